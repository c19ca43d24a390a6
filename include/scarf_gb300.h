/*
 * scarf_gb300 -- C ABI of the GB300 (sm_103a) graph-construction path of scarf.
 *
 * Every entry point takes caller-owned DEVICE pointers (plain pointers and
 * sizes, no C++ or torch types), an explicit cudaStream_t passed as void*, and
 * returns an int status (SG_OK = 0, negative on error; the message is in
 * sg_last_error(), which is per host thread). Calls are asynchronous on the
 * given stream unless stated otherwise; completion means the caller has
 * synchronised that stream. The library never frees caller memory. Scratch
 * memory belongs to the handle: it grows on demand up to the handle's HBM
 * budget and is reused by later calls, so calls made with one handle must be
 * issued on one stream (or be ordered by the caller). One handle per host
 * thread.
 *
 * Reference paths are relative to the scarf project root (v0.32.3).
 */
#ifndef SCARF_GB300_H
#define SCARF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_handle sg_handle;

enum {
  SG_OK = 0,
  SG_ERR_ARG = -1,         /* bad shape, size, pointer or flag */
  SG_ERR_OOM = -2,         /* device allocation failed */
  SG_ERR_CUDA = -3,        /* a CUDA runtime / library call failed */
  SG_ERR_TIMEOUT = -4,     /* a bounded device wait ran out */
  SG_ERR_BUDGET = -5,      /* scratch would exceed the handle's HBM budget */
  SG_ERR_UNSUPPORTED = -6  /* valid request this build does not implement */
};

/* element types */
enum { SG_F32 = 0, SG_BF16 = 1, SG_F64 = 2 };
/* numeric forms */
enum { SG_PLAIN = 0, SG_PRECISION = 1 };
/* sg_normalize_csr flags */
#define SG_NORM_LOG1P 1u          /* log_transform=True   (scarf/assay.py:54-64) */
#define SG_NORM_RENORM_SUBSET 2u  /* renormalize_subset=True (scarf/assay.py:818-823) */
/* sg_fuzzy_union flags */
#define SG_UNION_UPPER_ONLY 1u    /* load_graph(upper_only=True): triu (graph_datastore.py:1071-1072) */

int sg_version(void);
const char* sg_last_error(void);

/* Create a handle on `device` whose scratch may grow to `hbm_budget_bytes`
 * (0 = no limit). No reference counterpart: scarf holds no device state. */
int sg_create(int device, size_t hbm_budget_bytes, sg_handle** out);
int sg_destroy(sg_handle* h);
/* Bytes of scratch the handle holds now. */
size_t sg_workspace_bytes(const sg_handle* h);

/* Diagnostics (no reference counterpart): number of this library's kernels
 * launched by the process so far; per-kernel device time measured with CUDA
 * events around the named launches while profiling is on. Names:
 * "normalize", "cov_simt", "cov_tc", "project", "knn_simt", "knn_tc",
 * "rerank", "smooth", "union". sg_profile_query synchronises the recorded
 * events. */
unsigned long long sg_kernel_launches(void);
int sg_profile(sg_handle* h, int enable);

/* Autotuning (no reference counterpart): with enable != 0, the first
 * precision-form sg_knn of a shape bucket (log2 of the query rows, log2 of the
 * reference rows, d, candidate-list length, self-kNN or not) with at least
 * 1e9 query-reference pairs times three reference split counts (each with and
 * without the locality order for a self-kNN) and keeps the fastest for later
 * calls of that bucket on this handle. Off by default: the first call of a
 * bucket then costs three to six calls. sg_knn_last_splits returns the split
 * count of the last precision-form sg_knn. */
int sg_set_autotune(sg_handle* h, int enable);
int sg_knn_last_splits(const sg_handle* h);
/* 1 when the last precision-form sg_knn on the handle ran its self-kNN in the
 * locality order (rows sorted by their nearest pilot row, each CTA starting
 * its reference scan at its own rows), else 0. The autotuner times a
 * self-kNN with and without it. */
int sg_knn_last_locality(const sg_handle* h);
int sg_profile_reset(sg_handle* h);

/* Bounded-wait test hooks (no reference counterpart). Every mbarrier wait of
 * the tensor-core kernels gives up after a number of polls (2^22 by default),
 * raises the kernel's error flag, lets the CTA's own copies and MMAs finish,
 * frees its tensor memory and returns; the call then returns SG_ERR_TIMEOUT
 * and the context stays usable. sg_set_wait_limit sets that poll limit for
 * later calls on the handle (0 = the default). sg_test_idle_mma makes the
 * next precision-form sg_knn on the handle launch its kernel with the MMA
 * issuer idle, so that the copy and epilogue waits run out on a barrier that
 * nothing arrives at; it faults nothing and leaves no work in flight. */
int sg_set_wait_limit(sg_handle* h, uint32_t polls);
int sg_test_idle_mma(sg_handle* h);
int sg_profile_query(sg_handle* h, const char* name, double* total_ms, long long* count);

/* a1+a3 -- library-size normalisation of CSR counts with the feature gather,
 * fused with the column sums of the written values.
 * Replaces RNAassay.normed (scarf/assay.py:780-828) with norm_lib_size /
 * norm_lib_size_log (scarf/assay.py:41-64) and the two statistics passes of
 * make_graph (scarf/datastore/graph_datastore.py:767-796).
 *   indptr[n_rows+1]: row r's entries are indices/data[indptr[r]-indptr[0] ..
 *   indptr[r+1]-indptr[0]); col_map[n_genes]: output column of a gene or -1.
 *   s_r = integer sum of the mapped counts (0 -> 1) when SG_NORM_RENORM_SUBSET,
 *   else n_counts[r]. out[r*ld_out + j] = log1p(size_factor*c/s_r) (or without
 *   log1p), written as SG_F32 or SG_BF16. Columns with missing_mask[j] != 0
 *   take fill_value instead (mapping_utils.py:208 fills 1.0); missing_mask may
 *   be NULL. libsize_out[n_rows] (int64, may be NULL) receives s_r for the
 *   renormalised form. colsum/colsumsq (n_cols doubles, may be NULL) are
 *   ACCUMULATED with the sums of the written values, in a fixed order.
 *   indptr/indices/data may be device memory or page-locked host memory
 *   (cudaHostAlloc / cudaHostRegister): the kernel then reads the rows over
 *   the host link itself, with no staging copy. Pageable host memory is
 *   refused with SG_ERR_ARG. */
int sg_normalize_csr(sg_handle* h, const int64_t* indptr, const int32_t* indices,
                     const int32_t* data, int64_t n_rows, const int32_t* col_map,
                     int64_t n_genes, int32_t n_cols, const uint8_t* missing_mask,
                     float fill_value, const double* n_counts, double size_factor,
                     uint32_t flags, void* out, int64_t ld_out, int32_t out_dtype,
                     int64_t* libsize_out, double* colsum, double* colsumsq, void* stream);

/* a3 -- mu = sum/n, sigma = sqrt(sumsq/n - mu^2) (population std), then
 * clean_array: NaN/inf -> 0 and sigma == 0 -> 1 (scarf/utils.py:143-153,
 * graph_datastore.py:767-796). f32 copies (may be NULL) feed the kernels. */
int sg_zstats(sg_handle* h, const double* colsum, const double* colsumsq, int64_t n_rows,
              int32_t n_cols, double* mu, double* sigma, float* mu32, float* sigma32,
              void* stream);

/* a4 -- scatter of the z-scaled rows, z = (x - mu)/sigma, over rows with
 * row_mask[r] != 0 (row_mask may be NULL = all): cov (n_cols^2 doubles,
 * symmetric, row-major) and zsum (n_cols doubles) are ACCUMULATED.
 * SG_PLAIN: FP32 SIMT products; SG_PRECISION: 3xBF16 split products on the
 * tcgen05 tensor cores with FP32 accumulation. Partials are reduced in FP64.
 * Replaces the IncrementalPCA fit of AnnStream._fit_pca (scarf/ann.py:207-256). */
int sg_covariance(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld,
                  const float* mu32, const float* sigma32, const uint8_t* row_mask,
                  int32_t precision, double* cov, double* zsum, void* stream);

/* a4 -- principal axes of the centred scatter cov - zsum zsum^T / n_used by an
 * FP64 eigendecomposition on the device. comps[n_cols*n_comp] (row-major,
 * column c = c-th largest) with the largest-magnitude entry of each component
 * positive (scikit-learn svd_flip(u_based_decision=False)); evals[n_comp]
 * descending; evr[n_comp] = eval / trace (explained_variance_ratio_);
 * loadings32[n_cols*ld_l] = the first n_load components as float32 (the
 * reference's loadings = components_[:-1].T, ann.py:256). Synchronises the
 * stream. Any output pointer except comps may be NULL. */
int sg_pca_basis(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                 int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                 int32_t n_load, float* loadings32, int32_t ld_l, void* stream);

/* a4 -- the same outputs as sg_pca_basis from a mixed-precision solver: an
 * FP32 partial eigendecomposition of the centred scatter (the n_comp + 16
 * largest pairs), then an FP64 Rayleigh-Ritz step on that subspace (FP64
 * Cholesky-QR, FP64 Q^T A Q and its FP64 eigendecomposition). Separated
 * components agree with sg_pca_basis to FP32 eigenvector accuracy.
 * Synchronises the stream. No counterpart in the reference beyond the
 * IncrementalPCA fit it also replaces (scarf/ann.py:207-256). */
int sg_pca_basis_mixed(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                       int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                       int32_t n_load, float* loadings32, int32_t ld_l, void* stream);

/* a4 -- the same outputs as sg_pca_basis from a Chebyshev-filtered block
 * subspace iteration: FP32 GEMMs apply Chebyshev polynomials of the centred
 * scatter (damped on [0, cut], cut = the block's smallest Ritz value) to a
 * block of ~2.5 (n_comp + 16) columns, re-orthonormalised by FP32
 * Cholesky-QR2 after each segment; an FP32 Rayleigh-Ritz step picks the
 * n_comp + 16 largest Ritz vectors and the FP64 Rayleigh-Ritz step of
 * sg_pca_basis_mixed refines them. When a wanted FP64 Ritz pair has a
 * residual ||A v - w v|| above 1e-4 of the largest eigenvalue, or the matrix
 * is too small for the block, the result comes from sg_pca_basis_mixed.
 * Synchronises the stream. No counterpart in the reference beyond the
 * IncrementalPCA fit it also replaces (scarf/ann.py:207-256). */
int sg_pca_basis_filter(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                        int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                        int32_t n_load, float* loadings32, int32_t ld_l, void* stream);

/* Max relative FP64 residual of the wanted pairs in the last
 * sg_pca_basis_filter call on this handle: NaN when the call took the dense
 * route for a small matrix, infinity when it fell back to it. No counterpart
 * in the reference. */
double sg_pca_filter_residual(const sg_handle* h);

/* a5 -- the reducer ((x - mu)/sigma) . L (scarf/ann.py:129-138, :191-192):
 * scores[r*ld_s + c], c < d (columns d..ld_s-1 are written 0). bf16_out (may be
 * NULL) receives a BF16 copy with row stride ld_b (zero padded).
 * SG_PLAIN: FP32 SIMT products of the centred values. SG_PRECISION (d <= 64):
 * x . (L/sigma) - mu^T (L/sigma) on the tcgen05 tensor cores, each factor split
 * into BF16 hi + lo and the products hi.hi + hi.lo + lo.hi accumulated in FP32
 * (about 1e-5 of the scores' scale); x must then be finite. */
int sg_project(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld,
               const float* mu32, const float* sigma32, const float* loadings32, int32_t d,
               int32_t ld_l, float* scores, int32_t ld_s, void* bf16_out, int32_t ld_b,
               int32_t precision, void* stream);

/* a6/a7/a10 -- exact squared-L2 kNN of queries[nq x d] (row stride ld) against
 * refs[nr x d], replacing the hnswlib index (scarf/ann.py:14-28, :290-326) and
 * AnnStream.transform_ann (scarf/ann.py:194-205).
 * self_offset >= 0: query q is reference row self_offset+q; k+1 neighbours are
 *   found and self is removed with fix_knn_query's rule (scarf/ann.py:31-52):
 *   column 0 if it is self, else the first self position, else the last
 *   column; *n_missed (device int64, ACCUMULATED) counts rows whose first hit
 *   was not self, i.e. self_query_knn's recall (scarf/knn_utils.py:23-76).
 * self_offset < 0: plain query of k neighbours (run_mapping,
 *   scarf/datastore/mapping_datastore.py:198-208); n_missed may be NULL.
 * precision SG_PLAIN: FP32 candidate distances; SG_PRECISION: BF16 tcgen05
 * distance GEMM. Both keep k(+1)+margin candidates per query and re-rank them
 * with exact FP32 sum((q-r)^2), ties by index. idx_out[nq*k] int64,
 * dist_out[nq*k] float32 (hnswlib 'l2' returns squared distances). */
int sg_knn(sg_handle* h, const float* queries, int64_t nq, const float* refs, int64_t nr,
           int32_t d, int32_t ld, int32_t k, int64_t self_offset, int32_t margin,
           int32_t precision, int64_t* idx_out, float* dist_out, int64_t* n_missed,
           void* stream);

/* a8 -- smoothen_dists (scarf/knn_utils.py:89-159) over umap-learn's
 * smooth_knn_dist and compute_membership_strengths, chunk by chunk of
 * chunk_rows rows: rho/sigma per row (sigma sum from column 1), weights in
 * float32, weight 0 where the neighbour index equals the chunk-local row, then
 * zero weights replaced by global_min = min(1, smallest non-zero weight of each
 * chunk holding a zero). edges_out[n*k*2] int64 pairs (row, col) in row-major
 * order (the (n*k, 2) u8 dataset), w_out[n*k] float64. */
int sg_smooth(sg_handle* h, const int64_t* knn_idx, const float* knn_dist, int64_t n,
              int32_t k, double local_connectivity, double bandwidth, int64_t chunk_rows,
              int64_t* edges_out, double* w_out, void* stream);

/* sg_smooth for callers that must not have device memory allocated on their
 * behalf (a host that owns the whole HBM budget through its own pool, a
 * latency-critical loop that cannot take cudaMalloc's device-wide
 * synchronisation, a plugin host that forbids allocations outside its
 * allocator). No counterpart in the reference: scarf never touches a device.
 * Same arguments and results as sg_smooth without a handle; runs on the
 * current device. Its scratch (three words per chunk of rows) is a fixed
 * array of static device memory in the library (256 KB, held on every GPU
 * that loads the library until the process exits): at most 2^14 chunks
 * (n / chunk_rows, rounded up) per call, larger requests return SG_ERR_ARG.
 * Nothing is allocated or freed. The first call on a device (and the first
 * call under a context other than the one of the last lookup) looks up the
 * array's device address with cudaGetSymbolAddress; make that first call
 * before any stream capture. A device reset between calls is not supported.
 * All calls share the one array, so calls whose work overlaps on the GPU
 * (other streams, other host threads) race: order them. */
int sg_smooth_noalloc(const int64_t* knn_idx, const float* knn_dist, int64_t n, int32_t k,
                      double local_connectivity, double bandwidth, int64_t chunk_rows,
                      int64_t* edges_out, double* w_out, void* stream);

/* a9 -- fuzzy union of the graph G given as COO (edges[nnz*2] int64 pairs,
 * w[nnz] float64, k edges per row in row-major order; use_k < k keeps the first
 * use_k of each row as _store_to_sparse does, graph_datastore.py:474-511;
 * duplicates are summed): U = mix*(G + G^T - G o G^T) + (1-mix)*(G o G^T)
 * with zeros removed (umap.py:118-123; mix = 1 is load_graph's symmetrize,
 * graph_datastore.py:1052-1055). FP64 with the reference's operation order,
 * so values are bit-identical to scipy's. Output CSR with sorted column
 * indices: indptr_out[n+1] (int64; indptr_out[n] is the nnz), indices_out and
 * data_out with room for `capacity` entries (2*nnz always suffices).
 * nnz < 2^30. */
int sg_fuzzy_union(sg_handle* h, const int64_t* edges, const double* w, int64_t nnz, int64_t n,
                   int32_t k, int32_t use_k, double mix, uint32_t flags, int64_t* indptr_out,
                   int32_t* indices_out, double* data_out, int64_t capacity, void* stream);

/* b2 -- the mapping service (run_mapping's query, scarf/datastore/
 * mapping_datastore.py:198-208, with align_features' fill of absent features,
 * scarf/mapping_utils.py:148-214) as a native continuous-batching server, for
 * hosts that are not Python. The reference is caller-owned device memory that
 * must outlive the server: mu32/sigma32 (n_feats), loadings32 (n_feats x ld_l,
 * the first d columns used), ref_scores (n_ref x ld_ref). The query panel is
 * fixed per server: col_map[n_genes] maps a target gene to its reference
 * feature or -1, missing_mask[n_feats] != 0 marks features the target lacks
 * (filled with 1.0 after normalisation); both are host arrays, copied.
 * norm_flags are sg_normalize_csr's; precision is the form of sg_project and
 * sg_knn (margin 16 in the precision form). n_workers threads each own a CUDA
 * stream, a library handle and batch buffers on `device`.
 * Requests are admitted in arrival order while the HBM they need (rows x
 * (normalised row + scores + results) + 8 bytes per non-zero) fits
 * hbm_budget_bytes; one that cannot fit alone finishes with SG_ERR_BUDGET.
 * Each batch takes up to max_batch_rows rows from the admitted requests,
 * shortest remaining first, so large requests are served in row slices and
 * small ones that arrive meanwhile join the next batch; a row's result does
 * not depend on its batch. */
typedef struct sg_server sg_server;
int sg_serve_create(int device, const float* mu32, const float* sigma32, const float* loadings32,
                    int32_t n_feats, int32_t d, int32_t ld_l, const float* ref_scores, int64_t n_ref,
                    int32_t ld_ref, const int32_t* col_map, int64_t n_genes, const uint8_t* missing_mask,
                    int32_t k, int32_t precision, double size_factor, uint32_t norm_flags,
                    int32_t max_batch_rows, size_t hbm_budget_bytes, int32_t n_workers, sg_server** out);
/* Queue n_rows target cells given as HOST CSR (indptr[n_rows+1] int64 with
 * row r's entries at indices/data[indptr[r]-indptr[0] ..]); the arrays must
 * stay valid and unchanged until the request is done. *request_id names it. */
int sg_serve_submit(sg_server* s, const int64_t* indptr, const int32_t* indices, const int32_t* data,
                    int64_t n_rows, int64_t* request_id);
/* *done = 1 once the request has finished (with results or an error). */
int sg_serve_poll(sg_server* s, int64_t request_id, int32_t* done);
/* Block until the request is done or timeout_ms passes (SG_ERR_TIMEOUT). */
int sg_serve_wait(sg_server* s, int64_t request_id, int64_t timeout_ms);
/* The finished request's k nearest reference rows (idx_out, int64) and squared
 * distances (dist_out, float32), n_rows x k host arrays; releases the request.
 * Returns the request's own status (SG_ERR_BUDGET, a CUDA error, ...). */
int sg_serve_result(sg_server* s, int64_t request_id, int64_t* idx_out, float* dist_out);
/* GPU batches run and rows mapped so far (either pointer may be NULL). */
int sg_serve_stats(sg_server* s, int64_t* batches, int64_t* rows);
/* Stop the workers after their current batch and free the server; requests
 * not yet done are abandoned. */
int sg_serve_destroy(sg_server* s);

/* f2 -- decoding of scarf's zarr chunks on the device: numcodecs Blosc frames
 * (c-blosc 1.x layout, LZ4 codec, with bit shuffle, byte shuffle or none,
 * split or whole blocks, or plain copies), as scarf's create_zarr_dataset
 * writes them (scarf/writers.py:58-89; dense uint32 counts at :164-204).
 * frames: HOST bytes, frame f at [frame_offsets[f], frame_offsets[f+1]);
 * frame f decodes into the DEVICE buffer out (out_bytes long) at byte
 * out_starts[f] (HOST array), its header's uncompressed size long. Headers are
 * checked on the host; the LZ4 streams are decoded one warp each and the
 * shuffles undone on the device. A malformed stream returns SG_ERR_ARG (every
 * device read and write is bounds-checked). Synchronises the stream. */
int sg_blosc_decode(sg_handle* h, const uint8_t* frames, const int64_t* frame_offsets, int32_t n_frames,
                    void* out, int64_t out_bytes, const int64_t* out_starts, void* stream);

/* f2 -- CSR rows of one band of decoded dense chunks (device memory): chunk k
 * of the band (k < ceil(n_cols / chunk_cols)) is chunk_rows x chunk_cols
 * uint32 in C order at chunks + k * chunk_rows * chunk_cols and covers
 * columns [k * chunk_cols, ...) of a matrix n_cols wide. Rows [0, n_rows) of
 * the band become indptr_out[n_rows + 1] (int64, starting at indptr_base) and,
 * in ascending column order, indices_out (int32) and data_out (int32; a count
 * above 2^31 - 1 is SG_ERR_ARG). *nnz_out receives the band's non-zeros; with
 * capacity 0 only indptr_out and *nnz_out are written (a counting pass).
 * Synchronises the stream. */
int sg_chunks_to_csr(sg_handle* h, const uint32_t* chunks, int64_t n_rows, int32_t chunk_rows,
                     int32_t chunk_cols, int64_t n_cols, int64_t indptr_base, int64_t* indptr_out,
                     int32_t* indices_out, int32_t* data_out, int64_t capacity, int64_t* nnz_out,
                     void* stream);

/* f2, writing -- one Blosc1 frame per chunk of device bytes, in the format
 * scarf's create_zarr_dataset writes through numcodecs (scarf/writers.py:
 * 58-89): LZ4 codec, blocks not split, bit shuffle (shuffle = 2), byte
 * shuffle (1) or none (0); a one-byte type is stored unshuffled. Chunk c is
 * src[chunk_offsets[c] - chunk_offsets[0], chunk_offsets[c + 1] -
 * chunk_offsets[0]) (src a device pointer, chunk_offsets a host array of
 * n_chunks + 1 non-decreasing offsets, each chunk below 2^31 - 64 bytes).
 * blocksize: bytes per Blosc block, a multiple of typesize, at most 32768.
 * The frames are written back to back into the host buffer frames_out
 * (frames_capacity bytes, at least sg_blosc_encode_bound(...)), frame c at
 * frame_offsets_out[c] (host, n_chunks + 1 entries). A block whose LZ4 stream
 * would not be shorter than the block is stored as it is. Synchronises the
 * stream. */
int sg_blosc_encode(sg_handle* h, const void* src, const int64_t* chunk_offsets, int32_t n_chunks, int32_t typesize,
                    int32_t shuffle, int32_t blocksize, void* frames_out, int64_t frames_capacity,
                    int64_t* frame_offsets_out, void* stream);

/* Host only: a frames_capacity that sg_blosc_encode always fits in (-1 for a
 * bad argument). */
int64_t sg_blosc_encode_bound(const int64_t* chunk_offsets, int32_t n_chunks, int32_t blocksize);

/* f1 -- the MiniBatchKMeans step of make_graph (scarf/ann.py:328-346):
 * MiniBatchKMeans(n_clusters=k, random_state=seed, batch_size=block_rows)
 * partial_fit over the row blocks of x[n x d] (row stride ld, a multiple of 4)
 * in order, then predict for every row. The first block initialises the
 * centres (its rows in order when it has exactly k rows, else greedy
 * k-means++); each block then moves the centres it is nearest to with
 * scikit-learn's count-weighted update (FP64) and reassigns centres below
 * 0.01 x the largest weight every 10 k rows or while one has no weight.
 * Random draws come from a counter hash of `seed`, not numpy's generator.
 * centers_out[k*d] float64 (row-major), labels_out[n] int32. 1 <= k <= 2048,
 * k <= block_rows <= 4096, d <= 64. */
int sg_kmeans_minibatch(sg_handle* h, const float* x, int64_t n, int32_t d, int32_t ld, int32_t k,
                        int32_t block_rows, uint64_t seed, double* centers_out, int32_t* labels_out,
                        void* stream);

/* f4 -- calc_snn (scarf/knn_utils.py:195-211): snn_out[i*k + j] =
 * |set(indices[i]) & set(indices[m])| / (k - 1) with m = indices[i*k + j]
 * (int64, row-major n x k; a negative m counts from the end, an m outside
 * [-n, n) scores 0). 2 <= k <= 64. */
int sg_calc_snn(sg_handle* h, const int64_t* indices, int64_t n, int32_t k, double* snn_out, void* stream);

/* f4 -- merge_graphs + weight_sort_indices (scarf/knn_utils.py:214-274) of
 * n_graphs kNN graphs of n rows and k neighbours each, given as host arrays
 * of device pointers: indices[g] (n x k int64), w[g] (n x k float64) and
 * snn[g] (n x k float64, from sg_calc_snn). Per row the candidates are ordered
 * by w + snn, largest first (ties: the later candidate first), the first
 * occurrence of each neighbour is kept, and the first k go to out_indices /
 * out_w (n x k; -1 / 0 pad a row with fewer than k distinct neighbours).
 * 1 <= n_graphs <= 8, n_graphs * k <= 128. */
int sg_merge_graphs(sg_handle* h, int32_t n_graphs, const int64_t* const* indices, const double* const* w,
                    const double* const* snn, int64_t n, int32_t k, int64_t* out_indices, double* out_w,
                    void* stream);

/* f3 -- the UMAP layout of the fused graph (scarf/umap.py:41-115: umap-learn's
 * optimize_layout_euclidean with move_other=True, densMAP off): n_epochs
 * epochs of attraction along the edges head[i] -> tail[i] (int32, E edges,
 * sampled every epochs_per_sample[i] epochs (float64, as umap-learn's
 * make_epochs_per_sample returns them); <= 0 never) and repulsion from
 * negative_sample_rate random vertices per sample, on embedding[n_vertices x
 * dim] float32 in place. a, b: the curve parameters (find_ab_params); gamma:
 * repulsion strength; alpha decays linearly from initial_alpha. The sampling
 * schedule is kept in float64 as umap-learn keeps it. Negative samples are
 * drawn from a counter hash of (seed, epoch, edge, sample).
 * sequential == 0: all edges of an epoch are processed concurrently, their
 * float32 steps added to the embedding atomically (reads may be stale, as in
 * umap-learn's parallel mode). sequential != 0: one thread runs the loop in
 * edge order with umap-learn's float64 gradient arithmetic on float32
 * coordinates, deterministically (small graphs: it is the reference
 * trajectory for tests). dim <= 8. */
int sg_umap_layout(sg_handle* h, const int32_t* head, const int32_t* tail, const double* epochs_per_sample,
                   int64_t n_edges, int64_t n_vertices, int32_t dim, float* embedding, int32_t n_epochs, float a,
                   float b, float gamma, float initial_alpha, float negative_sample_rate, uint64_t seed,
                   int32_t sequential, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SCARF_GB300_H */
