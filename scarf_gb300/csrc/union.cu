// a9: fuzzy union U = mix*(G + G^T - G o G^T) + (1-mix)*(G o G^T) of a COO
// graph, as CSR with sorted column indices and zeros removed
// (scarf/umap.py:118-123; mix = 1 is load_graph's symmetrize,
// scarf/datastore/graph_datastore.py:1052-1055).
//
// Every kept edge e = (r, c, w) lands twice in per-row buckets: as an "out"
// item in bucket r and as an "in" item in bucket c. An item is one 64-bit key
// (column << 33 | tag << 32 | e), so sorting a bucket groups its entries by
// column, puts G's entries before G^T's and keeps input order among
// duplicates. Buckets are sorted by a warp-level bitonic network in shared
// memory (<= 256 items) or by a CTA-level bitonic network over a padded scratch
// region (larger buckets). A warp-wide walk over each sorted bucket then yields
// a = sum of G's weights and b = sum of G^T's for every column, and the value
// in FP64 with the operation order of scipy's sparse add/multiply (no fused
// multiply-add), so the result is bit-identical to the reference's.
#include "common.cuh"

namespace {

constexpr int kSmallBucket = 256;
constexpr unsigned long long kPad = ~0ull;

__device__ __forceinline__ bool keep_edge(int64_t e, int k, int use_k) { return use_k >= k || (e % k) < use_k; }

__global__ void degree_kernel(const int64_t* __restrict__ edges, int64_t nnz, int64_t n, int k, int use_k,
                              int* __restrict__ deg, unsigned long long* __restrict__ bad) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nnz; e += int64_t(gridDim.x) * blockDim.x) {
    if (!keep_edge(e, k, use_k)) continue;
    const int64_t r = edges[2 * e], c = edges[2 * e + 1];
    if (r < 0 || r >= n || c < 0 || c >= n) {
      atomicAdd(bad, 1ull);
      continue;
    }
    atomicAdd(&deg[r], 1);
    atomicAdd(&deg[c], 1);
  }
}

// ---- exclusive scan of n ints into n+1 int64 (three phases) --------------
constexpr int kScanTile = 1024;

__global__ void scan_tiles_kernel(const int* __restrict__ in, int64_t n, long long* __restrict__ tile_sums) {
  __shared__ long long red[256];
  const int64_t a = int64_t(blockIdx.x) * kScanTile;
  long long s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += 256)
    if (a + i < n) s += in[a + i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = red[0];
}

__global__ void scan_sums_kernel(long long* __restrict__ tile_sums, int64_t ntiles) {
  // one CTA: exclusive scan in place, 1024 at a time
  __shared__ long long buf[1024];
  long long carry = 0;
  for (int64_t b = 0; b < ntiles; b += 1024) {
    const int64_t i = b + threadIdx.x;
    long long v = i < ntiles ? tile_sums[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      long long t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < ntiles) tile_sums[i] = carry + buf[threadIdx.x] - v;
    carry += buf[1023];
    __syncthreads();
  }
}

__global__ void scan_apply_kernel(const int* __restrict__ in, int64_t n, const long long* __restrict__ tile_off,
                                  int64_t* __restrict__ out) {
  __shared__ long long buf[kScanTile];
  const int64_t a = int64_t(blockIdx.x) * kScanTile;
  const int i = threadIdx.x;  // 1024 threads
  const long long v = (a + i < n) ? in[a + i] : 0;
  buf[i] = v;
  __syncthreads();
  for (int o = 1; o < kScanTile; o <<= 1) {
    long long t = i >= o ? buf[i - o] : 0;
    __syncthreads();
    buf[i] += t;
    __syncthreads();
  }
  if (a + i < n) out[a + i] = tile_off[blockIdx.x] + buf[i] - v;
  if (a + i == n - 1) out[n] = tile_off[blockIdx.x] + buf[i];
}

__global__ void scatter_kernel(const int64_t* __restrict__ edges, int64_t nnz, int64_t n, int k, int use_k,
                               const int64_t* __restrict__ bptr, int* __restrict__ cursor,
                               unsigned long long* __restrict__ items) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nnz; e += int64_t(gridDim.x) * blockDim.x) {
    if (!keep_edge(e, k, use_k)) continue;
    const int64_t r = edges[2 * e], c = edges[2 * e + 1];
    if (r < 0 || r >= n || c < 0 || c >= n) continue;
    const unsigned long long lo = static_cast<unsigned long long>(static_cast<uint32_t>(e));
    const int64_t pr = bptr[r] + atomicAdd(&cursor[r], 1);
    items[pr] = (static_cast<unsigned long long>(c) << 33) | lo;               // G entry (r, c)
    const int64_t pc = bptr[c] + atomicAdd(&cursor[c], 1);
    items[pc] = (static_cast<unsigned long long>(r) << 33) | (1ull << 32) | lo;  // G^T entry (c, r)
  }
}

// warp per bucket; buckets above kSmallBucket are queued for the CTA sorter
__global__ void sort_small_kernel(unsigned long long* __restrict__ items, const int64_t* __restrict__ bptr, int64_t n,
                                  int* __restrict__ big, int* __restrict__ nbig) {
  __shared__ unsigned long long sh[8][kSmallBucket];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = int64_t(blockIdx.x) * 8 + warp;
  if (r >= n) return;
  const int64_t a = bptr[r];
  const int size = int(bptr[r + 1] - a);
  if (size <= 1) return;
  if (size > kSmallBucket) {
    if (lane == 0) big[atomicAdd(nbig, 1)] = int(r);
    return;
  }
  int P = 2;
  while (P < size) P <<= 1;
  unsigned long long* s = sh[warp];
  for (int i = lane; i < P; i += 32) s[i] = i < size ? items[a + i] : kPad;
  __syncwarp();
  for (int kk = 2; kk <= P; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long x = s[i], y = s[l];
          const bool up = (i & kk) == 0;
          if ((x > y) == up) {
            s[i] = y;
            s[l] = x;
          }
        }
      }
      __syncwarp();
    }
  }
  for (int i = lane; i < size; i += 32) items[a + i] = s[i];
}

// CTA per large bucket: bitonic network over a padded copy in scratch
__global__ void sort_big_kernel(unsigned long long* __restrict__ items, const int64_t* __restrict__ bptr,
                                const int* __restrict__ big, const int* __restrict__ nbig,
                                unsigned long long* __restrict__ pad) {
  const int cnt = *nbig;
  for (int b = blockIdx.x; b < cnt; b += gridDim.x) {
    const int64_t r = big[b];
    const int64_t a = bptr[r];
    const int64_t size = bptr[r + 1] - a;
    int64_t P = 2;
    while (P < size) P <<= 1;
    unsigned long long* s = pad + 2 * a;  // region [2a, 2a + P) lies inside [2a, 2*bptr[r+1])
    for (int64_t i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < size ? items[a + i] : kPad;
    __syncthreads();
    for (int64_t kk = 2; kk <= P; kk <<= 1) {
      for (int64_t j = kk >> 1; j > 0; j >>= 1) {
        for (int64_t i = threadIdx.x; i < P; i += blockDim.x) {
          const int64_t l = i ^ j;
          if (l > i) {
            const unsigned long long x = s[i], y = s[l];
            const bool up = (i & kk) == 0;
            if ((x > y) == up) {
              s[i] = y;
              s[l] = x;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int64_t i = threadIdx.x; i < size; i += blockDim.x) items[a + i] = s[i];
    __syncthreads();
  }
}

// value of one column group, scipy's operation order
__device__ __forceinline__ double union_value(bool has_a, bool has_b, double a, double b, double mix) {
  double u;
  if (has_a && has_b) u = __dsub_rn(__dadd_rn(a, b), __dmul_rn(a, b));
  else u = has_a ? a : b;
  double v = __dmul_rn(mix, u);
  if (has_a && has_b) v = __dadd_rn(v, __dmul_rn(__dsub_rn(1.0, mix), __dmul_rn(a, b)));
  return v;
}

// Warp per row: the bucket is read 32 items at a time (coalesced); the
// first item of each column group (its head) sums the group's G and G^T
// weights in bucket order, which is scipy's order, and the kept values are
// compacted in column order with a ballot.
template <bool kWrite>
__global__ void walk_kernel(const unsigned long long* __restrict__ items, const int64_t* __restrict__ bptr, int64_t n,
                            const double* __restrict__ w, double mix, unsigned flags, int* __restrict__ count,
                            const int64_t* __restrict__ optr, int32_t* __restrict__ oind, double* __restrict__ odat,
                            int64_t capacity) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (r >= n) return;  // whole warps
  const int64_t a = bptr[r], b = bptr[r + 1];
  const bool upper = flags & SG_UNION_UPPER_ONLY;
  int64_t o = kWrite ? optr[r] : 0;
  int cnt = 0;
  for (int64_t base = a; base < b; base += 32) {
    const int64_t p = base + lane;
    const bool valid = p < b;
    const unsigned long long key = valid ? items[p] : 0ull;
    const long long col = static_cast<long long>(key >> 33);
    long long prev = __shfl_up_sync(0xffffffffu, col, 1);
    if (lane == 0) prev = p > a ? static_cast<long long>(items[p - 1] >> 33) : -1;
    bool keep = false;
    double v = 0.0;
    if (valid && col != prev) {
      double sa = 0.0, sb = 0.0;
      bool ha = false, hb = false;
      for (int64_t q = p; q < b; ++q) {
        const unsigned long long it = q == p ? key : items[q];
        if (static_cast<long long>(it >> 33) != col) break;
        const double wv = w[it & 0xffffffffull];
        if ((it >> 32) & 1ull) {
          sb = hb ? __dadd_rn(sb, wv) : wv;
          hb = true;
        } else {
          sa = ha ? __dadd_rn(sa, wv) : wv;
          ha = true;
        }
      }
      v = union_value(ha, hb, sa, sb, mix);
      keep = v != 0.0 && (!upper || col >= r);
    }
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    if (kWrite && keep) {
      const int64_t pos = o + __popc(ball & ((1u << lane) - 1u));
      if (pos < capacity) {
        oind[pos] = int32_t(col);
        odat[pos] = v;
      }
    }
    o += __popc(ball);
    cnt += __popc(ball);
  }
  if (!kWrite && lane == 0) count[r] = cnt;
}

}  // namespace

extern "C" int sg_fuzzy_union(sg_handle* h, const int64_t* edges, const double* w, int64_t nnz, int64_t n, int32_t k,
                              int32_t use_k, double mix, uint32_t flags, int64_t* indptr_out, int32_t* indices_out,
                              double* data_out, int64_t capacity, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(indptr_out && (nnz == 0 || (edges && w)), "sg_fuzzy_union: null pointer argument");
  SG_ARG(n >= 1 && n < (int64_t(1) << 31), "sg_fuzzy_union: n=%lld outside [1, 2^31)", (long long)n);
  // per-row bucket degrees, cursors and walk counts are 32-bit: with fewer
  // than 2^30 edges no bucket (at most 2 * nnz items) can overflow them
  SG_ARG(nnz >= 0 && nnz < (int64_t(1) << 30), "sg_fuzzy_union: nnz=%lld outside [0, 2^30)", (long long)nnz);
  SG_ARG(k >= 1, "sg_fuzzy_union: k must be >= 1");
  if (use_k < 1) use_k = 1;
  if (use_k > k) use_k = k;
  const int64_t total = 2 * nnz;
  const int64_t ntiles = sg::ceil_div(n, kScanTile);
  const size_t need = sg::Carver::need(sizeof(int) * n) * 2 + sg::Carver::need(sizeof(int64_t) * (n + 1)) +
                      sg::Carver::need(sizeof(long long) * (ntiles + 1)) +
                      sg::Carver::need(sizeof(unsigned long long) * (total + 1)) +
                      sg::Carver::need(sizeof(unsigned long long) * (2 * total + 2)) +
                      sg::Carver::need(sizeof(int) * (n + 1)) + 512;
  int status;
  void* wsp = sg::ws_get(h, need, &status);
  if (!wsp) return status;
  sg::Carver cv(wsp);
  int* deg = cv.take<int>(n);
  int* cursor = cv.take<int>(n);
  int64_t* bptr = cv.take<int64_t>(n + 1);
  long long* tsum = cv.take<long long>(ntiles + 1);
  unsigned long long* items = cv.take<unsigned long long>(total + 1);
  unsigned long long* pad = cv.take<unsigned long long>(2 * total + 2);
  int* big = cv.take<int>(n + 1);
  int* nbig = cv.take<int>(1);
  unsigned long long* bad = cv.take<unsigned long long>(1);

  sg::ProfScope prof(h, "union", st);
  SG_CUDA(cudaMemsetAsync(deg, 0, sizeof(int) * n, st));
  SG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * n, st));
  SG_CUDA(cudaMemsetAsync(nbig, 0, sizeof(int), st));
  SG_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st));
  const int eg = int(std::min<int64_t>(sg::ceil_div(std::max<int64_t>(nnz, 1), 256), int64_t(h->sm_count) * 16));
  degree_kernel<<<eg, 256, 0, st>>>(edges, nnz, n, k, use_k, deg, bad);
  SG_LAUNCH_CHECK();
  auto scan = [&](const int* in, int64_t* out) -> int {
    scan_tiles_kernel<<<unsigned(ntiles), 256, 0, st>>>(in, n, tsum);
    SG_LAUNCH_CHECK();
    scan_sums_kernel<<<1, 1024, 0, st>>>(tsum, ntiles);
    SG_LAUNCH_CHECK();
    scan_apply_kernel<<<unsigned(ntiles), kScanTile, 0, st>>>(in, n, tsum, out);
    SG_LAUNCH_CHECK();
    return SG_OK;
  };
  int rc = scan(deg, bptr);
  if (rc) return rc;
  scatter_kernel<<<eg, 256, 0, st>>>(edges, nnz, n, k, use_k, bptr, cursor, items);
  SG_LAUNCH_CHECK();
  sort_small_kernel<<<unsigned(sg::ceil_div(n, 8)), 256, 0, st>>>(items, bptr, n, big, nbig);
  SG_LAUNCH_CHECK();
  sort_big_kernel<<<unsigned(h->sm_count), 1024, 0, st>>>(items, bptr, big, nbig, pad);
  SG_LAUNCH_CHECK();
  walk_kernel<false><<<sg::ceil_div_i(n, 8), 256, 0, st>>>(items, bptr, n, w, mix, flags, deg, nullptr, nullptr,
                                                              nullptr, 0);
  SG_LAUNCH_CHECK();
  rc = scan(deg, indptr_out);
  if (rc) return rc;
  walk_kernel<true><<<sg::ceil_div_i(n, 8), 256, 0, st>>>(items, bptr, n, w, mix, flags, nullptr, indptr_out,
                                                             indices_out, data_out, capacity);
  SG_LAUNCH_CHECK();
  unsigned long long hbad = 0;
  int64_t hnnz = 0;
  SG_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaMemcpyAsync(&hnnz, indptr_out + n, sizeof(hnnz), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (hbad) return sg::fail(SG_ERR_ARG, "sg_fuzzy_union: %llu edges have a row or column outside [0, %lld)", hbad, (long long)n);
  if (hnnz > capacity)
    return sg::fail(SG_ERR_ARG, "sg_fuzzy_union: the union has %lld entries, more than capacity %lld", (long long)hnnz,
                    (long long)capacity);
  return SG_OK;
}
