// a1 + a3: CSR library-size normalisation with the feature gather, fused with
// deterministic per-CTA column sums; FP64 reduction of the sums; z-statistics.
//
// Layout: one warp builds one dense output row in shared memory (the HVG
// counts are scattered into it, the integer library size is reduced across the
// warp, then the row is transformed in place and streamed out with 16-byte
// stores). After every round of `nwarps` rows the CTA folds the rows into
// per-column float32 accumulators held in shared memory, each column owned by
// one thread, always in the same order -- so the statistics are reproducible
// run to run. Per-CTA partials are reduced in FP64 in a fixed order.
#include "common.cuh"

#include <initializer_list>
#include <utility>

namespace {

constexpr int kRounds = 8;  // rows per warp per CTA

// CM: element type of the gene -> column map (int16_t when the output has
// fewer than 32768 columns, so that the map stays resident in L1)
template <bool kBf16, typename CM>
__global__ void normalize_kernel(const int64_t* __restrict__ indptr,
                                 const int32_t* __restrict__ indices,
                                 const int32_t* __restrict__ data, int64_t n_rows,
                                 const CM* __restrict__ col_map, int64_t n_genes, int n_cols, int vec,
                                 int pitch, const uint8_t* __restrict__ missing, float fill,
                                 const double* __restrict__ n_counts, float sf, unsigned flags,
                                 void* __restrict__ out, int64_t ld_out,
                                 int64_t* __restrict__ libsize_out, float* __restrict__ part_sum,
                                 float* __restrict__ part_sq) {
  extern __shared__ __align__(16) float smem[];
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* acc_s = smem;
  float* acc_q = smem + pitch;
  float* rows = smem + 2 * pitch;
  float* row = rows + warp * pitch;
  const bool renorm = flags & SG_NORM_RENORM_SUBSET;
  const bool do_log = flags & SG_NORM_LOG1P;
  const int64_t base = indptr[0];
  const int64_t row0 = int64_t(blockIdx.x) * nwarps * kRounds;

  for (int j = threadIdx.x; j < pitch; j += blockDim.x) {
    acc_s[j] = 0.f;
    acc_q[j] = 0.f;
  }

  for (int rnd = 0; rnd < kRounds; ++rnd) {
    const int64_t r = row0 + int64_t(rnd) * nwarps + warp;
    const bool valid = r < n_rows;
    float4* row4 = reinterpret_cast<float4*>(row);
    for (int j = lane; j < pitch / 4; j += 32) row4[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    long long s = 0;
    if (valid) {
      const int64_t p0 = indptr[r] - base, p1 = indptr[r + 1] - base;
      auto take = [&](int g, int c) {
        const int m = (unsigned)g < (unsigned long long)n_genes ? int(col_map[g]) : -1;
        if ((unsigned)m < (unsigned)n_cols) {
          s += c;
          atomicAdd(&row[m], float(c));
        }
      };
      if (vec) {
        // up to 3 entries before the first 16-byte boundary, then 16-byte
        // loads of indices and counts (two pairs in flight per lane), then
        // each lane's partial last block
        const int mis = int((reinterpret_cast<uintptr_t>(indices + p0) & 15) >> 2);
        const int64_t pa = min(p1, p0 + ((4 - mis) & 3));
        if (p0 + lane < pa) take(indices[p0 + lane], data[p0 + lane]);
        int64_t q = pa + 4 * lane;
        for (; q + 131 < p1; q += 256) {
          const int4 g0 = *reinterpret_cast<const int4*>(indices + q);
          const int4 c0 = *reinterpret_cast<const int4*>(data + q);
          const int4 g1 = *reinterpret_cast<const int4*>(indices + q + 128);
          const int4 c1 = *reinterpret_cast<const int4*>(data + q + 128);
          take(g0.x, c0.x); take(g0.y, c0.y); take(g0.z, c0.z); take(g0.w, c0.w);
          take(g1.x, c1.x); take(g1.y, c1.y); take(g1.z, c1.z); take(g1.w, c1.w);
        }
        for (; q + 3 < p1; q += 128) {
          const int4 g0 = *reinterpret_cast<const int4*>(indices + q);
          const int4 c0 = *reinterpret_cast<const int4*>(data + q);
          take(g0.x, c0.x); take(g0.y, c0.y); take(g0.z, c0.z); take(g0.w, c0.w);
        }
        for (int64_t e = q; e < p1 && e < q + 4; ++e) take(indices[e], data[e]);
      } else {
        int64_t p = p0 + lane;
        for (; p + 96 < p1; p += 128) {
          const int g0 = indices[p], g1 = indices[p + 32], g2 = indices[p + 64], g3 = indices[p + 96];
          const int c0 = data[p], c1 = data[p + 32], c2 = data[p + 64], c3 = data[p + 96];
          take(g0, c0); take(g1, c1); take(g2, c2); take(g3, c3);
        }
        for (; p < p1; p += 32) take(indices[p], data[p]);
      }
    }
    s = warp_sum_ll(s);
    double scal;
    if (renorm) {
      scal = (s == 0) ? 1.0 : double(s);
    } else {
      scal = valid ? n_counts[r] : 1.0;
    }
    const float sc = float(scal);
    __syncwarp();
    if (valid) {
      for (int j = lane; j < n_cols; j += 32) {
        float c = row[j];
        float v;
        if (c == 0.f && sc != 0.f) {
          v = 0.f;
        } else {
          v = __fdiv_rn(sf * c, sc);
          if (do_log) v = log1pf(v);
        }
        if (missing && missing[j]) v = fill;
        row[j] = v;
      }
      if (libsize_out && renorm && lane == 0) libsize_out[r] = (s == 0) ? 1 : s;
    }
    __syncwarp();
    if (valid) {
      if (kBf16) {
        __nv_bfloat16* o = static_cast<__nv_bfloat16*>(out) + r * ld_out;
        for (int j = lane * 2; j < n_cols; j += 64) {
          float a = row[j];
          float b = (j + 1 < n_cols) ? row[j + 1] : 0.f;
          if (j + 1 < n_cols) {
            *reinterpret_cast<__nv_bfloat162*>(o + j) = __floats2bfloat162_rn(a, b);
          } else {
            o[j] = __float2bfloat16_rn(a);
          }
        }
      } else {
        float4* o4 = reinterpret_cast<float4*>(static_cast<float*>(out) + r * ld_out);
        const int full = n_cols / 4;
        for (int j = lane; j < full; j += 32) o4[j] = row4[j];
        for (int j = full * 4 + lane; j < n_cols; j += 32) static_cast<float*>(out)[r * ld_out + j] = row[j];
      }
    }
    __syncthreads();
    // fold this round's rows into the column accumulators (fixed order)
    const int64_t left = n_rows - (row0 + int64_t(rnd) * nwarps);
    const int nvalid = left <= 0 ? 0 : (left < nwarps ? int(left) : nwarps);
    for (int j = threadIdx.x; j < n_cols; j += blockDim.x) {
      float a = acc_s[j], b = acc_q[j];
      for (int w = 0; w < nvalid; ++w) {
        float v = rows[w * pitch + j];
        a += v;
        b = fmaf(v, v, b);
      }
      acc_s[j] = a;
      acc_q[j] = b;
    }
    __syncthreads();
  }
  if (part_sum) {
    for (int j = threadIdx.x; j < n_cols; j += blockDim.x) {
      part_sum[int64_t(blockIdx.x) * n_cols + j] = acc_s[j];
      part_sq[int64_t(blockIdx.x) * n_cols + j] = acc_q[j];
    }
  }
}

// FP32 output without fused statistics: the same per-row arithmetic as
// normalize_kernel, but every warp walks its own rows (grid-stride) with no
// CTA-wide barrier, so a long row never holds the other warps of its CTA.
// The column statistics then come from colstats_kernel over the output.
template <typename CM>
__global__ void __launch_bounds__(256)
normalize_rows_kernel(const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                      const int32_t* __restrict__ data, int64_t n_rows, const CM* __restrict__ col_map,
                      int64_t n_genes, int n_cols, int vec, int pitch, const uint8_t* __restrict__ missing, float fill,
                      const double* __restrict__ n_counts, float sf, unsigned flags, float* __restrict__ out,
                      int64_t ld_out, int64_t* __restrict__ libsize_out) {
  extern __shared__ __align__(16) float smem[];
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* row = smem + warp * pitch;
  float4* row4 = reinterpret_cast<float4*>(row);
  const bool renorm = flags & SG_NORM_RENORM_SUBSET;
  const bool do_log = flags & SG_NORM_LOG1P;
  const int64_t base = indptr[0];
  const int64_t stride = int64_t(gridDim.x) * nwarps;
  for (int64_t r = int64_t(blockIdx.x) * nwarps + warp; r < n_rows; r += stride) {
    for (int j = lane; j < pitch / 4; j += 32) row4[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    long long s = 0;
    const int64_t p0 = indptr[r] - base, p1 = indptr[r + 1] - base;
    auto take = [&](int g, int c) {
      const int m = (unsigned)g < (unsigned long long)n_genes ? int(col_map[g]) : -1;
      if ((unsigned)m < (unsigned)n_cols) {
        s += c;
        atomicAdd(&row[m], float(c));
      }
    };
    if (vec) {
      const int mis = int((reinterpret_cast<uintptr_t>(indices + p0) & 15) >> 2);
      const int64_t pa = min(p1, p0 + ((4 - mis) & 3));
      if (p0 + lane < pa) take(indices[p0 + lane], data[p0 + lane]);
      int64_t q = pa + 4 * lane;
      // four 16-byte pairs in flight per lane
      for (; q + 387 < p1; q += 512) {
        int4 g[4], c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          g[u] = __ldcs(reinterpret_cast<const int4*>(indices + q + 128 * u));
          c[u] = __ldcs(reinterpret_cast<const int4*>(data + q + 128 * u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          take(g[u].x, c[u].x); take(g[u].y, c[u].y); take(g[u].z, c[u].z); take(g[u].w, c[u].w);
        }
      }
      for (; q + 3 < p1; q += 128) {
        const int4 g0 = __ldcs(reinterpret_cast<const int4*>(indices + q));
        const int4 c0 = __ldcs(reinterpret_cast<const int4*>(data + q));
        take(g0.x, c0.x); take(g0.y, c0.y); take(g0.z, c0.z); take(g0.w, c0.w);
      }
      for (int64_t e = q; e < p1 && e < q + 4; ++e) take(indices[e], data[e]);
    } else {
      int64_t p = p0 + lane;
      for (; p + 96 < p1; p += 128) {
        const int g0 = indices[p], g1 = indices[p + 32], g2 = indices[p + 64], g3 = indices[p + 96];
        const int c0 = data[p], c1 = data[p + 32], c2 = data[p + 64], c3 = data[p + 96];
        take(g0, c0); take(g1, c1); take(g2, c2); take(g3, c3);
      }
      for (; p < p1; p += 32) take(indices[p], data[p]);
    }
    s = warp_sum_ll(s);
    const double scal = renorm ? ((s == 0) ? 1.0 : double(s)) : n_counts[r];
    const float sc = float(scal);
    __syncwarp();
    float4* o4 = reinterpret_cast<float4*>(out + r * ld_out);
    for (int j4 = lane; j4 < pitch / 4; j4 += 32) {
      float4 c4 = row4[j4];
      float* cv = reinterpret_cast<float*>(&c4);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = 4 * j4 + u;
        float v;
        if (cv[u] == 0.f && sc != 0.f) {
          v = 0.f;
        } else {
          v = __fdiv_rn(sf * cv[u], sc);
          if (do_log) v = log1pf(v);
        }
        if (missing && j < n_cols && missing[j]) v = fill;
        cv[u] = j < n_cols ? v : 0.f;
      }
      if (4 * j4 + 3 < n_cols) {
        __stcs(o4 + j4, c4);
      } else {
        for (int u = 0; u < 4 && 4 * j4 + u < n_cols; ++u) out[r * ld_out + 4 * j4 + u] = cv[u];
      }
    }
    if (libsize_out && renorm && lane == 0) libsize_out[r] = (s == 0) ? 1 : s;
    __syncwarp();
  }
}

// Per-CTA column sums of x and x^2 over rows [blockIdx.x * rows, +rows), one
// thread per column slice, rows in order (reproducible run to run).
__global__ void __launch_bounds__(256)
colstats_kernel(const float* __restrict__ x, int64_t n_rows, int n_cols, int64_t ld, int rows,
                float* __restrict__ part_sum, float* __restrict__ part_sq) {
  const int64_t r0 = int64_t(blockIdx.x) * rows;
  const int64_t r1 = min(n_rows, r0 + rows);
  for (int j = threadIdx.x; j < n_cols; j += blockDim.x) {
    float a = 0.f, b = 0.f;
    for (int64_t r = r0; r < r1; ++r) {
      const float v = __ldcs(x + r * ld + j);
      a += v;
      b = fmaf(v, v, b);
    }
    part_sum[int64_t(blockIdx.x) * n_cols + j] = a;
    part_sq[int64_t(blockIdx.x) * n_cols + j] = b;
  }
}

// Stage 1 of the FP64 reduction: group g sums partial rows [g*per, (g+1)*per).
__global__ void partial_reduce1(const float* __restrict__ ps, const float* __restrict__ pq, int nparts,
                                int n_cols, int per, double* __restrict__ gs, double* __restrict__ gq) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int g = blockIdx.y;
  if (j >= n_cols) return;
  const int a = g * per, b = min(nparts, a + per);
  double s = 0.0, q = 0.0;
  for (int c = a; c < b; ++c) {
    s += double(ps[int64_t(c) * n_cols + j]);
    q += double(pq[int64_t(c) * n_cols + j]);
  }
  gs[int64_t(g) * n_cols + j] = s;
  gq[int64_t(g) * n_cols + j] = q;
}

// Stage 2: groups in order, accumulated into the caller's sums.
__global__ void partial_reduce2(const double* __restrict__ gs, const double* __restrict__ gq, int ngroups,
                                int n_cols, double* __restrict__ colsum, double* __restrict__ colsumsq) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cols) return;
  double s = 0.0, q = 0.0;
  for (int g = 0; g < ngroups; ++g) {
    s += gs[int64_t(g) * n_cols + j];
    q += gq[int64_t(g) * n_cols + j];
  }
  colsum[j] += s;
  colsumsq[j] += q;
}

__device__ __forceinline__ double clean_value(double v, double fill) {
  if (isnan(v) || isinf(v)) v = 0.0;
  if (v == 0.0) v = fill;
  return v;
}

__global__ void narrow_map_kernel(const int32_t* __restrict__ in, int64_t n, int n_cols, int16_t* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = int16_t((in[i] < 0 || in[i] >= n_cols) ? -1 : in[i]);
}

__global__ void zstats_kernel(const double* __restrict__ colsum, const double* __restrict__ colsumsq,
                              double n, int n_cols, double* __restrict__ mu, double* __restrict__ sigma,
                              float* __restrict__ mu32, float* __restrict__ sigma32) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cols) return;
  double m = colsum[j] / n;
  double var = colsumsq[j] / n - m * m;
  double sd = isnan(var) ? var : sqrt(var > 0.0 ? var : 0.0);
  m = clean_value(m, 0.0);
  sd = clean_value(sd, 1.0);
  if (mu) mu[j] = m;
  if (sigma) sigma[j] = sd;
  if (mu32) mu32[j] = float(m);
  if (sigma32) sigma32[j] = float(sd);
}

// A CSR array the kernels may read: device memory of this handle's device,
// managed memory, or page-locked host memory mapped at the same address
// (read over the host link). Pageable host memory is refused.
int check_readable(const sg_handle* h, const void* p, const char* what) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return sg::fail(SG_ERR_ARG, "sg_normalize_csr: %s is not a CUDA-visible pointer", what);
  }
  switch (a.type) {
    case cudaMemoryTypeDevice:
      if (a.device != h->device)
        return sg::fail(SG_ERR_ARG, "sg_normalize_csr: %s lives on device %d, the handle on %d", what, a.device,
                        h->device);
      return SG_OK;
    case cudaMemoryTypeManaged:
      return SG_OK;
    case cudaMemoryTypeHost:
      if (a.devicePointer != p)
        return sg::fail(SG_ERR_ARG, "sg_normalize_csr: page-locked %s is not mapped at its host address", what);
      return SG_OK;
    default:
      return sg::fail(SG_ERR_ARG, "sg_normalize_csr: %s is pageable host memory (pass device or page-locked memory)",
                      what);
  }
}

}  // namespace

extern "C" int sg_normalize_csr(sg_handle* h, const int64_t* indptr, const int32_t* indices,
                                const int32_t* data, int64_t n_rows, const int32_t* col_map,
                                int64_t n_genes, int32_t n_cols, const uint8_t* missing_mask,
                                float fill_value, const double* n_counts, double size_factor,
                                uint32_t flags, void* out, int64_t ld_out, int32_t out_dtype,
                                int64_t* libsize_out, double* colsum, double* colsumsq,
                                void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(n_rows >= 0 && n_cols > 0 && n_genes > 0, "sg_normalize_csr: bad sizes (n_rows=%lld n_cols=%d n_genes=%lld)",
         (long long)n_rows, n_cols, (long long)n_genes);
  SG_ARG(indptr && col_map && out, "sg_normalize_csr: null indptr/col_map/out");
  SG_ARG(out_dtype == SG_F32 || out_dtype == SG_BF16, "sg_normalize_csr: out_dtype must be SG_F32 or SG_BF16");
  SG_ARG(ld_out >= n_cols, "sg_normalize_csr: ld_out (%lld) < n_cols (%d)", (long long)ld_out, n_cols);
  SG_ARG((flags & SG_NORM_RENORM_SUBSET) || n_counts, "sg_normalize_csr: n_counts needed without SG_NORM_RENORM_SUBSET");
  SG_ARG((colsum == nullptr) == (colsumsq == nullptr), "sg_normalize_csr: colsum and colsumsq go together");
  if (out_dtype == SG_F32)
    SG_ARG(ld_out % 4 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0,
           "sg_normalize_csr: float32 output needs ld_out %% 4 == 0 and 16-byte alignment");
  else
    SG_ARG(ld_out % 2 == 0 && (reinterpret_cast<uintptr_t>(out) & 3) == 0,
           "sg_normalize_csr: bf16 output needs an even ld_out and 4-byte alignment");
  if (n_rows == 0) return SG_OK;
  SG_ARG(indices && data, "sg_normalize_csr: null indices/data");
  for (const auto& pa : {std::make_pair(static_cast<const void*>(indptr), "indptr"),
                         std::make_pair(static_cast<const void*>(indices), "indices"),
                         std::make_pair(static_cast<const void*>(data), "data")}) {
    const int rc = check_readable(h, pa.first, pa.second);
    if (rc) return rc;
  }

  const int pitch = (n_cols + 3) & ~3;
  const size_t row_bytes = size_t(pitch) * sizeof(float);
  const bool f32 = out_dtype == SG_F32;
  // FP32 output: barrier-free rows, then column statistics over the output
  // (kStatRows rows per CTA); BF16 output: the fused kernel, whose statistics
  // come from the unrounded values
  constexpr int kStatRows = 256;
  int nwarps = 8;
  while (nwarps > 1 && (size_t(nwarps) + (f32 ? 0 : 2)) * row_bytes > h->smem_optin) --nwarps;
  const size_t smem = (size_t(nwarps) + (f32 ? 0 : 2)) * row_bytes;
  if (smem > h->smem_optin)
    return sg::fail(SG_ERR_UNSUPPORTED, "sg_normalize_csr: %d output columns exceed the shared-memory row buffer", n_cols);
  const int64_t rows_per_cta = int64_t(nwarps) * kRounds;
  const int nblocks = f32 ? sg::ceil_div_i(n_rows, kStatRows) : sg::ceil_div_i(n_rows, rows_per_cta);

  const bool narrow = n_cols < 32768;
  float* ps = nullptr;
  float* pq = nullptr;
  double* gs = nullptr;
  double* gq = nullptr;
  int16_t* map16 = nullptr;
  int ngroups = 0, per = 0;
  {
    per = 32;
    ngroups = colsum ? sg::ceil_div_i(nblocks, per) : 0;
    const size_t need = (colsum ? 2 * sg::Carver::need(size_t(nblocks) * n_cols * sizeof(float)) +
                                      2 * sg::Carver::need(size_t(ngroups) * n_cols * sizeof(double))
                                : 0) +
                        (narrow ? sg::Carver::need(size_t(n_genes) * sizeof(int16_t)) : 0) + 256;
    int status;
    void* w = sg::ws_get(h, need, &status);
    if (!w) return status;
    sg::Carver cv(w);
    if (colsum) {
      ps = cv.take<float>(size_t(nblocks) * n_cols);
      pq = cv.take<float>(size_t(nblocks) * n_cols);
      gs = cv.take<double>(size_t(ngroups) * n_cols);
      gq = cv.take<double>(size_t(ngroups) * n_cols);
    }
    if (narrow) map16 = cv.take<int16_t>(size_t(n_genes));
  }
  if (narrow) {
    narrow_map_kernel<<<sg::ceil_div_i(n_genes, 256), 256, 0, st>>>(col_map, n_genes, n_cols, map16);
    SG_LAUNCH_CHECK();
  }
  // 16-byte loads need indices and counts equally aligned
  const int vec = ((reinterpret_cast<uintptr_t>(indices) ^ reinterpret_cast<uintptr_t>(data)) & 15) == 0 ? 1 : 0;
  const float sf = float(size_factor);
  sg::ProfScope prof(h, "normalize", st);
  auto launch_rows = [&](auto kern, const auto* map) -> int {
    SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nwarps * 32, smem));
    const int64_t grid = std::min<int64_t>(sg::ceil_div(n_rows, nwarps), int64_t(std::max(1, per_sm)) * h->sm_count);
    kern<<<unsigned(grid), nwarps * 32, smem, st>>>(indptr, indices, data, n_rows, map, n_genes, n_cols, vec, pitch,
                                                    missing_mask, fill_value, n_counts, sf, flags,
                                                    static_cast<float*>(out), ld_out, libsize_out);
    SG_LAUNCH_CHECK();
    return SG_OK;
  };
  auto launch = [&](auto kern, const auto* map) -> int {
    SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    kern<<<nblocks, nwarps * 32, smem, st>>>(indptr, indices, data, n_rows, map, n_genes, n_cols, vec, pitch,
                                             missing_mask, fill_value, n_counts, sf, flags, out, ld_out, libsize_out,
                                             ps, pq);
    SG_LAUNCH_CHECK();
    return SG_OK;
  };
  int rc;
  if (f32) {
    rc = narrow ? launch_rows(normalize_rows_kernel<int16_t>, map16) : launch_rows(normalize_rows_kernel<int32_t>, col_map);
    if (rc) return rc;
    if (colsum) {
      colstats_kernel<<<nblocks, 256, 0, st>>>(static_cast<const float*>(out), n_rows, n_cols, ld_out, kStatRows, ps,
                                               pq);
      SG_LAUNCH_CHECK();
    }
  } else {
    rc = narrow ? launch(normalize_kernel<true, int16_t>, map16) : launch(normalize_kernel<true, int32_t>, col_map);
  }
  if (rc) return rc;
  if (colsum) {
    dim3 g1(sg::ceil_div_i(n_cols, 256), ngroups);
    partial_reduce1<<<g1, 256, 0, st>>>(ps, pq, nblocks, n_cols, per, gs, gq);
    SG_LAUNCH_CHECK();
    partial_reduce2<<<sg::ceil_div_i(n_cols, 256), 256, 0, st>>>(gs, gq, ngroups, n_cols, colsum, colsumsq);
    SG_LAUNCH_CHECK();
  }
  return SG_OK;
}

extern "C" int sg_zstats(sg_handle* h, const double* colsum, const double* colsumsq, int64_t n_rows,
                         int32_t n_cols, double* mu, double* sigma, float* mu32, float* sigma32,
                         void* stream) {
  SG_HANDLE_CHECK(h);
  SG_ARG(colsum && colsumsq && n_cols > 0 && n_rows > 0, "sg_zstats: bad arguments");
  zstats_kernel<<<sg::ceil_div_i(n_cols, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      colsum, colsumsq, double(n_rows), n_cols, mu, sigma, mu32, sigma32);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
