// a4 + a5: scatter (covariance) of the z-scaled rows, FP64 eigendecomposition
// of it on the device (cuSOLVER syevdx, top n_comp pairs), the svd_flip sign
// convention, and the reducer projection ((x - mu)/sigma) . L.
//
// Plain covariance: FP32 SIMT, 128x128 output tiles of the upper triangle,
// 8x8 register micro-tiles, rows split into K-chunks whose float32 partials are
// reduced in FP64 in a fixed order. The z-transform (and the PCA row mask) is
// applied while staging each 16-row slab into shared memory.
#include "common.cuh"
#include "symeig.h"

#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

// SG_EIG_DEBUG (off unless defined at compile time) traces the filtered
// eigensolver's schedule to stderr.
#ifdef SG_EIG_DEBUG
#define EIG_DBG(...) std::fprintf(stderr, __VA_ARGS__)
#else
#define EIG_DBG(...) ((void)0)
#endif
#include <vector>

bool sg_project_tc_supported(const float* x, int64_t ld, int d);  // proj_tc.cu
int sg_project_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld, const float* mu32,
                  const float* sigma32, const float* loadings32, int32_t d, int32_t ld_l, float* scores, int32_t ld_s,
                  __nv_bfloat16* sb, int32_t ld_b, cudaStream_t st);  // proj_tc.cu
int sg_covariance_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld,
                     const float* mu32, const float* sigma32, const uint8_t* row_mask, double* cov,
                     double* zsum, cudaStream_t st);  // cov_tc.cu

namespace {

constexpr int CT = 128;  // covariance output tile
constexpr int CBK = 16;  // rows per shared-memory slab

__device__ __forceinline__ float zval(float x, float m, float s) { return __fdiv_rn(x - m, s); }

// t-th tile (row-major) of the upper triangle of a T x T tile grid
__device__ __forceinline__ int2 upper_tile(int t, int T) {
  for (int i = 0; i < T; ++i) {
    const int cnt = T - i;
    if (t < cnt) return make_int2(i, i + t);
    t -= cnt;
  }
  return make_int2(T - 1, T - 1);
}

// grid: (n_upper_tiles, n_splits). Tile t enumerates (ti, tj) with tj >= ti.
__global__ void __launch_bounds__(256, 2)
cov_simt_kernel(const float* __restrict__ x, int64_t n_rows, int n_cols, int64_t ld,
                const float* __restrict__ mu, const float* __restrict__ sg, const uint8_t* __restrict__ mask,
                int T, int64_t rows_per_split, float* __restrict__ part,
                int n_pad, float* __restrict__ zpart) {
  __shared__ __align__(16) float As[2][CBK][CT];
  __shared__ __align__(16) float Bs[2][CBK][CT];
  const int tid = threadIdx.x;
  const int2 t = upper_tile(blockIdx.x, T);
  const int i0 = t.x * CT, j0 = t.y * CT;
  const bool diag = t.x == t.y;
  const int64_t r_begin = int64_t(blockIdx.y) * rows_per_split;
  const int64_t r_end = min(n_rows, r_begin + rows_per_split);
  const int tx = tid & 15, ty = tid >> 4;
  // loader mapping: slab row lk = tid / 16, 8 columns from (tid % 16) * 8
  const int lk = tid >> 4, lc = (tid & 15) * 8;

  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
  float zs[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) zs[a] = 0.f;

  float ra[8], rb[8];
  auto load = [&](int64_t r0) {
    const int64_t r = r0 + lk;
    const bool ok = r < r_end && (mask == nullptr || mask[r] != 0);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int ca = i0 + lc + q, cb = j0 + lc + q;
      ra[q] = (ok && ca < n_cols) ? zval(x[r * ld + ca], mu[ca], sg[ca]) : 0.f;
      rb[q] = (ok && cb < n_cols) ? zval(x[r * ld + cb], mu[cb], sg[cb]) : 0.f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      As[buf][lk][lc + q] = ra[q];
      Bs[buf][lk][lc + q] = rb[q];
    }
    if (diag) {
#pragma unroll
      for (int q = 0; q < 8; ++q) zs[q] += ra[q];
    }
  };

  int buf = 0;
  if (r_begin < r_end) {
    load(r_begin);
    store(0);
  }
  __syncthreads();
  for (int64_t r0 = r_begin; r0 < r_end; r0 += CBK) {
    const bool more = r0 + CBK < r_end;
    if (more) load(r0 + CBK);
#pragma unroll
    for (int kk = 0; kk < CBK; ++kk) {
      float a[8], b[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
      a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
      a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
      b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
      b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
      for (int p = 0; p < 8; ++p)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  // write the float32 partial tile
  float* P = part + int64_t(blockIdx.y) * n_pad * n_pad;
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const int gi = i0 + (p < 4 ? ty * 4 + p : 64 + ty * 4 + p - 4);
    float4 lo = make_float4(acc[p][0], acc[p][1], acc[p][2], acc[p][3]);
    float4 hi = make_float4(acc[p][4], acc[p][5], acc[p][6], acc[p][7]);
    *reinterpret_cast<float4*>(&P[int64_t(gi) * n_pad + j0 + tx * 4]) = lo;
    *reinterpret_cast<float4*>(&P[int64_t(gi) * n_pad + j0 + 64 + tx * 4]) = hi;
  }
  if (diag) {
    // column sums of z over this split: 16 loader rows share each column
    __syncthreads();
    float* red = &As[0][0][0];  // 16 x 128 floats
#pragma unroll
    for (int q = 0; q < 8; ++q) red[lk * CT + lc + q] = zs[q];
    __syncthreads();
    if (tid < CT) {
      float s = 0.f;
      for (int r = 0; r < CBK; ++r) s += red[r * CT + tid];
      zpart[int64_t(blockIdx.y) * n_pad + i0 + tid] = s;
    }
  }
}

// FP64 sum over splits (fixed order) of the upper-triangle tiles; the result
// is added to cov[i][j] and mirrored to cov[j][i].
__global__ void cov_reduce_kernel(const float* __restrict__ part, int nsplit, int n_pad, int n_cols, int T,
                                  double* __restrict__ cov) {
  const int2 t = upper_tile(blockIdx.x, T);
  for (int e = threadIdx.x; e < CT * CT; e += blockDim.x) {
    const int i = t.x * CT + e / CT, j = t.y * CT + e % CT;
    if (i >= n_cols || j >= n_cols || j < i) continue;
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += double(part[int64_t(p) * n_pad * n_pad + int64_t(i) * n_pad + j]);
    cov[int64_t(i) * n_cols + j] += s;
    if (i != j) cov[int64_t(j) * n_cols + i] += s;
  }
}

__global__ void zsum_reduce_kernel(const float* __restrict__ zpart, int nsplit, int n_pad, int n_cols,
                                   double* __restrict__ zsum) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cols) return;
  double s = 0.0;
  for (int p = 0; p < nsplit; ++p) s += double(zpart[int64_t(p) * n_pad + j]);
  zsum[j] += s;
}

// centred scatter A = cov - zsum zsum^T / n, and its trace
__global__ void center_kernel(const double* __restrict__ cov, const double* __restrict__ zsum, double inv_n,
                              int n, double* __restrict__ A) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * n) return;
  const int i = int(e / n), j = int(e % n);
  const double c = zsum ? zsum[i] * zsum[j] * inv_n : 0.0;
  A[e] = cov[e] - c;
}

__global__ void trace_kernel(const double* __restrict__ A, int n, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += A[int64_t(i) * n + i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// One CTA per output component c (descending eigenvalue order).
__global__ void basis_kernel(const double* __restrict__ V, const double* __restrict__ W, int n, int m,
                             const double* __restrict__ trace, double* __restrict__ comps,
                             double* __restrict__ evals, double* __restrict__ evr, int n_load,
                             float* __restrict__ L32, int ld_l) {
  __shared__ double bv[256];
  __shared__ int bi[256];
  const int c = blockIdx.x;
  const int src = m - 1 - c;  // syevdx returns ascending order
  const double* v = V + int64_t(src) * n;  // column-major eigenvectors
  double best = -1.0;
  int besti = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = fabs(v[i]);
    if (a > best) { best = a; besti = i; }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = besti;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double a = bv[threadIdx.x + o];
      const int ai = bi[threadIdx.x + o];
      if (a > bv[threadIdx.x] || (a == bv[threadIdx.x] && ai < bi[threadIdx.x])) {
        bv[threadIdx.x] = a;
        bi[threadIdx.x] = ai;
      }
    }
    __syncthreads();
  }
  const double sgn = v[bi[0]] < 0.0 ? -1.0 : 1.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double val = sgn * v[i];
    comps[int64_t(i) * m + c] = val;
    if (L32 && c < n_load) L32[int64_t(i) * ld_l + c] = float(val);
  }
  if (L32 && c < n_load) {
    for (int i = threadIdx.x; i < n && c == 0; i += blockDim.x)
      for (int cc = n_load; cc < ld_l; ++cc) L32[int64_t(i) * ld_l + cc] = 0.f;
  }
  if (threadIdx.x == 0) {
    if (evals) evals[c] = W[src];
    if (evr) evr[c] = W[src] / *trace;
  }
}

// ||y - w v|| / |w_max| for one Ritz pair per CTA (y = A v)
__global__ void ritz_residual_kernel(const double* __restrict__ Y, const double* __restrict__ V,
                                     const double* __restrict__ W, const double* __restrict__ wmax, int n,
                                     double* __restrict__ out) {
  __shared__ double red[256];
  const int c = blockIdx.x;
  const double w = W[c];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = Y[int64_t(c) * n + i] - w * V[int64_t(c) * n + i];
    s += r * r;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = sqrt(red[0]) / fabs(*wmax);
}

__global__ void f64_to_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t ne) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < ne) b[e] = float(a[e]);
}

__global__ void f32_to_f64_kernel(const float* __restrict__ a, double* __restrict__ b, int64_t ne) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < ne) b[e] = double(a[e]);
}

// ---- projection -----------------------------------------------------------
constexpr int PR = 128;  // rows per CTA
constexpr int PC = 64;   // output columns per CTA
constexpr int PK = 32;   // features per slab

__global__ void __launch_bounds__(256)
project_kernel(const float* __restrict__ x, int64_t n_rows, int n_cols, int64_t ld, const float* __restrict__ mu,
               const float* __restrict__ sg, const float* __restrict__ L, int d, int ld_l,
               float* __restrict__ scores, int ld_s, __nv_bfloat16* __restrict__ sb, int ld_b) {
  __shared__ __align__(16) float As[PK][PR + 4];
  __shared__ __align__(16) float Bs[PK][PC];
  const int tid = threadIdx.x;
  const int64_t r0 = int64_t(blockIdx.x) * PR;
  const int c0 = blockIdx.y * PC;
  const int tx = tid & 15, ty = tid >> 4;
  float acc[8][4];
#pragma unroll
  for (int p = 0; p < 8; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = 0.f;
  const int lr = tid >> 1, lj = (tid & 1) * 16;
  for (int j0 = 0; j0 < n_cols; j0 += PK) {
    const int64_t r = r0 + lr;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = j0 + lj + q;
      As[lj + q][lr] = (r < n_rows && j < n_cols) ? zval(x[r * ld + j], mu[j], sg[j]) : 0.f;
    }
    for (int e = tid; e < PK * PC; e += 256) {
      const int jj = e / PC, cc = e % PC;
      const int j = j0 + jj, c = c0 + cc;
      Bs[jj][cc] = (j < n_cols && c < d) ? L[int64_t(j) * ld_l + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < PK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[4] = {b0.x, b0.y, b0.z, b0.w};
#pragma unroll
      for (int p = 0; p < 8; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const int64_t r = r0 + (p < 4 ? ty * 4 + p : 64 + ty * 4 + p - 4);
    if (r >= n_rows) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + tx * 4 + q;
      const float v = c < d ? acc[p][q] : 0.f;
      if (c < ld_s) scores[r * ld_s + c] = v;
      if (sb && c < ld_b) sb[r * ld_b + c] = __float2bfloat16_rn(v);
    }
  }
}


__global__ void pad_cols_kernel(float* __restrict__ s, int64_t n_rows, int from, int ld,
                                __nv_bfloat16* __restrict__ sb, int from_b, int ld_b) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  for (int c = from; c < ld; ++c) s[r * ld + c] = 0.f;
  if (sb)
    for (int c = from_b; c < ld_b; ++c) sb[r * ld_b + c] = __float2bfloat16_rn(0.f);
}


}  // namespace


void sg_solver_destroy(sg_handle* h) {
  if (h->blas) cublasDestroy(static_cast<cublasHandle_t>(h->blas));
  h->blas = nullptr;
  if (h->solver) cusolverDnDestroy(static_cast<cusolverDnHandle_t>(h->solver));
  if (h->solver_work) cudaFree(h->solver_work);
  h->solver = nullptr;
  h->solver_work = nullptr;
}

extern "C" int sg_covariance(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld,
                             const float* mu32, const float* sigma32, const uint8_t* row_mask,
                             int32_t precision, double* cov, double* zsum, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(x && mu32 && sigma32 && cov && zsum, "sg_covariance: null pointer argument");
  SG_ARG(n_rows >= 0 && n_cols > 0 && ld >= n_cols, "sg_covariance: bad sizes");
  SG_ARG(precision == SG_PLAIN || precision == SG_PRECISION, "sg_covariance: unknown precision %d", precision);
  if (n_rows == 0) return SG_OK;
  if (precision == SG_PRECISION) return sg_covariance_tc(h, x, n_rows, n_cols, ld, mu32, sigma32, row_mask, cov, zsum, st);

  const int T = sg::ceil_div_i(n_cols, CT);
  const int n_pad = T * CT;
  const int ntile = T * (T + 1) / 2;
  int64_t rows_per_split = 8192;
  const int64_t want_ctas = int64_t(h->sm_count) * 4;
  while (rows_per_split > 512 && ntile * sg::ceil_div(n_rows, rows_per_split) < want_ctas) rows_per_split /= 2;
  rows_per_split = ((rows_per_split + CBK - 1) / CBK) * CBK;
  const int nsplit = int(sg::ceil_div(n_rows, rows_per_split));

  const size_t part_bytes = size_t(nsplit) * n_pad * n_pad * sizeof(float);
  const size_t need = sg::Carver::need(part_bytes) + sg::Carver::need(size_t(nsplit) * n_pad * sizeof(float));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  float* part = cv.take<float>(size_t(nsplit) * n_pad * n_pad);
  float* zpart = cv.take<float>(size_t(nsplit) * n_pad);
  dim3 grid(ntile, nsplit);
  sg::ProfScope prof(h, "cov_simt", st);
  cov_simt_kernel<<<grid, 256, 0, st>>>(x, n_rows, n_cols, ld, mu32, sigma32, row_mask, T, rows_per_split, part,
                                        n_pad, zpart);
  SG_LAUNCH_CHECK();
  cov_reduce_kernel<<<ntile, 256, 0, st>>>(part, nsplit, n_pad, n_cols, T, cov);
  SG_LAUNCH_CHECK();
  zsum_reduce_kernel<<<sg::ceil_div_i(n_cols, 256), 256, 0, st>>>(zpart, nsplit, n_pad, n_cols, zsum);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_pca_basis(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                            int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                            int32_t n_load, float* loadings32, int32_t ld_l, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(cov && comps && n_cols > 0 && n_used > 0, "sg_pca_basis: bad arguments");
  SG_ARG(n_comp >= 1 && n_comp <= n_cols, "sg_pca_basis: n_comp=%d outside [1, %d]", n_comp, n_cols);
  SG_ARG(!loadings32 || (n_load >= 0 && n_load <= n_comp && ld_l >= n_load), "sg_pca_basis: bad loadings shape");
  const int n = n_cols;
  if (!h->solver) {
    cusolverDnHandle_t s;
    if (cusolverDnCreate(&s) != CUSOLVER_STATUS_SUCCESS) return sg::fail(SG_ERR_CUDA, "cusolverDnCreate failed");
    h->solver = s;
  }
  cusolverDnHandle_t sol = static_cast<cusolverDnHandle_t>(h->solver);
  if (cusolverDnSetStream(sol, st) != CUSOLVER_STATUS_SUCCESS) return sg::fail(SG_ERR_CUDA, "cusolverDnSetStream failed");

  const size_t abytes = sizeof(double) * size_t(n) * n;
  int status;
  void* w = sg::ws_get(h, sg::Carver::need(abytes) + sg::Carver::need(sizeof(double) * n) + 1024, &status);
  if (!w) return status;
  sg::Carver cv(w);
  double* A = cv.take<double>(size_t(n) * n);
  double* W = cv.take<double>(n);
  double* tr = cv.take<double>(1);
  int* info = cv.take<int>(1);
  const int64_t ne = int64_t(n) * n;
  center_kernel<<<sg::ceil_div_i(ne, 256), 256, 0, st>>>(cov, zsum, 1.0 / double(n_used), n, A);
  SG_LAUNCH_CHECK();
  trace_kernel<<<1, 256, 0, st>>>(A, n, tr);
  SG_LAUNCH_CHECK();
  const int il = n - n_comp + 1, iu = n;
  int meig = 0, lwork = 0;
  if (cusolverDnDsyevdx_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER, n, A, n,
                                   0.0, 0.0, il, iu, &meig, W, &lwork) != CUSOLVER_STATUS_SUCCESS)
    return sg::fail(SG_ERR_CUDA, "cusolverDnDsyevdx_bufferSize failed");
  const size_t wbytes = sizeof(double) * size_t(lwork);
  if (h->solver_work_bytes < wbytes) {
    if (h->solver_work) cudaFree(h->solver_work);
    h->solver_work = nullptr;
    h->solver_work_bytes = 0;
    if (h->budget && wbytes + h->ws_bytes > h->budget)
      return sg::fail(SG_ERR_BUDGET, "eigensolver workspace of %zu bytes exceeds the HBM budget", wbytes);
    SG_CUDA(cudaMalloc(&h->solver_work, wbytes));
    h->solver_work_bytes = wbytes;
  }
  sg::ProfScope prof(h, "eigh", st);
  cusolverStatus_t cs = cusolverDnDsyevdx(sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER, n,
                                          A, n, 0.0, 0.0, il, iu, &meig, W, static_cast<double*>(h->solver_work), lwork,
                                          info);
  if (cs != CUSOLVER_STATUS_SUCCESS) return sg::fail(SG_ERR_CUDA, "cusolverDnDsyevdx failed (status %d)", int(cs));
  int hinfo = 0;
  SG_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (hinfo != 0) return sg::fail(SG_ERR_CUDA, "cusolverDnDsyevdx: info=%d", hinfo);
  if (meig != n_comp) return sg::fail(SG_ERR_CUDA, "cusolverDnDsyevdx returned %d of %d eigenpairs", meig, n_comp);
  basis_kernel<<<n_comp, 256, 0, st>>>(A, W, n, n_comp, tr, comps, evals, evr, n_load, loadings32, ld_l);
  SG_LAUNCH_CHECK();
  SG_CUDA(cudaStreamSynchronize(st));
  return SG_OK;
}

namespace {

int solver_work(sg_handle* h, size_t wbytes) {
  if (h->solver_work_bytes >= wbytes) return SG_OK;
  if (h->solver_work) cudaFree(h->solver_work);
  h->solver_work = nullptr;
  h->solver_work_bytes = 0;
  if (h->budget && wbytes + h->ws_bytes > h->budget)
    return sg::fail(SG_ERR_BUDGET, "eigensolver workspace of %zu bytes exceeds the HBM budget", wbytes);
  SG_CUDA(cudaMalloc(&h->solver_work, wbytes));
  h->solver_work_bytes = wbytes;
  return SG_OK;
}

#define SG_BLAS(call)                                                                              \
  do {                                                                                             \
    cublasStatus_t s_ = (call);                                                                    \
    if (s_ != CUBLAS_STATUS_SUCCESS) return sg::fail(SG_ERR_CUDA, "%s failed (status %d)", #call, int(s_)); \
  } while (0)
#define SG_SOLVER(call)                                                                            \
  do {                                                                                             \
    cusolverStatus_t s_ = (call);                                                                  \
    if (s_ != CUSOLVER_STATUS_SUCCESS) return sg::fail(SG_ERR_CUDA, "%s failed (status %d)", #call, int(s_)); \
  } while (0)

}  // namespace

// Mixed-precision principal axes: an FP32 partial eigendecomposition of the
// centred scatter (top n_comp + 16 pairs), then an FP64 Rayleigh-Ritz step on
// that subspace (FP64 Cholesky-QR orthonormalisation, FP64 Q^T A Q and its
// FP64 eigendecomposition), so eigenvalues and vectors are FP64 Ritz pairs.
namespace {

// FP64 Rayleigh-Ritz on the subspace spanned by the m columns of Q (n x m,
// FP64, overwritten): FP64 Cholesky-QR orthonormalisation, B = Q^T A Q and
// its FP64 eigendecomposition; V = Q U holds the Ritz vectors and W the Ritz
// values, both in ascending order. When `resid` is given, it receives
// max_c ||A v_c - w_c v_c|| / max|w| over the top n_top Ritz pairs (host value;
// this synchronises the stream).
int rayleigh_ritz_fp64(sg_handle* h, cusolverDnHandle_t sol, cublasHandle_t blas, const double* A, int n, int m,
                       double* Q, double* Y, double* V, double* G, double* B, double* W, int* info, int lwork_d,
                       int n_top, double* resid, double* rcol, cudaStream_t st) {
  const double one = 1.0, zero = 0.0;
  sg::ProfScope prof(h, "eig_rr64", st);
  // Q <- Q R^-1 with Q^T Q = L L^T (R = L^T): FP64 Cholesky-QR
  SG_BLAS(cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, Q, n, Q, n, &zero, G, m));
  SG_SOLVER(cusolverDnDpotrf(sol, CUBLAS_FILL_MODE_LOWER, m, G, m, static_cast<double*>(h->solver_work),
                             int(h->solver_work_bytes / sizeof(double)), info));
  SG_BLAS(cublasDtrsm(blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, m, &one, G,
                      m, Q, n));
  // Rayleigh quotient B = Q^T A Q and its FP64 eigendecomposition, on the
  // host: at these sizes a device solver is bound by launch latency
  SG_BLAS(cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, n, &one, A, n, Q, n, &zero, Y, n));
  SG_BLAS(cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, Q, n, Y, n, &zero, B, m));
  {
    const size_t mm = static_cast<size_t>(m) * static_cast<size_t>(m);
    std::vector<double> hb(mm), hu(mm), hw(static_cast<size_t>(m));
    SG_CUDA(cudaMemcpyAsync(hb.data(), B, sizeof(double) * mm, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    if (sg::symeig_host(m, hb.data(), hw.data(), hu.data()) != 0)
      return sg::fail(SG_ERR_CUDA, "Rayleigh-Ritz: the host QL iteration did not converge (m=%d)", m);
    SG_CUDA(cudaMemcpyAsync(B, hu.data(), sizeof(double) * mm, cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaMemcpyAsync(W, hw.data(), sizeof(double) * size_t(m), cudaMemcpyHostToDevice, st));
    SG_CUDA(cudaStreamSynchronize(st));  // the host buffers go out of scope
  }
  (void)lwork_d;
  SG_BLAS(cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, m, &one, Q, n, B, m, &zero, V, n));
  if (resid) {
    // A V = (A Q) U; the residual of Ritz pair c is (A Q) u_c - w_c v_c
    SG_BLAS(cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, m, &one, Y, n, B, m, &zero, Q, n));
    ritz_residual_kernel<<<n_top, 256, 0, st>>>(Q + size_t(m - n_top) * n, V + size_t(m - n_top) * n, W + (m - n_top),
                                                W + (m - 1), n, rcol);
    SG_LAUNCH_CHECK();
    std::vector<double> hr(static_cast<size_t>(n_top));
    SG_CUDA(cudaMemcpyAsync(hr.data(), rcol, sizeof(double) * size_t(n_top), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    double mx = 0.0;
    for (double v : hr) mx = std::isfinite(v) ? std::max(mx, v) : INFINITY;
    *resid = mx;
  }
  return SG_OK;
}

int check_info(const int* info, int count, cudaStream_t st, const char* what) {
  std::vector<int> hi(static_cast<size_t>(count));
  SG_CUDA(cudaMemcpyAsync(hi.data(), info, sizeof(int) * size_t(count), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < count; ++i)
    if (hi[size_t(i)] != 0) return sg::fail(SG_ERR_CUDA, "%s: factorisation %d info=%d", what, i, hi[size_t(i)]);
  return SG_OK;
}

int solver_handles(sg_handle* h, cudaStream_t st, cusolverDnHandle_t* sol, cublasHandle_t* blas) {
  if (!h->solver) {
    cusolverDnHandle_t s;
    SG_SOLVER(cusolverDnCreate(&s));
    h->solver = s;
  }
  if (!h->blas) {
    cublasHandle_t b;
    SG_BLAS(cublasCreate(&b));
    // the BF16x9 emulated GEMMs here only see finite operands (a non-finite
    // block fails the Ritz and residual checks downstream), so the library's
    // scan-and-patch passes for infinities and NaNs are switched off
    SG_BLAS(cublasSetEmulationSpecialValuesSupport(b, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE));
    h->blas = b;
  }
  *sol = static_cast<cusolverDnHandle_t>(h->solver);
  *blas = static_cast<cublasHandle_t>(h->blas);
  SG_SOLVER(cusolverDnSetStream(*sol, st));
  SG_BLAS(cublasSetStream(*blas, st));
  return SG_OK;
}

}  // namespace

// Mixed-precision principal axes: an FP32 partial eigendecomposition of the
// centred scatter (top n_comp + 16 pairs), then an FP64 Rayleigh-Ritz step on
// that subspace (FP64 Cholesky-QR orthonormalisation, FP64 Q^T A Q and its
// FP64 eigendecomposition), so eigenvalues and vectors are FP64 Ritz pairs.
extern "C" int sg_pca_basis_mixed(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                                  int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                                  int32_t n_load, float* loadings32, int32_t ld_l, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(cov && comps && n_cols > 0 && n_used > 0, "sg_pca_basis_mixed: bad arguments");
  SG_ARG(n_comp >= 1 && n_comp <= n_cols, "sg_pca_basis_mixed: n_comp=%d outside [1, %d]", n_comp, n_cols);
  SG_ARG(!loadings32 || (n_load >= 0 && n_load <= n_comp && ld_l >= n_load),
         "sg_pca_basis_mixed: bad loadings shape");
  const int n = n_cols;
  const int m = std::min(n, n_comp + 16);
  cusolverDnHandle_t sol;
  cublasHandle_t blas;
  int rc = solver_handles(h, st, &sol, &blas);
  if (rc) return rc;
  const size_t nn = size_t(n) * n, nm = size_t(n) * m, mm = size_t(m) * m;
  const size_t need = sg::Carver::need(nn * 8) + sg::Carver::need(nn * 4) + 3 * sg::Carver::need(nm * 8) +
                      2 * sg::Carver::need(mm * 8) + 2 * sg::Carver::need(size_t(n) * 8) + 1024;
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  double* A = cv.take<double>(nn);
  float* A32 = cv.take<float>(nn);
  double* Q = cv.take<double>(nm);
  double* Y = cv.take<double>(nm);
  double* V = cv.take<double>(nm);
  double* G = cv.take<double>(mm);
  double* B = cv.take<double>(mm);
  float* W32 = cv.take<float>(n);
  double* W = cv.take<double>(n);
  double* tr = cv.take<double>(1);
  int* info = cv.take<int>(4);
  SG_CUDA(cudaMemsetAsync(info, 0, 4 * sizeof(int), st));
  const int64_t ne = int64_t(nn);
  center_kernel<<<sg::ceil_div_i(ne, 256), 256, 0, st>>>(cov, zsum, 1.0 / double(n_used), n, A);
  SG_LAUNCH_CHECK();
  trace_kernel<<<1, 256, 0, st>>>(A, n, tr);
  SG_LAUNCH_CHECK();
  f64_to_f32_kernel<<<sg::ceil_div_i(ne, 256), 256, 0, st>>>(A, A32, ne);
  SG_LAUNCH_CHECK();
  sg::ProfScope prof(h, "eigh", st);
  const int il = n - m + 1, iu = n;
  int meig = 0, lwork = 0;
  SG_SOLVER(cusolverDnSsyevdx_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER,
                                         n, A32, n, 0.f, 0.f, il, iu, &meig, W32, &lwork));
  int lwork_d = 0;
  SG_SOLVER(cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, B, m, W, &lwork_d));
  const size_t wb = std::max(sizeof(float) * size_t(lwork), sizeof(double) * size_t(lwork_d));
  rc = solver_work(h, wb);
  if (rc) return rc;
  SG_SOLVER(cusolverDnSsyevdx(sol, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER, n, A32, n,
                              0.f, 0.f, il, iu, &meig, W32, static_cast<float*>(h->solver_work), lwork, info + 2));
  if (meig != m) return sg::fail(SG_ERR_CUDA, "cusolverDnSsyevdx returned %d of %d eigenpairs", meig, m);
  f32_to_f64_kernel<<<sg::ceil_div_i(int64_t(nm), 256), 256, 0, st>>>(A32, Q, int64_t(nm));
  SG_LAUNCH_CHECK();
  rc = rayleigh_ritz_fp64(h, sol, blas, A, n, m, Q, Y, V, G, B, W, info, lwork_d, n_comp, nullptr, nullptr, st);
  if (rc) return rc;
  rc = check_info(info, 3, st, "sg_pca_basis_mixed");
  if (rc) return rc;
  // the n_comp largest Ritz pairs are the last n_comp columns (ascending order)
  basis_kernel<<<n_comp, 256, 0, st>>>(V + size_t(m - n_comp) * n, W + (m - n_comp), n, n_comp, tr, comps, evals,
                                       evr, n_load, loadings32, ld_l);
  SG_LAUNCH_CHECK();
  SG_CUDA(cudaStreamSynchronize(st));
  return SG_OK;
}

namespace {

// uniform(-1, 1) block from a counter hash (the SplitMix64 finaliser)
__global__ void random_block_kernel(float* __restrict__ X, int64_t ne, uint64_t seed) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  uint64_t z = uint64_t(e) * 0x9E3779B97F4A7C15ull + seed;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  X[e] = float(int32_t(uint32_t(z >> 32))) * (1.0f / 2147483648.0f);
}

// largest absolute row sum (an upper bound of the spectral radius)
__global__ void absrow_max_kernel(const float* __restrict__ A, int n, float* __restrict__ out) {
  __shared__ float red[256];
  float mx = 0.f;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    float s = 0.f;
    for (int j = threadIdx.x; j < n; j += blockDim.x) s += fabsf(A[int64_t(i) * n + j]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    mx = fmaxf(mx, red[0]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(reinterpret_cast<int*>(out), __float_as_int(mx));  // non-negative floats
}

// Column scaling for Cholesky-QR: with d = diag(Y^T Y), G <- D G D and
// Y <- Y D for D = diag(d)^(-1/2), so the Gram matrix has a unit diagonal (a
// non-positive d_j leaves column j unscaled; the factorisation then fails).
__global__ void gram_scale_kernel(float* __restrict__ G, const float* __restrict__ diag, int m) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(m) * m) return;
  const int i = int(e % m), j = int(e / m);
  const float di = diag[i], dj = diag[j];
  G[e] *= (di > 0.f ? rsqrtf(di) : 1.f) * (dj > 0.f ? rsqrtf(dj) : 1.f);
}

__global__ void diag_copy_kernel(const float* __restrict__ G, float* __restrict__ diag, int m) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) diag[j] = G[int64_t(j) * m + j];
}

__global__ void col_rscale_kernel(float* __restrict__ Y, const float* __restrict__ diag, int n, int m) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(n) * m) return;
  const float g = diag[e / n];
  Y[e] *= g > 0.f ? rsqrtf(g) : 1.f;
}

// Rayleigh quotients of the block's last K columns from the first filter
// product C = a1 A X - X: x^T A x = (x^T c + x^T x) / a1
__global__ void tail_rq_kernel(const float* __restrict__ X, const float* __restrict__ C, int n, int m, int K, float a1,
                               float* __restrict__ out) {
  __shared__ float red[2][256];
  const int j = m - K + blockIdx.x;
  float s = 0.f, q = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float x = X[int64_t(j) * n + i];
    s = fmaf(x, C[int64_t(j) * n + i], s);
    q = fmaf(x, x, q);
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = q;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = (red[0][0] + red[1][0]) / (a1 * red[1][0]);
}

// v <- v / |v| and *rq = v^T y / v^T v (y = A v), one CTA
__global__ void normalize_rq_kernel(float* __restrict__ v, const float* __restrict__ y, int n, float* __restrict__ rq) {
  __shared__ float red[2][1024];
  float a = 0.f, q = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a = fmaf(v[i], v[i], a);
    q = fmaf(v[i], y[i], q);
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = q;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  const float nn = red[0][0];
  if (threadIdx.x == 0) *rq = red[1][0] / nn;
  const float inv = nn > 0.f ? rsqrtf(nn) : 1.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] *= inv;
}

// reverse the column order of an m x m column-major matrix
__global__ void reverse_cols_kernel(float* __restrict__ G, int m) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int half = m / 2;
  if (e >= int64_t(half) * m) return;
  const int j = int(e / m), i = int(e % m);
  const int64_t a = int64_t(j) * m + i, b = int64_t(m - 1 - j) * m + i;
  const float t = G[a];
  G[a] = G[b];
  G[b] = t;
}

struct FilterBufs {
  float* X;   // n x m, orthonormal block
  float* P;   // n x m scratch
  float* Q;   // n x m scratch
  float* G;   // m x m
  float* W;   // m Ritz values
  float* D;   // m diagonal of the Gram matrix
  float* R;   // Rayleigh quotients of the last columns
  int* info;  // one slot per factorisation
  int n_info;
  int cap_info;
  syevjInfo_t jac = nullptr;  // Jacobi settings for blocks of up to kJacobiMax columns
};

// Blocks up to this width take cuSOLVER's Jacobi eigensolver in the FP32
// Rayleigh-Ritz step (1.56 against 1.98 ms at 128 on a GB300; at 192 the
// divide-and-conquer solver is faster, 1.55 against 2.7 ms).
constexpr int kJacobiMax = 128;

struct JacobiGuard {
  syevjInfo_t p = nullptr;
  ~JacobiGuard() {
    if (p) cusolverDnDestroySyevjInfo(p);
  }
};

// Y <- Y D L^-T with (Y D)^T (Y D) = L L^T and D the column scaling, in place
// (FP32 Cholesky-QR on unit-norm columns), `passes` times. The first columns
// keep their span: the block stays ordered with its dominant directions
// first. One pass leaves the columns orthogonal to ~u cond(Y)^2, enough
// between filter segments; two passes make them orthonormal to FP32.
int cholqr_f32(sg_handle* h, cusolverDnHandle_t sol, cublasHandle_t blas, float* Y, int n, int m, FilterBufs& b,
               int passes, cudaStream_t st) {
  const float one = 1.f, zero = 0.f;
  sg::ProfScope prof(h, "eig_qr", st);
  for (int pass = 0; pass < passes; ++pass) {
    SG_BLAS(cublasSgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, Y, n, Y, n, &zero, b.G, m));
    int* inf = b.info + std::min(b.n_info, b.cap_info - 3);
    ++b.n_info;
    diag_copy_kernel<<<sg::ceil_div_i(m, 256), 256, 0, st>>>(b.G, b.D, m);
    SG_LAUNCH_CHECK();
    gram_scale_kernel<<<sg::ceil_div_i(int64_t(m) * m, 256), 256, 0, st>>>(b.G, b.D, m);
    SG_LAUNCH_CHECK();
    col_rscale_kernel<<<sg::ceil_div_i(int64_t(n) * m, 256), 256, 0, st>>>(Y, b.D, n, m);
    SG_LAUNCH_CHECK();
    SG_SOLVER(cusolverDnSpotrf(sol, CUBLAS_FILL_MODE_LOWER, m, b.G, m, static_cast<float*>(h->solver_work),
                               int(h->solver_work_bytes / sizeof(float)), inf));
    SG_BLAS(cublasStrsm(blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, m, &one,
                        b.G, m, Y, n));
  }
  return SG_OK;
}

constexpr int kTailCols = 8;

// C = alpha A B + beta C for the filter's n x n by n x m products: FP32 inputs
// and outputs, computed by cuBLAS as FP32 emulated with BF16 splits on the
// tensor cores (the accuracy of an FP32 GEMM, about 20% faster here)
cublasStatus_t filter_gemm(cublasHandle_t blas, int n, int m, const float* alpha, const float* A, const float* B,
                           const float* beta, float* C) {
  return cublasGemmEx(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, n, alpha, A, CUDA_R_32F, n, B, CUDA_R_32F, n, beta, C,
                      CUDA_R_32F, n, CUBLAS_COMPUTE_32F_EMULATED_16BFX9, CUBLAS_GEMM_DEFAULT);
}

// One filter segment on the block X: X <- orth(T_deg((2A - cut I)/cut) X),
// the Chebyshev polynomial that is bounded by 1 on [0, cut] and grows fastest
// above it. Recurrence: Y1 = (2/cut) A X - X, Y_{k+1} = (4/cut) A Y_k - 2 Y_k - Y_{k-1}.
// *tail_rq receives the smallest Rayleigh quotient of the input block's last
// kTailCols columns (host value; synchronises).
int filter_segment(sg_handle* h, cusolverDnHandle_t sol, cublasHandle_t blas, const float* A32, int n, int m, int deg,
                   double cut, FilterBufs& b, cudaStream_t st, float* tail_rq, int qr_passes) {
  const float a1 = float(2.0 / cut), a2 = float(4.0 / cut), m1 = -1.f, m2 = -2.f, one = 1.f;
  float* prev = b.X;
  float* cur = b.P;
  const int K = std::min(kTailCols, m);
  {
    sg::ProfScope prof_f(h, "eig_filter", st);
    SG_CUDA(cudaMemcpyAsync(cur, prev, sizeof(float) * size_t(n) * m, cudaMemcpyDeviceToDevice, st));
    SG_BLAS(filter_gemm(blas, n, m, &a1, A32, prev, &m1, cur));
    tail_rq_kernel<<<K, 256, 0, st>>>(prev, cur, n, m, K, a1, b.R);
    SG_LAUNCH_CHECK();
    for (int k = 2; k <= deg; ++k) {
      // prev <- -prev - 2 cur, then prev <- (4/cut) A cur + prev
      SG_BLAS(cublasSgeam(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, &m1, prev, n, &m2, cur, n, prev, n));
      SG_BLAS(filter_gemm(blas, n, m, &a2, A32, cur, &one, prev));
      std::swap(prev, cur);
    }
  }
  int rc = cholqr_f32(h, sol, blas, cur, n, m, b, qr_passes, st);
  if (rc) return rc;
  // the tail quotients are read once the segment's work is queued
  float hr[kTailCols];
  SG_CUDA(cudaMemcpyAsync(hr, b.R, sizeof(float) * size_t(K), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  float mn = INFINITY;
  for (int k = 0; k < K; ++k) mn = std::isfinite(hr[k]) ? std::min(mn, hr[k]) : mn;
  *tail_rq = mn;
  if (cur != b.X) {
    // keep X as the block; the other two buffers stay scratch
    if (cur == b.P) std::swap(b.X, b.P);
    else std::swap(b.X, b.Q);
  }
  return SG_OK;
}

// FP32 Rayleigh-Ritz of the block: X <- X U (Ritz vectors, descending: the
// dominant directions first); the Ritz values, ascending, are copied to `wh`
// (host, synchronising).
int ritz_f32(sg_handle* h, cusolverDnHandle_t sol, cublasHandle_t blas, const float* A32, int n, int m, FilterBufs& b,
             int lwork_s, std::vector<float>& wh, bool vectors, cudaStream_t st) {
  const float one = 1.f, zero = 0.f;
  sg::ProfScope prof(h, "eig_rr32", st);
  SG_BLAS(filter_gemm(blas, n, m, &one, A32, b.X, &zero, b.P));
  SG_BLAS(cublasSgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, b.X, n, b.P, n, &zero, b.G, m));
  int* inf = b.info + std::min(b.n_info, b.cap_info - 1);
  ++b.n_info;
  const cusolverEigMode_t mode = vectors ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
  if (b.jac && m <= kJacobiMax)
    SG_SOLVER(cusolverDnSsyevj(sol, mode, CUBLAS_FILL_MODE_LOWER, m, b.G, m, b.W, static_cast<float*>(h->solver_work),
                               int(h->solver_work_bytes / sizeof(float)), inf, b.jac));
  else
    SG_SOLVER(cusolverDnSsyevd(sol, mode, CUBLAS_FILL_MODE_LOWER, m, b.G, m, b.W, static_cast<float*>(h->solver_work),
                               lwork_s, inf));
  if (vectors) {
    reverse_cols_kernel<<<sg::ceil_div_i(int64_t(m / 2) * m, 256), 256, 0, st>>>(b.G, m);
    SG_LAUNCH_CHECK();
    SG_BLAS(cublasSgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, n, m, m, &one, b.X, n, b.G, m, &zero, b.P, n));
    std::swap(b.X, b.P);
  }
  wh.resize(size_t(m));
  SG_CUDA(cudaMemcpyAsync(wh.data(), b.W, sizeof(float) * size_t(m), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  return SG_OK;
}

// degree s of the largest s <= smax with T_s(t) <= bound (t >= 1)
int cheb_degree(double t, double bound, int smax) {
  int s = 1;
  for (int k = 2; k <= smax; ++k) {
    if (std::cosh(k * std::acosh(std::max(1.0, t))) > bound) break;
    s = k;
  }
  return s;
}

}  // namespace

// Principal axes by Chebyshev-filtered block subspace iteration: FP32 cuBLAS
// GEMMs apply Chebyshev polynomials of the centred scatter, damped on [0, cut],
// to an m-wide block kept in descending order (dominant directions first),
// re-orthogonalised by column-scaled FP32 Cholesky-QR after each segment. The
// cut starts at the block's smallest Ritz value (never above its m-th
// eigenvalue) and rises with the Rayleigh quotients of its last columns,
// capped below the wanted pairs, so no wanted pair is damped. An FP32
// Rayleigh-Ritz step picks the top n_comp + 16 Ritz vectors and the FP64
// Rayleigh-Ritz step of the mixed solver refines them. If the FP64 residual
// of a wanted pair exceeds 1e-4 of the largest eigenvalue, or the problem is
// too small for the block, the mixed solver runs instead.
extern "C" int sg_pca_basis_filter(sg_handle* h, const double* cov, const double* zsum, int64_t n_used,
                                   int32_t n_cols, int32_t n_comp, double* comps, double* evals, double* evr,
                                   int32_t n_load, float* loadings32, int32_t ld_l, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(cov && comps && n_cols > 0 && n_used > 0, "sg_pca_basis_filter: bad arguments");
  SG_ARG(n_comp >= 1 && n_comp <= n_cols, "sg_pca_basis_filter: n_comp=%d outside [1, %d]", n_comp, n_cols);
  SG_ARG(!loadings32 || (n_load >= 0 && n_load <= n_comp && ld_l >= n_load),
         "sg_pca_basis_filter: bad loadings shape");
  const int n = n_cols;
  const int p = n_comp + 16;
  const int m = int(sg::ceil_div(std::max<int64_t>(p + 64, (5 * int64_t(p)) / 2), 32) * 32);
  h->eig_resid = NAN;
  if (m > 256 || 2 * m > n || n_used < 4 * int64_t(m))
    return sg_pca_basis_mixed(h, cov, zsum, n_used, n_cols, n_comp, comps, evals, evr, n_load, loadings32, ld_l,
                              stream);
  cusolverDnHandle_t sol;
  cublasHandle_t blas;
  int rc = solver_handles(h, st, &sol, &blas);
  if (rc) return rc;
  const size_t nn = size_t(n) * n, nm = size_t(n) * m, np = size_t(n) * p, pp = size_t(p) * p;
  const int cap_info = 128;
  const size_t need = sg::Carver::need(nn * 8) + sg::Carver::need(nn * 4) + 3 * sg::Carver::need(nm * 4) +
                      sg::Carver::need(size_t(m) * m * 4) + 2 * sg::Carver::need(size_t(m) * 4) +
                      sg::Carver::need(kTailCols * 4) + sg::Carver::need(nn * 4) + sg::Carver::need(size_t(n) * 12) +
                      sg::Carver::need(8) +
                      3 * sg::Carver::need(np * 8) + 2 * sg::Carver::need(pp * 8) + sg::Carver::need(size_t(p) * 8) +
                      sg::Carver::need(size_t(p) * 8) + sg::Carver::need(16) + sg::Carver::need(cap_info * 4);
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  double* A = cv.take<double>(nn);
  float* A32 = cv.take<float>(nn);
  FilterBufs b;
  b.X = cv.take<float>(nm);
  b.P = cv.take<float>(nm);
  b.Q = cv.take<float>(nm);
  b.G = cv.take<float>(size_t(m) * m);
  b.W = cv.take<float>(size_t(m));
  b.D = cv.take<float>(size_t(m));
  b.R = cv.take<float>(size_t(kTailCols));
  float* A32d = cv.take<float>(nn);       // the scatter with the locked pair deflated
  float* lv = cv.take<float>(size_t(n) * 3);  // the locked vector and two recurrence buffers
  float* lrq = cv.take<float>(2);
  double* Qd = cv.take<double>(np);
  double* Yd = cv.take<double>(np);
  double* Vd = cv.take<double>(np);
  double* Gd = cv.take<double>(pp);
  double* Bd = cv.take<double>(pp);
  double* Wd = cv.take<double>(size_t(p));
  double* rcol = cv.take<double>(size_t(p));
  double* tr = cv.take<double>(2);
  b.info = cv.take<int>(cap_info);
  b.n_info = 0;
  b.cap_info = cap_info;
  SG_CUDA(cudaMemsetAsync(b.info, 0, sizeof(int) * cap_info, st));
  const int64_t ne = int64_t(nn);
  center_kernel<<<sg::ceil_div_i(ne, 256), 256, 0, st>>>(cov, zsum, 1.0 / double(n_used), n, A);
  SG_LAUNCH_CHECK();
  trace_kernel<<<1, 256, 0, st>>>(A, n, tr);
  SG_LAUNCH_CHECK();
  f64_to_f32_kernel<<<sg::ceil_div_i(ne, 256), 256, 0, st>>>(A, A32, ne);
  SG_LAUNCH_CHECK();
  sg::ProfScope prof(h, "eigh", st);
  float* rowmax = reinterpret_cast<float*>(tr + 1);
  SG_CUDA(cudaMemsetAsync(rowmax, 0, sizeof(float), st));
  absrow_max_kernel<<<std::min(n, 4 * h->sm_count), 256, 0, st>>>(A32, n, rowmax);
  SG_LAUNCH_CHECK();
  random_block_kernel<<<sg::ceil_div_i(int64_t(nm), 256), 256, 0, st>>>(b.X, int64_t(nm), 0x5CA2F00Dull);
  SG_LAUNCH_CHECK();
  // workspace: FP32 potrf / syevd of m, FP64 potrf / syevd of p
  int lw_potrf = 0, lw_s = 0, lw_d = 0, lw_dp = 0;
  SG_SOLVER(cusolverDnSpotrf_bufferSize(sol, CUBLAS_FILL_MODE_LOWER, m, b.G, m, &lw_potrf));
  SG_SOLVER(cusolverDnSsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, b.G, m, b.W, &lw_s));
  JacobiGuard jac;
  if (m <= kJacobiMax) {
    SG_SOLVER(cusolverDnCreateSyevjInfo(&jac.p));
    SG_SOLVER(cusolverDnXsyevjSetTolerance(jac.p, 0.0));   // machine accuracy
    SG_SOLVER(cusolverDnXsyevjSetMaxSweeps(jac.p, 20));
    int lw_j = 0;
    SG_SOLVER(cusolverDnSsyevj_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, b.G, m, b.W,
                                          &lw_j, jac.p));
    lw_s = std::max(lw_s, lw_j);
    b.jac = jac.p;
  }
  SG_SOLVER(cusolverDnDsyevd_bufferSize(sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, p, Bd, p, Wd, &lw_d));
  SG_SOLVER(cusolverDnDpotrf_bufferSize(sol, CUBLAS_FILL_MODE_LOWER, p, Gd, p, &lw_dp));
  const size_t wb = std::max(std::max(sizeof(float) * size_t(lw_potrf), sizeof(float) * size_t(lw_s)),
                             std::max(sizeof(double) * size_t(lw_d), sizeof(double) * size_t(lw_dp)));
  rc = solver_work(h, wb);
  if (rc) return rc;
  rc = cholqr_f32(h, sol, blas, b.X, n, m, b, 2, st);
  if (rc) return rc;
  double hd[2];
  SG_CUDA(cudaMemcpyAsync(hd, tr, sizeof(double), cudaMemcpyDeviceToHost, st));
  float hrow = 0.f;
  SG_CUDA(cudaMemcpyAsync(&hrow, rowmax, sizeof(float), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  const double trace = hd[0];
  // phase A: the mean eigenvalue as the cut, degrees bounded by the row-sum bound
  double cut = std::max(trace / n, 1e-30);
  int deg = cheb_degree(2.0 * double(hrow) / cut - 1.0, 1e3, 8);
  EIG_DBG("filter: n=%d m=%d p=%d trace/n=%g rowmax=%g degA=%d\n", n, m, p, cut, double(hrow), deg);
  float rq = 0.f;
  for (int s = 0; s < 2; ++s) {  // the second leaves X orthonormal for the Rayleigh-Ritz step
    rc = filter_segment(h, sol, blas, A32, n, m, deg, cut, b, st, &rq, s == 1 ? 2 : 1);
    if (rc) return rc;
  }
  // phase B: cut from the block's smallest Ritz value, degree from its largest
  std::vector<float> th;
  rc = ritz_f32(h, sol, blas, A32, n, m, b, lw_s, th, true, st);
  if (rc) return rc;
  bool ok = th[0] > 0.f && std::isfinite(th[size_t(m - 1)]);
  EIG_DBG("filter: RR1 ok=%d theta_min=%g theta_max=%g\n", int(ok), double(th[0]), double(th[size_t(m - 1)]));
  double resid = INFINITY;
  if (ok) {
    // The cut starts at the block's smallest Ritz value (never above its
    // m-th eigenvalue) and rises with the smallest Rayleigh quotient of the
    // block's last columns as the block converges, capped at 0.99 x the Ritz
    // value of pair n_comp + 8, which is a lower bound of that eigenvalue: no
    // wanted pair is ever damped.
    cut = double(th[0]);
    double theta_w = double(th[size_t(m - std::min(m, n_comp + 8))]);
    double cut_cap = 0.99 * theta_w;
    double theta_max = 1.05 * double(th[size_t(m - 1)]);
    // Degree budget: each segment amplifies pair n_comp over the damped
    // interval by about exp(deg * acosh(t)), t = 2 theta_c / cut - 1 for the
    // cut it ran with; stop when the product reaches 1e10. A flat spectrum
    // near the cut (many cells: a narrow Marchenko-Pastur bulk) gets more
    // segments, a well separated one fewer.
    double theta_c = double(th[size_t(m - std::min(m, n_comp))]);
    // Lock a leading spike: when the largest Ritz value is far above the cut
    // (t > 3) and 1.5 x the next, its growth alone would hold every segment to
    // a low degree. Its vector is polished by one Chebyshev segment of its
    // own (cut at the next Ritz value) and deflated from a copy of the
    // scatter; the other m - 1 columns are filtered with the deflated
    // operator, whose largest eigenvalue is then the next one.
    const float* Aop = A32;
    int L = 0, ma = m;
    {
      const double t1 = double(th[size_t(m - 1)]), t2 = double(th[size_t(m - 2)]);
      if (2.0 * t1 / cut - 1.0 > 3.0 && t1 >= 1.5 * t2 && n_comp >= 2) L = 1;
      if (L) {
        const float one = 1.f, zero = 0.f, mtwo = -2.f, mone = -1.f;
        float* v = lv;
        float* y0 = lv + n;
        float* y1 = lv + 2 * n;
        SG_CUDA(cudaMemcpyAsync(v, b.X, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, st));
        const double cl = t2;  // a lower bound of the second eigenvalue
        const int dl = std::min(24, int(std::ceil(std::acosh(1e8) / std::acosh(2.0 * t1 / cl - 1.0))));
        const float a1 = float(2.0 / cl), a2 = float(4.0 / cl);
        // y0 = v, y1 = (2/c) A v - v, y_{k+1} = (4/c) A y_k - 2 y_k - y_{k-1}
        SG_CUDA(cudaMemcpyAsync(y0, v, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, st));
        SG_CUDA(cudaMemcpyAsync(y1, v, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, st));
        SG_BLAS(cublasSgemv(blas, CUBLAS_OP_N, n, n, &a1, A32, n, v, 1, &mone, y1, 1));
        float* pr = y0;
        float* cr = y1;
        for (int k = 2; k <= dl; ++k) {
          SG_BLAS(cublasSscal(blas, n, &mone, pr, 1));
          SG_BLAS(cublasSaxpy(blas, n, &mtwo, cr, 1, pr, 1));
          SG_BLAS(cublasSgemv(blas, CUBLAS_OP_N, n, n, &a2, A32, n, cr, 1, &one, pr, 1));
          std::swap(pr, cr);
        }
        SG_CUDA(cudaMemcpyAsync(v, cr, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, st));
        normalize_rq_kernel<<<1, 1024, 0, st>>>(v, v, n, lrq + 1);  // unit length
        SG_LAUNCH_CHECK();
        SG_BLAS(cublasSgemv(blas, CUBLAS_OP_N, n, n, &one, A32, n, v, 1, &zero, y0, 1));
        normalize_rq_kernel<<<1, 1024, 0, st>>>(v, y0, n, lrq);  // Rayleigh quotient of the unit vector
        SG_LAUNCH_CHECK();
        float hrq = 0.f;
        SG_CUDA(cudaMemcpyAsync(&hrq, lrq, sizeof(float), cudaMemcpyDeviceToHost, st));
        SG_CUDA(cudaStreamSynchronize(st));
        if (!(hrq > 0.f) || !std::isfinite(hrq)) {
          L = 0;
        } else {
          // deflated operator A - theta v v^T, and the active block X[:, 1:m]
          SG_CUDA(cudaMemcpyAsync(A32d, A32, sizeof(float) * nn, cudaMemcpyDeviceToDevice, st));
          const float mth = -hrq;
          SG_BLAS(cublasSger(blas, n, n, &mth, v, 1, v, 1, A32d, n));
          SG_CUDA(cudaMemcpyAsync(b.P, b.X + n, sizeof(float) * size_t(n) * (m - 1), cudaMemcpyDeviceToDevice, st));
          std::swap(b.X, b.P);
          Aop = A32d;
          ma = m - 1;
          theta_max = 1.05 * t2;
          EIG_DBG("filter: locked theta=%g (RR1 %g), next %g, polish degree %d\n", double(hrq), t1, t2, dl);
        }
      }
    }
    const double target = std::log(1e10);
    double gain = 0.0;
    int done = 0, segs = 0;
    bool refreshed = false;
    EIG_DBG("filter: RR1 theta_min=%g theta_c=%g theta_w=%g theta_max=%g\n", double(th[0]), theta_c, theta_w,
            double(th[size_t(m - 1)]));
    // long segments while the dominant directions lead the block (their
    // growth over the weakest column at most 1e5), then two short ones
    // (growth at most 1e2) that leave the block accurate to FP32
    for (int polish = 0; gain < target || polish < 2; ++segs) {
      const double t_max = 2.0 * theta_max / cut - 1.0;
      const bool last = gain >= target;
      const int d = cheb_degree(t_max, last ? 1e2 : 1e5, 8);
      rc = filter_segment(h, sol, blas, Aop, n, ma, d, cut, b, st, &rq, last && polish == 1 ? 2 : 1);
      if (rc) return rc;
      if (!last) {
        gain += d * std::acosh(std::max(1.0, 2.0 * theta_c / cut - 1.0));
        done += d;
      }
      EIG_DBG("filter: seg %d deg %d cut %g tail_rq %g gain %g\n", segs, d, cut, double(rq), gain);
      if (!last && !refreshed && std::isfinite(rq) && double(rq) > cut_cap && gain > 0.25 * target) {
        // The cap, from Ritz values of a barely filtered block, holds the cut
        // below the block's tail: fresh Ritz values (of the orthonormalised
        // block, which they also put in descending order) give a higher,
        // still valid cap and a better rate estimate.
        rc = cholqr_f32(h, sol, blas, b.X, n, ma, b, 1, st);
        if (rc) return rc;
        rc = ritz_f32(h, sol, blas, Aop, n, ma, b, lw_s, th, true, st);
        if (rc) return rc;
        refreshed = true;
        if (th[0] > 0.f && std::isfinite(th[size_t(ma - 1)])) {
          // pairs n_comp + 8 and n_comp overall are pairs n_comp + 8 - L and n_comp - L of the active block
          theta_w = std::max(theta_w, double(th[size_t(ma - std::min(ma, n_comp + 8 - L))]));
          theta_c = std::max(theta_c, double(th[size_t(ma - std::min(ma, n_comp - L))]));
          theta_max = std::max(theta_max, 1.05 * double(th[size_t(ma - 1)]));
          cut_cap = 0.99 * theta_w;
        }
        EIG_DBG("filter: refresh theta_c=%g theta_w=%g\n", theta_c, theta_w);
      }
      if (std::isfinite(rq)) cut = std::min(cut_cap, std::max(cut, double(rq)));
      if (last) ++polish;
      if (done >= 240 && !last) gain = target;  // degree cap
    }
    if (L) {
      // the locked vector back in front of the active block, orthonormalised
      // together, for the Rayleigh-Ritz step on the undeflated scatter
      SG_CUDA(cudaMemcpyAsync(b.P, lv, sizeof(float) * size_t(n), cudaMemcpyDeviceToDevice, st));
      SG_CUDA(cudaMemcpyAsync(b.P + n, b.X, sizeof(float) * size_t(n) * ma, cudaMemcpyDeviceToDevice, st));
      std::swap(b.X, b.P);
      rc = cholqr_f32(h, sol, blas, b.X, n, m, b, 2, st);
      if (rc) return rc;
    }
    rc = ritz_f32(h, sol, blas, A32, n, m, b, lw_s, th, true, st);
    if (rc) return rc;
    // the top p Ritz vectors (the first p columns) -> FP64 Rayleigh-Ritz with a residual check
    f32_to_f64_kernel<<<sg::ceil_div_i(int64_t(np), 256), 256, 0, st>>>(b.X, Qd, int64_t(np));
    SG_LAUNCH_CHECK();
    rc = rayleigh_ritz_fp64(h, sol, blas, A, n, p, Qd, Yd, Vd, Gd, Bd, Wd, b.info + cap_info - 2, lw_d, n_comp,
                            &resid, rcol, st);
    if (rc) return rc;
    std::vector<int> hi(static_cast<size_t>(cap_info));
    SG_CUDA(cudaMemcpyAsync(hi.data(), b.info, sizeof(int) * cap_info, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < cap_info; ++i)
      if (hi[size_t(i)] != 0) {
        EIG_DBG("filter: factorisation slot %d info=%d (of %d used)\n", i, hi[size_t(i)], b.n_info);
        ok = false;
      }
    EIG_DBG("filter: RR2 theta_min=%g theta_max=%g resid=%g\n", double(th[0]), double(th[size_t(m - 1)]), resid);
    ok = ok && b.n_info < cap_info - 3 && resid <= 1e-4;
  }
  h->eig_resid = ok ? resid : INFINITY;
  if (!ok)
    return sg_pca_basis_mixed(h, cov, zsum, n_used, n_cols, n_comp, comps, evals, evr, n_load, loadings32, ld_l,
                              stream);
  basis_kernel<<<n_comp, 256, 0, st>>>(Vd + size_t(p - n_comp) * n, Wd + (p - n_comp), n, n_comp, tr, comps, evals,
                                       evr, n_load, loadings32, ld_l);
  SG_LAUNCH_CHECK();
  SG_CUDA(cudaStreamSynchronize(st));
  return SG_OK;
}

extern "C" int sg_project(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld,
                          const float* mu32, const float* sigma32, const float* loadings32, int32_t d,
                          int32_t ld_l, float* scores, int32_t ld_s, void* bf16_out, int32_t ld_b,
                          int32_t precision, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(x && mu32 && sigma32 && loadings32 && scores, "sg_project: null pointer argument");
  SG_ARG(n_rows >= 0 && n_cols > 0 && ld >= n_cols && d > 0 && ld_l >= d && ld_s >= d, "sg_project: bad sizes");
  SG_ARG(!bf16_out || ld_b >= d, "sg_project: ld_b < d");
  SG_ARG(precision == SG_PLAIN || precision == SG_PRECISION, "sg_project: unknown precision %d", precision);
  if (n_rows == 0) return SG_OK;
  // the precision form on the tensor cores; rows of x that TMA cannot address
  // (an unaligned base or row stride) take the FP32 SIMT kernel instead
  if (precision == SG_PRECISION && sg_project_tc_supported(x, ld, d))
    return sg_project_tc(h, x, n_rows, n_cols, ld, mu32, sigma32, loadings32, d, ld_l, scores, ld_s,
                         static_cast<__nv_bfloat16*>(bf16_out), ld_b, st);
  SG_ARG(precision == SG_PLAIN || d <= 64, "sg_project: the precision form supports d <= 64");
  const int ccols = std::max<int>(ld_s, bf16_out ? ld_b : 0);
  sg::ProfScope prof(h, "project", st);
  dim3 grid(sg::ceil_div_i(n_rows, PR), sg::ceil_div_i(std::min<int>(ccols, sg::ceil_div_i(d, PC) * PC), PC));
  project_kernel<<<grid, 256, 0, st>>>(x, n_rows, n_cols, ld, mu32, sigma32, loadings32, d, ld_l, scores, ld_s,
                                       static_cast<__nv_bfloat16*>(bf16_out), ld_b);
  SG_LAUNCH_CHECK();
  const int covered = int(grid.y) * PC;
  if (covered < ld_s || (bf16_out && covered < ld_b)) {
    pad_cols_kernel<<<sg::ceil_div_i(n_rows, 256), 256, 0, st>>>(scores, n_rows, std::min(covered, ld_s), ld_s,
                                                                 static_cast<__nv_bfloat16*>(bf16_out),
                                                                 std::min(covered, bf16_out ? ld_b : 0), ld_b);
    SG_LAUNCH_CHECK();
  }
  return SG_OK;
}

extern "C" double sg_pca_filter_residual(const sg_handle* h) { return h ? h->eig_resid : NAN; }
