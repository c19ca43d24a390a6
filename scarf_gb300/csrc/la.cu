// Small dense linear algebra of the PCA eigensolver (see la.cuh).
#include "la.cuh"

#include <algorithm>
#include <cmath>

namespace sg {
namespace la {
namespace {

constexpr int GBM = 64, GBN = 64, GBK = 16;

int sm_count() {
  static int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

// K splits for an m x n output: enough CTAs for about two waves, at least 256
// of K per split
int gemm_splits(int m, int n, int k) {
  const int64_t tiles = int64_t((m + GBM - 1) / GBM) * ((n + GBN - 1) / GBN);
  const int64_t want = (2 * int64_t(sm_count()) + tiles - 1) / tiles;
  const int64_t cap = std::max<int64_t>(1, k / 256);
  return int(std::max<int64_t>(1, std::min(want, cap)));
}

// C tile (64 x 64) of alpha op(A) B + beta C, or its partial over one split of
// K into part[split] (column-major m x n) when part is given. 256 threads,
// each a 4 x 4 micro-tile; K staged through shared memory 16 at a time.
template <typename T, bool TA>
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, int kps, T alpha, const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
            T beta, T* __restrict__ C, int ldc, T* __restrict__ part) {
  __shared__ __align__(16) T As[GBK][GBM + 4];
  __shared__ __align__(16) T Bs[GBK][GBN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int i0 = blockIdx.x * GBM, j0 = blockIdx.y * GBN;
  const int kb = blockIdx.z * kps, ke = min(K, kb + kps);
  T acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
  for (int k0 = kb; k0 < ke; k0 += GBK) {
#pragma unroll
    for (int r = 0; r < (GBM * GBK) / 256; ++r) {
      const int e = tid + 256 * r;
      int ii, kk;
      if (!TA) {  // consecutive threads: consecutive rows of A (column-major)
        ii = e % GBM;
        kk = e / GBM;
      } else {    // op(A)(i, k) = A[k + i lda]: consecutive threads, consecutive k
        kk = e % GBK;
        ii = e / GBK;
      }
      const int i = i0 + ii, k = k0 + kk;
      T v = T(0);
      if (i < M && k < ke) v = TA ? A[k + int64_t(i) * lda] : A[i + int64_t(k) * lda];
      As[kk][ii] = v;
    }
#pragma unroll
    for (int r = 0; r < (GBK * GBN) / 256; ++r) {
      const int e = tid + 256 * r;
      const int kk = e % GBK, jj = e / GBK;
      const int k = k0 + kk, j = j0 + jj;
      Bs[kk][jj] = (j < N && k < ke) ? B[k + int64_t(j) * ldb] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[kk][tx * 4 + q];
        b[q] = Bs[kk][ty * 4 + q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = i0 + tx * 4 + p;
    if (i >= M) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + ty * 4 + q;
      if (j >= N) continue;
      if (part) {
        part[int64_t(blockIdx.z) * M * N + i + int64_t(j) * M] = acc[p][q];
      } else {
        T v = alpha * acc[p][q];
        if (beta != T(0)) v = fma(beta, C[i + int64_t(j) * ldc], v);
        C[i + int64_t(j) * ldc] = v;
      }
    }
  }
}

// C = alpha sum_z part[z] + beta C, the splits added in order
template <typename T>
__global__ void gemm_reduce_kernel(int M, int N, int ns, T alpha, const T* __restrict__ part, T beta,
                                   T* __restrict__ C, int ldc) {
  const int64_t mn = int64_t(M) * N;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < mn; e += int64_t(gridDim.x) * blockDim.x) {
    T s = T(0);
    for (int z = 0; z < ns; ++z) s += part[int64_t(z) * mn + e];
    const int64_t i = e % M, j = e / M;
    T v = alpha * s;
    if (beta != T(0)) v = fma(beta, C[i + j * ldc], v);
    C[i + j * ldc] = v;
  }
}

// row-major packed lower triangle: element (i, k), k <= i
__device__ __forceinline__ int low_idx(int i, int k) { return i * (i + 1) / 2 + k; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Cholesky (Crout order: column j from the finished columns before it), one
// CTA; the factor is built in shared memory and written to G's lower triangle
template <typename T>
__global__ void __launch_bounds__(1024) potrf_kernel(int m, T* __restrict__ G, int ldg, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char potrf_smem[];
  T* L = reinterpret_cast<T*>(potrf_smem);
  __shared__ int bad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
  for (int e = tid; e < m * (m + 1) / 2; e += blockDim.x) {
    // decode (i, k) of packed index e
    int i = int((sqrtf(8.f * float(e) + 1.f) - 1.f) * 0.5f);
    while (i * (i + 1) / 2 > e) --i;
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    const int k = e - i * (i + 1) / 2;
    L[e] = G[i + int64_t(k) * ldg];
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (warp == 0) {
      T s = T(0);
      for (int k = lane; k < j; k += 32) s = fma(L[low_idx(j, k)], L[low_idx(j, k)], s);
      s = warp_sum(s);
      if (lane == 0) {
        const T d = L[low_idx(j, j)] - s;
        if (!(d > T(0))) bad = j + 1;
        else L[low_idx(j, j)] = sqrt(d);
      }
    }
    __syncthreads();
    if (bad) break;
    const T djj = L[low_idx(j, j)];
    for (int i = j + 1 + warp; i < m; i += nw) {
      T s = T(0);
      for (int k = lane; k < j; k += 32) s = fma(L[low_idx(i, k)], L[low_idx(j, k)], s);
      s = warp_sum(s);
      if (lane == 0) L[low_idx(i, j)] = (L[low_idx(i, j)] - s) / djj;
    }
    __syncthreads();
  }
  if (tid == 0) *info = bad;
  if (bad) return;
  for (int e = tid; e < m * (m + 1) / 2; e += blockDim.x) {
    int i = int((sqrtf(8.f * float(e) + 1.f) - 1.f) * 0.5f);
    while (i * (i + 1) / 2 > e) --i;
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    const int k = e - i * (i + 1) / 2;
    G[i + int64_t(k) * ldg] = L[e];
  }
}

// Y <- Y L^-T: row r solves z L^T = y by forward substitution, z_j =
// (y_j - sum_{k<j} L_jk z_k) / L_jj, in place (a thread per row; L packed in
// shared memory, read by every thread at the same address)
template <typename T>
__global__ void trsm_rlt_kernel(int n, int m, const T* __restrict__ G, int ldg, T* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T* L = reinterpret_cast<T*>(trsm_smem);
  for (int e = threadIdx.x; e < m * (m + 1) / 2; e += blockDim.x) {
    int i = int((sqrtf(8.f * float(e) + 1.f) - 1.f) * 0.5f);
    while (i * (i + 1) / 2 > e) --i;
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    const int k = e - i * (i + 1) / 2;
    L[e] = G[i + int64_t(k) * ldg];
  }
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  T* y = Y + r;
  for (int j = 0; j < m; ++j) {
    const T* lj = L + low_idx(j, 0);
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
    int k = 0;
    for (; k + 3 < j; k += 4) {
      s0 = fma(lj[k], y[int64_t(k) * n], s0);
      s1 = fma(lj[k + 1], y[int64_t(k + 1) * n], s1);
      s2 = fma(lj[k + 2], y[int64_t(k + 2) * n], s2);
      s3 = fma(lj[k + 3], y[int64_t(k + 3) * n], s3);
    }
    for (; k < j; ++k) s0 = fma(lj[k], y[int64_t(k) * n], s0);
    y[int64_t(j) * n] = (y[int64_t(j) * n] - ((s0 + s1) + (s2 + s3))) / lj[j];
  }
}

// ---- cyclic Jacobi in round-robin order (one CTA) ------------------------
// A (mp x mp, mp even) as its packed upper triangle in shared memory; V in
// shared memory (mp <= 192) or global scratch. Each round rotates mp/2
// disjoint pairs at once: the 2 x 2 blocks of A between two pairs get the row
// rotation of one and the column rotation of the other, the diagonal block of
// a pair the Jacobi update that zeroes its off-diagonal entry (Numerical
// Recipes' t = tan formulas), and the columns of V the pair's rotation.
constexpr int kJacobiSmemV = 192;
constexpr int kJacobiMaxSweeps = 16;

__device__ __forceinline__ int up_idx(int x, int y, int mp) {  // x <= y
  return x * mp - x * (x - 1) / 2 + (y - x);
}
__device__ __forceinline__ float& aref(float* A, int x, int y, int mp) {
  return x <= y ? A[up_idx(x, y, mp)] : A[up_idx(y, x, mp)];
}
__device__ __forceinline__ int player(int t, int r, int mp) { return t == 0 ? 0 : ((t - 1 + r) % (mp - 1)) + 1; }

template <bool kSmemV>
__global__ void __launch_bounds__(1024)
syev_jacobi_kernel(int m, int mp, const float* __restrict__ Ain, int lda, float* __restrict__ W, float* __restrict__ Vout,
                   float* __restrict__ Vg, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char jac_smem[];
  float* A = reinterpret_cast<float*>(jac_smem);                      // mp (mp + 1) / 2
  float* V = kSmemV ? A + mp * (mp + 1) / 2 : Vg;                     // mp x mp, column-major
  float* rc = (kSmemV ? V + mp * mp : A + mp * (mp + 1) / 2);         // [mp/2] cos
  float* rs = rc + mp / 2;                                            // [mp/2] sin
  float* rt = rs + mp / 2;                                            // [mp/2] tan
  int* rp = reinterpret_cast<int*>(rt + mp / 2);
  int* rq = rp + mp / 2;
  __shared__ float red[2][32];
  __shared__ int stop;
  const int tid = threadIdx.x, nt = blockDim.x, P = mp / 2;
  // the lower triangle of the input; the padding row and column are zero
  for (int x = 0; x < mp; ++x)
    for (int y = x + tid; y < mp; y += nt) A[up_idx(x, y, mp)] = (x < m && y < m) ? Ain[y + int64_t(x) * lda] : 0.f;
  for (int e = tid; e < mp * mp; e += nt) V[e] = (e % mp == e / mp) ? 1.f : 0.f;
  if (tid == 0) stop = 0;
  __syncthreads();
  int sweep = 0;
  for (; sweep < kJacobiMaxSweeps; ++sweep) {
    for (int r = 0; r < mp - 1; ++r) {
      if (tid < P) {
        int p = player(tid, r, mp), q = player(mp - 1 - tid, r, mp);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        const float apq = aref(A, p, q, mp);
        float c = 1.f, s = 0.f, t = 0.f;
        if (apq != 0.f) {
          const float theta = (aref(A, q, q, mp) - aref(A, p, p, mp)) / (2.f * apq);
          const float at = fabsf(theta);
          t = at > 1e18f ? 0.5f / theta : (theta >= 0.f ? 1.f : -1.f) / (at + sqrtf(fmaf(theta, theta, 1.f)));
          c = rsqrtf(fmaf(t, t, 1.f));
          s = t * c;
        }
        rp[tid] = p;
        rq[tid] = q;
        rc[tid] = c;
        rs[tid] = s;
        rt[tid] = t;
      }
      __syncthreads();
      // blocks (a, b), a <= b, of the P x P pair grid (upper triangle, row-major)
      const int U = P * (P + 1) / 2;
      for (int u = tid; u < U; u += nt) {
        int a = 0;
        {
          // row a: first u' = a P - a (a - 1) / 2
          float fa = (float(2 * P + 1) - sqrtf(float(2 * P + 1) * float(2 * P + 1) - 8.f * float(u))) * 0.5f;
          a = max(0, min(P - 1, int(fa)));
          while (a > 0 && a * P - a * (a - 1) / 2 > u) --a;
          while (a + 1 < P && (a + 1) * P - (a + 1) * a / 2 <= u) ++a;
        }
        const int b = a + (u - (a * P - a * (a - 1) / 2));
        const int pa = rp[a], qa = rq[a];
        if (a == b) {
          const float apq = aref(A, pa, qa, mp), t = rt[a];
          aref(A, pa, pa, mp) -= t * apq;
          aref(A, qa, qa, mp) += t * apq;
          aref(A, pa, qa, mp) = 0.f;
        } else {
          const int pb = rp[b], qb = rq[b];
          const float ca = rc[a], sa = rs[a], cb = rc[b], sb = rs[b];
          const float x00 = aref(A, pa, pb, mp), x01 = aref(A, pa, qb, mp);
          const float x10 = aref(A, qa, pb, mp), x11 = aref(A, qa, qb, mp);
          // columns (pair b), then rows (pair a)
          const float y00 = cb * x00 - sb * x01, y01 = sb * x00 + cb * x01;
          const float y10 = cb * x10 - sb * x11, y11 = sb * x10 + cb * x11;
          aref(A, pa, pb, mp) = ca * y00 - sa * y10;
          aref(A, qa, pb, mp) = sa * y00 + ca * y10;
          aref(A, pa, qb, mp) = ca * y01 - sa * y11;
          aref(A, qa, qb, mp) = sa * y01 + ca * y11;
        }
      }
      for (int u = tid; u < P * mp; u += nt) {
        const int k = u / mp, row = u - k * mp;
        const int p = rp[k], q = rq[k];
        const float c = rc[k], s = rs[k];
        const float vp = V[row + p * mp], vq = V[row + q * mp];
        V[row + p * mp] = c * vp - s * vq;
        V[row + q * mp] = s * vp + c * vq;
      }
      __syncthreads();
    }
    // off-diagonal and diagonal mass
    float off = 0.f, dg = 0.f;
    for (int x = 0; x < mp; ++x)
      for (int y = x + tid; y < mp; y += nt) {
        const float v = A[up_idx(x, y, mp)];
        if (y == x) dg = fmaf(v, v, dg);
        else off = fmaf(v, v, off);
      }
    off = warp_sum(off);
    dg = warp_sum(dg);
    if ((tid & 31) == 0) {
      red[0][tid >> 5] = off;
      red[1][tid >> 5] = dg;
    }
    __syncthreads();
    if (tid == 0) {
      float o = 0.f, d = 0.f;
      for (int w = 0; w < (nt >> 5); ++w) {
        o += red[0][w];
        d += red[1][w];
      }
      stop = o <= 1e-14f * d ? 1 : 0;  // off-diagonal norm below 1e-7 of the diagonal's
    }
    __syncthreads();
    if (stop) break;
  }
  // eigenvalues ascending (ties by index), the padding pair left out
  for (int x = tid; x < m; x += nt) {
    const float vx = A[up_idx(x, x, mp)];
    int rank = 0;
    for (int y = 0; y < m; ++y) {
      const float vy = A[up_idx(y, y, mp)];
      rank += (vy < vx) || (vy == vx && y < x);
    }
    W[rank] = vx;
    for (int row = 0; row < m; ++row) Vout[row + int64_t(rank) * m] = V[row + x * mp];
  }
  if (tid == 0) *info = stop ? 0 : -1;  // 0: converged
}

__global__ void symv_kernel(int n, float alpha, const float* __restrict__ A, const float* __restrict__ x, float beta,
                            float* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // a warp per output: column j of the symmetric A
  if (j >= n) return;
  const float* col = A + int64_t(j) * n;
  float s = 0.f;
  for (int i = lane; i < n; i += 32) s = fmaf(col[i], x[i], s);
  s = warp_sum(s);
  if (lane == 0) y[j] = beta != 0.f ? fmaf(beta, y[j], alpha * s) : alpha * s;
}

__global__ void syr_kernel(int n, const float* __restrict__ A, float th, const float* __restrict__ v,
                           float* __restrict__ out) {
  const int64_t nn = int64_t(n) * n;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nn; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = e % n, j = e / n;
    out[e] = fmaf(th * v[i], v[j], A[e]);
  }
}

__global__ void cheb_combine_kernel(int64_t n, float* __restrict__ prev, const float* __restrict__ cur) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x)
    prev[e] = fmaf(-2.f, cur[e], -prev[e]);
}

unsigned grid_for(int64_t n, int per = 256) {
  return unsigned(std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, int64_t(sm_count()) * 16)));
}

}  // namespace

size_t gemm_scratch(int m, int n, int k) {
  const int ns = gemm_splits(m, n, k);
  return ns > 1 ? size_t(ns) * size_t(m) * size_t(n) : 0;
}

template <typename T>
int gemm(bool trans_a, int m, int n, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc,
         T* scratch, cudaStream_t st) {
  if (m <= 0 || n <= 0) return SG_OK;
  const int ns = scratch ? gemm_splits(m, n, k) : 1;
  const int kps = ((k + ns - 1) / ns + GBK - 1) / GBK * GBK;
  const int nsplit = std::max(1, (k + kps - 1) / kps);
  dim3 grid(unsigned((m + GBM - 1) / GBM), unsigned((n + GBN - 1) / GBN), unsigned(nsplit));
  T* part = nsplit > 1 ? scratch : nullptr;
  if (trans_a)
    gemm_kernel<T, true><<<grid, 256, 0, st>>>(m, n, k, kps, alpha, A, lda, B, ldb, beta, C, ldc, part);
  else
    gemm_kernel<T, false><<<grid, 256, 0, st>>>(m, n, k, kps, alpha, A, lda, B, ldb, beta, C, ldc, part);
  SG_LAUNCH_CHECK();
  if (part) {
    gemm_reduce_kernel<T><<<grid_for(int64_t(m) * n), 256, 0, st>>>(m, n, nsplit, alpha, part, beta, C, ldc);
    SG_LAUNCH_CHECK();
  }
  return SG_OK;
}

template int gemm<float>(bool, int, int, int, float, const float*, int, const float*, int, float, float*, int, float*,
                         cudaStream_t);
template int gemm<double>(bool, int, int, int, double, const double*, int, const double*, int, double, double*, int,
                          double*, cudaStream_t);

template <typename T>
int potrf(int m, T* G, int ldg, int* info, cudaStream_t st) {
  SG_ARG(m >= 1 && m <= 256, "potrf: m=%d outside [1, 256]", m);
  const size_t smem = sizeof(T) * size_t(m) * (m + 1) / 2;
  SG_CUDA(cudaFuncSetAttribute(potrf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  potrf_kernel<T><<<1, 1024, smem, st>>>(m, G, ldg, info);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
template int potrf<float>(int, float*, int, int*, cudaStream_t);
template int potrf<double>(int, double*, int, int*, cudaStream_t);

template <typename T>
int trsm_rlt(int n, int m, const T* G, int ldg, T* Y, cudaStream_t st) {
  SG_ARG(m >= 1 && m <= 256, "trsm: m=%d outside [1, 256]", m);
  if (n <= 0) return SG_OK;
  const size_t smem = sizeof(T) * size_t(m) * (m + 1) / 2;
  SG_CUDA(cudaFuncSetAttribute(trsm_rlt_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  trsm_rlt_kernel<T><<<unsigned((n + 31) / 32), 32, smem, st>>>(n, m, G, ldg, Y);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
template int trsm_rlt<float>(int, int, const float*, int, float*, cudaStream_t);
template int trsm_rlt<double>(int, int, const double*, int, double*, cudaStream_t);

int syev_f32(int m, const float* A, int lda, float* W, float* V, float* scratch, int* info, cudaStream_t st) {
  SG_ARG(m >= 1 && m <= 256, "syev: m=%d outside [1, 256]", m);
  const int mp = (m + 1) / 2 * 2;
  const bool smem_v = mp <= kJacobiSmemV;
  SG_ARG(smem_v || scratch, "syev: m=%d needs scratch for the vectors", m);
  const size_t smem = sizeof(float) * (size_t(mp) * (mp + 1) / 2 + (smem_v ? size_t(mp) * mp : 0) + 3 * (mp / 2)) +
                      sizeof(int) * 2 * (mp / 2);
  if (smem_v) {
    SG_CUDA(cudaFuncSetAttribute(syev_jacobi_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    syev_jacobi_kernel<true><<<1, 1024, smem, st>>>(m, mp, A, lda, W, V, nullptr, info);
  } else {
    SG_CUDA(cudaFuncSetAttribute(syev_jacobi_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    syev_jacobi_kernel<false><<<1, 1024, smem, st>>>(m, mp, A, lda, W, V, scratch, info);
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}

int symv_f32(int n, float alpha, const float* A, const float* x, float beta, float* y, cudaStream_t st) {
  symv_kernel<<<unsigned((int64_t(n) * 32 + 255) / 256), 256, 0, st>>>(n, alpha, A, x, beta, y);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

int syr_f32(int n, const float* A, float theta_neg, const float* v, float* A_out, cudaStream_t st) {
  syr_kernel<<<grid_for(int64_t(n) * n), 256, 0, st>>>(n, A, theta_neg, v, A_out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

int cheb_combine_f32(int64_t n, float* prev, const float* cur, cudaStream_t st) {
  cheb_combine_kernel<<<grid_for(n), 256, 0, st>>>(n, prev, cur);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

}  // namespace la
}  // namespace sg
