// a8: smoothen_dists (scarf/knn_utils.py:89-159) over the published
// umap-learn smooth_knn_dist / compute_membership_strengths, in float32.
//
// Kernel 1 (one CTA per chunk of `chunk_rows` rows): the FP64 sum of the
// chunk's distances (the sigma floor of rows whose rho is 0) and the chunk's
// zero flag / minimum, reset.
// Kernel 2 (128 rows per CTA): the rows' distances are staged through shared
// memory with coalesced loads; one thread per row finds rho and sigma; then
// each warp writes the edges and weights of its rows, lanes across the k
// neighbours (coalesced 16-byte edge stores). Per chunk it records whether a
// weight is zero and the smallest non-zero weight (atomicMin on the float
// bits; positive floats order like their bit patterns).
// Kernel 3 (one CTA per chunk holding a zero): global_min = min(1, minima of
// the chunks holding a zero), written over that chunk's zero weights.
//
// sigma is a bisection on sum_{j>=1} exp(-max(0, d_j - rho)/sigma) =
// log2(k)*bandwidth (the sum starts at column 1), stopping within 1e-5, with
// float32 lo/hi/mid. umap-learn compiles this loop with numba's fastmath, so
// its own sums carry no fixed rounding; here each term is one reciprocal
// multiply and one hardware exp2 (relative error ~1e-7 per term, far inside
// the 1e-5 stopping band). The weights themselves use IEEE division and expf.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

namespace {

constexpr int kRowsPerCta = 128;
constexpr int kMaxK = 128;
constexpr float kLog2e = 1.4426950408889634f;

__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// one CTA per chunk: FP64 sum of its distances; zero flag and minimum reset
__global__ void chunk_stats_kernel(const float* __restrict__ dist, int64_t n, int k, int64_t chunk_rows,
                                   double* __restrict__ chunk_sum, unsigned* __restrict__ chunk_min,
                                   int* __restrict__ chunk_zero) {
  const int64_t c = blockIdx.x;
  const int64_t a = c * chunk_rows * k, b = min(n, (c + 1) * chunk_rows) * int64_t(k);
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t e = a + threadIdx.x; e < b; e += blockDim.x) s += double(dist[e]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    chunk_sum[c] = red[0];
    chunk_min[c] = 0x7f800000u;
    chunk_zero[c] = 0;
  }
}

__global__ void __launch_bounds__(kRowsPerCta)
smooth_kernel(const int64_t* __restrict__ idx, const float* __restrict__ dist, int64_t n, int k, double lc,
              double target, int64_t chunk_rows, const double* __restrict__ chunk_sum, int64_t* __restrict__ edges,
              bool edges16, double* __restrict__ w_out, unsigned* __restrict__ chunk_min,
              int* __restrict__ chunk_zero) {
  extern __shared__ float sd[];  // kRowsPerCta * pitch distances, then rho and sigma per row
  const int pitch = k | 1;       // odd: thread-per-row reads hit distinct banks
  float* s_rho = sd + kRowsPerCta * pitch;
  float* s_sig = s_rho + kRowsPerCta;
  const int64_t r0 = int64_t(blockIdx.x) * kRowsPerCta;
  const int nrows = int(min(int64_t(kRowsPerCta), n - r0));
  for (int e = threadIdx.x; e < nrows * k; e += blockDim.x) {
    const int rr = e / k, j = e - rr * k;
    sd[rr * pitch + j] = dist[r0 * k + e];
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < nrows) {
    const int64_t row = r0 + t;
    const float* d = sd + t * pitch;
    const float inf = __int_as_float(0x7f800000);
    // rho: the local_connectivity-th non-zero distance (interpolated)
    int nnz = 0;
    for (int j = 0; j < k; ++j) nnz += d[j] > 0.f;
    const int index = int(floor(lc));
    const double interp = lc - double(index);  // a float64 scalar in the reference
    float rho = 0.f;
    if (double(nnz) >= lc) {
      if (index > 0) {
        int seen = 0;
        float prev = 0.f, at = 0.f;
        for (int j = 0; j < k; ++j) {
          if (d[j] > 0.f) {
            ++seen;
            if (seen == index) prev = d[j];
            if (seen == index + 1) { at = d[j]; break; }
          }
        }
        rho = prev;
        if (interp > 1e-5) rho = float(double(rho) + interp * double(at - prev));
      } else {
        float first = 0.f;
        for (int j = 0; j < k; ++j)
          if (d[j] > 0.f) { first = d[j]; break; }
        rho = float(interp * double(first));
      }
    } else if (nnz > 0) {
      float mx = 0.f;
      for (int j = 0; j < k; ++j)
        if (d[j] > 0.f) mx = fmaxf(mx, d[j]);
      rho = mx;
    }
    // sigma: bisection with float32 lo/hi/mid; the sum skips column 0
    float lo = 0.f, hi = inf, mid = 1.f;
    for (int it = 0; it < 64; ++it) {
      const float sc = -rcp_approx(mid) * kLog2e;
      float psum = 0.f;
      for (int j = 1; j < k; ++j) {
        const float dd = d[j] - rho;
        psum += dd > 0.f ? ex2_approx(dd * sc) : 1.f;
      }
      if (fabs(double(psum) - target) < 1e-5) break;
      if (double(psum) > target) {
        hi = mid;
        mid = (lo + hi) / 2.f;
      } else {
        lo = mid;
        if (hi == inf) mid *= 2.f;
        else mid = (lo + hi) / 2.f;
      }
    }
    float sigma = mid;
    const int64_t chunk = row / chunk_rows;
    if (rho > 0.f) {
      float s = 0.f;
      for (int j = 0; j < k; ++j) s += d[j];
      const double lim = 1e-3 * (double(s) / k);
      if (double(sigma) < lim) sigma = float(lim);
    } else {
      const int64_t cr = min(chunk_rows, n - chunk * chunk_rows);
      const double lim = 1e-3 * (chunk_sum[chunk] / double(cr * k));
      if (double(sigma) < lim) sigma = float(lim);
    }
    s_rho[t] = rho;
    s_sig[t] = sigma;
  }
  __syncthreads();
  // weights (compute_membership_strengths), a warp per row, lanes over the
  // neighbours; the self test uses the chunk-local row number, as the
  // reference passes global neighbour indices
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int rr = warp; rr < nrows; rr += kRowsPerCta / 32) {
    const int64_t row = r0 + rr;
    const int64_t chunk = row / chunk_rows;
    const int64_t local = row - chunk * chunk_rows;
    const float rho = s_rho[rr], sigma = s_sig[rr];
    bool any_zero = false;
    unsigned mn = 0x7f800000u;
    for (int j = lane; j < k; j += 32) {
      const int64_t e = row * k + j;
      const int64_t nb = idx[e];
      const float dj = sd[rr * pitch + j];
      float v;
      if (nb == local) v = 0.f;
      else if (dj - rho <= 0.f || sigma == 0.f) v = 1.f;
      else v = expf(-__fdiv_rn(dj - rho, sigma));
      if (edges16) {
        reinterpret_cast<longlong2*>(edges)[e] = make_longlong2(row, nb);
      } else {
        edges[2 * e] = row;
        edges[2 * e + 1] = nb;
      }
      w_out[e] = double(v);
      if (v == 0.f) any_zero = true;
      else mn = min(mn, __float_as_uint(v));
    }
    any_zero = __any_sync(0xffffffffu, any_zero);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    if (lane == 0) {
      if (any_zero && !chunk_zero[chunk]) atomicOr(&chunk_zero[chunk], 1);
      if (mn < 0x7f800000u) atomicMin(&chunk_min[chunk], mn);
    }
  }
}

// One CTA per chunk: a chunk holding a zero weight computes global_min over
// all chunks holding one and writes it over its zero weights.
__global__ void fix_zeros_kernel(double* __restrict__ w_out, int64_t n, int k, int64_t chunk_rows, int64_t nchunks,
                                 const unsigned* __restrict__ chunk_min, const int* __restrict__ chunk_zero) {
  const int64_t c = blockIdx.x;
  if (!chunk_zero[c]) return;
  __shared__ float red[256];
  float m = 1.f;
  for (int64_t i = threadIdx.x; i < nchunks; i += blockDim.x)
    if (chunk_zero[i]) m = fminf(m, __uint_as_float(chunk_min[i]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fminf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  const double g = double(red[0]);
  const int64_t a = c * chunk_rows * k, b = min(n, (c + 1) * chunk_rows) * int64_t(k);
  for (int64_t e = a + threadIdx.x; e < b; e += blockDim.x)
    if (w_out[e] == 0.0) w_out[e] = g;
}

size_t smooth_smem(int k) { return sizeof(float) * (size_t(kRowsPerCta) * size_t(k | 1) + 2 * kRowsPerCta); }

// the three launches of one smoothing call over the chunk scratch given
int launch_smooth(const int64_t* knn_idx, const float* knn_dist, int64_t n, int k, double lc, double bw,
                  int64_t chunk_rows, int64_t nchunks, int64_t* edges_out, double* w_out, double* csum,
                  unsigned* cmin, int* czero, sg_handle* h, cudaStream_t st) {
  chunk_stats_kernel<<<unsigned(nchunks), 256, 0, st>>>(knn_dist, n, k, chunk_rows, csum, cmin, czero);
  SG_LAUNCH_CHECK();
  const double target = log2(double(k)) * bw;
  const size_t smem = smooth_smem(k);
  SG_CUDA(cudaFuncSetAttribute(smooth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  sg::ProfScope prof(h, "smooth", st);
  smooth_kernel<<<sg::ceil_div_i(n, kRowsPerCta), kRowsPerCta, smem, st>>>(
      knn_idx, knn_dist, n, k, lc, target, chunk_rows, csum, edges_out,
      (reinterpret_cast<uintptr_t>(edges_out) & 15u) == 0, w_out, cmin, czero);
  SG_LAUNCH_CHECK();
  fix_zeros_kernel<<<unsigned(nchunks), 256, 0, st>>>(w_out, n, k, chunk_rows, nchunks, cmin, czero);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

// rows * k * 24 bytes of output must stay far from int64 overflow
constexpr int64_t kMaxSmoothRows = int64_t(1) << 40;

}  // namespace

extern "C" int sg_smooth(sg_handle* h, const int64_t* knn_idx, const float* knn_dist, int64_t n, int32_t k,
                         double local_connectivity, double bandwidth, int64_t chunk_rows, int64_t* edges_out,
                         double* w_out, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(knn_idx && knn_dist && edges_out && w_out, "sg_smooth: null pointer argument");
  SG_ARG(n >= 0 && n < kMaxSmoothRows, "sg_smooth: n=%lld outside [0, 2^40)", (long long)n);
  SG_ARG(k >= 1 && k <= kMaxK, "sg_smooth: k=%d outside [1, %d]", k, kMaxK);
  SG_ARG(chunk_rows >= 1, "sg_smooth: chunk_rows must be >= 1");
  if (n == 0) return SG_OK;
  const int64_t nchunks = sg::ceil_div(n, chunk_rows);
  SG_ARG(nchunks < (int64_t(1) << 31), "sg_smooth: too many chunks");
  const size_t need = sg::Carver::need(sizeof(double) * nchunks) + 2 * sg::Carver::need(sizeof(unsigned) * nchunks);
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  double* csum = cv.take<double>(nchunks);
  unsigned* cmin = cv.take<unsigned>(nchunks);
  int* czero = cv.take<int>(nchunks);
  return launch_smooth(knn_idx, knn_dist, n, k, local_connectivity, bandwidth, chunk_rows, nchunks, edges_out, w_out,
                       csum, cmin, czero, h, st);
}

// ---------------------------------------------------------------------------
// Smoothing without any device allocation.
//
// Some callers cannot let a library allocate device memory: a host that owns
// the whole HBM budget through its own pool (a serving process sized to the
// last byte), code that must not take cudaMalloc's implicit device-wide
// synchronisation in a latency-critical loop, or a plugin host that forbids
// allocations outside its allocator. For them, sg_smooth_noalloc does what
// sg_smooth does with its scratch -- three words per chunk of rows -- held in
// a fixed array that belongs to this file (static device memory, reserved on
// every GPU that loads the library until the process exits): at most
// kNoallocMaxChunks = 2^14 chunks per call, 256 KB per GPU.
namespace {

constexpr int64_t kNoallocMaxChunks = int64_t(1) << 14;
constexpr size_t kNoallocSum = sizeof(double) * size_t(kNoallocMaxChunks);
constexpr size_t kNoallocU32 = sizeof(unsigned) * size_t(kNoallocMaxChunks);
constexpr size_t kNoallocBytes = kNoallocSum + 2 * kNoallocU32;

static __device__ __align__(256) unsigned char g_smooth_scratch[kNoallocBytes];

// Device address of g_smooth_scratch per device, looked up on first use with
// that device current, and again whenever the current context differs from
// the one it was looked up in (a context made by cuCtxCreate, say).
struct NoallocSlot {
  CUcontext ctx;
  void* addr;
};
std::mutex g_noalloc_mu;
NoallocSlot g_noalloc[64] = {};

CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    return static_cast<PFN_cuCtxGetCurrent_v4000>(nullptr);
  }();
  CUcontext c = nullptr;
  if (fn) fn(&c);
  return c;
}

}  // namespace

extern "C" int sg_smooth_noalloc(const int64_t* knn_idx, const float* knn_dist, int64_t n, int32_t k,
                                 double local_connectivity, double bandwidth, int64_t chunk_rows,
                                 int64_t* edges_out, double* w_out, void* stream) {
  sg::clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(knn_idx && knn_dist && edges_out && w_out, "sg_smooth_noalloc: null pointer argument");
  SG_ARG(n >= 0 && n < kMaxSmoothRows, "sg_smooth_noalloc: n=%lld outside [0, 2^40)", (long long)n);
  SG_ARG(k >= 1 && k <= kMaxK, "sg_smooth_noalloc: k=%d outside [1, %d]", k, kMaxK);
  SG_ARG(chunk_rows >= 1, "sg_smooth_noalloc: chunk_rows must be >= 1");
  if (n == 0) return SG_OK;
  const int64_t nchunks = sg::ceil_div(n, chunk_rows);
  SG_ARG(nchunks <= kNoallocMaxChunks,
         "sg_smooth_noalloc: %lld chunks exceed the fixed scratch limit of %lld; use larger chunk_rows or sg_smooth",
         (long long)nchunks, (long long)kNoallocMaxChunks);
  int dev = 0;
  SG_CUDA(cudaGetDevice(&dev));
  SG_ARG(dev >= 0 && dev < 64, "sg_smooth_noalloc: device ordinal %d not supported", dev);
  char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    // cudaGetSymbolAddress also makes the runtime's context current on this
    // thread, so the context is read after it
    if (!g_noalloc[dev].addr || g_noalloc[dev].ctx != current_context()) {
      void* p = nullptr;
      SG_CUDA(cudaGetSymbolAddress(&p, g_smooth_scratch));
      g_noalloc[dev] = {current_context(), p};
    }
    base = static_cast<char*>(g_noalloc[dev].addr);
  }
  double* csum = reinterpret_cast<double*>(base);
  unsigned* cmin = reinterpret_cast<unsigned*>(base + kNoallocSum);
  int* czero = reinterpret_cast<int*>(base + kNoallocSum + kNoallocU32);
  // the previous call's contents stay in the array: chunk_stats_kernel
  // rewrites every chunk's sum, flag and minimum before anything reads them
  return launch_smooth(knn_idx, knn_dist, n, k, local_connectivity, bandwidth, chunk_rows, nchunks, edges_out, w_out,
                       csum, cmin, czero, nullptr, st);
}
