// a8: smoothen_dists (scarf/knn_utils.py:89-159) over the published
// umap-learn smooth_knn_dist / compute_membership_strengths, in float32 with
// the per-row operation order of those numba loops.
//
// Kernel 1: one thread per row (rows staged through shared memory with
// coalesced loads): rho, sigma by 64-step bisection on
// sum_{j>=1} exp(-max(0, d_j - rho)/sigma) = log2(k)*bandwidth, the sigma
// floor, then the k weights. Per chunk of `chunk_rows` rows it records whether
// a weight is zero and the smallest non-zero weight (atomicMin on the float
// bits; positive floats order like their bit patterns).
// Kernel 2: global_min = min(1, chunk minima of chunks holding a zero); the
// zero weights of those chunks are replaced.
// A chunk-mean pre-pass supplies the floor of rows whose rho is 0.
#include "common.cuh"

#include <mutex>

namespace {

constexpr int kRowsPerCta = 128;
constexpr int kMaxK = 128;

__global__ void chunk_sum_kernel(const float* __restrict__ dist, int64_t n, int k, int64_t chunk_rows,
                                 double* __restrict__ chunk_sum) {
  // one CTA per chunk
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
  if (threadIdx.x == 0) chunk_sum[c] = red[0];
}

__global__ void __launch_bounds__(kRowsPerCta)
smooth_kernel(const int64_t* __restrict__ idx, const float* __restrict__ dist, int64_t n, int k, double lc,
              double target, int64_t chunk_rows, const double* __restrict__ chunk_sum, int64_t* __restrict__ edges,
              double* __restrict__ w_out, float* __restrict__ w32, unsigned* __restrict__ chunk_min,
              int* __restrict__ chunk_zero) {
  extern __shared__ float sd[];  // kRowsPerCta * (k + 1)
  const int pitch = k + 1;
  const int64_t r0 = int64_t(blockIdx.x) * kRowsPerCta;
  const int nrows = int(min(int64_t(kRowsPerCta), n - r0));
  for (int e = threadIdx.x; e < nrows * k; e += blockDim.x) {
    const int rr = e / k, j = e % k;
    sd[rr * pitch + j] = dist[(r0 + rr) * k + j];
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t >= nrows) return;
  const int64_t row = r0 + t;
  const float* d = sd + t * pitch;
  const float inf = __int_as_float(0x7f800000);

  // rho (smooth_knn_dist): the local_connectivity-th non-zero distance
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

  // sigma: bisection with float32 lo/hi/mid/psum (the sum skips column 0)
  float lo = 0.f, hi = inf, mid = 1.f;
  for (int it = 0; it < 64; ++it) {
    float psum = 0.f;
    for (int j = 1; j < k; ++j) {
      const float dd = d[j] - rho;
      psum += dd > 0.f ? expf(-__fdiv_rn(dd, mid)) : 1.f;
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

  // weights (compute_membership_strengths); the self test uses the
  // chunk-local row number, as the reference passes global neighbour indices
  const int64_t local = row - chunk * chunk_rows;
  bool any_zero = false;
  unsigned mn = 0x7f800000u;
  for (int j = 0; j < k; ++j) {
    const int64_t nb = idx[row * k + j];
    float v;
    if (nb == local) {
      v = 0.f;
    } else if (d[j] - rho <= 0.f || sigma == 0.f) {
      v = 1.f;
    } else {
      v = expf(-__fdiv_rn(d[j] - rho, sigma));
    }
    const int64_t e = row * k + j;
    edges[2 * e] = row;
    edges[2 * e + 1] = nb;
    w32[e] = v;
    w_out[e] = double(v);
    if (v == 0.f) any_zero = true;
    else mn = min(mn, __float_as_uint(v));
  }
  if (any_zero) atomicOr(&chunk_zero[chunk], 1);
  atomicMin(&chunk_min[chunk], mn);
}

__global__ void init_chunks_kernel(unsigned* __restrict__ chunk_min, int* __restrict__ chunk_zero, int64_t nchunks) {
  const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c < nchunks) {
    chunk_min[c] = 0x7f800000u;
    chunk_zero[c] = 0;
  }
}

// global_min over chunks (one CTA), then the zero weights of flagged chunks
__global__ void global_min_kernel(const unsigned* __restrict__ chunk_min, const int* __restrict__ chunk_zero,
                                  int64_t nchunks, float* __restrict__ gmin) {
  __shared__ float red[256];
  float m = 1.f;
  for (int64_t c = threadIdx.x; c < nchunks; c += blockDim.x)
    if (chunk_zero[c]) m = fminf(m, __uint_as_float(chunk_min[c]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fminf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *gmin = red[0];
}

__global__ void fix_zeros_kernel(const float* __restrict__ w32, double* __restrict__ w_out, int64_t n, int k,
                                 int64_t chunk_rows, const int* __restrict__ chunk_zero,
                                 const float* __restrict__ gmin) {
  const int64_t c = blockIdx.x;
  if (!chunk_zero[c]) return;
  const int64_t a = c * chunk_rows * k, b = min(n, (c + 1) * chunk_rows) * int64_t(k);
  const double g = double(*gmin);
  for (int64_t e = a + threadIdx.x; e < b; e += blockDim.x)
    if (w32[e] == 0.f) w_out[e] = g;
}

}  // namespace

extern "C" int sg_smooth(sg_handle* h, const int64_t* knn_idx, const float* knn_dist, int64_t n, int32_t k,
                         double local_connectivity, double bandwidth, int64_t chunk_rows, int64_t* edges_out,
                         double* w_out, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(knn_idx && knn_dist && edges_out && w_out, "sg_smooth: null pointer argument");
  SG_ARG(n >= 0 && k >= 1 && k <= kMaxK, "sg_smooth: k=%d outside [1, %d]", k, kMaxK);
  SG_ARG(chunk_rows >= 1, "sg_smooth: chunk_rows must be >= 1");
  if (n == 0) return SG_OK;
  const int64_t nchunks = sg::ceil_div(n, chunk_rows);
  const size_t need = sg::Carver::need(sizeof(float) * size_t(n) * k) + sg::Carver::need(sizeof(double) * nchunks) +
                      2 * sg::Carver::need(sizeof(unsigned) * nchunks) + 256;
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  float* w32 = cv.take<float>(size_t(n) * k);
  double* csum = cv.take<double>(nchunks);
  unsigned* cmin = cv.take<unsigned>(nchunks);
  int* czero = cv.take<int>(nchunks);
  float* gmin = cv.take<float>(1);
  SG_ARG(nchunks < (int64_t(1) << 31), "sg_smooth: too many chunks");
  init_chunks_kernel<<<sg::ceil_div_i(nchunks, 256), 256, 0, st>>>(cmin, czero, nchunks);
  SG_LAUNCH_CHECK();
  chunk_sum_kernel<<<unsigned(nchunks), 256, 0, st>>>(knn_dist, n, k, chunk_rows, csum);
  SG_LAUNCH_CHECK();
  const double target = log2(double(k)) * bandwidth;
  const size_t smem = sizeof(float) * kRowsPerCta * (k + 1);
  SG_CUDA(cudaFuncSetAttribute(smooth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  sg::ProfScope prof(h, "smooth", st);
  smooth_kernel<<<sg::ceil_div_i(n, kRowsPerCta), kRowsPerCta, smem, st>>>(
      knn_idx, knn_dist, n, k, local_connectivity, target, chunk_rows, csum, edges_out, w_out, w32, cmin,
      czero);
  SG_LAUNCH_CHECK();
  global_min_kernel<<<1, 256, 0, st>>>(cmin, czero, nchunks, gmin);
  SG_LAUNCH_CHECK();
  fix_zeros_kernel<<<unsigned(nchunks), 256, 0, st>>>(w32, w_out, n, k, chunk_rows, czero, gmin);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Smoothing without any device allocation.
//
// Some callers cannot let a library allocate device memory: a host that owns
// the whole HBM budget through its own pool (a serving process sized to the
// last byte), code that must not take cudaMalloc's implicit device-wide
// synchronisation in a latency-critical loop, or a plugin host that forbids
// allocations outside its allocator. For them, sg_smooth_noalloc does what
// sg_smooth does with its scratch held in a fixed array that belongs to this
// file (static device memory, reserved on every GPU that loads the library
// until the process exits): at most kNoallocMaxEdges = 2^21 edges (n * k) and
// kNoallocMaxChunks = 2^14 chunks per call, about 8.3 MB per GPU.
namespace {

constexpr int64_t kNoallocMaxEdges = int64_t(1) << 21;
constexpr int64_t kNoallocMaxChunks = int64_t(1) << 14;
constexpr size_t kNoallocW32 = sizeof(float) * size_t(kNoallocMaxEdges);
constexpr size_t kNoallocSum = sizeof(double) * size_t(kNoallocMaxChunks);
constexpr size_t kNoallocU32 = sizeof(unsigned) * size_t(kNoallocMaxChunks);
constexpr size_t kNoallocBytes = kNoallocW32 + kNoallocSum + 2 * kNoallocU32 + 256;

static __device__ __align__(256) unsigned char g_smooth_scratch[kNoallocBytes];

// device address of g_smooth_scratch per device, looked up on first use
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

}  // namespace

extern "C" int sg_smooth_noalloc(const int64_t* knn_idx, const float* knn_dist, int64_t n, int32_t k,
                                 double local_connectivity, double bandwidth, int64_t chunk_rows,
                                 int64_t* edges_out, double* w_out, void* stream) {
  sg::clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(knn_idx && knn_dist && edges_out && w_out, "sg_smooth_noalloc: null pointer argument");
  SG_ARG(n >= 0 && k >= 1 && k <= kMaxK, "sg_smooth_noalloc: k=%d outside [1, %d]", k, kMaxK);
  SG_ARG(chunk_rows >= 1, "sg_smooth_noalloc: chunk_rows must be >= 1");
  if (n == 0) return SG_OK;
  const int64_t nchunks = sg::ceil_div(n, chunk_rows);
  SG_ARG(n * k <= kNoallocMaxEdges,
         "sg_smooth_noalloc: %lld edges (n*k) exceed the fixed scratch limit of %lld; use sg_smooth",
         (long long)(n * k), (long long)kNoallocMaxEdges);
  SG_ARG(nchunks <= kNoallocMaxChunks,
         "sg_smooth_noalloc: %lld chunks exceed the fixed scratch limit of %lld; use larger chunk_rows or sg_smooth",
         (long long)nchunks, (long long)kNoallocMaxChunks);
  int dev = 0;
  SG_CUDA(cudaGetDevice(&dev));
  SG_ARG(dev >= 0 && dev < 64, "sg_smooth_noalloc: device ordinal %d not supported", dev);
  char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      SG_CUDA(cudaGetSymbolAddress(&p, g_smooth_scratch));
      g_noalloc_addr[dev] = p;
    }
    base = static_cast<char*>(g_noalloc_addr[dev]);
  }
  float* w32 = reinterpret_cast<float*>(base);
  double* csum = reinterpret_cast<double*>(base + kNoallocW32);
  unsigned* cmin = reinterpret_cast<unsigned*>(base + kNoallocW32 + kNoallocSum);
  int* czero = reinterpret_cast<int*>(base + kNoallocW32 + kNoallocSum + kNoallocU32);
  float* gmin = reinterpret_cast<float*>(base + kNoallocW32 + kNoallocSum + 2 * kNoallocU32);
  // the previous call's contents stay in the array: every piece read below is
  // first written in this call (chunk flags and minima by init_chunks_kernel,
  // chunk sums, float weights and the global minimum by their kernels)
  init_chunks_kernel<<<sg::ceil_div_i(nchunks, 256), 256, 0, st>>>(cmin, czero, nchunks);
  SG_LAUNCH_CHECK();
  chunk_sum_kernel<<<unsigned(nchunks), 256, 0, st>>>(knn_dist, n, k, chunk_rows, csum);
  SG_LAUNCH_CHECK();
  const double target = log2(double(k)) * bandwidth;
  const size_t smem = sizeof(float) * kRowsPerCta * (k + 1);
  SG_CUDA(cudaFuncSetAttribute(smooth_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  smooth_kernel<<<sg::ceil_div_i(n, kRowsPerCta), kRowsPerCta, smem, st>>>(
      knn_idx, knn_dist, n, k, local_connectivity, target, chunk_rows, csum, edges_out, w_out, w32, cmin,
      czero);
  SG_LAUNCH_CHECK();
  global_min_kernel<<<1, 256, 0, st>>>(cmin, czero, nchunks, gmin);
  SG_LAUNCH_CHECK();
  fix_zeros_kernel<<<unsigned(nchunks), 256, 0, st>>>(w32, w_out, n, k, chunk_rows, czero, gmin);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
