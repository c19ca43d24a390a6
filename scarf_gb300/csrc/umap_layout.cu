// f3: the UMAP layout scarf runs on the fused graph (scarf/umap.py:41-115,
// simplicial_set_embedding -> umap-learn optimize_layout_euclidean with
// move_other=True, densMAP off). Restated from umap-learn's published
// algorithm (umap/layouts.py, 0.5 line):
//
//   every epoch n, every edge i with epoch_of_next_sample[i] <= n:
//     attraction   coefficient -2ab d^(2(b-1)) / (a d^(2b) + 1) on d = |y_j - y_k|^2
//                  (0 when d = 0), per coordinate clipped to [-4, 4], applied
//                  to y_j (+) and y_k (-), scaled by alpha
//     repulsion    int((n - next_negative[i]) / (epochs_per_sample[i] / rate))
//                  random vertices k': coefficient 2 gamma b / ((0.001 + d)
//                  (a d^b + 1)), clipped, on y_j only (4 per coordinate when
//                  d = 0 and k' != j, nothing when k' = j)
//   alpha = initial_alpha * (1 - n / n_epochs) after epoch n.
// The 4-per-coordinate push of a negative sample that sits exactly on the
// head vertex is the else branch of the 0.5 line's repulsion loop; scarf's
// requirements leave umap-learn unpinned, and a release that sets that
// step to 0 differs only for coincident points.
//
// One thread per edge and epoch, all edges of an epoch concurrently. Each
// thread follows its own copy of the head vertex through the edge's updates
// (as the sequential loop does) and adds every step to the embedding with an
// atomic add, so concurrent updates of a vertex accumulate instead of
// overwriting one another; reads of other vertices may be stale, as in
// umap-learn's parallel mode. The layout is a sample of the same stochastic
// process, not the sequential run's exact trajectory. Negative samples come
// from a counter hash of the seed, the epoch, the edge and the sample number.
#include "common.cuh"

namespace {

constexpr int kUmapMaxDim = 8;

// SplitMix64's output function of seed + v * golden ratio
__device__ __forceinline__ uint64_t ul_mix(uint64_t seed, uint64_t v) {
  uint64_t z = seed + v * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// the draw of sample p of edge i in epoch n: one mixing round per input, so
// no two (epoch, edge, sample) triples share a key
__device__ __forceinline__ uint64_t ul_hash(uint64_t seed, uint64_t epoch, uint64_t edge, uint64_t p) {
  return ul_mix(ul_mix(ul_mix(seed, epoch), edge), p);
}

__device__ __forceinline__ float clip4(float v) { return fminf(4.f, fmaxf(-4.f, v)); }

__global__ void umap_init_kernel(const double* __restrict__ eps, int64_t ne, double rate, double* __restrict__ next,
                                 double* __restrict__ next_neg, double* __restrict__ eps_neg) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= ne) return;
  next[i] = eps[i];
  eps_neg[i] = eps[i] / rate;
  next_neg[i] = eps_neg[i];
}

// the negative sample p of edge i in epoch n
__device__ __forceinline__ int64_t neg_vertex(uint64_t seed, int epoch, int64_t i, int p, int64_t nv) {
  return int64_t(ul_hash(seed, uint64_t(epoch), uint64_t(i), uint64_t(p)) % uint64_t(nv));
}

__global__ void umap_epoch_kernel(float* __restrict__ y, int dim, const int32_t* __restrict__ head,
                                  const int32_t* __restrict__ tail, const double* __restrict__ eps,
                                  double* __restrict__ next, double* __restrict__ next_neg,
                                  const double* __restrict__ eps_neg, int64_t ne, int64_t nv, int epoch, float a,
                                  float b, float gamma, float alpha, uint64_t seed) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < ne; i += int64_t(gridDim.x) * blockDim.x) {
    if (eps[i] <= 0.0 || next[i] > double(epoch)) continue;  // edges of weight 0 never sample
    const int64_t j = head[i], k = tail[i];
    float* yj = y + j * dim;
    float* yk = y + k * dim;
    float cur[kUmapMaxDim];
    float d2 = 0.f;
    for (int d = 0; d < dim; ++d) {
      cur[d] = yj[d];
      const float t = cur[d] - yk[d];
      d2 += t * t;
    }
    float gc = 0.f;
    if (d2 > 0.f) gc = -2.f * a * b * powf(d2, b - 1.f) / (a * powf(d2, b) + 1.f);
    for (int d = 0; d < dim; ++d) {
      const float g = clip4(gc * (cur[d] - yk[d]));
      cur[d] += g * alpha;
      atomicAdd(&yj[d], g * alpha);
      atomicAdd(&yk[d], -g * alpha);
    }
    next[i] += eps[i];
    const int nneg = int((double(epoch) - next_neg[i]) / eps_neg[i]);
    for (int p = 0; p < nneg; ++p) {
      const int64_t kk = neg_vertex(seed, epoch, i, p, nv);
      const float* yo = y + kk * dim;
      float e2 = 0.f;
      for (int d = 0; d < dim; ++d) {
        const float t = cur[d] - yo[d];
        e2 += t * t;
      }
      float rc;
      if (e2 > 0.f) rc = 2.f * gamma * b / ((0.001f + e2) * (a * powf(e2, b) + 1.f));
      else if (j == kk) continue;
      else rc = 0.f;
      for (int d = 0; d < dim; ++d) {
        const float g = rc > 0.f ? clip4(rc * (cur[d] - yo[d])) : 4.f;
        cur[d] += g * alpha;
        atomicAdd(&yj[d], g * alpha);
      }
    }
    next_neg[i] += double(nneg) * eps_neg[i];
  }
}

// The deterministic mode: one thread runs umap-learn's sequential loop
// (edges in order, every update applied at once, move_other=True) with the
// arithmetic of its numba code -- float32 coordinates and differences,
// float64 squared distances, gradient coefficients, alpha and sampling
// schedule -- and the same negative-sample draws as the parallel mode. For
// small graphs: it is the reference trajectory that the parallel mode is a
// concurrent sample of.
__device__ __forceinline__ double sq_dist64(const float* u, const float* v, int dim) {
  double r = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double t = double(__fsub_rn(u[d], v[d]));
    r = __dadd_rn(r, __dmul_rn(t, t));
  }
  return r;
}

__global__ void umap_sequential_kernel(float* __restrict__ y, int dim, const int32_t* __restrict__ head,
                                       const int32_t* __restrict__ tail, const double* __restrict__ eps,
                                       double* __restrict__ next, double* __restrict__ next_neg,
                                       const double* __restrict__ eps_neg, int64_t ne, int64_t nv, int n_epochs,
                                       double a, double b, double gamma, double initial_alpha, uint64_t seed) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  auto clip = [](double v) { return v > 4.0 ? 4.0 : (v < -4.0 ? -4.0 : v); };
  double alpha = initial_alpha;
  for (int n = 0; n < n_epochs; ++n) {
    for (int64_t i = 0; i < ne; ++i) {
      if (eps[i] <= 0.0 || next[i] > double(n)) continue;
      const int64_t j = head[i], k = tail[i];
      float* cur = y + j * dim;
      float* oth = y + k * dim;
      const double d2 = sq_dist64(cur, oth, dim);
      double gc = 0.0;
      if (d2 > 0.0) gc = -2.0 * a * b * pow(d2, b - 1.0) / (a * pow(d2, b) + 1.0);
      for (int d = 0; d < dim; ++d) {
        const double g = clip(__dmul_rn(gc, double(__fsub_rn(cur[d], oth[d]))));
        cur[d] = float(__dadd_rn(double(cur[d]), __dmul_rn(g, alpha)));
        oth[d] = float(__dadd_rn(double(oth[d]), __dmul_rn(-g, alpha)));
      }
      next[i] += eps[i];
      const int nneg = int((double(n) - next_neg[i]) / eps_neg[i]);
      for (int p = 0; p < nneg; ++p) {
        const int64_t kk = neg_vertex(seed, n, i, p, nv);
        const float* o = y + kk * dim;
        const double e2 = sq_dist64(cur, o, dim);
        double rc;
        if (e2 > 0.0) rc = 2.0 * gamma * b / ((0.001 + e2) * (a * pow(e2, b) + 1.0));
        else if (j == kk) continue;
        else rc = 0.0;
        for (int d = 0; d < dim; ++d) {
          const double g = rc > 0.0 ? clip(__dmul_rn(rc, double(__fsub_rn(cur[d], o[d])))) : 4.0;
          cur[d] = float(__dadd_rn(double(cur[d]), __dmul_rn(g, alpha)));
        }
      }
      next_neg[i] += double(nneg) * eps_neg[i];
    }
    alpha = initial_alpha * (1.0 - double(n) / double(n_epochs));
  }
}

}  // namespace

extern "C" int sg_umap_layout(sg_handle* h, const int32_t* head, const int32_t* tail,
                              const double* epochs_per_sample, int64_t n_edges, int64_t n_vertices, int32_t dim,
                              float* embedding, int32_t n_epochs, float a, float b, float gamma, float initial_alpha,
                              float negative_sample_rate, uint64_t seed, int32_t sequential, void* stream) {
  SG_HANDLE_CHECK(h);
  SG_ARG(head && tail && epochs_per_sample && embedding, "sg_umap_layout: null pointer argument");
  SG_ARG(n_edges >= 0 && n_vertices >= 1, "sg_umap_layout: bad sizes");
  SG_ARG(dim >= 1 && dim <= kUmapMaxDim, "sg_umap_layout: dim=%d outside [1, %d]", dim, kUmapMaxDim);
  SG_ARG(n_epochs >= 1 && negative_sample_rate > 0.f, "sg_umap_layout: need n_epochs >= 1 and a positive rate");
  if (n_edges == 0) return SG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* buf = nullptr;
  const size_t need = 3 * sg::Carver::need(sizeof(double) * size_t(n_edges));
  SG_CUDA(cudaMallocAsync(&buf, need, st));
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{buf, st};
  sg::Carver cv(buf);
  double* next = cv.take<double>(size_t(n_edges));
  double* next_neg = cv.take<double>(size_t(n_edges));
  double* eps_neg = cv.take<double>(size_t(n_edges));
  sg::ProfScope prof(h, "umap_layout", st);
  umap_init_kernel<<<sg::ceil_div_i(n_edges, 256), 256, 0, st>>>(epochs_per_sample, n_edges,
                                                                 double(negative_sample_rate), next, next_neg,
                                                                 eps_neg);
  SG_LAUNCH_CHECK();
  if (sequential) {
    umap_sequential_kernel<<<1, 1, 0, st>>>(embedding, dim, head, tail, epochs_per_sample, next, next_neg, eps_neg,
                                            n_edges, n_vertices, n_epochs, double(a), double(b), double(gamma),
                                            double(initial_alpha), seed);
    SG_LAUNCH_CHECK();
    return SG_OK;
  }
  const unsigned grid = unsigned(std::min<int64_t>(sg::ceil_div(n_edges, 256), int64_t(h->sm_count) * 16));
  float alpha = initial_alpha;
  for (int n = 0; n < n_epochs; ++n) {
    umap_epoch_kernel<<<grid, 256, 0, st>>>(embedding, dim, head, tail, epochs_per_sample, next, next_neg, eps_neg,
                                            n_edges, n_vertices, n, a, b, gamma, alpha, seed);
    SG_LAUNCH_CHECK();
    alpha = initial_alpha * (1.f - float(n) / float(n_epochs));
  }
  return SG_OK;
}
