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

__global__ void umap_init_kernel(const float* __restrict__ eps, int64_t ne, float rate, float* __restrict__ next,
                                 float* __restrict__ next_neg, float* __restrict__ eps_neg) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= ne) return;
  next[i] = eps[i];
  eps_neg[i] = eps[i] / rate;
  next_neg[i] = eps_neg[i];
}

__global__ void umap_epoch_kernel(float* __restrict__ y, int dim, const int32_t* __restrict__ head,
                                  const int32_t* __restrict__ tail, const float* __restrict__ eps,
                                  float* __restrict__ next, float* __restrict__ next_neg,
                                  const float* __restrict__ eps_neg, int64_t ne, int64_t nv, int epoch, float a,
                                  float b, float gamma, float alpha, uint64_t seed) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < ne; i += int64_t(gridDim.x) * blockDim.x) {
    if (eps[i] <= 0.f || next[i] > float(epoch)) continue;  // edges of weight 0 never sample
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
    const int nneg = int((float(epoch) - next_neg[i]) / eps_neg[i]);
    for (int p = 0; p < nneg; ++p) {
      const int64_t kk = int64_t(ul_hash(seed, uint64_t(epoch), uint64_t(i), uint64_t(p)) % uint64_t(nv));
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
    next_neg[i] += float(nneg) * eps_neg[i];
  }
}

}  // namespace

extern "C" int sg_umap_layout(sg_handle* h, const int32_t* head, const int32_t* tail, const float* epochs_per_sample,
                              int64_t n_edges, int64_t n_vertices, int32_t dim, float* embedding, int32_t n_epochs,
                              float a, float b, float gamma, float initial_alpha, float negative_sample_rate,
                              uint64_t seed, void* stream) {
  SG_HANDLE_CHECK(h);
  SG_ARG(head && tail && epochs_per_sample && embedding, "sg_umap_layout: null pointer argument");
  SG_ARG(n_edges >= 0 && n_vertices >= 1, "sg_umap_layout: bad sizes");
  SG_ARG(dim >= 1 && dim <= kUmapMaxDim, "sg_umap_layout: dim=%d outside [1, %d]", dim, kUmapMaxDim);
  SG_ARG(n_epochs >= 1 && negative_sample_rate > 0.f, "sg_umap_layout: need n_epochs >= 1 and a positive rate");
  if (n_edges == 0) return SG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* buf = nullptr;
  const size_t need = 3 * sg::Carver::need(sizeof(float) * size_t(n_edges));
  SG_CUDA(cudaMallocAsync(&buf, need, st));
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{buf, st};
  sg::Carver cv(buf);
  float* next = cv.take<float>(size_t(n_edges));
  float* next_neg = cv.take<float>(size_t(n_edges));
  float* eps_neg = cv.take<float>(size_t(n_edges));
  sg::ProfScope prof(h, "umap_layout", st);
  umap_init_kernel<<<sg::ceil_div_i(n_edges, 256), 256, 0, st>>>(epochs_per_sample, n_edges, negative_sample_rate,
                                                                 next, next_neg, eps_neg);
  SG_LAUNCH_CHECK();
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
