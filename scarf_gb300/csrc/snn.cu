// f4: shared-nearest-neighbour scores and the merge of kNN graphs used by
// integrate_assays (scarf/knn_utils.py:195-274: calc_snn, weight_sort_indices,
// merge_graphs).
//
//   calc_snn      snn[i][j] = |set(indices[i]) & set(indices[m])| / (k - 1),
//                 m = indices[i][j] (a negative m counts from the end, as a
//                 numba index does); one thread per (i, j), O(k^2) on the
//                 k <= 64 entries of the two rows.
//   merge_graphs  per row: the k neighbours of every graph, ordered by
//                 weight + snn, largest first (ties: the later candidate first,
//                 the reverse of a stable ascending argsort), the first
//                 occurrence of each neighbour kept, the first k of them out;
//                 one thread per row.
#include "common.cuh"

namespace {

constexpr int kSnnMaxK = 64;
constexpr int kMergeMaxGraphs = 8;
constexpr int kMergeMaxCand = 128;

__global__ void calc_snn_kernel(const int64_t* __restrict__ idx, int64_t n, int k, double* __restrict__ snn) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n * k) return;
  const int64_t i = e / k;
  const int64_t* a = idx + i * k;
  int64_t m = idx[e];
  if (m < 0) m += n;
  int cnt = 0;
  if (m >= 0 && m < n) {
    const int64_t* b = idx + m * k;
    for (int p = 0; p < k; ++p) {
      const int64_t v = a[p];
      bool dup = false;
      for (int q = 0; q < p && !dup; ++q) dup = a[q] == v;
      if (dup) continue;
      bool in_b = false;
      for (int q = 0; q < k && !in_b; ++q) in_b = b[q] == v;
      cnt += in_b ? 1 : 0;
    }
  }
  snn[e] = double(cnt) / double(k - 1);
}

struct MergeArgs {
  const int64_t* idx[kMergeMaxGraphs];
  const double* w[kMergeMaxGraphs];
  const double* snn[kMergeMaxGraphs];
};

__global__ void merge_graphs_kernel(MergeArgs g, int ng, int64_t n, int k, int64_t* __restrict__ out_idx,
                                    double* __restrict__ out_w) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = ng * k;
  int order[kMergeMaxCand];
  double wn[kMergeMaxCand];
  for (int t = 0; t < c; ++t) {
    const int gi = t / k, j = t - gi * k;
    wn[t] = g.w[gi][i * k + j] + g.snn[gi][i * k + j];
    order[t] = t;
  }
  // insertion sort: larger weight first, then the later candidate first
  for (int a = 1; a < c; ++a) {
    const int v = order[a];
    const double wv = wn[v];
    int b = a - 1;
    while (b >= 0 && (wn[order[b]] < wv || (wn[order[b]] == wv && order[b] < v))) {
      order[b + 1] = order[b];
      --b;
    }
    order[b + 1] = v;
  }
  int kept = 0;
  for (int a = 0; a < c && kept < k; ++a) {
    const int t = order[a];
    const int gi = t / k, j = t - gi * k;
    const int64_t v = g.idx[gi][i * k + j];
    bool seen = false;
    for (int q = 0; q < kept && !seen; ++q) seen = out_idx[i * k + q] == v;
    if (seen) continue;
    out_idx[i * k + kept] = v;
    out_w[i * k + kept] = g.w[gi][i * k + j];
    ++kept;
  }
  for (; kept < k; ++kept) {  // fewer than k distinct neighbours: padding the caller checks
    out_idx[i * k + kept] = -1;
    out_w[i * k + kept] = 0.0;
  }
}

}  // namespace

extern "C" int sg_calc_snn(sg_handle* h, const int64_t* indices, int64_t n, int32_t k, double* snn_out,
                           void* stream) {
  SG_HANDLE_CHECK(h);
  SG_ARG(indices && snn_out, "sg_calc_snn: null pointer argument");
  SG_ARG(n >= 1 && k >= 2 && k <= kSnnMaxK, "sg_calc_snn: need n >= 1 and 2 <= k <= %d", kSnnMaxK);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  sg::ProfScope prof(h, "calc_snn", st);
  calc_snn_kernel<<<sg::ceil_div_i(n * k, 256), 256, 0, st>>>(indices, n, k, snn_out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

extern "C" int sg_merge_graphs(sg_handle* h, int32_t n_graphs, const int64_t* const* indices, const double* const* w,
                               const double* const* snn, int64_t n, int32_t k, int64_t* out_indices, double* out_w,
                               void* stream) {
  SG_HANDLE_CHECK(h);
  SG_ARG(indices && w && snn && out_indices && out_w, "sg_merge_graphs: null pointer argument");
  SG_ARG(n_graphs >= 1 && n_graphs <= kMergeMaxGraphs, "sg_merge_graphs: n_graphs=%d outside [1, %d]", n_graphs,
         kMergeMaxGraphs);
  SG_ARG(n >= 1 && k >= 1 && int64_t(n_graphs) * k <= kMergeMaxCand,
         "sg_merge_graphs: need n >= 1 and n_graphs * k <= %d", kMergeMaxCand);
  MergeArgs g{};
  for (int t = 0; t < n_graphs; ++t) {
    SG_ARG(indices[t] && w[t] && snn[t], "sg_merge_graphs: null pointer for graph %d", t);
    g.idx[t] = indices[t];
    g.w[t] = w[t];
    g.snn[t] = snn[t];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  sg::ProfScope prof(h, "merge_graphs", st);
  merge_graphs_kernel<<<sg::ceil_div_i(n, 128), 128, 0, st>>>(g, n_graphs, n, k, out_indices, out_w);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
