// Shared definitions of the scarf_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstddef>
#include <limits>
#include <vector>

#include "../../include/scarf_gb300.h"

struct sg_handle {
  int device = 0;
  int sm_count = 0;
  size_t smem_optin = 0;
  size_t budget = 0;         // 0 = unlimited
  void* ws = nullptr;        // scratch arena, grown on demand
  size_t ws_bytes = 0;
  void* solver = nullptr;    // cusolverDnHandle_t, created on first use
  void* blas = nullptr;      // cublasHandle_t, created on first use
  void* solver_work = nullptr;
  size_t solver_work_bytes = 0;
  // max relative FP64 residual of the last sg_pca_basis_filter call
  // (NaN: it used the dense route; infinity: it fell back to it)
  double eig_resid = std::numeric_limits<double>::quiet_NaN();
  // kNN split autotuning (off unless sg_set_autotune(h, 1)): the chosen split
  // count per (log2 query rows, log2 reference rows, d, list length) bucket
  bool autotune = false;
  struct KnnTune {
    int qb, rb, d, kc, nsplit, loc;
    bool self;
  };
  std::vector<KnnTune> knn_tune;
  int last_knn_splits = 0;
  int last_knn_locality = 0;
  // bounded-wait test hooks (sg_set_wait_limit, sg_test_idle_mma): the poll
  // limit of the tensor-core kernels' mbarrier waits (0 = the default), and a
  // one-shot switch that keeps the next precision kNN's MMA issuer idle
  uint32_t wait_limit = 0;
  bool idle_mma_once = false;
  // kernel timing (off unless sg_profile(h, 1)): events around named launches
  bool prof = false;
  struct ProfRec {
    const char* name;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof_pending;
  struct ProfSum {
    const char* name;
    double ms;
    int64_t count;
  };
  std::vector<ProfSum> prof_done;
};

namespace sg {

int fail(int status, const char* fmt, ...);
void count_launch();

// Times the launches issued on `st` while in scope when the handle profiles.
struct ProfScope {
  sg_handle* h;
  const char* name;
  cudaStream_t st;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(sg_handle* h_, const char* n, cudaStream_t s) : h(h_), name(n), st(s) {
    if (h && h->prof && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
      cudaEventRecord(a, st);
  }
  ~ProfScope() {
    if (a && b) {
      cudaEventRecord(b, st);
      h->prof_pending.push_back({name, a, b});
    }
  }
};
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void clear_error();

// Scratch of at least `bytes`, 256-byte aligned; grows the arena (after a
// device synchronisation) when needed. nullptr on failure with the error set.
void* ws_get(sg_handle* h, size_t bytes, int* status);

// Carves consecutive 256-byte-aligned pieces out of one scratch block.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base(static_cast<char*>(b)) {}
  template <class T>
  T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base + off);
    off += (count * sizeof(T) + 255) & ~size_t(255);
    return p;
  }
  static size_t need(size_t bytes) { return (bytes + 255) & ~size_t(255); }
};

inline int ceil_div_i(int64_t a, int64_t b) { return int((a + b - 1) / b); }
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace sg

#define SG_ARG(cond, ...)                                   \
  do {                                                      \
    if (!(cond)) return sg::fail(SG_ERR_ARG, __VA_ARGS__);  \
  } while (0)

#define SG_CUDA(call)                                                   \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return sg::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define SG_LAUNCH_CHECK()  \
  do {                     \
    SG_CUDA(cudaGetLastError()); \
    sg::count_launch();    \
  } while (0)

#define SG_HANDLE_CHECK(h)                                            \
  do {                                                                \
    if (!(h)) return sg::fail(SG_ERR_ARG, "null sg_handle");          \
    sg::clear_error();                                                \
    SG_CUDA(cudaSetDevice((h)->device));                              \
  } while (0)

// ---- device helpers --------------------------------------------------------
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}
