// Handle, error and scratch management of the C ABI.
#include "common.cuh"

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

namespace {
thread_local char g_err[1024] = {0};
std::atomic<unsigned long long> g_launches{0};

void prof_drain(sg_handle* h) {
  for (auto& r : h->prof_pending) {
    float ms = 0.f;
    cudaEventSynchronize(r.b);
    cudaEventElapsedTime(&ms, r.a, r.b);
    bool found = false;
    for (auto& s : h->prof_done)
      if (strcmp(s.name, r.name) == 0) {
        s.ms += ms;
        s.count += 1;
        found = true;
      }
    if (!found) h->prof_done.push_back({r.name, double(ms), 1});
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  h->prof_pending.clear();
}
}  // namespace

namespace sg {

void clear_error() { g_err[0] = 0; }

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int fail(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  const char* base = strrchr(file, '/');
  int st = (e == cudaErrorMemoryAllocation) ? SG_ERR_OOM : SG_ERR_CUDA;
  snprintf(g_err, sizeof(g_err), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e),
           base ? base + 1 : file, line);
  return st;
}

void* ws_get(sg_handle* h, size_t bytes, int* status) {
  *status = SG_OK;
  if (bytes == 0) bytes = 256;
  if (h->ws && h->ws_bytes >= bytes) return h->ws;
  size_t want = bytes + bytes / 8;  // headroom against regrowth
  if (h->budget && want > h->budget) want = bytes;
  if (h->budget && bytes > h->budget) {
    *status = fail(SG_ERR_BUDGET, "scratch of %zu bytes exceeds the handle's HBM budget of %zu bytes",
                   bytes, h->budget);
    return nullptr;
  }
  if (h->ws) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      *status = cuda_fail(e, "cudaDeviceSynchronize", __FILE__, __LINE__);
      return nullptr;
    }
    cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *status = fail(SG_ERR_OOM, "cudaMalloc of %zu scratch bytes failed: %s", want, cudaGetErrorString(e));
    return nullptr;
  }
  h->ws = p;
  h->ws_bytes = want;
  return p;
}

}  // namespace sg

void sg_solver_destroy(sg_handle* h);  // pca.cu

extern "C" {

int sg_version(void) { return 1; }

const char* sg_last_error(void) { return g_err; }

int sg_create(int device, size_t hbm_budget_bytes, sg_handle** out) {
  sg::clear_error();
  if (!out) return sg::fail(SG_ERR_ARG, "sg_create: null output pointer");
  *out = nullptr;
  int ndev = 0;
  SG_CUDA(cudaGetDeviceCount(&ndev));
  SG_ARG(device >= 0 && device < ndev, "sg_create: device %d out of range (%d devices)", device, ndev);
  SG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SG_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return sg::fail(SG_ERR_UNSUPPORTED, "sg_create: device %d is sm_%d%d; this library is built for sm_103a (GB300)",
                    device, prop.major, prop.minor);
  sg_handle* h = new sg_handle();
  h->device = device;
  h->sm_count = prop.multiProcessorCount;
  h->smem_optin = prop.sharedMemPerBlockOptin;
  h->budget = hbm_budget_bytes;
  *out = h;
  return SG_OK;
}

int sg_destroy(sg_handle* h) {
  if (!h) return SG_OK;
  cudaSetDevice(h->device);
  prof_drain(h);
  sg_solver_destroy(h);
  if (h->ws) cudaFree(h->ws);
  delete h;
  return SG_OK;
}

size_t sg_workspace_bytes(const sg_handle* h) { return h ? h->ws_bytes : 0; }

unsigned long long sg_kernel_launches(void) { return g_launches.load(); }

int sg_set_autotune(sg_handle* h, int enable) {
  if (!h) return sg::fail(SG_ERR_ARG, "null sg_handle");
  h->autotune = enable != 0;
  return SG_OK;
}

int sg_knn_last_splits(const sg_handle* h) { return h ? h->last_knn_splits : 0; }

int sg_knn_last_locality(const sg_handle* h) { return h ? h->last_knn_locality : 0; }

int sg_set_wait_limit(sg_handle* h, uint32_t polls) {
  if (!h) return sg::fail(SG_ERR_ARG, "null sg_handle");
  h->wait_limit = polls;
  return SG_OK;
}

int sg_test_idle_mma(sg_handle* h) {
  if (!h) return sg::fail(SG_ERR_ARG, "null sg_handle");
  h->idle_mma_once = true;
  return SG_OK;
}

int sg_profile(sg_handle* h, int enable) {
  if (!h) return sg::fail(SG_ERR_ARG, "null sg_handle");
  cudaSetDevice(h->device);
  prof_drain(h);
  h->prof = enable != 0;
  return SG_OK;
}

int sg_profile_reset(sg_handle* h) {
  if (!h) return sg::fail(SG_ERR_ARG, "null sg_handle");
  cudaSetDevice(h->device);
  prof_drain(h);
  h->prof_done.clear();
  return SG_OK;
}

int sg_profile_query(sg_handle* h, const char* name, double* total_ms, long long* count) {
  if (!h || !name || !total_ms || !count) return sg::fail(SG_ERR_ARG, "sg_profile_query: null argument");
  cudaSetDevice(h->device);
  prof_drain(h);
  *total_ms = 0.0;
  *count = 0;
  for (auto& s : h->prof_done)
    if (strcmp(s.name, name) == 0) {
      *total_ms = s.ms;
      *count = s.count;
    }
  return SG_OK;
}

}  // extern "C"
