// The mapping service behind the C ABI (sg_serve_*): continuous batching of
// run_mapping queries (scarf/datastore/mapping_datastore.py:198-208) over a
// device-resident reference, for hosts that are not Python.
//
// A request is a CSR block of target cells on the host (the caller keeps the
// arrays valid until the request is done). Requests are admitted by the HBM
// they would need; each worker thread (its own CUDA stream, library handle
// and device buffers) takes up to max_batch_rows rows from the pending
// requests, shortest remaining first (ties by arrival), so a large request is
// served in row slices while small ones that arrive meanwhile join the next
// batch. A batch is: the slices' CSR copied to the device, sg_normalize_csr
// onto the reference features (absent features filled with 1.0,
// scarf/mapping_utils.py:208), sg_project with the reference's mu, sigma and
// loadings, sg_knn (k neighbours, no self rule) against the reference
// scores, and the results copied back into the request's host result arrays.
// Rows are independent, so a row's result does not depend on its batch.
#include "common.cuh"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

struct Request {
  int64_t id = 0;
  const int64_t* indptr = nullptr;
  const int32_t* indices = nullptr;
  const int32_t* data = nullptr;
  int64_t n_rows = 0;
  int64_t next_row = 0;   // first row not yet handed to a batch
  int64_t rows_done = 0;
  size_t bytes = 0;       // admission cost
  bool admitted = false;
  bool done = false;
  int status = SG_OK;
  std::string error;
  std::vector<int64_t> idx;
  std::vector<float> dist;
};

struct Slice {
  std::shared_ptr<Request> r;
  int64_t a, b;  // rows [a, b)
};

// device buffers of one worker, grown on demand
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int grow(size_t want) {
    if (want <= n) return SG_OK;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    SG_CUDA(cudaMalloc(&p, want * sizeof(T)));
    n = want;
    return SG_OK;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

struct sg_server {
  int device = 0;
  // reference (caller-owned device arrays)
  const float* mu = nullptr;
  const float* sigma = nullptr;
  const float* loadings = nullptr;
  const float* ref_scores = nullptr;
  int32_t n_feats = 0, d = 0, ld_l = 0, ld_ref = 0;
  int64_t n_ref = 0;
  // query panel (server-owned device copies)
  int32_t* d_cmap = nullptr;
  uint8_t* d_missing = nullptr;
  int64_t n_genes = 0;
  int32_t k = 0, precision = 0, margin = 0, max_rows = 0;
  double size_factor = 1000.0;
  uint32_t flags = 0;
  size_t budget = 0, in_use = 0;
  size_t bytes_per_row = 0;
  // scheduling state
  std::mutex mu_;
  std::condition_variable cv;
  std::vector<std::shared_ptr<Request>> pending;  // admitted, rows left to batch
  std::vector<std::shared_ptr<Request>> queued;   // waiting for HBM budget
  std::map<int64_t, std::shared_ptr<Request>> all;
  int64_t next_id = 1;
  bool stopping = false;
  std::atomic<int64_t> batches{0}, rows{0};
  std::vector<std::thread> workers;
  std::string init_error;
  int init_status = SG_OK;
};

namespace {

size_t request_cost(const sg_server* s, const Request& r) {
  const int64_t nnz = r.n_rows ? r.indptr[r.n_rows] - r.indptr[0] : 0;
  return size_t(r.n_rows) * s->bytes_per_row + size_t(nnz) * 8;
}

// admit queued requests in arrival order while they fit the budget (lock held)
void admit(sg_server* s) {
  while (!s->queued.empty()) {
    auto& r = s->queued.front();
    if (s->in_use + r->bytes > s->budget && s->in_use > 0) break;
    s->in_use += r->bytes;
    r->admitted = true;
    s->pending.push_back(r);
    s->queued.erase(s->queued.begin());
  }
}

// up to max_rows rows from the pending requests, shortest remaining first (lock held)
std::vector<Slice> take_batch(sg_server* s) {
  std::vector<std::shared_ptr<Request>> order;
  for (auto& r : s->pending)
    if (r->next_row < r->n_rows) order.push_back(r);
  std::stable_sort(order.begin(), order.end(), [](const std::shared_ptr<Request>& a, const std::shared_ptr<Request>& b) {
    const int64_t ra = a->n_rows - a->next_row, rb = b->n_rows - b->next_row;
    return ra != rb ? ra < rb : a->id < b->id;
  });
  std::vector<Slice> batch;
  int64_t room = s->max_rows;
  for (auto& r : order) {
    if (room == 0) break;
    const int64_t take = std::min<int64_t>(room, r->n_rows - r->next_row);
    batch.push_back({r, r->next_row, r->next_row + take});
    r->next_row += take;
    room -= take;
  }
  return batch;
}

// results of a finished batch (or its error) into the requests (lock held)
void complete(sg_server* s, const std::vector<Slice>& batch, const int64_t* hidx, const float* hdist, int status,
              const char* msg) {
  int64_t off = 0;
  for (const auto& sl : batch) {
    Request& r = *sl.r;
    const int64_t n = sl.b - sl.a;
    if (status == SG_OK) {
      memcpy(r.idx.data() + sl.a * s->k, hidx + off * s->k, sizeof(int64_t) * n * s->k);
      memcpy(r.dist.data() + sl.a * s->k, hdist + off * s->k, sizeof(float) * n * s->k);
    } else if (r.status == SG_OK) {
      r.status = status;
      r.error = msg;
    }
    off += n;
    r.rows_done += n;
    if (r.rows_done == r.n_rows) {
      r.done = true;
      s->in_use -= r.bytes;
      s->pending.erase(std::remove(s->pending.begin(), s->pending.end(), sl.r), s->pending.end());
    }
  }
  admit(s);
  s->cv.notify_all();
}

void worker_main(sg_server* s) {
  cudaSetDevice(s->device);
  sg_handle* h = nullptr;
  cudaStream_t st = nullptr;
  // the admission budget governs the requests' data; the library's own
  // scratch for a batch (operand packing, candidate lists) is the handle's
  int rc = sg_create(s->device, 0, &h);
  if (rc == SG_OK && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) rc = SG_ERR_CUDA;
  if (rc != SG_OK) {
    std::lock_guard<std::mutex> lock(s->mu_);
    s->init_status = rc;
    s->init_error = sg_last_error();
    s->stopping = true;
    s->cv.notify_all();
    if (h) sg_destroy(h);
    return;
  }
  const int64_t ld = (s->n_feats + 3) / 4 * 4;
  DevBuf<int64_t> d_ip, d_idx, d_miss;
  DevBuf<int32_t> d_ind, d_dat;
  DevBuf<float> d_x, d_sc, d_dist;
  int64_t* h_ip = nullptr;
  int64_t* h_idx = nullptr;
  float* h_dist = nullptr;
  const size_t rows_cap = size_t(s->max_rows);
  bool ok = cudaMallocHost(&h_ip, sizeof(int64_t) * (rows_cap + 1)) == cudaSuccess &&
            cudaMallocHost(&h_idx, sizeof(int64_t) * rows_cap * s->k) == cudaSuccess &&
            cudaMallocHost(&h_dist, sizeof(float) * rows_cap * s->k) == cudaSuccess;
  if (ok) ok = d_ip.grow(rows_cap + 1) == SG_OK && d_x.grow(rows_cap * ld) == SG_OK &&
               d_sc.grow(rows_cap * s->ld_ref) == SG_OK && d_idx.grow(rows_cap * s->k) == SG_OK &&
               d_dist.grow(rows_cap * s->k) == SG_OK && d_miss.grow(1) == SG_OK;
  for (;;) {
    std::vector<Slice> batch;
    {
      std::unique_lock<std::mutex> lock(s->mu_);
      s->cv.wait(lock, [&] {
        if (s->stopping) return true;
        for (auto& r : s->pending)
          if (r->next_row < r->n_rows) return true;
        return false;
      });
      if (s->stopping) break;
      batch = take_batch(s);
    }
    int status = ok ? SG_OK : SG_ERR_OOM;
    std::string msg = ok ? "" : "sg_serve: a worker could not allocate its batch buffers";
    int64_t nrows = 0, nnz = 0;
    if (status == SG_OK) {
      h_ip[0] = 0;
      for (const auto& sl : batch) {
        const Request& r = *sl.r;
        const int64_t q0 = r.indptr[0];
        for (int64_t i = sl.a; i < sl.b; ++i) {
          const int64_t len = r.indptr[i + 1] - r.indptr[i];
          h_ip[nrows + 1] = h_ip[nrows] + len;
          ++nrows;
        }
        nnz += r.indptr[sl.b] - q0 - (r.indptr[sl.a] - q0);
      }
      status = d_ind.grow(size_t(std::max<int64_t>(nnz, 1)));
      if (status == SG_OK) status = d_dat.grow(size_t(std::max<int64_t>(nnz, 1)));
      int64_t pos = 0;
      auto cu = [&](cudaError_t e) {
        if (e != cudaSuccess && status == SG_OK) {
          status = SG_ERR_CUDA;
          msg = std::string("sg_serve: ") + cudaGetErrorString(e);
        }
      };
      if (status == SG_OK) {
        cu(cudaMemcpyAsync(d_ip.p, h_ip, sizeof(int64_t) * (nrows + 1), cudaMemcpyHostToDevice, st));
        for (const auto& sl : batch) {
          const Request& r = *sl.r;
          const int64_t q0 = r.indptr[0];
          const int64_t p0 = r.indptr[sl.a] - q0, p1 = r.indptr[sl.b] - q0;
          if (p1 > p0) {
            cu(cudaMemcpyAsync(d_ind.p + pos, r.indices + p0, sizeof(int32_t) * (p1 - p0), cudaMemcpyHostToDevice,
                               st));
            cu(cudaMemcpyAsync(d_dat.p + pos, r.data + p0, sizeof(int32_t) * (p1 - p0), cudaMemcpyHostToDevice, st));
          }
          pos += p1 - p0;
        }
      }
      if (status == SG_OK)
        status = sg_normalize_csr(h, d_ip.p, d_ind.p, d_dat.p, nrows, s->d_cmap, s->n_genes, s->n_feats,
                                  s->d_missing, 1.0f, nullptr, s->size_factor, s->flags, d_x.p, ld, SG_F32, nullptr,
                                  nullptr, nullptr, st);
      if (status == SG_OK)
        status = sg_project(h, d_x.p, nrows, s->n_feats, ld, s->mu, s->sigma, s->loadings, s->d, s->ld_l, d_sc.p,
                            s->ld_ref, nullptr, 0, s->precision, st);
      if (status == SG_OK)
        status = sg_knn(h, d_sc.p, nrows, s->ref_scores, s->n_ref, s->d, s->ld_ref, s->k, -1, s->margin,
                        s->precision, d_idx.p, d_dist.p, d_miss.p, st);
      if (status == SG_OK) {
        cu(cudaMemcpyAsync(h_idx, d_idx.p, sizeof(int64_t) * nrows * s->k, cudaMemcpyDeviceToHost, st));
        cu(cudaMemcpyAsync(h_dist, d_dist.p, sizeof(float) * nrows * s->k, cudaMemcpyDeviceToHost, st));
        cu(cudaStreamSynchronize(st));
      } else if (msg.empty()) {
        msg = sg_last_error();
      }
    }
    std::lock_guard<std::mutex> lock(s->mu_);
    complete(s, batch, h_idx, h_dist, status, msg.c_str());
    s->batches += 1;
    s->rows += nrows;
  }
  if (h_ip) cudaFreeHost(h_ip);
  if (h_idx) cudaFreeHost(h_idx);
  if (h_dist) cudaFreeHost(h_dist);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  sg_destroy(h);
}

}  // namespace

extern "C" {

int sg_serve_create(int device, const float* mu32, const float* sigma32, const float* loadings32, int32_t n_feats,
                    int32_t d, int32_t ld_l, const float* ref_scores, int64_t n_ref, int32_t ld_ref,
                    const int32_t* col_map, int64_t n_genes, const uint8_t* missing_mask, int32_t k,
                    int32_t precision, double size_factor, uint32_t norm_flags, int32_t max_batch_rows,
                    size_t hbm_budget_bytes, int32_t n_workers, sg_server** out) {
  sg::clear_error();
  SG_ARG(out && mu32 && sigma32 && loadings32 && ref_scores && col_map && missing_mask,
         "sg_serve_create: null pointer argument");
  *out = nullptr;
  SG_ARG(n_feats > 0 && d > 0 && ld_l >= d && ld_ref >= d && n_ref >= 1 && n_genes >= 1,
         "sg_serve_create: bad reference sizes");
  SG_ARG(k >= 1 && k <= n_ref, "sg_serve_create: k=%d outside [1, n_ref]", k);
  SG_ARG(precision == SG_PLAIN || precision == SG_PRECISION, "sg_serve_create: unknown precision %d", precision);
  SG_ARG(max_batch_rows >= 1 && n_workers >= 1 && n_workers <= 16, "sg_serve_create: bad batch rows or workers");
  SG_ARG(hbm_budget_bytes > 0, "sg_serve_create: the HBM budget must be positive");
  for (int64_t g = 0; g < n_genes; ++g)
    SG_ARG(col_map[g] >= -1 && col_map[g] < n_feats, "sg_serve_create: col_map[%lld] out of range", (long long)g);
  SG_CUDA(cudaSetDevice(device));
  auto* s = new sg_server();
  s->device = device;
  s->mu = mu32;
  s->sigma = sigma32;
  s->loadings = loadings32;
  s->ref_scores = ref_scores;
  s->n_feats = n_feats;
  s->d = d;
  s->ld_l = ld_l;
  s->ld_ref = ld_ref;
  s->n_ref = n_ref;
  s->n_genes = n_genes;
  s->k = k;
  s->precision = precision;
  s->margin = precision == SG_PRECISION ? 16 : 0;
  s->max_rows = max_batch_rows;
  s->size_factor = size_factor;
  s->flags = norm_flags;
  s->budget = hbm_budget_bytes;
  const size_t ld = size_t(n_feats + 3) / 4 * 4;
  s->bytes_per_row = 8 + ld * 4 + size_t(ld_ref) * 4 + size_t(k) * 12;
  if (cudaMalloc(&s->d_cmap, sizeof(int32_t) * n_genes) != cudaSuccess ||
      cudaMalloc(&s->d_missing, n_feats) != cudaSuccess ||
      cudaMemcpy(s->d_cmap, col_map, sizeof(int32_t) * n_genes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(s->d_missing, missing_mask, n_feats, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    if (s->d_cmap) cudaFree(s->d_cmap);
    if (s->d_missing) cudaFree(s->d_missing);
    delete s;
    return sg::fail(SG_ERR_OOM, "sg_serve_create: could not place the gene panel on the device");
  }
  for (int w = 0; w < n_workers; ++w) s->workers.emplace_back(worker_main, s);
  *out = s;
  return SG_OK;
}

int sg_serve_submit(sg_server* s, const int64_t* indptr, const int32_t* indices, const int32_t* data, int64_t n_rows,
                    int64_t* request_id) {
  sg::clear_error();
  SG_ARG(s && indptr && request_id && n_rows >= 0, "sg_serve_submit: bad argument");
  const int64_t nnz = n_rows ? indptr[n_rows] - indptr[0] : 0;
  SG_ARG(nnz >= 0 && (nnz == 0 || (indices && data)), "sg_serve_submit: bad CSR");
  auto r = std::make_shared<Request>();
  r->indptr = indptr;
  r->indices = indices;
  r->data = data;
  r->n_rows = n_rows;
  r->idx.assign(size_t(n_rows) * s->k, -1);
  r->dist.assign(size_t(n_rows) * s->k, 0.f);
  r->bytes = request_cost(s, *r);
  std::lock_guard<std::mutex> lock(s->mu_);
  if (s->init_status != SG_OK) return sg::fail(s->init_status, "sg_serve: %s", s->init_error.c_str());
  r->id = s->next_id++;
  *request_id = r->id;
  s->all[r->id] = r;
  if (r->bytes > s->budget) {
    r->status = SG_ERR_BUDGET;
    r->error = "sg_serve: the request needs " + std::to_string(r->bytes) + " bytes of HBM, more than the budget of " +
               std::to_string(s->budget);
    r->done = true;
  } else if (n_rows == 0) {
    r->done = true;
  } else {
    s->queued.push_back(r);
    admit(s);
  }
  s->cv.notify_all();
  return SG_OK;
}

int sg_serve_poll(sg_server* s, int64_t request_id, int32_t* done) {
  sg::clear_error();
  SG_ARG(s && done, "sg_serve_poll: null argument");
  std::lock_guard<std::mutex> lock(s->mu_);
  auto it = s->all.find(request_id);
  SG_ARG(it != s->all.end(), "sg_serve_poll: unknown request %lld", (long long)request_id);
  *done = it->second->done ? 1 : 0;
  return SG_OK;
}

int sg_serve_wait(sg_server* s, int64_t request_id, int64_t timeout_ms) {
  sg::clear_error();
  SG_ARG(s, "sg_serve_wait: null server");
  std::unique_lock<std::mutex> lock(s->mu_);
  auto it = s->all.find(request_id);
  SG_ARG(it != s->all.end(), "sg_serve_wait: unknown request %lld", (long long)request_id);
  auto r = it->second;
  const bool done = s->cv.wait_for(lock, std::chrono::milliseconds(std::max<int64_t>(0, timeout_ms)),
                                   [&] { return r->done || s->init_status != SG_OK; });
  if (!r->done && s->init_status != SG_OK) return sg::fail(s->init_status, "sg_serve: %s", s->init_error.c_str());
  if (!done) return sg::fail(SG_ERR_TIMEOUT, "sg_serve_wait: request %lld not done within %lld ms",
                             (long long)request_id, (long long)timeout_ms);
  return SG_OK;
}

int sg_serve_result(sg_server* s, int64_t request_id, int64_t* idx_out, float* dist_out) {
  sg::clear_error();
  SG_ARG(s, "sg_serve_result: null server");
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lock(s->mu_);
    auto it = s->all.find(request_id);
    SG_ARG(it != s->all.end(), "sg_serve_result: unknown request %lld", (long long)request_id);
    SG_ARG(it->second->done, "sg_serve_result: request %lld is not done", (long long)request_id);
    r = it->second;
    s->all.erase(it);
  }
  if (r->status != SG_OK) return sg::fail(r->status, "%s", r->error.c_str());
  SG_ARG(r->n_rows == 0 || (idx_out && dist_out), "sg_serve_result: null output buffer");
  if (r->n_rows) {
    memcpy(idx_out, r->idx.data(), sizeof(int64_t) * r->idx.size());
    memcpy(dist_out, r->dist.data(), sizeof(float) * r->dist.size());
  }
  return SG_OK;
}

int sg_serve_stats(sg_server* s, int64_t* batches, int64_t* rows) {
  sg::clear_error();
  SG_ARG(s, "sg_serve_stats: null server");
  if (batches) *batches = s->batches.load();
  if (rows) *rows = s->rows.load();
  return SG_OK;
}

int sg_serve_destroy(sg_server* s) {
  if (!s) return SG_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu_);
    s->stopping = true;
    s->cv.notify_all();
  }
  for (auto& t : s->workers) t.join();
  cudaSetDevice(s->device);
  cudaFree(s->d_cmap);
  cudaFree(s->d_missing);
  delete s;
  return SG_OK;
}

}  // extern "C"
