// f1: the MiniBatchKMeans step of make_graph (scarf/ann.py:328-346): one
// partial_fit per row block of the reduced data, in order, then predict for
// every row. Follows scikit-learn 1.6.1's MiniBatchKMeans with n_init=3 (which
// partial_fit does not use), reassignment_ratio 0.01 and unit sample weights
// (sklearn/cluster/_kmeans.py: partial_fit, _mini_batch_step, _random_reassign,
// _kmeans_plusplus; sklearn/cluster/_k_means_minibatch.pyx:
// _minibatch_update_dense).
//
//   init     the first block's rows by greedy k-means++ (2 + ln k local
//            trials); when the block has exactly k rows that picks every row,
//            and the centres are taken in row order.
//   step     labels = nearest centre (sg_knn, k = 1: exact FP32 squared
//            distances, ties to the smaller index); for every centre with
//            members c <- (c * w + sum of members in row order) * (1 / (w + n))
//            in FP64 and w += n; then, every 10 k rows of blocks or while a
//            centre has no weight, the centres below 0.01 x the largest weight
//            (at most half the block's rows, smallest weights first) move to
//            distinct random rows of the block and take the smallest remaining
//            weight.
//   predict  labels of all rows against the final centres (sg_knn, k = 1).
//
// Random draws come from a counter hash (SplitMix64's finaliser) of the seed,
// a stream number and an index, not from numpy's generator, so runs are
// reproducible but differ from scikit-learn's wherever it draws.
#include "common.cuh"

#include <algorithm>
#include <cmath>

extern "C" int sg_knn(sg_handle* h, const float* queries, int64_t nq, const float* refs, int64_t nr, int32_t d,
                      int32_t ld, int32_t k, int64_t self_offset, int32_t margin, int32_t precision,
                      int64_t* idx_out, float* dist_out, int64_t* n_missed, void* stream);

namespace {

__global__ void km_narrow_kernel(const int64_t* __restrict__ a, int64_t n, int32_t* __restrict__ b) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) b[i] = int32_t(a[i]);
}

constexpr int kKmMaxK = 2048;      // centres
constexpr int kKmMaxBlock = 4096;  // rows per block
constexpr int kKmThreads = 1024;

__host__ __device__ __forceinline__ uint64_t km_hash(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t z = seed + (stream * 0x100000000ull + i) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double km_unit(uint64_t seed, uint64_t stream, uint64_t i) {
  return double(km_hash(seed, stream, i) >> 11) * (1.0 / 9007199254740992.0);
}

// Fit state on the device (one stream-ordered allocation per fit).
struct KmState {
  double* c64;      // k x d centres
  float* c32;       // k x ld centres (FP32 copy the assignment reads)
  double* w;        // k weights
  long long* since; // rows since the last reassignment check
  int64_t* lab;     // block labels (int64, from sg_knn)
  float* dist;      // block distances
  int* cnt;         // k: members per centre in this block
  int* off;         // k + 1: first member of each centre in perm
  int* perm;        // block rows grouped by centre, row order within
  int* flag;        // 1: this step checks for reassignment
};

__device__ __forceinline__ double sq_dist_rows(const float* __restrict__ a, const float* __restrict__ b, int d) {
  double s = 0.0;
  for (int j = 0; j < d; ++j) {
    const double t = double(a[j]) - double(b[j]);
    s += t * t;
  }
  return s;
}

// Greedy k-means++ over the block's rows (one CTA): D2 = squared distance to
// the nearest chosen centre; each round draws 2 + ln k candidates with
// probability proportional to D2 and keeps the one that lowers the potential
// sum most (first on ties).
__global__ void __launch_bounds__(kKmThreads)
km_plusplus_kernel(const float* __restrict__ x, int ld, int rows, int d, int k, uint64_t seed, int trials,
                   KmState s) {
  extern __shared__ double sm[];
  double* d2 = sm;                                   // rows
  double* csum = d2 + rows;                          // max(rows, blockDim): prefix sums, reduction scratch
  double* pot = csum + (rows > kKmThreads ? rows : kKmThreads);  // trials
  int* cid = reinterpret_cast<int*>(pot + trials);  // trials
  __shared__ int chosen;
  __shared__ double total;
  const int tid = threadIdx.x;
  if (tid == 0) chosen = int(km_unit(seed, 1, 0) * rows) % rows;
  __syncthreads();
  for (int c = 0; c < k; ++c) {
    // centre c is row `chosen`
    const float* xc = x + int64_t(chosen) * ld;
    for (int j = tid; j < d; j += blockDim.x) s.c64[int64_t(c) * d + j] = double(xc[j]);
    for (int i = tid; i < rows; i += blockDim.x) {
      const double t = sq_dist_rows(x + int64_t(i) * ld, xc, d);
      d2[i] = c == 0 ? t : fmin(d2[i], t);
    }
    __syncthreads();
    if (c + 1 == k) break;
    // prefix sums of d2 in row order (one thread: rows <= 4096)
    if (tid == 0) {
      double acc = 0.0;
      for (int i = 0; i < rows; ++i) {
        acc += d2[i];
        csum[i] = acc;
      }
      total = acc;
    }
    __syncthreads();
    if (tid < trials) {
      const double r = km_unit(seed, 2 + uint64_t(c), uint64_t(tid)) * total;
      int lo = 0, hi = rows - 1;  // first index with csum > r (searchsorted, side left on csum >= r)
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (csum[mid] < r) lo = mid + 1;
        else hi = mid;
      }
      cid[tid] = lo;
      pot[tid] = 0.0;
    }
    __syncthreads();
    // potential of each candidate: sum over rows of min(d2, dist to candidate)
    for (int t = 0; t < trials; ++t) {
      const float* xt = x + int64_t(cid[t]) * ld;
      double part = 0.0;
      for (int i = tid; i < rows; i += blockDim.x) part += fmin(d2[i], sq_dist_rows(x + int64_t(i) * ld, xt, d));
      // fixed-order block reduction through csum (reused as scratch)
      csum[tid] = part;
      __syncthreads();
      for (int wdt = blockDim.x / 2; wdt > 0; wdt >>= 1) {
        if (tid < wdt) csum[tid] += csum[tid + wdt];
        __syncthreads();
      }
      if (tid == 0) pot[t] = csum[0];
      __syncthreads();
    }
    if (tid == 0) {
      int best = 0;
      for (int t = 1; t < trials; ++t)
        if (pot[t] < pot[best]) best = t;
      chosen = cid[best];
    }
    __syncthreads();
  }
}

// Centres = the block's rows in order (k rows): k-means++ picks every row.
__global__ void km_rows_init_kernel(const float* __restrict__ x, int ld, int k, int d, KmState s) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(k) * d) return;
  const int64_t c = e / d;
  const int j = int(e - c * d);
  s.c64[e] = double(x[c * ld + j]);
}

__global__ void km_to_f32_kernel(int k, int d, int ld, KmState s) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(k) * ld) return;
  const int64_t c = e / ld;
  const int j = int(e - c * ld);
  s.c32[e] = j < d ? float(s.c64[c * d + j]) : 0.f;
}

// A mini-batch step after the block's labels are known, in three launches:
// km_group_kernel (one CTA) counts and groups the rows by centre and makes
// scikit-learn's reassignment decision; km_move_kernel (all SMs, one thread
// per centre coordinate) applies the count-weighted update; km_reassign_kernel
// (one CTA) adds the counts to the weights and, when due, reassigns light
// centres. The serial parts read shared memory only.
__global__ void __launch_bounds__(kKmThreads)
km_group_kernel(int rows, int k, int batch_size, KmState s) {
  extern __shared__ int smi[];
  int* cnt = smi;          // k
  int* labs = cnt + k;     // rows (-1 outside [0, k))
  __shared__ int any_zero;
  const int tid = threadIdx.x;
  if (tid == 0) any_zero = 0;
  for (int c = tid; c < k; c += blockDim.x) cnt[c] = 0;
  for (int i = tid; i < rows; i += blockDim.x) {
    const int64_t c = s.lab[i];
    labs[i] = (c >= 0 && c < k) ? int(c) : -1;  // none outside from a valid kNN
  }
  __syncthreads();
  for (int c = tid; c < k; c += blockDim.x)
    if (s.w[c] == 0.0) any_zero = 1;
  for (int i = tid; i < rows; i += blockDim.x)
    if (labs[i] >= 0) atomicAdd(&cnt[labs[i]], 1);
  __syncthreads();
  for (int c = tid; c < k; c += blockDim.x) s.cnt[c] = cnt[c];
  __syncthreads();
  if (tid == 0) {
    // _random_reassign: counted in whole blocks of the first block's size
    long long since = *s.since + batch_size;
    int flag = 0;
    if (any_zero || since >= 10ll * k) {
      since = 0;
      flag = 1;
    }
    *s.since = since;
    *s.flag = flag;
    int acc = 0;
    for (int c = 0; c < k; ++c) {
      const int n = cnt[c];
      s.off[c] = acc;
      cnt[c] = acc;  // running position
      acc += n;
    }
    s.off[k] = acc;
    for (int i = 0; i < rows; ++i) {  // stable: row order within each centre
      const int c = labs[i];
      if (c >= 0) s.perm[cnt[c]++] = i;
    }
  }
}

// _minibatch_update_dense: c <- (c * w + members in row order) * (1 / (w + n)), FP64
__global__ void km_move_kernel(const float* __restrict__ x, int ld, int d, int k, KmState s) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(k) * d) return;
  const int c = int(e / d), j = int(e - int64_t(c) * d);
  const int n = s.cnt[c];
  if (n == 0) return;
  const double w = s.w[c];
  double v = s.c64[e] * w;
  const int o = s.off[c];
  for (int m = o; m < o + n; ++m) v += double(x[int64_t(s.perm[m]) * ld + j]);
  v *= 1.0 / (w + double(n));
  s.c64[e] = v;
  s.c32[int64_t(c) * ld + j] = float(v);
}

__global__ void __launch_bounds__(kKmThreads)
km_reassign_kernel(const float* __restrict__ x, int ld, int rows, int d, int k, uint64_t seed, long long step,
                   KmState s) {
  extern __shared__ double smd[];
  double* ws = smd;                                                         // k
  unsigned long long* key = reinterpret_cast<unsigned long long*>(ws + k);  // kKmMaxBlock
  int* order = reinterpret_cast<int*>(key + kKmMaxBlock);                   // k
  __shared__ int n_re;
  __shared__ double wmin_rest;
  const int tid = threadIdx.x;
  for (int c = tid; c < k; c += blockDim.x) {
    const double w = s.w[c] + double(s.cnt[c]);
    ws[c] = w;
    s.w[c] = w;
  }
  if (*s.flag == 0) return;  // uniform
  __syncthreads();
  if (tid == 0) {
    double mx = 0.0;
    for (int c = 0; c < k; ++c) mx = fmax(mx, ws[c]);
    // candidates: weight < 0.01 x max; at most int(0.5 * rows), smallest
    // weights first (index order on ties), then back in index order
    int m = 0;
    for (int c = 0; c < k; ++c)
      if (ws[c] < 0.01 * mx) order[m++] = c;
    const int cap = int(0.5 * rows);
    if (m > cap) {
      for (int a = 1; a < m; ++a) {
        const int v = order[a];
        int b = a - 1;
        while (b >= 0 && ws[order[b]] > ws[v]) {
          order[b + 1] = order[b];
          --b;
        }
        order[b + 1] = v;
      }
      m = cap;
      for (int a = 1; a < m; ++a) {
        const int v = order[a];
        int b = a - 1;
        while (b >= 0 && order[b] > v) {
          order[b + 1] = order[b];
          --b;
        }
        order[b + 1] = v;
      }
    }
    n_re = m;
    double mn = INFINITY;
    int fi = 0;
    for (int c = 0; c < k; ++c) {
      if (fi < m && order[fi] == c) ++fi;
      else mn = fmin(mn, ws[c]);
    }
    wmin_rest = mn;
  }
  __syncthreads();
  const int m = n_re;
  if (m == 0) return;
  // distinct rows of the block, uniformly: the m smallest hash keys (the row
  // index in the low 12 bits keeps them distinct), by a bitonic sort
  int P = 1;
  while (P < rows) P <<= 1;
  for (int i = tid; i < P; i += blockDim.x)
    key[i] = i < rows ? (km_hash(seed, 0x80000000ull + uint64_t(step), uint64_t(i)) & ~0xFFFull) | uint64_t(i)
                      : ~0ull;
  __syncthreads();
  for (int size = 2; size <= P; size <<= 1) {
    for (int j = size >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long a = key[i], b = key[l];
          if ((a > b) == ((i & size) == 0)) {
            key[i] = b;
            key[l] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int64_t e = tid; e < int64_t(m) * d; e += blockDim.x) {
    const int a = int(e / d), j = int(e - int64_t(a) * d);
    const int row = int(key[a] & 0xFFFull);  // the row index in the key's low bits
    const float v = x[int64_t(row) * ld + j];
    s.c64[int64_t(order[a]) * d + j] = double(v);
    s.c32[int64_t(order[a]) * ld + j] = v;
  }
  for (int a = tid; a < m; a += blockDim.x) s.w[order[a]] = wmin_rest;
}

}  // namespace

extern "C" int sg_kmeans_minibatch(sg_handle* h, const float* x, int64_t n, int32_t d, int32_t ld, int32_t k,
                                   int32_t block_rows, uint64_t seed, double* centers_out, int32_t* labels_out,
                                   void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(x && centers_out && labels_out, "sg_kmeans_minibatch: null pointer argument");
  SG_ARG(d >= 1 && d <= 64 && ld >= d && ld % 4 == 0, "sg_kmeans_minibatch: need 1 <= d <= 64, ld >= d, ld % 4 == 0");
  SG_ARG(k >= 1 && k <= kKmMaxK, "sg_kmeans_minibatch: k=%d outside [1, %d]", k, kKmMaxK);
  SG_ARG(block_rows >= 1 && block_rows <= kKmMaxBlock, "sg_kmeans_minibatch: block_rows=%d outside [1, %d]",
         block_rows, kKmMaxBlock);
  SG_ARG(n >= 1 && n < (int64_t(1) << 31), "sg_kmeans_minibatch: n=%lld outside [1, 2^31)", (long long)n);
  const int first = int(std::min<int64_t>(n, block_rows));
  SG_ARG(first >= k, "sg_kmeans_minibatch: the first block has %d rows, fewer than k=%d", first, k);
  // state in its own allocation: the kNN calls below use the handle's workspace
  const size_t need = sg::Carver::need(sizeof(double) * size_t(k) * d) + sg::Carver::need(sizeof(float) * size_t(k) * ld) +
                      sg::Carver::need(sizeof(double) * size_t(k)) + sg::Carver::need(sizeof(long long)) +
                      sg::Carver::need(sizeof(int64_t) * size_t(n)) + sg::Carver::need(sizeof(float) * size_t(n)) +
                      sg::Carver::need(sizeof(int) * size_t(k)) + sg::Carver::need(sizeof(int) * size_t(k + 1)) +
                      sg::Carver::need(sizeof(int) * size_t(block_rows)) + sg::Carver::need(sizeof(int));
  void* buf = nullptr;
  SG_CUDA(cudaMallocAsync(&buf, need, st));
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{buf, st};
  sg::Carver cv(buf);
  KmState s;
  s.c64 = cv.take<double>(size_t(k) * d);
  s.c32 = cv.take<float>(size_t(k) * ld);
  s.w = cv.take<double>(size_t(k));
  s.since = cv.take<long long>(1);
  s.lab = cv.take<int64_t>(size_t(n));
  s.dist = cv.take<float>(size_t(n));
  s.cnt = cv.take<int>(size_t(k));
  s.off = cv.take<int>(size_t(k + 1));
  s.perm = cv.take<int>(size_t(block_rows));
  s.flag = cv.take<int>(1);
  SG_CUDA(cudaMemsetAsync(s.w, 0, sizeof(double) * size_t(k), st));
  SG_CUDA(cudaMemsetAsync(s.since, 0, sizeof(long long), st));
  sg::ProfScope prof(h, "kmeans", st);
  if (first == k) {
    km_rows_init_kernel<<<sg::ceil_div_i(int64_t(k) * d, 256), 256, 0, st>>>(x, ld, k, d, s);
    SG_LAUNCH_CHECK();
  } else {
    const int trials = 2 + int(std::log(double(k)));
    const size_t smem = sizeof(double) * (size_t(first) + size_t(std::max(first, kKmThreads)) + size_t(trials)) +
                        sizeof(int) * size_t(trials);
    SG_CUDA(cudaFuncSetAttribute(km_plusplus_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    km_plusplus_kernel<<<1, kKmThreads, smem, st>>>(x, ld, first, d, k, seed, trials, s);
    SG_LAUNCH_CHECK();
  }
  const unsigned g32 = unsigned(sg::ceil_div_i(int64_t(k) * ld, 256));
  km_to_f32_kernel<<<g32, 256, 0, st>>>(k, d, ld, s);
  SG_LAUNCH_CHECK();
  const size_t smem_g = sizeof(int) * size_t(k + block_rows);
  const size_t smem_r = sizeof(double) * size_t(k) + sizeof(unsigned long long) * size_t(kKmMaxBlock) +
                        sizeof(int) * size_t(k);
  SG_CUDA(cudaFuncSetAttribute(km_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_g)));
  SG_CUDA(cudaFuncSetAttribute(km_reassign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_r)));
  const unsigned gmove = unsigned(sg::ceil_div_i(int64_t(k) * d, 256));
  long long step = 0;
  for (int64_t r0 = 0; r0 < n; r0 += block_rows, ++step) {
    const int rows = int(std::min<int64_t>(block_rows, n - r0));
    const float* xb = x + r0 * ld;
    int rc = sg_knn(h, xb, rows, s.c32, k, d, ld, 1, -1, 0, SG_PLAIN, s.lab, s.dist, nullptr, st);
    if (rc) return rc;
    km_group_kernel<<<1, kKmThreads, smem_g, st>>>(rows, k, first, s);
    SG_LAUNCH_CHECK();
    km_move_kernel<<<gmove, 256, 0, st>>>(xb, ld, d, k, s);
    SG_LAUNCH_CHECK();
    km_reassign_kernel<<<1, kKmThreads, smem_r, st>>>(xb, ld, rows, d, k, seed, step, s);
    SG_LAUNCH_CHECK();
  }
  SG_CUDA(cudaMemcpyAsync(centers_out, s.c64, sizeof(double) * size_t(k) * d, cudaMemcpyDeviceToDevice, st));
  // predict: the nearest final centre of every row
  int rc = sg_knn(h, x, n, s.c32, k, d, ld, 1, -1, 16, SG_PRECISION, s.lab, s.dist, nullptr, st);
  if (rc) return rc;
  km_narrow_kernel<<<sg::ceil_div_i(n, 256), 256, 0, st>>>(s.lab, n, labels_out);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
