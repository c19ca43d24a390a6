// a6/a7/a10: exact squared-L2 kNN.
//
// Stage 1 (candidates): a CTA owns 128 queries and sweeps a range of reference
// rows in tiles of 128. The distance tile is a 128x128 FP32 SIMT product
// (8x8 register micro-tiles over the transposed, zero-padded scores staged in
// shared memory with cp.async double buffering), turned into the ranking key
// |r|^2 - 2 q.r (|q|^2 is constant per query) and written to shared memory;
// then every query row is scanned by two threads, each keeping a sorted
// top-KC list in registers behind a threshold test. Candidate lists go to
// scratch. The precision form computes the same tile with the BF16 tcgen05
// kernel of knn_tc.cu.
// Stage 2 (re-rank): one warp per query recomputes exact FP32 sum((q-r)^2) for
// every candidate, keeps the kq best by (distance, index), and applies
// fix_knn_query's self-removal rule (scarf/ann.py:31-52) before writing k.
#include "common.cuh"

#include <algorithm>

int sg_knn_tc(sg_handle* h, const float* queries, int64_t nq, const float* refs, int64_t nr, int d, int ld, int kq,
              int k, int64_t self_offset, int margin, int64_t* idx_out, float* dist_out, unsigned long long* nmiss,
              cudaStream_t st);  // knn_tc.cu

namespace {

constexpr int QT_ = 128;  // queries per CTA
constexpr int RT_ = 128;  // refs per tile
constexpr int DS_PITCH = RT_ + 4;
constexpr int kMaxD = 64;
constexpr int BUFS = 24;  // candidate buffer slots per (query row, half)

template <int KC>
struct TopK {
  float d[KC];
  int i[KC];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int j = 0; j < KC; ++j) {
      d[j] = __int_as_float(0x7f800000);
      i[j] = -1;
    }
  }
  __device__ __forceinline__ float worst() const { return d[KC - 1]; }
  // insert (v, vi) into the ascending list; v < worst() must hold
  __device__ __forceinline__ void insert(float v, int vi) {
    bool placed = false;
#pragma unroll
    for (int j = KC - 1; j >= 1; --j) {
      const bool sh = d[j - 1] > v;
      const float nd = sh ? d[j - 1] : v;
      const int ni = sh ? i[j - 1] : vi;
      if (!placed) {
        d[j] = nd;
        i[j] = ni;
      }
      placed = placed || !sh;
    }
    if (!placed) {
      d[0] = v;
      i[0] = vi;
    }
  }
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// transposed, zero-padded copy: out[c * ldo + r] = in[r * ld + c]; norms[r] = |in_r|^2 (inf for padding)
__global__ void transpose_pad_kernel(const float* __restrict__ in, int64_t n, int d, int ld, float* __restrict__ out,
                                     int64_t ldo, float* __restrict__ norms) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= ldo) return;
  float s = 0.f;
  for (int c = 0; c < d; ++c) {
    const float v = r < n ? in[r * ld + c] : 0.f;
    out[int64_t(c) * ldo + r] = v;
    s = fmaf(v, v, s);
  }
  if (norms) norms[r] = r < n ? s : __int_as_float(0x7f800000);
}

template <int KC>
__global__ void __launch_bounds__(256, 1)
knn_simt_kernel(const float* __restrict__ QT, int64_t ldq, const float* __restrict__ RT, int64_t ldr,
                const float* __restrict__ rn, int d, int64_t nq, int64_t nr, int64_t refs_per_split,
                int* __restrict__ cand, int64_t nq_pad) {
  extern __shared__ __align__(16) float sm[];
  float* Qs = sm;                         // [d][128]
  float* Rs = Qs + kMaxD * QT_;           // [2][d][128]
  float* Ds = Rs + 2 * kMaxD * RT_;       // [128][DS_PITCH]
  float* Ns = Ds + QT_ * DS_PITCH;        // [2][128] reference norms
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t q0 = int64_t(blockIdx.x) * QT_;
  const int64_t s_begin = int64_t(blockIdx.y) * refs_per_split;
  const int64_t s_end = min(nr, s_begin + refs_per_split);
  const int my_row = tid & 127, half = tid >> 7;
  float* bk = Ns + 2 * RT_ + tid;                                  // slot s: bk[s * 256]
  int* bi = reinterpret_cast<int*>(Ns + 2 * RT_ + BUFS * 256) + tid;

  TopK<KC> top;
  top.init();
  float thr = __int_as_float(0x7f800000);
  int cnt = 0;
  // merge the buffered candidates into the sorted register list
  auto compact = [&]() {
    for (int s2 = 0; s2 < cnt; ++s2) {
      const float v = bk[s2 * 256];
      if (v < top.worst()) top.insert(v, bi[s2 * 256]);
    }
    cnt = 0;
    thr = top.worst();
  };

  // queries once
  for (int e = tid; e < d * (QT_ / 4); e += 256) {
    const int c = e / (QT_ / 4), v = e % (QT_ / 4);
    cp_async16(&Qs[c * QT_ + v * 4], &QT[int64_t(c) * ldq + q0 + v * 4]);
  }
  auto load_tile = [&](int buf, int64_t r0) {
    float* R = Rs + buf * kMaxD * RT_;
    for (int e = tid; e < d * (RT_ / 4); e += 256) {
      const int c = e / (RT_ / 4), v = e % (RT_ / 4);
      cp_async16(&R[c * RT_ + v * 4], &RT[int64_t(c) * ldr + r0 + v * 4]);
    }
    if (tid < RT_ / 4) cp_async16(&Ns[buf * RT_ + tid * 4], &rn[r0 + tid * 4]);
  };
  int buf = 0;
  if (s_begin < s_end) load_tile(0, s_begin);
  cp_async_commit();

  for (int64_t r0 = s_begin; r0 < s_end; r0 += RT_) {
    cp_async_wait_all();
    __syncthreads();  // tile `buf` visible; previous phase 2 done with Ds
    if (r0 + RT_ < s_end) load_tile(buf ^ 1, r0 + RT_);
    cp_async_commit();
    const float* R = Rs + buf * kMaxD * RT_;
    float acc[8][8];
#pragma unroll
    for (int p = 0; p < 8; ++p)
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[p][q] = 0.f;
#pragma unroll 2
    for (int c = 0; c < d; ++c) {
      const float4 a0 = *reinterpret_cast<const float4*>(&Qs[c * QT_ + ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&Qs[c * QT_ + 64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&R[c * RT_ + tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&R[c * RT_ + 64 + tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int p = 0; p < 8; ++p)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    // ranking key |r|^2 - 2 q.r; refs outside this split are excluded
    const float* N = Ns + buf * RT_;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int row = p < 4 ? ty * 4 + p : 64 + ty * 4 + p - 4;
      float o[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int col = q < 4 ? tx * 4 + q : 64 + tx * 4 + q - 4;
        const bool in = r0 + col < s_end;
        o[q] = in ? fmaf(-2.f, acc[p][q], N[col]) : __int_as_float(0x7f800000);
      }
      *reinterpret_cast<float4*>(&Ds[row * DS_PITCH + tx * 4]) = make_float4(o[0], o[1], o[2], o[3]);
      *reinterpret_cast<float4*>(&Ds[row * DS_PITCH + 64 + tx * 4]) = make_float4(o[4], o[5], o[6], o[7]);
    }
    __syncthreads();
    // phase 2: filter this thread's half row into its candidate buffer
    const float* D = Ds + my_row * DS_PITCH + half * 64;
    const int base = int(r0) + half * 64;
#pragma unroll 2
    for (int c = 0; c < 64; c += 8) {
      if (__any_sync(0xffffffffu, cnt > BUFS - 8)) compact();
      const float4 v0 = *reinterpret_cast<const float4*>(&D[c]);
      const float4 v1 = *reinterpret_cast<const float4*>(&D[c + 4]);
      const float kk[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
      const float m = fminf(fminf(fminf(kk[0], kk[1]), fminf(kk[2], kk[3])),
                            fminf(fminf(kk[4], kk[5]), fminf(kk[6], kk[7])));
      if (m < thr) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (kk[q] < thr) {
            bk[cnt * 256] = kk[q];
            bi[cnt * 256] = base + c + q;
            ++cnt;
          }
        }
      }
    }
    buf ^= 1;
  }
  compact();
  cp_async_wait_all();
  const int64_t q = q0 + my_row;
  int* out = cand + ((int64_t(blockIdx.y) * 2 + half) * nq_pad + q) * KC;
#pragma unroll
  for (int j = 0; j < KC; ++j) out[j] = top.i[j];
}

// Sorted list of (distance bits << 32 | index) keys: a total order that puts
// equal distances in index order.
template <int KQ>
struct KeyList {
  unsigned long long k[KQ];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int j = 0; j < KQ; ++j) k[j] = ~0ull;
  }
  __device__ __forceinline__ unsigned long long worst() const { return k[KQ - 1]; }
  __device__ __forceinline__ void insert(unsigned long long v) {  // v < worst()
    bool placed = false;
#pragma unroll
    for (int j = KQ - 1; j >= 1; --j) {
      const bool sh = k[j - 1] > v;
      const unsigned long long nk = sh ? k[j - 1] : v;
      if (!placed) k[j] = nk;
      placed = placed || !sh;
    }
    if (!placed) k[0] = v;
  }
  __device__ __forceinline__ void pop() {
#pragma unroll
    for (int j = 0; j < KQ - 1; ++j) k[j] = k[j + 1];
    k[KQ - 1] = ~0ull;
  }
};

// Ascending bitonic sort of the warp's 32 * SLOTS keys, element lane + 32 s in
// v[s]: partners in other lanes through shuffles, partners in the same lane
// (distance >= 32) by a local compare-exchange.
template <int SLOTS>
__device__ __forceinline__ void warp_bitonic_sort(unsigned long long (&v)[SLOTS], int lane) {
  constexpr int N = 32 * SLOTS;
#pragma unroll
  for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
    for (int j = size >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
          const int t = s ^ (j >> 5);
          if (t > s) {
            const bool up = ((lane + 32 * s) & size) == 0;
            const unsigned long long a = v[s], b = v[t];
            const bool sw = (a > b) == up;
            v[s] = sw ? b : a;
            v[t] = sw ? a : b;
          }
        }
      } else {
#pragma unroll
        for (int s = 0; s < SLOTS; ++s) {
          const int i = lane + 32 * s;
          const unsigned long long w = __shfl_xor_sync(0xffffffffu, v[s], j);
          const bool keep_min = ((i & size) == 0) == ((i & j) == 0);
          const bool lt = v[s] < w;
          v[s] = (lt == keep_min) ? v[s] : w;
        }
      }
    }
  }
}

// Re-rank for at most 32 * SLOTS candidates per query: each lane scores
// candidates lane + 32 s, the warp sorts the keys, and every lane writes its
// own output positions; the self rule uses ballots. The same keys in the same
// total order as the list merge below, so the same output.
// Exact FP32 sum over c < d of (q[c] - r[c])^2, accumulated in the order
// c = 0 .. d-1; the reference row is read 16 bytes at a time when its rows are
// 16-byte aligned (each lane reads its own candidate row, so wide loads cut
// the L1 wavefronts of the gather by four).
__device__ __forceinline__ float rerank_dist(const float* __restrict__ qv, const float* __restrict__ r, int d,
                                             bool vec) {
  float acc = 0.f;
  int c = 0;
  if (vec) {
    const float4* r4 = reinterpret_cast<const float4*>(r);
    for (; c + 3 < d; c += 4) {
      const float4 v = __ldg(r4 + (c >> 2));
      float df = qv[c] - v.x;
      acc = fmaf(df, df, acc);
      df = qv[c + 1] - v.y;
      acc = fmaf(df, df, acc);
      df = qv[c + 2] - v.z;
      acc = fmaf(df, df, acc);
      df = qv[c + 3] - v.w;
      acc = fmaf(df, df, acc);
    }
  }
  for (; c < d; ++c) {
    const float df = qv[c] - __ldg(r + c);
    acc = fmaf(df, df, acc);
  }
  return acc;
}

template <int SLOTS>
__global__ void __launch_bounds__(128)
rerank_sort_kernel(const float* __restrict__ queries, const float* __restrict__ refs, int d, int ld, int64_t nq,
                   const int* __restrict__ cand, int nlists, int kc, int64_t nq_pad, int kq, int k,
                   int64_t self_offset, int64_t* __restrict__ idx_out, float* __restrict__ dist_out,
                   unsigned long long* __restrict__ nmiss) {
  __shared__ float qs[4][kMaxD];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = int64_t(blockIdx.x) * 4 + warp;
  if (q >= nq) return;  // whole warps
  for (int c = lane; c < d; c += 32) qs[warp][c] = queries[q * ld + c];
  __syncwarp();
  const bool vec = (ld & 3) == 0 && (reinterpret_cast<uintptr_t>(refs) & 15) == 0;
  const int total = nlists * kc;
  unsigned long long v[SLOTS];
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) {
    v[s] = ~0ull;
    const int e = lane + 32 * s;
    if (e >= total) continue;
    const int ci = cand[(int64_t(e / kc) * nq_pad + q) * kc + e % kc];
    if (ci < 0) continue;
    const float acc = rerank_dist(qs[warp], refs + int64_t(ci) * ld, d, vec);
    v[s] = (static_cast<unsigned long long>(__float_as_uint(acc)) << 32) | unsigned(ci);
  }
  warp_bitonic_sort<SLOTS>(v, lane);
  // the self rule: drop position 0 when it is self, else the first self among
  // the first kq (a miss), else the last of them (a miss)
  int drop = -1;
  if (self_offset >= 0) {
    const unsigned self = unsigned(self_offset + q);
    int first = -1;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      const bool hit = lane + 32 * s < kq && v[s] != ~0ull && unsigned(v[s] & 0xffffffffu) == self;
      const unsigned b = __ballot_sync(0xffffffffu, hit);
      if (first < 0 && b) first = 32 * s + __ffs(int(b)) - 1;
    }
    if (first == 0) {
      drop = 0;
    } else {
      if (lane == 0) atomicAdd(nmiss, 1ull);
      drop = first > 0 ? first : kq - 1;
    }
  }
#pragma unroll
  for (int s = 0; s < SLOTS; ++s) {
    const int p = lane + 32 * s;
    if (p >= kq || p == drop) continue;
    const int o = drop >= 0 && p > drop ? p - 1 : p;
    if (o >= k) continue;
    idx_out[q * k + o] = v[s] == ~0ull ? -1 : int64_t(v[s] & 0xffffffffu);
    dist_out[q * k + o] = v[s] == ~0ull ? __int_as_float(0x7f800000) : __uint_as_float(unsigned(v[s] >> 32));
  }
}

// Stage 2: exact re-rank and self fix. One warp per query; every lane keeps a
// sorted key list of the candidates it scored, and the warp merges the 32
// lists by kq rounds of a warp-wide minimum over the list heads.
template <int KQ>
__global__ void __launch_bounds__(128)
rerank_kernel(const float* __restrict__ queries, const float* __restrict__ refs, int d, int ld, int64_t nq,
              const int* __restrict__ cand, int nlists, int kc, int64_t nq_pad, int kq, int k, int64_t self_offset,
              int64_t* __restrict__ idx_out, float* __restrict__ dist_out, unsigned long long* __restrict__ nmiss) {
  __shared__ float qs[4][kMaxD];
  __shared__ unsigned long long sel[4][64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q = int64_t(blockIdx.x) * 4 + warp;
  if (q >= nq) return;
  for (int c = lane; c < d; c += 32) qs[warp][c] = queries[q * ld + c];
  __syncwarp();
  KeyList<KQ> top;
  top.init();
  const int total = nlists * kc;
  for (int e = lane; e < total; e += 32) {
    const int l = e / kc, j = e % kc;
    const int ci = cand[(int64_t(l) * nq_pad + q) * kc + j];
    if (ci < 0) continue;
    const float s = rerank_dist(qs[warp], refs + int64_t(ci) * ld, d, false);
    const unsigned long long key = (static_cast<unsigned long long>(__float_as_uint(s)) << 32) | unsigned(ci);
    if (key < top.worst()) top.insert(key);
  }
  for (int t = 0; t < kq; ++t) {
    const unsigned long long head = top.k[0];
    const unsigned long long m = warp_min_u64(head);
    if (lane == 0) sel[warp][t] = m;
    if (m != ~0ull && head == m) top.pop();
  }
  __syncwarp();
  if (lane == 0) {
    const unsigned long long* S = sel[warp];
    int drop = -1;
    if (self_offset >= 0) {
      const unsigned self = unsigned(self_offset + q);
      const bool first_self = S[0] != ~0ull && unsigned(S[0] & 0xffffffffu) == self;
      if (!first_self) {
        atomicAdd(nmiss, 1ull);
        for (int p = 1; p < kq; ++p)
          if (S[p] != ~0ull && unsigned(S[p] & 0xffffffffu) == self) {
            drop = p;
            break;
          }
        if (drop < 0) drop = kq - 1;
      } else {
        drop = 0;
      }
    }
    int o = 0;
    for (int p = 0; p < kq && o < k; ++p) {
      if (p == drop) continue;
      const unsigned long long v = S[p];
      idx_out[q * k + o] = v == ~0ull ? -1 : int64_t(v & 0xffffffffu);
      dist_out[q * k + o] = v == ~0ull ? __int_as_float(0x7f800000) : __uint_as_float(unsigned(v >> 32));
      ++o;
    }
  }
}

template <int KC>
int launch_simt(const float* QT, int64_t ldq, const float* RT, int64_t ldr, const float* rn, int d, int64_t nq,
                int64_t nr, int64_t rps, int nsplit, int* cand, int64_t nq_pad, cudaStream_t st) {
  const size_t smem = sizeof(float) * (size_t(kMaxD) * QT_ + 2 * size_t(kMaxD) * RT_ + QT_ * DS_PITCH + 2 * RT_) +
                      size_t(BUFS) * 256 * 8;
  SG_CUDA(cudaFuncSetAttribute(knn_simt_kernel<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  dim3 grid(unsigned(nq_pad / QT_), unsigned(nsplit));
  knn_simt_kernel<KC><<<grid, 256, smem, st>>>(QT, ldq, RT, ldr, rn, d, nq, nr, rps, cand, nq_pad);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

template <int KQ>
int launch_rerank(const float* queries, const float* refs, int d, int ld, int64_t nq, const int* cand, int nlists,
                  int kc, int64_t nq_pad, int kq, int k, int64_t self_offset, int64_t* idx_out, float* dist_out,
                  unsigned long long* nmiss, cudaStream_t st) {
  rerank_kernel<KQ><<<unsigned(sg::ceil_div(nq, 4)), 128, 0, st>>>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad,
                                                                    kq, k, self_offset, idx_out, dist_out, nmiss);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

}  // namespace

// Shared by the tcgen05 candidate path: re-rank `nlists` candidate lists.
int sg_rerank(const float* queries, const float* refs, int d, int ld, int64_t nq, const int* cand, int nlists, int kc,
              int64_t nq_pad, int kq, int k, int64_t self_offset, int64_t* idx_out, float* dist_out,
              unsigned long long* nmiss, cudaStream_t st) {
  const int total = nlists * kc;
  if (kq <= 64 && total <= 128) {
    const unsigned grid = unsigned(sg::ceil_div(nq, 4));
    if (total <= 64)
      rerank_sort_kernel<2><<<grid, 128, 0, st>>>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k,
                                                  self_offset, idx_out, dist_out, nmiss);
    else
      rerank_sort_kernel<4><<<grid, 128, 0, st>>>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k,
                                                  self_offset, idx_out, dist_out, nmiss);
    SG_LAUNCH_CHECK();
    return SG_OK;
  }
  if (kq <= 16) return launch_rerank<16>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k, self_offset, idx_out, dist_out, nmiss, st);
  if (kq <= 32) return launch_rerank<32>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k, self_offset, idx_out, dist_out, nmiss, st);
  return launch_rerank<64>(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k, self_offset, idx_out, dist_out, nmiss, st);
}

extern "C" int sg_knn(sg_handle* h, const float* queries, int64_t nq, const float* refs, int64_t nr, int32_t d,
                      int32_t ld, int32_t k, int64_t self_offset, int32_t margin, int32_t precision,
                      int64_t* idx_out, float* dist_out, int64_t* n_missed, void* stream) {
  SG_HANDLE_CHECK(h);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SG_ARG(queries && refs && idx_out && dist_out, "sg_knn: null pointer argument");
  SG_ARG(d >= 1 && d <= kMaxD, "sg_knn: d=%d outside [1, %d]", d, kMaxD);
  SG_ARG(ld >= d, "sg_knn: ld < d");
  SG_ARG(nq >= 0 && nr >= 1 && nr < (int64_t(1) << 31), "sg_knn: bad nq/nr");
  SG_ARG(k >= 1, "sg_knn: k must be >= 1");
  SG_ARG(margin >= 0, "sg_knn: margin must be >= 0");
  SG_ARG(precision == SG_PLAIN || precision == SG_PRECISION, "sg_knn: unknown precision %d", precision);
  const bool self = self_offset >= 0;
  SG_ARG(!self || n_missed, "sg_knn: n_missed needed for a self query");
  const int kq = k + (self ? 1 : 0);
  SG_ARG(kq <= nr, "sg_knn: %d neighbours requested from %lld references", kq, (long long)nr);
  SG_ARG(kq <= 64, "sg_knn: k=%d too large (k + self <= 64)", k);
  if (nq == 0) return SG_OK;
  if (precision == SG_PRECISION) {
    unsigned long long* nm_p = reinterpret_cast<unsigned long long*>(n_missed);
    return sg_knn_tc(h, queries, nq, refs, nr, d, ld, kq, k, self_offset, margin, idx_out, dist_out,
                     self ? nm_p : nullptr, st);
  }
  int kc = kq + margin;
  kc = kc <= 16 ? 16 : kc <= 32 ? 32 : 64;
  SG_ARG(kq + margin <= 64, "sg_knn: k + margin too large (<= 64 candidates per list)");

  const int64_t nq_pad = sg::ceil_div(nq, QT_) * QT_;
  const int64_t nr_pad = sg::ceil_div(nr, RT_) * RT_;
  const int qtiles = int(nq_pad / QT_);
  // splits of the reference range: enough CTAs to fill the GPU for some waves
  int nsplit = std::max<int>(1, int(std::lround(double(h->sm_count) * 8 / qtiles)));
  const int64_t max_split = std::max<int64_t>(1, nr_pad / (RT_ * 4));
  nsplit = int(std::min<int64_t>(nsplit, max_split));
  nsplit = std::min(nsplit, 256);
  int64_t rps = sg::ceil_div(sg::ceil_div(nr, nsplit), RT_) * RT_;
  nsplit = int(sg::ceil_div(nr, rps));

  const bool same = (queries == refs) && (nq == nr);
  int status;
  const size_t cand_bytes = sizeof(int) * size_t(nsplit) * 2 * nq_pad * kc;
  const size_t need = sg::Carver::need(sizeof(float) * size_t(d) * nr_pad) + sg::Carver::need(sizeof(float) * nr_pad) +
                      (same ? 0 : sg::Carver::need(sizeof(float) * size_t(d) * nq_pad)) + sg::Carver::need(cand_bytes) +
                      sg::Carver::need(sizeof(unsigned long long));
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  float* RT = cv.take<float>(size_t(d) * nr_pad);
  float* rn = cv.take<float>(nr_pad);
  float* QT = same ? RT : cv.take<float>(size_t(d) * nq_pad);
  int* cand = cv.take<int>(size_t(nsplit) * 2 * nq_pad * kc);
  unsigned long long* nm = cv.take<unsigned long long>(1);

  const int nlists = 2 * nsplit;
  transpose_pad_kernel<<<sg::ceil_div_i(nr_pad, 256), 256, 0, st>>>(refs, nr, d, ld, RT, nr_pad, rn);
  SG_LAUNCH_CHECK();
  if (!same) {
    transpose_pad_kernel<<<sg::ceil_div_i(nq_pad, 256), 256, 0, st>>>(queries, nq, d, ld, QT, nq_pad, nullptr);
    SG_LAUNCH_CHECK();
  }
  int rc;
  {
  sg::ProfScope prof(h, "knn_simt", st);
  if (kc == 16) rc = launch_simt<16>(QT, nq_pad, RT, nr_pad, rn, d, nq, nr, rps, nsplit, cand, nq_pad, st);
  else if (kc == 32) rc = launch_simt<32>(QT, nq_pad, RT, nr_pad, rn, d, nq, nr, rps, nsplit, cand, nq_pad, st);
  else rc = launch_simt<64>(QT, nq_pad, RT, nr_pad, rn, d, nq, nr, rps, nsplit, cand, nq_pad, st);
  }
  if (rc != SG_OK) return rc;
  sg::ProfScope prof(h, "rerank", st);
  unsigned long long* nmiss = self ? reinterpret_cast<unsigned long long*>(n_missed) : nm;
  return sg_rerank(queries, refs, d, ld, nq, cand, nlists, kc, nq_pad, kq, k, self_offset, idx_out, dist_out, nmiss, st);
}
