// a6/a7 precision form: BF16 distance tiles on the tcgen05 tensor cores.
//
// One CTA owns 256 queries (two 128-row query tiles, one TMEM lane per query
// of each) and a range of reference rows.
//   warp 0      TMA producer: the BF16 query tiles once, then 128-row reference
//               tiles into a 4-stage shared-memory ring (128B swizzle, K = 64).
//   warp 1      MMA issuer (one thread): per reference tile, D0 = Q0 . R^T and
//               D1 = Q1 . R^T (128 x 128 each) as tcgen05.mma kind::f16 K=16
//               steps into one of two TMEM accumulator pairs (2 x 256 columns),
//               committed to the ring's empty barrier and to the accumulator's
//               full barrier. Each reference tile read from L2 feeds 256 queries.
//   warps 2-9   epilogue, two per TMEM lane quarter (one per query tile): each
//               reads its 32 queries' 128 columns 64 at a time with tcgen05.ld,
//               takes the ranking key |r|^2 - 2 q.r, tests it against the
//               query's current threshold and keeps one register top-KC list
//               per query; the accumulator is handed back as soon as it has been
//               read, so the MMAs of tile t+1 overlap the epilogue of tile t.
// Every mbarrier wait is bounded: on expiry the kernel raises an error flag,
// drains its own TMA copies and MMAs (again bounded), frees TMEM and returns.
// The candidates are re-ranked exactly in FP32 by knn.cu.
#include "tc_ptx.cuh"

#include <type_traits>

#include <algorithm>

int sg_rerank(const float* queries, const float* refs, int d, int ld, int64_t nq, const int* cand, int nlists, int kc,
              int64_t nq_pad, int kq, int k, int64_t self_offset, int64_t* idx_out, float* dist_out,
              unsigned long long* nmiss, cudaStream_t st);  // knn.cu

namespace {

using namespace tc;

constexpr int BM = 128;           // queries per tile (TMEM lanes)
constexpr int QT = 2;             // query tiles per CTA
constexpr int BQ = BM * QT;       // queries per CTA
constexpr int BN = 128;           // references per tile
constexpr int BK = 64;
constexpr int STAGES = 4;
constexpr uint32_t A_BYTES = BQ * BK * 2;
constexpr uint32_t A_TILE_BYTES = BM * BK * 2;
constexpr uint32_t B_BYTES = BN * BK * 2;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_COLS = QT * BN;  // one accumulator pair
constexpr int EPI_WARPS = 4 * QT;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int BUF = 48;  // candidate buffer slots per query
__host__ __device__ constexpr size_t smem_bytes(int) {
  return 1024 /*align*/ + A_BYTES + STAGES * B_BYTES + 256 /*barriers*/ + EPI_WARPS * BN * 4 /*rn*/ +
         size_t(BUF) * BQ * 8 /*buffers*/;
}
static_assert(smem_bytes(0) <= 227 * 1024, "shared memory budget");
static_assert(2 * ACC_COLS <= TMEM_COLS, "two accumulator pairs");

// Instruction descriptor, kind::f16: D F32, A/B BF16, both K-major, N, M.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);

// min of three floats in one PTX instruction (sm_100 and later)
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Order-preserving map of a float to uint32 (for atomicMin across CTAs) and back.
__device__ __forceinline__ uint32_t key_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float bits_key(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

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
  // Sorted insert of v (< worst()) after any equal keys. Slot j changes when
  // d[j] > v and then takes slot j-1's entry when that one is also above v,
  // else v: every slot is decided from the old list alone, with no chain
  // between slots.
  __device__ __forceinline__ void insert(float v, int vi) {
#pragma unroll
    for (int j = KC - 1; j >= 1; --j) {
      const bool gt = d[j] > v;
      const bool up = d[j - 1] > v;
      const float nd = up ? d[j - 1] : v;
      const int ni = up ? i[j - 1] : vi;
      d[j] = gt ? nd : d[j];
      i[j] = gt ? ni : i[j];
    }
    if (d[0] > v) {
      d[0] = v;
      i[0] = vi;
    }
  }
};

// SHARE: the lists of a query in different CTAs (reference splits) share
// their worst keys through `qbound` (worth it with several splits; with one
// the extra state costs more than the candidates it saves)
template <int KC, bool SHARE>
__global__ void __launch_bounds__(THREADS, 1)
knn_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              const float* __restrict__ rn, int64_t nr, int64_t rps, int* __restrict__ cand, int64_t nq_pad,
              int fold, unsigned* __restrict__ qbound, int* __restrict__ err, uint32_t wait_limit, int idle_mma,
              const int* __restrict__ perm, int64_t nq) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = su32(smem_raw);
  uint8_t* sm = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* sA = sm;
  uint8_t* sB = sm + A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + A_BYTES + STAGES * B_BYTES);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* a_full = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(a_full + 1);
  float* rn_s = reinterpret_cast<float*>(sm + A_BYTES + STAGES * B_BYTES + 256);
  float* bufk = rn_s + EPI_WARPS * BN;                         // [BUF][BQ]
  int* bufi = reinterpret_cast<int*>(bufk + BUF * BQ);         // [BUF][BQ]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q0 = int64_t(blockIdx.x) * BQ;
  const int64_t s_begin = int64_t(blockIdx.y) * rps;
  const int64_t s_end = min(nr, s_begin + rps);
  const int ntiles = int((s_end - s_begin + BN - 1) / BN);
  // With a locality order (perm != null: queries and references are the same
  // rows, both sorted so that neighbours sit close together), the CTA starts
  // at the reference tile of its own queries and wraps around, so that its
  // candidate lists fill with near neighbours first and few later keys pass.
  int t0 = 0;
  if (perm != nullptr && ntiles > 0) {
    const int64_t diag = (q0 - s_begin) / BN;
    t0 = int(diag < 0 ? 0 : (diag >= ntiles ? ntiles - 1 : diag));
  }
  auto tile_at = [&](int t) -> int64_t {
    const int u = t + t0;
    return s_begin + int64_t(u >= ntiles ? u - ntiles : u) * BN;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], EPI_WARPS);
    }
    mbar_init(a_full, 1);
    fence_barrier_init();
  }
  if (warp == 1) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      tma_prefetch(&tmA);
      tma_prefetch(&tmB);
      mbar_expect_tx(a_full, A_BYTES);
      tma_load_2d(sA, &tmA, a_full, 0, int(q0));
      int issued = 0;
      for (int t = 0; t < ntiles; ++t) {
        const int s = t % STAGES;
        const uint32_t ph = (t / STAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1, wait_limit)) break;
        mbar_expect_tx(&full[s], B_BYTES);
        tma_load_2d(sB + s * B_BYTES, &tmB, &full[s], 0, int(tile_at(t)));
        ++issued;
      }
      // on the error path, let this CTA's own copies land before leaving
      if (*reinterpret_cast<volatile int*>(err)) {
        for (int t = max(0, issued - STAGES); t < issued; ++t) {
          for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(&full[t % STAGES], (t / STAGES) & 1); ++it) {
          }
        }
        for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(a_full, 0); ++it) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && !idle_mma) {
      int issued = 0;
      if (mbar_wait(a_full, 0, err, 2, wait_limit)) {
        tc_fence_after();
        const uint64_t adesc0 = smem_desc_sw128(su32(sA));
        const uint64_t adesc1 = smem_desc_sw128(su32(sA + A_TILE_BYTES));
        for (int t = 0; t < ntiles; ++t) {
          const int s = t % STAGES;
          const uint32_t ph = (t / STAGES) & 1;
          const int b = t & 1;
          const uint32_t aph = (t >> 1) & 1;
          if (!mbar_wait(&acc_empty[b], aph ^ 1u, err, 3, wait_limit)) break;
          if (!mbar_wait(&full[s], ph, err, 4, wait_limit)) break;
          tc_fence_after();
          const uint64_t bdesc = smem_desc_sw128(su32(sB + s * B_BYTES));
          const uint32_t d0 = tmem + uint32_t(b) * ACC_COLS;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            mma_bf16(d0, adesc0 + uint64_t(2 * kk), bdesc + uint64_t(2 * kk), kIdesc, kk > 0 ? 1u : 0u);
            mma_bf16(d0 + uint32_t(BN), adesc1 + uint64_t(2 * kk), bdesc + uint64_t(2 * kk), kIdesc,
                     kk > 0 ? 1u : 0u);
          }
          mma_commit(&empty[s]);
          mma_commit(&acc_full[b]);
          ++issued;
        }
      }
      if (issued > 0 && *reinterpret_cast<volatile int*>(err)) {
        // let the last MMAs finish before TMEM is released
        const int t = issued - 1;
        for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(&acc_full[t & 1], (t >> 1) & 1); ++it) {
        }
      }
    }
  } else {
    const int quarter = warp & 3;      // TMEM lanes [32*quarter, 32*quarter+32) are this warp's
    const int sel = (warp - 2) >> 2;   // query tile: accumulator columns [BN*sel, BN*sel + BN)
    const int row = sel * BM + quarter * 32 + lane;  // query of this thread within the CTA
    float* my_rn = rn_s + (warp - 2) * BN;
    float* bk = bufk + row;  // slot s of this query's buffer: bk[s * BQ]
    int* bi = bufi + row;
    TopK<KC> top;
    top.init();
    // Every list of a query (its reference splits in other CTAs) holds keys of
    // that query, so each full list's worst key bounds the query's final
    // KC-th key from above: a candidate at or above the smallest of them
    // cannot make the query's top KC. The splits share their worst keys
    // through `qbound` (atomicMin on an order-preserving encoding); it only
    // decreases, so a stale value is still a valid bound.
    unsigned* qb = qbound + q0 + row;
    float shared = __int_as_float(0x7f800000);  // smallest worst key of the other lists
    float published = shared;
    float thr = shared;
    int cnt = 0;
    // merge the buffered candidates into the sorted register list, then
    // publish the list's worst key
    auto compact = [&]() {
      for (int s2 = 0; s2 < cnt; ++s2) {
        const float v = bk[s2 * BQ];
        if (v < top.worst() && (!SHARE || v < shared)) top.insert(v, bi[s2 * BQ]);
      }
      cnt = 0;
      const float w = top.worst();
      if (SHARE && w < published) {
        published = w;
        atomicMin(qb, key_bits(w));
      }
      thr = SHARE ? fminf(w, shared) : w;
    };
    // filter one chunk of 32 accumulator columns into the buffer; kRn: add
    // |r|^2 here (not folded into the MMA). References past the last one
    // carry an enormous key (a +inf norm, or a huge folded norm), so the last
    // tile needs no mask. Four independent 8-key minima, then one branch per
    // chunk: after the first tiles almost no chunk holds a passing key.
    auto process = [&](auto rn_tag, const uint32_t (&r)[32], int ch, int64_t r0) {
      constexpr bool kRn = decltype(rn_tag)::value;
      const int cbase = int(r0) + ch * 32;
      float kk[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        float key = __uint_as_float(r[q]);
        if (kRn) key += my_rn[ch * 32 + q];  // the accumulator is -2 q.r (the queries are scaled by -2)
        kk[q] = key;
      }
      float m8[4];
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const float* k8 = kk + 8 * g;
        m8[g] = fmin3(fmin3(k8[0], k8[1], k8[2]), fmin3(k8[3], k8[4], k8[5]), fminf(k8[6], k8[7]));
      }
      if (fminf(fmin3(m8[0], m8[1], m8[2]), m8[3]) < thr) {
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          if (m8[g] < thr) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              if (kk[8 * g + q] < thr) {
                bk[cnt * BQ] = kk[8 * g + q];
                bi[cnt * BQ] = cbase + 8 * g + q;
                ++cnt;
              }
            }
          }
        }
      }
    };
    constexpr int NCH = BN / 32;
    static_assert(NCH == 4, "the tile loop below handles two 64-column halves");
    auto tiles = [&](auto rn_tag) {
      constexpr bool kRn = decltype(rn_tag)::value;
      for (int t = 0; t < ntiles; ++t) {
        const int b = t & 1;
        const uint32_t aph = (t >> 1) & 1;
        const int64_t r0 = tile_at(t);
        if (kRn) {
          __syncwarp();  // every lane has read the last tile's norms
          reinterpret_cast<float4*>(my_rn)[lane] = __ldg(reinterpret_cast<const float4*>(rn + r0) + lane);
        }
        if (SHARE) {
          shared = fminf(shared, bits_key(__ldcg(qb)));
          thr = fminf(thr, shared);
        }
        bool ok = mbar_wait(&acc_full[b], aph, err, 5, wait_limit);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) return;
        tc_fence_after();
        __syncwarp();
        const uint32_t tbase = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b) * ACC_COLS + uint32_t(sel * BN);
        // two 64-column loads per tile into one register buffer (fewer
        // round trips to TMEM than four 32-column loads, double-buffered,
        // and 2-4% faster at 1M x 1M)
        uint32_t ra[32], rb[32];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          tmem_ld64(tbase + uint32_t(64 * half), ra, rb);
          tmem_wait_ld(ra, rb);
          if (half == 1) {
            // the tile is in registers: hand the accumulator back before
            // filtering its second half, so the MMAs of tile t+2 start earlier
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
          }
          if (__any_sync(0xffffffffu, cnt > BUF - 32)) compact();
          process(rn_tag, ra, 2 * half, r0);
          if (__any_sync(0xffffffffu, cnt > BUF - 32)) compact();
          process(rn_tag, rb, 2 * half + 1, r0);
        }
      }
    };
    // padding references carry |r|^2 = +inf (unfolded) or a huge folded norm
    if (fold) tiles(std::false_type{});
    else tiles(std::true_type{});
    compact();
    // list `split` of every query: nsplit lists per query
    // back to the caller's row order: the list of query perm[q], with the
    // caller's reference numbers
    const int64_t qpos = q0 + row;
    const int64_t qout = (perm != nullptr && qpos < nq) ? int64_t(perm[qpos]) : qpos;
    int* out = cand + (int64_t(blockIdx.y) * nq_pad + qout) * KC;
    // padding rows (index nr and up) carry enormous keys but still fill the
    // slots of a list whose split has fewer than KC references: they are
    // not candidates (-1, which the re-rank skips)
#pragma unroll
    for (int j = 0; j < KC; ++j) {
      const int ix = top.i[j];
      out[j] = (ix >= 0 && ix < nr) ? (perm != nullptr ? perm[ix] : ix) : -1;
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// BF16 operands, zero padded to 64 columns and n_pad rows.
// refs: the rounded rows; with `fold`, columns d, d+1, d+2 carry |r_b|^2 split
//   into three BF16 terms (hi, mid, lo), so that the product with the query's
//   ones gives the norm to ~2^-24 relative, and padding rows carry 1e38 there;
//   norms[] = |r_b|^2 (+inf for padding).
// queries: -2 * rounded rows (exact in BF16) and, with `fold`, ones in columns
//   d..d+2. The accumulator is then |r|^2 - 2 q.r directly.
// Both operands are packed 64 rows per CTA: the rows (gathered through perm
// when given) are staged in shared memory with coalesced loads, each row's
// norm is summed by one thread in column order, and the BF16 rows leave in
// 16-byte stores. kRef: the references as described above, and their FP32
// norms (+inf for padding rows); otherwise the queries.
constexpr int PR = 64;  // rows per packing CTA

template <bool kRef>
__global__ void __launch_bounds__(256)
pack_bf16_kernel(const float* __restrict__ in, int64_t n, int d, int ld, int fold, __nv_bfloat16* __restrict__ out,
                 int64_t n_pad, float* __restrict__ norms, const int* __restrict__ perm) {
  __shared__ float rows[PR][BK + 1];
  __shared__ float nrm[PR];
  const int64_t r0 = int64_t(blockIdx.x) * PR;
  const int tid = threadIdx.x;
  for (int task = tid; task < PR * BK; task += 256) {
    const int rr = task >> 6, c = task & (BK - 1);
    const int64_t r = r0 + rr;
    float v = 0.f;
    if (r < n && c < d) {
      const int64_t src = perm != nullptr ? int64_t(perm[r]) : r;
      v = in[src * ld + c];
    }
    rows[rr][c] = v;
  }
  __syncthreads();
  if (kRef && tid < PR) {
    const int64_t r = r0 + tid;
    float sum = 0.f;
    for (int c = 0; c < d; ++c) {
      const float bf = __bfloat162float(__float2bfloat16_rn(rows[tid][c]));
      sum = fmaf(bf, bf, sum);
    }
    nrm[tid] = sum;
    if (r < n_pad) norms[r] = r < n ? sum : __int_as_float(0x7f800000);
  }
  __syncthreads();
  for (int task = tid; task < PR * (BK / 8); task += 256) {
    const int rr = task >> 3, c0 = (task & 7) * 8;
    const int64_t r = r0 + rr;
    if (r >= n_pad) continue;
    const bool real = r < n;
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int c = c0 + e;
      __nv_bfloat16 b;
      if (kRef) {
        b = __float2bfloat16_rn(0.f);
        if (c < d) {
          b = __float2bfloat16_rn(rows[rr][c]);
        } else if (fold && c < d + 3) {
          if (!real) {
            if (c == d) b = __float2bfloat16_rn(1e38f);  // padding: a key no query keeps
          } else {
            const float sum = nrm[rr];
            const __nv_bfloat16 hi = __float2bfloat16_rn(sum);
            const float rem1 = sum - __bfloat162float(hi);
            const __nv_bfloat16 mid = __float2bfloat16_rn(rem1);
            const __nv_bfloat16 lo = __float2bfloat16_rn(rem1 - __bfloat162float(mid));
            b = c == d ? hi : (c == d + 1 ? mid : lo);
          }
        }
      } else {
        if (c < d) {
          const float v = __bfloat162float(__float2bfloat16_rn(rows[rr][c]));
          b = __float2bfloat16_rn(-2.f * v);
        } else {
          b = __float2bfloat16_rn((fold && c < d + 3) ? 1.f : 0.f);
        }
      }
      o[e] = b;
    }
    *reinterpret_cast<uint4*>(out + r * BK + c0) = *reinterpret_cast<const uint4*>(o);
  }
}

// ---- locality order of a self-kNN ---------------------------------------
// The rows are sorted (stably) by their nearest pilot, a strided sample of the
// rows; queries and references then share that order, and each CTA meets its
// own neighbourhood in its first reference tiles (see knn_tc_kernel).
constexpr int kMaxPilots = 128;
constexpr int kSortRows = 512;  // rows per counting-sort block

// nearest pilot of every row by |p|^2 - 2 x.p (ties to the smaller pilot);
// pilots = rows 0, stride, 2 stride, ... staged as -2p (zero padded to BK)
__global__ void nearest_pilot_kernel(const float* __restrict__ x, int64_t n, int d, int ld, int64_t stride, int np,
                                     int* __restrict__ pid) {
  __shared__ float sp[kMaxPilots * BK];
  __shared__ float pn[kMaxPilots];
  for (int i = threadIdx.x; i < np * BK; i += blockDim.x) {
    const int p = i / BK, c = i - p * BK;
    sp[i] = c < d ? -2.f * x[int64_t(p) * stride * ld + c] : 0.f;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    float q = 0.f;
    for (int c = 0; c < d; ++c) q = fmaf(sp[p * BK + c], sp[p * BK + c], q);
    pn[p] = 0.25f * q;
  }
  __syncthreads();
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float xr[BK];
#pragma unroll
  for (int c = 0; c < BK; ++c) xr[c] = c < d ? x[r * ld + c] : 0.f;
  float best = __int_as_float(0x7f800000);
  int bi = 0;
  for (int p = 0; p < np; ++p) {
    float acc = pn[p];
#pragma unroll
    for (int c = 0; c < BK; ++c) acc = fmaf(xr[c], sp[p * BK + c], acc);
    if (acc < best) {
      best = acc;
      bi = p;
    }
  }
  pid[r] = bi;
}

// rows of each counting-sort block per pilot: hist[pilot * nblk + block]
__global__ void bin_count_kernel(const int* __restrict__ pid, int64_t n, int np, int* __restrict__ hist, int nblk) {
  __shared__ int cnt[kMaxPilots];
  for (int i = threadIdx.x; i < np; i += blockDim.x) cnt[i] = 0;
  __syncthreads();
  const int64_t a = int64_t(blockIdx.x) * kSortRows, b = min(n, a + kSortRows);
  for (int64_t r = a + threadIdx.x; r < b; r += blockDim.x) atomicAdd(&cnt[pid[r]], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < np; i += blockDim.x) hist[int64_t(i) * nblk + blockIdx.x] = cnt[i];
}

// exclusive scan of hist in (pilot, block) order; one CTA of 1024 threads
__global__ void __launch_bounds__(1024) bin_scan_kernel(int* __restrict__ hist, int64_t total) {
  __shared__ int part[1024];
  const int64_t per = (total + 1023) / 1024;
  const int64_t a = int64_t(threadIdx.x) * per, b = min(total, a + per);
  int sum = 0;
  for (int64_t i = a; i < b; ++i) sum += hist[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int64_t i = a; i < b; ++i) {
    const int v = hist[i];
    hist[i] = run;
    run += v;
  }
}

// stable scatter: one warp per counting-sort block, its rows 32 at a time in order
__global__ void bin_scatter_kernel(const int* __restrict__ pid, int64_t n, int np, const int* __restrict__ off,
                                   int nblk, int* __restrict__ perm) {
  __shared__ int cur[kMaxPilots];
  const int lane = threadIdx.x;
  for (int i = lane; i < np; i += 32) cur[i] = off[int64_t(i) * nblk + blockIdx.x];
  __syncwarp();
  const int64_t a = int64_t(blockIdx.x) * kSortRows, b = min(n, a + kSortRows);
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t base = a; base < b; base += 32) {
    const int64_t r = base + lane;
    const bool live = r < b;
    const int p = live ? pid[r] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, p);
    if (live) perm[cur[p] + __popc(peers & lt)] = int(r);
    __syncwarp();
    if (live && (peers & lt) == 0u) cur[p] += __popc(peers);
    __syncwarp();
  }
}

__global__ void add_count_kernel(unsigned long long* __restrict__ dst, const unsigned long long* __restrict__ src) {
  *dst += *src;
}

// pilots used for n rows (0: no locality order)
int pilots_for(int64_t n) {
  if (n < (int64_t(1) << 15)) return 0;
  return int(std::min<int64_t>(kMaxPilots, std::max<int64_t>(16, n / 4096)));
}

int locality_order(const float* x, int64_t n, int d, int ld, int np, int* pid, int* hist, int* perm,
                   cudaStream_t st) {
  const int nblk = sg::ceil_div_i(n, kSortRows);
  nearest_pilot_kernel<<<sg::ceil_div_i(n, 128), 128, 0, st>>>(x, n, d, ld, n / np, np, pid);
  SG_LAUNCH_CHECK();
  bin_count_kernel<<<nblk, 256, 0, st>>>(pid, n, np, hist, nblk);
  SG_LAUNCH_CHECK();
  bin_scan_kernel<<<1, 1024, 0, st>>>(hist, int64_t(np) * nblk);
  SG_LAUNCH_CHECK();
  bin_scatter_kernel<<<nblk, 32, 0, st>>>(pid, n, np, hist, nblk, perm);
  SG_LAUNCH_CHECK();
  return SG_OK;
}

template <int KC>
int launch_tc(const CUtensorMap& a, const CUtensorMap& b, const float* rn, int64_t nr, int64_t rps, int nsplit,
              int* cand, int64_t nq_pad, int fold, unsigned* qbound, int* err, uint32_t wait_limit, int idle_mma,
              const int* perm, int64_t nq, cudaStream_t st) {
  const size_t smem = smem_bytes(KC);
  dim3 grid(unsigned(nq_pad / BQ), unsigned(nsplit));
  if (nsplit > 1) {
    SG_CUDA(cudaFuncSetAttribute(knn_tc_kernel<KC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    knn_tc_kernel<KC, true><<<grid, THREADS, smem, st>>>(a, b, rn, nr, rps, cand, nq_pad, fold, qbound, err, wait_limit,
                                                           idle_mma, perm, nq);
  } else {
    SG_CUDA(cudaFuncSetAttribute(knn_tc_kernel<KC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    knn_tc_kernel<KC, false><<<grid, THREADS, smem, st>>>(a, b, rn, nr, rps, cand, nq_pad, fold, qbound, err, wait_limit,
                                                           idle_mma, perm, nq);
  }
  SG_LAUNCH_CHECK();
  return SG_OK;
}

}  // namespace

// Precision-form kNN: BF16 candidates on the tensor cores, exact FP32 re-rank.
int sg_knn_tc(sg_handle* h, const float* queries, int64_t nq, const float* refs, int64_t nr, int d, int ld, int kq,
              int k, int64_t self_offset, int margin, int64_t* idx_out, float* dist_out, unsigned long long* nmiss,
              cudaStream_t st) {
  if (d > BK) return sg::fail(SG_ERR_ARG, "sg_knn: the precision form supports d <= %d", BK);
  int kc = kq + margin;
  if (kc > 64) return sg::fail(SG_ERR_ARG, "sg_knn: k + margin too large (<= 64 candidates per list)");
  kc = kc <= 16 ? 16 : kc <= 32 ? 32 : kc <= 40 ? 40 : kc <= 48 ? 48 : 64;
  const int64_t nq_pad = sg::ceil_div(nq, BQ) * BQ;
  const int64_t nr_pad = sg::ceil_div(nr, BN) * BN;
  if (nr_pad >= (int64_t(1) << 31) || nq_pad >= (int64_t(1) << 31)) return sg::fail(SG_ERR_ARG, "sg_knn: too many rows");
  const int qtiles = int(nq_pad / BQ);
  // reference splits per query tile: the heuristic fills ~4 CTAs (1024 queries) per SM
  auto splits_for = [&](int want) {
    int ns = std::max(1, want);
    ns = int(std::min<int64_t>(ns, std::max<int64_t>(1, nr_pad / (BN * 8))));
    ns = std::min(ns, 256);
    const int64_t rps_ = sg::ceil_div(sg::ceil_div(nr, ns), BN) * BN;
    return int(sg::ceil_div(nr, rps_));
  };
  const int ns0 = splits_for(int(std::lround(double(h->sm_count) * 4 / qtiles)));
  auto ilog2 = [](int64_t v) {
    int r = 0;
    while ((int64_t(1) << (r + 1)) <= v) ++r;
    return r;
  };
  const int qb = ilog2(nq_pad), rb = ilog2(nr_pad);
  // self-kNN (the queries are the references): the rows can be put in a
  // locality order (see pilots_for); the autotuner decides whether it pays
  const int np_self = (queries == refs && nq == nr && self_offset == 0) ? pilots_for(nr) : 0;
  int tuned = 0, tuned_loc = 1;
  for (const auto& e : h->knn_tune)
    if (e.qb == qb && e.rb == rb && e.d == d && e.kc == kc && e.self == (np_self > 0)) {
      tuned = e.nsplit;
      tuned_loc = e.loc;
    }
  auto run = [&](int nsplit, int loc, unsigned long long* miss) -> int {
  const int np = loc ? np_self : 0;
  const int nblk = np ? sg::ceil_div_i(nr, kSortRows) : 0;
  const int64_t rps = sg::ceil_div(sg::ceil_div(nr, nsplit), BN) * BN;
  const int fold = d <= BK - 3 ? 1 : 0;
  const size_t need = sg::Carver::need(size_t(nr_pad) * BK * 2) + sg::Carver::need(size_t(nr_pad) * 4) +
                      sg::Carver::need(size_t(nq_pad) * BK * 2) +
                      sg::Carver::need(sizeof(int) * size_t(nsplit) * nq_pad * kc) + sg::Carver::need(sizeof(int)) +
                      sg::Carver::need(sizeof(unsigned) * size_t(nq_pad)) +
                      (np ? 2 * sg::Carver::need(sizeof(int) * size_t(nr)) +
                                sg::Carver::need(sizeof(int) * size_t(np) * nblk)
                          : 0);
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  __nv_bfloat16* Rb = cv.take<__nv_bfloat16>(size_t(nr_pad) * BK);
  float* rn = cv.take<float>(nr_pad);
  __nv_bfloat16* Qb = cv.take<__nv_bfloat16>(size_t(nq_pad) * BK);
  int* cand = cv.take<int>(size_t(nsplit) * nq_pad * kc);
  int* err = cv.take<int>(1);
  unsigned* qbound = cv.take<unsigned>(size_t(nq_pad));
  int* perm = nullptr;
  if (np) {
    int* pid = cv.take<int>(size_t(nr));
    perm = cv.take<int>(size_t(nr));
    int* hist = cv.take<int>(size_t(np) * nblk);
    const int rc0 = locality_order(refs, nr, d, ld, np, pid, hist, perm, st);
    if (rc0) return rc0;
  }
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  // all ones: decodes to NaN, which fminf ignores (no bound yet)
  SG_CUDA(cudaMemsetAsync(qbound, 0xFF, sizeof(unsigned) * size_t(nq_pad), st));
  pack_bf16_kernel<true><<<sg::ceil_div_i(nr_pad, PR), 256, 0, st>>>(refs, nr, d, ld, fold, Rb, nr_pad, rn, perm);
  SG_LAUNCH_CHECK();
  pack_bf16_kernel<false><<<sg::ceil_div_i(nq_pad, PR), 256, 0, st>>>(queries, nq, d, ld, fold, Qb, nq_pad, nullptr,
                                                                       perm);
  SG_LAUNCH_CHECK();
  CUtensorMap ta, tb;
  int rc = make_map(&ta, Qb, nq_pad, BQ);
  if (rc) return rc;
  rc = make_map(&tb, Rb, nr_pad, BN);
  if (rc) return rc;
  const uint32_t wl = h->wait_limit ? h->wait_limit : WAIT_LIMIT;
  const int idle = h->idle_mma_once ? 1 : 0;
  h->idle_mma_once = false;
  {
  sg::ProfScope prof(h, "knn_tc", st);
  if (kc == 16) rc = launch_tc<16>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, fold, qbound, err, wl, idle, perm, nq, st);
  else if (kc == 32) rc = launch_tc<32>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, fold, qbound, err, wl, idle, perm, nq, st);
  else if (kc == 40) rc = launch_tc<40>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, fold, qbound, err, wl, idle, perm, nq, st);
  else if (kc == 48) rc = launch_tc<48>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, fold, qbound, err, wl, idle, perm, nq, st);
  else rc = launch_tc<64>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, fold, qbound, err, wl, idle, perm, nq, st);
  }
  if (rc) return rc;
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_TIMEOUT, "sg_knn: a tensor-core pipeline wait expired (stage %d)", herr);
  sg::ProfScope prof(h, "rerank", st);
  h->last_knn_splits = nsplit;
  h->last_knn_locality = np > 0 ? 1 : 0;
  return sg_rerank(queries, refs, d, ld, nq, cand, nsplit, kc, nq_pad, kq, k, self_offset, idx_out, dist_out,
                   miss, st);
  };
  if (tuned) return run(tuned, tuned_loc, nmiss);
  if (!h->autotune || double(nq) * double(nr) < 1e9) return run(ns0, 1, nmiss);
  // Autotune the (split count, locality order) pair for this (query rows,
  // reference rows, d, list length, self) bucket: time the heuristic split
  // count, half and double of it, each with and without the locality order
  // for a self-kNN (kernel + re-rank), once, and keep the fastest. Every
  // candidate returns the same exact top k, so the last run's outputs stand;
  // its miss count alone is added to n_missed.
  struct Cand {
    int ns, loc;
  };
  std::vector<Cand> cands;
  for (int c : {ns0, splits_for(std::max(1, ns0 / 2)), splits_for(ns0 * 2)})
    for (int loc : {1, 0}) {
      if (loc == 0 && np_self == 0) continue;
      bool dup = false;
      for (const Cand& e : cands) dup |= (e.ns == c && e.loc == (np_self ? loc : 1));
      if (!dup) cands.push_back({c, np_self ? loc : 1});
    }
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  unsigned long long* trial_miss = nullptr;
  if (nmiss) SG_CUDA(cudaMallocAsync(&trial_miss, sizeof(unsigned long long), st));
  Cand best = cands[0];
  float best_ms = INFINITY;
  int rc = SG_OK;
  for (const Cand& c : cands) {
    if (trial_miss) SG_CUDA(cudaMemsetAsync(trial_miss, 0, sizeof(unsigned long long), st));
    SG_CUDA(cudaEventRecord(e0, st));
    rc = run(c.ns, c.loc, trial_miss);
    if (rc) break;
    SG_CUDA(cudaEventRecord(e1, st));
    SG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    SG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  if (rc == SG_OK && trial_miss) {
    add_count_kernel<<<1, 1, 0, st>>>(nmiss, trial_miss);
    SG_LAUNCH_CHECK();
  }
  if (trial_miss) cudaFreeAsync(trial_miss, st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  h->knn_tune.push_back({qb, rb, d, kc, best.ns, best.loc, np_self > 0});
  return SG_OK;
}
