// a4, precision form: 3xBF16 split covariance on the tcgen05 tensor cores.
//
// zsplit: z = (x - mu)/sigma in float32 (rows outside the PCA mask are 0),
//   split into hi = bf16(z) and lo = bf16(z - hi), and written transposed
//   (feature-major, cells contiguous: the K-major operand layout), with
//   per-tile column sums of z for the centring term.
// gemm: D[128 x 256] tile of Z^T Z for the tiles that touch the upper
//   triangle, K = a split of the cells in steps of 64; per step three
//   products hi.hi + hi.lo + lo.hi (12 tcgen05.mma kind::f16 K=16) fed by a
//   2-stage TMA ring (4 tiles per stage). Each stage lands in three parts with
//   their own barriers, the two hi tiles first, so that the four hi.hi
//   products start while the lo tiles are still in flight (4 % faster than
//   one barrier for the whole 96 KB stage). The FP32 TMEM accumulator covers
//   one chunk of CHUNK_STEPS steps (1024 cells) only: two accumulators
//   alternate, and while the MMAs fill one, the epilogue warps add the other
//   into the CTA's partial tile, held as unevaluated float pairs (hi + lo,
//   error-free TwoSum additions). A long FP32 accumulation drifts, since the
//   many equal small terms of the zero counts of a gene all round the same
//   way; short chunks bound that drift to the size of the 3xBF16 residual.
//   Partials are reduced over the splits in FP64 in a fixed order.
#include "tc_ptx.cuh"

#include <initializer_list>

namespace {

using namespace tc;

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BK = 64;
constexpr int STAGES = 2;
constexpr uint32_t A_BYTES = BM * BK * 2;
constexpr uint32_t B_BYTES = BN * BK * 2;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr uint32_t ACC_COLS = 256;
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
constexpr int CHUNK_STEPS = 16;
constexpr int TILE_ELEMS = BM * BN;

// (hi, lo) += v with hi + lo exact to the pair's precision (Knuth's TwoSum)
__device__ __forceinline__ void pair_add(float& hi, float& lo, float v) {
  const float s = __fadd_rn(hi, v);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb));
  hi = s;
  lo = __fadd_rn(lo, e);
}
constexpr size_t SMEM_BYTES = 1024 + size_t(STAGES) * STAGE_BYTES + 256;
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);
constexpr int ZT = 64;  // zsplit tile

// The value z takes on a zero count of column c, shifted by delta_c so that
// it is a BF16 number: those entries then split exactly (lo = 0) and their
// many equal products carry no representation error. The scatter of the
// shifted values is corrected back in FP64 (cov_shift_kernel).
__device__ __forceinline__ float zero_shift(float mu, float sg) {
  const float z0 = __fdiv_rn(0.f - mu, sg);
  return z0 - __bfloat162float(__float2bfloat16_rn(z0));
}

constexpr int ZR = 128;  // cells per zsplit tile

// z' = (x - mu)/sigma - delta for a tile of 128 cells x 64 features: the rows
// read 16 lanes per row (16-byte vectors when kVec: rows 16-byte aligned),
// the column sums of z per 64-cell half in row order (the partials of 64-row
// tiles), and the transposed hi/lo values written two cells per lane (128 B
// per warp store, 256 B per feature and tile).
template <bool kVec>
__global__ void __launch_bounds__(256)
zsplit_kernel(const float* __restrict__ x, int64_t n_rows, int n_cols, int64_t ld, const float* __restrict__ mu,
              const float* __restrict__ sg, const uint8_t* __restrict__ mask, __nv_bfloat16* __restrict__ hi,
              __nv_bfloat16* __restrict__ lo, int64_t n_pad, float* __restrict__ zpart, int h_pad) {
  __shared__ float t[ZR][ZT + 1];
  __shared__ float smu[ZT], ssg[ZT], dl[ZT];
  __shared__ uint8_t valid[ZR];
  const int64_t r0 = int64_t(blockIdx.x) * ZR;
  const int c0 = blockIdx.y * ZT;
  const int tid = threadIdx.x;
  if (tid < ZT) {
    const int c = c0 + tid;
    smu[tid] = c < n_cols ? mu[c] : 0.f;
    ssg[tid] = c < n_cols ? sg[c] : 1.f;
    dl[tid] = c < n_cols ? zero_shift(mu[c], sg[c]) : 0.f;
  }
  if (tid < ZR) {
    const int64_t r = r0 + tid;
    valid[tid] = (r < n_rows && (mask == nullptr || mask[r] != 0)) ? 1 : 0;
  }
  __syncthreads();
  // 128 rows x 16 groups of 4 features: 8 per thread, 16 lanes per row
#pragma unroll
  for (int i = 0; i < (ZR * ZT / 4) / 256; ++i) {
    const int task = tid + 256 * i;
    const int rr = task >> 4, g = task & 15;
    const int c = c0 + 4 * g;
    float e4[4] = {0.f, 0.f, 0.f, 0.f};
    if (valid[rr] && c < n_cols) {
      const float* src = x + (r0 + rr) * ld + c;
      if (kVec) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(src));
        e4[0] = v.x;
        e4[1] = v.y;
        e4[2] = v.z;
        e4[3] = v.w;
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          if (c + e < n_cols) e4[e] = __ldg(src + e);
      }
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int cc = 4 * g + e;
      t[rr][cc] = (valid[rr] && c + e < n_cols) ? __fdiv_rn(e4[e] - smu[cc], ssg[cc]) : 0.f;
    }
  }
  __syncthreads();
  // column sums of z over each 64-row half, rows in order
  if (tid < 2 * ZT) {
    const int c = tid & (ZT - 1), hh = tid >> 6;
    if (r0 + hh * ZT < n_pad) {
      float s = 0.f;
      for (int rr = 0; rr < ZT; ++rr) s += t[hh * ZT + rr][c];
      zpart[(int64_t(blockIdx.x) * 2 + hh) * h_pad + c0 + c] = s;
    }
  }
  // transposed split writes: feature cc, cells 2p and 2p+1 of the tile
  for (int task = tid; task < ZT * (ZR / 2); task += 256) {
    const int cc = task >> 6, p = task & 63;
    const int rr = 2 * p;
    if (r0 + rr >= n_pad) continue;
    __nv_bfloat16 h2[2], l2[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float z = valid[rr + e] ? t[rr + e][cc] - dl[cc] : 0.f;
      h2[e] = __float2bfloat16_rn(z);
      l2[e] = __float2bfloat16_rn(z - __bfloat162float(h2[e]));
    }
    const int64_t o = int64_t(c0 + cc) * n_pad + r0 + rr;
    *reinterpret_cast<__nv_bfloat162*>(hi + o) = __halves2bfloat162(h2[0], h2[1]);
    *reinterpret_cast<__nv_bfloat162*>(lo + o) = __halves2bfloat162(l2[0], l2[1]);
  }
}

// tile t of the 128 x 256 tiles whose column block reaches the diagonal
__device__ __forceinline__ int2 cov_tile(int t, int TI, int TJ) {
  for (int i = 0; i < TI; ++i) {
    const int j0 = (i * BM) / BN;
    const int cnt = TJ - j0;
    if (t < cnt) return make_int2(i, j0 + t);
    t -= cnt;
  }
  return make_int2(TI - 1, TJ - 1);
}

__global__ void __launch_bounds__(192, 1)
cov_tc_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
              const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, int TI, int TJ,
              int64_t steps_per_split, int64_t total_steps, float* __restrict__ part, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = su32(smem_raw);
  uint8_t* sm = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + STAGES * STAGE_BYTES);
  uint64_t* fullH = bars;                   // [STAGES]: A hi and B hi landed
  uint64_t* fullBl = bars + STAGES;         // [STAGES]: B lo landed
  uint64_t* fullAl = bars + 2 * STAGES;     // [STAGES]: A lo landed
  uint64_t* empty = bars + 3 * STAGES;
  uint64_t* acc_full = bars + 4 * STAGES;   // [2]: chunk accumulated in TMEM buffer b
  uint64_t* acc_empty = acc_full + 2;       // [2]: buffer b read out by the 4 epilogue warps
  uint64_t* mma_done = acc_empty + 2;       // every MMA of this CTA has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int2 tile = cov_tile(blockIdx.x, TI, TJ);
  const int64_t k_begin = int64_t(blockIdx.y) * steps_per_split;
  const int64_t k_end = min(total_steps, k_begin + steps_per_split);
  const int nsteps = int(k_end - k_begin);
  const int nchunks = (nsteps + CHUNK_STEPS - 1) / CHUNK_STEPS;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&fullH[s], 1);
      mbar_init(&fullBl[s], 1);
      mbar_init(&fullAl[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);
    }
    mbar_init(mma_done, 1);
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
      tma_prefetch(&mAh);
      tma_prefetch(&mAl);
      tma_prefetch(&mBh);
      tma_prefetch(&mBl);
      int issued = 0;
      for (int t = 0; t < nsteps; ++t) {
        const int s = t % STAGES;
        const uint32_t ph = (t / STAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) break;
        uint8_t* st = sm + s * STAGE_BYTES;
        const int kx = int((k_begin + t) * BK);
        // hi halves first: the hi.hi products start while the lo halves land
        mbar_expect_tx(&fullH[s], A_BYTES + B_BYTES);
        tma_load_2d(st, &mAh, &fullH[s], kx, tile.x * BM);
        tma_load_2d(st + 2 * A_BYTES, &mBh, &fullH[s], kx, tile.y * BN);
        mbar_expect_tx(&fullBl[s], B_BYTES);
        tma_load_2d(st + 2 * A_BYTES + B_BYTES, &mBl, &fullBl[s], kx, tile.y * BN);
        mbar_expect_tx(&fullAl[s], A_BYTES);
        tma_load_2d(st + A_BYTES, &mAl, &fullAl[s], kx, tile.x * BM);
        ++issued;
      }
      if (*reinterpret_cast<volatile int*>(err)) {
        for (int t = max(0, issued - STAGES); t < issued; ++t)
          for (uint64_t* fb : {fullH, fullBl, fullAl})
            for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(&fb[t % STAGES], (t / STAGES) & 1); ++it) {
            }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      for (int t = 0; t < nsteps; ++t) {
        const int c = t / CHUNK_STEPS, tl = t - c * CHUNK_STEPS, b = c & 1;
        const uint32_t dacc = tmem + uint32_t(b) * ACC_COLS;
        if (tl == 0) {
          // the epilogue has read this buffer's previous chunk (first use: passes)
          if (!mbar_wait(&acc_empty[b], ((c >> 1) & 1) ^ 1u, err, 4)) break;
          tc_fence_after();
        }
        const int s = t % STAGES;
        const uint32_t ph = (t / STAGES) & 1;
        uint8_t* st = sm + s * STAGE_BYTES;
        const uint64_t ah = smem_desc_sw128(su32(st));
        const uint64_t al = smem_desc_sw128(su32(st + A_BYTES));
        const uint64_t bh = smem_desc_sw128(su32(st + 2 * A_BYTES));
        const uint64_t bl = smem_desc_sw128(su32(st + 2 * A_BYTES + B_BYTES));
        if (!mbar_wait(&fullH[s], ph, err, 2)) break;
        tc_fence_after();
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk)
          mma_bf16(dacc, ah + uint64_t(2 * kk), bh + uint64_t(2 * kk), kIdesc, (tl > 0 || kk > 0) ? 1u : 0u);
        if (!mbar_wait(&fullBl[s], ph, err, 2)) break;
        tc_fence_after();
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) mma_bf16(dacc, ah + uint64_t(2 * kk), bl + uint64_t(2 * kk), kIdesc, 1u);
        if (!mbar_wait(&fullAl[s], ph, err, 2)) break;
        tc_fence_after();
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) mma_bf16(dacc, al + uint64_t(2 * kk), bh + uint64_t(2 * kk), kIdesc, 1u);
        mma_commit(&empty[s]);
        if (tl == CHUNK_STEPS - 1 || t == nsteps - 1) mma_commit(&acc_full[b]);
      }
      // TMEM is released only after every MMA issued above has completed
      mma_commit(mma_done);
      for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(mma_done, 0); ++it) {
      }
    }
  } else {
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;
    // the CTA's partial tile as two column-major float planes (hi, lo): a
    // warp's 32 rows of one column are 128 contiguous bytes in each
    float* P = part + (int64_t(blockIdx.y) * gridDim.x + blockIdx.x) * (2 * TILE_ELEMS) + row;
    const uint32_t tq = tmem + (uint32_t(quarter * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < nchunks; ++c) {
      const int b = c & 1;
      const bool ok = mbar_wait(&acc_full[b], (c >> 1) & 1, err, 3);
      if (!__all_sync(0xffffffffu, ok)) break;
      tc_fence_after();
      const uint32_t tb = tq + uint32_t(b) * ACC_COLS;
#pragma unroll 1
      for (int ch = 0; ch < BN / 32; ++ch) {
        uint32_t r[32];
        tmem_ld32(tb + uint32_t(ch * 32), r);
        tmem_wait_ld(r);
        float* oh = P + ch * 32 * BM;
        float* ol = oh + TILE_ELEMS;
        if (c == 0) {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            oh[q * BM] = __uint_as_float(r[q]);
            ol[q * BM] = 0.f;
          }
        } else {
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            float hi = oh[q * BM], lo = ol[q * BM];
            pair_add(hi, lo, __uint_as_float(r[q]));
            oh[q * BM] = hi;
            ol[q * BM] = lo;
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
    }
    if (nchunks == 0) {
#pragma unroll 1
      for (int q = 0; q < BN; ++q) P[q * BM] = P[TILE_ELEMS + q * BM] = 0.f;
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// FP64 sum over the splits (fixed order) of the partial tiles; the upper
// triangle is added to cov and mirrored.
__global__ void __launch_bounds__(256)
cov_tc_reduce_kernel(const float* __restrict__ part, int nsplit, int ntile, int TI, int TJ, int n_cols,
                     double* __restrict__ cov) {
  const int t = blockIdx.y;
  const int2 tl = cov_tile(t, TI, TJ);
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= TILE_ELEMS) return;
  const int i = tl.x * BM + (e % BM), j = tl.y * BN + (e / BM);
  if (i >= n_cols || j >= n_cols || j < i) return;
  double s = 0.0;
  for (int p = 0; p < nsplit; ++p) {
    const float* q = part + (int64_t(p) * ntile + t) * (2 * TILE_ELEMS) + e;
    s += double(q[0]) + double(q[TILE_ELEMS]);
  }
  cov[int64_t(j) * n_cols + i] += s;
  if (i != j) cov[int64_t(i) * n_cols + j] += s;
}

// Column sums of z from the 64-row tile partials, in FP64 and a fixed order:
// groups of kZGroup tiles (more for very tall inputs, so that the groups fit
// one grid dimension) in parallel, tiles in order within a group, then the
// groups in order.
constexpr int kZGroup = 128;

__global__ void zpart_group_kernel(const float* __restrict__ zpart, int ntiles, int group, int h_pad, int n_cols,
                                   double* __restrict__ gsum) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cols) return;
  const int t0 = blockIdx.y * group, t1 = min(ntiles, t0 + group);
  double s = 0.0;
  for (int t = t0; t < t1; ++t) s += double(zpart[int64_t(t) * h_pad + j]);
  gsum[int64_t(blockIdx.y) * n_cols + j] = s;
}

__global__ void zpart_reduce_kernel(const double* __restrict__ gsum, int ngroups, int n_cols,
                                    double* __restrict__ zsum, double* __restrict__ zcall) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_cols) return;
  double s = 0.0;
  for (int g = 0; g < ngroups; ++g) s += gsum[int64_t(g) * n_cols + j];
  zsum[j] += s;
  zcall[j] = s;
}

__global__ void count_rows_kernel(const uint8_t* __restrict__ mask, int64_t n_rows,
                                  unsigned long long* __restrict__ count) {
  unsigned long long c = 0;
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n_rows; r += int64_t(gridDim.x) * blockDim.x)
    c += mask[r] != 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// Undo the zero shift: with z' = z - delta over the m valid rows and Z = sum z,
// sum z_a z_b = sum z'_a z'_b + delta_b Z_a + delta_a Z_b - m delta_a delta_b.
// The expression is symmetric in (a, b) term by term, so cov stays symmetric.
__global__ void cov_shift_kernel(const float* __restrict__ mu, const float* __restrict__ sg,
                                 const double* __restrict__ zcall, const unsigned long long* __restrict__ count,
                                 int64_t n_valid, int n_cols, double* __restrict__ cov) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (b >= n_cols) return;
  const double m = count ? double(*count) : double(n_valid);
  const double da = double(zero_shift(mu[a], sg[a])), db = double(zero_shift(mu[b], sg[b]));
  cov[int64_t(a) * n_cols + b] += (db * zcall[a] + da * zcall[b]) - m * (da * db);
}

}  // namespace

int sg_covariance_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld, const float* mu32,
                     const float* sigma32, const uint8_t* row_mask, double* cov, double* zsum, cudaStream_t st) {
  const int h_pad = int(sg::ceil_div(n_cols, BN) * BN);
  const int64_t n_pad = sg::ceil_div(n_rows, BK) * BK;
  const int64_t total_steps = n_pad / BK;
  if (n_pad >= (int64_t(1) << 31)) return sg::fail(SG_ERR_ARG, "sg_covariance: too many rows for one call");
  const int TI = h_pad / BM, TJ = h_pad / BN;
  int ntile = 0;
  for (int i = 0; i < TI; ++i) ntile += TJ - (i * BM) / BN;
  // K splits: enough CTAs for several waves, at least 8 steps each
  int64_t want = std::max<int64_t>(1, (int64_t(h->sm_count) * 6 + ntile - 1) / ntile);
  int64_t sps = std::max<int64_t>(8, sg::ceil_div(total_steps, want));
  const int nsplit = int(sg::ceil_div(total_steps, sps));
  const int zt = int(n_pad / ZT);
  const int zgroup = std::max(kZGroup, sg::ceil_div_i(zt, 65535));
  const size_t need = 2 * sg::Carver::need(size_t(h_pad) * n_pad * 2) +
                      sg::Carver::need(size_t(nsplit) * ntile * TILE_ELEMS * 2 * sizeof(float)) +
                      sg::Carver::need(size_t(zt) * h_pad * 4) + sg::Carver::need(size_t(n_cols) * 8) +
                      sg::Carver::need(size_t(sg::ceil_div_i(zt, zgroup)) * n_cols * 8) +
                      sg::Carver::need(sizeof(unsigned long long)) +
                      sg::Carver::need(sizeof(int));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  __nv_bfloat16* zh = cv.take<__nv_bfloat16>(size_t(h_pad) * n_pad);
  __nv_bfloat16* zl = cv.take<__nv_bfloat16>(size_t(h_pad) * n_pad);
  float* part = cv.take<float>(size_t(nsplit) * ntile * TILE_ELEMS * 2);
  float* zpart = cv.take<float>(size_t(zt) * h_pad);
  double* zcall = cv.take<double>(size_t(n_cols));
  const int zgroups = sg::ceil_div_i(zt, zgroup);
  double* gsum = cv.take<double>(size_t(zgroups) * n_cols);
  unsigned long long* count = cv.take<unsigned long long>(1);
  int* err = cv.take<int>(1);
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (row_mask) {
    SG_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
    count_rows_kernel<<<std::min<int64_t>(4 * h->sm_count, sg::ceil_div(n_rows, 256)), 256, 0, st>>>(row_mask, n_rows,
                                                                                                 count);
    SG_LAUNCH_CHECK();
  }
  {
    sg::ProfScope prof(h, "zsplit", st);
    const dim3 zgrid(unsigned(sg::ceil_div(n_pad, ZR)), unsigned(h_pad / ZT));
    if (ld % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0)
      zsplit_kernel<true><<<zgrid, 256, 0, st>>>(x, n_rows, n_cols, ld, mu32, sigma32, row_mask, zh, zl, n_pad, zpart,
                                                  h_pad);
    else
      zsplit_kernel<false><<<zgrid, 256, 0, st>>>(x, n_rows, n_cols, ld, mu32, sigma32, row_mask, zh, zl, n_pad, zpart,
                                                   h_pad);
    SG_LAUNCH_CHECK();
  }
  CUtensorMap mAh, mAl, mBh, mBl;
  int rc = make_map(&mAh, zh, h_pad, BM, n_pad, BK);
  if (!rc) rc = make_map(&mAl, zl, h_pad, BM, n_pad, BK);
  if (!rc) rc = make_map(&mBh, zh, h_pad, BN, n_pad, BK);
  if (!rc) rc = make_map(&mBl, zl, h_pad, BN, n_pad, BK);
  if (rc) return rc;
  {
    sg::ProfScope prof(h, "cov_tc", st);
    SG_CUDA(cudaFuncSetAttribute(cov_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM_BYTES)));
    cov_tc_kernel<<<dim3(unsigned(ntile), unsigned(nsplit)), 192, SMEM_BYTES, st>>>(mAh, mAl, mBh, mBl, TI, TJ, sps,
                                                                                 total_steps, part, err);
    SG_LAUNCH_CHECK();
  }
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_TIMEOUT, "sg_covariance: a tensor-core pipeline wait expired (stage %d)", herr);
  cov_tc_reduce_kernel<<<dim3(unsigned(TILE_ELEMS / 256), unsigned(ntile)), 256, 0, st>>>(part, nsplit, ntile, TI, TJ,
                                                                                         n_cols, cov);
  SG_LAUNCH_CHECK();
  zpart_group_kernel<<<dim3(unsigned(sg::ceil_div_i(n_cols, 256)), unsigned(zgroups)), 256, 0, st>>>(
      zpart, zt, zgroup, h_pad, n_cols, gsum);
  SG_LAUNCH_CHECK();
  zpart_reduce_kernel<<<sg::ceil_div_i(n_cols, 256), 256, 0, st>>>(gsum, zgroups, n_cols, zsum, zcall);
  SG_LAUNCH_CHECK();
  cov_shift_kernel<<<dim3(unsigned(sg::ceil_div_i(n_cols, 256)), unsigned(n_cols)), 256, 0, st>>>(
      mu32, sigma32, zcall, row_mask ? count : nullptr, n_rows, n_cols, cov);
  SG_LAUNCH_CHECK();
  return SG_OK;
}
