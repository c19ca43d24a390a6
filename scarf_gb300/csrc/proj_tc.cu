// a5, precision form: the reducer ((x - mu)/sigma) . L (scarf/ann.py:129-138,
// :191-192) on the tcgen05 tensor cores, as x . L' - b with L' = L / sigma
// per feature and b = mu^T L'.
//
// Persistent CTAs, one per SM, each taking 128-row tiles of x in turn:
//   warp 0       TMA producer: per 64-feature chunk the BF16 hi and lo halves
//                of L'^T (64 score columns x 64 features, 128B swizzle).
//   warp 1       MMA issuer (one thread): per chunk, four K=16 steps of three
//                products hi.hi + hi.lo + lo.hi (M=128, N=64) into one of two
//                TMEM accumulators (64 FP32 columns each), so that the next
//                tile accumulates while the last one is written out.
//   warps 2-9    converters: read the tile's chunk of x once from HBM with
//                16-byte loads, split each value into hi = bf16(x) and
//                lo = bf16(x - hi), and store both into the K-major
//                128B-swizzled layout the MMA reads (16-byte chunk c of row r
//                at r * 128 + ((c ^ (r % 8)) * 16)).
//   warps 10-13  epilogue, one per TMEM lane quarter: read the accumulator,
//                subtract b, write the FP32 scores (and the BF16 copy).
// b is summed in FP64 from the same split L' the MMAs use. Every mbarrier
// wait is bounded: on expiry the kernel raises an error flag, lets its own
// copies and MMAs finish, frees its tensor memory and returns.
#include "tc_ptx.cuh"

namespace {

using namespace tc;

constexpr int PM = 128;                       // rows per tile (TMEM lanes)
constexpr int PN = 64;                        // score columns, d <= 64 (zero padded)
constexpr int PK = 64;                        // features per chunk (one 128-byte BF16 row)
constexpr int PSTAGES = 4;
constexpr uint32_t A_HALF = PM * PK * 2;      // 16 KB
constexpr uint32_t B_HALF = PN * PK * 2;      // 8 KB
constexpr uint32_t STAGE = 2 * A_HALF + 2 * B_HALF;
constexpr int CONV_WARPS = 8;
constexpr int EPI_WARPS = 4;
constexpr int THREADS = 64 + 32 * (CONV_WARPS + EPI_WARPS);
constexpr int CONV_THREADS = 32 * CONV_WARPS;
constexpr uint32_t ACC_COLS = PN;
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
constexpr size_t SMEM_BYTES = 1024 + size_t(PSTAGES) * STAGE + 256 + PN * sizeof(float);
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory budget");
static_assert((PM * PK / 8) % CONV_THREADS == 0, "converter work split");
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(PN >> 3) << 17) | (uint32_t(PM >> 4) << 24);

__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return uint32_t(__bfloat16_as_ushort(a)) | (uint32_t(__bfloat16_as_ushort(b)) << 16);
}

__global__ void __launch_bounds__(THREADS, 1)
proj_tc_kernel(const __grid_constant__ CUtensorMap tmLh, const __grid_constant__ CUtensorMap tmLl,
               const float* __restrict__ x, int64_t n_rows, int n_cols, int64_t ld, int nk, int64_t ntiles,
               const float* __restrict__ bsh, int d, float* __restrict__ scores, int ld_s,
               __nv_bfloat16* __restrict__ sb, int ld_b, bool vec, int* __restrict__ err, uint32_t wait_limit) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = su32(smem_raw);
  uint8_t* sm = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + PSTAGES * STAGE);
  uint64_t* full = bars;
  uint64_t* empty = bars + PSTAGES;
  uint64_t* acc_full = bars + 2 * PSTAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  float* s_b = reinterpret_cast<float*>(sm + PSTAGES * STAGE + 256);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int my_tiles = ntiles > blockIdx.x ? int((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < PSTAGES; ++s) {
      mbar_init(&full[s], CONV_WARPS + 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], EPI_WARPS);
    }
    mbar_init(mma_done, 1);
    fence_barrier_init();
  }
  for (int c = threadIdx.x; c < PN; c += blockDim.x) s_b[c] = c < d ? bsh[c] : 0.f;
  if (warp == 1) {
    tmem_alloc(tmem_slot, TMEM_COLS);
    tmem_relinquish();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int total = my_tiles * nk;  // chunks this CTA streams

  if (warp == 0) {
    if (lane == 0) {
      tma_prefetch(&tmLh);
      tma_prefetch(&tmLl);
      int issued = 0;
      for (int g = 0; g < total; ++g) {
        const int s = g % PSTAGES;
        const uint32_t ph = (g / PSTAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1, wait_limit)) break;
        uint8_t* stg = sm + s * STAGE;
        const int kc = g % nk;
        mbar_expect_tx(&full[s], 2 * B_HALF);
        tma_load_2d(stg + 2 * A_HALF, &tmLh, &full[s], kc * PK, 0);
        tma_load_2d(stg + 2 * A_HALF + B_HALF, &tmLl, &full[s], kc * PK, 0);
        ++issued;
      }
      if (*reinterpret_cast<volatile int*>(err)) {
        // this CTA's own copies land before it leaves
        for (int g = max(0, issued - PSTAGES); g < issued; ++g)
          for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(&full[g % PSTAGES], (g / PSTAGES) & 1); ++it) {
          }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int issued = 0;
      for (int li = 0; li < my_tiles; ++li) {
        const int b = li & 1;
        if (!mbar_wait(&acc_empty[b], ((li >> 1) & 1) ^ 1u, err, 3, wait_limit)) break;
        tc_fence_after();
        const uint32_t dacc = tmem + uint32_t(b) * ACC_COLS;
        bool ok = true;
        for (int kc = 0; kc < nk; ++kc) {
          const int g = li * nk + kc;
          const int s = g % PSTAGES;
          if (!mbar_wait(&full[s], (g / PSTAGES) & 1, err, 2, wait_limit)) {
            ok = false;
            break;
          }
          tc_fence_after();
          uint8_t* stg = sm + s * STAGE;
          const uint64_t ah = smem_desc_sw128(su32(stg));
          const uint64_t al = smem_desc_sw128(su32(stg + A_HALF));
          const uint64_t bh = smem_desc_sw128(su32(stg + 2 * A_HALF));
          const uint64_t bl = smem_desc_sw128(su32(stg + 2 * A_HALF + B_HALF));
#pragma unroll
          for (int kk = 0; kk < PK / 16; ++kk) {
            const uint64_t o = uint64_t(2 * kk);
            mma_bf16(dacc, ah + o, bh + o, kIdesc, (kc > 0 || kk > 0) ? 1u : 0u);
            mma_bf16(dacc, ah + o, bl + o, kIdesc, 1u);
            mma_bf16(dacc, al + o, bh + o, kIdesc, 1u);
          }
          mma_commit(&empty[s]);
          ++issued;
        }
        if (!ok) break;
        mma_commit(&acc_full[b]);
      }
      if (issued > 0) {
        // tensor memory is released only after every MMA issued above has completed
        mma_commit(mma_done);
        for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(mma_done, 0); ++it) {
        }
      }
    }
  } else if (warp < 2 + CONV_WARPS) {
    const int ct = threadIdx.x - 64;
    for (int g = 0; g < total; ++g) {
      const int s = g % PSTAGES;
      const uint32_t ph = (g / PSTAGES) & 1;
      const bool ok = mbar_wait(&empty[s], ph ^ 1u, err, 4, wait_limit);
      if (!__all_sync(0xffffffffu, ok)) break;
      const int li = g / nk, kc = g - li * nk;
      const int64_t row0 = (int64_t(blockIdx.x) + int64_t(li) * gridDim.x) * PM;
      uint8_t* ahi = sm + s * STAGE;
      uint8_t* alo = ahi + A_HALF;
#pragma unroll
      for (int i = 0; i < (PM * PK / 8) / CONV_THREADS; ++i) {
        const int item = ct + CONV_THREADS * i;
        const int r = item >> 3, c8 = item & 7;
        const int64_t grow = row0 + r;
        const int f0 = kc * PK + c8 * 8;
        float v[8];
        if (grow < n_rows && vec && f0 + 8 <= n_cols) {
          const float4* p = reinterpret_cast<const float4*>(x + grow * ld + f0);
          const float4 u0 = __ldcs(p), u1 = __ldcs(p + 1);
          v[0] = u0.x; v[1] = u0.y; v[2] = u0.z; v[3] = u0.w;
          v[4] = u1.x; v[5] = u1.y; v[6] = u1.z; v[7] = u1.w;
        } else {
#pragma unroll
          for (int q = 0; q < 8; ++q) v[q] = (grow < n_rows && f0 + q < n_cols) ? x[grow * ld + f0 + q] : 0.f;
        }
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * q]), h1 = __float2bfloat16_rn(v[2 * q + 1]);
          const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * q] - __bfloat162float(h0));
          const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * q + 1] - __bfloat162float(h1));
          hw[q] = pack2(h0, h1);
          lw[q] = pack2(l0, l1);
        }
        const uint32_t off = uint32_t(r) * 128u + (uint32_t(c8 ^ (r & 7)) << 4);
        *reinterpret_cast<uint4*>(ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      // the generic-proxy stores must be visible to the tensor cores' reads
      fence_async_shared();
      __syncwarp();
      if (lane == 0) mbar_arrive(&full[s]);
    }
  } else {
    const int quarter = warp & 3;
    const uint32_t tq = tmem + (uint32_t(quarter * 32) << 16);
    for (int li = 0; li < my_tiles; ++li) {
      const int b = li & 1;
      const bool ok = mbar_wait(&acc_full[b], (li >> 1) & 1, err, 5, wait_limit);
      if (!__all_sync(0xffffffffu, ok)) break;
      tc_fence_after();
      uint32_t ra[32], rb[32];
      tmem_ld32(tq + uint32_t(b) * ACC_COLS, ra);
      tmem_ld32(tq + uint32_t(b) * ACC_COLS + 32u, rb);
      tmem_wait_ld(ra);
      tmem_wait_ld(rb);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
      const int64_t row = (int64_t(blockIdx.x) + int64_t(li) * gridDim.x) * PM + quarter * 32 + lane;
      if (row < n_rows) {
        float* o = scores + row * ld_s;
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const float v = c < d ? __uint_as_float(ra[c]) - s_b[c] : 0.f;
          if (c < ld_s) o[c] = v;
          if (sb != nullptr && c < ld_b) sb[row * ld_b + c] = __float2bfloat16_rn(v);
        }
#pragma unroll
        for (int c = 32; c < 64; ++c) {
          const float v = c < d ? __uint_as_float(rb[c - 32]) - s_b[c] : 0.f;
          if (c < ld_s) o[c] = v;
          if (sb != nullptr && c < ld_b) sb[row * ld_b + c] = __float2bfloat16_rn(v);
        }
        for (int c = 64; c < ld_s; ++c) o[c] = 0.f;
        if (sb != nullptr)
          for (int c = 64; c < ld_b; ++c) sb[row * ld_b + c] = __float2bfloat16_rn(0.f);
      }
    }
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// L'^T = (L / sigma)^T split into BF16 hi and lo (PN x k_pad, zero padded),
// and b = mu^T (hi + lo) summed in FP64; one CTA per score column.
__global__ void split_loadings_kernel(const float* __restrict__ L, int h, int ld_l, int d,
                                      const float* __restrict__ mu, const float* __restrict__ sg, int k_pad,
                                      __nv_bfloat16* __restrict__ lh, __nv_bfloat16* __restrict__ ll,
                                      float* __restrict__ b) {
  __shared__ double part[256];
  const int c = blockIdx.x;
  double acc = 0.0;
  for (int j = threadIdx.x; j < k_pad; j += blockDim.x) {
    const float lp = (c < d && j < h) ? __fdiv_rn(L[int64_t(j) * ld_l + c], sg[j]) : 0.f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(lp);
    const __nv_bfloat16 lo = __float2bfloat16_rn(lp - __bfloat162float(hi));
    lh[int64_t(c) * k_pad + j] = hi;
    ll[int64_t(c) * k_pad + j] = lo;
    if (j < h) acc += double(mu[j]) * (double(__bfloat162float(hi)) + double(__bfloat162float(lo)));
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) b[c] = float(part[0]);
}

}  // namespace

int sg_project_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld, const float* mu32,
                  const float* sigma32, const float* loadings32, int32_t d, int32_t ld_l, float* scores, int32_t ld_s,
                  __nv_bfloat16* sb, int32_t ld_b, cudaStream_t st) {
  if (d > PN) return sg::fail(SG_ERR_ARG, "sg_project: the precision form supports d <= %d", PN);
  const int nk = sg::ceil_div_i(n_cols, PK);
  const int k_pad = nk * PK;
  const int64_t ntiles = sg::ceil_div(n_rows, PM);
  const size_t need = 2 * sg::Carver::need(size_t(PN) * k_pad * 2) + sg::Carver::need(sizeof(float) * PN) +
                      sg::Carver::need(sizeof(int));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  __nv_bfloat16* lh = cv.take<__nv_bfloat16>(size_t(PN) * k_pad);
  __nv_bfloat16* ll = cv.take<__nv_bfloat16>(size_t(PN) * k_pad);
  float* bsh = cv.take<float>(PN);
  int* err = cv.take<int>(1);
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  sg::ProfScope prof(h, "project", st);
  split_loadings_kernel<<<PN, 256, 0, st>>>(loadings32, n_cols, ld_l, d, mu32, sigma32, k_pad, lh, ll, bsh);
  SG_LAUNCH_CHECK();
  CUtensorMap tmh, tml;
  int rc = make_map(&tmh, lh, PN, PN, k_pad, PK);
  if (!rc) rc = make_map(&tml, ll, PN, PN, k_pad, PK);
  if (rc) return rc;
  // 16-byte loads of x need a 16-byte aligned base and a row stride of whole float4s
  const bool vec = (reinterpret_cast<uintptr_t>(x) & 15u) == 0 && (ld & 3) == 0;
  const unsigned grid = unsigned(std::min<int64_t>(ntiles, h->sm_count));
  const uint32_t wl = h->wait_limit ? h->wait_limit : WAIT_LIMIT;
  SG_CUDA(cudaFuncSetAttribute(proj_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM_BYTES)));
  proj_tc_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(tmh, tml, x, n_rows, n_cols, ld, nk, ntiles, bsh, d, scores, ld_s,
                                                    sb, ld_b, vec, err, wl);
  SG_LAUNCH_CHECK();
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_TIMEOUT, "sg_project: a tensor-core pipeline wait expired (stage %d)", herr);
  return SG_OK;
}
