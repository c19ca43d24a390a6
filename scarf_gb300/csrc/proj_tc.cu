// a5, precision form: the reducer ((x - mu)/sigma) . L (scarf/ann.py:129-138,
// :191-192) on the tcgen05 tensor cores, as x . L' - b with L' = L / sigma
// per feature and b = mu^T L'.
//
// Persistent CTAs, one per SM, each taking 128-row tiles of x in turn:
//   warp 0       TMA producer of x: per 64-feature chunk of the tile, the
//                fp32 block (128 rows x 64 features, 32 KB; rows and features
//                past the matrix read as zeros) into a 3-stage staging ring.
//   warp 1       MMA issuer (one thread): per chunk, four K=16 steps of three
//                products hi.hi + hi.lo + lo.hi (M=128, N=64) into one of two
//                TMEM accumulators (64 FP32 columns each), so that the next
//                tile accumulates while the last one is written out.
//   warp 2       TMA producer of the loadings: per chunk the BF16 hi and lo
//                halves of L'^T (64 score columns x 64 features, 128B swizzle).
//   warps 3-10   converters: split each staged value into hi = bf16(x) and
//                lo = bf16(x - hi) and store both into the K-major
//                128B-swizzled layout the MMA reads (16-byte chunk c of row r
//                at r * 128 + ((c ^ (r % 8)) * 16)).
//   warps 11-14  epilogue, one per TMEM lane quarter: read the accumulator,
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
constexpr int XSTAGES = 3;                    // fp32 staging ring
constexpr int PSTAGES = 2;                    // BF16 operand ring
constexpr uint32_t X_BYTES = PM * PK * 4;     // 32 KB
constexpr uint32_t A_HALF = PM * PK * 2;      // 16 KB
constexpr uint32_t B_HALF = PN * PK * 2;      // 8 KB
constexpr uint32_t STAGE = 2 * A_HALF + 2 * B_HALF;
constexpr int CONV_WARPS = 8;
constexpr int EPI_WARPS = 4;
constexpr int CONV0 = 3;                      // first converter warp
constexpr int EPI0 = CONV0 + CONV_WARPS;      // first epilogue warp
constexpr int THREADS = 32 * (EPI0 + EPI_WARPS);
constexpr int CONV_THREADS = 32 * CONV_WARPS;
constexpr uint32_t ACC_COLS = PN;
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
constexpr size_t SMEM_BYTES = 1024 + size_t(XSTAGES) * X_BYTES + size_t(PSTAGES) * STAGE + 256 + PN * sizeof(float);
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory budget");
static_assert((PM * PK / 4) % CONV_THREADS == 0, "converter work split");
static_assert(EPI0 % 4 == 3, "the epilogue warps cover the four TMEM lane quarters");
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(PN >> 3) << 17) | (uint32_t(PM >> 4) << 24);

__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return uint32_t(__bfloat16_as_ushort(a)) | (uint32_t(__bfloat16_as_ushort(b)) << 16);
}

__global__ void __launch_bounds__(THREADS, 1)
proj_tc_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmLh,
               const __grid_constant__ CUtensorMap tmLl, int64_t n_rows, int nk, int64_t ntiles,
               const float* __restrict__ bsh, int d, float* __restrict__ scores, int ld_s,
               __nv_bfloat16* __restrict__ sb, int ld_b, int* __restrict__ err, uint32_t wait_limit) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = su32(smem_raw);
  uint8_t* sm = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* xs = sm;                                        // [XSTAGES][X_BYTES]
  uint8_t* ab = sm + XSTAGES * X_BYTES;                    // [PSTAGES][STAGE]
  uint64_t* bars = reinterpret_cast<uint64_t*>(ab + PSTAGES * STAGE);
  uint64_t* x_full = bars;
  uint64_t* x_empty = x_full + XSTAGES;
  uint64_t* full = x_empty + XSTAGES;
  uint64_t* empty = full + PSTAGES;
  uint64_t* acc_full = empty + PSTAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  float* s_b = reinterpret_cast<float*>(ab + PSTAGES * STAGE + 256);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int my_tiles = ntiles > blockIdx.x ? int((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < XSTAGES; ++s) {
      mbar_init(&x_full[s], 1);
      mbar_init(&x_empty[s], CONV_WARPS);
    }
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

  if (warp == 0 || warp == 2) {
    // the two TMA producers: x (warp 0) and the loadings (warp 2)
    if (lane == 0) {
      const bool is_x = warp == 0;
      const int nst = is_x ? XSTAGES : PSTAGES;
      uint64_t* fb = is_x ? x_full : full;
      uint64_t* eb = is_x ? x_empty : empty;
      if (is_x) tma_prefetch(&tmX);
      else {
        tma_prefetch(&tmLh);
        tma_prefetch(&tmLl);
      }
      int issued = 0;
      for (int g = 0; g < total; ++g) {
        const int s = g % nst;
        if (!mbar_wait(&eb[s], ((g / nst) & 1) ^ 1u, err, is_x ? 1 : 6, wait_limit)) break;
        const int li = g / nk, kc = g - li * nk;
        if (is_x) {
          const int64_t row0 = (int64_t(blockIdx.x) + int64_t(li) * gridDim.x) * PM;
          mbar_expect_tx(&fb[s], X_BYTES);
          tma_load_2d(xs + s * X_BYTES, &tmX, &fb[s], kc * PK, int(row0));
        } else {
          uint8_t* stg = ab + s * STAGE;
          mbar_expect_tx(&fb[s], 2 * B_HALF);
          tma_load_2d(stg + 2 * A_HALF, &tmLh, &fb[s], kc * PK, 0);
          tma_load_2d(stg + 2 * A_HALF + B_HALF, &tmLl, &fb[s], kc * PK, 0);
        }
        ++issued;
      }
      if (*reinterpret_cast<volatile int*>(err)) {
        // this CTA's own copies land before it leaves
        for (int g = max(0, issued - nst); g < issued; ++g)
          for (uint32_t it = 0; it < WAIT_LIMIT && !mbar_try_wait(&fb[g % nst], (g / nst) & 1); ++it) {
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
          uint8_t* stg = ab + s * STAGE;
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
  } else if (warp < EPI0) {
    // thread t of a pair (t, t^1) reads one float4 of a row; together the
    // pair holds the 8 values of one 16-byte BF16 chunk: the even thread
    // stores its hi chunk, the odd thread the lo chunk
    const int ct = threadIdx.x - 32 * CONV0;
    const bool odd = lane & 1;
    for (int g = 0; g < total; ++g) {
      const int xsg = g % XSTAGES, s = g % PSTAGES;
      bool ok = mbar_wait(&x_full[xsg], (g / XSTAGES) & 1, err, 4, wait_limit);
      ok = ok && mbar_wait(&empty[s], ((g / PSTAGES) & 1) ^ 1u, err, 7, wait_limit);
      if (!__all_sync(0xffffffffu, ok)) break;
      const float* xst = reinterpret_cast<const float*>(xs + xsg * X_BYTES);
      uint8_t* ahi = ab + s * STAGE;
      uint8_t* alo = ahi + A_HALF;
#pragma unroll
      for (int i = 0; i < (PM * PK / 4) / CONV_THREADS; ++i) {
        const int item = ct + CONV_THREADS * i;       // float4 index within the block
        const int r = item >> 4, q = item & 15;       // row, float4 within the row
        const float4 v = *reinterpret_cast<const float4*>(xst + r * PK + q * 4);
        const float f[4] = {v.x, v.y, v.z, v.w};
        uint32_t hw[2], lw[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const __nv_bfloat16 h0 = __float2bfloat16_rn(f[2 * j]), h1 = __float2bfloat16_rn(f[2 * j + 1]);
          hw[j] = pack2(h0, h1);
          lw[j] = pack2(__float2bfloat16_rn(f[2 * j] - __bfloat162float(h0)),
                        __float2bfloat16_rn(f[2 * j + 1] - __bfloat162float(h1)));
        }
        // even thread: its hi words + the partner's hi words; odd: partner's lo + its lo
        const uint32_t s0 = odd ? hw[0] : lw[0], s1 = odd ? hw[1] : lw[1];
        const uint32_t p0 = __shfl_xor_sync(0xffffffffu, s0, 1), p1 = __shfl_xor_sync(0xffffffffu, s1, 1);
        const int c8 = q >> 1;
        const uint32_t off = uint32_t(r) * 128u + (uint32_t(c8 ^ (r & 7)) << 4);
        if (!odd) *reinterpret_cast<uint4*>(ahi + off) = make_uint4(hw[0], hw[1], p0, p1);
        else *reinterpret_cast<uint4*>(alo + off) = make_uint4(p0, p1, lw[0], lw[1]);
      }
      // the generic-proxy stores must be visible to the tensor cores' reads
      fence_async_shared();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&full[s]);
        mbar_arrive(&x_empty[xsg]);
      }
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

// 2-D FP32 tensor map over x (n_rows x n_cols, row stride ld floats), box 64
// features x 128 rows, no swizzle; reads past the matrix fill with zeros
int make_x_map(CUtensorMap* tm, const float* x, int64_t n_rows, int n_cols, int64_t ld) {
  auto fn = encode_fn();
  if (!fn) return sg::fail(SG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t gdim[2] = {cuuint64_t(n_cols), cuuint64_t(n_rows)};
  cuuint64_t gstride[1] = {cuuint64_t(ld) * 4};
  cuuint32_t box[2] = {cuuint32_t(PK), cuuint32_t(PM)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(x), gdim, gstride, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return sg::fail(SG_ERR_CUDA, "cuTensorMapEncodeTiled (x) failed (%d)", int(r));
  return SG_OK;
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

bool sg_project_tc_supported(const float* x, int64_t ld, int d) {
  // the TMA map of x needs a 16-byte aligned base and a row stride of whole 16-byte units
  return d <= PN && (reinterpret_cast<uintptr_t>(x) & 15u) == 0 && (ld & 3) == 0;
}

int sg_project_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld, const float* mu32,
                  const float* sigma32, const float* loadings32, int32_t d, int32_t ld_l, float* scores, int32_t ld_s,
                  __nv_bfloat16* sb, int32_t ld_b, cudaStream_t st) {
  if (!sg_project_tc_supported(x, ld, d))
    return sg::fail(SG_ERR_ARG, "sg_project: the precision form needs d <= %d and 16-byte aligned rows of x", PN);
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
  CUtensorMap tmx, tmh, tml;
  int rc = make_x_map(&tmx, x, n_rows, n_cols, ld);
  if (!rc) rc = make_map(&tmh, lh, PN, PN, k_pad, PK);
  if (!rc) rc = make_map(&tml, ll, PN, PN, k_pad, PK);
  if (rc) return rc;
  const unsigned grid = unsigned(std::min<int64_t>(ntiles, h->sm_count));
  const uint32_t wl = h->wait_limit ? h->wait_limit : WAIT_LIMIT;
  SG_CUDA(cudaFuncSetAttribute(proj_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM_BYTES)));
  proj_tc_kernel<<<grid, THREADS, SMEM_BYTES, st>>>(tmx, tmh, tml, n_rows, nk, ntiles, bsh, d, scores, ld_s, sb, ld_b,
                                                    err, wl);
  SG_LAUNCH_CHECK();
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_TIMEOUT, "sg_project: a tensor-core pipeline wait expired (stage %d)", herr);
  return SG_OK;
}
