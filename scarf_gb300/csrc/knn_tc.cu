// a6/a7 precision form: BF16 distance tiles on the tcgen05 tensor cores.
//
// One CTA owns 128 queries (one TMEM lane each) and a range of reference rows.
//   warp 0      TMA producer: the BF16 query tile once, then 256-row reference
//               tiles into a 4-stage shared-memory ring (128B swizzle, K = 64).
//   warp 1      MMA issuer (one thread): D[128x256] = Q . R^T as four
//               tcgen05.mma kind::f16 K=16 steps into one of two TMEM
//               accumulators (2 x 256 columns), committed to the ring's empty
//               barrier and to the accumulator's full barrier.
//   warps 2-5   epilogue: tcgen05.ld 32 columns at a time, ranking key
//               |r|^2 - 2 q.r, threshold test, register top-KC insertion; the
//               accumulator is handed back as soon as it has been read, so the
//               MMA of tile t+1 overlaps the epilogue of tile t.
// Every mbarrier wait is bounded: on expiry the kernel raises an error flag,
// drains its own TMA copies and MMAs (again bounded), frees TMEM and returns.
// The candidates are re-ranked exactly in FP32 by knn.cu.
#include "common.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

int sg_rerank(const float* queries, const float* refs, int d, int ld, int64_t nq, const int* cand, int nlists, int kc,
              int64_t nq_pad, int kq, int k, int64_t self_offset, int64_t* idx_out, float* dist_out,
              unsigned long long* nmiss, cudaStream_t st);  // knn.cu

namespace {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BK = 64;
constexpr int STAGES = 4;
constexpr uint32_t A_BYTES = BM * BK * 2;
constexpr uint32_t B_BYTES = BN * BK * 2;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr size_t SMEM_BYTES = 1024 /*align*/ + A_BYTES + STAGES * B_BYTES + 256 /*barriers*/ + 4 * BN * 4 /*rn*/;

__device__ __forceinline__ uint32_t su32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the limit expires (the error flag is then raised)
// or when another thread has already raised it.
__device__ __noinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err, int code) {
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(b, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*reinterpret_cast<volatile int*>(err)) return false;
      if (it >= WAIT_LIMIT) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
          "r"(su32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(su32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void tma_prefetch(const CUtensorMap* tm) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tm)) : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "setp.ne.b32 P, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, P;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;            // leading byte offset (unused for this layout)
  d |= uint64_t(1024 >> 4) << 32;    // stride byte offset
  d |= uint64_t(1) << 46;            // version
  d |= uint64_t(2) << 61;            // SWIZZLE_128B
  return d;
}
// Instruction descriptor, kind::f16: D F32, A/B BF16, both K-major, N, M.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);

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

template <int KC>
__global__ void __launch_bounds__(192, 1)
knn_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              const float* __restrict__ rn, int64_t nr, int64_t rps, int* __restrict__ cand, int64_t nq_pad,
              int* __restrict__ err) {
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

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t q0 = int64_t(blockIdx.x) * BM;
  const int64_t s_begin = int64_t(blockIdx.y) * rps;
  const int64_t s_end = min(nr, s_begin + rps);
  const int ntiles = int((s_end - s_begin + BN - 1) / BN);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);
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
        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) break;
        mbar_expect_tx(&full[s], B_BYTES);
        tma_load_2d(sB + s * B_BYTES, &tmB, &full[s], 0, int(s_begin + int64_t(t) * BN));
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
    if (lane == 0) {
      int issued = 0;
      if (mbar_wait(a_full, 0, err, 2)) {
        tc_fence_after();
        const uint64_t adesc = smem_desc_sw128(su32(sA));
        for (int t = 0; t < ntiles; ++t) {
          const int s = t % STAGES;
          const uint32_t ph = (t / STAGES) & 1;
          const int b = t & 1;
          const uint32_t aph = (t >> 1) & 1;
          if (!mbar_wait(&acc_empty[b], aph ^ 1u, err, 3)) break;
          if (!mbar_wait(&full[s], ph, err, 4)) break;
          tc_fence_after();
          const uint64_t bdesc = smem_desc_sw128(su32(sB + s * B_BYTES));
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(tmem + uint32_t(b * BN), adesc + uint64_t(2 * kk), bdesc + uint64_t(2 * kk), kIdesc,
                     kk > 0 ? 1u : 0u);
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
    const int quarter = warp & 3;  // TMEM lanes [32*quarter, 32*quarter+32) are this warp's
    const int row = quarter * 32 + lane;
    float* my_rn = rn_s + (warp - 2) * BN;
    TopK<KC> top;
    top.init();
    for (int t = 0; t < ntiles; ++t) {
      const int b = t & 1;
      const uint32_t aph = (t >> 1) & 1;
      const int64_t r0 = s_begin + int64_t(t) * BN;
      const float4* src = reinterpret_cast<const float4*>(rn + r0);
      reinterpret_cast<float4*>(my_rn)[lane * 2] = __ldg(src + lane * 2);
      reinterpret_cast<float4*>(my_rn)[lane * 2 + 1] = __ldg(src + lane * 2 + 1);
      bool ok = mbar_wait(&acc_full[b], aph, err, 5);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      tc_fence_after();
      __syncwarp();
      const uint32_t tbase = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b * BN);
#pragma unroll 1
      for (int ch = 0; ch < BN / 32; ++ch) {
        uint32_t r[32];
        __syncwarp();
        tmem_ld32(tbase + uint32_t(ch * 32), r);
        tmem_wait_ld();
        const float* nrm = my_rn + ch * 32;
        const int cbase = int(r0) + ch * 32;
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          const float4 nv = *reinterpret_cast<const float4*>(nrm + j);
          const float k0 = fmaf(-2.f, __uint_as_float(r[j]), nv.x);
          const float k1 = fmaf(-2.f, __uint_as_float(r[j + 1]), nv.y);
          const float k2 = fmaf(-2.f, __uint_as_float(r[j + 2]), nv.z);
          const float k3 = fmaf(-2.f, __uint_as_float(r[j + 3]), nv.w);
          if (fminf(fminf(k0, k1), fminf(k2, k3)) < top.worst()) {
            if (k0 < top.worst()) top.insert(k0, cbase + j);
            if (k1 < top.worst()) top.insert(k1, cbase + j + 1);
            if (k2 < top.worst()) top.insert(k2, cbase + j + 2);
            if (k3 < top.worst()) top.insert(k3, cbase + j + 3);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
      __syncwarp();
    }
    int* out = cand + (int64_t(blockIdx.y) * nq_pad + q0 + row) * KC;
#pragma unroll
    for (int j = 0; j < KC; ++j) out[j] = top.i[j];
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// BF16 copy of float32 rows, zero padded to 64 columns and to n_pad rows;
// norms are those of the rounded rows (+inf for padding rows).
__global__ void to_bf16_kernel(const float* __restrict__ in, int64_t n, int d, int ld, __nv_bfloat16* __restrict__ out,
                               int64_t n_pad, float* __restrict__ norms) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n_pad) return;
  float s = 0.f;
  __nv_bfloat16* o = out + r * BK;
  for (int c = 0; c < BK; ++c) {
    const float v = (r < n && c < d) ? in[r * ld + c] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    o[c] = b;
    const float bf = __bfloat162float(b);
    s = fmaf(bf, bf, s);
  }
  if (norms) norms[r] = r < n ? s : __int_as_float(0x7f800000);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int make_map(CUtensorMap* tm, const void* base, int64_t rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return sg::fail(SG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t gdim[2] = {cuuint64_t(BK), cuuint64_t(rows)};
  cuuint64_t gstride[1] = {cuuint64_t(BK) * 2};
  cuuint32_t box[2] = {cuuint32_t(BK), cuuint32_t(box_rows)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), gdim, gstride, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return sg::fail(SG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
  return SG_OK;
}

template <int KC>
int launch_tc(const CUtensorMap& a, const CUtensorMap& b, const float* rn, int64_t nr, int64_t rps, int nsplit,
              int* cand, int64_t nq_pad, int* err, cudaStream_t st) {
  SG_CUDA(cudaFuncSetAttribute(knn_tc_kernel<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SMEM_BYTES)));
  dim3 grid(unsigned(nq_pad / BM), unsigned(nsplit));
  knn_tc_kernel<KC><<<grid, 192, SMEM_BYTES, st>>>(a, b, rn, nr, rps, cand, nq_pad, err);
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
  kc = kc <= 16 ? 16 : kc <= 32 ? 32 : kc <= 48 ? 48 : 64;
  const int64_t nq_pad = sg::ceil_div(nq, BM) * BM;
  const int64_t nr_pad = sg::ceil_div(nr, BN) * BN;
  if (nr_pad >= (int64_t(1) << 31) || nq_pad >= (int64_t(1) << 31)) return sg::fail(SG_ERR_ARG, "sg_knn: too many rows");
  const int qtiles = int(nq_pad / BM);
  int nsplit = std::max<int>(1, int(std::lround(double(h->sm_count) * 8 / qtiles)));
  nsplit = int(std::min<int64_t>(nsplit, std::max<int64_t>(1, nr_pad / (BN * 4))));
  nsplit = std::min(nsplit, 256);
  const int64_t rps = sg::ceil_div(sg::ceil_div(nr, nsplit), BN) * BN;
  nsplit = int(sg::ceil_div(nr, rps));
  const bool same = (queries == refs) && (nq == nr);
  const size_t need = sg::Carver::need(size_t(nr_pad) * BK * 2) + sg::Carver::need(size_t(nr_pad) * 4) +
                      (same ? 0 : sg::Carver::need(size_t(nq_pad) * BK * 2)) +
                      sg::Carver::need(sizeof(int) * size_t(nsplit) * nq_pad * kc) + sg::Carver::need(sizeof(int));
  int status;
  void* w = sg::ws_get(h, need, &status);
  if (!w) return status;
  sg::Carver cv(w);
  __nv_bfloat16* Rb = cv.take<__nv_bfloat16>(size_t(nr_pad) * BK);
  float* rn = cv.take<float>(nr_pad);
  __nv_bfloat16* Qb = same ? Rb : cv.take<__nv_bfloat16>(size_t(nq_pad) * BK);
  int* cand = cv.take<int>(size_t(nsplit) * nq_pad * kc);
  int* err = cv.take<int>(1);
  SG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  to_bf16_kernel<<<sg::ceil_div_i(nr_pad, 256), 256, 0, st>>>(refs, nr, d, ld, Rb, nr_pad, rn);
  SG_LAUNCH_CHECK();
  if (!same) {
    to_bf16_kernel<<<sg::ceil_div_i(nq_pad, 256), 256, 0, st>>>(queries, nq, d, ld, Qb, nq_pad, nullptr);
    SG_LAUNCH_CHECK();
  }
  CUtensorMap ta, tb;
  int rc = make_map(&ta, Qb, same ? nr_pad : nq_pad, BM);
  if (rc) return rc;
  rc = make_map(&tb, Rb, nr_pad, BN);
  if (rc) return rc;
  {
  sg::ProfScope prof(h, "knn_tc", st);
  if (kc == 16) rc = launch_tc<16>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, err, st);
  else if (kc == 32) rc = launch_tc<32>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, err, st);
  else if (kc == 48) rc = launch_tc<48>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, err, st);
  else rc = launch_tc<64>(ta, tb, rn, nr, rps, nsplit, cand, nq_pad, err, st);
  }
  if (rc) return rc;
  int herr = 0;
  SG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA(cudaStreamSynchronize(st));
  if (herr) return sg::fail(SG_ERR_TIMEOUT, "sg_knn: a tensor-core pipeline wait expired (stage %d)", herr);
  sg::ProfScope prof(h, "rerank", st);
  return sg_rerank(queries, refs, d, ld, nq, cand, nsplit, kc, nq_pad, kq, k, self_offset, idx_out, dist_out, nmiss,
                   st);
}
