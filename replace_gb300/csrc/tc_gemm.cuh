// Tensor-core GEMM on the fifth-generation (tcgen05) path (header: the
// kernel template and its launchers, instantiated with the epilogues of the
// users in tc_gemm.cu and poisson_gemm.cu).
//   D (M x N, fp32) = A (M x K, bf16) * B (N x K, bf16)^T
// with A and B stored K-contiguous (row-major M x K and N x K).  One CTA
// computes a 128 x BN tile of D:
//   * a TMA producer thread streams 128 x 64 tiles of A and BN x 64 tiles of
//     B into a shared-memory ring of 192 KB (eight stages at BN = 64, six at
//     128, four at 256; 128-byte swizzle, the layout the MMA descriptors
//     expect), one mbarrier per stage for "full";
//   * an MMA thread issues tcgen05.mma (kind::f16, bf16 inputs, fp32
//     accumulator in tensor memory, M = 128, N = BN, K = 16 per
//     instruction) and commits each stage back to its "empty" mbarrier;
//   * after the last commit all four warps read the accumulator from tensor
//     memory (tcgen05.ld, 32 rows per warp, 32 columns at a time) and hand
//     it to the epilogue: a row-major epilogue (Epi::kRowMajor) gets one
//     element per lane with the lanes on 32 consecutive columns of one row
//     (the warp's 32 x 32 block goes through a shared-memory transpose), so
//     its stores coalesce; otherwise each thread gets its row's 32 columns.
// Every mbarrier wait is bounded: on time-out the CTA records an error,
// drains the copies it issued (again bounded), frees its tensor memory and
// returns, so a fault in the pipeline can never hang the GPU.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "gpl_internal.h"

namespace gpl {
namespace tc {

constexpr int kTcM = 128;
constexpr int kTcK = 64;                 // one 128-byte swizzle row of bf16
constexpr int kTcThreads = 128;
constexpr long long kWaitPolls = 1ll << 24;        // bounded mbarrier polls

// Ring depth: 192 KB of stages.  Each k-tile is little MMA work, so the
// loads in flight (not the tensor pipe) set the pace.
template <int BN>
constexpr int tc_stages() { return (192 * 1024) / ((kTcM + BN) * kTcK * 2); }

template <int BN>
struct TcSmem {
  static constexpr int ST = tc_stages<BN>();
  __nv_bfloat16 a[ST][kTcM * kTcK];
  __nv_bfloat16 b[ST][BN * kTcK];
  float scratch[kTcThreads / 32][32 * 33];   // the epilogue's per-warp transpose
  uint64_t full[ST];
  uint64_t empty[ST];
  uint64_t done;
  uint32_t tmem_base;
};
template <int BN>
constexpr size_t tc_smem_bytes() { return sizeof(TcSmem<BN>) + 1024; }   // + alignment slack

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of the given parity; false after kWaitPolls polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (long long i = 0; i < kWaitPolls; i++)
    if (mbar_try(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(saddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(saddr(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand with 128-byte swizzle,
// rows of 128 B, 8-row atoms 1024 B apart (stride byte offset), descriptor
// version 1, layout type 2 (128-byte swizzle).
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
  const uint32_t a = saddr(p);
  uint64_t d = 0;
  d |= (uint64_t)((a & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;                 // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset
  d |= (uint64_t)1 << 46;                 // descriptor version
  d |= (uint64_t)2 << 61;                 // 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N = BN, M = kTcM.
template <int BN>
constexpr uint32_t idesc_of() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

// 32 consecutive fp32 columns of this warp's 32 accumulator rows.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

template <int BN, class Epi>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int K, Epi epi,
              int* err) {
  static_assert(BN == 64 || BN == 128 || BN == 256, "N tile");
  constexpr int kTcStages = TcSmem<BN>::ST;
  static_assert(kTcStages >= 2, "ring depth");
  constexpr uint32_t kBytesA = kTcM * kTcK * 2, kBytesB = BN * kTcK * 2;
  extern __shared__ unsigned char smem_raw[];
  TcSmem<BN>& S =
      *reinterpret_cast<TcSmem<BN>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * BN;
  const int kt_n = K / kTcK;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kTcStages; s++) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], 1);
    }
    mbar_init(&S.done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {   // tensor memory: BN fp32 columns x 128 lanes
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&S.tmem_base)),
                 "r"((uint32_t)BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;
  bool ok = true;
  if (warp == 0 && lane == 0) {
    // producer: stage s holds k-tile kt while kt % kTcStages == s
    int issued = 0;
    for (int kt = 0; kt < kt_n; kt++) {
      const int s = kt % kTcStages;
      if (kt >= kTcStages && !mbar_wait(&S.empty[s], ((kt / kTcStages) - 1) & 1)) { ok = false; break; }
      mbar_expect_tx(&S.full[s], kBytesA + kBytesB);
      tma_load_2d(S.a[s], &ta, kt * kTcK, m0, &S.full[s]);
      tma_load_2d(S.b[s], &tb, kt * kTcK, n0, &S.full[s]);
      issued = kt + 1;
    }
    if (!ok) {
      // drain: the copies of the last stages issued must land before the
      // CTA releases its shared memory
      for (int kt = (issued > kTcStages ? issued - kTcStages : 0); kt < issued; kt++)
        mbar_wait(&S.full[kt % kTcStages], (kt / kTcStages) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    for (int kt = 0; kt < kt_n; kt++) {
      const int s = kt % kTcStages;
      if (!mbar_wait(&S.full[s], (kt / kTcStages) & 1)) { ok = false; break; }
      tc_fence_after();
      const uint64_t da = smem_desc(S.a[s]), db = smem_desc(S.b[s]);
#pragma unroll
      for (int kk = 0; kk < kTcK / 16; kk++)   // 16 bf16 = 32 bytes = 2 descriptor units
        tc_mma(tmem, da + 2 * kk, db + 2 * kk, idesc_of<BN>(), (kt | kk) ? 1u : 0u);
      tc_commit(&S.empty[s]);
    }
    tc_commit(&S.done);   // arrives when every MMA issued above has completed
  }
  __syncwarp();
  // warp-uniform: tcgen05.ld below is a warp-collective instruction
  const bool got = __all_sync(0xffffffffu, mbar_wait(&S.done, 0));
  tc_fence_after();
  if (got) {
    float v[32];
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    float* scr = S.scratch[warp];
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      tmem_ld32(tmem + lane_base + (uint32_t)c, v);
      if constexpr (Epi::kRowMajor) {
#pragma unroll
        for (int i = 0; i < 32; i++) scr[lane * 33 + i] = v[i];
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; r++) epi.at(m0 + warp * 32 + r, n0 + c + lane, scr[r * 33 + lane]);
        __syncwarp();
      } else {
        epi(m0 + warp * 32 + lane, n0 + c, v);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN)
                 : "memory");
  if ((!ok || !got) && err) atomicExch(err, 1);
}

inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::mutex mu;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// K-major bf16 operand of `rows` x K (row stride ld elements) as a TMA map
// with 64 x box_rows boxes.
inline int encode_operand(CUtensorMap* map, const void* base, int rows, int K, int ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) { set_error("cuTensorMapEncodeTiled is not available"); return GPL_ERR_CUDA; }
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed"); return GPL_ERR_CUDA; }
  return GPL_OK;
}

// A GEMM whose operands are fixed (tensor maps encoded once): prepare() sets
// the kernel's shared-memory limit outside any stream capture; launch()
// only enqueues the kernel, so it can be captured in a CUDA graph.
template <int BN, class Epi>
struct TcPlan {
  CUtensorMap ta, tb;
  int M = 0, N = 0, K = 0;
  int prepare(const void* a, int lda, const void* b, int ldb, int m, int n, int k) {
    if (m <= 0 || n <= 0 || k <= 0 || m % kTcM || n % BN || k % kTcK || lda < k || ldb < k || lda % 8 ||
        ldb % 8 || ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15)) {
      set_error("tensor-core GEMM plan: bad shape or alignment");
      return GPL_ERR_INVALID_ARG;
    }
    M = m; N = n; K = k;
    int rc = encode_operand(&ta, a, m, k, lda, kTcM);
    if (!rc) rc = encode_operand(&tb, b, n, k, ldb, BN);
    if (rc) return rc;
    GPL_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc_smem_bytes<BN>()));
    return GPL_OK;
  }
  void launch(const Epi& epi, int* err, cudaStream_t s) const {
    k_tc_gemm<BN, Epi><<<dim3(N / BN, M / kTcM), kTcThreads, tc_smem_bytes<BN>(), s>>>(ta, tb, K, epi, err);
  }
};

template <int BN, class Epi>
int launch_tc_gemm(const void* a, int lda, const void* b, int ldb, int M, int N, int K, const Epi& epi, int* err,
                   cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0 || M % kTcM || N % BN || K % kTcK || lda < K || ldb < K || lda % 8 || ldb % 8) {
    set_error("tensor-core GEMM: M must be a multiple of 128, N of the N tile, K of 64; rows 16-byte strided");
    return GPL_ERR_INVALID_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) {
    set_error("tensor-core GEMM: operands must be 16-byte aligned");
    return GPL_ERR_INVALID_ARG;
  }
  CUtensorMap ta, tb;
  int rc = encode_operand(&ta, a, M, K, lda, kTcM);
  if (!rc) rc = encode_operand(&tb, b, N, K, ldb, BN);
  if (rc) return rc;
  constexpr size_t smem = tc_smem_bytes<BN>();
  GPL_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_tc_gemm<BN, Epi><<<dim3(N / BN, M / kTcM), kTcThreads, smem, s>>>(ta, tb, K, epi, err);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}


}  // namespace tc
}  // namespace gpl
