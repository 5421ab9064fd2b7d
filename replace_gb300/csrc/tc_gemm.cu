// The diagnostic entry point of the tensor-core GEMM (gpl_tc_gemm_bf16):
// row-major fp32 output.
#include "tc_gemm.cuh"

namespace gpl {
namespace {

// Row-major fp32 output (the diagnostic GEMM).
struct EpiStore {
  float* d;
  int ldd;
  __device__ __forceinline__ void operator()(int row, int col0, const float (&v)[32]) const {
    float4* p = reinterpret_cast<float4*>(d + (size_t)row * ldd + col0);
#pragma unroll
    for (int i = 0; i < 8; i++) p[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  }
};

}  // namespace
}  // namespace gpl

using namespace gpl;

extern "C" gpl_status gpl_tc_gemm_bf16(const void* a, const void* b, float* d, int32_t m, int32_t n, int32_t k,
                                       int32_t* error_flag, void* stream) {
  if (!a || !b || !d) { set_error("null argument"); return GPL_ERR_INVALID_ARG; }
  EpiStore e{d, n};
  // a 64-wide N tile where a 128-wide one would leave SMs idle
  if (n % 128 == 0 && (int64_t)(m / 128) * (n / 128) >= 148)
    return (gpl_status)tc::launch_tc_gemm<128>(a, k, b, k, m, n, k, e, error_flag, (cudaStream_t)stream);
  return (gpl_status)tc::launch_tc_gemm<64>(a, k, b, k, m, n, k, e, error_flag, (cudaStream_t)stream);
}
