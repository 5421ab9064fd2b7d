// The diagnostic entry point of the tensor-core GEMM (gpl_tc_gemm_bf16):
// row-major fp32 output.
#include "tc_gemm.cuh"

namespace gpl {
namespace {

// Row-major fp32 output (the diagnostic GEMM): lanes on consecutive columns.
struct EpiStore {
  static constexpr bool kRowMajor = true;
  float* d;
  int ldd;
  __device__ __forceinline__ void at(int row, int col, float v) const { d[(size_t)row * ldd + col] = v; }
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
