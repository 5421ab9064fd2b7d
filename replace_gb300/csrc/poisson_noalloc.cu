// gpl_poisson_solve_noalloc: the Poisson solve of gpl_poisson_solve for
// callers that must not allocate device memory during the call -- a
// placement server that admits jobs against a fixed HBM budget and accounts
// for every byte up front, a host framework whose caching allocator already
// owns the device's memory, or a latency-critical loop that cannot absorb
// the device-wide synchronisation that cudaMalloc / cudaFree may cause.
//
// Its scratch (three transform planes and the twiddle/frequency tables) is a
// file-scope __device__ array of fixed size, so every GPU that loads this
// library holds kScratchBytes (about 3.1 MB) until the process exits.  The
// entry point calls no cudaMalloc, cudaFree or allocating library routine.
//
// Set-up: host code cannot pass the array's name to a kernel (on the host it
// is only a stand-in symbol, not a device address), so the first call on each
// device, with that device current, asks the runtime for the array's device
// address (cudaGetSymbolAddress) and caches it.  That first call should come
// before any stream capture.  The cached address belongs to the device's
// context: after cudaDeviceReset the next call sees a new context and looks
// the address up again (so that call, too, should precede any capture).
//
// Sharing: every call uses the same array and leaves its contents behind.
// Nothing in it needs to start at zero: each call rewrites the tables and all
// three planes before reading them.  Calls that overlap on the GPU (for
// example on two streams) race on the array; callers must order them.
#include <cuda_runtime.h>

#include <mutex>

#include "gpl_internal.h"

namespace gpl {
namespace {

constexpr int kNoAllocMaxBins = 512 * 512;     // largest nx * ny accepted
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kPlane = align256((size_t)kNoAllocMaxBins * sizeof(float));
constexpr size_t kOffSpec = 0;
constexpr size_t kOffP1 = kOffSpec + kPlane;
constexpr size_t kOffP2 = kOffP1 + kPlane;
constexpr size_t kOffWx = kOffP2 + kPlane;
constexpr size_t kOffWy = kOffWx + align256(kFftMax * sizeof(float));
constexpr size_t kOffW4x = kOffWy + align256(kFftMax * sizeof(float));
constexpr size_t kOffW4y = kOffW4x + align256(kFftMax * sizeof(float2));
constexpr size_t kOffTw = kOffW4y + align256(kFftMax * sizeof(float2));
constexpr size_t kScratchBytes = kOffTw + align256((kFftMax / 2) * sizeof(float2));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[64] = {nullptr};
unsigned long long g_ctx[64] = {0};    // context each cached address belongs to

// Tables of FFT::init (src/fft.cpp:78-90) and of the transforms, written into
// the scratch array for this call's grid.
__global__ void k_noalloc_tables(int nx, int ny, int bsx, int bsy, unsigned char* base) {
  float* wx = reinterpret_cast<float*>(base + kOffWx);
  float* wy = reinterpret_cast<float*>(base + kOffWy);
  float2* w4x = reinterpret_cast<float2*>(base + kOffW4x);
  float2* w4y = reinterpret_cast<float2*>(base + kOffW4y);
  float2* tw = reinterpret_cast<float2*>(base + kOffTw);
  const int n = max(max(nx, ny), kFftMax / 2);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double s, c;
    if (k < nx) {
      wx[k] = (float)(3.141592653589793 * (double)(float)k / (double)(float)nx);
      sincospi(-(double)k / (2.0 * nx), &s, &c);
      w4x[k] = make_float2((float)c, (float)s);
    }
    if (k < ny) {
      wy[k] = (float)(3.141592653589793 * (double)(float)k / (double)(float)ny *
                      (double)(float)bsy / (double)(float)bsx);
      sincospi(-(double)k / (2.0 * ny), &s, &c);
      w4y[k] = make_float2((float)c, (float)s);
    }
    if (k < kFftMax / 2) {
      sincospi(-2.0 * (double)k / (double)kFftMax, &s, &c);
      tw[k] = make_float2((float)c, (float)s);
    }
  }
}

}  // namespace
}  // namespace gpl

using namespace gpl;

extern "C" gpl_status gpl_poisson_solve_noalloc(int32_t nx, int32_t ny, int32_t bsx, int32_t bsy,
                                                const float* density, float* phi, float* fx,
                                                float* fy, void* stream) {
  auto pow2 = [](int v) { return v >= 2 && v <= kFftMax && (v & (v - 1)) == 0; };
  if (!pow2(nx) || !pow2(ny) || bsx <= 0 || bsy <= 0 || !density || !fx || !fy) {
    set_error("gpl_poisson_solve_noalloc: sizes must be powers of two in [2, 4096], bin sizes "
              "positive, density/field pointers non-null");
    return GPL_ERR_INVALID_ARG;
  }
  if ((int64_t)nx * ny > kNoAllocMaxBins) {
    set_error("gpl_poisson_solve_noalloc: nx * ny = " + std::to_string((int64_t)nx * ny) +
              " exceeds the fixed scratch limit of " + std::to_string(kNoAllocMaxBins) +
              " bins (512 x 512); use gpl_poisson_solve for larger grids");
    return GPL_ERR_INVALID_ARG;
  }
  int dev = 0;
  GPL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return GPL_ERR_INVALID_ARG; }
  GPL_CUDA(cudaSetDevice(dev));         // initialises the device's context if needed
  const unsigned long long ctx = current_context_id();
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev] || g_ctx[dev] != ctx) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error(std::string("gpl_poisson_solve_noalloc: cudaGetSymbolAddress failed: ") +
                  cudaGetErrorString(e));
        return GPL_ERR_CUDA;
      }
      g_addr[dev] = p;
      g_ctx[dev] = ctx;
    }
    base = static_cast<unsigned char*>(g_addr[dev]);
  }
  cudaStream_t s = (cudaStream_t)stream;
  k_noalloc_tables<<<8, 256, 0, s>>>(nx, ny, bsx, bsy, base);
  GPL_CUDA(cudaGetLastError());
  PoissonGrid g;
  g.nx = nx; g.ny = ny; g.size_x = bsx; g.size_y = bsy;
  g.core_lx = g.core_ly = 0; g.core_ux = nx * bsx; g.core_uy = ny * bsy;
  g.wx = reinterpret_cast<const float*>(base + kOffWx);
  g.wy = reinterpret_cast<const float*>(base + kOffWy);
  g.w4x = reinterpret_cast<const float2*>(base + kOffW4x);
  g.w4y = reinterpret_cast<const float2*>(base + kOffW4y);
  g.tw = reinterpret_cast<const float2*>(base + kOffTw);
  int rc = poisson_passes(g, nullptr, nullptr, nullptr, 1.0f, density, nullptr, nullptr,
                          reinterpret_cast<float*>(base + kOffSpec),
                          reinterpret_cast<float*>(base + kOffP1),
                          reinterpret_cast<float*>(base + kOffP2), nullptr, fx, fy, phi, s, nullptr);
  return (gpl_status)rc;
}
