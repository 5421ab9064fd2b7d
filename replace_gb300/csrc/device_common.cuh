// Device helpers shared by the placement kernels.
#pragma once

#include <cuda_runtime.h>

#include "gpl_internal.h"

namespace gpl {

// Bin column/row bounds of the reference's BinGrid (src/nesterovBase.cpp:684-711):
// uniform binSize steps from the core corner, the last one clipped.
struct BinGeom {
  int core_lx, core_ly, core_ux, core_uy, size_x, size_y, cnt_x, cnt_y;
  __device__ __forceinline__ int lo_x(int a) const { return core_lx + a * size_x; }
  __device__ __forceinline__ int hi_x(int a) const { return min(core_lx + (a + 1) * size_x, core_ux); }
  __device__ __forceinline__ int lo_y(int c) const { return core_ly + c * size_y; }
  __device__ __forceinline__ int hi_y(int c) const { return min(core_ly + (c + 1) * size_y, core_uy); }
  // getDensityMinMaxIdxX/Y (src/nesterovBase.cpp:822-841), clamped to the
  // grid so that a coordinate outside the core cannot index outside it.
  __device__ __forceinline__ void range(int lx, int ux, int ly, int uy, int& x0, int& x1, int& y0,
                                        int& y1) const {
    const int dl = lx - core_lx, du = ux - core_lx;
    x0 = dl / size_x;
    x1 = ((du >= size_x ? du % size_x : du) == 0) ? du / size_x : du / size_x + 1;
    const int el = ly - core_ly, eu = uy - core_ly;
    y0 = el / size_y;
    y1 = ((eu >= size_y ? eu % size_y : eu) == 0) ? eu / size_y : eu / size_y + 1;
    x0 = max(x0, 0); y0 = max(y0, 0);
    x1 = min(x1, cnt_x); y1 = min(y1, cnt_y);
  }
  // getOverlapDensityArea (src/nesterovBase.cpp:1533-1547)
  __device__ __forceinline__ float overlap(int a, int c, int lx, int ux, int ly, int uy) const {
    const int rlx = max(lo_x(a), lx), rux = min(hi_x(a), ux);
    const int rly = max(lo_y(c), ly), ruy = min(hi_y(c), uy);
    if (rlx >= rux || rly >= ruy) return 0.0f;
    return __fmul_rn((float)(rux - rlx), (float)(ruy - rly));
  }
};

// GCell::setDensityCenterLocation: float centre truncated to int, then the
// density rectangle is centre -/+ half size (src/nesterovBase.cpp:164-179).
__device__ __forceinline__ void density_rect(float2 c, int2 h, int& lx, int& ux, int& ly, int& uy) {
  const int cx = __float2int_rz(c.x), cy = __float2int_rz(c.y);
  lx = cx - h.x; ux = cx + h.x; ly = cy - h.y; uy = cy + h.y;
}

// getDensityCoordiLayoutInsideX/Y (src/nesterovBase.cpp:1270-1297)
__device__ __forceinline__ float inside(float c, int h, int lo, int hi) {
  float adj = c;
  const float hf = (float)h;
  if (__fsub_rn(c, hf) < (float)lo) adj = (float)(lo + h);
  if (__fadd_rn(c, hf) > (float)hi) adj = (float)(hi - h);
  return adj;
}

// fastExp (src/nesterovBase.cpp:1568-1582): (1 + a/1024)^1024 by ten
// squarings.  The reference's first step is evaluated in double; for a float
// argument 1 + a/1024 rounded once to float is the same value.
// Element i of a small pointer array held in kernel parameters, by selects:
// indexing a parameter array with a run-time index makes the compiler copy
// the whole parameter block to local memory.
template <class T>
__device__ __forceinline__ T pick4(T const (&a)[4], int i) {
  return i == 0 ? a[0] : i == 1 ? a[1] : i == 2 ? a[2] : a[3];
}
template <class T>
__device__ __forceinline__ T pick2(T const (&a)[2], int i) {
  return i == 0 ? a[0] : a[1];
}

// float -> int64 truncation and int64 -> float rounding through 32-bit
// conversions when the value fits (the same results; the 64-bit conversions
// run on the FP64 pipe, which is narrow on this part).
__device__ __forceinline__ unsigned long long trunc_u64(float f) {   // f >= 0
  return f < 4294967296.0f ? (unsigned long long)__float2uint_rz(f) : (unsigned long long)(long long)f;
}
__device__ __forceinline__ float ll_to_float(long long v) {
  return (v >= 0 && v < 2147483648ll) ? __int2float_rn((int)v) : __ll2float_rn(v);
}

__device__ __forceinline__ float fast_exp(float a) {
  a = __fadd_rn(1.0f, __fmul_rn(a, 0.0009765625f));
#pragma unroll
  for (int i = 0; i < 10; i++) a = __fmul_rn(a, a);
  return a;
}

// Block sums of N values; thread 0 writes out_base[k * stride + index]
// (index defaults to the block index).
template <int N>
__device__ __forceinline__ void block_reduce_n(double (&v)[N], double* out_base, int stride,
                                               double* sh /* [32*N] */, int index = -1) {
  if (index < 0) index = blockIdx.x;
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) sh[k * 32 + wid] = v[k];
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) {
      double x = lane < nw ? sh[k * 32 + lane] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) out_base[k * stride + index] = x;
    }
  }
  __syncthreads();
}

// Sum of p[0..n) by one block in a fixed order (thread-strided, then fixed
// trees); reads bypass L1 because other blocks wrote the values.  The result
// is returned to every thread.
__device__ __forceinline__ double block_sum_ordered(const double* p, int n, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += __ldcg(p + i);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[0] = v;
  }
  __syncthreads();
  const double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ long long block_sum_ordered_ll(const long long* p, int n, long long* sh) {
  long long v = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += __ldcg(p + i);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sh[lane] : 0ll;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[0] = v;
  }
  __syncthreads();
  const long long r = sh[0];
  __syncthreads();
  return r;
}

}  // namespace gpl
