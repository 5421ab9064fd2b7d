// Weighted-average (WA) wirelength model: NesterovBase::updateWireLengthForceWA
// (src/nesterovBase.cpp:1304-1360), the per-pin gradient of
// getWireLengthGradientPinWA (:1383-1440, JingWei's thesis eq. 4.13) and the
// integer HPWL of NesterovBase::getHpwl (:1508-1516).
//
// Nets are split once per job by degree: nets of up to kSmallNet pins are
// processed one per thread (their exponential sums are accumulated in the
// reference's pin order, so the per-net sums are the reference's values);
// larger nets are processed one per warp (bounding box by warp min/max, sums
// by warp shuffles).  Each pin's gradient is written to pin_grad; the gcell
// kernel sums a cell's pins in the instance's pin order.
#include <climits>

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace gpl {

namespace {

constexpr int kBlock = 256;

struct WaArgs {
  const int32_t* nets;        // net list of this launch (small or large)
  int n_nets;
  const int32_t* net_start;
  const int32_t* pin_g;
  const int2* pin_off;
  const float2* slp;
  float cx, cy;               // wire-length coefficients (1/gamma)
  float bar;                  // minWireLengthForceBar
  float2* pin_grad;
  long long* part_i;          // HPWL partials, this launch's blocks start at part_offset
  int part_offset;
};

// Pin centre: gcell pins follow the truncated density centre
// (GPin::updateDensityLocation, src/nesterovBase.cpp:411-415); other pins
// keep their fixed position.
__device__ __forceinline__ int2 pin_pos(const WaArgs& A, int q) {
  const int g = __ldg(&A.pin_g[q]);
  const int2 o = __ldg(&A.pin_off[q]);
  if (g < 0) return o;
  const float2 c = __ldg(&A.slp[g]);
  return make_int2(__float2int_rz(c.x) + o.x, __float2int_rz(c.y) + o.y);
}

struct WaSums { float s[8]; };

// getWireLengthGradientPinWA for one pin given its net's sums.
__device__ __forceinline__ float2 pin_gradient(int2 p, int lx, int ux, int ly, int uy,
                                               const WaSums& S, float cx, float cy, float bar) {
  float gminx = 0.f, gmaxx = 0.f, gminy = 0.f, gmaxy = 0.f;
  const float x = (float)p.x, y = (float)p.y;
  const float eminx = __fmul_rn((float)(lx - p.x), cx);
  const float emaxx = __fmul_rn((float)(p.x - ux), cx);
  const float eminy = __fmul_rn((float)(ly - p.y), cy);
  const float emaxy = __fmul_rn((float)(p.y - uy), cy);
  if (eminx > bar) {
    const float e = fast_exp(eminx), s0 = S.s[0];
    gminx = (s0 * (e * (1.0f - cx * x)) + cx * e * S.s[1]) / (s0 * s0);
  }
  if (emaxx > bar) {
    const float e = fast_exp(emaxx), s0 = S.s[2];
    gmaxx = (s0 * (e * (1.0f + cx * x)) - cx * e * S.s[3]) / (s0 * s0);
  }
  if (eminy > bar) {
    const float e = fast_exp(eminy), s0 = S.s[4];
    gminy = (s0 * (e * (1.0f - cy * y)) + cy * e * S.s[5]) / (s0 * s0);
  }
  if (emaxy > bar) {
    const float e = fast_exp(emaxy), s0 = S.s[6];
    gmaxy = (s0 * (e * (1.0f + cy * y)) - cy * e * S.s[7]) / (s0 * s0);
  }
  return make_float2(gminx - gmaxx, gminy - gmaxy);
}

// Accumulate one pin into the eight WA sums (src/nesterovBase.cpp:1320-1355).
__device__ __forceinline__ void pin_sums(int2 p, int lx, int ux, int ly, int uy, float cx, float cy,
                                         float bar, WaSums& S) {
  const float eminx = __fmul_rn((float)(lx - p.x), cx);
  const float emaxx = __fmul_rn((float)(p.x - ux), cx);
  const float eminy = __fmul_rn((float)(ly - p.y), cy);
  const float emaxy = __fmul_rn((float)(p.y - uy), cy);
  if (eminx > bar) { const float e = fast_exp(eminx); S.s[0] = __fadd_rn(S.s[0], e); S.s[1] = __fadd_rn(S.s[1], __fmul_rn((float)p.x, e)); }
  if (emaxx > bar) { const float e = fast_exp(emaxx); S.s[2] = __fadd_rn(S.s[2], e); S.s[3] = __fadd_rn(S.s[3], __fmul_rn((float)p.x, e)); }
  if (eminy > bar) { const float e = fast_exp(eminy); S.s[4] = __fadd_rn(S.s[4], e); S.s[5] = __fadd_rn(S.s[5], __fmul_rn((float)p.y, e)); }
  if (emaxy > bar) { const float e = fast_exp(emaxy); S.s[6] = __fadd_rn(S.s[6], e); S.s[7] = __fadd_rn(S.s[7], __fmul_rn((float)p.y, e)); }
}

__global__ void __launch_bounds__(kBlock) k_wa_small(WaArgs A) {
  __shared__ long long sh[32];
  const int t = blockIdx.x * kBlock + threadIdx.x;
  long long hp = 0;
  if (t < A.n_nets) {
    const int n = A.nets[t];
    const int s = A.net_start[n], e = A.net_start[n + 1];
    int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
    for (int q = s; q < e; q++) {
      const int2 p = pin_pos(A, q);
      lx = min(lx, p.x); ux = max(ux, p.x); ly = min(ly, p.y); uy = max(uy, p.y);
    }
    WaSums S;
#pragma unroll
    for (int k = 0; k < 8; k++) S.s[k] = 0.0f;
    for (int q = s; q < e; q++) pin_sums(pin_pos(A, q), lx, ux, ly, uy, A.cx, A.cy, A.bar, S);
    for (int q = s; q < e; q++)
      A.pin_grad[q] = pin_gradient(pin_pos(A, q), lx, ux, ly, uy, S, A.cx, A.cy, A.bar);
    hp = (long long)((ux - lx) + (uy - ly));
  }
  block_reduce_ll(hp, &A.part_i[A.part_offset + blockIdx.x], sh);
}

// One warp per net.
__global__ void __launch_bounds__(kBlock) k_wa_large(WaArgs A) {
  __shared__ long long sh[32];
  const int w = (blockIdx.x * kBlock + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  long long hp = 0;
  if (w < A.n_nets) {
    const int n = A.nets[w];
    const int s = A.net_start[n], e = A.net_start[n + 1];
    int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
    for (int q = s + lane; q < e; q += 32) {
      const int2 p = pin_pos(A, q);
      lx = min(lx, p.x); ux = max(ux, p.x); ly = min(ly, p.y); uy = max(uy, p.y);
    }
    lx = __reduce_min_sync(0xffffffffu, lx);
    ly = __reduce_min_sync(0xffffffffu, ly);
    ux = __reduce_max_sync(0xffffffffu, ux);
    uy = __reduce_max_sync(0xffffffffu, uy);
    WaSums S;
#pragma unroll
    for (int k = 0; k < 8; k++) S.s[k] = 0.0f;
    for (int q = s + lane; q < e; q += 32) pin_sums(pin_pos(A, q), lx, ux, ly, uy, A.cx, A.cy, A.bar, S);
#pragma unroll
    for (int k = 0; k < 8; k++)
      for (int o = 16; o > 0; o >>= 1) S.s[k] += __shfl_xor_sync(0xffffffffu, S.s[k], o);
    for (int q = s + lane; q < e; q += 32)
      A.pin_grad[q] = pin_gradient(pin_pos(A, q), lx, ux, ly, uy, S, A.cx, A.cy, A.bar);
    if (lane == 0) hp = (long long)((ux - lx) + (uy - ly));
  }
  block_reduce_ll(hp, &A.part_i[A.part_offset + blockIdx.x], sh);
}

}  // namespace

int net_blocks(const DeviceModel& d) {
  return (d.n_net_small + kBlock - 1) / kBlock + (d.n_net_large * 32 + kBlock - 1) / kBlock;
}

int launch_wa(DeviceModel& d, const EvalArgs& a, cudaStream_t s, Timer& t) {
  WaArgs A;
  A.net_start = d.net_start;
  A.pin_g = d.pin_g;
  A.pin_off = d.pin_off;
  A.slp = a.slp;
  A.cx = a.wl_coef_x; A.cy = a.wl_coef_y;
  A.bar = a.min_wl_force_bar;
  A.pin_grad = d.pin_grad;
  A.part_i = d.part_i;
  const int b_small = (d.n_net_small + kBlock - 1) / kBlock;
  const int b_large = (d.n_net_large * 32 + kBlock - 1) / kBlock;
  t.begin(kKWa);
  if (b_small) {
    A.nets = d.net_small; A.n_nets = d.n_net_small; A.part_offset = 0;
    k_wa_small<<<b_small, kBlock, 0, s>>>(A);
  }
  if (b_large) {
    A.nets = d.net_large; A.n_nets = d.n_net_large; A.part_offset = b_small;
    k_wa_large<<<b_large, kBlock, 0, s>>>(A);
  }
  t.end(kKWa);
  t.count((b_small ? 1 : 0) + (b_large ? 1 : 0));
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

}  // namespace gpl
