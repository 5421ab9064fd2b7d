// Weighted-average (WA) wirelength model: NesterovBase::updateWireLengthForceWA
// (src/nesterovBase.cpp:1304-1360), the per-pin gradient of
// getWireLengthGradientPinWA (:1383-1440, JingWei's thesis eq. 4.13) and the
// integer HPWL of NesterovBase::getHpwl (:1508-1516).
//
// Nets are bucketed once per job by degree d into group widths G = 2, 4, 8,
// 16, 32 (the smallest G >= d); a net is handled by G consecutive lanes of a
// warp, one pin per lane.  Nets of up to 64 and 128 pins take a warp with two
// and four pins per lane, still in registers.  On the device, nets are numbered in bucket order
// (within a bucket by their lowest gcell index, so that consecutive warps
// touch nearby cells) and pins are renumbered so that each net's pins are
// contiguous in that order: pin records are read and pin gradients written
// with coalesced accesses.  The lane keeps its pin's position and four
// exponentials in registers: bounding box and the eight WA sums are group
// reductions (xor shuffles inside the aligned G-lane group), and the pin
// gradient follows without re-reading anything.  For groups of 8 lanes or
// more the eight sums are reduced by halving exchanges (each step sends half
// of the values still held, so 8 values take 4 + 2 + 1 + ... shuffles instead
// of 8 per step) and then broadcast.  Nets of more than 128 pins take a warp
// each and loop over their pins.  One launch covers all buckets (the block
// index selects the bucket), so warps never mix net sizes.
//
// Optional per-net weights (GNet::customWeight, src/nesterovBase.h:210-212)
// scale each pin gradient as it is written.  They are a compile-time variant
// of the kernel: the unweighted one keeps its register count (48 -> 40 per
// thread, six blocks of 256 threads per SM instead of five).
#include <climits>
#include <cstring>

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace gpl {

namespace {

constexpr int kBlock = 256;

struct WaArgs {
  int bucket_start[kWaBuckets + 1];   // first (bucket-ordered) net of each bucket
  int block_start[kWaBuckets + 1];    // first block of each bucket
  const int32_t* net_start;     // pin CSR of the bucket-ordered nets
  const int4* pins;             // (gcell or -1, x offset or position, y ..., unused)
  float2* slp_all[4];
  const EvalCtl* ctl;
  float bar;                    // minWireLengthForceBar
  float2* pin_grad;             // device pin order
  const float* net_w;           // per-net weights (bucket order), weighted variant only
  long long* hpwl_total;        // kHpwlLanes spread accumulators (stride kHpwlStride)
};

// This evaluation's coordinates and wire-length coefficients (1/gamma), read
// from the control record; kept apart from the (constant) kernel parameters.
template <bool kW>
struct WaEval {
  const float2* slp;
  const float* w;               // per-net weights (kW only)
  float cx, cy;
};

// Net k's weight times a pin gradient (the weighted sum that timing-driven
// placers form per gcell: weight x getWireLengthGradientPinWA).
template <bool kW>
__device__ __forceinline__ float2 weighed(const WaEval<kW>& V, int k, float2 g) {
  if constexpr (!kW) return g;
  const float w = __ldg(&V.w[k]);
  return make_float2(__fmul_rn(g.x, w), __fmul_rn(g.y, w));
}

// Pin centre: gcell pins follow the truncated density centre
// (GPin::updateDensityLocation, src/nesterovBase.cpp:411-415); other pins
// keep their fixed position.
template <bool kW>
__device__ __forceinline__ int2 pin_pos(const WaEval<kW>& V, const int4& r) {
  if (r.x < 0) return make_int2(r.y, r.z);
  const float2 c = __ldg(&V.slp[r.x]);
  return make_int2(__float2int_rz(c.x) + r.y, __float2int_rz(c.y) + r.z);
}

// The four WA exponentials of one pin (src/nesterovBase.cpp:1320-1355);
// a direction whose exponent is not above minWireLengthForceBar contributes 0
// and has its flag cleared.
struct PinExp {
  float e[4];      // min x, max x, min y, max y
  unsigned flags;  // bit k set: e[k] is used
};

__device__ __forceinline__ PinExp pin_exps(int2 p, int lx, int ux, int ly, int uy, float cx, float cy,
                                           float bar) {
  PinExp r;
  const float a[4] = {__fmul_rn((float)(lx - p.x), cx), __fmul_rn((float)(p.x - ux), cx),
                      __fmul_rn((float)(ly - p.y), cy), __fmul_rn((float)(p.y - uy), cy)};
  r.flags = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    r.e[k] = 0.0f;
    if (a[k] > bar) { r.e[k] = fast_exp(a[k]); r.flags |= 1u << k; }
  }
  return r;
}

// getWireLengthGradientPinWA (src/nesterovBase.cpp:1383-1440) regrouped per
// net.  With the net's sums S[0..3] = (sum e, sum x e) for min x and max x
// (S[4..7] the same for y), the min-x term (s e (1 - c x) + c e S1) / s^2 is
// e (A + B x) with A = 1/s + c S1 / s^2 and B = -c/s (max x: A = 1/s -
// c S1 / s^2, B = c/s), so a pin costs one multiply-add and one multiply per
// direction once the net's A and B are known.  The sums of exponentials are
// in [1, degree] (the extreme pin contributes exp(0) = 1, every term is at
// most 1), so the fast reciprocal (2 ulp) is safe; a direction whose
// exponent fell below the force bar has e = 0 and contributes 0.
struct NetCoef {
  float a[4], b[4];
};

__device__ __forceinline__ NetCoef net_coef(const float* S, float cx, float cy) {
  NetCoef K;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float c = k < 2 ? cx : cy;
    const float inv = __fdividef(1.0f, S[2 * k]);
    const float m = __fmul_rn(__fmul_rn(__fmul_rn(c, S[2 * k + 1]), inv), inv);
    const bool lo = (k & 1) == 0;          // min side
    K.a[k] = lo ? __fadd_rn(inv, m) : __fsub_rn(inv, m);
    K.b[k] = lo ? __fmul_rn(-c, inv) : __fmul_rn(c, inv);
  }
  return K;
}

// (The arithmetic of this and net_coef is spelled out with rounding
// intrinsics, so that every kernel that inlines it -- the per-job WA kernel
// and the batched one -- computes the same values: left to the compiler, a
// multiply and an add may be fused in one kernel and not in the other.)
__device__ __forceinline__ float2 pin_gradient(int2 p, const PinExp& E, const NetCoef& K) {
  const float x = (float)p.x, y = (float)p.y;
  const float g0 = __fmul_rn(E.e[0], __fmaf_rn(K.b[0], x, K.a[0]));
  const float g1 = __fmul_rn(E.e[1], __fmaf_rn(K.b[1], x, K.a[1]));
  const float g2 = __fmul_rn(E.e[2], __fmaf_rn(K.b[2], y, K.a[2]));
  const float g3 = __fmul_rn(E.e[3], __fmaf_rn(K.b[3], y, K.a[3]));
  return make_float2(__fsub_rn(g0, g1), __fsub_rn(g2, g3));
}

__device__ __forceinline__ void sums_of(int2 p, const PinExp& E, float* S) {
  S[0] = E.e[0]; S[1] = __fmul_rn((float)p.x, E.e[0]);
  S[2] = E.e[1]; S[3] = __fmul_rn((float)p.x, E.e[1]);
  S[4] = E.e[2]; S[5] = __fmul_rn((float)p.y, E.e[2]);
  S[6] = E.e[3]; S[7] = __fmul_rn((float)p.y, E.e[3]);
}

// Sums of S[0..7] over each aligned G-lane group (G = 8, 16 or 32), returned
// to every lane of the group.  Halving exchanges: at offset G/2 a lane keeps
// the half of its values selected by its own offset bit and sends the other
// half, so after three steps each lane holds one partial sum (index given by
// three bits of its lane number); the remaining offsets finish that sum, and
// eight shuffles broadcast the totals.  The order is fixed, so the result is
// the same run to run.
template <int G>
__device__ __forceinline__ void group_sum8(float (&S)[8]) {
  static_assert(G == 8 || G == 16 || G == 32, "group width");
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  constexpr int o1 = G / 2, o2 = G / 4, o3 = G / 8;
  float T[4], U[2], V;
  {
    const bool hi = lane & o1;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const float keep = hi ? S[4 + j] : S[j], send = hi ? S[j] : S[4 + j];
      T[j] = keep + __shfl_xor_sync(full, send, o1);
    }
  }
  {
    const bool hi = lane & o2;
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const float keep = hi ? T[2 + j] : T[j], send = hi ? T[j] : T[2 + j];
      U[j] = keep + __shfl_xor_sync(full, send, o2);
    }
  }
  {
    const bool hi = lane & o3;
    const float keep = hi ? U[1] : U[0], send = hi ? U[0] : U[1];
    V = keep + __shfl_xor_sync(full, send, o3);
  }
#pragma unroll
  for (int o = o3 / 2; o > 0; o >>= 1) V += __shfl_xor_sync(full, V, o);
  // value index k is held by the lanes whose offset bits o1, o2, o3 spell k
  const int base = lane & ~(G - 1);
#pragma unroll
  for (int k = 0; k < 8; k++)
    S[k] = __shfl_sync(full, V, base + ((k & 4) ? o1 : 0) + ((k & 2) ? o2 : 0) + ((k & 1) ? o3 : 0));
}

// The exponentials of both pins of a two-pin net, equal to pin_exps of each
// pin: in every direction one pin is the extreme (exponent exactly 0, and
// fast_exp(0) = 1 exactly), so only the other pin's exponential is computed,
// one fast_exp per direction instead of two.
__device__ __forceinline__ void pair_exps(int2 p0, int2 p1, int lx, int ux, int ly, int uy, float cx, float cy,
                                          float bar, PinExp& E0, PinExp& E1) {
  const float a0[4] = {__fmul_rn((float)(lx - p0.x), cx), __fmul_rn((float)(p0.x - ux), cx),
                       __fmul_rn((float)(ly - p0.y), cy), __fmul_rn((float)(p0.y - uy), cy)};
  const float a1[4] = {__fmul_rn((float)(lx - p1.x), cx), __fmul_rn((float)(p1.x - ux), cx),
                       __fmul_rn((float)(ly - p1.y), cy), __fmul_rn((float)(p1.y - uy), cy)};
  E0.flags = E1.flags = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    // the smaller exponent is the non-extreme pin's (or 0 for a tie)
    const float am = fminf(a0[k], a1[k]);
    const float v = am > bar ? fast_exp(am) : 0.0f;
    E0.e[k] = 0.0f;
    E1.e[k] = 0.0f;
    if (a0[k] > bar) { E0.e[k] = a0[k] == am ? v : 1.0f; E0.flags |= 1u << k; }
    if (a1[k] > bar) { E1.e[k] = a1[k] == am ? v : 1.0f; E1.flags |= 1u << k; }
  }
}

// Nets of one or two pins (the most common kind): one thread per net, both
// pins in registers; the same values as a two-lane group (the group's sums
// are S0 + S1 in either lane, and float addition commutes).
template <bool kW>
__device__ __forceinline__ long long wa_pair(const WaArgs& A, const WaEval<kW>& V, int local_block) {
  const int k = A.bucket_start[0] + local_block * kBlock + threadIdx.x;
  if (k >= A.bucket_start[1]) return 0ll;
  const int s = __ldg(&A.net_start[k]), e = __ldg(&A.net_start[k + 1]);
  const int2 p0 = pin_pos(V, __ldg(&A.pins[s]));
  if (e - s == 1) {
    const PinExp E = pin_exps(p0, p0.x, p0.x, p0.y, p0.y, V.cx, V.cy, A.bar);
    float S[8];
    sums_of(p0, E, S);
    A.pin_grad[s] = weighed(V, k, pin_gradient(p0, E, net_coef(S, V.cx, V.cy)));
    return 0ll;
  }
  const int2 p1 = pin_pos(V, __ldg(&A.pins[s + 1]));
  const int lx = min(p0.x, p1.x), ux = max(p0.x, p1.x), ly = min(p0.y, p1.y), uy = max(p0.y, p1.y);
  PinExp E0, E1;
  pair_exps(p0, p1, lx, ux, ly, uy, V.cx, V.cy, A.bar, E0, E1);
  float S[8], T[8];
  sums_of(p0, E0, S);
  sums_of(p1, E1, T);
#pragma unroll
  for (int t = 0; t < 8; t++) S[t] += T[t];
  float2* g = A.pin_grad + s;
  const NetCoef K = net_coef(S, V.cx, V.cy);
  g[0] = weighed(V, k, pin_gradient(p0, E0, K));
  g[1] = weighed(V, k, pin_gradient(p1, E1, K));
  return (long long)((ux - lx) + (uy - ly));
}

// One net per G-lane group, one pin per lane.
template <int G, bool kW>
__device__ __forceinline__ long long wa_group(const WaArgs& A, const WaEval<kW>& V, int bucket,
                                              int local_block) {
  const int per_block = kBlock / G;
  const int grp = threadIdx.x / G, li = threadIdx.x % G;
  const int k = A.bucket_start[bucket] + local_block * per_block + grp;
  const bool net_ok = k < A.bucket_start[bucket + 1];
  int s = 0, e = 0;
  if (net_ok) {
    s = __ldg(&A.net_start[k]);
    e = __ldg(&A.net_start[k + 1]);
  }
  const int q = s + li;
  const bool valid = net_ok && q < e;
  int4 r = make_int4(-1, 0, 0, -1);
  if (valid) r = __ldg(&A.pins[q]);
  const int2 p = valid ? pin_pos(V, r) : make_int2(0, 0);
  int lx = valid ? p.x : INT_MAX, ux = valid ? p.x : INT_MIN;
  int ly = valid ? p.y : INT_MAX, uy = valid ? p.y : INT_MIN;
  if constexpr (G == 32) {
    lx = __reduce_min_sync(0xffffffffu, lx);
    ux = __reduce_max_sync(0xffffffffu, ux);
    ly = __reduce_min_sync(0xffffffffu, ly);
    uy = __reduce_max_sync(0xffffffffu, uy);
  } else {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      lx = min(lx, __shfl_xor_sync(0xffffffffu, lx, o));
      ux = max(ux, __shfl_xor_sync(0xffffffffu, ux, o));
      ly = min(ly, __shfl_xor_sync(0xffffffffu, ly, o));
      uy = max(uy, __shfl_xor_sync(0xffffffffu, uy, o));
    }
  }
  PinExp E;
  float S[8];
  if (valid) {
    E = pin_exps(p, lx, ux, ly, uy, V.cx, V.cy, A.bar);
    sums_of(p, E, S);
  } else {
    E.flags = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) E.e[t] = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; t++) S[t] = 0.0f;
  }
  if constexpr (G >= 8) {
    group_sum8<G>(S);
  } else {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
      for (int t = 0; t < 8; t++) S[t] += __shfl_xor_sync(0xffffffffu, S[t], o);
  }
  if (valid) A.pin_grad[q] = weighed(V, k, pin_gradient(p, E, net_coef(S, V.cx, V.cy)));
  return (net_ok && li == 0) ? (long long)((ux - lx) + (uy - ly)) : 0ll;
}

// One warp per net of up to 32 P pins, P pins per lane kept in registers.
template <int P, bool kW>
__device__ __forceinline__ long long wa_warp(const WaArgs& A, const WaEval<kW>& V, int bucket,
                                             int local_block) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int k = A.bucket_start[bucket] + local_block * (kBlock / 32) + (threadIdx.x >> 5);
  if (k >= A.bucket_start[bucket + 1]) return 0ll;           // warp-uniform
  const int s = __ldg(&A.net_start[k]), e = __ldg(&A.net_start[k + 1]);
  int2 p[P];
  bool ok[P];
  int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
#pragma unroll
  for (int j = 0; j < P; j++) {
    const int q = s + lane + 32 * j;
    ok[j] = q < e;
    p[j] = ok[j] ? pin_pos(V, __ldg(&A.pins[q])) : make_int2(0, 0);
    if (ok[j]) { lx = min(lx, p[j].x); ux = max(ux, p[j].x); ly = min(ly, p[j].y); uy = max(uy, p[j].y); }
  }
  lx = __reduce_min_sync(full, lx);
  ly = __reduce_min_sync(full, ly);
  ux = __reduce_max_sync(full, ux);
  uy = __reduce_max_sync(full, uy);
  PinExp E[P];
  float S[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int j = 0; j < P; j++) {
    if (ok[j]) {
      E[j] = pin_exps(p[j], lx, ux, ly, uy, V.cx, V.cy, A.bar);
      float t[8];
      sums_of(p[j], E[j], t);
#pragma unroll
      for (int i = 0; i < 8; i++) S[i] = __fadd_rn(S[i], t[i]);
    }
  }
  group_sum8<32>(S);
  const NetCoef K = net_coef(S, V.cx, V.cy);
#pragma unroll
  for (int j = 0; j < P; j++)
    if (ok[j]) A.pin_grad[s + lane + 32 * j] = weighed(V, k, pin_gradient(p[j], E[j], K));
  return lane == 0 ? (long long)((ux - lx) + (uy - ly)) : 0ll;
}

// One warp per net of more than 128 pins; lanes stride over the pins.
template <bool kW>
__device__ __forceinline__ long long wa_huge(const WaArgs& A, const WaEval<kW>& V, int bucket,
                                             int local_block) {
  const int lane = threadIdx.x & 31;
  const int k = A.bucket_start[bucket] + local_block * (kBlock / 32) + (threadIdx.x >> 5);
  if (k >= A.bucket_start[bucket + 1]) return 0ll;           // warp-uniform
  const int s = __ldg(&A.net_start[k]), e = __ldg(&A.net_start[k + 1]);
  int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
  for (int q = s + lane; q < e; q += 32) {
    const int2 p = pin_pos(V, __ldg(&A.pins[q]));
    lx = min(lx, p.x); ux = max(ux, p.x); ly = min(ly, p.y); uy = max(uy, p.y);
  }
  lx = __reduce_min_sync(0xffffffffu, lx);
  ly = __reduce_min_sync(0xffffffffu, ly);
  ux = __reduce_max_sync(0xffffffffu, ux);
  uy = __reduce_max_sync(0xffffffffu, uy);
  float S[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int q = s + lane; q < e; q += 32) {
    const int2 p = pin_pos(V, __ldg(&A.pins[q]));
    const PinExp E = pin_exps(p, lx, ux, ly, uy, V.cx, V.cy, A.bar);
    float t[8];
    sums_of(p, E, t);
#pragma unroll
    for (int j = 0; j < 8; j++) S[j] = __fadd_rn(S[j], t[j]);
  }
#pragma unroll
  for (int j = 0; j < 8; j++)
    for (int o = 16; o > 0; o >>= 1) S[j] += __shfl_xor_sync(0xffffffffu, S[j], o);
  const NetCoef K = net_coef(S, V.cx, V.cy);
  for (int q = s + lane; q < e; q += 32) {
    const int4 r = __ldg(&A.pins[q]);
    const int2 p = pin_pos(V, r);
    const PinExp E = pin_exps(p, lx, ux, ly, uy, V.cx, V.cy, A.bar);
    A.pin_grad[q] = weighed(V, k, pin_gradient(p, E, K));
  }
  return lane == 0 ? (long long)((ux - lx) + (uy - ly)) : 0ll;
}

// Buckets 0-5 (nets of up to 64 pins) in one launch; buckets 6-7 (larger
// nets, rare) in a second one, so that their larger register footprint does
// not lower the occupancy of the common case.
constexpr int kWaSplit = 6;

// The unweighted common-net variant is held to 32 registers (seven resident
// blocks of 256 threads per SM instead of six: 71.1 -> 65.4 us at a million
// cells); at 32 registers the weighted one spills (4 bytes), so it keeps six
// blocks per SM (40 registers, no spill); the large-net variants keep their
// registers.
// Block vb of the small-net (kLarge = false) or large-net launch; shared by
// the per-job launch and the batched one.
template <bool kLarge, bool kW>
__device__ __forceinline__ void wa_body(const WaArgs& A, int vb) {
  WaEval<kW> V;
  {
    const EvalCtl* C = A.ctl;
    const int i = C->i_eval;
    V.slp = i == 0 ? A.slp_all[0] : i == 1 ? A.slp_all[1] : i == 2 ? A.slp_all[2] : A.slp_all[3];
    V.cx = C->wl_coef_x;
    V.cy = C->wl_coef_y;
    V.w = A.net_w;
  }
  const int gb = vb + (kLarge ? A.block_start[kWaSplit] : 0);
  int bucket = kLarge ? kWaSplit : 0;
  const int last = kLarge ? kWaBuckets - 1 : kWaSplit - 1;
  while (bucket < last && gb >= A.block_start[bucket + 1]) bucket++;
  const int lb = gb - A.block_start[bucket];
  long long hp = 0;
  if constexpr (!kLarge) {
    switch (bucket) {
      case 0: hp = wa_pair(A, V, lb); break;
      case 1: hp = wa_group<4, kW>(A, V, 1, lb); break;
      case 2: hp = wa_group<8, kW>(A, V, 2, lb); break;
      case 3: hp = wa_group<16, kW>(A, V, 3, lb); break;
      case 4: hp = wa_group<32, kW>(A, V, 4, lb); break;
      default: hp = wa_warp<2, kW>(A, V, 5, lb); break;
    }
  } else {
    if (bucket == 6) hp = wa_warp<4, kW>(A, V, 6, lb);
    else hp = wa_huge(A, V, 7, lb);
  }
  // HPWL is an integer sum, exact in any order: each warp adds its nets'
  // total with one 64-bit atomic, spread over kHpwlLanes accumulators (no
  // block barrier; the gcell kernel sums and clears them)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) hp += __shfl_xor_sync(0xffffffffu, hp, o);
  if ((threadIdx.x & 31) == 0 && hp != 0) {
    const int lane_slot = (gb * (kBlock / 32) + (threadIdx.x >> 5)) % kHpwlLanes;
    atomicAdd(reinterpret_cast<unsigned long long*>(A.hpwl_total + lane_slot * kHpwlStride),
              (unsigned long long)hp);
  }
}

template <bool kLarge, bool kW>
__global__ void __launch_bounds__(kBlock, kLarge ? 1 : (kW ? 6 : 7)) k_wa(const __grid_constant__ WaArgs A) {
  wa_body<kLarge, kW>(A, (int)blockIdx.x);
}

}  // namespace

// bucket 0: a thread per net; 1-4: lane groups of 2 << bucket; 5-7: a warp per net
int wa_nets_per_block(int bucket) { return bucket == 0 ? kBlock : bucket < 5 ? kBlock / (2 << bucket) : kBlock / 32; }

int net_blocks(const DeviceModel& d) { return d.wa_block_start[kWaBuckets]; }

namespace {
WaArgs wa_args(const DeviceModel& d, const EvalArgs& a) {
  WaArgs A;
  for (int b = 0; b <= kWaBuckets; b++) {
    A.bucket_start[b] = d.wa_bucket_start[b];
    A.block_start[b] = d.wa_block_start[b];
  }
  A.net_start = d.net_start;
  A.pins = d.pins;
  for (int k = 0; k < 4; k++) A.slp_all[k] = d.slp[k];
  A.ctl = d.ctl;
  A.bar = a.min_wl_force_bar;
  A.pin_grad = d.pin_grad;
  A.net_w = d.net_w;
  A.hpwl_total = d.hpwl_total;
  return A;
}

// Batched form: work items (instance, block of the instance's small- or
// large-net launch); the block body is the per-job kernel's.
template <bool kLarge, bool kW>
__global__ void __launch_bounds__(kBlock, kLarge ? 1 : 5)
    k_wa_batch(const WaArgs* args, const int4* items, const int* count) {
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    wa_body<kLarge, kW>(args[it.x], it.y);
  }
}
}  // namespace

size_t wa_batch_args_bytes() { return sizeof(WaArgs); }

void wa_launch_blocks(const DeviceModel& d, int* small, int* large) {
  *small = d.wa_block_start[kWaSplit];
  *large = d.wa_block_start[kWaBuckets] - *small;
}

void write_wa_batch_args(const DeviceModel& d, const EvalArgs& a, void* dst) {
  const WaArgs A = wa_args(d, a);
  memcpy(dst, &A, sizeof(A));
}

int launch_wa_batch(bool large, bool weighted, const void* args, const int4* items, const int* count, int grid,
                    cudaStream_t s) {
  const WaArgs* A = static_cast<const WaArgs*>(args);
  if (large) {
    if (weighted) k_wa_batch<true, true><<<grid, kBlock, 0, s>>>(A, items, count);
    else k_wa_batch<true, false><<<grid, kBlock, 0, s>>>(A, items, count);
  } else {
    if (weighted) k_wa_batch<false, true><<<grid, kBlock, 0, s>>>(A, items, count);
    else k_wa_batch<false, false><<<grid, kBlock, 0, s>>>(A, items, count);
  }
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

int launch_wa(DeviceModel& d, const EvalArgs& a, cudaStream_t s, Timer& t) {
  const WaArgs A = wa_args(d, a);
  const int small = d.wa_block_start[kWaSplit];
  const int large = d.wa_block_start[kWaBuckets] - small;
  t.begin(kKWa);
  if (d.net_weighted) {
    if (small) k_wa<false, true><<<small, kBlock, 0, s>>>(A);
    if (large) k_wa<true, true><<<large, kBlock, 0, s>>>(A);
  } else {
    if (small) k_wa<false, false><<<small, kBlock, 0, s>>>(A);
    if (large) k_wa<true, false><<<large, kBlock, 0, s>>>(A);
  }
  t.end(kKWa);
  t.count((small ? 1 : 0) + (large ? 1 : 0));
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

}  // namespace gpl
