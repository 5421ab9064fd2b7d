// Density scatter (BinGrid::updateBinsGCellDensityArea, src/nesterovBase.cpp:746-798)
// fused with the Nesterov predictor (src/nesterovPlace.cpp:338-362), the
// per-gcell gradient kernel (getDensityGradient :1458-1478 + the WA gradient
// sum :1363-1375 + NesterovPlace::updateGradients src/nesterovPlace.cpp:206-273
// + the step-length distances :555-571, 598-607), and the FP64 finalize.
//
// The scatter adds, per (gcell, covered bin), the truncated int64 value of
// the float overlap area times the density scale (times the target density
// for macros) -- the reference's exact per-contribution arithmetic.  Integer
// addition is associative, so atomics give bit-exact, order-independent bin
// areas.  Lanes of a warp that hit the same bin are combined first
// (__match_any_sync), which matters when many cells sit on the same bins
// (all cells start at the core centre).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "device_common.cuh"

namespace gpl {

namespace {

constexpr int kBlock = 256;
constexpr int kBigBins = 64;          // cells covering more bins go to the big-cell kernels
constexpr int kCellBlocksPerSm = 6;   // the gcell kernel's residency (40 registers, a few spilled)

struct ScatterArgs {
  BinGeom geo;
  int n_g;
  float td;
  const int2* half;
  const float* scale;
  const uint8_t* kind;
  float2* slp[4];
  float2* sum[4];
  float2* coordi[2];
  unsigned long long* area[2];  // two sets of inst [nb], filler [nb]
  const EvalCtl* ctl;
};

__device__ __forceinline__ float2 predict_one(const ScatterArgs& A, const EvalCtl& C, int g, int2 h) {
  const float2 cs = pick4(A.slp, C.i_src)[g], sg = pick4(A.sum, C.i_src)[g], cc = pick2(A.coordi, C.c_cur)[g];
  float nx = __fadd_rn(cs.x, __fmul_rn(C.step, sg.x));
  float ny = __fadd_rn(cs.y, __fmul_rn(C.step, sg.y));
  float sx = __fadd_rn(nx, __fmul_rn(C.coeff, __fsub_rn(nx, cc.x)));
  float sy = __fadd_rn(ny, __fmul_rn(C.coeff, __fsub_rn(ny, cc.y)));
  const BinGeom& G = A.geo;
  pick2(A.coordi, C.c_next)[g] = make_float2(inside(nx, h.x, G.core_lx, G.core_ux), inside(ny, h.y, G.core_ly, G.core_uy));
  float2 s = make_float2(inside(sx, h.x, G.core_lx, G.core_ux), inside(sy, h.y, G.core_ly, G.core_uy));
  pick4(A.slp, C.i_eval)[g] = s;
  return s;
}

// ------------------------------------------------------------ tile order
// The scatter visits gcells tile by tile: a tile is tile_w x tile_h bins, and
// the gcells whose centres lie in it (at the last ordering) are consecutive
// in `order`.  A block takes a chunk of at most d.chunk gcells of one tile
// (the tile side and chunk size are tuned per job, see nesterov_init) and
// accumulates their bin areas in a shared-memory window over the
// tile and a margin; the window's non-zero bins then go to the global areas
// with one 64-bit atomic each.  Bins outside the window (cells that moved
// away, large cells) go to the global areas directly.  The int64 sums do not
// depend on the order, so the ordering only changes the number of global
// atomics, never a result.

constexpr int kTileMargin = 2;

struct OrderArgs {
  BinGeom geo;
  int n_g, tile_w, tile_h, tiles_x, tiles_y;
  const float2* slp;            // the coordinates to order by, or (slp == nullptr)
  const float2* slp_all[4];     // slot ctl->i_src of these (the device loop)
  const EvalCtl* ctl;
  int chunk;                    // gcells per chunk (at most)
  int32_t* tile_count;
  int32_t* tile_start;
  int32_t* order;
  int4* chunks;
  int32_t* n_chunks;
};

__device__ __forceinline__ int tile_of(const OrderArgs& O, float2 c) {
  const BinGeom& G = O.geo;
  const int bx = min(max((__float2int_rz(c.x) - G.core_lx) / G.size_x, 0), G.cnt_x - 1);
  const int by = min(max((__float2int_rz(c.y) - G.core_ly) / G.size_y, 0), G.cnt_y - 1);
  return (by / O.tile_h) * O.tiles_x + bx / O.tile_w;
}

__device__ __forceinline__ const float2* order_coords(const OrderArgs& O) {
  return O.slp ? O.slp : pick4(O.slp_all, O.ctl->i_src);
}

// Lanes of a warp on the same tile add their count with one atomic.
__global__ void __launch_bounds__(kBlock) k_order_count(OrderArgs O) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  const float2* slp = order_coords(O);
  const int t = g < O.n_g ? tile_of(O, slp[g]) : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, t);    // every lane takes part
  if (t >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&O.tile_count[t], __popc(peers));
}

// One block: exclusive scan of the tile counts into tile_start, fill cursors
// (tile_count := tile_start), and the chunk table (tiles cut into chunks of
// at most O.chunk gcells).
constexpr int kOrderScanT = 1024;
__global__ void __launch_bounds__(kOrderScanT) k_order_scan(OrderArgs O) {
  __shared__ int32_t sc[kOrderScanT], sk[kOrderScanT];
  const int nt = O.tiles_x * O.tiles_y;
  const int per = (nt + kOrderScanT - 1) / kOrderScanT;
  const int lo = min((int)threadIdx.x * per, nt), hi = min(lo + per, nt);
  int cells = 0, chunks = 0;
  for (int t = lo; t < hi; t++) {
    const int c = O.tile_count[t];
    cells += c;
    chunks += (c + O.chunk - 1) / O.chunk;
  }
  sc[threadIdx.x] = cells;
  sk[threadIdx.x] = chunks;
  __syncthreads();
  for (int o = 1; o < kOrderScanT; o <<= 1) {
    const int x = threadIdx.x >= o ? sc[threadIdx.x - o] : 0;
    const int y = threadIdx.x >= o ? sk[threadIdx.x - o] : 0;
    __syncthreads();
    sc[threadIdx.x] += x;
    sk[threadIdx.x] += y;
    __syncthreads();
  }
  int at = sc[threadIdx.x] - cells, ck = sk[threadIdx.x] - chunks;
  for (int t = lo; t < hi; t++) {
    const int c = O.tile_count[t];
    O.tile_start[t] = at;
    O.tile_count[t] = at;
    for (int f = 0; f < c; f += O.chunk) O.chunks[ck++] = make_int4(t, at + f, at + min(f + O.chunk, c), 0);
    at += c;
  }
  if (threadIdx.x == kOrderScanT - 1) {
    O.tile_start[nt] = sc[kOrderScanT - 1];
    *O.n_chunks = sk[kOrderScanT - 1];
  }
}

__global__ void __launch_bounds__(kBlock) k_order_fill(OrderArgs O) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const float2* slp = order_coords(O);
  const int t = g < O.n_g ? tile_of(O, slp[g]) : -1;
  const unsigned peers = __match_any_sync(0xffffffffu, t);    // every lane takes part
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (t >= 0 && lane == leader) base = atomicAdd(&O.tile_count[t], __popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);               // every lane takes part
  if (t >= 0) O.order[base + __popc(peers & ((1u << lane) - 1u))] = g;
}

struct TileArgs {
  int tile_w, tile_h, tiles_x;
  const int32_t* order;
  const int4* chunks;
  const int32_t* n_chunks;
};

// updateGCellDensityCenterLocation + updateBinsGCellDensityArea
// (src/nesterovBase.cpp:746-819, 1198-1207): one chunk of one tile per block.
// Per (gcell, bin) the area is (int64)(float overlap * scale [* td for a
// macro]), added into the inst or filler set.  The predictor runs here for
// every gcell (big ones included; their bins are left to k_scatter_big).
// The body of one block (chunk vb); `win` is the block's dynamic shared
// window.  Shared by the per-job launch and the batched one.
__device__ __forceinline__ void scatter_body(const ScatterArgs& A, const TileArgs& T, int vb, unsigned* win) {
  if (vb >= *T.n_chunks) return;                   // block-uniform
  const EvalCtl C = *A.ctl;
  unsigned long long* area = pick2(A.area, C.area_cur);
  const BinGeom& G = A.geo;
  const int nb = G.cnt_x * G.cnt_y;
  const int4 ch = T.chunks[vb];
  const int ox = (ch.x % T.tiles_x) * T.tile_w - kTileMargin;
  const int oy = (ch.x / T.tiles_x) * T.tile_h - kTileMargin;
  const int wx = T.tile_w + 2 * kTileMargin, wy = T.tile_h + 2 * kTileMargin, wn = wx * wy;
  unsigned* win_hi = win + 2 * wn;
  for (int i = threadIdx.x; i < 4 * wn; i += blockDim.x) win[i] = 0u;
  __syncthreads();
  for (int idx = ch.y + threadIdx.x; idx < ch.z; idx += blockDim.x) {
    const int g = T.order[idx];
    const int2 h = A.half[g];
    const float2 c = C.predict ? predict_one(A, C, g, h) : pick4(A.slp, C.i_eval)[g];
    const int k = A.kind[g];
    if (k & 4) continue;                           // big cell: k_scatter_big
    int lx, ux, ly, uy, x0, x1, y0, y1;
    density_rect(c, h, lx, ux, ly, uy);
    G.range(lx, ux, ly, uy, x0, x1, y0, y1);
    const float sc = A.scale[g];
    const int half = (k & 3) == 2 ? 1 : 0;
    for (int cc = y0; cc < y1; cc++) {
      for (int a = x0; a < x1; a++) {
        const float ov = G.overlap(a, cc, lx, ux, ly, uy);
        float f = __fmul_rn(ov, sc);
        if ((k & 3) == 1) f = __fmul_rn(f, A.td);          // macro: scale down by target density
        const unsigned long long v = trunc_u64(f);
        if (!v) continue;
        const int u = a - ox, w = cc - oy;
        if (u >= 0 && u < wx && w >= 0 && w < wy && v < (1ull << 32)) {
          // v < 2^32 split into 16-bit halves added to two 32-bit words: a
          // chunk has fewer than 2^16 gcells (set_scatter_shape), one addition
          // each per bin, so neither word can wrap; the adds return nothing
          const int i = half * wn + w * wx + u;
          atomicAdd(&win[i], (unsigned)(v & 0xffffu));
          atomicAdd(&win_hi[i], (unsigned)(v >> 16));
        } else {
          atomicAdd(&area[half * nb + cc * G.cnt_x + a], v);
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * wn; i += blockDim.x) {
    const unsigned long long v = (unsigned long long)win[i] + ((unsigned long long)win_hi[i] << 16);
    if (!v) continue;
    const int half = i >= wn ? 1 : 0, r = i - half * wn;
    const int a = ox + r % wx, cc = oy + r / wx;      // inside the grid: only in-grid bins were added
    atomicAdd(&area[half * nb + cc * G.cnt_x + a], v);
  }
}

__global__ void __launch_bounds__(kBlock, 5) k_scatter(ScatterArgs A, TileArgs T) {
  extern __shared__ unsigned win[];                // [2][wy][wx] low 16-bit sums, then high 16-bit sums
  scatter_body(A, T, (int)blockIdx.x, win);
}

// One block per big cell (macros): threads stride over its bins.
__device__ __forceinline__ void scatter_big_body(const ScatterArgs& A, const int32_t* big, int vb) {
  const EvalCtl C = *A.ctl;
  unsigned long long* area = pick2(A.area, C.area_cur);
  const int g = big[vb];
  const BinGeom& G = A.geo;
  const int nb = G.cnt_x * G.cnt_y;
  const int2 h = A.half[g];
  // k_scatter has already written this cell's predicted coordinates; the
  // block recomputes them with the same arithmetic instead of reading them
  float2 c;
  if (C.predict) {
    __shared__ float2 cs;
    if (threadIdx.x == 0) cs = predict_one(A, C, g, h);
    __syncthreads();
    c = cs;
  } else {
    c = pick4(A.slp, C.i_eval)[g];
  }
  int lx, ux, ly, uy, x0, x1, y0, y1;
  density_rect(c, h, lx, ux, ly, uy);
  G.range(lx, ux, ly, uy, x0, x1, y0, y1);
  if (x1 <= x0 || y1 <= y0) return;
  const int nbx = x1 - x0, total = nbx * (y1 - y0);
  const int k = A.kind[g];
  const float sc = A.scale[g];
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int a = x0 + t % nbx, cc = y0 + t / nbx;
    float f = __fmul_rn(G.overlap(a, cc, lx, ux, ly, uy), sc);
    if ((k & 3) == 1) f = __fmul_rn(f, A.td);
    const long long v = (long long)trunc_u64(f);
    if (v) atomicAdd(&area[((k & 3) == 2 ? nb : 0) + cc * G.cnt_x + a], (unsigned long long)v);
  }
}

__global__ void __launch_bounds__(kBlock) k_scatter_big(ScatterArgs A, const int32_t* big, int n_big) {
  scatter_big_body(A, big, (int)blockIdx.x);
}

struct CellArgs {
  BinGeom geo;
  int n_g;
  const int2* half;
  const float* scale;
  const uint8_t* kind;
  float2* slp[4];
  float2* sum[4];
  const EvalCtl* ctl;
  const float2* field;        // (Ex, Ey) per bin
  const int32_t* g_pin_start;
  const int32_t* g_pins;      // device pin index of each gcell pin slot
  const float2* pin_grad;     // device pin order
  const float2* precond;      // (#pins, dx*dy)
  const int32_t* big_idx;
  float2* d_big;
  float min_precond;
  float2* wl_out;
  float2* d_out;
  double* part;               // [kPartSlots][stride]
  int stride;
  int n_ovf_blocks, n_phi_blocks;
  unsigned* counters;
  long long* hpwl_total;
  double* part_total;         // [kPartSlots] scratch of the final reduction
  EvalResult* out;
};

// Density gradient of one big cell, reduced over a block (fixed tree order).
__device__ __forceinline__ void dgrad_big_body(const CellArgs& A, const int32_t* big, int vb) {
  __shared__ float sx[kBlock], sy[kBlock];
  const int g = big[vb];
  const BinGeom& G = A.geo;
  const EvalCtl C = *A.ctl;
  int lx, ux, ly, uy, x0, x1, y0, y1;
  density_rect(pick4(A.slp, C.i_eval)[g], A.half[g], lx, ux, ly, uy);
  G.range(lx, ux, ly, uy, x0, x1, y0, y1);
  const int nbx = max(x1 - x0, 0), total = nbx * max(y1 - y0, 0);
  const float sc = A.scale[g];
  float ex = 0.0f, ey = 0.0f;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int a = x0 + t % nbx, cc = y0 + t / nbx;
    const float ov = __fmul_rn(G.overlap(a, cc, lx, ux, ly, uy), sc);
    const float2 f = A.field[cc * G.cnt_x + a];
    ex = __fadd_rn(ex, __fmul_rn(ov, f.x));
    ey = __fadd_rn(ey, __fmul_rn(ov, f.y));
  }
  sx[threadIdx.x] = ex; sy[threadIdx.x] = ey;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) { sx[threadIdx.x] += sx[threadIdx.x + s]; sy[threadIdx.x] += sy[threadIdx.x + s]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) A.d_big[vb] = make_float2(sx[0], sy[0]);
}

__global__ void __launch_bounds__(kBlock) k_dgrad_big(CellArgs A, const int32_t* big, int n_big) {
  dgrad_big_body(A, big, (int)blockIdx.x);
}

// One gcell per thread, grid-stride over a grid sized to the SM count; the
// block partial sums are reduced by the last block to finish (threadfence +
// counter), in a fixed order, so there is no separate reduction launch and
// the result is the same run to run.
// Block vb of a launch of vgrid blocks.
__device__ __forceinline__ void cell_body(const CellArgs& A, int vb, int vgrid) {
  __shared__ double sh[32 * kPartSlots];
  __shared__ bool last;
  // per-thread sums in float over the thread's few gcells; FP64 from the
  // warp sums on (the FP64 pipe is narrow on this part)
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};      // |wl|, |d|, coord dist^2, grad dist^2
  int bad = 0;
  const BinGeom& G = A.geo;
  const EvalCtl C = *A.ctl;
  // restrict-qualified views (inputs and outputs are distinct arrays), so
  // the loads of a thread's next gcell can be issued before the stores of
  // its previous one
  const float2* __restrict__ slp = pick4(A.slp, C.i_eval);
  float2* __restrict__ sum_out = C.write_sum ? pick4(A.sum, C.i_eval) : nullptr;
  const float2* __restrict__ ref_slp = C.i_ref >= 0 ? pick4(A.slp, C.i_ref) : nullptr;
  const float2* __restrict__ ref_sum = C.i_ref >= 0 ? pick4(A.sum, C.i_ref) : nullptr;
  float2* __restrict__ wl_out = C.write_wd ? A.wl_out : nullptr;
  float2* __restrict__ d_out = C.write_wd ? A.d_out : nullptr;
  const float2* __restrict__ pin_grad = A.pin_grad;
  const int32_t* __restrict__ g_pins = A.g_pins;
  const int32_t* __restrict__ g_pin_start = A.g_pin_start;
  const float2* __restrict__ field = A.field;
  const int2* __restrict__ half = A.half;
  const uint8_t* __restrict__ kind = A.kind;
  const float* __restrict__ scale = A.scale;
  const float2* __restrict__ precond = A.precond;
  const float lam = C.density_penalty;
  const int lane = threadIdx.x & 31;
  // warp-uniform grid-stride loop: the warps gather the pins of cells with
  // more than 32 pins (macros) together
#pragma unroll 2
  for (int base = vb * kBlock + (threadIdx.x & ~31); base < A.n_g; base += vgrid * kBlock) {
    const int g = base + lane;
    const bool valid = g < A.n_g;
    int ps = 0, pe = 0;
    float2 w = make_float2(0.0f, 0.0f);
    if (valid) {
      ps = g_pin_start[g];
      pe = g_pin_start[g + 1];
      if (pe - ps <= 32) {
        // WA gradient: the cell's pins in instance pin order, four slots'
        // loads in flight at a time (the sums stay in slot order)
        for (int t = ps; t < pe; t += 4) {
          int q[4];
#pragma unroll
          for (int u = 0; u < 4; u++) q[u] = t + u < pe ? g_pins[t + u] : -1;
          float2 pg[4];
#pragma unroll
          for (int u = 0; u < 4; u++) pg[u] = q[u] >= 0 ? pin_grad[q[u]] : make_float2(0.0f, 0.0f);
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (q[u] >= 0) {
              w.x = __fadd_rn(w.x, pg[u].x);
              w.y = __fadd_rn(w.y, pg[u].y);
            }
        }
      }
    }
    unsigned many = __ballot_sync(0xffffffffu, pe - ps > 32);
    while (many) {
      const int src = __ffs(many) - 1;
      many &= many - 1;
      const int s0 = __shfl_sync(0xffffffffu, ps, src), s1 = __shfl_sync(0xffffffffu, pe, src);
      float2 part = make_float2(0.0f, 0.0f);
      for (int t = s0 + lane; t < s1; t += 32) {
        const float2 pg = pin_grad[g_pins[t]];
        part.x = __fadd_rn(part.x, pg.x);
        part.y = __fadd_rn(part.y, pg.y);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        part.x = __fadd_rn(part.x, __shfl_xor_sync(0xffffffffu, part.x, o));
        part.y = __fadd_rn(part.y, __shfl_xor_sync(0xffffffffu, part.y, o));
      }
      if (lane == src) w = part;
    }
    if (!valid) continue;
    const float2 c = slp[g];
    const int k = kind[g];
    // density gradient: sum over covered bins of overlap * scale * field
    float2 d = make_float2(0.0f, 0.0f);
    if (k & 4) {
      d = A.d_big[A.big_idx[g]];
    } else {
      int lx, ux, ly, uy, x0, x1, y0, y1;
      density_rect(c, half[g], lx, ux, ly, uy);
      G.range(lx, ux, ly, uy, x0, x1, y0, y1);
      const float sc = scale[g];
      for (int a = x0; a < x1; a++) {
        for (int cc = y0; cc < y1; cc++) {
          const float ov = __fmul_rn(G.overlap(a, cc, lx, ux, ly, uy), sc);
          const float2 f = field[cc * G.cnt_x + a];
          d.x = __fadd_rn(d.x, __fmul_rn(ov, f.x));
          d.y = __fadd_rn(d.y, __fmul_rn(ov, f.y));
        }
      }
    }
    float2 s = make_float2(__fadd_rn(w.x, __fmul_rn(lam, d.x)), __fadd_rn(w.y, __fmul_rn(lam, d.y)));
    const float2 pc = precond[g];
    float px = __fadd_rn(pc.x, __fmul_rn(lam, pc.y));
    float py = px;
    if (px <= A.min_precond) px = A.min_precond;
    if (py <= A.min_precond) py = A.min_precond;
    s.x = __fdiv_rn(s.x, px);
    s.y = __fdiv_rn(s.y, py);
    if (sum_out) sum_out[g] = s;
    if (wl_out) wl_out[g] = w;
    if (d_out) d_out[g] = d;
    const float aw = fabsf(w.x) + fabsf(w.y);
    const float ad = fabsf(d.x) + fabsf(d.y);
    acc[0] += aw;
    acc[1] += ad;
    if (ref_slp) {
      const float2 r = ref_slp[g], q = ref_sum[g];
      // getDistance (src/nesterovPlace.cpp:598-607): float differences
      const float dx = c.x - r.x, dy = c.y - r.y;
      const float gx = s.x - q.x, gy = s.y - q.y;
      // rounding spelled out: the per-job and the batched kernel inline
      // this body, and must not fuse differently
      acc[2] = __fadd_rn(acc[2], __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
      acc[3] = __fadd_rn(acc[3], __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)));
    }
    if (!isfinite(aw) || !isfinite(ad)) bad = 1;
  }
  {
    // warp sums (float, fixed xor tree), then the block's warps in order in FP64
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    const int any_bad = __any_sync(0xffffffffu, bad);
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < 4; k++) sh[k * 32 + wid] = (double)acc[k];
      sh[4 * 32 + wid] = any_bad ? 1.0 : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
      double t = 0.0;
      for (int w8 = 0; w8 < nw; w8++) t += sh[threadIdx.x * 32 + w8];
      A.part[(size_t)(kPartWl + threadIdx.x) * A.stride + vb] = t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&A.counters[0], 1u) == (unsigned)vgrid - 1;
  }
  __syncthreads();
  if (!last) return;
  // final reduction (the last block): every partial is visible after the
  // fence; all slots are loaded in one pass so the loads overlap
  double tot[kPartSlots];
#pragma unroll
  for (int slot = 0; slot < kPartSlots; slot++) tot[slot] = 0.0;
  const int n_max = max(max(vgrid, A.n_ovf_blocks), A.n_phi_blocks);
  for (int i = threadIdx.x; i < n_max; i += blockDim.x) {
#pragma unroll
    for (int slot = 0; slot < kPartSlots; slot++) {
      const int n = slot == kPartOverflow ? A.n_ovf_blocks
                                          : (slot == kPartPhi ? A.n_phi_blocks : vgrid);
      if (i < n) tot[slot] += __ldcg(A.part + (size_t)slot * A.stride + i);
    }
  }
  // the WA kernel's HPWL accumulators: one per lane of the first warp,
  // summed by shuffles and cleared for the next evaluation
  static_assert(kHpwlLanes == 32, "one HPWL accumulator per lane");
  long long hpwl = 0;
  if (threadIdx.x < 32) {
    hpwl = __ldcg(A.hpwl_total + threadIdx.x * kHpwlStride);
    A.hpwl_total[threadIdx.x * kHpwlStride] = 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) hpwl += __shfl_xor_sync(0xffffffffu, hpwl, o);
  }
  block_reduce_n<kPartSlots>(tot, A.part_total, 1, sh, 0);   // thread 0 writes part_total[k]
  if (threadIdx.x == 0) {
    for (int slot = 0; slot < kPartSlots; slot++) tot[slot] = A.part_total[slot];
    EvalResult r;
    r.overflow = tot[kPartOverflow];
    r.wl_sum = tot[kPartWl];
    r.d_sum = tot[kPartD];
    r.coord_dist = tot[kPartCoordDist];
    r.grad_dist = tot[kPartGradDist];
    r.sum_phi = tot[kPartPhi];
    r.nan_flag = tot[kPartNan];
    r.hpwl = hpwl;
    // getStepLength / getDistance (src/nesterovPlace.cpp:555-571, 598-607)
    const float cd = (float)sqrt(r.coord_dist / (2.0 * A.n_g));
    const float gd = (float)sqrt(r.grad_dist / (2.0 * A.n_g));
    r.new_step_length = cd / gd;
    r.pad = 0;
    *A.out = r;
    A.counters[0] = 0u;
  }
}

__global__ void __launch_bounds__(kBlock, kCellBlocksPerSm) k_cell(CellArgs A) {
  cell_body(A, (int)blockIdx.x, (int)gridDim.x);
}

// sum over bins of phi * (nonPlace + inst + filler) in FP64
// (NesterovBase::updateDensityForceBin, src/nesterovBase.cpp:1494-1505)
__global__ void __launch_bounds__(kBlock) k_sum_phi(const float* phi, const unsigned long long* area,
                                                   const int64_t* nonplace, int nb, double* part) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (int b = blockIdx.x * kBlock + threadIdx.x; b < nb; b += gridDim.x * kBlock)
    v[0] += (double)phi[b] * (double)(nonplace[b] + (long long)area[b] + (long long)area[nb + b]);
  block_reduce_n<1>(v, part, 0, sh);
}

BinGeom geom(const DeviceModel& d) {
  BinGeom G;
  G.core_lx = d.core_lx; G.core_ly = d.core_ly; G.core_ux = d.core_ux; G.core_uy = d.core_uy;
  G.size_x = d.size_x; G.size_y = d.size_y; G.cnt_x = d.cnt_x; G.cnt_y = d.cnt_y;
  return G;
}

}  // namespace

int cell_blocks(const DeviceModel& d) { return (d.n_g + kBlock - 1) / kBlock; }

namespace {
ScatterArgs scatter_args(const DeviceModel& d) {
  ScatterArgs A;
  A.geo = geom(d);
  A.n_g = d.n_g;
  A.td = d.target_density;
  A.half = d.g_half; A.scale = d.g_scale; A.kind = d.g_kind;
  for (int k = 0; k < 4; k++) { A.slp[k] = d.slp[k]; A.sum[k] = d.sum[k]; }
  A.coordi[0] = d.coordi[0]; A.coordi[1] = d.coordi[1];
  A.area[0] = d.area[0]; A.area[1] = d.area[1];
  A.ctl = d.ctl;
  return A;
}

TileArgs tile_args(const DeviceModel& d) {
  TileArgs T;
  T.tile_w = d.tile_w; T.tile_h = d.tile_h; T.tiles_x = d.tiles_x;
  T.order = d.order; T.chunks = d.chunks; T.n_chunks = d.n_chunks;
  return T;
}

CellArgs cell_args(const DeviceModel& d, const EvalArgs& a, int n_phi_blocks) {
  CellArgs A;
  A.geo = geom(d);
  A.n_g = d.n_g;
  A.half = d.g_half; A.scale = d.g_scale; A.kind = d.g_kind;
  for (int k = 0; k < 4; k++) { A.slp[k] = d.slp[k]; A.sum[k] = d.sum[k]; }
  A.ctl = d.ctl;
  A.field = d.field;
  A.g_pin_start = d.g_pin_start;
  A.g_pins = d.g_pins;
  A.pin_grad = d.pin_grad;
  A.precond = d.g_precond;
  A.big_idx = d.g_big_idx; A.d_big = d.d_big;
  A.min_precond = a.min_precond;
  A.wl_out = d.wl_out; A.d_out = d.d_out;
  A.part = d.part;
  A.stride = d.part_stride;
  A.n_ovf_blocks = poisson_blocks_a(d.cnt_x, d.cnt_y);
  A.n_phi_blocks = n_phi_blocks;
  A.counters = d.counters;
  A.hpwl_total = d.hpwl_total;
  A.part_total = d.part_total;
  A.out = d.result;
  return A;
}
}  // namespace

int launch_scatter(DeviceModel& d, const EvalArgs& a, cudaStream_t s, Timer& t) {
  const ScatterArgs A = scatter_args(d);
  const TileArgs T = tile_args(d);
  (void)a;
  t.begin(kKScatter);
  k_scatter<<<d.max_chunks, kBlock, scatter_smem(d), s>>>(A, T);
  if (d.n_big) k_scatter_big<<<d.n_big, kBlock, 0, s>>>(A, d.big_cells, d.n_big);
  t.end(kKScatter);
  t.count(d.n_big ? 2 : 1);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

void tile_grid(int cnt_x, int cnt_y, int side, int* tw, int* th, int* tx, int* ty) {
  *tw = std::min(side, cnt_x);
  *th = std::min(side, cnt_y);
  *tx = (cnt_x + *tw - 1) / *tw;
  *ty = (cnt_y + *th - 1) / *th;
}

// every tile's chunks: one per `chunk` gcells, plus one per tile for the
// partial last chunks
int scatter_max_chunks(int n_g, int tiles, int chunk) { return tiles + (n_g + chunk - 1) / chunk; }

bool set_scatter_shape(DeviceModel& d, int side, int chunk) {
  int tw, th, tx, ty;
  tile_grid(d.cnt_x, d.cnt_y, side, &tw, &th, &tx, &ty);
  const int mc = scatter_max_chunks(d.n_g, tx * ty, chunk);
  if (tx * ty > d.tile_cap || mc > d.chunk_cap || chunk <= 0 || chunk >= 65536) return false;
  d.tile_w = tw; d.tile_h = th; d.tiles_x = tx; d.tiles_y = ty;
  d.chunk = chunk;
  d.max_chunks = mc;
  return true;
}

// the window: two 32-bit words (16-bit split) per bin of the tile and its margin
size_t scatter_smem(const DeviceModel& d) {
  return (size_t)4 * (d.tile_w + 2 * kTileMargin) * (d.tile_h + 2 * kTileMargin) * 4;
}

int scatter_prepare_device() {
  static int done = 0;   // per process (one device in use)
  if (done) return GPL_OK;
  const int side = kTileSides[sizeof(kTileSides) / sizeof(kTileSides[0]) - 1];
  const int smem = 4 * (side + 2 * kTileMargin) * (side + 2 * kTileMargin) * 4;
  GPL_CUDA(cudaFuncSetAttribute(k_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  done = 1;
  return GPL_OK;
}

int launch_tile_order(DeviceModel& d, int slot, cudaStream_t s, Timer& t) {
  OrderArgs O;
  O.geo = geom(d);
  O.n_g = d.n_g;
  O.tile_w = d.tile_w; O.tile_h = d.tile_h; O.tiles_x = d.tiles_x; O.tiles_y = d.tiles_y;
  // slot < 0: the slot the control record's predictor starts from
  O.slp = slot >= 0 ? d.slp[slot] : nullptr;
  for (int k = 0; k < 4; k++) O.slp_all[k] = d.slp[k];
  O.ctl = d.ctl;
  O.chunk = d.chunk;
  O.tile_count = d.tile_count; O.tile_start = d.tile_start; O.order = d.order;
  O.chunks = d.chunks; O.n_chunks = d.n_chunks;
  t.begin(kKOther);
  GPL_CUDA(cudaMemsetAsync(d.tile_count, 0, sizeof(int32_t) * d.tiles_x * d.tiles_y, s));
  k_order_count<<<cell_blocks(d), kBlock, 0, s>>>(O);
  k_order_scan<<<1, kOrderScanT, 0, s>>>(O);
  k_order_fill<<<cell_blocks(d), kBlock, 0, s>>>(O);
  t.end(kKOther);
  t.count(3);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

// The gcell kernel's grid-stride loop runs on one wave of resident blocks
// (kCellBlocksPerSm per SM at its register count), so its last-block
// reduction waits for no second wave.
int cell_grid(const DeviceModel& d) { return std::max(1, std::min(cell_blocks(d), d.sm_count * kCellBlocksPerSm)); }

int launch_cell(DeviceModel& d, const EvalArgs& a, int n_phi_blocks, cudaStream_t s, Timer& t) {
  const CellArgs A = cell_args(d, a, n_phi_blocks);
  t.begin(kKCell);
  if (d.n_big) k_dgrad_big<<<d.n_big, kBlock, 0, s>>>(A, d.big_cells, d.n_big);
  k_cell<<<cell_grid(d), kBlock, 0, s>>>(A);
  t.end(kKCell);
  t.count(d.n_big ? 2 : 1);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

namespace {
// updateInitialPrevSLPCoordi (src/nesterovPlace.cpp:492-512):
// prev = inside(cur + coef * sum), one clamp per axis.
__global__ void __launch_bounds__(kBlock) k_initial_prev(BinGeom G, int n_g, const int2* half,
                                                         const float2* cur, const float2* sum, float coef,
                                                         float2* out) {
  const int g = blockIdx.x * kBlock + threadIdx.x;
  if (g >= n_g) return;
  const int2 h = half[g];
  const float2 c = cur[g], s = sum[g];
  const float x = __fadd_rn(c.x, __fmul_rn(coef, s.x));
  const float y = __fadd_rn(c.y, __fmul_rn(coef, s.y));
  out[g] = make_float2(inside(x, h.x, G.core_lx, G.core_ux), inside(y, h.y, G.core_ly, G.core_uy));
}
}  // namespace

int launch_initial_prev(DeviceModel& d, const float2* cur_slp, const float2* cur_sum, float coef,
                        float2* out, cudaStream_t s, Timer& t) {
  t.begin(kKOther);
  k_initial_prev<<<cell_blocks(d), kBlock, 0, s>>>(geom(d), d.n_g, d.g_half, cur_slp, cur_sum, coef, out);
  t.end(kKOther);
  t.count(1);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

int launch_sum_phi(DeviceModel& d, int area_set, cudaStream_t s, Timer& t, int* n_blocks) {
  const int nb = d.cnt_x * d.cnt_y;
  const int blocks = std::min((nb + kBlock - 1) / kBlock, d.part_stride);
  t.begin(kKOther);
  k_sum_phi<<<blocks, kBlock, 0, s>>>(d.phi, d.area[area_set], d.nonplace, nb,
                                     d.part + (size_t)kPartPhi * d.part_stride);
  t.end(kKOther);
  t.count(1);
  GPL_CUDA(cudaGetLastError());
  *n_blocks = blocks;
  return GPL_OK;
}

// ------------------------------------------------------------ batched form
// Many jobs' evaluations in one launch per phase: a persistent grid whose
// blocks take work items (instance, block of that instance's own launch,
// that launch's grid) from a table and run the same block body as the
// per-job kernels, on the instance's arguments (kept in device memory).  A
// job's blocks therefore compute exactly what its own launch computes.
namespace {

struct ScatterBatchArgs {
  ScatterArgs A;
  TileArgs T;
  const int32_t* big;
};

struct CellBatchArgs {
  CellArgs A;
  const int32_t* big;
};

__global__ void __launch_bounds__(kBlock, 5) k_scatter_batch(const ScatterBatchArgs* args, const int4* items,
                                                             const int* count) {
  extern __shared__ unsigned win[];
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    const ScatterBatchArgs& a = args[it.x];
    scatter_body(a.A, a.T, it.y, win);
    __syncthreads();                  // the window is the next item's
  }
}

__global__ void __launch_bounds__(kBlock) k_scatter_big_batch(const ScatterBatchArgs* args, const int4* items,
                                                              const int* count) {
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    scatter_big_body(args[it.x].A, args[it.x].big, it.y);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kBlock) k_dgrad_big_batch(const CellBatchArgs* args, const int4* items,
                                                            const int* count) {
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    dgrad_big_body(args[it.x].A, args[it.x].big, it.y);
    __syncthreads();
  }
}

// (fewer resident blocks than the per-job kernel: the work-item loop and the
// arguments read from memory need the registers)
__global__ void __launch_bounds__(kBlock, 4) k_cell_batch(const CellBatchArgs* args,
                                                                         const int4* items, const int* count) {
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    cell_body(args[it.x].A, it.y, it.z);
    __syncthreads();
  }
}

}  // namespace

size_t scatter_batch_args_bytes() { return sizeof(ScatterBatchArgs); }
size_t cell_batch_args_bytes() { return sizeof(CellBatchArgs); }

void write_scatter_batch_args(const DeviceModel& d, void* dst) {
  ScatterBatchArgs x;
  x.A = scatter_args(d);
  x.T = tile_args(d);
  x.big = d.big_cells;
  memcpy(dst, &x, sizeof(x));
}

void write_cell_batch_args(const DeviceModel& d, const EvalArgs& a, void* dst) {
  CellBatchArgs x;
  x.A = cell_args(d, a, 0);
  x.big = d.big_cells;
  memcpy(dst, &x, sizeof(x));
}

int scatter_batch_prepare_device() {
  static int done = 0;
  if (done) return GPL_OK;
  const int side = kTileSides[sizeof(kTileSides) / sizeof(kTileSides[0]) - 1];
  const int smem = 4 * (side + 2 * kTileMargin) * (side + 2 * kTileMargin) * 4;
  GPL_CUDA(cudaFuncSetAttribute(k_scatter_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  done = 1;
  return GPL_OK;
}

int launch_density_batch(int phase, const void* args, const int4* items, const int* count, int grid,
                         size_t smem, cudaStream_t s) {
  switch (phase) {
    case kBScatter:
      k_scatter_batch<<<grid, kBlock, smem, s>>>(static_cast<const ScatterBatchArgs*>(args), items, count);
      break;
    case kBScatterBig:
      k_scatter_big_batch<<<grid, kBlock, 0, s>>>(static_cast<const ScatterBatchArgs*>(args), items, count);
      break;
    case kBDgradBig:
      k_dgrad_big_batch<<<grid, kBlock, 0, s>>>(static_cast<const CellBatchArgs*>(args), items, count);
      break;
    case kBCell:
      k_cell_batch<<<grid, kBlock, 0, s>>>(static_cast<const CellBatchArgs*>(args), items, count);
      break;
    default:
      set_error("launch_density_batch: unknown phase");
      return GPL_ERR_INVALID_ARG;
  }
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

}  // namespace gpl
