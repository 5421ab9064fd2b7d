// Initial place: InitialPlace::doBicgstabPlace (src/initialPlace.cpp:56-105).
//
// Each round builds the bound-to-bound (B2B) system of createSparseMatrix
// (:185-378) on the device and solves it for x and y with BiCGSTAB
// (van der Vorst's algorithm with Eigen's stopping and restart rules, the
// reference's solver, src/initialPlace.cpp:78-86).
//
// Matrix assembly.  The reference enumerates, per net, every pin pair in
// which at least one pin is a bound pin (first pin at the net's minimum or
// maximum coordinate, updatePinInfo :128-182) and adds triplets.  Seen from
// one movable pin p, its partners are all other pins of the net when p is a
// bound pin, and the net's bound pins otherwise (pins on p's own instance
// excluded).  Row i of the matrix therefore gathers, over the instance's pins
// and their partners: the diagonal weight, the right-hand side, and one
// off-diagonal entry per movable partner.  Rows are built in two passes
// (count, prefix scan, fill); duplicate columns stay separate entries (the
// product is the same sum).  Each row is written by one thread in a fixed
// order, so the system is deterministic.
//
// Solver.  Vectors are FP32 (as the reference's float Eigen vectors); inner
// products and the rho / alpha / omega scalars are FP64.  Both axes run in
// the same launches (blockIdx.y = axis).  The scalar steps are done by the
// last block of each reduction kernel, so the host only polls a done flag
// (or, with device_loop, one-thread kernels take the host's decisions
// inside one graph).  The batched form runs the same block bodies for many
// jobs from a work table (run_initial_place_batch).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <vector>

#include "device_common.cuh"

namespace gpl {
namespace {

constexpr int kB = 256;

struct BiState {
  double rho, rho_old, alpha, w, r0sq, rhs_sq, tol2, rr, dot_r0r;
  int i, restarts, done, need_restart, zero_x;
  int par;                 // kernel-per-phase form: which p / v buffer holds the current iterate
  int pad[2];
};

struct IpDev {
  int n_mov = 0, n_pins = 0, n_nets = 0;
  // netlist (host pin order)
  int32_t* net_start;      // [n_nets + 1]
  int32_t* pin_net;        // [n_pins]
  int32_t* pin_mov;        // movable instance index of the pin, -1 otherwise
  int32_t* pin_inst;       // instance index (any kind), -1 for IO
  int2* pin_off;           // offset from the instance centre (movable pins)
  int2* pin_fix;           // fixed position (other pins)
  int32_t* mov_pin_start;  // [n_mov + 1] pins of each movable instance (instance pin order)
  int32_t* mov_pins;
  // state
  int2* ctr;               // movable instance centres
  int2* pos;               // pin positions this round
  int4* bound;             // per net: first min-x, max-x, min-y, max-y pin (or -1)
  int n_mp = 0;            // movable pin slots (mov_pins)
  int32_t* cnt;            // [2][n_mp] entries contributed by each movable pin slot
  int32_t* slot_off;       // [2][n_mp + 1] exclusive prefix of cnt (entry offsets)
  float* slot_diag;        // [2][n_mp] diagonal and right-hand side parts per slot
  float* slot_rhs;
  int32_t* rowptr;         // [2][n_mov + 1]
  int32_t* scan_part;      // block sums of the scan
  int32_t* col;            // [2][nnz_cap]
  uint16_t* col16;         // [2][nnz_cap] column - the block's x window start (blocks with a window)
  float* val;
  float* diag;             // [2][n_mov]
  float* b;                // [2][n_mov]
  float *x, *r, *r0, *s, *t;   // [2][n_mov]
  float *p, *v;            // [2 buffers][2][n_mov] (the grid and cluster forms use buffer 0)
  double* part;            // [2][slots][parts]
  double* cpart;           // cooperative solve: [4 phases][2 axes][2][parts]
  struct GridBar* bar;     // cooperative solve: grid barrier
  unsigned* counters;      // [2][8]
  struct IpLoop* loop;     // the device loop's state (kernel-per-phase form)
  BiState* st;             // [2]
  BiState* st_h;           // pinned mirror
  int parts = 0;
  int rows_blk = 0;        // rows per block of the kernel-per-phase SpMV (a multiple of 32)
  int2* win;               // [2][parts] x window (first index, length) of each SpMV block; length 0: none
  size_t nnz_cap = 0;
  char* mem = nullptr;
  size_t bytes = 0;
};

struct IpParams {
  int max_fanout, min_diff;
  float weight_scale;
  int max_iter;
};

// ------------------------------------------------------------ assembly
__device__ __forceinline__ void ip_pos_body(const IpDev& D, int vb) {
  const int q = vb * kB + threadIdx.x;
  if (q >= D.n_pins) return;
  const int m = D.pin_mov[q];
  if (m >= 0) {
    const int2 c = D.ctr[m], o = D.pin_off[q];
    D.pos[q] = make_int2(c.x + o.x, c.y + o.y);
  } else {
    D.pos[q] = D.pin_fix[q];
  }
}

// updatePinInfo: the first pin (in net order) at a strict new minimum or
// maximum keeps the flag, i.e. the first occurrence of the extreme value.
__device__ __forceinline__ void ip_bound_body(const IpDev& D, int vb) {
  const int n = vb * kB + threadIdx.x;
  if (n >= D.n_nets) return;
  int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
  int4 b = make_int4(-1, -1, -1, -1);
  for (int q = D.net_start[n]; q < D.net_start[n + 1]; q++) {
    const int2 p = D.pos[q];
    if (lx > p.x) { lx = p.x; b.x = q; }
    if (ux < p.x) { ux = p.x; b.y = q; }
    if (ly > p.y) { ly = p.y; b.z = q; }
    if (uy < p.y) { uy = p.y; b.w = q; }
  }
  D.bound[n] = b;
}

__device__ __forceinline__ bool net_used(const IpDev& D, const IpParams& P, int n, int& deg) {
  deg = D.net_start[n + 1] - D.net_start[n];
  return deg > 1 && deg < P.max_fanout;
}

__device__ __forceinline__ float pair_weight(const IpParams& P, float net_w, int a, int b) {
  const int diff = abs(a - b);
  return diff > P.min_diff ? net_w / diff : net_w / P.min_diff;
}

// Visit the partners of pin q (movable, instance inst) for one axis.
template <class F>
__device__ __forceinline__ void for_partners(const IpDev& D, int q, int n, int axis, F f) {
  const int4 bd = D.bound[n];
  const int b0 = axis ? bd.z : bd.x, b1 = axis ? bd.w : bd.y;
  const int inst = D.pin_inst[q];
  if (q == b0 || q == b1) {
    for (int r = D.net_start[n]; r < D.net_start[n + 1]; r++)
      if (r != q && D.pin_inst[r] != inst) f(r);
  } else {
    if (b0 >= 0 && D.pin_inst[b0] != inst) f(b0);
    if (b1 >= 0 && b1 != b0 && D.pin_inst[b1] != inst) f(b1);
  }
}

// One movable pin slot t of the B2B assembly: pin q of net n.  A bound pin's
// partners are the other pins of the net (of other instances), a plain pin's
// the net's two bound pins.  Slots are in instance-pin order, so a row of
// the matrix is the concatenation of its instance's slots.
struct Slot {
  int q, n, inst, s, e;
  bool used, bound;
};

__device__ __forceinline__ Slot slot_of(const IpDev& D, const IpParams& P, int t, int axis) {
  Slot c;
  c.q = D.mov_pins[t];
  c.n = D.pin_net[c.q];
  int deg;
  c.used = net_used(D, P, c.n, deg);
  c.s = D.net_start[c.n];
  c.e = D.net_start[c.n + 1];
  c.inst = D.pin_inst[c.q];
  const int4 bd = D.bound[c.n];
  c.bound = c.q == (axis ? bd.z : bd.x) || c.q == (axis ? bd.w : bd.y);
  return c;
}

// Partner lists longer than this (bound pins of large nets) are walked by the
// whole warp, lanes striding over the net's pins.
constexpr int kLongList = 32;

// Entries each slot contributes (movable partners); lanes take one slot each,
// long partner lists are counted by the warp together.
__device__ __forceinline__ void ip_count_body(const IpDev& D, const IpParams& P, int vb, int vgrid, int axis) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (int w = vb * kB + (threadIdx.x & ~31); w < D.n_mp; w += vgrid * kB) {
    const int t = w + lane;
    int c = 0;
    bool lng = false;
    Slot sl{};
    if (t < D.n_mp) {
      sl = slot_of(D, P, t, axis);
      if (sl.used) {
        if (sl.bound && sl.e - sl.s > kLongList) lng = true;
        else for_partners(D, sl.q, sl.n, axis, [&](int r) { if (D.pin_mov[r] >= 0) c++; });
      }
    }
    unsigned longs = __ballot_sync(full, lng);
    while (longs) {
      const int src = __ffs(longs) - 1;
      longs &= longs - 1;
      const int q = __shfl_sync(full, sl.q, src), inst = __shfl_sync(full, sl.inst, src);
      const int ls = __shfl_sync(full, sl.s, src), le = __shfl_sync(full, sl.e, src);
      int part = 0;
      for (int r = ls + lane; r < le; r += 32)
        if (r != q && D.pin_inst[r] != inst && D.pin_mov[r] >= 0) part++;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(full, part, o);
      if (lane == src) c = part;
    }
    if (t < D.n_mp) D.cnt[axis * D.n_mp + t] = c;
  }
}

// exclusive scan of cnt[axis] into rowptr[axis] (three kernels)
__device__ __forceinline__ void scan_blocks_body(const int32_t* in, int32_t* out, int32_t* part, int n, int vb,
                                                 int vgrid, int axis) {
  __shared__ int32_t sh[kB];
  const int i = vb * kB + threadIdx.x;
  const int v = i < n ? in[axis * n + i] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kB; o <<= 1) {
    const int x = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += x;
    __syncthreads();
  }
  if (i < n) out[axis * (n + 1) + i] = sh[threadIdx.x] - v;     // exclusive within the block
  if (threadIdx.x == kB - 1) part[axis * vgrid + vb] = sh[kB - 1];
}

// Exclusive scan of the block sums (one block of kScanT threads per axis:
// contiguous chunks per thread, then a scan of the chunk sums); the total
// goes to out[n].
constexpr int kScanT = 1024;
__device__ __forceinline__ void scan_parts_body(int32_t* part, int nparts, int32_t* out, int n, int axis) {
  __shared__ int32_t sh[kScanT];
  int32_t* pp = part + axis * nparts;
  const int chunk = (nparts + kScanT - 1) / kScanT;
  const int lo = min(threadIdx.x * chunk, nparts), hi = min(lo + chunk, nparts);
  int sum = 0;
  for (int k = lo; k < hi; k++) sum += pp[k];
  sh[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < kScanT; o <<= 1) {
    const int x = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += x;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - sum;
  for (int k = lo; k < hi; k++) {
    const int v = pp[k];
    pp[k] = run;
    run += v;
  }
  if (threadIdx.x == kScanT - 1) out[axis * (n + 1) + n] = sh[kScanT - 1];
}

__device__ __forceinline__ void scan_add_body(int32_t* rowptr, const int32_t* part, int n, int vb, int vgrid,
                                              int axis) {
  const int i = vb * kB + threadIdx.x;
  if (i < n) rowptr[axis * (n + 1) + i] += part[axis * vgrid + vb];
}

// Row pointers: a row starts at its instance's first slot.
__device__ __forceinline__ void ip_rowptr_body(const IpDev& D, int vb, int axis) {
  const int i = vb * kB + threadIdx.x;
  if (i > D.n_mov) return;
  const int t = i < D.n_mov ? D.mov_pin_start[i] : D.n_mp;
  D.rowptr[axis * (D.n_mov + 1) + i] = D.slot_off[axis * (D.n_mp + 1) + t];
}

// createSparseMatrix (src/initialPlace.cpp:221-374), one slot per lane: the
// off-diagonal entries of movable partners at the slot's offset (partner
// order), and the slot's parts of the diagonal and the right-hand side.  Long
// partner lists: the warp walks the net 32 pins at a time and compacts the
// entries in pin order with ballots.
// counters[kFillOverflow]: set if an entry fell outside the entry bound of
// ip_sizes (never expected: the bound is exact for the partner rule); the
// entry is dropped and the initial place reports an error.
constexpr int kFillOverflow = 7;

__device__ __forceinline__ void ip_fill_body(const IpDev& D, const IpParams& P, int vb, int vgrid, int axis) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int32_t* col = D.col + axis * D.nnz_cap;
  float* val = D.val + axis * D.nnz_cap;
  for (int w = vb * kB + (threadIdx.x & ~31); w < D.n_mp; w += vgrid * kB) {
    const int t = w + lane;
    float diag = 0.0f, rhs = 0.0f;
    bool lng = false;
    Slot sl{};
    int at = 0, pq = 0, off_q = 0;
    float net_w = 0.0f;
    if (t < D.n_mp) {
      sl = slot_of(D, P, t, axis);
      at = D.slot_off[axis * (D.n_mp + 1) + t];
      const int i = D.pin_mov[sl.q];
      const int2 ci = D.ctr[i];
      pq = axis ? D.pos[sl.q].y : D.pos[sl.q].x;
      off_q = pq - (axis ? ci.y : ci.x);
      net_w = sl.used ? P.weight_scale / (sl.e - sl.s - 1) : 0.0f;
      if (sl.used) {
        if (sl.bound && sl.e - sl.s > kLongList) {
          lng = true;
        } else {
          for_partners(D, sl.q, sl.n, axis, [&](int r) {
            const int pr = axis ? D.pos[r].y : D.pos[r].x;
            const float wgt = pair_weight(P, net_w, pq, pr);
            diag += wgt;
            const int j = D.pin_mov[r];
            if (j >= 0) {
              if ((size_t)at < D.nnz_cap) {
                col[at] = j;
                val[at] = -wgt;
              } else {
                D.counters[kFillOverflow] = 1u;
              }
              at++;
              const int2 cj = D.ctr[j];
              const int off_r = pr - (axis ? cj.y : cj.x);
              rhs = __fmaf_rn(-wgt, (float)(off_q - off_r), rhs);
            } else {
              rhs = __fmaf_rn(wgt, (float)(pr - off_q), rhs);
            }
          });
        }
      }
    }
    unsigned longs = __ballot_sync(full, lng);
    while (longs) {
      const int src = __ffs(longs) - 1;
      longs &= longs - 1;
      const int q = __shfl_sync(full, sl.q, src), inst = __shfl_sync(full, sl.inst, src);
      const int ls = __shfl_sync(full, sl.s, src), le = __shfl_sync(full, sl.e, src);
      const int spq = __shfl_sync(full, pq, src), soff = __shfl_sync(full, off_q, src);
      const float snw = __shfl_sync(full, net_w, src);
      int sat = __shfl_sync(full, at, src);
      float dg = 0.0f, rh = 0.0f;
      for (int r0 = ls; r0 < le; r0 += 32) {
        const int r = r0 + lane;
        const bool partner = r < le && r != q && D.pin_inst[r] != inst;
        int j = -1;
        float wgt = 0.0f;
        if (partner) {
          const int pr = axis ? D.pos[r].y : D.pos[r].x;
          wgt = pair_weight(P, snw, spq, pr);
          dg += wgt;
          j = D.pin_mov[r];
          if (j >= 0) {
            const int2 cj = D.ctr[j];
            const int off_r = pr - (axis ? cj.y : cj.x);
            rh = __fmaf_rn(-wgt, (float)(soff - off_r), rh);
          } else {
            rh = __fmaf_rn(wgt, (float)(pr - soff), rh);
          }
        }
        const unsigned mv = __ballot_sync(full, partner && j >= 0);
        if (partner && j >= 0) {
          const int k = sat + __popc(mv & ((1u << lane) - 1u));
          if ((size_t)k < D.nnz_cap) {
            col[k] = j;
            val[k] = -wgt;
          } else {
            D.counters[kFillOverflow] = 1u;
          }
        }
        sat += __popc(mv);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dg += __shfl_xor_sync(full, dg, o);
        rh += __shfl_xor_sync(full, rh, o);
      }
      if (lane == src) { diag = dg; rhs = rh; }
    }
    if (t < D.n_mp) {
      D.slot_diag[axis * D.n_mp + t] = diag;
      D.slot_rhs[axis * D.n_mp + t] = rhs;
    }
  }
}

// Diagonal and right-hand side of each row: its slots' parts in pin order.
__device__ __forceinline__ void ip_rowsum_body(const IpDev& D, int vb, int axis) {
  const int i = vb * kB + threadIdx.x;
  if (i >= D.n_mov) return;
  float diag = 0.0f, rhs = 0.0f;
  for (int t = D.mov_pin_start[i]; t < D.mov_pin_start[i + 1]; t++) {
    diag += D.slot_diag[axis * D.n_mp + t];
    rhs += D.slot_rhs[axis * D.n_mp + t];
  }
  D.diag[axis * D.n_mov + i] = diag;
  D.b[axis * D.n_mov + i] = rhs;
}

// The x window of SpMV block vb: its own rows and every column its rows'
// entries read, as (first index, length), or length 0 when that is wider
// than kXWin (the block then gathers from global memory); for a block with
// a window, its entries' columns relative to the window start in 16 bits.
constexpr int kXWinMax = 5632;
__device__ __forceinline__ void ip_window_body(const IpDev& D, int vb, int axis) {
  __shared__ int sh[2][kB / 32];
  const int n = D.n_mov;
  const int r0 = vb * D.rows_blk, r1 = min(r0 + D.rows_blk, n);
  int lo = r0, hi = r1;
  if (r0 < r1) {
    const int32_t* rp = D.rowptr + axis * (n + 1);
    const int32_t* col = D.col + axis * D.nnz_cap;
    const int k1 = (int)min((size_t)rp[r1], D.nnz_cap);
    for (int k = rp[r0] + threadIdx.x; k < k1; k += blockDim.x) {
      const int c = col[k];
      lo = min(lo, c);
      hi = max(hi, c + 1);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = lo; sh[1][wid] = hi; }
  __syncthreads();
  __shared__ int s_lo;
  if (threadIdx.x == 0) {
    for (int w = 1; w < kB / 32; w++) { lo = min(lo, sh[0][w]); hi = max(hi, sh[1][w]); }
    const bool fits = r0 < r1 && hi - lo <= kXWinMax;
    D.win[axis * D.parts + vb] = make_int2(fits ? lo : 0, fits ? hi - lo : 0);
    s_lo = fits ? lo : -1;
  }
  __syncthreads();
  // the window-relative columns the SpMV reads (2 bytes an entry instead of 4)
  const int base = s_lo;
  if (base >= 0) {
    const int32_t* rp = D.rowptr + axis * (n + 1);
    const int32_t* col = D.col + axis * D.nnz_cap;
    uint16_t* col16 = D.col16 + axis * D.nnz_cap;
    const int k1 = (int)min((size_t)rp[r1], D.nnz_cap);
    for (int k = rp[r0] + threadIdx.x; k < k1; k += blockDim.x) col16[k] = (uint16_t)(col[k] - base);
  }
}

// The per-job launches of the assembly phases (blockIdx.y = axis); the
// batched form runs the same bodies from a work table.
__global__ void k_ip_pos(const __grid_constant__ IpDev D) { ip_pos_body(D, (int)blockIdx.x); }
__global__ void k_ip_bound(const __grid_constant__ IpDev D) { ip_bound_body(D, (int)blockIdx.x); }
__global__ void k_ip_count(const __grid_constant__ IpDev D, const __grid_constant__ IpParams P) {
  ip_count_body(D, P, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void k_scan_blocks(const int32_t* in, int32_t* out, int32_t* part, int n) {
  scan_blocks_body(in, out, part, n, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void __launch_bounds__(kScanT) k_scan_parts(int32_t* part, int nparts, int32_t* out, int n) {
  scan_parts_body(part, nparts, out, n, (int)blockIdx.x);
}
__global__ void k_scan_add(int32_t* rowptr, const int32_t* part, int n) {
  scan_add_body(rowptr, part, n, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void k_ip_rowptr(const __grid_constant__ IpDev D) { ip_rowptr_body(D, (int)blockIdx.x, (int)blockIdx.y); }
__global__ void k_ip_fill(const __grid_constant__ IpDev D, const __grid_constant__ IpParams P) {
  ip_fill_body(D, P, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void k_ip_rowsum(const __grid_constant__ IpDev D) { ip_rowsum_body(D, (int)blockIdx.x, (int)blockIdx.y); }
__global__ void k_ip_window(const __grid_constant__ IpDev D) { ip_window_body(D, (int)blockIdx.x, (int)blockIdx.y); }

// ------------------------------------------------------------ solver
// Sparse products: each warp takes windows of 32 consecutive rows (row
// w + lane on each lane), windows strided by the launch's thread count.
//
// Staged form (CSR-stream, Greathouse & Daga, SC'14): a window's rows are
// contiguous in the CSR arrays, so the lanes read the window's whole entry
// range with coalesced loads, put each product val * x[col] (rounded to
// float) in the warp's shared-memory stage, and then each lane adds its own
// row's products in entry order (rows of a bound pin of a large net have
// tens of entries; one in ten rows is such a row, so the stage takes them
// too).  A window whose range exceeds the stage takes the direct form: rows
// of up to kLongRow entries are summed by their own lane with the same
// rounded products in the same order, longer ones (a cell whose pins bound
// many large nets can have over a thousand) by the whole warp, lanes
// striding over the entries and then a shuffle tree, so one long row does
// not hold up the launch.  Which form a window takes depends on the matrix
// only, so every solver form computes the same products.
//
// The loads are what bounds these phases (a memory round trip is about a
// microsecond under load), so each window keeps many in flight: the next
// window's row pointers, diagonal and operands are fetched before the
// current window's entries are read, and the entries are read in batches of
// kBatch coalesced chunks of 32 entries whose index and value loads all
// precede the gathers that depend on them (16 where registers allow, fewer
// in the cooperative and cluster solves; the products are the same).
// kFromL2: read xv through L2 only (in the cooperative and cluster solves
// other blocks wrote it since this block last read it).
constexpr int kLongRow = 32;
constexpr int kStage = 1024;   // floats of shared memory per warp

// dynamic shared memory of a launch whose blocks have `threads` threads
constexpr size_t stage_bytes(int threads) { return (size_t)(threads / 32) * kStage * sizeof(float); }

// The kernel-per-phase SpMV gives each block a contiguous range of rows and
// stages the slice of the multiplied vector that the range's entries read
// (its x window: the lowest to the highest column, at most kXWin floats)
// in shared memory after the warps' product stages, so that the gathers hit
// shared memory instead of L1/L2.  A block whose window is wider reads the
// vector from global memory.  Product stages (32 KB) and window (22 KB) fit
// four blocks per SM, the occupancy the grid is sized for.
constexpr int kXWin = kXWinMax;
constexpr size_t spmv_bytes() { return stage_bytes(kB) + (size_t)kXWin * sizeof(float); }

// Row data of one window, fetched a window ahead.
struct RowFetch {
  int s, e;        // the lane's row entry range
  float acc;       // diag * x_i (the row's first term)
  float aux;       // the caller's per-row operand (read with the row)
};

// Starts moving a window's matrix entries (col and val, rows w .. w + 31)
// from DRAM into L2 while the warp works on the window before it: one bulk
// L2 prefetch per array, issued by lane 0, the range widened to 16-byte
// boundaries (it stays inside the arrays' 256-byte padding).
template <class C>
__device__ __forceinline__ void prefetch_window(const C* col, const float* val, const RowFetch& f, bool valid) {
  const unsigned full = 0xffffffffu;
  const unsigned m = __ballot_sync(full, valid);
  if (!m) return;
  const int last = 31 - __clz(m);
  const int base = __shfl_sync(full, f.s, 0);
  const int end = __shfl_sync(full, f.e, last);
  if ((threadIdx.x & 31) == 0 && end > base) {
    const uintptr_t c0 = reinterpret_cast<uintptr_t>(col + base) & ~uintptr_t(15);
    const uintptr_t c1 = (reinterpret_cast<uintptr_t>(col + end) + 15) & ~uintptr_t(15);
    const uintptr_t v0 = reinterpret_cast<uintptr_t>(val + base) & ~uintptr_t(15);
    const uintptr_t v1 = (reinterpret_cast<uintptr_t>(val + end) + 15) & ~uintptr_t(15);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(c0), "r"((unsigned)(c1 - c0)) : "memory");
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(v0), "r"((unsigned)(v1 - v0)) : "memory");
  }
}

// One window: returns the lane's row product (valid lanes).
template <bool kFromL2, int kBatch, class C, class Ld>
__device__ __forceinline__ float spmv_window(const C* __restrict__ col, const float* __restrict__ val,
                                             Ld ld, const RowFetch& f, bool valid, float* stage) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int s = f.s, e = f.e;
  float acc = f.acc;
  const bool long_row = e - s > kLongRow;
  // the window's entry range: lane 0 is always valid (the window starts in
  // range); the last valid lane ends it
  const int last = __popc(__ballot_sync(full, valid)) - 1;
  const int base = __shfl_sync(full, s, 0);
  const int total = __shfl_sync(full, e, last) - base;
  if (total <= kStage) {
    for (int c0 = 0; c0 < total; c0 += 32 * kBatch) {
      int cj[kBatch];
      float vj[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; b++) {
        const int k = c0 + 32 * b + lane;
        cj[b] = k < total ? (int)__ldg(col + base + k) : 0;
        vj[b] = k < total ? __ldg(val + base + k) : 0.0f;
      }
#pragma unroll
      for (int b = 0; b < kBatch; b++) {
        const int k = c0 + 32 * b + lane;
        if (k < total) stage[k] = __fmul_rn(vj[b], ld(cj[b]));
      }
    }
    __syncwarp();
    int k = s - base;
    const int ke = e - base;
    for (; k + 4 <= ke; k += 4) {
      const float a0 = stage[k], a1 = stage[k + 1], a2 = stage[k + 2], a3 = stage[k + 3];
      acc = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(acc, a0), a1), a2), a3);
    }
    for (; k < ke; k++) acc = __fadd_rn(acc, stage[k]);
    __syncwarp();                 // the stage is free for the warp's next window
    return acc;
  }
  if (!long_row) {
#pragma unroll 4
    for (int k = s; k < e; k++) acc = __fadd_rn(acc, __fmul_rn(val[k], ld(col[k])));
  }
  unsigned longs = __ballot_sync(full, long_row);
  while (longs) {
    const int src = __ffs(longs) - 1;
    longs &= longs - 1;
    const int ls = __shfl_sync(full, s, src), le = __shfl_sync(full, e, src);
    float part = 0.0f;
#pragma unroll 4
    for (int k = ls + lane; k < le; k += 32) part = __fmaf_rn(val[k], ld(col[k]), part);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part = __fadd_rn(part, __shfl_xor_sync(full, part, o));
    if (lane == src) acc = __fadd_rn(acc, part);
  }
  return acc;
}

// (A x)_i for the warp's windows w0, w0 + step, ... below n_end, x_j = gx(j);
// epi(i, value, aux[i]) for every row (kAuxX: aux_i = x_i).  All 32 lanes
// call it together (w0 is warp-uniform).  kWin: every x_j is read from
// xs[j - lo] (the block's x window in shared memory, which holds every
// column the rows read).
template <bool kFromL2 = false, int kBatch = 16, bool kPrefetch = true, bool kWin = false, bool kAuxX = false,
          class GX, class Epi>
__device__ __forceinline__ void spmv_rows(const IpDev& D, int axis, GX gx, const float* aux,
                                          int w0, int step, float* stage, Epi epi, int n_end = -1,
                                          const float* xs = nullptr, int lo = 0) {
  const int n = n_end < 0 ? D.n_mov : n_end;
  const int lane = threadIdx.x & 31;
  // entry columns: window-relative 16-bit in window mode, absolute otherwise
  auto ldc = [&](int c) { return kWin ? xs[c] : gx(c); };
  // the rows' own operands (absolute row index)
  auto ld = [&](int j) { return kWin ? xs[j - lo] : gx(j); };
  const int32_t* __restrict__ rp = D.rowptr + axis * (D.n_mov + 1);
  const int32_t* __restrict__ col = D.col + axis * D.nnz_cap;
  const uint16_t* __restrict__ col16 = D.col16 + axis * D.nnz_cap;
  const float* __restrict__ val = D.val + axis * D.nnz_cap;
  const float* __restrict__ dg = D.diag + axis * D.n_mov;
  auto fetch = [&](int w) {
    RowFetch f{0, 0, 0.0f, 0.0f};
    const int i = w + lane;
    if (i < n) {
      f.s = rp[i];
      f.e = rp[i + 1];
      const float xi = ld(i);
      f.acc = __fmul_rn(dg[i], xi);
      f.aux = kAuxX ? xi : (aux ? (kFromL2 ? __ldcg(aux + i) : aux[i]) : 0.0f);
    }
    return f;
  };
  // row data two windows ahead, matrix entries one window ahead (in L2)
  RowFetch cur = fetch(w0);
  RowFetch next = fetch(w0 + step);
  for (int w = w0; w < n; w += step) {
    if constexpr (kPrefetch) {
      if constexpr (kWin) prefetch_window(col16, val, next, w + step + lane < n);
      else prefetch_window(col, val, next, w + step + lane < n);
    }
    const RowFetch next2 = fetch(w + 2 * step);
    const int i = w + lane;
    float v;
    if constexpr (kWin) v = spmv_window<kFromL2, kBatch>(col16, val, ldc, cur, i < n, stage);
    else v = spmv_window<kFromL2, kBatch>(col, val, ldc, cur, i < n, stage);
    if (i < n) epi(i, v, cur.aux);
    cur = next;
    next = next2;
  }
}

// Vector phases: grid-stride streams with kVecUnroll elements of every array
// in flight per thread (the same elements per thread, in the same order, as
// a plain grid-stride loop).
constexpr int kVecUnroll = 4;

// p = r + beta (p - w v)
template <int U = kVecUnroll>
__device__ __forceinline__ void phase_p(float* p, const float* r, const float* v, float beta, float w,
                                        int i0, int step, int n) {
  for (int i = i0; i < n; i += U * step) {
    float rr[U], pp[U], vv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) { rr[u] = r[k]; pp[u] = p[k]; vv[u] = v[k]; }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) p[k] = __fmaf_rn(beta, __fmaf_rn(-w, vv[u], pp[u]), rr[u]);
    }
  }
}

// s = r - alpha v
template <int U = kVecUnroll>
__device__ __forceinline__ void phase_s(float* s, const float* r, const float* v, float alpha,
                                        int i0, int step, int n) {
  for (int i = i0; i < n; i += U * step) {
    float rr[U], vv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) { rr[u] = r[k]; vv[u] = v[k]; }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) s[k] = __fmaf_rn(-alpha, vv[u], rr[u]);
    }
  }
}

// x += alpha p + w s; r = s - w t; acc += (|r|^2, r0 . r)
template <int U = kVecUnroll>
__device__ __forceinline__ void phase_xr(float* x, float* r, const float* p, const float* s, const float* t,
                                         const float* r0, float alpha, float w, int i0, int step, int n,
                                         float (&acc)[2]) {
  for (int i = i0; i < n; i += U * step) {
    float xx[U], pp[U], ss[U], tt[U], qq[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) { xx[u] = x[k]; pp[u] = p[k]; ss[u] = s[k]; tt[u] = t[k]; qq[u] = r0[k]; }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int k = i + u * step;
      if (k < n) {
        x[k] = __fadd_rn(xx[u], __fmaf_rn(alpha, pp[u], __fmul_rn(w, ss[u])));
        const float ri = __fmaf_rn(-w, tt[u], ss[u]);
        r[k] = ri;
        acc[0] = __fmaf_rn(ri, ri, acc[0]);
        acc[1] = __fmaf_rn(qq[u], ri, acc[1]);
      }
    }
  }
}

// a vector read through L2 only (other blocks wrote it in the same launch)
struct L2Vec {
  const float* v;
  __device__ __forceinline__ float operator()(int j) const { return __ldcg(v + j); }
};

// the calling warp's stage in the launch's dynamic shared memory
__device__ __forceinline__ float* warp_stage() {
  extern __shared__ float stage_all[];
  return stage_all + (threadIdx.x >> 5) * kStage;
}

// The block's SpMV rows [r0, r1) and its x window: x_j = gx(j) over the
// window, written to shared memory (after the product stages) by the whole
// block.
struct BlockRows {
  int r0, r1, lo, span;
  const float* xs;
};
template <class GX>
__device__ __forceinline__ BlockRows block_rows(const IpDev& D, GX gx, int vb, int axis) {
  extern __shared__ float stage_all[];
  BlockRows b;
  b.r0 = vb * D.rows_blk;
  b.r1 = min(b.r0 + D.rows_blk, D.n_mov);
  const int2 w = D.win[axis * D.parts + vb];
  b.lo = w.x;
  b.span = w.y;
  float* xs = stage_all + (kB / 32) * kStage;
  for (int k = threadIdx.x; k < b.span; k += blockDim.x) xs[k] = gx(b.lo + k);
  __syncthreads();
  b.xs = xs;
  return b;
}

// buffer `par` of p or v (axis `axis`)
__device__ __forceinline__ float* pv_buf(float* base, const IpDev& D, int par, int axis) {
  return base + ((size_t)par * 2 + axis) * D.n_mov;
}

// block partial sums of up to 2 products, then the last block of this axis
// runs `fin` with the totals (fixed-order reduction)
template <int N, class Fin>
__device__ __forceinline__ void reduce_and_finish(const IpDev& D, int kernel_id, const float (&vf)[N], Fin fin,
                                                  int vb, int vgrid, int axis) {
  __shared__ double sh[32 * N];
  __shared__ bool last;
  double* part = D.part + (size_t)(axis * 2) * D.parts;
  double v[N];
#pragma unroll
  for (int k = 0; k < N; k++) v[k] = vf[k];      // the thread's rows in float, FP64 across threads
  block_reduce_n<N>(v, part, D.parts, sh, vb);
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&D.counters[axis * 8 + kernel_id], 1u) == (unsigned)vgrid - 1;
  }
  __syncthreads();
  if (!last) return;
  double tot[N];
#pragma unroll
  for (int k = 0; k < N; k++) tot[k] = 0.0;
  for (int b = threadIdx.x; b < vgrid; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < N; k++) tot[k] += __ldcg(part + (size_t)k * D.parts + b);
  __shared__ double tt[N];
  block_reduce_n<N>(tot, tt, 1, sh, 0);
  if (threadIdx.x == 0) {
    double r[N];
#pragma unroll
    for (int k = 0; k < N; k++) r[k] = tt[k];
    fin(D.st[axis], r);
    D.counters[axis * 8 + kernel_id] = 0u;
  }
}

// start of an iteration (Eigen's loop head): stop test, rho, restart test
__device__ __forceinline__ void loop_head(BiState& S, int max_iter) {
  const double eps2 = 1.1920928955078125e-07 * 1.1920928955078125e-07;
  if (!(S.rr > S.tol2 && S.i < max_iter)) { S.done = 1; return; }
  S.rho_old = S.rho;
  S.rho = S.dot_r0r;
  S.need_restart = fabs(S.rho) < eps2 * S.r0sq ? 1 : 0;
}

// r = b - A x (r0 = r when restarting), with |r|^2 and |b|^2
__device__ __forceinline__ void bi_residual_body(const IpDev& D, int init, int max_iter, int vb, int vgrid,
                                                 int axis) {
  float* stage = warp_stage();
  BiState& S = D.st[axis];
  if (!init && (S.done || !S.need_restart)) return;
  const int n = D.n_mov;
  const float* bb = D.b + axis * n;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  float* r0 = D.r0 + axis * n;
  float v[2] = {0.0f, 0.0f};
  auto gx = [&](int j) { return x[j]; };
  const BlockRows br = block_rows(D, gx, vb, axis);
  auto epi = [&](int i, float ax, float bi) {
    const float ri = bi - ax;
    r[i] = ri;
    r0[i] = ri;
    v[0] = __fmaf_rn(ri, ri, v[0]);
    v[1] = __fmaf_rn(bi, bi, v[1]);
  };
  const int w0 = br.r0 + (threadIdx.x & ~31);
  if (br.span) spmv_rows<false, 8, true, true>(D, axis, gx, bb, w0, kB, stage, epi, br.r1, br.xs, br.lo);
  else spmv_rows<false, 8, true, false>(D, axis, gx, bb, w0, kB, stage, epi, br.r1);
  reduce_and_finish<2>(D, 0, v, [&](BiState& s, const double* t) {
    if (init) {
      s.r0sq = t[0];
      s.rr = t[0];
      s.rhs_sq = t[1];
      s.rho = s.alpha = s.w = 1.0;
      s.dot_r0r = t[0];
      s.tol2 = 1.1920928955078125e-07 * 1.1920928955078125e-07 * t[1];
      s.i = 0; s.restarts = 0; s.done = 0; s.need_restart = 0; s.zero_x = 0; s.par = 0;
      if (t[1] == 0.0) { s.zero_x = 1; s.done = 1; s.rr = 0.0; }
      else loop_head(s, max_iter);
    } else {
      s.rho = s.r0sq = s.rr = t[0];
      if (s.restarts++ == 0) s.i = 0;
      s.need_restart = 0;
    }
  }, vb, vgrid, axis);
}

// p = r + beta (p - w v) and v = A p, alpha = rho / (r0 . v): the new p is
// computed where it is read (the block's x window, its own rows for Xr, the
// gathers of a block without a window) from the previous p and v, which
// therefore live in a second buffer (S.par selects the current one).
// kWB: entries per lane in flight in the window path (load scheduling only:
// the arithmetic does not depend on it).
template <int kWB = 8>
__device__ __forceinline__ void bi_pv_body(const IpDev& D, int vb, int vgrid, int axis) {
  float* stage = warp_stage();
  const BiState& S = D.st[axis];
  if (S.done) return;
  // beta once per block: FP64 division is slow on this part
  __shared__ float sc[2];
  if (threadIdx.x == 0) {
    const double beta = (S.rho / S.rho_old) * (S.alpha / S.w);
    sc[0] = (float)beta;                // Eigen's scalars are float
    sc[1] = (float)S.w;
  }
  __syncthreads();
  const float bf = sc[0], wf = sc[1];
  const int par = S.par;
  const float* po = pv_buf(D.p, D, par, axis);
  const float* vo = pv_buf(D.v, D, par, axis);
  float* pn = pv_buf(D.p, D, par ^ 1, axis);
  float* vn = pv_buf(D.v, D, par ^ 1, axis);
  const float* r = D.r + axis * D.n_mov;
  const float* r0 = D.r0 + axis * D.n_mov;
  auto gx = [&](int j) { return __fmaf_rn(bf, __fmaf_rn(-wf, vo[j], po[j]), r[j]); };
  const BlockRows br = block_rows(D, gx, vb, axis);
  for (int i = br.r0 + threadIdx.x; i < br.r1; i += blockDim.x) pn[i] = br.span ? br.xs[i - br.lo] : gx(i);
  float acc[1] = {0.0f};
  auto epi = [&](int i, float vi, float r0i) {
    vn[i] = vi;
    acc[0] = __fmaf_rn(r0i, vi, acc[0]);
  };
  const int w0 = br.r0 + (threadIdx.x & ~31);
  if (br.span) spmv_rows<false, kWB, true, true>(D, axis, gx, r0, w0, kB, stage, epi, br.r1, br.xs, br.lo);
  else spmv_rows<false, 4, true, false>(D, axis, gx, r0, w0, kB, stage, epi, br.r1);   // 3 gathers an entry
  reduce_and_finish<1>(D, 1, acc, [&](BiState& s, const double* t) { s.alpha = s.rho / t[0]; }, vb, vgrid, axis);
}

// s = r - alpha v and t = A s, omega = (t . s) / (t . t): s computed where it
// is read, as p in bi_pv_body; the block writes its own rows' s for Xr.
__device__ __forceinline__ void bi_st_body(const IpDev& D, int vb, int vgrid, int axis) {
  float* stage = warp_stage();
  const BiState& S = D.st[axis];
  if (S.done) return;
  const float af = (float)S.alpha;
  const float* vn = pv_buf(D.v, D, S.par ^ 1, axis);
  const float* r = D.r + axis * D.n_mov;
  float* s = D.s + axis * D.n_mov;
  float* t = D.t + axis * D.n_mov;
  auto gx = [&](int j) { return __fmaf_rn(-af, vn[j], r[j]); };
  const BlockRows br = block_rows(D, gx, vb, axis);
  for (int i = br.r0 + threadIdx.x; i < br.r1; i += blockDim.x) s[i] = br.span ? br.xs[i - br.lo] : gx(i);
  float acc[2] = {0.0f, 0.0f};
  auto epi = [&](int i, float ti, float si) {
    t[i] = ti;
    acc[0] = __fmaf_rn(ti, ti, acc[0]);
    acc[1] = __fmaf_rn(ti, si, acc[1]);
  };
  const int w0 = br.r0 + (threadIdx.x & ~31);
  if (br.span) spmv_rows<false, 8, true, true, true>(D, axis, gx, nullptr, w0, kB, stage, epi, br.r1, br.xs, br.lo);
  else spmv_rows<false, 4, true, false, true>(D, axis, gx, nullptr, w0, kB, stage, epi, br.r1);
  reduce_and_finish<2>(D, 2, acc, [&](BiState& st, const double* tt) {
    st.w = tt[0] > 0.0 ? tt[1] / tt[0] : 0.0;
  }, vb, vgrid, axis);
}

// x += alpha p + omega s; r = s - omega t; |r|^2 and r0 . r; next loop head
__device__ __forceinline__ void bi_xr_body(const IpDev& D, int max_iter, int vb, int vgrid, int axis) {
  const BiState& S = D.st[axis];
  if (S.done) return;
  const int n = D.n_mov;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  const float* p = pv_buf(D.p, D, S.par ^ 1, axis);
  const float* s = D.s + axis * n;
  const float* t = D.t + axis * n;
  const float* r0 = D.r0 + axis * n;
  const float af = (float)S.alpha, wf = (float)S.w;
  float acc[2] = {0.0f, 0.0f};
  phase_xr(x, r, p, s, t, r0, af, wf, vb * kB + threadIdx.x, vgrid * kB, n, acc);
  reduce_and_finish<2>(D, 3, acc, [&](BiState& st, const double* tt) {
    st.rr = tt[0];
    st.dot_r0r = tt[1];
    st.i++;
    st.par ^= 1;
    loop_head(st, max_iter);
  }, vb, vgrid, axis);
}

// The per-job launches of the solver phases (blockIdx.y = axis).
__global__ void __launch_bounds__(kB, 4) k_bi_residual(const __grid_constant__ IpDev D, int init, int max_iter) {
  bi_residual_body(D, init, max_iter, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void __launch_bounds__(kB, 4) k_bi_pv(const __grid_constant__ IpDev D) {
  bi_pv_body(D, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void __launch_bounds__(kB, 4) k_bi_st(const __grid_constant__ IpDev D) {
  bi_st_body(D, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}
__global__ void k_bi_xr(const __grid_constant__ IpDev D, int max_iter) {
  bi_xr_body(D, max_iter, (int)blockIdx.x, (int)gridDim.x, (int)blockIdx.y);
}

// ---------------------------------------------------- cooperative solve
// The whole BiCGSTAB solve of both axes as one cooperative launch: the
// phases of the kernel-per-phase loop (with the p and s updates as phases
// of their own) run in the same order, separated by grid barriers instead
// of kernel boundaries, on the same grid; the rows are strided over the
// blocks (the phase form's SpMV gives each block a contiguous range), so
// the dot products sum in another order and the iterates agree to rounding.
// Every block reduces the partials of both axes itself (same fixed order),
// so every block holds the same solver scalars and the loop ends in step
// across the grid.

struct GridBar {
  unsigned count, gen;
  int err, pad;
};

// At 64 ns per sleep this bounds a wait at about 2 s; a block that gives up
// sets err, and every block leaves at its next barrier.
constexpr unsigned long long kBarSpin = 1ull << 25;

__device__ __forceinline__ bool grid_barrier(GridBar* bar) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &bar->gen;
    volatile int* err = &bar->err;
    const unsigned g = *gen;
    __threadfence();
    const unsigned nb = gridDim.x * gridDim.y;
    if (atomicAdd(&bar->count, 1u) == nb - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g && *err == 0) {
        if (++spins > kBarSpin) { atomicExch(&bar->err, 1); break; }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = (*err == 0);
  }
  __syncthreads();
  return s_ok != 0;
}

// Block sums of float per-thread partials, in FP64 (block_reduce_n).
template <int N>
__device__ __forceinline__ void block_partials(const float (&vf)[N], double* out, int stride, double* sh) {
  double v[N];
#pragma unroll
  for (int k = 0; k < N; k++) v[k] = vf[k];
  block_reduce_n<N>(v, out, stride, sh);
}

__device__ __forceinline__ double* cpart(const IpDev& D, int phase, int axis) {
  return D.cpart + (size_t)((phase * 2 + axis) * 2) * D.parts;
}

// Totals of both axes for one phase, in every block (thread-strided over the
// block partials, then the block tree), as the last block of a kernel sums.
template <int N>
__device__ __forceinline__ void coop_totals(const IpDev& D, int phase, double (&tot)[2][N],
                                            double* sh, double* tt) {
  double v[2 * N];
#pragma unroll
  for (int k = 0; k < 2 * N; k++) v[k] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int k = 0; k < N; k++) v[a * N + k] += __ldcg(cpart(D, phase, a) + (size_t)k * D.parts + b);
  block_reduce_n<2 * N>(v, tt, 1, sh, 0);
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int k = 0; k < N; k++) tot[a][k] = tt[a * N + k];
}

__global__ void __launch_bounds__(kB, 4) k_bi_coop(IpDev D, int max_iter) {
  float* stage = warp_stage();
  __shared__ double sh[32 * 4];
  __shared__ double tt[4];
  __shared__ BiState S[2];
  const int axis = blockIdx.y;
  const int n = D.n_mov;
  if (threadIdx.x < 2) S[threadIdx.x] = D.st[threadIdx.x];
  __syncthreads();
  const float* bb = D.b + axis * n;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  float* r0 = D.r0 + axis * n;
  float* p = D.p + axis * n;
  float* v = D.v + axis * n;
  float* sv = D.s + axis * n;
  float* t = D.t + axis * n;
  const int i0 = blockIdx.x * kB + threadIdx.x, step = gridDim.x * kB;
  const int w0 = blockIdx.x * kB + (threadIdx.x & ~31);
  for (int it = 0; it <= 2 * max_iter + 2; it++) {
    if (S[0].done && S[1].done) break;
    // restart: r = r0 = b - A x
    if ((!S[0].done && S[0].need_restart) || (!S[1].done && S[1].need_restart)) {
      float acc[2] = {0.0f, 0.0f};
      if (!S[axis].done && S[axis].need_restart)
        spmv_rows<true, 4>(D, axis, L2Vec{x}, bb, w0, step, stage, [&](int i, float ax, float bi) {
          const float ri = bi - ax;
          r[i] = ri;
          r0[i] = ri;
          acc[0] = __fmaf_rn(ri, ri, acc[0]);
          acc[1] = __fmaf_rn(bi, bi, acc[1]);
        });
      block_partials<2>(acc, cpart(D, 3, axis), D.parts, sh);
      if (!grid_barrier(D.bar)) return;
      double tot[2][2];
      coop_totals<2>(D, 3, tot, sh, tt);
      if (threadIdx.x == 0)
        for (int a = 0; a < 2; a++) {
          BiState& q = S[a];
          if (q.done || !q.need_restart) continue;
          q.rho = q.r0sq = q.rr = tot[a][0];
          if (q.restarts++ == 0) q.i = 0;
          q.need_restart = 0;
        }
      __syncthreads();
    }
    const bool live = !S[axis].done;
    // p = r + beta (p - w v)
    if (live) {
      const float beta = (float)((S[axis].rho / S[axis].rho_old) * (S[axis].alpha / S[axis].w));
      const float w = (float)S[axis].w;
      phase_p<2>(p, r, v, beta, w, i0, step, n);
    }
    if (!grid_barrier(D.bar)) return;
    // v = A p, alpha = rho / (r0 . v)
    {
      float acc[1] = {0.0f};
      if (live)
        spmv_rows<true, 4>(D, axis, L2Vec{p}, r0, w0, step, stage, [&](int i, float vi, float r0i) {
          v[i] = vi;
          acc[0] = __fmaf_rn(r0i, vi, acc[0]);
        });
      block_partials<1>(acc, cpart(D, 0, axis), D.parts, sh);
      if (!grid_barrier(D.bar)) return;
      double tot[2][1];
      coop_totals<1>(D, 0, tot, sh, tt);
      if (threadIdx.x == 0)
        for (int a = 0; a < 2; a++)
          if (!S[a].done) S[a].alpha = S[a].rho / tot[a][0];
      __syncthreads();
    }
    // s = r - alpha v
    if (live) {
      const float alpha = (float)S[axis].alpha;
      phase_s<2>(sv, r, v, alpha, i0, step, n);
    }
    if (!grid_barrier(D.bar)) return;
    // t = A s, w = (t . s) / (t . t)
    {
      float acc[2] = {0.0f, 0.0f};
      if (live)
        spmv_rows<true, 4>(D, axis, L2Vec{sv}, sv, w0, step, stage, [&](int i, float ti, float si) {
          t[i] = ti;
          acc[0] = __fmaf_rn(ti, ti, acc[0]);
          acc[1] = __fmaf_rn(ti, si, acc[1]);
        });
      block_partials<2>(acc, cpart(D, 1, axis), D.parts, sh);
      if (!grid_barrier(D.bar)) return;
      double tot[2][2];
      coop_totals<2>(D, 1, tot, sh, tt);
      if (threadIdx.x == 0)
        for (int a = 0; a < 2; a++)
          if (!S[a].done) S[a].w = tot[a][0] > 0.0 ? tot[a][1] / tot[a][0] : 0.0;
      __syncthreads();
    }
    // x += alpha p + w s; r = s - w t; then the next loop head
    {
      float acc[2] = {0.0f, 0.0f};
      if (live) {
        const float alpha = (float)S[axis].alpha, w = (float)S[axis].w;
        phase_xr<2>(x, r, p, sv, t, r0, alpha, w, i0, step, n, acc);
      }
      block_partials<2>(acc, cpart(D, 2, axis), D.parts, sh);
      if (!grid_barrier(D.bar)) return;
      double tot[2][2];
      coop_totals<2>(D, 2, tot, sh, tt);
      if (threadIdx.x == 0)
        for (int a = 0; a < 2; a++) {
          BiState& q = S[a];
          if (q.done) continue;
          q.rr = tot[a][0];
          q.dot_r0r = tot[a][1];
          q.i++;
          loop_head(q, max_iter);
        }
      __syncthreads();
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 2) D.st[threadIdx.x] = S[threadIdx.x];
}

// --------------------------------------------------- cluster solve
// For systems of up to kClMaxRows instances: each axis is solved by one
// thread-block cluster of kClCtas CTAs.  The phases are those of k_bi_coop;
// they are separated by the hardware cluster barrier, and the reductions go
// through distributed shared memory: every CTA stores its block sum in its
// own shared slot, and after the barrier each CTA adds the slots of all CTAs
// in rank order, so all CTAs of the cluster hold the same scalars.  Vectors
// other CTAs wrote are read through L2 (spmv_warp<true>).
namespace cg = cooperative_groups;
constexpr int kClCtas = 8;
constexpr int kClThreads = 1024;
constexpr int kClMaxRows = 65536;

template <int N>
__device__ __forceinline__ void cluster_total(cg::cluster_group& cl, const float (&vf)[N], double* slot,
                                              double* sh, double* tot_sh, double (&tot)[N]) {
  double v[N];
#pragma unroll
  for (int k = 0; k < N; k++) v[k] = vf[k];
  block_reduce_n<N>(v, slot, 1, sh, 0);   // slot[k] = this CTA's sum
  cl.sync();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double t = 0.0;
      for (int r = 0; r < kClCtas; r++) t += cl.map_shared_rank(slot, r)[k];
      tot_sh[k] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) tot[k] = tot_sh[k];
}

__global__ void __cluster_dims__(kClCtas, 1, 1) __launch_bounds__(kClThreads, 1)
k_bi_cluster(IpDev D, int max_iter) {
  float* stage = warp_stage();
  cg::cluster_group cl = cg::this_cluster();
  __shared__ double sh[32 * 2];
  __shared__ double slot[4][2];
  __shared__ double tot_sh[2];
  __shared__ BiState S;
  const int axis = blockIdx.y;
  const int n = D.n_mov;
  if (threadIdx.x == 0) S = D.st[axis];
  __syncthreads();
  const float* bb = D.b + axis * n;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  float* r0 = D.r0 + axis * n;
  float* p = D.p + axis * n;
  float* v = D.v + axis * n;
  float* sv = D.s + axis * n;
  float* t = D.t + axis * n;
  const int lane = threadIdx.x & 31;
  const int w0 = (int)cl.block_rank() * kClThreads + (threadIdx.x & ~31);
  const int step = kClCtas * kClThreads;
  for (int it = 0; it <= 2 * max_iter + 2 && !S.done; it++) {
    // restart: r = r0 = b - A x
    if (S.need_restart) {
      float acc[2] = {0.0f, 0.0f};
      spmv_rows<true, 8, false>(D, axis, L2Vec{x}, bb, w0, step, stage, [&](int i, float ax, float bi) {
        const float ri = bi - ax;
        r[i] = ri;
        r0[i] = ri;
        acc[0] = __fmaf_rn(ri, ri, acc[0]);
        acc[1] = __fmaf_rn(bi, bi, acc[1]);
      });
      double tot[2];
      cluster_total<2>(cl, acc, slot[3], sh, tot_sh, tot);
      if (threadIdx.x == 0) {
        S.rho = S.r0sq = S.rr = tot[0];
        if (S.restarts++ == 0) S.i = 0;
        S.need_restart = 0;
      }
      __syncthreads();
    }
    // p = r + beta (p - w v)
    {
      const float beta = (float)((S.rho / S.rho_old) * (S.alpha / S.w));
      const float w = (float)S.w;
      phase_p<2>(p, r, v, beta, w, w0 + lane, step, n);
    }
    cl.sync();
    // v = A p, alpha = rho / (r0 . v)
    {
      float acc[1] = {0.0f};
      spmv_rows<true, 8, false>(D, axis, L2Vec{p}, r0, w0, step, stage, [&](int i, float vi, float r0i) {
        v[i] = vi;
        acc[0] = __fmaf_rn(r0i, vi, acc[0]);
      });
      double tot[1];
      cluster_total<1>(cl, acc, slot[0], sh, tot_sh, tot);
      if (threadIdx.x == 0) S.alpha = S.rho / tot[0];
      __syncthreads();
    }
    // s = r - alpha v
    {
      const float alpha = (float)S.alpha;
      phase_s<2>(sv, r, v, alpha, w0 + lane, step, n);
    }
    cl.sync();
    // t = A s, w = (t . s) / (t . t)
    {
      float acc[2] = {0.0f, 0.0f};
      spmv_rows<true, 8, false>(D, axis, L2Vec{sv}, sv, w0, step, stage, [&](int i, float ti, float si) {
        t[i] = ti;
        acc[0] = __fmaf_rn(ti, ti, acc[0]);
        acc[1] = __fmaf_rn(ti, si, acc[1]);
      });
      double tot[2];
      cluster_total<2>(cl, acc, slot[1], sh, tot_sh, tot);
      if (threadIdx.x == 0) S.w = tot[0] > 0.0 ? tot[1] / tot[0] : 0.0;
      __syncthreads();
    }
    // x += alpha p + w s; r = s - w t; then the next loop head
    {
      float acc[2] = {0.0f, 0.0f};
      const float alpha = (float)S.alpha, w = (float)S.w;
      phase_xr<2>(x, r, p, sv, t, r0, alpha, w, w0 + lane, step, n, acc);
      double tot[2];
      cluster_total<2>(cl, acc, slot[2], sh, tot_sh, tot);
      if (threadIdx.x == 0) {
        S.rr = tot[0];
        S.dot_r0r = tot[1];
        S.i++;
        loop_head(S, max_iter);
      }
      __syncthreads();
    }
  }
  if (cl.block_rank() == 0 && threadIdx.x == 0) D.st[axis] = S;
  cl.sync();   // no CTA leaves while another may still read its shared memory
}

// rhs == 0: Eigen sets x = 0; then the instances move to the solution
// (InitialPlace::updateCoordi :380-385, float -> int truncation)
__device__ __forceinline__ void ip_move_body(const IpDev& D, int vb) {
  const int i = vb * kB + threadIdx.x;
  if (i >= D.n_mov) return;
  const int n = D.n_mov;
  float x = D.x[i], y = D.x[n + i];
  if (D.st[0].zero_x) { x = 0.0f; D.x[i] = 0.0f; }
  if (D.st[1].zero_x) { y = 0.0f; D.x[n + i] = 0.0f; }
  D.ctr[i] = make_int2((int)x, (int)y);
}

// Start of one solve: the warm start is the instances' current centres
// (instLocVecX_ = inst->cx(), src/initialPlace.cpp:211-218) and, as every
// BiCGSTAB solve begins, p = v = 0.
__device__ __forceinline__ void ip_guess_body(const IpDev& D, int vb) {
  const int i = vb * kB + threadIdx.x;
  if (i >= D.n_mov) return;
  const int2 c = D.ctr[i];
  const int n = D.n_mov;
  D.x[i] = (float)c.x;
  D.x[n + i] = (float)c.y;
  D.p[i] = D.p[n + i] = 0.0f;
  D.v[i] = D.v[n + i] = 0.0f;
}

__global__ void k_ip_move(const __grid_constant__ IpDev D) { ip_move_body(D, (int)blockIdx.x); }
__global__ void k_ip_guess(const __grid_constant__ IpDev D) { ip_guess_body(D, (int)blockIdx.x); }

// ------------------------------------------------------------ batched form
// The phases of the kernel-per-phase solve for many jobs at once: block b of
// a batched launch takes work item items[b] = (job, block of the job's own
// launch, that launch's grid, axis) and runs the per-job kernel's body on
// the job's tables, so every job computes exactly what its own launches
// compute (the bodies spell their floating-point rounding out, so the
// arithmetic does not depend on the kernel they are compiled into).
enum IpPhase {
  kIpPos = 0, kIpBound, kIpCount, kIpScanBlocks, kIpScanAdd, kIpRowptr, kIpFill, kIpRowsum, kIpGuess,
  kIpResidualInit, kIpResidual, kIpPV, kIpST, kIpXr, kIpMove, kIpWindow
};

template <int Ph>
__global__ void __launch_bounds__(kB, 4) k_ipb(const IpDev* __restrict__ Ds, const IpParams* __restrict__ Ps,
                                            const int4* __restrict__ items) {
  // the job's tables in shared memory (IpDev is a few hundred bytes)
  __shared__ __align__(16) unsigned char raw[sizeof(IpDev)];
  static_assert(sizeof(IpDev) % 4 == 0, "IpDev is copied as words");
  const int4 it = items[blockIdx.x];
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(Ds + it.x);
    unsigned* dst = reinterpret_cast<unsigned*>(raw);
    for (int w = threadIdx.x; w < (int)(sizeof(IpDev) / 4); w += blockDim.x) dst[w] = src[w];
  }
  __syncthreads();
  const IpDev& D = *reinterpret_cast<const IpDev*>(raw);
  const int vb = it.y, vg = it.z, ax = it.w;
  if constexpr (Ph == kIpPos) ip_pos_body(D, vb);
  else if constexpr (Ph == kIpBound) ip_bound_body(D, vb);
  else if constexpr (Ph == kIpCount) { const IpParams P = Ps[it.x]; ip_count_body(D, P, vb, vg, ax); }
  else if constexpr (Ph == kIpScanBlocks) scan_blocks_body(D.cnt, D.slot_off, D.scan_part, D.n_mp, vb, vg, ax);
  else if constexpr (Ph == kIpScanAdd) scan_add_body(D.slot_off, D.scan_part, D.n_mp, vb, vg, ax);
  else if constexpr (Ph == kIpRowptr) ip_rowptr_body(D, vb, ax);
  else if constexpr (Ph == kIpFill) { const IpParams P = Ps[it.x]; ip_fill_body(D, P, vb, vg, ax); }
  else if constexpr (Ph == kIpRowsum) ip_rowsum_body(D, vb, ax);
  else if constexpr (Ph == kIpGuess) ip_guess_body(D, vb);
  else if constexpr (Ph == kIpResidualInit) bi_residual_body(D, 1, Ps[it.x].max_iter, vb, vg, ax);
  else if constexpr (Ph == kIpResidual) bi_residual_body(D, 0, Ps[it.x].max_iter, vb, vg, ax);
  else if constexpr (Ph == kIpPV) bi_pv_body<4>(D, vb, vg, ax);   // 4: no spills with the tables in shared memory
  else if constexpr (Ph == kIpST) bi_st_body(D, vb, vg, ax);
  else if constexpr (Ph == kIpXr) bi_xr_body(D, Ps[it.x].max_iter, vb, vg, ax);
  else if constexpr (Ph == kIpMove) ip_move_body(D, vb);
  else if constexpr (Ph == kIpWindow) ip_window_body(D, vb, ax);
}

// the scan of the block sums: one block of kScanT threads per (job, axis)
__global__ void __launch_bounds__(kScanT) k_ipb_scan_parts(const IpDev* __restrict__ Ds,
                                                           const int4* __restrict__ items) {
  const int4 it = items[blockIdx.x];
  const IpDev& D = Ds[it.x];
  scan_parts_body(D.scan_part, it.z, D.slot_off, D.n_mp, it.w);
}

// both solver states of every job into one array (one copy to the host)
__global__ void k_ipb_states(const IpDev* __restrict__ Ds, const int* __restrict__ jobs, int n, BiState* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < 2 * n) out[k] = Ds[jobs[k >> 1]].st[k & 1];
}

// ------------------------------------------------------------ device loop
// The rounds of the kernel-per-phase form as one CUDA graph: WHILE (rounds
// go on) { assembly; WHILE (a solve goes on) { 8 iterations; chunk tail };
// move; round tail }.  The one-thread tails take the decisions the host loop
// takes between its chunks and rounds (same tests, same values), so the host
// waits once per initial place instead of once per chunk.
struct IpLoop {
  int round, chunks, max_rounds, iter_limit;   // iter_limit: the host loop's 2 * max_iter + 2
  int finished, iters_x, iters_y;
  float err;
};

__global__ void k_ip_loop_head(IpLoop* L, int max_rounds, int iter_limit, cudaGraphConditionalHandle h_round) {
  IpLoop l{};
  l.max_rounds = max_rounds;
  l.iter_limit = iter_limit;
  *L = l;
  cudaGraphSetConditional(h_round, max_rounds > 0 ? 1u : 0u);
}

__global__ void k_ip_chunk_head(IpLoop* L, cudaGraphConditionalHandle h_chunk) {
  L->chunks = 0;
  cudaGraphSetConditional(h_chunk, 1u);
}

// after a chunk: another one while a solve goes on and the host loop's
// iteration bound allows (it counts 8 per chunk from 0)
__global__ void k_ip_chunk_tail(const BiState* st, IpLoop* L, cudaGraphConditionalHandle h_chunk) {
  const int n = ++L->chunks;
  const bool done = st[0].done && st[1].done;
  cudaGraphSetConditional(h_chunk, (!done && 8 * n <= L->iter_limit) ? 1u : 0u);
}

// after the move: the round's error (solver.error() = sqrt(|r|^2 / |b|^2),
// in double as on the host) and the stop test (src/initialPlace.cpp:93-99)
__global__ void k_ip_round_tail(const BiState* st, IpLoop* L, cudaGraphConditionalHandle h_round) {
  IpLoop l = *L;
  l.round++;
  const float ex = st[0].rhs_sq > 0 ? (float)sqrt(st[0].rr / st[0].rhs_sq) : 0.0f;
  const float ey = st[1].rhs_sq > 0 ? (float)sqrt(st[1].rr / st[1].rhs_sq) : 0.0f;
  l.err = ex < ey ? ey : ex;
  l.iters_x = st[0].i;
  l.iters_y = st[1].i;
  l.finished = ((l.err <= 1e-5 && l.round >= 5) || l.round >= l.max_rounds) ? 1 : 0;
  *L = l;
  cudaGraphSetConditional(h_round, l.finished ? 0u : 1u);
}

int blocks_for(int n) { return std::max(1, (n + kB - 1) / kB); }

}  // namespace

// Rows per thread of the SpMV phases when the grid is not capped.  Small
// systems (up to kSmallRows rows, latency-bound alone) take one row per
// thread: one SpMV window per warp, the shortest kernel; larger ones four
// (four windows per warp, the next one's row data fetched while the current
// one is summed).  The x + r phase of a small system runs on a quarter of
// the SpMV grid (four vector elements per thread, all in flight at once:
// no longer alone, and a quarter of the blocks' FP64 block reductions when
// many jobs run batched).
constexpr int kSmallRows = 65536;
int solve_rows(size_t n) { return n <= (size_t)kSmallRows ? 1 : 4; }

struct IpSizes {
  size_t nnz_cap = 1, bytes = 0;
  int grid = 1;        // SpMV blocks per axis
  int xr_grid = 1;     // x + r blocks per axis
  int parts = 1;       // block partials per axis and value (the larger grid)
  int rows_blk = 32;
};

// Scratch layout of run_initial_place (the sizes its carving below takes).
IpSizes ip_sizes(const HostModel& m, int grid_cap) {
  IpSizes z;
  const size_t nP = m.place_insts.size();
  size_t n_mp = 0;
  for (int i : m.place_insts) n_mp += m.inst_pin_start[i + 1] - m.inst_pin_start[i];
  // An upper bound of the off-diagonal entries per axis (see for_partners):
  // a net of degree d has at most two bound pins, each partnering at most
  // d - 1 pins, and every other pin partners at most the two bound pins, so
  // the net contributes at most 2 (d - 1) + 2 (d - 2) = 4 d - 6 entries (one
  // bound pin for both ends: (d - 1) + (d - 1) <= 4 d - 6 for d >= 2).
  size_t nnz = 0;
  for (int n = 0; n < m.n_nets; n++) {
    const size_t deg = m.net_start[n + 1] - m.net_start[n];
    if (deg > 1 && (int)deg < m.p.initial_place_max_fanout) nnz += 4 * deg - 6;
  }
  z.nnz_cap = std::max<size_t>(nnz, 1);
  // solve_rows rows per thread, at most grid_cap blocks per axis
  const size_t rows_per_block = (size_t)kB * solve_rows(nP);
  const int g0 = std::max(1, std::min((int)((nP + rows_per_block - 1) / rows_per_block), grid_cap));
  // the SpMV's contiguous row ranges: whole windows of 32 rows per block
  z.rows_blk = std::max(32, (int)((nP + g0 - 1) / g0 + 31) / 32 * 32);
  z.grid = std::max(1, (int)((nP + z.rows_blk - 1) / z.rows_blk));
  // x + r of a small system: four elements per thread, all in flight at
  // once (a larger grid for the capped large systems measured slower)
  z.xr_grid = nP <= (size_t)kSmallRows ? (z.grid + 3) / 4 : z.grid;
  z.parts = std::max(z.grid, z.xr_grid);
  const size_t scan_blocks = blocks_for((int)n_mp);
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += (b + 255) / 256 * 256 + 256; };
  add((m.n_nets + 1) * 4); add(m.n_pins * 4); add(m.n_pins * 4); add(m.n_pins * 4);
  add(m.n_pins * 8); add(m.n_pins * 8); add((nP + 1) * 4); add(n_mp * 4);
  add(nP * 8); add(m.n_pins * 8); add(m.n_nets * 16); add(2 * n_mp * 4); add(2 * (n_mp + 1) * 4);
  add(2 * n_mp * 4); add(2 * n_mp * 4); add(2 * (nP + 1) * 4);
  add(2 * scan_blocks * 4); add(2 * z.nnz_cap * 4); add(2 * z.nnz_cap * 2); add(2 * z.nnz_cap * 4);
  for (int k = 0; k < 7; k++) add(2 * nP * 4);
  for (int k = 0; k < 2; k++) add(2 * 2 * nP * 4);
  add(2 * 2 * (size_t)z.parts * 8); add(4 * 2 * 2 * (size_t)z.parts * 8); add(sizeof(GridBar));
  add(2 * (size_t)z.parts * 8);
  add(16 * 4); add(sizeof(IpLoop)); add(2 * sizeof(BiState));
  z.bytes = bytes;
  return z;
}

// (a cooperative grid has at most 8 blocks of kB threads per SM, 2 axes)
size_t initial_place_bytes(const HostModel& m, int sm_count) { return ip_sizes(m, sm_count * 8).bytes; }

// One job's initial place on the device: its scratch, tables and solver
// state (ip_setup), the rounds (run_initial_place's loop, or the batched
// form's lockstep rounds), and the read-back (ip_finish).
// offset of the device loop's state copy in the job's pinned ip_state block
constexpr size_t kIpLoopPinned = 512;

struct IpRun {
  HostModel* m = nullptr;
  cudaStream_t s = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaEvent_t sync_ev = nullptr;
  IpDev D;
  IpParams P;
  int nP = 0, nb_mov = 0, grid = 1, xr_grid = 1, scan_blocks = 1;
  bool cluster = false, coop = false;
  int coop_attr = 0, per_sm = 0;
  std::vector<int2> ctr;         // host centres (read back at the end)
  BiState* st_h = nullptr;       // pinned solver states [2] (+ GridBar)
  int rounds = 0, iters[2] = {0, 0}, coop_rounds = 0;
  float err = 0.0f;
  bool finished = false;         // the rounds are over (stop test or limit)
  double t_start = 0.0;
};

namespace {
double wall_now() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

int ip_setup(HostModel& m, cudaStream_t s, int sm_count, void* pinned, cudaMemPool_t pool, cudaEvent_t sync_ev,
             IpRun& R) {
  static_assert(2 * sizeof(BiState) + sizeof(GridBar) <= kIpLoopPinned &&
                    kIpLoopPinned + sizeof(IpLoop) <= sizeof(HostPinned::ip_state),
                "pinned solver state too small");
  R.m = &m;
  R.s = s;
  R.pool = pool;
  R.sync_ev = sync_ev;
  R.st_h = static_cast<BiState*>(pinned);
  R.t_start = wall_now();
  IpDev& D = R.D;
  const gpl_params& prm = m.p;
  const auto wall = wall_now;
  const double t_start = R.t_start;
  D.n_mov = (int)m.place_insts.size();
  D.n_pins = m.n_pins;
  D.n_nets = m.n_nets;
  const int nP = D.n_mov;
  // the per-pin host arrays are filled by a few threads (parallel_ranges)
  std::vector<int32_t> ext(m.n_insts, -1);
  for (int k = 0; k < nP; k++) ext[m.place_insts[k]] = k;
  RawArray<int32_t> pin_net(m.n_pins), pin_mov(m.n_pins);
  RawArray<int2> pin_off(m.n_pins), pin_fix(m.n_pins);
  std::vector<int32_t> mps(nP + 1, 0);
  for (int k = 0; k < nP; k++) {
    const int i = m.place_insts[k];
    mps[k + 1] = mps[k] + (m.inst_pin_start[i + 1] - m.inst_pin_start[i]);
  }
  RawArray<int32_t> mp(mps[nP]);
  RawArray<int2> ctr(nP);
  parallel_ranges(m.n_nets, [&](int a, int b) {
    for (int n = a; n < b; n++)
      for (int q = m.net_start[n]; q < m.net_start[n + 1]; q++) pin_net[q] = n;
  });
  parallel_ranges(m.n_pins, [&](int a, int b) {
    for (int q = a; q < b; q++) {
      const int i = m.pin_inst[q];
      pin_mov[q] = i >= 0 ? ext[i] : -1;
      pin_off[q] = make_int2(m.pin_ox[q], m.pin_oy[q]);
      pin_fix[q] = make_int2(m.pin_x[q], m.pin_y[q]);
    }
  });
  parallel_ranges(nP, [&](int a, int b) {
    for (int k = a; k < b; k++) {
      const int i = m.place_insts[k];
      int w = mps[k];
      for (int t = m.inst_pin_start[i]; t < m.inst_pin_start[i + 1]; t++) mp[w++] = m.inst_pins[t];
      ctr[k] = make_int2((m.ilx[i] + m.iux[i]) / 2, (m.ily[i] + m.iuy[i]) / 2);
    }
  });
  // The cooperative solve needs its whole grid (both axes) resident at once.
  int dev = 0, coop_attr = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop_attr, cudaDevAttrCooperativeLaunch, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bi_coop, kB, stage_bytes(kB));
  // the cluster solve's stages exceed the default dynamic shared-memory cap
  cudaFuncSetAttribute(k_bi_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_bytes(kClThreads));
  // the SpMV phases' product stages and x window exceed the default cap too
  for (const void* f : {(const void*)k_bi_residual, (const void*)k_bi_pv, (const void*)k_bi_st,
                        (const void*)k_ipb<kIpResidualInit>, (const void*)k_ipb<kIpResidual>,
                        (const void*)k_ipb<kIpPV>, (const void*)k_ipb<kIpST>})
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spmv_bytes());
  cudaGetLastError();
  // ip_solver: 0 auto, 1 kernel per phase, 2 cooperative grid, 3 cluster per axis
  const int mode = prm.ip_solver;
  // Auto is the phase form: it keeps the SpMV's gathers in L1 (the grid and
  // cluster forms must read vectors other blocks wrote in the same launch
  // through L2), which makes it the fastest form alone from about 50,000
  // instances up and, because its short kernels interleave with other jobs'
  // kernels, the best one under the placement server at every size.
  bool cluster = mode == 3 && nP <= kClMaxRows;
  bool coop = !cluster && coop_attr != 0 && per_sm > 0 && mode == 2;
  // the same grid either way, so both solvers give the same iterates
  const int grid_cap = (coop_attr != 0 && per_sm > 0) ? std::max(1, per_sm * sm_count / 2) : sm_count * 8;
  const IpSizes z = ip_sizes(m, grid_cap);
  D.nnz_cap = z.nnz_cap;
  const int nb_mov = blocks_for(nP);
  const int grid = z.grid;
  D.parts = z.parts;
  D.rows_blk = z.rows_blk;
  D.n_mp = (int)mp.size();
  const int scan_blocks = blocks_for(D.n_mp);
  const double t_host = wall();
  cudaError_t e = dev_alloc((void**)&D.mem, z.bytes, pool, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(std::string("initial place: device allocation failed: ") + cudaGetErrorString(e));
    return GPL_ERR_OUT_OF_MEMORY;
  }
  char* cur = D.mem;
  auto take = [&](size_t b) { char* r = cur; cur += (b + 255) / 256 * 256 + 256; return r; };
  D.net_start = (int32_t*)take((m.n_nets + 1) * 4);
  D.pin_net = (int32_t*)take(m.n_pins * 4);
  D.pin_mov = (int32_t*)take(m.n_pins * 4);
  D.pin_inst = (int32_t*)take(m.n_pins * 4);
  D.pin_off = (int2*)take(m.n_pins * 8);
  D.pin_fix = (int2*)take(m.n_pins * 8);
  D.mov_pin_start = (int32_t*)take((nP + 1) * 4);
  D.mov_pins = (int32_t*)take(mp.size() * 4);
  D.ctr = (int2*)take(nP * 8);
  D.pos = (int2*)take(m.n_pins * 8);
  D.bound = (int4*)take(m.n_nets * 16);
  D.cnt = (int32_t*)take(2 * (size_t)D.n_mp * 4);
  D.slot_off = (int32_t*)take(2 * ((size_t)D.n_mp + 1) * 4);
  D.slot_diag = (float*)take(2 * (size_t)D.n_mp * 4);
  D.slot_rhs = (float*)take(2 * (size_t)D.n_mp * 4);
  D.rowptr = (int32_t*)take(2 * (nP + 1) * 4);
  D.scan_part = (int32_t*)take(2 * scan_blocks * 4);
  D.col = (int32_t*)take(2 * D.nnz_cap * 4);
  D.col16 = (uint16_t*)take(2 * D.nnz_cap * 2);
  D.val = (float*)take(2 * D.nnz_cap * 4);
  D.diag = (float*)take(2 * nP * 4);
  D.b = (float*)take(2 * nP * 4);
  D.x = (float*)take(2 * nP * 4);
  D.r = (float*)take(2 * nP * 4);
  D.r0 = (float*)take(2 * nP * 4);
  D.p = (float*)take(2 * 2 * nP * 4);
  D.v = (float*)take(2 * 2 * nP * 4);
  D.s = (float*)take(2 * nP * 4);
  D.t = (float*)take(2 * nP * 4);
  D.part = (double*)take(2 * 2 * (size_t)D.parts * 8);
  D.cpart = (double*)take(4 * 2 * 2 * (size_t)D.parts * 8);
  D.bar = (GridBar*)take(sizeof(GridBar));
  D.win = (int2*)take(2 * (size_t)D.parts * 8);
  D.counters = (unsigned*)take(16 * 4);
  D.loop = (IpLoop*)take(sizeof(IpLoop));
  D.st = (BiState*)take(2 * sizeof(BiState));
  int rc = GPL_OK;
  auto up = [&](void* dst, const void* src, size_t b) {
    if (!rc && b && cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = GPL_ERR_CUDA;
  };
  up(D.net_start, m.net_start.data(), (m.n_nets + 1) * 4);
  up(D.pin_net, pin_net.data(), m.n_pins * 4);
  up(D.pin_mov, pin_mov.data(), m.n_pins * 4);
  up(D.pin_inst, m.pin_inst.data(), m.n_pins * 4);
  up(D.pin_off, pin_off.data(), m.n_pins * 8);
  up(D.pin_fix, pin_fix.data(), m.n_pins * 8);
  up(D.mov_pin_start, mps.data(), (nP + 1) * 4);
  up(D.mov_pins, mp.data(), mp.size() * 4);
  up(D.ctr, ctr.data(), nP * 8);
  if (!rc && cudaMemsetAsync(D.counters, 0, 16 * 4, s) != cudaSuccess) rc = GPL_ERR_CUDA;
  if (prm.verbose_level >= 2) {
    cudaStreamSynchronize(s);
    printf("[InitialPlace] host arrays %.2f ms, device scratch %.1f MB + uploads %.2f ms\n", t_host - t_start,
           z.bytes / 1e6, wall() - t_host);
  }
  if (rc) {
    set_error("initial place: upload failed");
    dev_free(D.mem, pool, s);
    D.mem = nullptr;
    return rc;
  }
  IpParams& P = R.P;
  P.max_fanout = prm.initial_place_max_fanout;
  P.min_diff = prm.initial_place_min_diff_length;
  P.weight_scale = prm.initial_place_net_weight_scale;
  P.max_iter = prm.initial_place_max_solver_iter;
  R.nP = nP;
  R.nb_mov = nb_mov;
  R.grid = grid;
  R.xr_grid = z.xr_grid;
  R.scan_blocks = scan_blocks;
  R.cluster = cluster;
  R.coop = coop;
  R.coop_attr = coop_attr;
  R.per_sm = per_sm;
  R.ctr.assign(ctr.data(), ctr.data() + nP);
  if (prm.verbose_level >= 2)
    printf("[InitialPlace] setup %.2f ms (host arrays, scratch, upload)\n", wall() - t_start);
  return GPL_OK;
}

// After the rounds: the solution's centres back to the host model (when a
// round ran), the scratch released, the statistics.
int ip_finish(IpRun& R, gpl_ip_stats* stats, int rc) {
  HostModel& m = *R.m;
  IpDev& D = R.D;
  const double t_end = wall_now();
  unsigned fill_overflow = 0;
  if (!rc && D.mem) {
    if (cudaMemcpyAsync(R.ctr.data(), D.ctr, R.nP * 8, cudaMemcpyDeviceToHost, R.s) != cudaSuccess ||
        cudaMemcpyAsync(&fill_overflow, D.counters + kFillOverflow, sizeof(unsigned), cudaMemcpyDeviceToHost, R.s) !=
            cudaSuccess ||
        host_wait(R.s, R.sync_ev) != cudaSuccess) rc = GPL_ERR_CUDA;
  }
  if (D.mem) dev_free(D.mem, R.pool, R.s);
  D.mem = nullptr;
  if (rc) { set_error("initial place: CUDA error"); return rc; }
  if (fill_overflow) { set_error("initial place: B2B entries exceeded their bound"); return GPL_ERR_CUDA; }
  if (R.rounds > 0)
    for (int k = 0; k < R.nP; k++) host_set_inst_center(m, m.place_insts[k], R.ctr[k].x, R.ctr[k].y);
  if (m.p.verbose_level >= 2) printf("[InitialPlace] read-back and release %.2f ms\n", wall_now() - t_end);
  if (stats) {
    stats->iterations = R.rounds;
    stats->last_error = R.err;
    stats->last_hpwl = 0;
    stats->solver_iters_x = R.iters[0];
    stats->solver_iters_y = R.iters[1];
    stats->cooperative_rounds = R.coop_rounds;
  }
  return GPL_OK;
}

// The round's end for one job: its solver states give the error
// (solver.error() = sqrt(|r|^2 / |b|^2)) and the stop test
// (src/initialPlace.cpp:93-99).
void ip_round_done(IpRun& R, int round, const BiState* st) {
  const float ex = st[0].rhs_sq > 0 ? (float)sqrt(st[0].rr / st[0].rhs_sq) : 0.0f;
  const float ey = st[1].rhs_sq > 0 ? (float)sqrt(st[1].rr / st[1].rhs_sq) : 0.0f;
  R.err = std::max(ex, ey);
  R.iters[0] = st[0].i;
  R.iters[1] = st[1].i;
  R.rounds = round;
  if ((R.err <= 1e-5 && round >= 5) || round >= R.m->p.initial_place_max_iter) R.finished = true;
}

int run_initial_place(HostModel& m, cudaStream_t s, int sm_count, gpl_ip_stats* stats, Timer& timer,
                      void* pinned, cudaMemPool_t pool, cudaEvent_t sync_ev) {
  IpRun R;
  int rc = ip_setup(m, s, sm_count, pinned, pool, sync_ev, R);
  if (rc) return rc;
  const gpl_params& prm = m.p;
  IpDev& D = R.D;
  const IpParams& P = R.P;
  const int nP = R.nP, nb_mov = R.nb_mov, grid = R.grid, scan_blocks = R.scan_blocks;
  bool cluster = R.cluster, coop = R.coop;
  const int coop_attr = R.coop_attr, per_sm = R.per_sm, mode = prm.ip_solver;
  BiState* st_h = R.st_h;
  const dim3 g2(nb_mov, 2), gs(grid, 2), gx(R.xr_grid, 2);
  const auto wall = wall_now;
  double t_round = wall();
  // The round's assembly (12 kernels) and a chunk of 8 solver iterations of
  // the phase form (32 kernels) have fixed arguments for the whole job, so
  // each is captured once as a CUDA graph and replayed (one launch instead
  // of tens: small jobs are bound by launches).  Without graphs (use_graph 0,
  // kernel timing, or a failed capture) the same kernels are launched one
  // by one.
  auto assembly = [&]() {
    k_ip_pos<<<blocks_for(m.n_pins), kB, 0, s>>>(D);
    k_ip_bound<<<blocks_for(m.n_nets), kB, 0, s>>>(D);
    k_ip_count<<<dim3(scan_blocks, 2), kB, 0, s>>>(D, P);
    k_scan_blocks<<<dim3(scan_blocks, 2), kB, 0, s>>>(D.cnt, D.slot_off, D.scan_part, D.n_mp);
    k_scan_parts<<<2, kScanT, 0, s>>>(D.scan_part, scan_blocks, D.slot_off, D.n_mp);
    k_scan_add<<<dim3(scan_blocks, 2), kB, 0, s>>>(D.slot_off, D.scan_part, D.n_mp);
    k_ip_rowptr<<<dim3(blocks_for(nP + 1), 2), kB, 0, s>>>(D);
    k_ip_fill<<<dim3(scan_blocks, 2), kB, 0, s>>>(D, P);
    k_ip_rowsum<<<g2, kB, 0, s>>>(D);
    k_ip_guess<<<nb_mov, kB, 0, s>>>(D);
    k_ip_window<<<gs, kB, 0, s>>>(D);
    k_bi_residual<<<gs, kB, spmv_bytes(), s>>>(D, 1, P.max_iter);
  };
  auto phase_chunk = [&]() {
    for (int k = 0; k < 8; k++) {
      k_bi_residual<<<gs, kB, spmv_bytes(), s>>>(D, 0, P.max_iter);
      k_bi_pv<<<gs, kB, spmv_bytes(), s>>>(D);
      k_bi_st<<<gs, kB, spmv_bytes(), s>>>(D);
      k_bi_xr<<<gx, kB, 0, s>>>(D, P.max_iter);
    }
  };
  auto capture = [&](auto&& body) -> cudaGraphExec_t {
    if (!prm.use_graph || timer.enabled) return nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    body();
    if (cudaStreamEndCapture(s, &g) != cudaSuccess || !g || cudaGraphInstantiate(&e, g, 0) != cudaSuccess) e = nullptr;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return e;
  };
  // The whole initial place as one graph with conditional nodes (device_loop
  // 1; the phase form with graphs, no kernel timing, no per-round
  // printing): one launch and one wait.  Under the placement server the
  // host-driven rounds interleave better with the other jobs' kernels (64
  // small jobs: 0.96 s against 1.28 s), so it is not the default.  Any
  // failure to build it leaves the host loop below.
  if (!cluster && !coop && prm.use_graph && prm.device_loop && !timer.enabled && prm.verbose_level < 2 &&
      prm.initial_place_max_iter > 0) {
    // the unique node without dependents of a graph captured from one stream
    auto tail_of = [](cudaGraph_t gr) -> cudaGraphNode_t {
      size_t n = 0;
      if (cudaGraphGetNodes(gr, nullptr, &n) != cudaSuccess || n == 0) return nullptr;
      std::vector<cudaGraphNode_t> nodes(n);
      if (cudaGraphGetNodes(gr, nodes.data(), &n) != cudaSuccess) return nullptr;
      cudaGraphNode_t t = nullptr;
      int tails = 0;
      for (cudaGraphNode_t nd : nodes) {
        size_t k = 0;
        if (cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &k) != cudaSuccess) return nullptr;
        if (k == 0) { t = nd; tails++; }
      }
      return tails == 1 ? t : nullptr;
    };
    auto into = [&](cudaGraph_t gr, const cudaGraphNode_t* dep, auto&& body) {
      cudaGraph_t cap = nullptr;
      if (cudaStreamBeginCaptureToGraph(s, gr, dep, nullptr, dep ? 1 : 0, cudaStreamCaptureModeThreadLocal) !=
          cudaSuccess)
        return false;
      body();
      return cudaStreamEndCapture(s, &cap) == cudaSuccess;
    };
    auto add_while = [](cudaGraph_t gr, cudaGraphNode_t dep, cudaGraphConditionalHandle h, cudaGraphNode_t* node,
                        cudaGraph_t* body) {
      cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
      wp.conditional.handle = h;
      wp.conditional.type = cudaGraphCondTypeWhile;
      wp.conditional.size = 1;
      if (cudaGraphAddNode(node, gr, &dep, nullptr, 1, &wp) != cudaSuccess) return false;
      *body = wp.conditional.phGraph_out[0];
      return true;
    };
    IpLoop* L_h = reinterpret_cast<IpLoop*>(reinterpret_cast<unsigned char*>(st_h) + kIpLoopPinned);
    cudaGraph_t g = nullptr, body_r = nullptr, body_c = nullptr;
    cudaGraphNode_t head = nullptr, wr = nullptr, wc = nullptr, a_tail = nullptr;
    cudaGraphConditionalHandle h_round = 0, h_chunk = 0;
    cudaGraphExec_t loop_exec = nullptr;
    const int iter_limit = 2 * P.max_iter + 2;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    ok = ok && cudaGraphConditionalHandleCreate(&h_round, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
    ok = ok && cudaGraphConditionalHandleCreate(&h_chunk, g, 0, cudaGraphCondAssignDefault) == cudaSuccess;
    ok = ok && into(g, nullptr, [&] {
      k_ip_loop_head<<<1, 1, 0, s>>>(D.loop, prm.initial_place_max_iter, iter_limit, h_round);
    });
    ok = ok && (head = tail_of(g)) != nullptr;
    ok = ok && add_while(g, head, h_round, &wr, &body_r);
    ok = ok && into(body_r, nullptr, [&] {
      assembly();
      k_ip_chunk_head<<<1, 1, 0, s>>>(D.loop, h_chunk);
    });
    ok = ok && (a_tail = tail_of(body_r)) != nullptr;
    ok = ok && add_while(body_r, a_tail, h_chunk, &wc, &body_c);
    ok = ok && into(body_c, nullptr, [&] {
      phase_chunk();
      k_ip_chunk_tail<<<1, 1, 0, s>>>(D.st, D.loop, h_chunk);
    });
    ok = ok && into(body_r, &wc, [&] {
      k_ip_move<<<nb_mov, kB, 0, s>>>(D);
      k_ip_round_tail<<<1, 1, 0, s>>>(D.st, D.loop, h_round);
    });
    ok = ok && into(g, &wr, [&] {
      cudaMemcpyAsync(L_h, D.loop, sizeof(IpLoop), cudaMemcpyDeviceToHost, s);
    });
    ok = ok && cudaGraphInstantiate(&loop_exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (ok) {
      if (cudaGraphLaunch(loop_exec, s) != cudaSuccess || host_wait(s, sync_ev) != cudaSuccess) {
        rc = GPL_ERR_CUDA;
      } else {
        R.rounds = L_h->round;
        R.err = L_h->err;
        R.iters[0] = L_h->iters_x;
        R.iters[1] = L_h->iters_y;
        R.finished = L_h->finished != 0;
      }
      cudaGraphExecDestroy(loop_exec);
      return ip_finish(R, stats, rc);
    }
    if (loop_exec) cudaGraphExecDestroy(loop_exec);
    if (prm.verbose_level > 0) printf("[InitialPlace] device loop not built: the host drives the rounds\n");
  }
  cudaGraphExec_t assembly_exec = capture(assembly);
  cudaGraphExec_t chunk_exec = (!cluster && !coop) ? capture(phase_chunk) : nullptr;
  for (int round = 1; round <= prm.initial_place_max_iter && !rc; round++) {
    timer.begin(kKOther);
    if (assembly_exec) {
      if (cudaGraphLaunch(assembly_exec, s) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
    } else {
      assembly();
    }
    timer.end(kKOther);
    timer.count(12);
    bool solved = false;
    if (cluster) {
      // the whole solve of each axis in one cluster
      timer.begin(kKOther);
      k_bi_cluster<<<dim3(kClCtas, 2), kClThreads, stage_bytes(kClThreads), s>>>(D, P.max_iter);
      timer.end(kKOther);
      timer.count(1);
      const cudaError_t ce = cudaGetLastError();
      if (ce == cudaSuccess) {
        solved = true;
        R.coop_rounds++;
      } else {
        // not launched (no room for the cluster): the grid forms below
        if (prm.verbose_level > 0)
          printf("[InitialPlace] cluster solve not launched (%s)\n", cudaGetErrorString(ce));
        cluster = false;
        coop = coop_attr != 0 && per_sm > 0 && mode != 1;
      }
    }
    if (!solved && coop) {
      // the whole solve in one cooperative launch
      int max_iter = P.max_iter;
      void* args[] = {(void*)&D, (void*)&max_iter};
      cudaError_t ce = cudaMemsetAsync(D.bar, 0, sizeof(GridBar), s);
      timer.begin(kKOther);
      if (ce == cudaSuccess)
        ce = cudaLaunchCooperativeKernel((const void*)k_bi_coop, dim3(grid, 2), dim3(kB), args, stage_bytes(kB), s);
      timer.end(kKOther);
      timer.count(1);
      if (ce != cudaSuccess) {
        cudaGetLastError();            // not launched: the kernel-per-phase loop below
        if (prm.verbose_level > 0)
          printf("[InitialPlace] cooperative solve not launched (%s): one kernel per phase\n",
                 cudaGetErrorString(ce));
        coop = false;
      } else {
        GridBar* bar_h = reinterpret_cast<GridBar*>(st_h + 2);
        if (cudaMemcpyAsync(bar_h, D.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            host_wait(s, sync_ev) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
        if (bar_h->err == 0) {
          solved = true;
          R.coop_rounds++;
        } else {
          // a barrier wait ran out: solve this round again phase by phase
          coop = false;
          k_ip_guess<<<nb_mov, kB, 0, s>>>(D);
          k_bi_residual<<<gs, kB, spmv_bytes(), s>>>(D, 1, P.max_iter);
          timer.count(2);
        }
      }
    }
    // BiCGSTAB phase by phase: chunks of iterations, then poll the done flags
    for (int it = 0; !solved && it <= 2 * P.max_iter + 2; it += 8) {
      timer.begin(kKOther);
      if (chunk_exec) {
        if (cudaGraphLaunch(chunk_exec, s) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      } else {
        phase_chunk();
      }
      timer.end(kKOther);
      timer.count(32);
      if (cudaGetLastError() != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      if (cudaMemcpyAsync(st_h, D.st, 2 * sizeof(BiState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          host_wait(s, sync_ev) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      if (st_h[0].done && st_h[1].done) break;
    }
    if (rc) break;
    k_ip_move<<<nb_mov, kB, 0, s>>>(D);
    timer.count(1);
    if (cudaMemcpyAsync(st_h, D.st, 2 * sizeof(BiState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        host_wait(s, sync_ev) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
    ip_round_done(R, round, st_h);
    if (prm.verbose_level >= 2) {
      const double t = wall();
      printf("[InitialPlace] Iter: %d error: %g solver iterations: %d %d (%.2f ms)\n", round, R.err, R.iters[0],
             R.iters[1], t - t_round);
      t_round = t;
    }
    if (R.finished) break;
  }
  if (assembly_exec) cudaGraphExecDestroy(assembly_exec);
  if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
  (void)nP;
  return ip_finish(R, stats, rc);
}

// ------------------------------------------------------------ batched form
// The rounds of many jobs in lockstep: every round, each member's assembly
// phases run as one launch per phase over the work table, then chunks of
// eight solver iterations (four launches each) until every member's two
// solves are done (a member that finished early skips the later chunks'
// blocks: every phase body returns at once on a finished solve, as it does
// in the job's own chunks), then the move; then each member's error and stop
// test as run_initial_place takes them.  A member leaves when its rounds
// end.  Each membership's assembly and chunk are captured as CUDA graphs.
namespace {

enum IpTable { kTPos = 0, kTBound, kTScan, kTParts, kTRowptr, kTRowsum, kTMov, kTSolve, kTVec, kTTables };

// the work items of one member in each table
void ip_items(const IpRun& R, int k, std::vector<int4> (&t)[kTTables]) {
  const HostModel& m = *R.m;
  for (int b = 0; b < blocks_for(m.n_pins); b++) t[kTPos].push_back(make_int4(k, b, 0, 0));
  for (int b = 0; b < blocks_for(m.n_nets); b++) t[kTBound].push_back(make_int4(k, b, 0, 0));
  for (int a = 0; a < 2; a++) {
    for (int b = 0; b < R.scan_blocks; b++) t[kTScan].push_back(make_int4(k, b, R.scan_blocks, a));
    t[kTParts].push_back(make_int4(k, 0, R.scan_blocks, a));
    for (int b = 0; b < blocks_for(R.nP + 1); b++) t[kTRowptr].push_back(make_int4(k, b, 0, a));
    for (int b = 0; b < R.nb_mov; b++) t[kTRowsum].push_back(make_int4(k, b, R.nb_mov, a));
    for (int b = 0; b < R.grid; b++) t[kTSolve].push_back(make_int4(k, b, R.grid, a));
    for (int b = 0; b < R.xr_grid; b++) t[kTVec].push_back(make_int4(k, b, R.xr_grid, a));
  }
  for (int b = 0; b < R.nb_mov; b++) t[kTMov].push_back(make_int4(k, b, 0, 0));
}

size_t ip_item_count(const IpRun& R) {
  const HostModel& m = *R.m;
  return (size_t)blocks_for(m.n_pins) + blocks_for(m.n_nets) +
         2 * ((size_t)R.scan_blocks + 1 + blocks_for(R.nP + 1) + R.nb_mov + R.grid + R.xr_grid) + R.nb_mov;
}

using IpBatchKernel = void (*)(const IpDev*, const IpParams*, const int4*);

}  // namespace

int run_initial_place_batch(IpBatchJob* jobs, int n, int sm_count, int64_t* launches) {
  std::vector<IpRun> R(n);
  std::vector<char> active(n, 0);
  size_t max_items = 0;
  bool verbose = false;
  for (int k = 0; k < n; k++) verbose |= jobs[k].m->p.verbose_level >= 2;
  const double t_start = wall_now();
  for (int k = 0; k < n; k++) {
    IpBatchJob& J = jobs[k];
    J.status = GPL_OK;
    if (J.m->p.initial_place_max_iter <= 0) continue;
    J.status = ip_setup(*J.m, J.s, sm_count, J.pinned, J.pool, J.sync_ev, R[k]);
    if (!J.status && host_wait(J.s, J.sync_ev) != cudaSuccess) J.status = ip_finish(R[k], nullptr, GPL_ERR_CUDA);
    if (J.status) continue;
    active[k] = 1;
    max_items += ip_item_count(R[k]);
  }
  int rc = GPL_OK;
  cudaStream_t bs = nullptr;
  char* dmem = nullptr;
  char* hmem = nullptr;
  cudaGraphExec_t assembly_exec = nullptr, chunk_exec = nullptr;
  long long nl = 0;
  std::vector<int> mem;
  for (int k = 0; k < n; k++)
    if (active[k]) mem.push_back(k);
  if (!mem.empty()) {
    // device: the members' tables and parameters, the work items, the
    // member list and the gathered solver states; pinned: items, list, states
    const size_t b_ds = (size_t)n * sizeof(IpDev), b_ps = (size_t)n * sizeof(IpParams);
    const size_t b_items = max_items * sizeof(int4), b_list = (size_t)n * sizeof(int),
                 b_st = 2 * (size_t)n * sizeof(BiState);
    auto rnd = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_ps = rnd(b_ds), o_items = o_ps + rnd(b_ps), o_list = o_items + rnd(b_items),
                 o_st = o_list + rnd(b_list), total = o_st + rnd(b_st);
    const size_t h_list = rnd(b_items), h_st = h_list + rnd(b_list), h_total = h_st + rnd(b_st);
    std::vector<IpDev> ds(n);
    std::vector<IpParams> ps(n);
    int maxit = 0;
    for (int k : mem) {
      ds[k] = R[k].D;
      ps[k] = R[k].P;
      maxit = std::max(maxit, R[k].P.max_iter);
    }
    if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc((void**)&dmem, total) != cudaSuccess || cudaMallocHost((void**)&hmem, h_total) != cudaSuccess ||
        cudaMemcpyAsync(dmem, ds.data(), b_ds, cudaMemcpyHostToDevice, bs) != cudaSuccess ||
        cudaMemcpyAsync(dmem + o_ps, ps.data(), b_ps, cudaMemcpyHostToDevice, bs) != cudaSuccess ||
        cudaStreamSynchronize(bs) != cudaSuccess) {
      cudaGetLastError();
      set_error("batched initial place: setup failed");
      rc = GPL_ERR_CUDA;
    }
    const IpDev* d_ds = reinterpret_cast<const IpDev*>(dmem);
    const IpParams* d_ps = reinterpret_cast<const IpParams*>(dmem + o_ps);
    const int4* d_items = reinterpret_cast<const int4*>(dmem + o_items);
    const int* d_list = reinterpret_cast<const int*>(dmem + o_list);
    BiState* d_st = reinterpret_cast<BiState*>(dmem + o_st);
    int4* h_items = reinterpret_cast<int4*>(hmem);
    int* h_lst = reinterpret_cast<int*>(hmem + h_list);
    const BiState* h_states = reinterpret_cast<const BiState*>(hmem + h_st);
    int off[kTTables] = {}, cnt[kTTables] = {};
    int n_mem = 0;
    auto L = [&](IpBatchKernel kern, int table, size_t smem) {
      if (!cnt[table]) return;
      kern<<<cnt[table], kB, smem, bs>>>(d_ds, d_ps, d_items + off[table]);
      nl++;
    };
    auto gather = [&]() {
      k_ipb_states<<<(2 * n_mem + 127) / 128, 128, 0, bs>>>(d_ds, d_list, n_mem, d_st);
      nl++;
      cudaMemcpyAsync(hmem + h_st, d_st, 2 * (size_t)n_mem * sizeof(BiState), cudaMemcpyDeviceToHost, bs);
    };
    auto assembly = [&]() {
      L(k_ipb<kIpPos>, kTPos, 0);
      L(k_ipb<kIpBound>, kTBound, 0);
      L(k_ipb<kIpCount>, kTScan, 0);
      L(k_ipb<kIpScanBlocks>, kTScan, 0);
      if (cnt[kTParts]) {
        k_ipb_scan_parts<<<cnt[kTParts], kScanT, 0, bs>>>(d_ds, d_items + off[kTParts]);
        nl++;
      }
      L(k_ipb<kIpScanAdd>, kTScan, 0);
      L(k_ipb<kIpRowptr>, kTRowptr, 0);
      L(k_ipb<kIpFill>, kTScan, 0);
      L(k_ipb<kIpRowsum>, kTRowsum, 0);
      L(k_ipb<kIpGuess>, kTMov, 0);
      L(k_ipb<kIpWindow>, kTSolve, 0);
      L(k_ipb<kIpResidualInit>, kTSolve, spmv_bytes());
    };
    auto chunk = [&]() {
      for (int k = 0; k < 8; k++) {
        L(k_ipb<kIpResidual>, kTSolve, spmv_bytes());
        L(k_ipb<kIpPV>, kTSolve, spmv_bytes());
        L(k_ipb<kIpST>, kTSolve, spmv_bytes());
        L(k_ipb<kIpXr>, kTVec, 0);
      }
      gather();
    };
    // a captured body launches its kernels once per replay: count them
    // when replayed, not when captured
    auto capture = [&](auto&& body, long long& per_replay) -> cudaGraphExec_t {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t e = nullptr;
      const long long before = nl;
      if (cudaStreamBeginCapture(bs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      body();
      if (cudaStreamEndCapture(bs, &g) != cudaSuccess || !g || cudaGraphInstantiate(&e, g, 0) != cudaSuccess)
        e = nullptr;
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      per_replay = nl - before;
      nl = before;
      return e;
    };
    auto replay = [&](cudaGraphExec_t e, auto&& body, long long per_replay) {
      if (e) {
        if (cudaGraphLaunch(e, bs) != cudaSuccess) return false;
        nl += per_replay;
      } else {
        body();
      }
      return cudaGetLastError() == cudaSuccess;
    };
    long long n_assembly = 0, n_chunk = 0;
    bool layout_changed = true;
    if (verbose) printf("[InitialPlace] batched: %d jobs set up in %.2f ms\n", (int)mem.size(), wall_now() - t_start);
    for (int round = 1; !rc && !mem.empty(); round++) {
      const double t_round = wall_now();
      int chunks = 0;
      if (layout_changed) {
        // the members' work items and list (pinned), then up to the device
        std::vector<int4> t[kTTables];
        for (int q = 0; q < (int)mem.size(); q++) ip_items(R[mem[q]], mem[q], t);
        int at = 0;
        for (int tb = 0; tb < kTTables; tb++) {
          off[tb] = at;
          cnt[tb] = (int)t[tb].size();
          std::copy(t[tb].begin(), t[tb].end(), h_items + at);
          at += cnt[tb];
        }
        n_mem = (int)mem.size();
        std::copy(mem.begin(), mem.end(), h_lst);
        if (cudaMemcpyAsync(dmem + o_items, h_items, (size_t)at * sizeof(int4), cudaMemcpyHostToDevice, bs) !=
                cudaSuccess ||
            cudaMemcpyAsync(dmem + o_list, h_lst, (size_t)n_mem * sizeof(int), cudaMemcpyHostToDevice, bs) !=
                cudaSuccess) { rc = GPL_ERR_CUDA; break; }
        if (assembly_exec) cudaGraphExecDestroy(assembly_exec);
        if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
        assembly_exec = capture(assembly, n_assembly);
        chunk_exec = capture(chunk, n_chunk);
        layout_changed = false;
      }
      if (!replay(assembly_exec, assembly, n_assembly)) { rc = GPL_ERR_CUDA; break; }
      for (int it = 0; it <= 2 * maxit + 2; it += 8) {
        if (!replay(chunk_exec, chunk, n_chunk) || cudaStreamSynchronize(bs) != cudaSuccess) {
          rc = GPL_ERR_CUDA;
          break;
        }
        chunks++;
        bool all = true;
        for (int q = 0; q < n_mem && all; q++) all = h_states[2 * q].done && h_states[2 * q + 1].done;
        if (all) break;
      }
      if (rc) break;
      L(k_ipb<kIpMove>, kTMov, 0);
      gather();
      if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(bs) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      std::vector<int> next;
      for (int q = 0; q < n_mem; q++) {
        IpRun& r = R[mem[q]];
        ip_round_done(r, round, h_states + 2 * q);
        if (r.m->p.verbose_level >= 2)
          printf("[InitialPlace] Iter: %d error: %g solver iterations: %d %d (batched, %d jobs)\n", round, r.err,
                 r.iters[0], r.iters[1], n_mem);
        if (!r.finished) next.push_back(mem[q]);
      }
      if (verbose)
        printf("[InitialPlace] batched round %d: %d jobs, %d chunks of 8 solver iterations, %.2f ms\n", round, n_mem,
               chunks, wall_now() - t_round);
      layout_changed = next.size() != mem.size();
      mem.swap(next);
    }
    if (rc) {
      cudaGetLastError();
      set_error("batched initial place: CUDA error");
    }
  }
  if (assembly_exec) cudaGraphExecDestroy(assembly_exec);
  if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
  if (bs) cudaStreamSynchronize(bs);
  if (dmem) cudaFree(dmem);
  if (hmem) cudaFreeHost(hmem);
  if (bs) cudaStreamDestroy(bs);
  const double t_end = wall_now();
  for (int k = 0; k < n; k++)
    if (active[k]) jobs[k].status = ip_finish(R[k], jobs[k].stats, rc);
  if (verbose) printf("[InitialPlace] batched: read-back of %d jobs %.2f ms\n", n, wall_now() - t_end);
  if (launches) *launches = nl;
  // a failure of the batch itself (its tables, stream or kernels) is also
  // the call's status; every job's own status says what happened to it
  return rc;
}

}  // namespace gpl
