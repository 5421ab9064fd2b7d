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
// last block of each reduction kernel, so the host only polls a done flag.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
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
  int pad[3];
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
  int32_t* cnt;            // [2][n_mov] row lengths (off-diagonal entries)
  int32_t* rowptr;         // [2][n_mov + 1]
  int32_t* scan_part;      // block sums of the scan
  int32_t* col;            // [2][nnz_cap]
  float* val;
  float* diag;             // [2][n_mov]
  float* b;                // [2][n_mov]
  float *x, *r, *r0, *p, *v, *s, *t;   // [2][n_mov]
  double* part;            // [2][slots][parts]
  unsigned* counters;      // [2][8]
  BiState* st;             // [2]
  BiState* st_h;           // pinned mirror
  int parts = 0;
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
__global__ void k_ip_pos(IpDev D) {
  const int q = blockIdx.x * kB + threadIdx.x;
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
__global__ void k_ip_bound(IpDev D) {
  const int n = blockIdx.x * kB + threadIdx.x;
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

__global__ void k_ip_count(IpDev D, IpParams P) {
  const int i = blockIdx.x * kB + threadIdx.x;
  const int axis = blockIdx.y;
  if (i >= D.n_mov) return;
  int c = 0;
  for (int t = D.mov_pin_start[i]; t < D.mov_pin_start[i + 1]; t++) {
    const int q = D.mov_pins[t];
    const int n = D.pin_net[q];
    int deg;
    if (!net_used(D, P, n, deg)) continue;
    for_partners(D, q, n, axis, [&](int r) { if (D.pin_mov[r] >= 0) c++; });
  }
  D.cnt[axis * D.n_mov + i] = c;
}

// exclusive scan of cnt[axis] into rowptr[axis] (three kernels)
__global__ void k_scan_blocks(const int32_t* in, int32_t* out, int32_t* part, int n) {
  __shared__ int32_t sh[kB];
  const int axis = blockIdx.y;
  const int i = blockIdx.x * kB + threadIdx.x;
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
  if (threadIdx.x == kB - 1) part[axis * gridDim.x + blockIdx.x] = sh[kB - 1];
}

__global__ void k_scan_parts(int32_t* part, int nparts, int32_t* rowptr, int n) {
  const int axis = blockIdx.x;
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < nparts; k++) {
      const int v = part[axis * nparts + k];
      part[axis * nparts + k] = run;
      run += v;
    }
    rowptr[axis * (n + 1) + n] = run;
  }
}

__global__ void k_scan_add(int32_t* rowptr, const int32_t* part, int n) {
  const int axis = blockIdx.y;
  const int i = blockIdx.x * kB + threadIdx.x;
  if (i < n) rowptr[axis * (n + 1) + i] += part[axis * gridDim.x + blockIdx.x];
}

// createSparseMatrix, one row per thread (src/initialPlace.cpp:221-374)
__global__ void k_ip_fill(IpDev D, IpParams P) {
  const int i = blockIdx.x * kB + threadIdx.x;
  const int axis = blockIdx.y;
  if (i >= D.n_mov) return;
  const int2 ci = D.ctr[i];
  int w_at = D.rowptr[axis * (D.n_mov + 1) + i];
  int32_t* col = D.col + axis * D.nnz_cap;
  float* val = D.val + axis * D.nnz_cap;
  float diag = 0.0f, rhs = 0.0f;
  for (int t = D.mov_pin_start[i]; t < D.mov_pin_start[i + 1]; t++) {
    const int q = D.mov_pins[t];
    const int n = D.pin_net[q];
    int deg;
    if (!net_used(D, P, n, deg)) continue;
    const float net_w = P.weight_scale / (deg - 1);
    const int pq = axis ? D.pos[q].y : D.pos[q].x;
    const int off_q = pq - (axis ? ci.y : ci.x);
    for_partners(D, q, n, axis, [&](int r) {
      const int pr = axis ? D.pos[r].y : D.pos[r].x;
      const float w = pair_weight(P, net_w, pq, pr);
      diag += w;
      const int j = D.pin_mov[r];
      if (j >= 0) {
        col[w_at] = j;
        val[w_at] = -w;
        w_at++;
        const int2 cj = D.ctr[j];
        const int off_r = pr - (axis ? cj.y : cj.x);
        rhs += -w * (float)(off_q - off_r);
      } else {
        rhs += w * (float)(pr - off_q);
      }
    });
  }
  D.diag[axis * D.n_mov + i] = diag;
  D.b[axis * D.n_mov + i] = rhs;
}

// ------------------------------------------------------------ solver
__device__ __forceinline__ float spmv_row(const IpDev& D, int axis, int i, const float* xv) {
  const int s = D.rowptr[axis * (D.n_mov + 1) + i], e = D.rowptr[axis * (D.n_mov + 1) + i + 1];
  const int32_t* col = D.col + axis * D.nnz_cap;
  const float* val = D.val + axis * D.nnz_cap;
  float acc = D.diag[axis * D.n_mov + i] * xv[i];
  for (int k = s; k < e; k++) acc += val[k] * xv[col[k]];
  return acc;
}

// block partial sums of up to 2 products, then the last block of this axis
// runs `fin` with the totals (fixed-order reduction)
template <int N, class Fin>
__device__ __forceinline__ void reduce_and_finish(IpDev& D, int kernel_id, double (&v)[N], Fin fin) {
  __shared__ double sh[32 * N];
  __shared__ bool last;
  const int axis = blockIdx.y;
  double* part = D.part + (size_t)(axis * 2) * D.parts;
  block_reduce_n<N>(v, part, D.parts, sh);
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&D.counters[axis * 8 + kernel_id], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  double tot[N];
#pragma unroll
  for (int k = 0; k < N; k++) tot[k] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
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
__global__ void k_bi_residual(IpDev D, int init, int max_iter) {
  const int axis = blockIdx.y;
  BiState& S = D.st[axis];
  if (!init && (S.done || !S.need_restart)) return;
  const int n = D.n_mov;
  const float* bb = D.b + axis * n;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  float* r0 = D.r0 + axis * n;
  double v[2] = {0.0, 0.0};
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB) {
    const float ri = bb[i] - spmv_row(D, axis, i, x);
    r[i] = ri;
    r0[i] = ri;
    v[0] += (double)ri * ri;
    v[1] += (double)bb[i] * bb[i];
  }
  reduce_and_finish<2>(D, 0, v, [&](BiState& s, const double* t) {
    if (init) {
      s.r0sq = t[0];
      s.rr = t[0];
      s.rhs_sq = t[1];
      s.rho = s.alpha = s.w = 1.0;
      s.dot_r0r = t[0];
      s.tol2 = 1.1920928955078125e-07 * 1.1920928955078125e-07 * t[1];
      s.i = 0; s.restarts = 0; s.done = 0; s.need_restart = 0; s.zero_x = 0;
      if (t[1] == 0.0) { s.zero_x = 1; s.done = 1; s.rr = 0.0; }
      else loop_head(s, max_iter);
    } else {
      s.rho = s.r0sq = s.rr = t[0];
      if (s.restarts++ == 0) s.i = 0;
      s.need_restart = 0;
    }
  });
}

__global__ void k_bi_p(IpDev D) {
  const int axis = blockIdx.y;
  const BiState& S = D.st[axis];
  if (S.done) return;
  const double beta = (S.rho / S.rho_old) * (S.alpha / S.w);
  const int n = D.n_mov;
  float* p = D.p + axis * n;
  const float* r = D.r + axis * n;
  const float* v = D.v + axis * n;
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB)
    p[i] = (float)(r[i] + beta * (p[i] - S.w * v[i]));
}

// v = A p, alpha = rho / (r0 . v)
__global__ void k_bi_v(IpDev D) {
  const int axis = blockIdx.y;
  if (D.st[axis].done) return;
  const int n = D.n_mov;
  const float* p = D.p + axis * n;
  float* v = D.v + axis * n;
  const float* r0 = D.r0 + axis * n;
  double acc[1] = {0.0};
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB) {
    const float vi = spmv_row(D, axis, i, p);
    v[i] = vi;
    acc[0] += (double)r0[i] * vi;
  }
  reduce_and_finish<1>(D, 1, acc, [&](BiState& s, const double* t) { s.alpha = s.rho / t[0]; });
}

__global__ void k_bi_s(IpDev D) {
  const int axis = blockIdx.y;
  const BiState& S = D.st[axis];
  if (S.done) return;
  const int n = D.n_mov;
  const float* r = D.r + axis * n;
  const float* v = D.v + axis * n;
  float* s = D.s + axis * n;
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB)
    s[i] = (float)(r[i] - S.alpha * v[i]);
}

// t = A s, omega = (t . s) / (t . t)
__global__ void k_bi_t(IpDev D) {
  const int axis = blockIdx.y;
  if (D.st[axis].done) return;
  const int n = D.n_mov;
  const float* s = D.s + axis * n;
  float* t = D.t + axis * n;
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB) {
    const float ti = spmv_row(D, axis, i, s);
    t[i] = ti;
    acc[0] += (double)ti * ti;
    acc[1] += (double)ti * s[i];
  }
  reduce_and_finish<2>(D, 2, acc, [&](BiState& st, const double* tt) {
    st.w = tt[0] > 0.0 ? tt[1] / tt[0] : 0.0;
  });
}

// x += alpha p + omega s; r = s - omega t; |r|^2 and r0 . r; next loop head
__global__ void k_bi_xr(IpDev D, int max_iter) {
  const int axis = blockIdx.y;
  const BiState& S = D.st[axis];
  if (S.done) return;
  const int n = D.n_mov;
  float* x = D.x + axis * n;
  float* r = D.r + axis * n;
  const float* p = D.p + axis * n;
  const float* s = D.s + axis * n;
  const float* t = D.t + axis * n;
  const float* r0 = D.r0 + axis * n;
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * kB + threadIdx.x; i < n; i += gridDim.x * kB) {
    x[i] = (float)(x[i] + S.alpha * p[i] + S.w * s[i]);
    const float ri = (float)(s[i] - S.w * t[i]);
    r[i] = ri;
    acc[0] += (double)ri * ri;
    acc[1] += (double)r0[i] * ri;
  }
  reduce_and_finish<2>(D, 3, acc, [&](BiState& st, const double* tt) {
    st.rr = tt[0];
    st.dot_r0r = tt[1];
    st.i++;
    loop_head(st, max_iter);
  });
}

// rhs == 0: Eigen sets x = 0; then the instances move to the solution
// (InitialPlace::updateCoordi :380-385, float -> int truncation)
__global__ void k_ip_move(IpDev D) {
  const int i = blockIdx.x * kB + threadIdx.x;
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
__global__ void k_ip_guess(IpDev D) {
  const int i = blockIdx.x * kB + threadIdx.x;
  if (i >= D.n_mov) return;
  const int2 c = D.ctr[i];
  const int n = D.n_mov;
  D.x[i] = (float)c.x;
  D.x[n + i] = (float)c.y;
  D.p[i] = D.p[n + i] = 0.0f;
  D.v[i] = D.v[n + i] = 0.0f;
}

int blocks_for(int n) { return std::max(1, (n + kB - 1) / kB); }

}  // namespace

// Runs the initial place on the device; on return the host model's
// instances (and pins) are at the solution.  stats may be null.
struct IpSizes {
  size_t nnz_cap = 1, bytes = 0;
  int grid = 1;
};

// Scratch layout of run_initial_place (the sizes its carving below takes).
IpSizes ip_sizes(const HostModel& m, int sm_count) {
  IpSizes z;
  const size_t nP = m.place_insts.size();
  size_t n_mp = 0;
  for (int i : m.place_insts) n_mp += m.inst_pin_start[i + 1] - m.inst_pin_start[i];
  // an upper bound of the off-diagonal entries: every movable pin of a used
  // net partners every other pin of that net
  size_t nnz = 0;
  for (int n = 0; n < m.n_nets; n++) {
    const size_t deg = m.net_start[n + 1] - m.net_start[n];
    if (deg > 1 && (int)deg < m.p.initial_place_max_fanout) nnz += deg * (deg - 1);
  }
  z.nnz_cap = std::max<size_t>(nnz, 1);
  const int nb_mov = blocks_for((int)nP);
  z.grid = std::max(1, std::min(nb_mov, sm_count * 8));
  const size_t scan_blocks = nb_mov;
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += (b + 255) / 256 * 256 + 256; };
  add((m.n_nets + 1) * 4); add(m.n_pins * 4); add(m.n_pins * 4); add(m.n_pins * 4);
  add(m.n_pins * 8); add(m.n_pins * 8); add((nP + 1) * 4); add(n_mp * 4);
  add(nP * 8); add(m.n_pins * 8); add(m.n_nets * 16); add(2 * nP * 4); add(2 * (nP + 1) * 4);
  add(2 * scan_blocks * 4); add(2 * z.nnz_cap * 4); add(2 * z.nnz_cap * 4);
  for (int k = 0; k < 9; k++) add(2 * nP * 4);
  add(2 * 2 * (size_t)z.grid * 8); add(16 * 4); add(2 * sizeof(BiState));
  z.bytes = bytes;
  return z;
}

size_t initial_place_bytes(const HostModel& m, int sm_count) { return ip_sizes(m, sm_count).bytes; }

int run_initial_place(HostModel& m, cudaStream_t s, int sm_count, gpl_ip_stats* stats, Timer& timer,
                      void* pinned, cudaMemPool_t pool) {
  static_assert(2 * sizeof(BiState) <= sizeof(HostPinned::ip_state), "pinned solver state too small");
  const gpl_params& prm = m.p;
  IpDev D;
  D.n_mov = (int)m.place_insts.size();
  D.n_pins = m.n_pins;
  D.n_nets = m.n_nets;
  const int nP = D.n_mov;
  std::vector<int32_t> ext(m.n_insts, -1);
  for (int k = 0; k < nP; k++) ext[m.place_insts[k]] = k;
  std::vector<int32_t> pin_net(m.n_pins), pin_mov(m.n_pins);
  std::vector<int2> pin_off(m.n_pins), pin_fix(m.n_pins);
  for (int n = 0; n < m.n_nets; n++)
    for (int q = m.net_start[n]; q < m.net_start[n + 1]; q++) pin_net[q] = n;
  for (int q = 0; q < m.n_pins; q++) {
    const int i = m.pin_inst[q];
    pin_mov[q] = i >= 0 ? ext[i] : -1;
    pin_off[q] = make_int2(m.pin_ox[q], m.pin_oy[q]);
    pin_fix[q] = make_int2(m.pin_x[q], m.pin_y[q]);
  }
  std::vector<int32_t> mps(nP + 1, 0), mp;
  for (int k = 0; k < nP; k++) {
    const int i = m.place_insts[k];
    for (int t = m.inst_pin_start[i]; t < m.inst_pin_start[i + 1]; t++) mp.push_back(m.inst_pins[t]);
    mps[k + 1] = (int)mp.size();
  }
  std::vector<int2> ctr(nP);
  for (int k = 0; k < nP; k++) {
    const int i = m.place_insts[k];
    ctr[k] = make_int2((m.ilx[i] + m.iux[i]) / 2, (m.ily[i] + m.iuy[i]) / 2);
  }
  const IpSizes z = ip_sizes(m, sm_count);
  D.nnz_cap = z.nnz_cap;
  const int nb_mov = blocks_for(nP);
  const int grid = z.grid;
  D.parts = grid;
  const int scan_blocks = nb_mov;
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
  D.cnt = (int32_t*)take(2 * nP * 4);
  D.rowptr = (int32_t*)take(2 * (nP + 1) * 4);
  D.scan_part = (int32_t*)take(2 * scan_blocks * 4);
  D.col = (int32_t*)take(2 * D.nnz_cap * 4);
  D.val = (float*)take(2 * D.nnz_cap * 4);
  D.diag = (float*)take(2 * nP * 4);
  D.b = (float*)take(2 * nP * 4);
  D.x = (float*)take(2 * nP * 4);
  D.r = (float*)take(2 * nP * 4);
  D.r0 = (float*)take(2 * nP * 4);
  D.p = (float*)take(2 * nP * 4);
  D.v = (float*)take(2 * nP * 4);
  D.s = (float*)take(2 * nP * 4);
  D.t = (float*)take(2 * nP * 4);
  D.part = (double*)take(2 * 2 * (size_t)D.parts * 8);
  D.counters = (unsigned*)take(16 * 4);
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
  BiState* st_h = static_cast<BiState*>(pinned);
  if (rc) {
    set_error("initial place: upload failed");
    dev_free(D.mem, pool, s);
    return rc;
  }
  IpParams P;
  P.max_fanout = prm.initial_place_max_fanout;
  P.min_diff = prm.initial_place_min_diff_length;
  P.weight_scale = prm.initial_place_net_weight_scale;
  P.max_iter = prm.initial_place_max_solver_iter;
  const dim3 g2(nb_mov, 2), gs(grid, 2);
  float err = 0.0f;
  int rounds = 0, iters[2] = {0, 0};
  for (int round = 1; round <= prm.initial_place_max_iter && !rc; round++) {
    timer.begin(kKOther);
    k_ip_pos<<<blocks_for(m.n_pins), kB, 0, s>>>(D);
    k_ip_bound<<<blocks_for(m.n_nets), kB, 0, s>>>(D);
    k_ip_count<<<g2, kB, 0, s>>>(D, P);
    k_scan_blocks<<<dim3(scan_blocks, 2), kB, 0, s>>>(D.cnt, D.rowptr, D.scan_part, nP);
    k_scan_parts<<<2, 32, 0, s>>>(D.scan_part, scan_blocks, D.rowptr, nP);
    k_scan_add<<<dim3(scan_blocks, 2), kB, 0, s>>>(D.rowptr, D.scan_part, nP);
    k_ip_fill<<<g2, kB, 0, s>>>(D, P);
    k_ip_guess<<<nb_mov, kB, 0, s>>>(D);
    k_bi_residual<<<gs, kB, 0, s>>>(D, 1, P.max_iter);
    timer.end(kKOther);
    timer.count(9);
    // BiCGSTAB: chunks of iterations, then poll the done flags
    for (int it = 0; it <= 2 * P.max_iter + 2; it += 8) {
      timer.begin(kKOther);
      for (int k = 0; k < 8; k++) {
        k_bi_residual<<<gs, kB, 0, s>>>(D, 0, P.max_iter);
        k_bi_p<<<gs, kB, 0, s>>>(D);
        k_bi_v<<<gs, kB, 0, s>>>(D);
        k_bi_s<<<gs, kB, 0, s>>>(D);
        k_bi_t<<<gs, kB, 0, s>>>(D);
        k_bi_xr<<<gs, kB, 0, s>>>(D, P.max_iter);
      }
      timer.end(kKOther);
      timer.count(48);
      if (cudaGetLastError() != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      if (cudaMemcpyAsync(st_h, D.st, 2 * sizeof(BiState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
      if (st_h[0].done && st_h[1].done) break;
    }
    if (rc) break;
    k_ip_move<<<nb_mov, kB, 0, s>>>(D);
    timer.count(1);
    if (cudaMemcpyAsync(st_h, D.st, 2 * sizeof(BiState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = GPL_ERR_CUDA; break; }
    // solver.error() = sqrt(|r|^2 / |b|^2)
    float ex = st_h[0].rhs_sq > 0 ? (float)sqrt(st_h[0].rr / st_h[0].rhs_sq) : 0.0f;
    float ey = st_h[1].rhs_sq > 0 ? (float)sqrt(st_h[1].rr / st_h[1].rhs_sq) : 0.0f;
    err = std::max(ex, ey);
    iters[0] = st_h[0].i; iters[1] = st_h[1].i;
    rounds = round;
    if (err <= 1e-5 && round >= 5) break;
  }
  if (!rc) {
    if (cudaMemcpyAsync(ctr.data(), D.ctr, nP * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) rc = GPL_ERR_CUDA;
  }
  dev_free(D.mem, pool, s);
  if (rc) { set_error("initial place: CUDA error"); return rc; }
  if (rounds > 0)
    for (int k = 0; k < nP; k++) host_set_inst_center(m, m.place_insts[k], ctr[k].x, ctr[k].y);
  if (stats) {
    stats->iterations = rounds;
    stats->last_error = err;
    stats->last_hpwl = 0;
    stats->solver_iters_x = iters[0];
    stats->solver_iters_y = iters[1];
  }
  return GPL_OK;
}

}  // namespace gpl
