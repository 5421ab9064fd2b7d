// Electrostatic Poisson solve on the bin grid: the semantics of FFT::doFFT
// (src/fft.cpp:112-177) -- a 2-D DCT-II of the bin density, spectral
// scaling, then an inverse DCT for the potential and mixed sine/cosine
// inverses for the field (Ooura ddct2d / ddsct2d / ddcst2d,
// src/fftsg2d.cpp:569-758) -- computed with shared-memory FFTs.
//
// Layout: every grid array is row-major by y (bin index j*nx + i, the
// reference's BinGrid order); x is the reference's first FFT index.
//
// Three passes, each reading and writing every bin once:
//   A (rows)    density from the int64 areas (+ FP64 overflow partials, and
//               zeroing of the other area buffer) -> DCT-II along x -> spec
//   B (columns) DCT-II along y, spectral solve (phi^ = rho^/(wx^2+wy^2)),
//               inverse along y: P1 = IDCT_y(phi^), P2 = IDST_y(wy*phi^)
//   C (rows)    phi = IDCT_x(P1), Ex = IDST_x(wx*P1), Ey = IDCT_x(P2)
// Real transforms are taken two at a time through one complex FFT (two rows
// or two columns packed as real and imaginary parts), using Makhoul's
// even/odd reordering for the DCT-II and its inverse for the DCT-III; an
// IDST is a DCT-III of the reversed input with alternating output signs.
//
// Two forms of the same passes: on 512 x 512 and 1024 x 1024 grids one warp
// per packed pair runs a register FFT (the "warp form", with the density in
// its own kernel before pass A); other grids use one packed pair per
// 256-thread block and radix-4 Stockham passes in shared memory.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "gpl_internal.h"

namespace gpl {

namespace {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// exp(sign * 2 pi i m / n) for 0 <= m < n from the half table tw[m] =
// exp(-2 pi i m / n), m < n/2 (the second half is the negated first half).
__device__ __forceinline__ float2 twiddle(const float2* tw, int m, int n, int sign) {
  const int h = n >> 1;
  float2 w = m < h ? tw[m] : make_float2(-tw[m - h].x, -tw[m - h].y);
  if (sign > 0) w.y = -w.y;
  return w;
}

// Stockham FFT over `batch` sequences of length n = 2^logn stored back to
// back in the shared buffer a; b is a same-size scratch buffer.  Returns the
// buffer that holds the result.  sign -1: forward, +1: unnormalised inverse.
// tw: the half table of this n in shared memory.  Radix-4 passes (one radix-2
// pass first when logn is odd): half as many passes, barriers and shared
// round trips as radix 2.  Pass with sub-transform size ns: element j of
// quarter r is multiplied by exp(sign 2 pi i r k / 4ns), k = j mod ns, and the
// 4-point DFT's outputs go to (j - k) * 4 + k + r ns.
__device__ float2* block_fft(float2* a, float2* b, int n, int logn, int batch, int sign,
                             const float2* __restrict__ tw) {
  int ns = 1, lns = 0;
  if (logn & 1) {
    const int half = n >> 1;
    const int total = half * batch;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int bi = idx >> (logn - 1);
      const int j = idx & (half - 1);
      const float2* in = a + bi * n;
      float2* out = b + bi * n;
      const float2 u = in[j], v = in[j + half];
      out[2 * j] = cadd(u, v);
      out[2 * j + 1] = csub(u, v);
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
    ns = 2;
    lns = 1;
  }
  if (logn < 2) return a;
  const int lq = logn - 2, q = 1 << lq;
  const int total = q * batch;
  for (; ns < n; ns <<= 2, lns += 2) {
    const int tstep_log = logn - 2 - lns;       // n / (4 ns) = 2^tstep_log
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int bi = idx >> lq;
      const int j = idx & (q - 1);
      const float2* in = a + bi * n;
      float2* out = b + bi * n;
      const int k = j & (ns - 1);
      float2 x0 = in[j], x1 = in[j + q], x2 = in[j + 2 * q], x3 = in[j + 3 * q];
      if (ns > 1) {
        const int m = k << tstep_log;
        x1 = cmul(x1, twiddle(tw, m, n, sign));
        x2 = cmul(x2, twiddle(tw, 2 * m, n, sign));
        x3 = cmul(x3, twiddle(tw, 3 * m, n, sign));
      }
      // 4-point DFT with W = exp(sign 2 pi i / 4) = sign * i
      const float2 a0 = cadd(x0, x2), a1 = csub(x0, x2);
      const float2 b0 = cadd(x1, x3), b1 = csub(x1, x3);
      const float2 wb1 = sign > 0 ? make_float2(-b1.y, b1.x) : make_float2(b1.y, -b1.x);
      const int o = ((j - k) << 2) + k;
      out[o] = cadd(a0, b0);
      out[o + ns] = cadd(a1, wb1);
      out[o + 2 * ns] = csub(a0, b0);
      out[o + 3 * ns] = csub(a1, wb1);
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
  }
  return a;
}

// The twiddles of a length-n FFT, exp(-2 pi i m / n) for m < n/2, copied into
// shared memory from the kFftMax table (the same values, read once per block).
__device__ __forceinline__ void load_twiddles(float2* tws, const float2* __restrict__ tw, int n) {
  const int stride = kFftMax / n;
  for (int m = threadIdx.x; m < n / 2; m += blockDim.x) tws[m] = __ldg(&tw[m * stride]);
}

// Makhoul position of element i of a length-n sequence: v[m] = x[2m],
// v[n-1-m] = x[2m+1].
__device__ __forceinline__ int makhoul_pos(int i, int n) { return (i & 1) ? n - 1 - (i >> 1) : (i >> 1); }

// DCT-II post-processing of a packed pair: from Z = FFT(v0 + i v1) at k and
// (n-k)%n, return (C0[k], C1[k]) with C[k] = Re(exp(-i pi k / 2n) V[k]).
__device__ __forceinline__ float2 dct2_post(float2 zk, float2 znk, float2 w4) {
  float2 zc = cconj(znk);
  float2 v0 = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
  // (Z - conj Z')/(2i) = (Im part, -Re part)/2 of (Z - conj Z')
  float2 d = csub(zk, zc);
  float2 v1 = make_float2(0.5f * d.y, -0.5f * d.x);
  return make_float2(w4.x * v0.x - w4.y * v0.y, w4.x * v1.x - w4.y * v1.y);
}

// DCT-III pre-processing coefficient c[k] for one real sequence a:
// c[0] = a[0], c[k] = 1/2 exp(+i pi k / 2n) (a[k] - i a[n-k]).
__device__ __forceinline__ float2 dct3_pre(float ak, float ank, float2 w4, int k) {
  if (k == 0) return make_float2(ak, 0.0f);
  float2 e = make_float2(0.5f * w4.x, -0.5f * w4.y);      // 1/2 conj(w4)
  return cmul(e, make_float2(ak, -ank));
}

__device__ __forceinline__ void block_reduce_add(double v, double* out, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) *out = v;
  }
  __syncthreads();
}

struct PassAArgs {
  int nx, ny, logn, pairs_per_block;
  int core_lx, core_ly, core_ux, core_uy, size_x, size_y;
  float td;
  unsigned long long* area_pair[2];  // two sets of inst [nb] then filler [nb]
  const EvalCtl* ctl;                // area_cur: the set to read (the other is zeroed)
  const int64_t* nonplace;
  const float* density_in;           // standalone mode: density given
  float* density;
  float* spec;
  double* part_overflow;
  const float2* tw;
  const float2* w4;                  // exp(-i pi k / 2nx), k < nx
};

// Block vb of pass A (smem: the block's dynamic shared memory); shared by the
// per-job launch and the batched one, as are the bodies of passes B and C.
// The pass bodies are compiled once (not inlined) and called by both
// kernels: inlined into two kernels, the same float expressions can be
// contracted into fused multiply-adds differently, and a job's result would
// then depend on which kernel ran it.
__device__ __noinline__ void poisson_a_body(const PassAArgs& A, int vb, float2* smem) {
  __shared__ double red[32];
  const int n = A.nx;
  const int rp_n = A.pairs_per_block;
  float2* buf0 = smem;
  float2* buf1 = smem + rp_n * n;
  float2* tws = smem + 2 * rp_n * n;                 // [n/2] twiddles
  load_twiddles(tws, A.tw, n);
  const int nb = A.nx * A.ny;
  float ovf_f = 0.0f;          // the thread's few bins in float; FP64 across threads
  const unsigned long long* area = nullptr;
  unsigned long long* area_clear = nullptr;
  if (A.ctl) {
    const int cur = A.ctl->area_cur;
    area = cur == 0 ? A.area_pair[0] : A.area_pair[1];
    area_clear = cur == 0 ? A.area_pair[1] : A.area_pair[0];
  }
  if (A.density_in) {
    for (int idx = threadIdx.x; idx < rp_n * n; idx += blockDim.x) {
      const int rp = idx / n, i = idx - rp * n;
      const int r = vb * rp_n + rp;
      float d0 = 0.0f, d1 = 0.0f;
      if (r < A.ny / 2) {
        d0 = A.density_in[(2 * r) * n + i];
        d1 = A.density_in[(2 * r + 1) * n + i];
      }
      buf0[rp * n + makhoul_pos(i, n)] = make_float2(d0, d1);
    }
  } else {
    // restrict-qualified views: the areas read and the set cleared (and the
    // density written) are distinct arrays, so the loads of later elements
    // can be issued before the stores of earlier ones
    const unsigned long long* __restrict__ ar = area;
    unsigned long long* __restrict__ ac = area_clear;
    const int64_t* __restrict__ np = A.nonplace;
    float* __restrict__ dens = A.density;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < rp_n * n; idx += blockDim.x) {
      const int rp = idx / n, i = idx - rp * n;
      const int r = vb * rp_n + rp;
      float dd[2] = {0.0f, 0.0f};
      if (r < A.ny / 2) {
        const int blx = A.core_lx + i * A.size_x;
        const int bux = min(blx + A.size_x, A.core_ux);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int j = 2 * r + h;
          const int b = j * n + i;
          const int bly = A.core_ly + j * A.size_y;
          const int buy = min(bly + A.size_y, A.core_uy);
          const long long bin_area = (long long)(bux - blx) * (long long)(buy - bly);
          const float cap = __fmul_rn(ll_to_float(bin_area), A.td);
          const float fi = ll_to_float((long long)ar[b]);
          const float ff = ll_to_float((long long)ar[nb + b]);
          const float fn = ll_to_float(np[b]);
          // BinGrid::updateBinsGCellDensityArea (src/nesterovBase.cpp:804-818)
          dd[h] = __fdiv_rn(__fadd_rn(__fadd_rn(fi, ff), fn), cap);
          ovf_f += fmaxf(0.0f, __fsub_rn(__fadd_rn(fi, fn), cap));
          ac[b] = 0ull;
          ac[nb + b] = 0ull;
          dens[b] = dd[h];
        }
      }
      buf0[rp * n + makhoul_pos(i, n)] = make_float2(dd[0], dd[1]);
    }
  }
  __syncthreads();
  float2* res = block_fft(buf0, buf1, n, A.logn, rp_n, -1, tws);
  for (int idx = threadIdx.x; idx < rp_n * n; idx += blockDim.x) {
    const int rp = idx / n, k = idx - rp * n;
    const int r = vb * rp_n + rp;
    if (r >= A.ny / 2) continue;
    const float2* z = res + rp * n;
    float2 c = dct2_post(z[k], z[(n - k) & (n - 1)], __ldg(&A.w4[k]));
    A.spec[(2 * r) * n + k] = c.x;
    A.spec[(2 * r + 1) * n + k] = c.y;
  }
  if (A.part_overflow) block_reduce_add((double)ovf_f, &A.part_overflow[vb], red);
}

__global__ void __launch_bounds__(256) k_poisson_a(const __grid_constant__ PassAArgs A) {
  extern __shared__ float2 smem[];
  poisson_a_body(A, (int)blockIdx.x, smem);
}

struct PassBArgs {
  int nx, ny, logn, col_pairs;       // column pairs per block
  const float* spec;
  float* p1;
  float* p2;
  const float* wx;
  const float* wy;
  const float2* tw;
  const float2* w4;                  // exp(-i pi k / 2ny), k < ny
  float scale;                       // 4 / (nx ny)
};

__device__ __noinline__ void poisson_b_body(const PassBArgs& B, int vb, float2* smem) {
  const int n = B.ny;
  const int cp = B.col_pairs;
  float2* s0 = smem;                 // [cp][n] work
  float2* s1 = smem + cp * n;        // [cp][n] scratch
  float2* s2 = smem + 2 * cp * n;    // [cp][n] spectrum: (phi^ col u0, phi^ col u1)
  float2* tws = smem + 3 * cp * n;   // [n/2] twiddles
  load_twiddles(tws, B.tw, n);
  const int u_base = vb * 2 * cp;
  // load: column pair q holds columns u_base + 2q, +1
#pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * cp * n; idx += blockDim.x) {
    const int v = idx / (2 * cp);           // row (y) index: consecutive threads read one row
    const int c = idx - v * 2 * cp;         // column within block
    const int q = c >> 1;
    const float val = B.spec[v * B.nx + u_base + c];
    float* slot = reinterpret_cast<float*>(&s0[q * n + makhoul_pos(v, n)]);
    slot[c & 1] = val;
  }
  __syncthreads();
  float2* res = block_fft(s0, s1, n, B.logn, cp, -1, tws);
  float2* other = (res == s0) ? s1 : s0;
  // DCT-II along y, then the spectral solve (src/fft.cpp:117-166)
  for (int idx = threadIdx.x; idx < cp * n; idx += blockDim.x) {
    const int q = idx / n, v = idx - q * n;
    const float2* z = res + q * n;
    float2 a = dct2_post(z[v], z[(n - v) & (n - 1)], __ldg(&B.w4[v]));
    float out[2];
    for (int h = 0; h < 2; h++) {
      const int u = u_base + 2 * q + h;
      float d = h ? a.y : a.x;
      if (u == 0) d *= 0.5f;
      if (v == 0) d *= 0.5f;
      d *= B.scale;
      float ph = 0.0f;
      if (u != 0 || v != 0) {
        const float wxu = __ldg(&B.wx[u]), wyv = __ldg(&B.wy[v]);
        ph = __fdiv_rn(d, __fadd_rn(__fmul_rn(wxu, wxu), __fmul_rn(wyv, wyv)));
      }
      out[h] = ph;
    }
    s2[q * n + v] = make_float2(out[0], out[1]);
  }
  __syncthreads();
  // P1 = IDCT_y(phi^) for both columns (one complex IFFT)
  for (int idx = threadIdx.x; idx < cp * n; idx += blockDim.x) {
    const int q = idx / n, k = idx - q * n;
    const float2* sp = s2 + q * n;
    const float2 w4 = __ldg(&B.w4[k]);
    float2 ak = sp[k], ank = k ? sp[n - k] : make_float2(0.f, 0.f);
    float2 c0 = dct3_pre(ak.x, ank.x, w4, k);
    float2 c1 = dct3_pre(ak.y, ank.y, w4, k);
    other[q * n + k] = make_float2(c0.x - c1.y, c0.y + c1.x);   // c0 + i c1
  }
  __syncthreads();
  float2* scratch = (other == s0) ? s1 : s0;
  res = block_fft(other, scratch, n, B.logn, cp, +1, tws);
  for (int idx = threadIdx.x; idx < 2 * cp * n; idx += blockDim.x) {
    const int v = idx / (2 * cp);
    const int c = idx - v * 2 * cp;
    const int q = c >> 1;
    const float2 w = res[q * n + makhoul_pos(v, n)];
    B.p1[v * B.nx + u_base + c] = (c & 1) ? w.y : w.x;
  }
  __syncthreads();
  // P2 = IDST_y(wy * phi^): DCT-III of b[k] = wy[n-k] phi^[n-k] (b[0] = 0)
  other = (res == s0) ? s1 : s0;
  for (int idx = threadIdx.x; idx < cp * n; idx += blockDim.x) {
    const int q = idx / n, k = idx - q * n;
    const float2* sp = s2 + q * n;
    const float2 w4 = __ldg(&B.w4[k]);
    float2 bk = make_float2(0.f, 0.f), bnk = make_float2(0.f, 0.f);
    if (k) {
      const float w = __ldg(&B.wy[n - k]);
      bk = make_float2(__fmul_rn(sp[n - k].x, w), __fmul_rn(sp[n - k].y, w));
      const float w2 = __ldg(&B.wy[k]);
      bnk = make_float2(__fmul_rn(sp[k].x, w2), __fmul_rn(sp[k].y, w2));
    }
    float2 c0 = dct3_pre(bk.x, bnk.x, w4, k);
    float2 c1 = dct3_pre(bk.y, bnk.y, w4, k);
    other[q * n + k] = make_float2(c0.x - c1.y, c0.y + c1.x);
  }
  __syncthreads();
  scratch = (other == s0) ? s1 : s0;
  res = block_fft(other, scratch, n, B.logn, cp, +1, tws);
  for (int idx = threadIdx.x; idx < 2 * cp * n; idx += blockDim.x) {
    const int v = idx / (2 * cp);
    const int c = idx - v * 2 * cp;
    const int q = c >> 1;
    const float2 w = res[q * n + makhoul_pos(v, n)];
    const float s = (v & 1) ? -1.0f : 1.0f;
    B.p2[v * B.nx + u_base + c] = s * ((c & 1) ? w.y : w.x);
  }
}

__global__ void __launch_bounds__(256) k_poisson_b(const __grid_constant__ PassBArgs B) {
  extern __shared__ float2 smem[];
  poisson_b_body(B, (int)blockIdx.x, smem);
}

struct PassCArgs {
  int nx, ny, logn, pairs_per_block;
  const float* p1;
  const float* p2;
  float2* field;          // (Ex, Ey) interleaved, may be null
  float* fx;              // or separate planes (standalone API)
  float* fy;
  float* phi;             // may be null
  const float* wx;
  const float2* tw;
  const float2* w4;       // exp(-i pi k / 2nx)
};

// One DCT-III (or IDST with sign flip) of a packed row pair held in smem
// rows a0/a1 (real inputs); writes packed c coefficients into dst.
__device__ __forceinline__ void build_dct3_pair(const float* a0, const float* a1, const float* wmul,
                                                bool reverse, float2* dst, int n, int k, float2 w4) {
  float x0k, x0nk, x1k, x1nk;
  if (!reverse) {
    x0k = a0[k]; x1k = a1[k];
    x0nk = k ? a0[n - k] : 0.f; x1nk = k ? a1[n - k] : 0.f;
  } else {
    // b[k] = w[n-k] a[n-k] for k >= 1, b[0] = 0
    if (k) {
      const float wa = wmul ? __ldg(&wmul[n - k]) : 1.0f;
      const float wb = wmul ? __ldg(&wmul[k]) : 1.0f;
      x0k = __fmul_rn(a0[n - k], wa); x1k = __fmul_rn(a1[n - k], wa);
      x0nk = __fmul_rn(a0[k], wb); x1nk = __fmul_rn(a1[k], wb);
    } else {
      x0k = x1k = x0nk = x1nk = 0.f;
    }
  }
  float2 c0 = dct3_pre(x0k, x0nk, w4, k);
  float2 c1 = dct3_pre(x1k, x1nk, w4, k);
  dst[k] = make_float2(c0.x - c1.y, c0.y + c1.x);
}

__device__ __noinline__ void poisson_c_body(const PassCArgs& C, int vb, float2* smem) {
  const int n = C.nx;
  const int rp_n = C.pairs_per_block;
  float* rows = reinterpret_cast<float*>(smem);       // [rp][4][n]: p1 row0, p1 row1, p2 row0, p2 row1
  float2* s0 = smem + rp_n * 2 * n;                    // [rp][n]
  float2* s1 = s0 + rp_n * n;                          // [rp][n]
  float2* tws = s1 + rp_n * n;                         // [n/2] twiddles
  load_twiddles(tws, C.tw, n);
#pragma unroll 4
  for (int idx = threadIdx.x; idx < rp_n * 2 * n; idx += blockDim.x) {
    const int rp = idx / (2 * n), t = idx - rp * 2 * n;
    const int h = t / n, i = t - h * n;
    const int r = vb * rp_n + rp;
    float a = 0.f, b = 0.f;
    if (r < C.ny / 2) {
      a = C.p1[(2 * r + h) * n + i];
      b = C.p2[(2 * r + h) * n + i];
    }
    rows[(rp * 4 + h) * n + i] = a;
    rows[(rp * 4 + 2 + h) * n + i] = b;
  }
  __syncthreads();
  // three transforms: 0 = phi (IDCT P1), 1 = Ex (IDST wx*P1), 2 = Ey (IDCT P2)
  for (int tr = (C.phi ? 0 : 1); tr < 3; tr++) {
    for (int idx = threadIdx.x; idx < rp_n * n; idx += blockDim.x) {
      const int rp = idx / n, k = idx - rp * n;
      const float* a0 = rows + (rp * 4 + (tr == 2 ? 2 : 0)) * n;
      const float* a1 = a0 + n;
      build_dct3_pair(a0, a1, tr == 1 ? C.wx : nullptr, tr == 1, s0 + rp * n, n, k, __ldg(&C.w4[k]));
    }
    __syncthreads();
    float2* res = block_fft(s0, s1, n, C.logn, rp_n, +1, tws);
    for (int idx = threadIdx.x; idx < rp_n * n; idx += blockDim.x) {
      const int rp = idx / n, m = idx - rp * n;
      const int r = vb * rp_n + rp;
      if (r >= C.ny / 2) continue;
      const float2 w = res[rp * n + makhoul_pos(m, n)];
      float v0 = w.x, v1 = w.y;
      if (tr == 1 && (m & 1)) { v0 = -v0; v1 = -v1; }
      const int b0 = (2 * r) * n + m, b1 = (2 * r + 1) * n + m;
      if (tr == 0) {
        C.phi[b0] = v0; C.phi[b1] = v1;
      } else if (C.field) {
        // Ex waits in the P1 rows (no longer read) and goes out with Ey as
        // one float2 per bin
        float* ex = rows + (rp * 4) * n;
        if (tr == 1) {
          ex[m] = v0; ex[n + m] = v1;
        } else {
          C.field[b0] = make_float2(ex[m], v0);
          C.field[b1] = make_float2(ex[n + m], v1);
        }
      } else {
        float* dst = tr == 1 ? C.fx : C.fy;
        dst[b0] = v0; dst[b1] = v1;
      }
    }
    __syncthreads();
    if (res != s0) { float2* t = s0; s0 = s1; s1 = t; }
  }
}

__global__ void __launch_bounds__(256) k_poisson_c(const __grid_constant__ PassCArgs C) {
  extern __shared__ float2 smem[];
  poisson_c_body(C, (int)blockIdx.x, smem);
}

// ---------------------------------------------------------------------------
// Warp form for 1024 x 1024 and 512 x 512 grids.  One warp runs one N-point
// FFT of a packed pair (two rows or two columns as real and imaginary parts)
// with N/32 elements per lane in registers, four-step: DFTs along n2 inside
// each lane, the twiddle W^(n1 k2), one transpose through padded shared
// memory, then 32-point DFTs along n1 (for N = 512 each of those is split
// over a lane pair: two 16-point DFTs and one radix-2 step by shuffle).  This
// replaces five shared-memory radix-4 passes with block barriers.
// Independent transforms of a pair run on separate warps (the column pass's
// two inverse transforms, the field pass's three), inputs and tables arrive
// by cp.async so that a warp waits for memory once, and the density comes
// from its own grid-wide kernel first (fusing it into the row pass was
// measured slower: its long blocks overlap worse with the WA kernel).

template <int N>
struct WarpFft {
  static_assert(N == 1024 || N == 512, "warp form sizes");
  static constexpr int kE = N / 32;                     // elements per lane
  static constexpr int kStride = kE + 1;                // padded transpose row
  static constexpr int kBuf = 2 * N > 2 * 32 * kStride ? 2 * N : 2 * 32 * kStride;   // floats per warp buffer
};

// exp(-2 pi i n1 k2 / N) at [k2 * 32 + n1], k2 < N/32: one coalesced row per k2.
__device__ __align__(16) float2 g_tw1024[1024];
__device__ __align__(16) float2 g_tw512[512];

template <int N>
__device__ __forceinline__ const float2* tw_table() {
  if constexpr (N == 1024) return g_tw1024;
  else return g_tw512;
}

template <int kBits>
__host__ __device__ constexpr int brev(int r) {
  int o = 0;
  for (int b = 0; b < kBits; b++) o |= ((r >> b) & 1) << (kBits - 1 - b);
  return o;
}

// cos and sin of 2 pi m / 32, m = 0..8 (the other octants by symmetry).
__host__ __device__ constexpr float cos32_oct(int m) {
  return m == 0 ? 1.0f : m == 1 ? 0.980785280403230449f : m == 2 ? 0.923879532511286756f
       : m == 3 ? 0.831469612302545237f : m == 4 ? 0.707106781186547524f
       : m == 5 ? 0.555570233019602225f : m == 6 ? 0.382683432365089772f
       : m == 7 ? 0.195090322016128268f : 0.0f;
}
__host__ __device__ constexpr float cos32(int m) {   // 0 <= m < 16
  return m <= 8 ? cos32_oct(m) : -cos32_oct(16 - m);
}
__host__ __device__ constexpr float sin32(int m) {   // 0 <= m < 16
  return m <= 8 ? cos32_oct(8 - m) : cos32_oct(m - 8);
}

// (re, im) times exp(kSign 2 pi i m / 32), m < 16 a compile-time constant.
template <int kSign>
__device__ __forceinline__ void rot32(float& re, float& im, int m) {
  if (m == 0) return;
  const float r = re, i = im;
  if (m == 8) {                     // exp(kSign i pi / 2) = kSign i
    re = kSign > 0 ? -i : i;
    im = kSign > 0 ? r : -r;
    return;
  }
  const float c = cos32(m), sn = kSign > 0 ? sin32(m) : -sin32(m);
  re = r * c - i * sn;
  im = r * sn + i * c;
}

// In-register M-point DFT (M = 16 or 32), radix-2 decimation in frequency:
// natural input order, register r ends with output brev(r).  Twiddles
// exp(kSign 2 pi i j / len) = exp(kSign 2 pi i (j 32/len) / 32) are
// compile-time constants after unrolling.
template <int M, int kSign>
__device__ __forceinline__ void dft_reg(float (&re)[M], float (&im)[M]) {
#pragma unroll
  for (int len = M; len >= 2; len >>= 1) {
    const int half = len >> 1;
#pragma unroll
    for (int start = 0; start < M; start += len) {
#pragma unroll
      for (int j = 0; j < half; j++) {
        const int a = start + j, b = a + half;
        const float ar = re[a], ai = im[a], br = re[b], bi = im[b];
        re[a] = ar + br;
        im[a] = ai + bi;
        re[b] = ar - br;
        im[b] = ai - bi;
        rot32<kSign>(re[b], im[b], j * (32 / len));
      }
    }
  }
}

// Asynchronous global -> shared copies (cp.async, sm_80+): a warp issues
// all of its inputs and tables at once and waits once, so each pass pays one
// memory latency instead of one per dependent load batch.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Copies n floats (n a multiple of 4 * 32, both pointers 16-byte aligned)
// with the calling warp's 16-byte cp.async.
__device__ __forceinline__ void warp_copy_async(float* dst, const float* src, int n) {
  const int l = threadIdx.x & 31;
  for (int t = 4 * l; t < n; t += 128) cp_async16(dst + t, src + t);
}

// N-point FFT of buf (natural order in and out, [WarpFft<N>::kBuf] floats,
// float2 view) by the calling warp; kSign -1 forward, +1 unnormalised
// inverse.  tws: the tw_table<N>() table in shared memory.
template <int N, int kSign>
__device__ __forceinline__ void warp_fft(float2* buf, const float2* tws) {
  constexpr int E = WarpFft<N>::kE, S = WarpFft<N>::kStride;
  constexpr int kBitsE = E == 32 ? 5 : 4;
  const int l = threadIdx.x & 31;
  float re[32], im[32];
  // stage 1: lane n1 = l holds x[n1 + 32 n2], n2 < E; DFT along n2
#pragma unroll
  for (int j = 0; j < E; j++) {
    const float2 v = buf[l + 32 * j];
    re[j] = v.x; im[j] = v.y;
  }
  if constexpr (E == 32) {
    dft_reg<32, kSign>(re, im);
  } else {
    float r16[16], i16[16];
#pragma unroll
    for (int j = 0; j < 16; j++) { r16[j] = re[j]; i16[j] = im[j]; }
    dft_reg<16, kSign>(r16, i16);
#pragma unroll
    for (int j = 0; j < 16; j++) { re[j] = r16[j]; im[j] = i16[j]; }
  }
  // twiddle W_N^(n1 k2), register r holding k2 = brev(r)
#pragma unroll
  for (int r = 1; r < E; r++) {
    float2 w = tws[brev<kBitsE>(r) * 32 + l];
    if (kSign > 0) w.y = -w.y;
    const float xr = re[r], xi = im[r];
    re[r] = xr * w.x - xi * w.y;
    im[r] = xr * w.y + xi * w.x;
  }
  __syncwarp();
  float* tr = reinterpret_cast<float*>(buf);
  float* ti = tr + 32 * S;
#pragma unroll
  for (int r = 0; r < E; r++) {
    tr[l * S + brev<kBitsE>(r)] = re[r];
    ti[l * S + brev<kBitsE>(r)] = im[r];
  }
  __syncwarp();
  if constexpr (E == 32) {
    // stage 2: lane k2 = l takes n1 = 0..31, a 32-point DFT, X[k2 + 32 k1]
#pragma unroll
    for (int n1 = 0; n1 < 32; n1++) {
      re[n1] = tr[n1 * S + l];
      im[n1] = ti[n1 * S + l];
    }
    __syncwarp();
    dft_reg<32, kSign>(re, im);
#pragma unroll
    for (int r = 0; r < 32; r++) buf[l + 32 * brev<5>(r)] = make_float2(re[r], im[r]);
  } else {
    // stage 2 for E = 16: lane pair (2 k2, 2 k2 + 1) takes the even and odd
    // n1 of column k2, one 16-point DFT each, then X[k] = E[k] + W^k O[k]
    // (even lane) and X[k + 16] = E[k] - W^k O[k] (odd lane), W = W_32
    const int k2 = l >> 1, odd = l & 1;
    float r16[16], i16[16];
#pragma unroll
    for (int i = 0; i < 16; i++) {
      r16[i] = tr[(2 * i + odd) * S + k2];
      i16[i] = ti[(2 * i + odd) * S + k2];
    }
    __syncwarp();
    dft_reg<16, kSign>(r16, i16);
#pragma unroll
    for (int r = 0; r < 16; r++) {
      const int k = brev<4>(r);
      const float pr = __shfl_xor_sync(0xffffffffu, r16[r], 1);
      const float pi = __shfl_xor_sync(0xffffffffu, i16[r], 1);
      // W^k O: O is the partner's value on the even lane, the own on the odd
      float orr = odd ? r16[r] : pr, oi = odd ? i16[r] : pi;
      rot32<kSign>(orr, oi, k);
      const float er = odd ? pr : r16[r], ei = odd ? pi : i16[r];
      const float xr = odd ? er - orr : er + orr, xi = odd ? ei - oi : ei + oi;
      buf[k2 + 16 * (k + 16 * odd)] = make_float2(xr, xi);
    }
  }
  __syncwarp();
}

// Density of every bin from the int64 areas, FP64 overflow partials (one per
// block) and the other area set cleared: pass A's first half.
__global__ void __launch_bounds__(256) k_poisson_dens(PassAArgs A) {
  __shared__ double red[32];
  const int nb = A.nx * A.ny;
  const int cur = A.ctl->area_cur;
  const unsigned long long* __restrict__ ar = cur == 0 ? A.area_pair[0] : A.area_pair[1];
  unsigned long long* __restrict__ ac = cur == 0 ? A.area_pair[1] : A.area_pair[0];
  const int64_t* __restrict__ np = A.nonplace;
  float* __restrict__ dens = A.density;
  float ovf = 0.0f;
#pragma unroll 4
  for (int b = blockIdx.x * 256 + threadIdx.x; b < nb; b += gridDim.x * 256) {
    const int j = b >> A.logn, i = b & (A.nx - 1);     // bin grids are powers of 2
    const int blx = A.core_lx + i * A.size_x, bux = min(blx + A.size_x, A.core_ux);
    const int bly = A.core_ly + j * A.size_y, buy = min(bly + A.size_y, A.core_uy);
    const long long bin_area = (long long)(bux - blx) * (long long)(buy - bly);
    const float cap = __fmul_rn(ll_to_float(bin_area), A.td);
    const float fi = ll_to_float((long long)ar[b]);
    const float ff = ll_to_float((long long)ar[nb + b]);
    const float fn = ll_to_float(np[b]);
    // BinGrid::updateBinsGCellDensityArea (src/nesterovBase.cpp:804-818)
    dens[b] = __fdiv_rn(__fadd_rn(__fadd_rn(fi, ff), fn), cap);
    ovf += fmaxf(0.0f, __fsub_rn(__fadd_rn(fi, fn), cap));
    ac[b] = 0ull;
    ac[nb + b] = 0ull;
  }
  if (A.part_overflow) block_reduce_add((double)ovf, &A.part_overflow[blockIdx.x], red);
}

// Pass A, warp form: DCT-II along x of row pair r (density rows 2r, 2r+1).
// Shared memory: FFT buffer, w4 and twiddle tables.
template <int N>
__global__ void __launch_bounds__(32) k_poisson_rows_w(PassAArgs A) {
  extern __shared__ float2 smem[];
  float2* buf = smem;
  float2* w4s = smem + WarpFft<N>::kBuf / 2;
  float2* tws = w4s + N;
  const int l = threadIdx.x;
  const int r = blockIdx.x;
  const float* d0 = (A.density_in ? A.density_in : A.density) + (size_t)(2 * r) * N;
  const float* d1 = d0 + N;
  // Makhoul order: v[m] = x[2m], v[n-1-m] = x[2m+1]
#pragma unroll 8
  for (int j = 0; j < N / 32; j++) {
    const int i = l + 32 * j;
    float* dst = reinterpret_cast<float*>(&buf[makhoul_pos(i, N)]);
    cp_async4(dst, d0 + i);
    cp_async4(dst + 1, d1 + i);
  }
  warp_copy_async(reinterpret_cast<float*>(w4s), reinterpret_cast<const float*>(A.w4), 2 * N);
  warp_copy_async(reinterpret_cast<float*>(tws), reinterpret_cast<const float*>(tw_table<N>()), 2 * N);
  cp_async_wait_all();
  __syncwarp();
  warp_fft<N, -1>(buf, tws);
  float* s0 = A.spec + (size_t)(2 * r) * N;
  float* s1 = s0 + N;
#pragma unroll 8
  for (int j = 0; j < N / 32; j++) {
    const int k = l + 32 * j;
    const float2 c = dct2_post(buf[k], buf[(N - k) & (N - 1)], w4s[k]);
    s0[k] = c.x;
    s1[k] = c.y;
  }
}

// Pass B, warp form: kP column pairs per block (2 kP adjacent columns; 32-byte
// row segments at kP = 4) and two warps per pair: warp (q, 0) takes the
// forward transform and the spectral solve of pair q, then the two inverse
// transforms (P1 and P2) run side by side on warps (q, 0) and (q, 1).
template <int N>
struct ColsShape {
  static constexpr int kP = N == 1024 ? 4 : 2;          // column pairs per block
  static constexpr int kThreads = 64 * kP;
  static constexpr int kH = kP / 2;                     // float4 segments per row
};

template <int N>
__global__ void __launch_bounds__(ColsShape<N>::kThreads) k_poisson_cols_w(PassBArgs B) {
  extern __shared__ float2 smem[];
  constexpr int kP = ColsShape<N>::kP, kT = ColsShape<N>::kThreads, kH = ColsShape<N>::kH;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int q = w >> 1, role = w & 1;
  constexpr int kBufF2 = WarpFft<N>::kBuf / 2;
  // [pair][role] FFT buffers, [pair] spectra, then the tables
  float2* buf = smem + (size_t)w * kBufF2;
  float2* spc = smem + (size_t)2 * kP * kBufF2 + (size_t)q * N;
  float2* w4s = smem + (size_t)kP * (2 * kBufF2 + N);    // [n] w4 (y)
  float2* tws = w4s + N;                                 // [n] twiddles
  float* wys = reinterpret_cast<float*>(tws + N);        // [n] wy
  const int u_base = blockIdx.x * 2 * kP;
  const int nx = B.nx;
  // inputs: 8-byte copies of column pairs into the pairs' role-0 buffers
  // (Makhoul order), and the block's tables
  for (int idx = threadIdx.x; idx < N * kP; idx += kT) {
    const int v = idx / kP, c = idx % kP;       // row v, pair c
    cp_async8(smem + (size_t)(2 * c) * kBufF2 + makhoul_pos(v, N), B.spec + (size_t)v * nx + u_base + 2 * c);
  }
  for (int t = 4 * threadIdx.x; t < 2 * N; t += 4 * kT) {
    cp_async16(reinterpret_cast<float*>(w4s) + t, reinterpret_cast<const float*>(B.w4) + t);
    cp_async16(reinterpret_cast<float*>(tws) + t, reinterpret_cast<const float*>(tw_table<N>()) + t);
  }
  for (int t = 4 * threadIdx.x; t < N; t += 4 * kT) cp_async16(wys + t, B.wy + t);
  const float wx0 = __ldg(&B.wx[u_base + 2 * q]), wx1 = __ldg(&B.wx[u_base + 2 * q + 1]);
  cp_async_wait_all();
  __syncthreads();
  if (role == 0) {
    warp_fft<N, -1>(buf, tws);
    // DCT-II along y, then the spectral solve (src/fft.cpp:117-166)
#pragma unroll 4
    for (int j = 0; j < N / 32; j++) {
      const int v = l + 32 * j;
      const float2 a = dct2_post(buf[v], buf[(N - v) & (N - 1)], w4s[v]);
      const float wyv = wys[v];
      float out[2];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int u = u_base + 2 * q + h;
        float d = h ? a.y : a.x;
        if (u == 0) d *= 0.5f;
        if (v == 0) d *= 0.5f;
        d *= B.scale;
        float ph = 0.0f;
        if (u != 0 || v != 0) {
          const float wxu = h ? wx1 : wx0;
          ph = __fdiv_rn(d, __fadd_rn(__fmul_rn(wxu, wxu), __fmul_rn(wyv, wyv)));
        }
        out[h] = ph;
      }
      spc[v] = make_float2(out[0], out[1]);
    }
  }
  __syncthreads();
  if (role == 0) {
    // P1 = IDCT_y(phi^) of both columns (one complex inverse FFT)
#pragma unroll 4
    for (int j = 0; j < N / 32; j++) {
      const int k = l + 32 * j;
      const float2 w4 = w4s[k];
      const float2 ak = spc[k], ank = k ? spc[N - k] : make_float2(0.f, 0.f);
      const float2 c0 = dct3_pre(ak.x, ank.x, w4, k);
      const float2 c1 = dct3_pre(ak.y, ank.y, w4, k);
      buf[k] = make_float2(c0.x - c1.y, c0.y + c1.x);
    }
  } else {
    // P2 = IDST_y(wy * phi^): DCT-III of b[k] = wy[n-k] phi^[n-k] (b[0] = 0)
#pragma unroll 4
    for (int j = 0; j < N / 32; j++) {
      const int k = l + 32 * j;
      const float2 w4 = w4s[k];
      float2 bk = make_float2(0.f, 0.f), bnk = make_float2(0.f, 0.f);
      if (k) {
        const float wa = wys[N - k];
        const float2 a = spc[N - k];
        bk = make_float2(__fmul_rn(a.x, wa), __fmul_rn(a.y, wa));
        const float wb = wys[k];
        const float2 b = spc[k];
        bnk = make_float2(__fmul_rn(b.x, wb), __fmul_rn(b.y, wb));
      }
      const float2 c0 = dct3_pre(bk.x, bnk.x, w4, k);
      const float2 c1 = dct3_pre(bk.y, bnk.y, w4, k);
      buf[k] = make_float2(c0.x - c1.y, c0.y + c1.x);
    }
  }
  __syncwarp();
  warp_fft<N, 1>(buf, tws);
  __syncthreads();
  // stores: P1 from the role-0 buffers, P2 (signs alternating in v) from
  // the role-1 buffers; a thread writes four columns (two pairs) as a float4
  for (int idx = threadIdx.x; idx < N * kH * 2; idx += kT) {
    const int h = idx % kH, out = (idx / kH) & 1, v = idx / (2 * kH);
    const int m = makhoul_pos(v, N);
    const float2* b0 = smem + (size_t)(2 * (2 * h) + out) * kBufF2;   // pair 2h, role out
    const float2* b1 = b0 + 2 * kBufF2;                               // pair 2h + 1
    const float2 x0 = b0[m], x1 = b1[m];
    const float sg = (out && (v & 1)) ? -1.0f : 1.0f;
    float* dst = out ? B.p2 : B.p1;
    *reinterpret_cast<float4*>(dst + (size_t)v * nx + u_base + 4 * h) =
        make_float4(sg * x0.x, sg * x0.y, sg * x1.x, sg * x1.y);
  }
}

// Pass C, warp form: two row pairs per block and one warp per transform of
// a pair (Ex = IDST_x(wx * P1), Ey = IDCT_x(P2), phi = IDCT_x(P1)); the
// block writes the field (Ex, Ey per bin) once all transforms are done.
constexpr int kWFieldPairs = 2;
constexpr int kWFieldThreads = 96 * kWFieldPairs;

template <int N>
__global__ void __launch_bounds__(kWFieldThreads) k_poisson_field_w(PassCArgs C) {
  extern __shared__ float2 smem[];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int p = w / 3, role = w % 3;            // role 0 Ex, 1 Ey, 2 phi
  constexpr int kBufF2 = WarpFft<N>::kBuf / 2;
  float2* buf = smem + (size_t)w * kBufF2;
  float* rows_all = reinterpret_cast<float*>(smem + (size_t)3 * kWFieldPairs * kBufF2);  // [pair][4][n]
  float2* w4s = reinterpret_cast<float2*>(rows_all + (size_t)kWFieldPairs * 4 * N);
  float2* tws = w4s + N;
  float* wxs = reinterpret_cast<float*>(tws + N);
  const int r0 = blockIdx.x * kWFieldPairs;
  // inputs: P1 and P2 rows of both pairs (contiguous per array), tables
  {
    const size_t base = (size_t)(2 * r0) * N;
    const int n = 2 * N * kWFieldPairs;       // floats per array
    for (int t = 4 * threadIdx.x; t < n; t += 4 * kWFieldThreads) {
      const int pp = t / (2 * N), o = t - pp * 2 * N;
      cp_async16(rows_all + (size_t)pp * 4 * N + o, C.p1 + base + t);
      cp_async16(rows_all + (size_t)pp * 4 * N + 2 * N + o, C.p2 + base + t);
    }
    for (int t = 4 * threadIdx.x; t < 2 * N; t += 4 * kWFieldThreads) {
      cp_async16(reinterpret_cast<float*>(w4s) + t, reinterpret_cast<const float*>(C.w4) + t);
      cp_async16(reinterpret_cast<float*>(tws) + t, reinterpret_cast<const float*>(tw_table<N>()) + t);
    }
    for (int t = 4 * threadIdx.x; t < N; t += 4 * kWFieldThreads) cp_async16(wxs + t, C.wx + t);
  }
  cp_async_wait_all();
  __syncthreads();
  const float* rows = rows_all + (size_t)p * 4 * N;
  if (role != 2 || C.phi) {
    const float* a0 = rows + (role == 1 ? 2 : 0) * N;
    const float* a1 = a0 + N;
#pragma unroll 4
    for (int j = 0; j < N / 32; j++) {
      const int k = l + 32 * j;
      float x0k, x0nk, x1k, x1nk;
      if (role != 0) {
        x0k = a0[k]; x1k = a1[k];
        x0nk = k ? a0[N - k] : 0.f; x1nk = k ? a1[N - k] : 0.f;
      } else if (k) {
        // b[k] = wx[n-k] a[n-k] for k >= 1, b[0] = 0
        const float wa = wxs[N - k], wb = wxs[k];
        x0k = __fmul_rn(a0[N - k], wa); x1k = __fmul_rn(a1[N - k], wa);
        x0nk = __fmul_rn(a0[k], wb); x1nk = __fmul_rn(a1[k], wb);
      } else {
        x0k = x1k = x0nk = x1nk = 0.f;
      }
      const float2 w4 = w4s[k];
      const float2 c0 = dct3_pre(x0k, x0nk, w4, k);
      const float2 c1 = dct3_pre(x1k, x1nk, w4, k);
      buf[k] = make_float2(c0.x - c1.y, c0.y + c1.x);
    }
    __syncwarp();
    warp_fft<N, 1>(buf, tws);
  }
  __syncthreads();
  // outputs, bin m of rows 2r and 2r + 1 of both pairs (IDST signs alternate)
  for (int idx = threadIdx.x; idx < kWFieldPairs * N; idx += kWFieldThreads) {
    const int pp = idx / N, m = idx - pp * N;
    const size_t b0 = (size_t)(2 * (r0 + pp)) * N;
    const int mp = makhoul_pos(m, N);
    const float2* bp = smem + (size_t)(3 * pp) * kBufF2;
    float2 ex = bp[mp];
    const float2 ey = bp[kBufF2 + mp];
    if (m & 1) { ex.x = -ex.x; ex.y = -ex.y; }
    if (C.field) {
      C.field[b0 + m] = make_float2(ex.x, ey.x);
      C.field[b0 + N + m] = make_float2(ex.y, ey.y);
    } else {
      C.fx[b0 + m] = ex.x; C.fx[b0 + N + m] = ex.y;
      C.fy[b0 + m] = ey.x; C.fy[b0 + N + m] = ey.y;
    }
    if (C.phi) {
      const float2 ph = bp[2 * kBufF2 + mp];
      C.phi[b0 + m] = ph.x; C.phi[b0 + N + m] = ph.y;
    }
  }
}

template <int N>
constexpr size_t smem_rows_w() { return (size_t)WarpFft<N>::kBuf * 4 + 2 * N * 8; }
template <int N>
constexpr size_t smem_cols_w() {
  return (size_t)ColsShape<N>::kP * (2 * WarpFft<N>::kBuf * 4 + N * 8) + 2 * N * 8 + N * 4;
}
template <int N>
constexpr size_t smem_field_w() {
  return (size_t)kWFieldPairs * (3 * WarpFft<N>::kBuf * 4 + 4 * N * 4) + 2 * N * 8 + N * 4;
}

// The sequence length of the warp form for this grid, or 0 (block form).
int warp_form(int nx, int ny) { return nx == ny && (nx == 1024 || nx == 512) ? nx : 0; }


int ilog2(int v) { int l = 0; while ((1 << l) < v) l++; return l; }

}  // namespace

// Row (column) pairs per block: as few as keep 256 threads busy, so that the
// grid has up to kMinPoissonBlocks blocks (several per SM) to hide the
// latency of the loads; small grids are spread over SMs instead of being
// serialised in a few blocks.
constexpr int kMinPoissonBlocks = 512;
int pairs_a(int nx, int ny) { return max(1, min(min(ny / 2, 2048 / nx), (ny / 2) / kMinPoissonBlocks)); }
int pairs_b(int nx, int ny) {
  return max(1, min(min(nx / 2, min(4, 4096 / ny)), (nx / 2) / kMinPoissonBlocks));
}
int pairs_c(int nx, int ny) { return pairs_a(nx, ny); }

size_t smem_a(int nx, int ny) { return ((size_t)2 * pairs_a(nx, ny) * nx + nx / 2) * sizeof(float2); }
size_t smem_b(int nx, int ny) { return ((size_t)3 * pairs_b(nx, ny) * ny + ny / 2) * sizeof(float2); }
size_t smem_c(int nx, int ny) { return ((size_t)4 * pairs_c(nx, ny) * nx + nx / 2) * sizeof(float2); }

// Blocks of the density pass (one FP64 overflow partial each): the warp
// form's grid-wide density kernel takes four bins per thread.
int poisson_blocks_a(int nx, int ny) {
  if (warp_form(nx, ny)) return nx * ny / 1024;
  int r = pairs_a(nx, ny);
  return (ny / 2 + r - 1) / r;
}

// The dynamic shared-memory limit is a per-device function attribute.
int poisson_prepare_device() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  GPL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return GPL_ERR_INVALID_ARG; }
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return GPL_OK;
  const int big = 200 * 1024;
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_a, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_b, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_c, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_cols_w<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_cols_w<1024>()));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_field_w<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_field_w<1024>()));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_cols_w<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_cols_w<512>()));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_field_w<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_field_w<512>()));
  for (int n : {1024, 512}) {
    // the warp form's twiddles, [k2 * 32 + n1] = exp(-2 pi i n1 k2 / n)
    std::vector<float2> t(n);
    for (int k2 = 0; k2 < n / 32; k2++)
      for (int n1 = 0; n1 < 32; n1++) {
        const double a = -2.0 * M_PI * (double)(n1 * k2) / (double)n;
        t[k2 * 32 + n1] = make_float2((float)cos(a), (float)sin(a));
      }
    if (n == 1024) GPL_CUDA(cudaMemcpyToSymbol(g_tw1024, t.data(), n * sizeof(float2)));
    else GPL_CUDA(cudaMemcpyToSymbol(g_tw512, t.data(), n * sizeof(float2)));
  }
  done[dev] = true;
  return GPL_OK;
}

namespace {
// Passes B and C of the block form, with the grids and dynamic shared memory
// of passes A, B and C.
void block_form_bc(const PoissonGrid& g, float* spec, float* p1, float* p2, float2* field, float* fx,
                   float* fy, float* phi, PassBArgs& B, PassCArgs& C, int grid[3], size_t smem[3]) {
  const int nx = g.nx, ny = g.ny;
  B.nx = nx; B.ny = ny; B.logn = ilog2(ny); B.col_pairs = pairs_b(nx, ny);
  B.spec = spec; B.p1 = p1; B.p2 = p2; B.wx = g.wx; B.wy = g.wy; B.tw = g.tw; B.w4 = g.w4y;
  B.scale = 4.0f / (float)nx / (float)ny;
  C.nx = nx; C.ny = ny; C.logn = ilog2(nx); C.pairs_per_block = pairs_c(nx, ny);
  C.p1 = p1; C.p2 = p2; C.field = field; C.fx = fx; C.fy = fy; C.phi = phi;
  C.wx = g.wx; C.tw = g.tw; C.w4 = g.w4x;
  grid[0] = poisson_blocks_a(nx, ny);
  grid[1] = nx / (2 * B.col_pairs);
  grid[2] = (ny / 2 + C.pairs_per_block - 1) / C.pairs_per_block;
  smem[0] = smem_a(nx, ny);
  smem[1] = smem_b(nx, ny);
  smem[2] = smem_c(nx, ny);
}

PassAArgs pass_a_args(const PoissonGrid& g, unsigned long long* const* area_pair, const EvalCtl* ctl,
                      const int64_t* nonplace, float td, const float* density_in, float* density,
                      double* part_overflow, float* spec) {
  PassAArgs A;
  A.nx = g.nx; A.ny = g.ny; A.logn = ilog2(g.nx); A.pairs_per_block = pairs_a(g.nx, g.ny);
  A.core_lx = g.core_lx; A.core_ly = g.core_ly; A.core_ux = g.core_ux; A.core_uy = g.core_uy;
  A.size_x = g.size_x; A.size_y = g.size_y; A.td = td;
  A.area_pair[0] = area_pair ? area_pair[0] : nullptr;
  A.area_pair[1] = area_pair ? area_pair[1] : nullptr;
  A.ctl = ctl; A.nonplace = nonplace;
  A.density_in = density_in; A.density = density; A.spec = spec;
  A.part_overflow = part_overflow; A.tw = g.tw; A.w4 = g.w4x;
  return A;
}

PoissonGrid job_grid(const DeviceModel& d) {
  PoissonGrid g;
  g.nx = d.cnt_x; g.ny = d.cnt_y; g.size_x = d.size_x; g.size_y = d.size_y;
  g.core_lx = d.core_lx; g.core_ly = d.core_ly; g.core_ux = d.core_ux; g.core_uy = d.core_uy;
  g.wx = d.wx; g.wy = d.wy; g.w4x = d.w4x; g.w4y = d.w4y; g.tw = d.twiddle;
  return g;
}

// Batched form of the block passes: work items (instance, block); each
// block runs the per-job kernel's body on its instance's arguments.
__global__ void __launch_bounds__(256) k_poisson_a_batch(const PassAArgs* args, const int4* items, const int* count) {
  extern __shared__ float2 smem[];
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    poisson_a_body(args[it.x], it.y, smem);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_poisson_b_batch(const PassBArgs* args, const int4* items, const int* count) {
  extern __shared__ float2 smem[];
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    poisson_b_body(args[it.x], it.y, smem);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_poisson_c_batch(const PassCArgs* args, const int4* items, const int* count) {
  extern __shared__ float2 smem[];
  const int n = *count;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {
    const int4 it = items[w];
    poisson_c_body(args[it.x], it.y, smem);
    __syncthreads();
  }
}
}  // namespace

size_t poisson_batch_args_bytes(int pass) {
  // the element size of the device arrays the batched kernels index
  return pass == 0 ? sizeof(PassAArgs) : pass == 1 ? sizeof(PassBArgs) : sizeof(PassCArgs);
}

bool write_poisson_batch_args(const DeviceModel& d, void* dst_a, void* dst_b, void* dst_c, int grid[3],
                              size_t smem[3]) {
  if (d.poisson_path != 1 || warp_form(d.cnt_x, d.cnt_y)) return false;
  const PoissonGrid g = job_grid(d);
  const PassAArgs A = pass_a_args(g, d.area, d.ctl, d.nonplace, d.target_density, nullptr, d.density,
                                  d.part + (size_t)kPartOverflow * d.part_stride, d.spec);
  PassBArgs B;
  PassCArgs C;
  block_form_bc(g, d.spec, d.p1, d.p2, d.field, nullptr, nullptr, nullptr, B, C, grid, smem);
  memcpy(dst_a, &A, sizeof(A));
  memcpy(dst_b, &B, sizeof(B));
  memcpy(dst_c, &C, sizeof(C));
  return true;
}

int poisson_batch_prepare_device() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  GPL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return GPL_ERR_INVALID_ARG; }
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return GPL_OK;
  const int big = 200 * 1024;
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_a_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_b_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  GPL_CUDA(cudaFuncSetAttribute(k_poisson_c_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
  done[dev] = true;
  return GPL_OK;
}

int launch_poisson_batch(int pass, const void* args, const int4* items, const int* count, int grid, size_t smem,
                         cudaStream_t s) {
  if (pass == 0) k_poisson_a_batch<<<grid, 256, smem, s>>>(static_cast<const PassAArgs*>(args), items, count);
  else if (pass == 1) k_poisson_b_batch<<<grid, 256, smem, s>>>(static_cast<const PassBArgs*>(args), items, count);
  else k_poisson_c_batch<<<grid, 256, smem, s>>>(static_cast<const PassCArgs*>(args), items, count);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

// The three passes on arbitrary device arrays.  Area mode (area != null):
// the density comes from the int64 areas; otherwise from density_in.
int poisson_passes(const PoissonGrid& g, unsigned long long* const* area_pair,
                   const EvalCtl* ctl, const int64_t* nonplace, float td,
                   const float* density_in, float* density, double* part_overflow,
                   float* spec, float* p1, float* p2, float2* field, float* fx, float* fy,
                   float* phi, cudaStream_t s, Timer* t) {
  int rc = poisson_prepare_device();
  if (rc) return rc;
  const int nx = g.nx, ny = g.ny;
  const PassAArgs A = pass_a_args(g, area_pair, ctl, nonplace, td, density_in, density, part_overflow, spec);
  if (const int wn = warp_form(nx, ny)) {
    const bool areas = area_pair && ctl;
    PassBArgs B;
    B.nx = nx; B.ny = ny; B.logn = ilog2(ny);
    B.spec = spec; B.p1 = p1; B.p2 = p2; B.wx = g.wx; B.wy = g.wy; B.tw = g.tw; B.w4 = g.w4y;
    B.scale = 4.0f / (float)nx / (float)ny;
    PassCArgs C;
    C.nx = nx; C.ny = ny; C.logn = ilog2(nx); C.pairs_per_block = kWFieldPairs;
    C.p1 = p1; C.p2 = p2; C.field = field; C.fx = fx; C.fy = fy; C.phi = phi;
    C.wx = g.wx; C.tw = g.tw; C.w4 = g.w4x;
    if (t) t->begin(kKPoissonA);
    if (areas) k_poisson_dens<<<poisson_blocks_a(nx, ny), 256, 0, s>>>(A);
    if (wn == 1024) k_poisson_rows_w<1024><<<ny / 2, 32, smem_rows_w<1024>(), s>>>(A);
    else k_poisson_rows_w<512><<<ny / 2, 32, smem_rows_w<512>(), s>>>(A);
    if (t) t->end(kKPoissonA);
    if (t) t->begin(kKPoissonB);
    if (wn == 1024) {
      B.col_pairs = ColsShape<1024>::kP;
      k_poisson_cols_w<1024><<<nx / (2 * ColsShape<1024>::kP), ColsShape<1024>::kThreads,
                               smem_cols_w<1024>(), s>>>(B);
    } else {
      B.col_pairs = ColsShape<512>::kP;
      k_poisson_cols_w<512><<<nx / (2 * ColsShape<512>::kP), ColsShape<512>::kThreads,
                              smem_cols_w<512>(), s>>>(B);
    }
    if (t) t->end(kKPoissonB);
    if (t) t->begin(kKPoissonC);
    if (wn == 1024) k_poisson_field_w<1024><<<ny / 2 / kWFieldPairs, kWFieldThreads, smem_field_w<1024>(), s>>>(C);
    else k_poisson_field_w<512><<<ny / 2 / kWFieldPairs, kWFieldThreads, smem_field_w<512>(), s>>>(C);
    if (t) t->end(kKPoissonC);
    if (t) t->count(areas ? 4 : 3);
    GPL_CUDA(cudaGetLastError());
    return GPL_OK;
  }
  PassBArgs B;
  PassCArgs C;
  int grid[3];
  size_t smem[3];
  block_form_bc(g, spec, p1, p2, field, fx, fy, phi, B, C, grid, smem);
  if (t) t->begin(kKPoissonA);
  k_poisson_a<<<grid[0], 256, smem[0], s>>>(A);
  if (t) t->end(kKPoissonA);
  if (t) t->begin(kKPoissonB);
  k_poisson_b<<<grid[1], 256, smem[1], s>>>(B);
  if (t) t->end(kKPoissonB);
  if (t) t->begin(kKPoissonC);
  k_poisson_c<<<grid[2], 256, smem[2], s>>>(C);
  if (t) t->end(kKPoissonC);
  if (t) t->count(3);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

int launch_poisson_job(DeviceModel& d, bool want_phi, cudaStream_t s, Timer& t) {
  if (d.poisson_path == 2 && d.pg) return launch_poisson_gemm(d, d.pg, want_phi, s, t);
  const PoissonGrid g = job_grid(d);
  return poisson_passes(g, d.area, d.ctl, d.nonplace, d.target_density, nullptr, d.density,
                        d.part + (size_t)kPartOverflow * d.part_stride, d.spec, d.p1, d.p2,
                        d.field, nullptr, nullptr, want_phi ? d.phi : nullptr, s, &t);
}

void make_w4(int n, std::vector<float2>& w) {
  w.resize(n);
  for (int k = 0; k < n; k++) {
    double a = -M_PI * (double)k / (2.0 * n);
    w[k] = make_float2((float)cos(a), (float)sin(a));
  }
}

// Scratch and tables of the standalone solve, cached per (device, grid).
namespace {
struct SolveCache {
  int device = -1, nx = 0, ny = 0, bsx = 0, bsy = 0;
  unsigned long long ctx = 0;   // context the memory belongs to
  char* mem = nullptr;
  float *spec = nullptr, *p1 = nullptr, *p2 = nullptr, *wx = nullptr, *wy = nullptr;
  float2 *w4x = nullptr, *w4y = nullptr, *tw = nullptr;
};
std::mutex g_cache_mu;
std::vector<std::unique_ptr<SolveCache>> g_cache;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
}  // namespace

unsigned long long current_context_id() {
  static CtxGetCurrentFn get_cur = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_cur || !get_id || get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

}  // namespace gpl

using namespace gpl;

extern "C" gpl_status gpl_poisson_solve(int32_t nx, int32_t ny, int32_t bsx, int32_t bsy,
                                        const float* density, float* phi, float* fx, float* fy,
                                        void* stream) {
  auto pow2 = [](int v) { return v >= 2 && v <= kFftMax && (v & (v - 1)) == 0; };
  if (!pow2(nx) || !pow2(ny) || bsx <= 0 || bsy <= 0 || !density || !fx || !fy) {
    set_error("gpl_poisson_solve: sizes must be powers of two in [2, 4096], bin sizes positive, "
              "density/field pointers non-null");
    return GPL_ERR_INVALID_ARG;
  }
  int dev = 0;
  GPL_CUDA(cudaGetDevice(&dev));
  GPL_CUDA(cudaSetDevice(dev));         // initialises the device's context if needed
  const unsigned long long ctx = current_context_id();
  cudaStream_t s = (cudaStream_t)stream;
  SolveCache* c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    // entries of a context that no longer exists (cudaDeviceReset) hold
    // memory that went with it: forget them without freeing
    for (auto& e : g_cache)
      if (e && e->device == dev && e->ctx != ctx) e.reset();
    g_cache.erase(std::remove(g_cache.begin(), g_cache.end(), nullptr), g_cache.end());
    for (auto& e : g_cache)
      if (e->device == dev && e->nx == nx && e->ny == ny && e->bsx == bsx && e->bsy == bsy) c = e.get();
    if (!c) {
      SolveCache e;
      e.device = dev; e.ctx = ctx; e.nx = nx; e.ny = ny; e.bsx = bsx; e.bsy = bsy;
      const size_t nb = (size_t)nx * ny;
      size_t bytes = 3 * nb * 4 + (nx + ny) * 4 + (nx + ny) * 8 + (kFftMax / 2) * 8 + 8 * 256;
      GPL_CUDA(cudaMalloc(&e.mem, bytes));
      char* q = e.mem;
      auto take = [&](size_t b) { char* r = q; q += ((b + 255) / 256) * 256; return r; };
      e.spec = (float*)take(nb * 4); e.p1 = (float*)take(nb * 4); e.p2 = (float*)take(nb * 4);
      e.wx = (float*)take(nx * 4); e.wy = (float*)take(ny * 4);
      e.w4x = (float2*)take(nx * 8); e.w4y = (float2*)take(ny * 8);
      e.tw = (float2*)take((kFftMax / 2) * 8);
      std::vector<float2> tw, w4x, w4y;
      std::vector<float> wx, wy;
      make_twiddle(tw); make_w4(nx, w4x); make_w4(ny, w4y); make_freq(nx, ny, bsx, bsy, wx, wy);
      GPL_CUDA(cudaMemcpy(e.wx, wx.data(), nx * 4, cudaMemcpyHostToDevice));
      GPL_CUDA(cudaMemcpy(e.wy, wy.data(), ny * 4, cudaMemcpyHostToDevice));
      GPL_CUDA(cudaMemcpy(e.w4x, w4x.data(), nx * 8, cudaMemcpyHostToDevice));
      GPL_CUDA(cudaMemcpy(e.w4y, w4y.data(), ny * 8, cudaMemcpyHostToDevice));
      GPL_CUDA(cudaMemcpy(e.tw, tw.data(), tw.size() * 8, cudaMemcpyHostToDevice));
      g_cache.emplace_back(new SolveCache(e));
      c = g_cache.back().get();
    }
  }
  PoissonGrid g;
  g.nx = nx; g.ny = ny; g.size_x = bsx; g.size_y = bsy;
  g.core_lx = g.core_ly = 0; g.core_ux = nx * bsx; g.core_uy = ny * bsy;
  g.wx = c->wx; g.wy = c->wy; g.w4x = c->w4x; g.w4y = c->w4y; g.tw = c->tw;
  int rc = poisson_passes(g, nullptr, nullptr, nullptr, 1.0f, density, nullptr, nullptr, c->spec,
                          c->p1, c->p2, nullptr, fx, fy, phi, s, nullptr);
  return (gpl_status)rc;
}
