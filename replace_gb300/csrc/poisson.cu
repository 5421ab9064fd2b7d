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
#include <cuda_runtime.h>

#include <cmath>
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

__global__ void __launch_bounds__(256) k_poisson_a(PassAArgs A) {
  extern __shared__ float2 smem[];
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
      const int r = blockIdx.x * rp_n + rp;
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
      const int r = blockIdx.x * rp_n + rp;
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
    const int r = blockIdx.x * rp_n + rp;
    if (r >= A.ny / 2) continue;
    const float2* z = res + rp * n;
    float2 c = dct2_post(z[k], z[(n - k) & (n - 1)], __ldg(&A.w4[k]));
    A.spec[(2 * r) * n + k] = c.x;
    A.spec[(2 * r + 1) * n + k] = c.y;
  }
  if (A.part_overflow) block_reduce_add((double)ovf_f, &A.part_overflow[blockIdx.x], red);
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

__global__ void __launch_bounds__(256) k_poisson_b(PassBArgs B) {
  extern __shared__ float2 smem[];
  const int n = B.ny;
  const int cp = B.col_pairs;
  float2* s0 = smem;                 // [cp][n] work
  float2* s1 = smem + cp * n;        // [cp][n] scratch
  float2* s2 = smem + 2 * cp * n;    // [cp][n] spectrum: (phi^ col u0, phi^ col u1)
  float2* tws = smem + 3 * cp * n;   // [n/2] twiddles
  load_twiddles(tws, B.tw, n);
  const int u_base = blockIdx.x * 2 * cp;
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

__global__ void __launch_bounds__(256) k_poisson_c(PassCArgs C) {
  extern __shared__ float2 smem[];
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
    const int r = blockIdx.x * rp_n + rp;
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
      const int r = blockIdx.x * rp_n + rp;
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

int poisson_blocks_a(int nx, int ny) { int r = pairs_a(nx, ny); return (ny / 2 + r - 1) / r; }

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
  done[dev] = true;
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
  PassAArgs A;
  A.nx = nx; A.ny = ny; A.logn = ilog2(nx); A.pairs_per_block = pairs_a(nx, ny);
  A.core_lx = g.core_lx; A.core_ly = g.core_ly; A.core_ux = g.core_ux; A.core_uy = g.core_uy;
  A.size_x = g.size_x; A.size_y = g.size_y; A.td = td;
  A.area_pair[0] = area_pair ? area_pair[0] : nullptr;
  A.area_pair[1] = area_pair ? area_pair[1] : nullptr;
  A.ctl = ctl; A.nonplace = nonplace;
  A.density_in = density_in; A.density = density; A.spec = spec;
  A.part_overflow = part_overflow; A.tw = g.tw; A.w4 = g.w4x;
  if (t) t->begin(kKPoissonA);
  k_poisson_a<<<poisson_blocks_a(nx, ny), 256, smem_a(nx, ny), s>>>(A);
  if (t) t->end(kKPoissonA);
  PassBArgs B;
  B.nx = nx; B.ny = ny; B.logn = ilog2(ny); B.col_pairs = pairs_b(nx, ny);
  B.spec = spec; B.p1 = p1; B.p2 = p2; B.wx = g.wx; B.wy = g.wy; B.tw = g.tw; B.w4 = g.w4y;
  B.scale = 4.0f / (float)nx / (float)ny;
  if (t) t->begin(kKPoissonB);
  k_poisson_b<<<nx / (2 * B.col_pairs), 256, smem_b(nx, ny), s>>>(B);
  if (t) t->end(kKPoissonB);
  PassCArgs C;
  C.nx = nx; C.ny = ny; C.logn = ilog2(nx); C.pairs_per_block = pairs_c(nx, ny);
  C.p1 = p1; C.p2 = p2; C.field = field; C.fx = fx; C.fy = fy; C.phi = phi;
  C.wx = g.wx; C.tw = g.tw; C.w4 = g.w4x;
  if (t) t->begin(kKPoissonC);
  k_poisson_c<<<(ny / 2 + C.pairs_per_block - 1) / C.pairs_per_block, 256, smem_c(nx, ny), s>>>(C);
  if (t) t->end(kKPoissonC);
  if (t) t->count(3);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

int launch_poisson_job(DeviceModel& d, bool want_phi, cudaStream_t s, Timer& t) {
  if (d.poisson_path == 2 && d.pg) return launch_poisson_gemm(d, d.pg, want_phi, s, t);
  PoissonGrid g;
  g.nx = d.cnt_x; g.ny = d.cnt_y; g.size_x = d.size_x; g.size_y = d.size_y;
  g.core_lx = d.core_lx; g.core_ly = d.core_ly; g.core_ux = d.core_ux; g.core_uy = d.core_uy;
  g.wx = d.wx; g.wy = d.wy; g.w4x = d.w4x; g.w4y = d.w4y; g.tw = d.twiddle;
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
  char* mem = nullptr;
  float *spec = nullptr, *p1 = nullptr, *p2 = nullptr, *wx = nullptr, *wy = nullptr;
  float2 *w4x = nullptr, *w4y = nullptr, *tw = nullptr;
};
std::mutex g_cache_mu;
std::vector<std::unique_ptr<SolveCache>> g_cache;
}  // namespace

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
  cudaStream_t s = (cudaStream_t)stream;
  SolveCache* c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (auto& e : g_cache)
      if (e->device == dev && e->nx == nx && e->ny == ny && e->bsx == bsx && e->bsy == bsy) c = e.get();
    if (!c) {
      SolveCache e;
      e.device = dev; e.nx = nx; e.ny = ny; e.bsx = bsx; e.bsy = bsy;
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
