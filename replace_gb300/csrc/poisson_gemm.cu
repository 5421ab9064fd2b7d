// The Poisson solve of updateDensityForceBin (src/nesterovBase.cpp:1481-1506,
// src/fft.cpp:112-177) as dense transforms on the tensor cores: every 1-D
// DCT-II / DCT-III / DST of the solve is a product with a constant n x n
// matrix, computed by the tcgen05 GEMM (tc_gemm.cuh) in bf16 with a
// three-term split: x = x0 + x1 + x2 (bf16 each, 24 significant bits in
// all: x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1), both
// differences exact in fp32), and
//   A * B ~ a0 b0 + a0 b1 + a0 b2 + a1 b0 + a1 b1 + a2 b0,
// the six products of order <= 2, as one GEMM over K' = 6K with A stored as
// [a2 | a1 | a1 | a0 | a0 | a0] and B as [b0 | b1 | b0 | b2 | b1 | b0] along
// K, accumulated in fp32.  The dropped terms are near 2^-24 of each product.
// The order matters: the tensor core's fp32 accumulation truncates, with an
// error that grows with the accumulated length and the accumulator's size
// (measured: 3e-7 relative at K = 256, 1.7e-6 at 1024, 2.3e-5 at 6144).
// The small products go first, while the accumulator is small, and the
// leading a0 b0 block last, so the result's error is about that of one
// K-long product (a first layout with a0 b0 first gave 5e-5 on the field at
// 1024 x 1024).  Data layout, with rows listed first (D = A * B^T):
//   G1  T[j][u]   = rho[j][.]  . C2x[u][.]         density rows, DCT-II along x
//   G2  S[u][v]   = T^T[u][.]  . C2y[v][.]         DCT-II along y -> spectrum^T;
//                                                  the epilogue solves and
//                                                  stores phi^T
//   G34 P[y'][u]  = [C3y; SWy][y'][.] . phi^T[u][.] DCT-III and wy-weighted DST
//                                                  along y (P1 and P2 stacked)
//   G6  Ex[y][x]  = P1[y][.] . SWx[x][.]           wx-weighted DST along x
//   G7  Ey[y][x]  = P2[y][.] . C3x[x][.]           DCT-III along x
//   G5  phi[y][x] = P1[y][.] . C3x[x][.]           (only when phi is wanted)
// The x-field's y-transform is P1 scaled by wx[u] (wx depends on u only), so
// its weight moves into SWx and no GEMM of its own is needed.
#include <cuda_bf16.h>

#include <memory>

#include "device_common.cuh"
#include "gpl_internal.h"
#include "tc_gemm.cuh"

namespace gpl {

namespace {

constexpr int kPgThreads = 256;

// Terms of the split along K (operand width kSplit * k for k values):
// 6 = three bf16 terms per value and the six products of order <= 2;
// 3 = two terms per value (hi, lo) and the products hi hi, hi lo, lo hi.
#ifndef GPL_PG_SPLIT
#define GPL_PG_SPLIT 6
#endif
constexpr int kSplit = GPL_PG_SPLIT;

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& t0, __nv_bfloat16& t1, __nv_bfloat16& t2) {
  t0 = __float2bfloat16_rn(x);
  const float r1 = __fsub_rn(x, __bfloat162float(t0));      // exact
  t1 = __float2bfloat16_rn(r1);
  t2 = __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(t1)));
}

// Column c of a split operand row of width k, smallest products first.
// kSplit 6: A [t2 | t1 | t1 | t0 | t0 | t0], B [t0 | t1 | t0 | t2 | t1 | t0]
// (products t2 t0, t1 t1, t1 t0, t0 t2, t0 t1, t0 t0).  kSplit 3: A
// [t1 | t0 | t0], B [t0 | t1 | t0] (t1 t0, t0 t1, t0 t0).
__device__ __forceinline__ void put_a(__nv_bfloat16* row, int k, int c, float x) {
  __nv_bfloat16 t0, t1, t2;
  split_bf16(x, t0, t1, t2);
  if constexpr (kSplit == 6) {
    row[c] = t2; row[k + c] = t1; row[2 * k + c] = t1;
    row[3 * k + c] = t0; row[4 * k + c] = t0; row[5 * k + c] = t0;
  } else {
    row[c] = t1; row[k + c] = t0; row[2 * k + c] = t0;
  }
}
__device__ __forceinline__ void put_b(__nv_bfloat16* row, int k, int c, float x) {
  __nv_bfloat16 t0, t1, t2;
  split_bf16(x, t0, t1, t2);
  if constexpr (kSplit == 6) {
    row[c] = t0; row[k + c] = t1; row[2 * k + c] = t0;
    row[3 * k + c] = t2; row[4 * k + c] = t1; row[5 * k + c] = t0;
  } else {
    row[c] = t0; row[k + c] = t1; row[2 * k + c] = t0;
  }
}

// Constant matrices, evaluated in double with exact argument reduction:
// kind 0 C2[m][k] = cos(pi (k + 1/2) m / n), 1 C3[m][k] = cos(pi k (m + 1/2) / n),
// 2 S[m][k] = sin(pi k (m + 1/2) / n) * w[k] (k >= 1; 0 for k = 0).
__global__ void k_pg_matrix(__nv_bfloat16* out, int rows, int n, int kind, int pattern, const float* w,
                            int row0) {
  const size_t total = (size_t)rows * n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / n), k = (int)(t - (size_t)m * n);
    long long num;
    if (kind == 0) num = (long long)(2 * k + 1) * m;
    else num = (long long)k * (2 * m + 1);
    num %= 4ll * n;                                 // angle = pi * num / (2n), period 2 pi
    double s, c;
    sincospi((double)num / (2.0 * n), &s, &c);
    double v = kind == 2 ? (k ? s * (double)w[k] : 0.0) : c;
    __nv_bfloat16* row = out + (size_t)(row0 + m) * kSplit * n;
    if (pattern == 0) put_a(row, n, k, (float)v);
    else put_b(row, n, k, (float)v);
  }
}

struct PgArgs {
  int nx, ny;
  int core_lx, core_ly, core_ux, core_uy, size_x, size_y;
  float td;
  unsigned long long* area_pair[2];
  const EvalCtl* ctl;
  const int64_t* nonplace;
  float* density;
  double* part_overflow;
  __nv_bfloat16* rho_a;       // [ny][kSplit nx]
};

// Density of every bin from the int64 areas (as pass A of the FFT path),
// FP64 overflow partials (one per block), the other area set cleared, and
// the density rows written as the first GEMM's A operand.
__global__ void __launch_bounds__(kPgThreads) k_pg_density(PgArgs A) {
  __shared__ double red[32];
  const int nb = A.nx * A.ny;
  const int cur = A.ctl->area_cur;
  const unsigned long long* __restrict__ ar = cur == 0 ? A.area_pair[0] : A.area_pair[1];
  unsigned long long* __restrict__ ac = cur == 0 ? A.area_pair[1] : A.area_pair[0];
  float ovf = 0.0f;
  for (int b = blockIdx.x * kPgThreads + threadIdx.x; b < nb; b += gridDim.x * kPgThreads) {
    const int j = b / A.nx, i = b - j * A.nx;
    const int blx = A.core_lx + i * A.size_x, bux = min(blx + A.size_x, A.core_ux);
    const int bly = A.core_ly + j * A.size_y, buy = min(bly + A.size_y, A.core_uy);
    const long long bin_area = (long long)(bux - blx) * (long long)(buy - bly);
    const float cap = __fmul_rn(ll_to_float(bin_area), A.td);
    const float fi = ll_to_float((long long)ar[b]);
    const float ff = ll_to_float((long long)ar[nb + b]);
    const float fn = ll_to_float(A.nonplace[b]);
    // BinGrid::updateBinsGCellDensityArea (src/nesterovBase.cpp:804-818)
    const float d = __fdiv_rn(__fadd_rn(__fadd_rn(fi, ff), fn), cap);
    ovf += fmaxf(0.0f, __fsub_rn(__fadd_rn(fi, fn), cap));
    ac[b] = 0ull;
    ac[nb + b] = 0ull;
    A.density[b] = d;
    // The transforms take d - 1: a constant changes only the (0, 0)
    // coefficient, which the solve sets to zero, and the density's mean is
    // close to 1 (the fillers fill the free space to the target density), so
    // the sums the tensor cores accumulate -- and their truncation error --
    // shrink to the density's fluctuations.
    put_a(A.rho_a + (size_t)j * kSplit * A.nx, A.nx, i, __fsub_rn(d, 1.0f));
  }
  double v = ovf;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kPgThreads / 32; w++) t += red[w];
    A.part_overflow[blockIdx.x] = t;
  }
}

// G1 epilogue: T[j][u0 + t] -> T^T[u][j] as an A operand (rows u, width ny);
// each thread's row j is a column of the output, so the lanes' stores of one
// output row are consecutive.
struct EpiT {
  static constexpr bool kRowMajor = false;
  __nv_bfloat16* out;
  int ny;
  __device__ __forceinline__ void operator()(int j, int u0, const float (&v)[32]) const {
#pragma unroll
    for (int t = 0; t < 32; t++) put_a(out + (size_t)(u0 + t) * kSplit * ny, ny, j, v[t]);
  }
};

// G2 epilogue: the spectral solve of FFT::doFFT (src/fft.cpp:117-166) on
// S[u][v] (x frequency u, y frequency v), stored as phi^T[u][v], a B operand.
struct EpiS {
  static constexpr bool kRowMajor = true;
  __nv_bfloat16* out;
  int nx, ny;
  const float* wx;
  const float* wy;
  float scale;
  __device__ __forceinline__ void at(int u, int vv, float s) const {
    float d = s;
    if (u == 0) d *= 0.5f;
    if (vv == 0) d *= 0.5f;
    d *= scale;
    float ph = 0.0f;
    if (u != 0 || vv != 0) {
      const float wxu = __ldg(wx + u), wyv = __ldg(wy + vv);
      ph = __fdiv_rn(d, __fadd_rn(__fmul_rn(wxu, wxu), __fmul_rn(wyv, wyv)));
    }
    put_b(out + (size_t)u * kSplit * ny, ny, vv, ph);
  }
};

// G34 epilogue: P[y'][u] stored as an A operand (rows y', width nx).
struct EpiP {
  static constexpr bool kRowMajor = true;
  __nv_bfloat16* out;
  int nx;
  __device__ __forceinline__ void at(int y, int u, float v) const { put_a(out + (size_t)y * kSplit * nx, nx, u, v); }
};

// G5/G6/G7 epilogue: one component of the field (or phi) at [y][x].
struct EpiF {
  static constexpr bool kRowMajor = true;
  float* base;        // field as floats (component c of bin b at 2 b + c), or phi
  int nx, stride, comp;
  __device__ __forceinline__ void at(int y, int x, float v) const {
    base[((size_t)y * nx + x) * stride + comp] = v;
  }
};

}  // namespace

// Per-job state of the GEMM path: operands and prepared GEMM plans.
struct PoissonGemm {
  int nx = 0, ny = 0;
  char* mem = nullptr;
  size_t bytes = 0;
  __nv_bfloat16 *c2x, *c2y, *a34, *swx, *c3x;     // constants
  __nv_bfloat16 *rho, *txt, *phit, *p12;          // data
  int* err = nullptr;
  tc::TcPlan<64, EpiT> g1;
  tc::TcPlan<64, EpiS> g2;
  tc::TcPlan<128, EpiP> g34;   // M = 2 ny: 128-wide N tiles keep it to one wave
  tc::TcPlan<64, EpiF> g6, g7, g5;
};

bool poisson_gemm_eligible(int nx, int ny) {
  return nx >= 128 && ny >= 128 && nx % 128 == 0 && ny % 128 == 0 && nx <= kFftMax && ny <= kFftMax;
}

void poisson_gemm_free(PoissonGemm* pg, cudaMemPool_t pool, cudaStream_t s) {
  if (!pg) return;
  dev_free(pg->mem, pool, s);
  delete pg;
}

int64_t poisson_gemm_bytes(int nx, int ny) {
  const size_t xk = kSplit * (size_t)nx, yk = kSplit * (size_t)ny;
  size_t b = 0;
  b += (size_t)nx * xk + (size_t)ny * yk + 2 * (size_t)ny * yk + 2 * (size_t)nx * xk;   // constants
  b += (size_t)ny * xk + (size_t)nx * yk + (size_t)nx * yk + 2 * (size_t)ny * xk;       // data
  return (int64_t)(b * 2 + 16 * 256);
}

// Builds the constant operands and the GEMM plans for the job's grid.
int poisson_gemm_setup(DeviceModel& d, PoissonGemm** out, cudaMemPool_t pool, cudaStream_t s) {
  *out = nullptr;
  const int nx = d.cnt_x, ny = d.cnt_y;
  if (!poisson_gemm_eligible(nx, ny)) { set_error("GEMM Poisson path: grid not eligible"); return GPL_ERR_INVALID_ARG; }
  std::unique_ptr<PoissonGemm> pg(new PoissonGemm());
  pg->nx = nx; pg->ny = ny;
  const size_t xk = kSplit * (size_t)nx, yk = kSplit * (size_t)ny;
  pg->bytes = (size_t)poisson_gemm_bytes(nx, ny);
  cudaError_t e = dev_alloc((void**)&pg->mem, pg->bytes, pool, s);
  if (e != cudaSuccess) { cudaGetLastError(); set_error("GEMM Poisson path: device allocation failed"); return GPL_ERR_OUT_OF_MEMORY; }
  char* cur = pg->mem;
  auto take = [&](size_t elems) {
    __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(cur);
    cur += (elems * 2 + 255) / 256 * 256;
    return p;
  };
  pg->c2x = take((size_t)nx * xk);
  pg->c2y = take((size_t)ny * yk);
  pg->a34 = take(2 * (size_t)ny * yk);
  pg->swx = take((size_t)nx * xk);
  pg->c3x = take((size_t)nx * xk);
  pg->rho = take((size_t)ny * xk);
  pg->txt = take((size_t)nx * yk);
  pg->phit = take((size_t)nx * yk);
  pg->p12 = take(2 * (size_t)ny * xk);
  pg->err = reinterpret_cast<int*>(cur);
  GPL_CUDA(cudaMemsetAsync(pg->err, 0, sizeof(int), s));
  const int grid = 4 * std::max(d.sm_count, 1);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->c2x, nx, nx, 0, 1, nullptr, 0);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->c2y, ny, ny, 0, 1, nullptr, 0);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->a34, ny, ny, 1, 0, nullptr, 0);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->a34, ny, ny, 2, 0, d.wy, ny);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->swx, nx, nx, 2, 1, d.wx, 0);
  k_pg_matrix<<<grid, kPgThreads, 0, s>>>(pg->c3x, nx, nx, 1, 1, nullptr, 0);
  GPL_CUDA(cudaGetLastError());
  int rc = pg->g1.prepare(pg->rho, (int)xk, pg->c2x, (int)xk, ny, nx, (int)xk);
  if (!rc) rc = pg->g2.prepare(pg->txt, (int)yk, pg->c2y, (int)yk, nx, ny, (int)yk);
  if (!rc) rc = pg->g34.prepare(pg->a34, (int)yk, pg->phit, (int)yk, 2 * ny, nx, (int)yk);
  if (!rc) rc = pg->g6.prepare(pg->p12, (int)xk, pg->swx, (int)xk, ny, nx, (int)xk);
  if (!rc) rc = pg->g7.prepare(pg->p12 + (size_t)ny * xk, (int)xk, pg->c3x, (int)xk, ny, nx, (int)xk);
  if (!rc) rc = pg->g5.prepare(pg->p12, (int)xk, pg->c3x, (int)xk, ny, nx, (int)xk);
  if (rc) { dev_free(pg->mem, pool, s); pg->mem = nullptr; return rc; }
  *out = pg.release();
  return GPL_OK;
}

int poisson_gemm_error(const PoissonGemm* pg, cudaStream_t s, int* flag) {
  *flag = 0;
  if (!pg) return GPL_OK;
  GPL_CUDA(cudaMemcpyAsync(flag, pg->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GPL_CUDA(cudaStreamSynchronize(s));
  return GPL_OK;
}

// One solve on the job's buffers (same inputs and outputs as the FFT
// passes of launch_poisson_job).
int launch_poisson_gemm(DeviceModel& d, PoissonGemm* pg, bool want_phi, cudaStream_t s, Timer& t) {
  const int nx = d.cnt_x, ny = d.cnt_y;
  PgArgs A;
  A.nx = nx; A.ny = ny;
  A.core_lx = d.core_lx; A.core_ly = d.core_ly; A.core_ux = d.core_ux; A.core_uy = d.core_uy;
  A.size_x = d.size_x; A.size_y = d.size_y; A.td = d.target_density;
  A.area_pair[0] = d.area[0]; A.area_pair[1] = d.area[1];
  A.ctl = d.ctl; A.nonplace = d.nonplace; A.density = d.density;
  A.part_overflow = d.part + (size_t)kPartOverflow * d.part_stride;
  A.rho_a = pg->rho;
  t.begin(kKPoissonA);
  k_pg_density<<<poisson_blocks_a(nx, ny), kPgThreads, 0, s>>>(A);
  pg->g1.launch(EpiT{pg->txt, ny}, pg->err, s);
  t.end(kKPoissonA);
  t.begin(kKPoissonB);
  pg->g2.launch(EpiS{pg->phit, nx, ny, d.wx, d.wy, 4.0f / (float)nx / (float)ny}, pg->err, s);
  pg->g34.launch(EpiP{pg->p12, nx}, pg->err, s);
  t.end(kKPoissonB);
  t.begin(kKPoissonC);
  float* field = reinterpret_cast<float*>(d.field);
  pg->g6.launch(EpiF{field, nx, 2, 0}, pg->err, s);
  pg->g7.launch(EpiF{field, nx, 2, 1}, pg->err, s);
  if (want_phi) pg->g5.launch(EpiF{d.phi, nx, 1, 0}, pg->err, s);
  t.end(kKPoissonC);
  t.count(want_phi ? 7 : 6);
  GPL_CUDA(cudaGetLastError());
  return GPL_OK;
}

}  // namespace gpl
