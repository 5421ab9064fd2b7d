// gpl_oracle.cpp - CPU restatement of RePlAce's global-placement path.
//
// TEST INFRASTRUCTURE ONLY.  This is the checker for the GB300 library: only
// the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
// The product never links, loads or calls it.
//
// It restates, in plain single-threaded C++, the reference's algorithm with
// the reference's arithmetic types (float where the reference uses float,
// the reference's double promotions where they occur, int64 bin areas):
//   PlacerBase bookkeeping          src/placerBase.cpp:606-758
//   NesterovBase init / fillers     src/nesterovBase.cpp:917-1155
//   BinGrid                         src/nesterovBase.cpp:631-868
//   density scatter + overflow      src/nesterovBase.cpp:746-819
//   Poisson solve (FFT::doFFT)      src/fft.cpp:47-177
//   WA wirelength + gradients       src/nesterovBase.cpp:1304-1454
//   density gradient                src/nesterovBase.cpp:1458-1478
//   NesterovPlace                   src/nesterovPlace.cpp:64-607
//   InitialPlace (B2B + BiCGSTAB)   src/initialPlace.cpp:56-385
// Deliberate differences, each stated where it occurs:
//   * the 2-D DCT/DST is computed in FP64 with an FFT of our own (the
//     reference uses Ooura's FP32 split-radix code); results are rounded to
//     float where the reference stores floats;
//   * BiCGSTAB (Eigen, not vendored) is restated from van der Vorst's
//     published algorithm with Eigen's documented stopping rule, FP32 vectors
//     and FP64 inner products.
// Parity of this restatement is pinned against the reference's own code run
// through oracle/refbuild (see tests/test_oracle.py).
#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../include/gpl.h"

namespace {

using std::vector;

const long double kSqrt2 = 1.414213562373095048801L;   // REPLACE_SQRT2
const long double kPi = 3.141592653589793238462L;      // REPLACE_FFT_PI

// ---------------------------------------------------------------- FFT / DCT
// Radix-2 complex FFT in double (sign -1: forward, +1: unnormalised inverse).
struct Fft {
  int n = 0;
  vector<std::complex<double>> tw;   // exp(-2 pi i k / n)
  vector<int> rev;
  void init(int nn) {
    n = nn;
    tw.resize(n / 2 > 0 ? n / 2 : 1);
    for (int k = 0; k < n / 2; k++) {
      double a = -2.0 * M_PI * k / n;
      tw[k] = std::complex<double>(cos(a), sin(a));
    }
    rev.assign(n, 0);
    int lg = 0;
    while ((1 << lg) < n) lg++;
    for (int i = 0; i < n; i++) {
      int r = 0;
      for (int b = 0; b < lg; b++) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
      rev[i] = r;
    }
  }
  void run(std::complex<double>* a, int sign) const {
    for (int i = 0; i < n; i++) if (i < rev[i]) std::swap(a[i], a[rev[i]]);
    for (int len = 2; len <= n; len <<= 1) {
      int step = n / len;
      for (int i = 0; i < n; i += len) {
        for (int k = 0; k < len / 2; k++) {
          std::complex<double> w = tw[k * step];
          if (sign > 0) w = std::conj(w);
          std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
          a[i + k] = u + v;
          a[i + k + len / 2] = u - v;
        }
      }
    }
  }
};

// DCT-II:  C[k] = sum_n x[n] cos(pi (n+1/2) k / N)        (Ooura ddct, isgn=-1)
// DCT-III: y[n] = sum_k a[k] cos(pi k (n+1/2) / N)        (Ooura ddct, isgn=+1)
// IDST:    y[n] = sum_{k=1..N} A[k] sin(pi k (n+1/2) / N), A[N] = a[0]
//                                                          (Ooura ddst, isgn=+1)
// Computed with Makhoul's reordering and an N-point complex FFT.
struct Dct1 {
  int n = 0;
  Fft fft;
  vector<std::complex<double>> buf;
  vector<std::complex<double>> w4;  // exp(-i pi k / (2N))
  void init(int nn) {
    n = nn;
    fft.init(n);
    buf.resize(n);
    w4.resize(n);
    for (int k = 0; k < n; k++) {
      double a = -M_PI * k / (2.0 * n);
      w4[k] = std::complex<double>(cos(a), sin(a));
    }
  }
  void dct2(const double* x, double* out) {
    if (n == 1) { out[0] = x[0]; return; }
    for (int m = 0; m < n / 2; m++) {
      buf[m] = x[2 * m];
      buf[n - 1 - m] = x[2 * m + 1];
    }
    fft.run(buf.data(), -1);
    for (int k = 0; k < n; k++) out[k] = (w4[k] * buf[k]).real();
  }
  void dct3(const double* a, double* out) {
    if (n == 1) { out[0] = a[0]; return; }
    buf[0] = a[0];
    for (int k = 1; k < n; k++)
      buf[k] = 0.5 * std::conj(w4[k]) * std::complex<double>(a[k], -a[n - k]);
    fft.run(buf.data(), +1);
    for (int m = 0; m < n / 2; m++) {
      out[2 * m] = buf[m].real();
      out[2 * m + 1] = buf[n - 1 - m].real();
    }
  }
  // a[0] holds A[N]
  void idst(const double* a, double* out) {
    vector<double> b(n);
    b[0] = 0.0;
    for (int k = 1; k < n; k++) b[k] = a[n - k];
    // A[N] term: sin(pi N (m+1/2)/N) = (-1)^m; folded in after the sign flip
    dct3(b.data(), out);
    for (int m = 0; m < n; m++) {
      double s = (m & 1) ? -1.0 : 1.0;
      out[m] = s * out[m] + a[0] * s;
    }
  }
};

enum Kind1D { K_DCT2, K_DCT3, K_IDST };

// Apply a 1-D transform along x (contiguous, length nx) or y (stride nx).
static void transform_axis(vector<double>& a, int nx, int ny, bool along_x, Kind1D kind) {
  int n = along_x ? nx : ny;
  int count = along_x ? ny : nx;
  Dct1 t;
  t.init(n);
  vector<double> in(n), out(n);
  for (int c = 0; c < count; c++) {
    for (int i = 0; i < n; i++) in[i] = along_x ? a[(size_t)c * nx + i] : a[(size_t)i * nx + c];
    if (kind == K_DCT2) t.dct2(in.data(), out.data());
    else if (kind == K_DCT3) t.dct3(in.data(), out.data());
    else t.idst(in.data(), out.data());
    for (int i = 0; i < n; i++) {
      if (along_x) a[(size_t)c * nx + i] = out[i];
      else a[(size_t)i * nx + c] = out[i];
    }
  }
}

// FFT::doFFT (src/fft.cpp:112-177) in FP64.  Arrays are row-major by y
// (index j * nx + i); x is the reference's first FFT index.
static void poisson_f64(int nx, int ny, int bsx, int bsy, const double* rho,
                        double* phi, double* ex, double* ey) {
  size_t nb = (size_t)nx * ny;
  vector<double> a(rho, rho + nb);
  transform_axis(a, nx, ny, true, K_DCT2);
  transform_axis(a, nx, ny, false, K_DCT2);
  // wx, wy as FFT::init computes them (long double, stored as float)
  vector<float> wx(nx), wy(ny), wx2(nx), wy2(ny);
  for (int i = 0; i < nx; i++) {
    wx[i] = (float)(kPi * (float)i / (float)nx);
    wx2[i] = wx[i] * wx[i];
  }
  for (int j = 0; j < ny; j++) {
    wy[j] = (float)(kPi * (float)j / (float)ny * (float)bsy / (float)bsx);
    wy2[j] = wy[j] * wy[j];
  }
  vector<double> p(nb), fx(nb), fy(nb);
  const double scale = 4.0 / nx / ny;
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      size_t k = (size_t)j * nx + i;
      double d = a[k];
      if (i == 0) d *= 0.5;
      if (j == 0) d *= 0.5;
      d *= scale;
      if (i == 0 && j == 0) {
        p[k] = fx[k] = fy[k] = 0.0;
      } else {
        double ph = d / ((double)wx2[i] + (double)wy2[j]);
        p[k] = ph;
        fx[k] = ph * wx[i];
        fy[k] = ph * wy[j];
      }
    }
  }
  // phi: IDCT in x and y; Ex: IDST in x, IDCT in y; Ey: IDCT in x, IDST in y
  transform_axis(p, nx, ny, true, K_DCT3);
  transform_axis(p, nx, ny, false, K_DCT3);
  transform_axis(fx, nx, ny, false, K_DCT3);
  transform_axis(fx, nx, ny, true, K_IDST);
  transform_axis(fy, nx, ny, true, K_DCT3);
  transform_axis(fy, nx, ny, false, K_IDST);
  std::copy(p.begin(), p.end(), phi);
  std::copy(fx.begin(), fx.end(), ex);
  std::copy(fy.begin(), fy.end(), ey);
}

// fastExp (src/nesterovBase.cpp:1568-1582): (1 + a/1024)^1024 by squaring;
// the first step is evaluated in double as in the reference.
static inline float fast_exp(float a) {
  a = (float)(1.0 + (double)a / 1024.0);
  for (int i = 0; i < 10; i++) a *= a;
  return a;
}

static inline int fast_modulo(int input, int ceil) { return input >= ceil ? input % ceil : input; }

struct FP { float x = 0, y = 0; FP() {} FP(float a, float b) : x(a), y(b) {} };

struct Oracle {
  gpl_params p;
  // ---- PlacerBase
  int coreLx, coreLy, coreUx, coreUy, siteW, siteH;
  int nInst = 0;
  vector<int> ilx, ily, iux, iuy;
  vector<uint8_t> ikind;
  vector<int> placeInsts;            // instance indices
  vector<int> nonPlaceInsts;
  int64_t placeArea = 0, stdArea = 0, macroArea = 0, nonPlaceArea = 0;
  int nPins = 0, nNets = 0;
  vector<int> pinInst, pinOx, pinOy, pinX, pinY, netStart;
  vector<int> instPinStart, instPins;
  // ---- NesterovBase
  bool nbReady = false;
  int nG = 0, nPlace = 0, nFill = 0, fillDx = 0, fillDy = 0;
  vector<int> glx, gly, gux, guy;          // real rectangle
  vector<int> gdlx, gdly, gdux, gduy;      // density rectangle
  vector<float> gscale;
  vector<uint8_t> gkind;                   // 0 std, 1 macro, 2 filler
  vector<int> gPinStart, gPins;            // gcell -> pins
  vector<int> gpx, gpy;                    // GPin centres
  // ---- BinGrid
  int cntX = 0, cntY = 0, sizeX = 0, sizeY = 0;
  vector<int> blx, bly, bux, buy;
  vector<int64_t> bNonPlace, bInst, bFill;
  vector<float> bDensity, bPhi, bEx, bEy;
  int64_t overflowArea = 0;
  double overflowF64 = 0.0;
  float sumPhi = 0.0f;
  double sumPhiF64 = 0.0;
  // ---- WA
  vector<float> nMinSX, nXMinSX, nMaxSX, nXMaxSX, nMinSY, nYMinSY, nMaxSY, nYMaxSY;
  vector<float> pMinX, pMaxX, pMinY, pMaxY;
  vector<uint8_t> pFlags;   // bit0 minX, bit1 maxX, bit2 minY, bit3 maxY
  // ---- NesterovPlace
  bool npReady = false;
  vector<FP> curSLP, curSLPWL, curSLPD, curSLPSum;
  vector<FP> nextSLP, nextSLPWL, nextSLPD, nextSLPSum;
  vector<FP> prevSLP, prevSLPWL, prevSLPD, prevSLPSum;
  vector<FP> curCoordi, nextCoordi;
  float wlGradSum = 0, dGradSum = 0, stepLength = 0, densityPenalty = 0;
  float baseWLCoef = 0, wlCoefX = 0, wlCoefY = 0, sumOverflow = 0;
  int64_t prevHpwl = 0;
  bool isDiverged = false;
  float curA = 1.0f, minSumOverflow = 1e30f, hpwlWithMinSumOverflow = 1e30f;
  bool isMaxPhiCoefChanged = false;
  float maxPhiCoef = 1.05f;
  int iter = 0, evals = 0, divergeCode = 0;
  bool finished = false;
  double wlGradSumF64 = 0, dGradSumF64 = 0;

  // ================================================================ setup
  int build(const gpl_netlist_desc* d, const gpl_params* pp) {
    p = *pp;
    maxPhiCoef = p.max_phi_coef;
    coreLx = d->core_lx; coreLy = d->core_ly; coreUx = d->core_ux; coreUy = d->core_uy;
    siteW = d->site_w; siteH = d->site_h;
    nInst = d->n_insts;
    ilx.assign(d->inst_lx, d->inst_lx + nInst);
    ily.assign(d->inst_ly, d->inst_ly + nInst);
    iux.assign(d->inst_ux, d->inst_ux + nInst);
    iuy.assign(d->inst_uy, d->inst_uy + nInst);
    ikind.assign(d->inst_kind, d->inst_kind + nInst);
    nPins = d->n_pins; nNets = d->n_nets;
    pinInst.assign(d->pin_inst, d->pin_inst + nPins);
    pinOx.assign(d->pin_ox, d->pin_ox + nPins);
    pinOy.assign(d->pin_oy, d->pin_oy + nPins);
    pinX.assign(d->pin_x, d->pin_x + nPins);
    pinY.assign(d->pin_y, d->pin_y + nPins);
    netStart.assign(d->net_start, d->net_start + nNets + 1);
    if (d->inst_pin_start) {
      instPinStart.assign(d->inst_pin_start, d->inst_pin_start + nInst + 1);
      instPins.assign(d->inst_pins, d->inst_pins + instPinStart[nInst]);
    } else {
      instPinStart.assign(nInst + 1, 0);
      for (int q = 0; q < nPins; q++) if (pinInst[q] >= 0) instPinStart[pinInst[q] + 1]++;
      for (int i = 0; i < nInst; i++) instPinStart[i + 1] += instPinStart[i];
      instPins.assign(instPinStart[nInst], 0);
      vector<int> fill(instPinStart.begin(), instPinStart.end() - 1);
      for (int q = 0; q < nPins; q++) if (pinInst[q] >= 0) instPins[fill[pinInst[q]]++] = q;
    }
    // PlacerBase::init areas (src/placerBase.cpp:639-680)
    for (int i = 0; i < nInst; i++) {
      int64_t a = (int64_t)(iux[i] - ilx[i]) * (int64_t)(iuy[i] - ily[i]);
      if (ikind[i] == GPL_INST_PLACE) {
        placeInsts.push_back(i);
        placeArea += a;
        if (iuy[i] - ily[i] > siteH * 6) macroArea += a; else stdArea += a;
      } else if (ikind[i] == GPL_INST_FIXED) {
        nonPlaceInsts.push_back(i);
        int rlx = std::max(coreLx, ilx[i]), rly = std::max(coreLy, ily[i]);
        int rux = std::min(coreUx, iux[i]), ruy = std::min(coreUy, iuy[i]);
        nonPlaceArea += (int64_t)(rux - rlx) * (int64_t)(ruy - rly);
      } else if (ikind[i] == GPL_INST_DUMMY) {
        nonPlaceInsts.push_back(i);
        nonPlaceArea += a;
      }
    }
    // PlacerBase::printInfo utilisation check (src/placerBase.cpp:936-956)
    int64_t coreArea = (int64_t)(coreUx - coreLx) * (int64_t)(coreUy - coreLy);
    float util = (float)placeArea / (coreArea - nonPlaceArea) * 100;
    if (util >= 100.1) return GPL_ERR_UTIL;
    return GPL_OK;
  }

  int instCx(int i) const { return (ilx[i] + iux[i]) / 2; }
  int instCy(int i) const { return (ily[i] + iuy[i]) / 2; }

  // Instance::setCenterLocation + Pin::updateLocation (src/placerBase.cpp:127-140)
  void setInstCenter(int i, int x, int y) {
    const int hx = (iux[i] - ilx[i]) / 2, hy = (iuy[i] - ily[i]) / 2;
    ilx[i] = x - hx; ily[i] = y - hy; iux[i] = x + hx; iuy[i] = y + hy;
    for (int k = instPinStart[i]; k < instPinStart[i + 1]; k++) {
      int q = instPins[k];
      pinX[q] = instCx(i) + pinOx[q];
      pinY[q] = instCy(i) + pinOy[q];
    }
  }

  // ============================================================ NesterovBase
  int initNesterovBase() {
    // GCells for placeable instances (src/nesterovBase.cpp:919-931)
    nPlace = (int)placeInsts.size();
    for (int k = 0; k < nPlace; k++) {
      int i = placeInsts[k];
      glx.push_back(ilx[i]); gly.push_back(ily[i]); gux.push_back(iux[i]); guy.push_back(iuy[i]);
      gkind.push_back((iuy[i] - ily[i]) > siteH * 6 ? 1 : 0);
    }
    int rc = initFillers();
    if (rc) return rc;
    nG = (int)glx.size();
    gdlx = glx; gdly = gly; gdux = gux; gduy = guy;
    // gcell pins (src/nesterovBase.cpp:977-986)
    gPinStart.assign(nG + 1, 0);
    for (int k = 0; k < nPlace; k++) {
      int i = placeInsts[k];
      gPinStart[k + 1] = gPinStart[k] + (instPinStart[i + 1] - instPinStart[i]);
    }
    for (int k = nPlace; k < nG; k++) gPinStart[k + 1] = gPinStart[k];
    gPins.clear();
    for (int k = 0; k < nPlace; k++) {
      int i = placeInsts[k];
      for (int t = instPinStart[i]; t < instPinStart[i + 1]; t++) gPins.push_back(instPins[t]);
    }
    gpx = pinX; gpy = pinY;
    initBins();
    // density size and scale (src/nesterovBase.cpp:1033-1061)
    gscale.resize(nG);
    for (int g = 0; g < nG; g++) {
      int dx = gux[g] - glx[g], dy = guy[g] - gly[g];
      float scaleX, scaleY, dsx, dsy;
      if (dx < kSqrt2 * sizeX) {
        scaleX = (float)dx / (float)(kSqrt2 * sizeX);
        dsx = (float)(kSqrt2 * (float)sizeX);
      } else { scaleX = 1.0f; dsx = (float)dx; }
      if (dy < kSqrt2 * sizeY) {
        scaleY = (float)dy / (float)(kSqrt2 * sizeY);
        dsy = (float)(kSqrt2 * (float)sizeY);
      } else { scaleY = 1.0f; dsy = (float)dy; }
      // GCell::setDensitySize (src/nesterovBase.cpp:182-191), int arguments
      int ddx = (int)dsx, ddy = (int)dsy;
      int cx = (gdux[g] + gdlx[g]) / 2, cy = (gduy[g] + gdly[g]) / 2;
      gdlx[g] = cx - ddx / 2; gdly[g] = cy - ddy / 2;
      gdux[g] = cx + ddx / 2; gduy[g] = cy + ddy / 2;
      gscale[g] = scaleX * scaleY;
    }
    // WA storage
    nMinSX.assign(nNets, 0); nXMinSX.assign(nNets, 0); nMaxSX.assign(nNets, 0); nXMaxSX.assign(nNets, 0);
    nMinSY.assign(nNets, 0); nYMinSY.assign(nNets, 0); nMaxSY.assign(nNets, 0); nYMaxSY.assign(nNets, 0);
    pMinX.assign(nPins, 0); pMaxX.assign(nPins, 0); pMinY.assign(nPins, 0); pMaxY.assign(nPins, 0);
    pFlags.assign(nPins, 0);
    nbReady = true;
    return GPL_OK;
  }

  // NesterovBase::initFillerGCells (src/nesterovBase.cpp:1066-1155)
  int initFillers() {
    vector<int> dxs, dys;
    for (int i : placeInsts) { dxs.push_back(iux[i] - ilx[i]); dys.push_back(iuy[i] - ily[i]); }
    std::sort(dxs.begin(), dxs.end());
    std::sort(dys.begin(), dys.end());
    int64_t dxSum = 0, dySum = 0;
    int minIdx = (int)(dxs.size() * 0.05);
    int maxIdx = (int)(dxs.size() * 0.95);
    for (int i = minIdx; i < maxIdx; i++) { dxSum += dxs[i]; dySum += dys[i]; }
    fillDx = (int)(dxSum / (maxIdx - minIdx));
    fillDy = (int)(dySum / (maxIdx - minIdx));
    int64_t coreArea = (int64_t)(coreUx - coreLx) * (int64_t)(coreUy - coreLy);
    int64_t whiteSpace = coreArea - nonPlaceArea;
    int64_t movable = (int64_t)(whiteSpace * p.target_density);
    int64_t totalFiller = movable - stdArea - (int64_t)(macroArea * p.target_density);
    if (totalFiller < 0) return GPL_ERR_FILLER_AREA;
    int fillerCnt = (int)(totalFiller / (int64_t)(fillDx * fillDy));
    std::mt19937 rv(0);
    int cdx = coreUx - coreLx, cdy = coreUy - coreLy;
    for (int i = 0; i < fillerCnt; i++) {
      auto rx = rv();
      auto ry = rv();
      int cx = (int)(rx % (unsigned)cdx + coreLx);
      int cy = (int)(ry % (unsigned)cdy + coreLy);
      glx.push_back(cx - fillDx / 2); gly.push_back(cy - fillDy / 2);
      gux.push_back(cx + fillDx / 2); guy.push_back(cy + fillDy / 2);
      gkind.push_back(2);
    }
    nFill = fillerCnt;
    return GPL_OK;
  }

  // BinGrid::initBins + updateBinsNonPlaceArea (src/nesterovBase.cpp:631-741)
  void initBins() {
    int64_t totalBinArea = (int64_t)(coreUx - coreLx) * (int64_t)(coreUy - coreLy);
    int64_t avgArea = placeArea / (int64_t)placeInsts.size();
    int64_t idealBinArea = (int64_t)std::round((float)avgArea / p.target_density);
    int idealBinCnt = (int)(totalBinArea / idealBinArea);
    int found = 2;
    for (found = 2; found <= 1024; found *= 2)
      if (found * found <= idealBinCnt && 4 * found * found > idealBinCnt) break;
    cntX = p.bin_grid_cnt_x > 0 ? p.bin_grid_cnt_x : found;
    cntY = p.bin_grid_cnt_y > 0 ? p.bin_grid_cnt_y : found;
    sizeX = (int)ceil((float)(coreUx - coreLx) / cntX);
    sizeY = (int)ceil((float)(coreUy - coreLy) / cntY);
    int nb = cntX * cntY;
    blx.resize(nb); bly.resize(nb); bux.resize(nb); buy.resize(nb);
    int x = coreLx, y = coreLy;
    for (int b = 0; b < nb; b++) {
      int sx = (x + sizeX > coreUx) ? coreUx - x : sizeX;
      int sy = (y + sizeY > coreUy) ? coreUy - y : sizeY;
      blx[b] = x; bly[b] = y; bux[b] = x + sx; buy[b] = y + sy;
      x += sizeX;
      if (x >= coreUx) { y += sizeY; x = coreLx; }
    }
    bNonPlace.assign(nb, 0); bInst.assign(nb, 0); bFill.assign(nb, 0);
    bDensity.assign(nb, 0); bPhi.assign(nb, 0); bEx.assign(nb, 0); bEy.assign(nb, 0);
    for (int i : nonPlaceInsts) {
      int lo_x = std::max((ilx[i] - coreLx) / sizeX, 0);
      int hi_x = std::min(fast_modulo(iux[i] - coreLx, sizeX) == 0 ? (iux[i] - coreLx) / sizeX
                                                                 : (iux[i] - coreLx) / sizeX + 1, cntX);
      int lo_y = std::max((ily[i] - coreLy) / sizeY, 0);
      int hi_y = std::min(fast_modulo(iuy[i] - coreLy, sizeY) == 0 ? (iuy[i] - coreLy) / sizeY
                                                                 : (iuy[i] - coreLy) / sizeY + 1, cntY);
      for (int a = lo_x; a < hi_x; a++) {
        for (int c = lo_y; c < hi_y; c++) {
          int b = c * cntX + a;
          int rlx = std::max(blx[b], ilx[i]), rly = std::max(bly[b], ily[i]);
          int rux = std::min(bux[b], iux[i]), ruy = std::min(buy[b], iuy[i]);
          int64_t ov = (rlx >= rux || rly >= ruy) ? 0 : (int64_t)(rux - rlx) * (int64_t)(ruy - rly);
          bNonPlace[b] += (int64_t)(ov * p.target_density);
        }
      }
    }
  }

  void binRange(int g, int& x0, int& x1, int& y0, int& y1) const {
    // getDensityMinMaxIdxX/Y (src/nesterovBase.cpp:822-841).  The reference
    // leaves the range unclamped and reads outside its bins for a cell that
    // sticks out of the core (undefined behaviour); the range is clamped to
    // the grid here, as the GPU does, which changes nothing for cells inside.
    x0 = (gdlx[g] - coreLx) / sizeX;
    x1 = fast_modulo(gdux[g] - coreLx, sizeX) == 0 ? (gdux[g] - coreLx) / sizeX
                                                  : (gdux[g] - coreLx) / sizeX + 1;
    y0 = (gdly[g] - coreLy) / sizeY;
    y1 = fast_modulo(gduy[g] - coreLy, sizeY) == 0 ? (gduy[g] - coreLy) / sizeY
                                                  : (gduy[g] - coreLy) / sizeY + 1;
    x0 = std::max(x0, 0); y0 = std::max(y0, 0);
    x1 = std::min(x1, cntX); y1 = std::min(y1, cntY);
  }

  float overlap(int b, int g) const {
    // getOverlapDensityArea (src/nesterovBase.cpp:1533-1547)
    int rlx = std::max(blx[b], gdlx[g]), rly = std::max(bly[b], gdly[g]);
    int rux = std::min(bux[b], gdux[g]), ruy = std::min(buy[b], gduy[g]);
    if (rlx >= rux || rly >= ruy) return 0.0f;
    return (float)(rux - rlx) * (float)(ruy - rly);
  }

  // GCell::setDensityCenterLocation + GPin::updateDensityLocation
  // (src/nesterovBase.cpp:164-179, 411-415); coordinates truncate to int.
  void setDensityCenters(const vector<FP>& c) {
    for (int g = 0; g < nG; g++) {
      int dcx = (int)c[g].x, dcy = (int)c[g].y;
      int hx = (gdux[g] - gdlx[g]) / 2, hy = (gduy[g] - gdly[g]) / 2;
      gdlx[g] = dcx - hx; gdly[g] = dcy - hy; gdux[g] = dcx + hx; gduy[g] = dcy + hy;
      int cx = (gdux[g] + gdlx[g]) / 2, cy = (gduy[g] + gdly[g]) / 2;
      for (int t = gPinStart[g]; t < gPinStart[g + 1]; t++) {
        int q = gPins[t];
        gpx[q] = cx + pinOx[q];
        gpy[q] = cy + pinOy[q];
      }
    }
  }

  // BinGrid::updateBinsGCellDensityArea (src/nesterovBase.cpp:746-819)
  void scatter() {
    int nb = cntX * cntY;
    std::fill(bInst.begin(), bInst.end(), 0);
    std::fill(bFill.begin(), bFill.end(), 0);
    for (int g = 0; g < nG; g++) {
      int x0, x1, y0, y1;
      binRange(g, x0, x1, y0, y1);
      for (int a = x0; a < x1; a++) {
        for (int c = y0; c < y1; c++) {
          int b = c * cntX + a;
          if (gkind[g] == 1) bInst[b] += (int64_t)(overlap(b, g) * gscale[g] * p.target_density);
          else if (gkind[g] == 0) bInst[b] += (int64_t)(overlap(b, g) * gscale[g]);
          else bFill[b] += (int64_t)(overlap(b, g) * gscale[g]);
        }
      }
    }
    overflowArea = 0;
    overflowF64 = 0.0;
    for (int b = 0; b < nb; b++) {
      int64_t binArea = (int64_t)(bux[b] - blx[b]) * (int64_t)(buy[b] - bly[b]);
      float cap = (float)binArea * p.target_density;
      bDensity[b] = ((float)bInst[b] + (float)bFill[b] + (float)bNonPlace[b]) / cap;
      float ov = std::max(0.0f, (float)bInst[b] + (float)bNonPlace[b] - cap);
      overflowArea = (int64_t)((float)overflowArea + ov);   // reference: float-evaluated +=
      overflowF64 += std::max(0.0, (double)bInst[b] + (double)bNonPlace[b] - (double)cap);
    }
  }

  // NesterovBase::updateDensityForceBin (src/nesterovBase.cpp:1481-1506)
  void densityForce() {
    size_t nb = (size_t)cntX * cntY;
    vector<double> rho(nb), ph(nb), fx(nb), fy(nb);
    for (size_t b = 0; b < nb; b++) rho[b] = bDensity[b];
    poisson_f64(cntX, cntY, sizeX, sizeY, rho.data(), ph.data(), fx.data(), fy.data());
    sumPhi = 0.0f;
    sumPhiF64 = 0.0;
    for (size_t b = 0; b < nb; b++) {
      bPhi[b] = (float)ph[b]; bEx[b] = (float)fx[b]; bEy[b] = (float)fy[b];
      sumPhi += bPhi[b] * (float)(bNonPlace[b] + bInst[b] + bFill[b]);
      sumPhiF64 += ph[b] * (double)(bNonPlace[b] + bInst[b] + bFill[b]);
    }
  }

  // NesterovBase::updateWireLengthForceWA (src/nesterovBase.cpp:1304-1360)
  void waForce(float cx_, float cy_) {
    const float bar = p.min_wire_length_force_bar;
    for (int n = 0; n < nNets; n++) {
      float s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, s6 = 0, s7 = 0;
      int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
      for (int q = netStart[n]; q < netStart[n + 1]; q++) {
        lx = std::min(gpx[q], lx); ly = std::min(gpy[q], ly);
        ux = std::max(gpx[q], ux); uy = std::max(gpy[q], uy);
      }
      for (int q = netStart[n]; q < netStart[n + 1]; q++) {
        pFlags[q] = 0;
        pMinX[q] = pMaxX[q] = pMinY[q] = pMaxY[q] = 0;
        float eMinX = (float)(lx - gpx[q]) * cx_;
        float eMaxX = (float)(gpx[q] - ux) * cx_;
        float eMinY = (float)(ly - gpy[q]) * cy_;
        float eMaxY = (float)(gpy[q] - uy) * cy_;
        if (eMinX > bar) { pMinX[q] = fast_exp(eMinX); pFlags[q] |= 1; s0 += pMinX[q]; s1 += (float)gpx[q] * pMinX[q]; }
        if (eMaxX > bar) { pMaxX[q] = fast_exp(eMaxX); pFlags[q] |= 2; s2 += pMaxX[q]; s3 += (float)gpx[q] * pMaxX[q]; }
        if (eMinY > bar) { pMinY[q] = fast_exp(eMinY); pFlags[q] |= 4; s4 += pMinY[q]; s5 += (float)gpy[q] * pMinY[q]; }
        if (eMaxY > bar) { pMaxY[q] = fast_exp(eMaxY); pFlags[q] |= 8; s6 += pMaxY[q]; s7 += (float)gpy[q] * pMaxY[q]; }
      }
      nMinSX[n] = s0; nXMinSX[n] = s1; nMaxSX[n] = s2; nXMaxSX[n] = s3;
      nMinSY[n] = s4; nYMinSY[n] = s5; nMaxSY[n] = s6; nYMaxSY[n] = s7;
    }
  }

  // getWireLengthGradientPinWA (src/nesterovBase.cpp:1383-1440); the
  // reference's double literals promote parts of the expression to double.
  FP pinGrad(int q, int n, float cx_, float cy_) const {
    float gMinX = 0, gMaxX = 0, gMinY = 0, gMaxY = 0;
    float x = (float)gpx[q], y = (float)gpy[q];
    if (pFlags[q] & 1) {
      float S = nMinSX[n], SX = nXMinSX[n];
      gMinX = (float)(((double)S * ((double)pMinX[q] * (1.0 - (double)(cx_ * x))) +
                       (double)(cx_ * pMinX[q] * SX)) / (double)(S * S));
    }
    if (pFlags[q] & 2) {
      float S = nMaxSX[n], SX = nXMaxSX[n];
      gMaxX = (float)(((double)S * ((double)pMaxX[q] * (1.0 + (double)(cx_ * x))) -
                       (double)(cx_ * pMaxX[q] * SX)) / (double)(S * S));
    }
    if (pFlags[q] & 4) {
      float S = nMinSY[n], SY = nYMinSY[n];
      gMinY = (float)(((double)S * ((double)pMinY[q] * (1.0 - (double)(cy_ * y))) +
                       (double)(cy_ * pMinY[q] * SY)) / (double)(S * S));
    }
    if (pFlags[q] & 8) {
      float S = nMaxSY[n], SY = nYMaxSY[n];
      gMaxY = (float)(((double)S * ((double)pMaxY[q] * (1.0 + (double)(cy_ * y))) -
                       (double)(cy_ * pMaxY[q] * SY)) / (double)(S * S));
    }
    return FP(gMinX - gMaxX, gMinY - gMaxY);
  }

  vector<int> pinNet;
  void buildPinNet() {
    pinNet.assign(nPins, 0);
    for (int n = 0; n < nNets; n++)
      for (int q = netStart[n]; q < netStart[n + 1]; q++) pinNet[q] = n;
  }

  // Per-net weights (GNet::customWeight, src/nesterovBase.h:210-212; stored
  // but not applied by the reference): empty = every weight 1, otherwise
  // each pin gradient is scaled by its net's weight before the gcell sum.
  vector<float> netW;

  FP wlGrad(int g, float cx_, float cy_) const {
    FP s;
    for (int t = gPinStart[g]; t < gPinStart[g + 1]; t++) {
      const int n = pinNet[gPins[t]];
      FP v = pinGrad(gPins[t], n, cx_, cy_);
      if (!netW.empty()) { v.x *= netW[n]; v.y *= netW[n]; }
      s.x += v.x; s.y += v.y;
    }
    return s;
  }

  FP densityGrad(int g) const {
    int x0, x1, y0, y1;
    binRange(g, x0, x1, y0, y1);
    FP e;
    for (int a = x0; a < x1; a++) {
      for (int c = y0; c < y1; c++) {
        int b = c * cntX + a;
        float ov = overlap(b, g) * gscale[g];
        e.x += ov * bEx[b];
        e.y += ov * bEy[b];
      }
    }
    return e;
  }

  int64_t hpwl() const {
    // NesterovBase::getHpwl (src/nesterovBase.cpp:1508-1516)
    int64_t h = 0;
    for (int n = 0; n < nNets; n++) {
      int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
      for (int q = netStart[n]; q < netStart[n + 1]; q++) {
        lx = std::min(gpx[q], lx); ly = std::min(gpy[q], ly);
        ux = std::max(gpx[q], ux); uy = std::max(gpy[q], uy);
      }
      h += (int64_t)((ux - lx) + (uy - ly));
    }
    return h;
  }

  // one evaluation: scatter, Poisson, WA (the EVAL of the loop)
  void evaluate(const vector<FP>& c) {
    setDensityCenters(c);
    scatter();
    densityForce();
    waForce(wlCoefX, wlCoefY);
    evals++;
  }

  // ============================================================ NesterovPlace
  // getDensityCoordiLayoutInsideX/Y (src/nesterovBase.cpp:1270-1297)
  float insideX(int g, float cx) const {
    float adj = cx;
    int h = (gdux[g] - gdlx[g]) / 2;
    if (cx - h < coreLx) adj = (float)(coreLx + h);
    if (cx + h > coreUx) adj = (float)(coreUx - h);
    return adj;
  }
  float insideY(int g, float cy) const {
    float adj = cy;
    int h = (gduy[g] - gdly[g]) / 2;
    if (cy - h < coreLy) adj = (float)(coreLy + h);
    if (cy + h > coreUy) adj = (float)(coreUy - h);
    return adj;
  }

  // NesterovPlace::updateGradients (src/nesterovPlace.cpp:206-273)
  void updateGradients(vector<FP>& sum, vector<FP>& wl, vector<FP>& dn) {
    wlGradSum = 0; dGradSum = 0;
    wlGradSumF64 = 0; dGradSumF64 = 0;
    for (int g = 0; g < nG; g++) {
      wl[g] = wlGrad(g, wlCoefX, wlCoefY);
      dn[g] = densityGrad(g);
      wlGradSum += std::fabs(wl[g].x);
      wlGradSum += std::fabs(wl[g].y);
      dGradSum += std::fabs(dn[g].x);
      dGradSum += std::fabs(dn[g].y);
      wlGradSumF64 += std::fabs((double)wl[g].x) + std::fabs((double)wl[g].y);
      dGradSumF64 += std::fabs((double)dn[g].x) + std::fabs((double)dn[g].y);
      sum[g].x = wl[g].x + densityPenalty * dn[g].x;
      sum[g].y = wl[g].y + densityPenalty * dn[g].y;
      float wlPre = (float)(gPinStart[g + 1] - gPinStart[g]);
      float dPre = (float)(gux[g] - glx[g]) * (float)(guy[g] - gly[g]);
      float px = wlPre + densityPenalty * dPre;
      float py = wlPre + densityPenalty * dPre;
      if (px <= p.min_preconditioner) px = p.min_preconditioner;
      if (py <= p.min_preconditioner) py = p.min_preconditioner;
      sum[g].x /= px;
      sum[g].y /= py;
    }
    if (std::isnan(wlGradSum) || std::isinf(wlGradSum) || std::isnan(dGradSum) || std::isinf(dGradSum))
      isDiverged = true;
  }

  float overflowRatio() const {
    return (float)overflowArea / (float)(stdArea + macroArea * p.target_density);
  }

  void updateWireLengthCoef(float overflow) {
    // src/nesterovPlace.cpp:474-490
    if (overflow > 1.0) wlCoefX = wlCoefY = 0.1f;
    else if (overflow < 0.1) wlCoefX = wlCoefY = 10.0f;
    else wlCoefX = wlCoefY = (float)(1.0 / pow(10.0, (overflow - 0.1) * 20 / 9.0 - 1.0));
    wlCoefX *= baseWLCoef;
    wlCoefY *= baseWLCoef;
  }

  static float distance(const vector<FP>& a, const vector<FP>& b) {
    float s = 0.0f;
    for (size_t i = 0; i < a.size(); i++) {
      s += (a[i].x - b[i].x) * (a[i].x - b[i].x);
      s += (a[i].y - b[i].y) * (a[i].y - b[i].y);
    }
    return (float)sqrt(s / (2.0 * a.size()));
  }

  float stepLengthOf(const vector<FP>& pc, const vector<FP>& pg, const vector<FP>& cc, const vector<FP>& cg) {
    float cd = distance(pc, cc);
    float gd = distance(pg, cg);
    return cd / gd;
  }

  // NesterovPlace::init (src/nesterovPlace.cpp:64-175)
  int initNesterovPlace() {
    buildPinNet();
    curSLP.assign(nG, FP()); curSLPWL = curSLPD = curSLPSum = curSLP;
    nextSLP = nextSLPWL = nextSLPD = nextSLPSum = curSLP;
    prevSLP = prevSLPWL = prevSLPD = prevSLPSum = curSLP;
    curCoordi = nextCoordi = curSLP;
    for (int g = 0; g < nG; g++) {
      // updateDensityCoordiLayoutInside (src/nesterovBase.cpp:1245-1268)
      float tlx = (float)gdlx[g], tly = (float)gdly[g];
      int ddx = gdux[g] - gdlx[g], ddy = gduy[g] - gdly[g];
      if (tlx < coreLx) tlx = (float)coreLx;
      if (tly < coreLy) tly = (float)coreLy;
      if (tlx + ddx > coreUx) tlx = (float)(coreUx - ddx);
      if (tly + ddy > coreUy) tly = (float)(coreUy - ddy);
      int nlx = (int)tlx, nly = (int)tly;
      gdux[g] = nlx + ddx; gduy[g] = nly + ddy; gdlx[g] = nlx; gdly[g] = nly;
      FP c((float)((gdux[g] + gdlx[g]) / 2), (float)((gduy[g] + gdly[g]) / 2));
      curSLP[g] = prevSLP[g] = curCoordi[g] = c;
    }
    setDensityCenters(curSLP);
    scatter();
    prevHpwl = hpwl();
    densityForce();
    baseWLCoef = p.init_wire_length_coef / ((float)(sizeX + sizeY) * 0.5);
    sumOverflow = overflowRatio();
    updateWireLengthCoef(sumOverflow);
    waForce(wlCoefX, wlCoefY);
    evals++;
    updateGradients(curSLPSum, curSLPWL, curSLPD);
    if (isDiverged) { npReady = true; divergeCode = GPL_ERR_DIVERGED_INIT; return GPL_ERR_DIVERGED_INIT; }
    for (int g = 0; g < nG; g++) {
      float px = curSLP[g].x + p.initial_prev_coordi_update_coef * curSLPSum[g].x;
      float py = curSLP[g].y + p.initial_prev_coordi_update_coef * curSLPSum[g].y;
      prevSLP[g] = FP(insideX(g, px), insideY(g, py));
    }
    evaluate(prevSLP);
    updateGradients(prevSLPSum, prevSLPWL, prevSLPD);
    if (isDiverged) { npReady = true; divergeCode = GPL_ERR_DIVERGED_INIT; return GPL_ERR_DIVERGED_INIT; }
    densityPenalty = (wlGradSum / dGradSum) * p.init_density_penalty;
    sumOverflow = overflowRatio();
    stepLength = stepLengthOf(prevSLP, prevSLPSum, curSLP, curSLPSum);
    if (p.verbose_level >= 3)
      printf("[oracle] InitialHPWL %lld BaseWireLengthCoef %g WireLengthCoef %g WLGradSum %g "
             "DensityGradSum %g InitDensityPenalty %g SumOverflow %g InitialStepLength %g\n",
             (long long)prevHpwl, baseWLCoef, wlCoefX, wlGradSum, dGradSum, densityPenalty,
             sumOverflow, stepLength);
    npReady = true;
    return GPL_OK;
  }

  float phiCoef(float scaledDiffHpwl) const {
    float r = (scaledDiffHpwl < 0) ? maxPhiCoef
                                   : (float)(maxPhiCoef * pow(maxPhiCoef, scaledDiffHpwl * -1.0));
    return std::max(p.min_phi_coef, r);
  }

  // NesterovPlace::doNesterovPlace (src/nesterovPlace.cpp:275-472), resumable
  int run(int maxIters, gpl_iter_log* log) {
    if (divergeCode == GPL_ERR_DIVERGED_INIT) { finished = true; return divergeCode; }
    int done = 0;
    for (; iter < p.nesterov_place_max_iter && !finished; iter++) {
      if (maxIters > 0 && done >= maxIters) break;
      done++;
      float prevA = curA;
      curA = (float)((1.0 + sqrt(4.0 * prevA * prevA + 1.0)) * 0.5);
      float coeff = (float)((prevA - 1.0) / curA);
      int bt = 0;
      for (bt = 0; bt < p.max_back_track; bt++) {
        for (int g = 0; g < nG; g++) {
          FP nc(curSLP[g].x + stepLength * curSLPSum[g].x, curSLP[g].y + stepLength * curSLPSum[g].y);
          FP ns(nc.x + coeff * (nc.x - curCoordi[g].x), nc.y + coeff * (nc.y - curCoordi[g].y));
          nextCoordi[g] = FP(insideX(g, nc.x), insideY(g, nc.y));
          nextSLP[g] = FP(insideX(g, ns.x), insideY(g, ns.y));
        }
        evaluate(nextSLP);
        updateGradients(nextSLPSum, nextSLPWL, nextSLPD);
        if (isDiverged) break;
        float ns = stepLengthOf(curSLP, curSLPSum, nextSLP, nextSLPSum);
        if (ns > stepLength * 0.95) { stepLength = ns; break; }
        stepLength = ns;
      }
      if (!isMaxPhiCoefChanged && sumOverflow < 0.35f) {
        isMaxPhiCoefChanged = true;
        maxPhiCoef = (float)(maxPhiCoef * 0.99);   // float *= double
      }
      if (p.max_back_track == bt) { divergeCode = GPL_ERR_DIVERGED_BACKTRACK; isDiverged = true; }
      // NaN/Inf inside the back-tracking loop: the reference leaves the
      // divergence code at 0 (src/nesterovPlace.cpp:371-374, 411-413)
      if (isDiverged) { finished = true; if (!divergeCode) divergeCode = GPL_ERR_DIVERGED_NAN; break; }
      // updateNextIter (src/nesterovPlace.cpp:514-553)
      std::swap(prevSLP, curSLP); std::swap(prevSLPWL, curSLPWL);
      std::swap(prevSLPD, curSLPD); std::swap(prevSLPSum, curSLPSum);
      std::swap(curSLP, nextSLP); std::swap(curSLPWL, nextSLPWL);
      std::swap(curSLPD, nextSLPD); std::swap(curSLPSum, nextSLPSum);
      std::swap(curCoordi, nextCoordi);
      sumOverflow = overflowRatio();
      updateWireLengthCoef(sumOverflow);
      int64_t h = hpwl();
      float pc = phiCoef((float)(h - prevHpwl) / p.reference_hpwl);
      prevHpwl = h;
      densityPenalty *= pc;
      if (log && log->count < log->capacity) {
        int k = log->count++;
        if (log->overflow) log->overflow[k] = sumOverflow;
        if (log->hpwl) log->hpwl[k] = prevHpwl;
        if (log->step_length) log->step_length[k] = stepLength;
        if (log->backtracks) log->backtracks[k] = bt + 1;
      }
      if (p.verbose_level > 0 && (iter == 0 || (iter + 1) % 10 == 0))
        printf("[NesterovSolve] Iter: %d overflow: %g HPWL: %lld\n", iter + 1, sumOverflow, (long long)prevHpwl);
      if (minSumOverflow > sumOverflow) { minSumOverflow = sumOverflow; hpwlWithMinSumOverflow = (float)prevHpwl; }
      if (sumOverflow < 0.3f && sumOverflow - minSumOverflow >= 0.02f &&
          hpwlWithMinSumOverflow * 1.2f < prevHpwl) {
        divergeCode = GPL_ERR_DIVERGED_PHI; isDiverged = true; finished = true; iter++; break;
      }
      if (iter > 50 && sumOverflow <= p.target_overflow) { finished = true; iter++; break; }
    }
    if (iter >= p.nesterov_place_max_iter) finished = true;
    return divergeCode;
  }

  // ============================================================ InitialPlace
  vector<uint8_t> bnd;   // bit0 minX, bit1 maxX, bit2 minY, bit3 maxY
  // InitialPlace::updatePinInfo (src/initialPlace.cpp:128-182)
  void updatePinInfo() {
    bnd.assign(nPins, 0);
    for (int n = 0; n < nNets; n++) {
      int qMinX = -1, qMinY = -1, qMaxX = -1, qMaxY = -1;
      int lx = INT_MAX, ly = INT_MAX, ux = INT_MIN, uy = INT_MIN;
      for (int q = netStart[n]; q < netStart[n + 1]; q++) {
        if (lx > pinX[q]) { if (qMinX >= 0) bnd[qMinX] &= ~1; lx = pinX[q]; qMinX = q; bnd[q] |= 1; }
        if (ux < pinX[q]) { if (qMaxX >= 0) bnd[qMaxX] &= ~2; ux = pinX[q]; qMaxX = q; bnd[q] |= 2; }
        if (ly > pinY[q]) { if (qMinY >= 0) bnd[qMinY] &= ~4; ly = pinY[q]; qMinY = q; bnd[q] |= 4; }
        if (uy < pinY[q]) { if (qMaxY >= 0) bnd[qMaxY] &= ~8; uy = pinY[q]; qMaxY = q; bnd[q] |= 8; }
      }
    }
  }

  struct Trip { int r, c; float v; };
  vector<int> extId;   // instance -> dense movable index or -1

  // InitialPlace::createSparseMatrix (src/initialPlace.cpp:185-378)
  void assemble(int axis, vector<Trip>& tr, vector<float>& rhs, vector<float>& x0) {
    const int nP = (int)placeInsts.size();
    rhs.assign(nP, 0.0f);
    x0.resize(nP);
    for (int k = 0; k < nP; k++) x0[k] = (float)(axis == 0 ? instCx(placeInsts[k]) : instCy(placeInsts[k]));
    tr.clear();
    const uint8_t bm = axis == 0 ? 3 : 12;
    const vector<int>& P = axis == 0 ? pinX : pinY;
    for (int n = 0; n < nNets; n++) {
      int s = netStart[n], e = netStart[n + 1];
      int deg = e - s;
      if (deg <= 1) continue;
      if (deg >= p.initial_place_max_fanout) continue;
      float w = p.initial_place_net_weight_scale / (deg - 1);
      for (int q1 = s; q1 < e; q1++) {
        for (int q2 = s; q2 < e; q2++) {
          if (q1 < q2) break;
          int i1 = pinInst[q1], i2 = pinInst[q2];
          if (i1 == i2) continue;
          if (!((bnd[q1] & bm) || (bnd[q2] & bm))) continue;
          int diff = std::abs(P[q1] - P[q2]);
          float wt = diff > p.initial_place_min_diff_length ? w / diff : w / p.initial_place_min_diff_length;
          bool m1 = i1 >= 0 && ikind[i1] == GPL_INST_PLACE;
          bool m2 = i2 >= 0 && ikind[i2] == GPL_INST_PLACE;
          int c1 = m1 ? (axis == 0 ? instCx(i1) : instCy(i1)) : 0;
          int c2 = m2 ? (axis == 0 ? instCx(i2) : instCy(i2)) : 0;
          if (m1 && m2) {
            int a = extId[i1], b = extId[i2];
            tr.push_back({a, a, wt}); tr.push_back({b, b, wt});
            tr.push_back({a, b, -wt}); tr.push_back({b, a, -wt});
            rhs[a] += -wt * ((P[q1] - c1) - (P[q2] - c2));
            rhs[b] += -wt * ((P[q2] - c2) - (P[q1] - c1));
          } else if (!m1 && m2) {
            int b = extId[i2];
            tr.push_back({b, b, wt});
            rhs[b] += wt * (P[q1] - (P[q2] - c2));
          } else if (m1 && !m2) {
            int a = extId[i1];
            tr.push_back({a, a, wt});
            rhs[a] += wt * (P[q2] - (P[q1] - c1));
          }
        }
      }
    }
  }

  // CSR from triplets with duplicates summed (Eigen setFromTriplets)
  static void toCsr(int n, vector<Trip>& tr, vector<int>& rp, vector<int>& ci, vector<float>& v) {
    std::stable_sort(tr.begin(), tr.end(), [](const Trip& a, const Trip& b) {
      return a.r != b.r ? a.r < b.r : a.c < b.c;
    });
    rp.assign(n + 1, 0); ci.clear(); v.clear();
    for (size_t k = 0; k < tr.size();) {
      size_t e = k;
      float s = 0.0f;
      while (e < tr.size() && tr[e].r == tr[k].r && tr[e].c == tr[k].c) { s += tr[e].v; e++; }
      ci.push_back(tr[k].c); v.push_back(s); rp[tr[k].r + 1]++;
      k = e;
    }
    for (int i = 0; i < n; i++) rp[i + 1] += rp[i];
  }

  static void spmv(const vector<int>& rp, const vector<int>& ci, const vector<float>& v,
                   const vector<float>& x, vector<float>& y) {
    int n = (int)rp.size() - 1;
    for (int i = 0; i < n; i++) {
      float s = 0.0f;
      for (int k = rp[i]; k < rp[i + 1]; k++) s += v[k] * x[ci[k]];
      y[i] = s;
    }
  }
  static double dot(const vector<float>& a, const vector<float>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); i++) s += (double)a[i] * (double)b[i];
    return s;
  }

  // BiCGSTAB (van der Vorst 1992), identity preconditioner, warm start;
  // stop when |r|^2 <= tol^2 |b|^2 (tol = FLT_EPSILON) or after maxIter;
  // restart from the true residual when rho becomes tiny.  Returns the
  // relative residual |r| / |b| (Eigen's solver.error()).
  static float bicgstab(const vector<int>& rp, const vector<int>& ci, const vector<float>& v,
                        const vector<float>& b, vector<float>& x, int maxIter, int* itersOut) {
    const int n = (int)b.size();
    const double tol = 1.1920928955078125e-07;
    vector<float> r(n), r0(n), p(n, 0.0f), vv(n, 0.0f), s(n), t(n), tmp(n);
    spmv(rp, ci, v, x, tmp);
    for (int i = 0; i < n; i++) r[i] = b[i] - tmp[i];
    r0 = r;
    double r0sq = dot(r0, r0);
    double rhsSq = dot(b, b);
    if (rhsSq == 0.0) { std::fill(x.begin(), x.end(), 0.0f); *itersOut = 0; return 0.0f; }
    double rho = 1, alpha = 1, w = 1;
    const double tol2 = tol * tol * rhsSq;
    const double eps2 = tol * tol;
    int it = 0, restarts = 0;
    while (dot(r, r) > tol2 && it < maxIter) {
      double rhoOld = rho;
      rho = dot(r0, r);
      if (std::fabs(rho) < eps2 * r0sq) {
        spmv(rp, ci, v, x, tmp);
        for (int i = 0; i < n; i++) r[i] = b[i] - tmp[i];
        r0 = r;
        rho = r0sq = dot(r, r);
        if (restarts++ == 0) it = 0;
      }
      double beta = (rho / rhoOld) * (alpha / w);
      for (int i = 0; i < n; i++) p[i] = (float)(r[i] + beta * (p[i] - w * vv[i]));
      spmv(rp, ci, v, p, vv);
      alpha = rho / dot(r0, vv);
      for (int i = 0; i < n; i++) s[i] = (float)(r[i] - alpha * vv[i]);
      spmv(rp, ci, v, s, t);
      double tt = dot(t, t);
      w = tt > 0.0 ? dot(t, s) / tt : 0.0;
      for (int i = 0; i < n; i++) x[i] = (float)(x[i] + alpha * p[i] + w * s[i]);
      for (int i = 0; i < n; i++) r[i] = (float)(s[i] - w * t[i]);
      it++;
    }
    *itersOut = it;
    return (float)sqrt(dot(r, r) / rhsSq);
  }

  // InitialPlace::doBicgstabPlace (src/initialPlace.cpp:56-105)
  int initialPlace(gpl_ip_stats* st) {
    if (!p.incremental_place_mode) {
      const int cx = (coreLx + coreUx) / 2, cy = (coreLy + coreUy) / 2;
      for (int i : placeInsts) setInstCenter(i, cx, cy);
    }
    extId.assign(nInst, -1);
    for (size_t k = 0; k < placeInsts.size(); k++) extId[placeInsts[k]] = (int)k;
    const int nP = (int)placeInsts.size();
    float err = 0.0f;
    int itx = 0, ity = 0, rounds = 0;
    for (int i = 1; i <= p.initial_place_max_iter; i++) {
      updatePinInfo();
      vector<Trip> tr;
      vector<float> bx, by, xx, xy;
      vector<int> rpx, cix, rpy, ciy;
      vector<float> vx, vy;
      assemble(0, tr, bx, xx);
      toCsr(nP, tr, rpx, cix, vx);
      assemble(1, tr, by, xy);
      toCsr(nP, tr, rpy, ciy, vy);
      float ex = bicgstab(rpx, cix, vx, bx, xx, p.initial_place_max_solver_iter, &itx);
      float ey = bicgstab(rpy, ciy, vy, by, xy, p.initial_place_max_solver_iter, &ity);
      err = std::max(ex, ey);
      for (int k = 0; k < nP; k++) setInstCenter(placeInsts[k], (int)xx[k], (int)xy[k]);
      rounds = i;
      if (err <= 1e-5 && i >= 5) break;
    }
    if (st) {
      st->iterations = rounds;
      st->last_error = err;
      st->last_hpwl = 0;
      st->solver_iters_x = itx;
      st->solver_iters_y = ity;
    }
    return GPL_OK;
  }
};

}  // namespace

extern "C" {

void* orc_create(const gpl_netlist_desc* d, const gpl_params* p, int* status) {
  Oracle* o = new Oracle();
  int rc = o->build(d, p);
  if (status) *status = rc;
  if (rc) { delete o; return nullptr; }
  return o;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

int orc_set_net_weights(void* h, const float* w, int64_t n) {
  Oracle* o = (Oracle*)h;
  if (!w) { o->netW.clear(); return 0; }
  if (n != o->nNets) return 1;
  o->netW.assign(w, w + n);
  return 0;
}

int orc_initial_place(void* h, gpl_ip_stats* st) { return ((Oracle*)h)->initialPlace(st); }

static void fill_info(Oracle* o, gpl_job_info* info) {
  if (!info) return;
  memset(info, 0, sizeof(*info));
  info->n_place_insts = o->nPlace;
  info->n_gcells = o->nG;
  info->n_fillers = o->nFill;
  info->bin_cnt_x = o->cntX; info->bin_cnt_y = o->cntY;
  info->bin_size_x = o->sizeX; info->bin_size_y = o->sizeY;
  info->filler_dx = o->fillDx; info->filler_dy = o->fillDy;
  info->place_insts_area = o->placeArea; info->std_insts_area = o->stdArea;
  info->macro_insts_area = o->macroArea; info->non_place_insts_area = o->nonPlaceArea;
}

// NesterovBase construction only (no NesterovPlace::init)
int orc_nesterov_base(void* h, gpl_job_info* info) {
  Oracle* o = (Oracle*)h;
  int rc = o->nbReady ? GPL_OK : o->initNesterovBase();
  if (rc == GPL_OK) { o->buildPinNet(); fill_info(o, info); }
  return rc;
}

int orc_nesterov_init(void* h, gpl_job_info* info) {
  Oracle* o = (Oracle*)h;
  int rc = o->nbReady ? GPL_OK : o->initNesterovBase();
  if (rc) return rc;
  fill_info(o, info);
  return o->initNesterovPlace();
}

int orc_nesterov_run(void* h, int max_iters, gpl_nesterov_stats* st, gpl_iter_log* log) {
  Oracle* o = (Oracle*)h;
  int rc = o->run(max_iters, log);
  if (st) {
    st->iterations = o->iter;
    st->evaluations = o->evals;
    st->finished = o->finished;
    st->status = o->divergeCode;
    st->overflow = o->sumOverflow;
    st->step_length = o->stepLength;
    st->density_penalty = o->densityPenalty;
    st->wire_length_coef = o->wlCoefX;
    st->hpwl = o->prevHpwl;
  }
  return rc;
}

// Reference-typed scalars of the last evaluation, in addition to gpl_eval_stats:
// [0] overflowArea as the reference accumulates it (float-evaluated int64)
// [1] sumPhi as the reference accumulates it (float)
// [2] wireLengthGradSum (float, sequential)  [3] densityGradSum (float, sequential)
int orc_eval(void* h, const float* xy, float cx, float cy, float* wl, float* dg,
             gpl_eval_stats* st, double* ref_scalars) {
  Oracle* o = (Oracle*)h;
  if (!o->nbReady) return GPL_ERR_BAD_STATE;
  vector<FP> c(o->nG);
  for (int g = 0; g < o->nG; g++) c[g] = FP(xy[2 * g], xy[2 * g + 1]);
  o->setDensityCenters(c);
  o->scatter();
  o->densityForce();
  o->waForce(cx, cy);
  double wsum = 0, dsum = 0;
  float wsf = 0, dsf = 0;
  for (int g = 0; g < o->nG; g++) {
    FP a = o->wlGrad(g, cx, cy);
    FP b = o->densityGrad(g);
    if (wl) { wl[2 * g] = a.x; wl[2 * g + 1] = a.y; }
    if (dg) { dg[2 * g] = b.x; dg[2 * g + 1] = b.y; }
    wsum += std::fabs((double)a.x) + std::fabs((double)a.y);
    dsum += std::fabs((double)b.x) + std::fabs((double)b.y);
    wsf += std::fabs(a.x); wsf += std::fabs(a.y);
    dsf += std::fabs(b.x); dsf += std::fabs(b.y);
  }
  if (st) {
    st->overflow_area_f64 = o->overflowF64;
    st->overflow_area = (int64_t)o->overflowF64;
    st->hpwl = o->hpwl();
    st->sum_phi = o->sumPhiF64;
    st->wire_length_grad_sum = wsum;
    st->density_grad_sum = dsum;
  }
  if (ref_scalars) {
    ref_scalars[0] = (double)o->overflowArea;
    ref_scalars[1] = (double)o->sumPhi;
    ref_scalars[2] = (double)wsf;
    ref_scalars[3] = (double)dsf;
  }
  return GPL_OK;
}

int orc_get_bins(void* h, int64_t* inst, int64_t* fill, int64_t* np, float* dens,
                 float* phi, float* ex, float* ey) {
  Oracle* o = (Oracle*)h;
  size_t nb = (size_t)o->cntX * o->cntY;
  for (size_t b = 0; b < nb; b++) {
    if (inst) inst[b] = o->bInst[b];
    if (fill) fill[b] = o->bFill[b];
    if (np) np[b] = o->bNonPlace[b];
    if (dens) dens[b] = o->bDensity[b];
    if (phi) phi[b] = o->bPhi[b];
    if (ex) ex[b] = o->bEx[b];
    if (ey) ey[b] = o->bEy[b];
  }
  return GPL_OK;
}

int orc_get_gcells(void* h, int32_t* drect, float* scale, uint8_t* kind) {
  Oracle* o = (Oracle*)h;
  for (int g = 0; g < o->nG; g++) {
    if (drect) { drect[4 * g] = o->gdlx[g]; drect[4 * g + 1] = o->gdly[g];
                 drect[4 * g + 2] = o->gdux[g]; drect[4 * g + 3] = o->gduy[g]; }
    if (scale) scale[g] = o->gscale[g];
    if (kind) kind[g] = o->gkind[g];
  }
  return GPL_OK;
}

int orc_get_gcell_coords(void* h, float* xy) {
  Oracle* o = (Oracle*)h;
  if ((int)o->curSLP.size() < o->nG) return GPL_ERR_BAD_STATE;   // before nesterov_init
  for (int g = 0; g < o->nG; g++) { xy[2 * g] = o->curSLP[g].x; xy[2 * g + 1] = o->curSLP[g].y; }
  return GPL_OK;
}

// NesterovPlace::updateDb (src/nesterovPlace.cpp:585-595); before the
// Nesterov stage, the instances' current (initial-place) locations.
int orc_get_inst_locations(void* h, int32_t* lx, int32_t* ly) {
  Oracle* o = (Oracle*)h;
  for (int i = 0; i < o->nInst; i++) { lx[i] = o->ilx[i]; ly[i] = o->ily[i]; }
  if (o->nbReady) {
    for (int k = 0; k < o->nPlace; k++) {
      int i = o->placeInsts[k];
      int dcx = (o->gdux[k] + o->gdlx[k]) / 2, dcy = (o->gduy[k] + o->gdly[k]) / 2;
      lx[i] = dcx - (o->gdux[k] - o->gdlx[k]) / 2;
      ly[i] = dcy - (o->gduy[k] - o->gdly[k]) / 2;
    }
  }
  return GPL_OK;
}

// Current pin centres as PlacerBase sees them (after the initial place)
int orc_get_pins(void* h, int32_t* x, int32_t* y) {
  Oracle* o = (Oracle*)h;
  for (int q = 0; q < o->nPins; q++) { x[q] = o->pinX[q]; y[q] = o->pinY[q]; }
  return GPL_OK;
}

// Standalone Poisson solve (FFT::doFFT) in FP64; arrays row-major by y.
void orc_poisson_f64(int nx, int ny, int bsx, int bsy, const double* rho, double* phi,
                     double* ex, double* ey) {
  poisson_f64(nx, ny, bsx, bsy, rho, phi, ex, ey);
}

// Direct O(N^2) per-axis transforms for validating the FFT path on small grids:
// kind 0 DCT-II, 1 DCT-III, 2 IDST (a[0] = A[N]); one vector of length n.
void orc_transform_direct(int kind, int n, const double* a, double* out) {
  for (int m = 0; m < n; m++) {
    long double s = 0;
    for (int k = 0; k < n; k++) {
      if (kind == 0) s += a[k] * cosl(kPi * (k + 0.5L) * m / n);
      else if (kind == 1) s += a[k] * cosl(kPi * k * (m + 0.5L) / n);
      else {
        int kk = k == 0 ? n : k;
        s += a[k] * sinl(kPi * kk * (m + 0.5L) / n);
      }
    }
    out[m] = (double)s;
  }
}

void orc_transform_fft(int kind, int n, const double* a, double* out) {
  Dct1 t;
  t.init(n);
  if (kind == 0) t.dct2(a, out);
  else if (kind == 1) t.dct3(a, out);
  else t.idst(a, out);
}

}  // extern "C"
