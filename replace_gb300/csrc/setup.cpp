// Host-side job setup: the once-per-job work of PlacerBase, NesterovBase and
// BinGrid.  It runs on the host in O(cells + pins + nonplace*bins) and must
// be bit-exact with the reference (integer geometry, mt19937 filler positions,
// float density scales), because every later kernel consumes its output.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <random>

#include "gpl_internal.h"

namespace gpl {

namespace {
const long double kSqrt2 = 1.414213562373095048801L;   // REPLACE_SQRT2

inline int fast_modulo(int input, int ceil) { return input >= ceil ? input % ceil : input; }
}  // namespace

// PlacerBase::init bookkeeping (src/placerBase.cpp:639-680) and the
// utilisation check of PlacerBase::printInfo (:936-956).
int build_placer_base(HostModel& m, const gpl_netlist_desc* d, const gpl_params* p) {
  if (!d || !p) { set_error("null netlist or params"); return GPL_ERR_INVALID_ARG; }
  if (d->n_insts <= 0 || d->n_nets < 0 || d->n_pins < 0 || !d->inst_lx || !d->inst_ly ||
      !d->inst_ux || !d->inst_uy || !d->inst_kind || !d->net_start ||
      (d->n_pins > 0 && (!d->pin_inst || !d->pin_ox || !d->pin_oy || !d->pin_x || !d->pin_y))) {
    set_error("incomplete netlist descriptor");
    return GPL_ERR_INVALID_ARG;
  }
  if (d->core_ux <= d->core_lx || d->core_uy <= d->core_ly || d->site_w <= 0 || d->site_h <= 0) {
    set_error("empty core area or site");
    return GPL_ERR_INVALID_ARG;
  }
  m.p = *p;
  m.core_lx = d->core_lx; m.core_ly = d->core_ly; m.core_ux = d->core_ux; m.core_uy = d->core_uy;
  m.site_w = d->site_w; m.site_h = d->site_h;
  m.n_insts = d->n_insts; m.n_pins = d->n_pins; m.n_nets = d->n_nets;
  m.ilx.assign(d->inst_lx, d->inst_lx + m.n_insts);
  m.ily.assign(d->inst_ly, d->inst_ly + m.n_insts);
  m.iux.assign(d->inst_ux, d->inst_ux + m.n_insts);
  m.iuy.assign(d->inst_uy, d->inst_uy + m.n_insts);
  m.ikind.assign(d->inst_kind, d->inst_kind + m.n_insts);
  m.net_start.assign(d->net_start, d->net_start + m.n_nets + 1);
  // the per-pin copies and checks in parallel ranges
  m.pin_inst.resize(m.n_pins); m.pin_ox.resize(m.n_pins); m.pin_oy.resize(m.n_pins);
  m.pin_x.resize(m.n_pins); m.pin_y.resize(m.n_pins);
  int bad_pin = 0;
  parallel_ranges(m.n_pins, [&](int a, int b) {
    const size_t w = (size_t)(b - a) * sizeof(int32_t);
    memcpy(m.pin_inst.data() + a, d->pin_inst + a, w);
    memcpy(m.pin_ox.data() + a, d->pin_ox + a, w);
    memcpy(m.pin_oy.data() + a, d->pin_oy + a, w);
    memcpy(m.pin_x.data() + a, d->pin_x + a, w);
    memcpy(m.pin_y.data() + a, d->pin_y + a, w);
    bool bad = false;
    for (int q = a; q < b; q++) bad |= m.pin_inst[q] < -1 || m.pin_inst[q] >= m.n_insts;
    if (bad) __atomic_store_n(&bad_pin, 1, __ATOMIC_RELAXED);
  });
  if (m.net_start[0] != 0 || m.net_start[m.n_nets] != m.n_pins) {
    set_error("net_start must run from 0 to n_pins");
    return GPL_ERR_INVALID_ARG;
  }
  for (int n = 0; n < m.n_nets; n++) {
    if (m.net_start[n + 1] < m.net_start[n]) { set_error("net_start not monotone"); return GPL_ERR_INVALID_ARG; }
    if (m.net_start[n + 1] == m.net_start[n]) {
      // NesterovBase::getHpwl over an empty net overflows int arithmetic in
      // the reference; such nets are rejected here.
      set_error("net without pins");
      return GPL_ERR_INVALID_ARG;
    }
  }
  if (bad_pin) { set_error("pin_inst out of range"); return GPL_ERR_INVALID_ARG; }
  if (d->inst_pin_start && d->inst_pins) {
    m.inst_pin_start.assign(d->inst_pin_start, d->inst_pin_start + m.n_insts + 1);
    int np = m.inst_pin_start[m.n_insts];
    if (np < 0 || np > m.n_pins) { set_error("inst_pin_start out of range"); return GPL_ERR_INVALID_ARG; }
    m.inst_pins.assign(d->inst_pins, d->inst_pins + np);
    for (int i = 0; i < m.n_insts; i++)
      if (m.inst_pin_start[i + 1] < m.inst_pin_start[i]) { set_error("inst_pin_start not monotone"); return GPL_ERR_INVALID_ARG; }
    if (m.inst_pin_start[0] < 0) { set_error("inst_pin_start out of range"); return GPL_ERR_INVALID_ARG; }
    // every instance pin listed exactly once, under its own instance (the
    // seen bitmap is shared by the ranges: atomic bit sets)
    std::vector<uint64_t> seen(((size_t)m.n_pins + 63) / 64, 0);
    int bad_owner = 0, twice = 0;
    long long inst_owned = 0;
    parallel_ranges(m.n_insts, [&](int a, int b) {
      bool bo = false, tw = false;
      for (int i = a; i < b && !bo; i++) {
        for (int k = m.inst_pin_start[i]; k < m.inst_pin_start[i + 1]; k++) {
          const int q = m.inst_pins[k];
          if (q < 0 || q >= m.n_pins || m.pin_inst[q] != i) { bo = true; break; }
          const uint64_t bit = 1ull << (q & 63);
          if (__atomic_fetch_or(&seen[q >> 6], bit, __ATOMIC_RELAXED) & bit) tw = true;
        }
      }
      if (bo) __atomic_store_n(&bad_owner, 1, __ATOMIC_RELAXED);
      if (tw) __atomic_store_n(&twice, 1, __ATOMIC_RELAXED);
    });
    if (bad_owner) { set_error("inst_pins inconsistent with pin_inst"); return GPL_ERR_INVALID_ARG; }
    if (twice) { set_error("inst_pins lists a pin twice"); return GPL_ERR_INVALID_ARG; }
    parallel_ranges(m.n_pins, [&](int a, int b) {
      long long c = 0;
      for (int q = a; q < b; q++) c += m.pin_inst[q] >= 0;
      __atomic_fetch_add(&inst_owned, c, __ATOMIC_RELAXED);
    });
    if (inst_owned != np) { set_error("inst_pins must list every pin of every instance"); return GPL_ERR_INVALID_ARG; }
  } else {
    m.inst_pin_start.assign(m.n_insts + 1, 0);
    for (int q = 0; q < m.n_pins; q++) if (m.pin_inst[q] >= 0) m.inst_pin_start[m.pin_inst[q] + 1]++;
    for (int i = 0; i < m.n_insts; i++) m.inst_pin_start[i + 1] += m.inst_pin_start[i];
    m.inst_pins.assign(m.inst_pin_start[m.n_insts], 0);
    std::vector<int32_t> fill(m.inst_pin_start.begin(), m.inst_pin_start.end() - 1);
    for (int q = 0; q < m.n_pins; q++) if (m.pin_inst[q] >= 0) m.inst_pins[fill[m.pin_inst[q]]++] = q;
  }
  for (int i = 0; i < m.n_insts; i++) {
    int64_t a = (int64_t)(m.iux[i] - m.ilx[i]) * (int64_t)(m.iuy[i] - m.ily[i]);
    switch (m.ikind[i]) {
      case GPL_INST_PLACE:
        m.place_insts.push_back(i);
        m.place_area += a;
        if (m.iuy[i] - m.ily[i] > m.site_h * 6) m.macro_area += a; else m.std_area += a;
        break;
      case GPL_INST_FIXED: {
        m.non_place_insts.push_back(i);
        int rlx = std::max(m.core_lx, m.ilx[i]), rly = std::max(m.core_ly, m.ily[i]);
        int rux = std::min(m.core_ux, m.iux[i]), ruy = std::min(m.core_uy, m.iuy[i]);
        if (rlx < rux && rly < ruy) m.non_place_area += (int64_t)(rux - rlx) * (int64_t)(ruy - rly);
        break;
      }
      case GPL_INST_DUMMY:
        m.non_place_insts.push_back(i);
        m.non_place_area += a;
        break;
      case GPL_INST_OUTSIDE:
        break;
      default:
        set_error("unknown instance kind");
        return GPL_ERR_INVALID_ARG;
    }
  }
  if (m.place_insts.empty()) { set_error("no movable instances"); return GPL_ERR_INVALID_ARG; }
  int64_t core_area = (int64_t)(m.core_ux - m.core_lx) * (int64_t)(m.core_uy - m.core_ly);
  float util = (float)m.place_area / (core_area - m.non_place_area) * 100;
  if (util >= 100.1) {
    set_error("Util exceeds 100%. Please double-check your die/row size");
    return GPL_ERR_UTIL;
  }
  return GPL_OK;
}

void host_set_inst_center(HostModel& m, int i, int x, int y) {
  // Instance::setCenterLocation (src/placerBase.cpp:127-140): the box keeps
  // 2*(dx/2) width.  The instance's pins are not stored: a movable
  // instance's pin is always its centre plus the pin offset.
  const int hx = (m.iux[i] - m.ilx[i]) / 2, hy = (m.iuy[i] - m.ily[i]) / 2;
  m.ilx[i] = x - hx; m.ily[i] = y - hy; m.iux[i] = x + hx; m.iuy[i] = y + hy;
}

void host_place_center(HostModel& m) {
  // InitialPlace::placeInstsCenter (src/initialPlace.cpp:108-115)
  const int cx = (m.core_lx + m.core_ux) / 2, cy = (m.core_ly + m.core_uy) / 2;
  for (int i : m.place_insts) host_set_inst_center(m, i, cx, cy);
}

// NesterovBase::init (src/nesterovBase.cpp:917-1062) with initFillerGCells
// (:1066-1155) and BinGrid::initBins / updateBinsNonPlaceArea (:631-741).
// Filler size and count (NesterovBase::initFillerGCells, src/nesterovBase.cpp:
// 1066-1155) and the bin grid (BinGrid::initBins, :631-717): the counts that
// size a job, independent of the instances' positions.
int nb_counts(const HostModel& m, NbCounts* c, const PlaceRects* rects) {
  const gpl_params& p = m.p;
  const int n_place = (int)m.place_insts.size();
  {
    std::vector<int> dxs, dys;
    dxs.reserve(n_place); dys.reserve(n_place);
    if (rects) {
      for (int k = 0; k < n_place; k++) { dxs.push_back(rects->ux[k] - rects->lx[k]); dys.push_back(rects->uy[k] - rects->ly[k]); }
    } else {
      for (int i : m.place_insts) { dxs.push_back(m.iux[i] - m.ilx[i]); dys.push_back(m.iuy[i] - m.ily[i]); }
    }
    int min_idx = (int)(dxs.size() * 0.05);
    int max_idx = (int)(dxs.size() * 0.95);
    if (max_idx <= min_idx) { set_error("too few movable instances for the filler size"); return GPL_ERR_INVALID_ARG; }
    // The reference sums ranks [min_idx, max_idx) of the sorted sizes.  Two
    // selections put exactly those ranks' values into [min_idx, max_idx)
    // (in some order), so the sum is the same without a full sort.
    auto mid_sum = [&](std::vector<int>& v) {
      std::nth_element(v.begin(), v.begin() + min_idx, v.end());
      std::nth_element(v.begin() + min_idx, v.begin() + max_idx, v.end());
      int64_t s = 0;
      for (int k = min_idx; k < max_idx; k++) s += v[k];
      return s;
    };
    const int64_t dx_sum = mid_sum(dxs), dy_sum = mid_sum(dys);
    c->fill_dx = (int)(dx_sum / (max_idx - min_idx));
    c->fill_dy = (int)(dy_sum / (max_idx - min_idx));
    int64_t core_area = (int64_t)(m.core_ux - m.core_lx) * (int64_t)(m.core_uy - m.core_ly);
    int64_t white = core_area - m.non_place_area;
    int64_t movable = (int64_t)(white * p.target_density);
    int64_t total_filler = movable - m.std_area - (int64_t)(m.macro_area * p.target_density);
    if (total_filler < 0) {
      set_error("Filler area is negative!! Please put higher target density or re-floorplan to have enough coreArea");
      return GPL_ERR_FILLER_AREA;
    }
    c->n_fill = (int)(total_filler / (int64_t)(c->fill_dx * c->fill_dy));
  }
  int64_t total_bin_area = (int64_t)(m.core_ux - m.core_lx) * (int64_t)(m.core_uy - m.core_ly);
  int64_t avg_area = m.place_area / (int64_t)n_place;
  int64_t ideal_bin_area = (int64_t)std::round((float)avg_area / p.target_density);
  if (ideal_bin_area <= 0) { set_error("degenerate ideal bin area"); return GPL_ERR_INVALID_ARG; }
  int ideal_bin_cnt = (int)(total_bin_area / ideal_bin_area);
  int found = 2;
  for (found = 2; found <= 1024; found *= 2)
    if (found * found <= ideal_bin_cnt && 4 * found * found > ideal_bin_cnt) break;
  c->cnt_x = p.bin_grid_cnt_x > 0 ? p.bin_grid_cnt_x : found;
  c->cnt_y = p.bin_grid_cnt_y > 0 ? p.bin_grid_cnt_y : found;
  auto pow2 = [](int v) { return v >= 2 && (v & (v - 1)) == 0; };
  if (!pow2(c->cnt_x) || !pow2(c->cnt_y) || c->cnt_x > kFftMax || c->cnt_y > kFftMax) {
    // The DCT (Ooura's and ours) needs power-of-two sizes.
    set_error("bin counts must be powers of two in [2, 4096]");
    return GPL_ERR_INVALID_ARG;
  }
  c->size_x = (int)ceil((float)(m.core_ux - m.core_lx) / c->cnt_x);
  c->size_y = (int)ceil((float)(m.core_uy - m.core_ly) / c->cnt_y);
  // BinGrid::initBins lays bins out by walking x in steps of binSize and
  // wrapping at the core edge; that walk yields cnt bins per row only if
  // (cnt - 1) * binSize < core width.  Finer grids misalign the reference's
  // bin indexing, so they are rejected.
  if ((int64_t)(c->cnt_x - 1) * c->size_x >= (m.core_ux - m.core_lx) ||
      (int64_t)(c->cnt_y - 1) * c->size_y >= (m.core_uy - m.core_ly)) {
    set_error("bin grid finer than the core allows (reference bin layout would wrap early)");
    return GPL_ERR_INVALID_ARG;
  }
  return GPL_OK;
}

PlaceRects place_rects(const HostModel& m) {
  PlaceRects r;
  const size_t n = m.place_insts.size();
  r.lx.resize(n); r.ly.resize(n); r.ux.resize(n); r.uy.resize(n);
  for (size_t k = 0; k < n; k++) {
    const int i = m.place_insts[k];
    r.lx[k] = m.ilx[i]; r.ly[k] = m.ily[i]; r.ux[k] = m.iux[i]; r.uy[k] = m.iuy[i];
  }
  return r;
}

// Everything of NesterovBase but the movable gcells' positions.  The
// movable instances' rectangles come from `rects` (a copy taken when their
// sizes are final: the initial place moves instances but keeps their sizes),
// so that this can run beside an initial place that moves the instances; it
// reads no other per-instance state that the initial place writes.
int build_nesterov_static(HostModel& m, const PlaceRects& rects) {
  const gpl_params& p = m.p;
  NbCounts nc;
  int rc = nb_counts(m, &nc, &rects);
  if (rc) return rc;
  m.glx.clear(); m.gly.clear(); m.gux.clear(); m.guy.clear(); m.gkind.clear();
  m.n_place = (int)m.place_insts.size();
  const size_t n_all = (size_t)m.n_place + (size_t)std::max(nc.n_fill, 0);
  m.glx.reserve(n_all); m.gly.reserve(n_all); m.gux.reserve(n_all); m.guy.reserve(n_all); m.gkind.reserve(n_all);
  for (int k = 0; k < m.n_place; k++) {
    m.glx.push_back(rects.lx[k]); m.gly.push_back(rects.ly[k]);
    m.gux.push_back(rects.ux[k]); m.guy.push_back(rects.uy[k]);
    m.gkind.push_back((rects.uy[k] - rects.ly[k]) > m.site_h * 6 ? 1 : 0);
  }
  // fillers: mt19937(0) centres
  m.fill_dx = nc.fill_dx;
  m.fill_dy = nc.fill_dy;
  {
    const int cnt = nc.n_fill;
    std::mt19937 rv(0);
    const int cdx = m.core_ux - m.core_lx, cdy = m.core_uy - m.core_ly;
    for (int k = 0; k < cnt; k++) {
      auto rx = rv();
      auto ry = rv();
      int cx = (int)(rx % (unsigned)cdx + m.core_lx);
      int cy = (int)(ry % (unsigned)cdy + m.core_ly);
      m.glx.push_back(cx - m.fill_dx / 2); m.gly.push_back(cy - m.fill_dy / 2);
      m.gux.push_back(cx + m.fill_dx / 2); m.guy.push_back(cy + m.fill_dy / 2);
      m.gkind.push_back(2);
    }
    m.n_fill = cnt;
  }
  m.n_g = (int)m.glx.size();
  // gcell -> pins in instance pin order; pin -> gcell (inst_pins lists
  // every pin of an instance exactly once, checked by build_placer_base)
  m.g_pin_start.assign(m.n_g + 1, 0);
  m.g_pins.clear();
  {
    std::vector<int32_t> g_of_inst(m.n_insts, -1);
    size_t total = 0;
    for (int k = 0; k < m.n_place; k++) {
      const int i = m.place_insts[k];
      g_of_inst[i] = k;
      total += m.inst_pin_start[i + 1] - m.inst_pin_start[i];
    }
    m.g_pins.reserve(total);
    for (int k = 0; k < m.n_place; k++) {
      const int i = m.place_insts[k];
      m.g_pins.insert(m.g_pins.end(), m.inst_pins.begin() + m.inst_pin_start[i],
                      m.inst_pins.begin() + m.inst_pin_start[i + 1]);
      m.g_pin_start[k + 1] = (int)m.g_pins.size();
    }
    m.pin_g.resize(m.n_pins);
    for (int q = 0; q < m.n_pins; q++) {
      const int i = m.pin_inst[q];
      m.pin_g[q] = i >= 0 ? g_of_inst[i] : -1;
    }
  }
  for (int k = m.n_place; k < m.n_g; k++) m.g_pin_start[k + 1] = m.g_pin_start[k];

  // bin grid
  m.cnt_x = nc.cnt_x; m.cnt_y = nc.cnt_y;
  m.size_x = nc.size_x; m.size_y = nc.size_y;
  const int nb = m.cnt_x * m.cnt_y;
  m.bin_nonplace.assign(nb, 0);
  auto bin_lo_x = [&](int a) { return m.core_lx + a * m.size_x; };
  auto bin_hi_x = [&](int a) { return std::min(m.core_lx + (a + 1) * m.size_x, m.core_ux); };
  auto bin_lo_y = [&](int c) { return m.core_ly + c * m.size_y; };
  auto bin_hi_y = [&](int c) { return std::min(m.core_ly + (c + 1) * m.size_y, m.core_uy); };
  for (int i : m.non_place_insts) {
    int lo_x = std::max((m.ilx[i] - m.core_lx) / m.size_x, 0);
    int hi_x = std::min(fast_modulo(m.iux[i] - m.core_lx, m.size_x) == 0
                            ? (m.iux[i] - m.core_lx) / m.size_x
                            : (m.iux[i] - m.core_lx) / m.size_x + 1, m.cnt_x);
    int lo_y = std::max((m.ily[i] - m.core_ly) / m.size_y, 0);
    int hi_y = std::min(fast_modulo(m.iuy[i] - m.core_ly, m.size_y) == 0
                            ? (m.iuy[i] - m.core_ly) / m.size_y
                            : (m.iuy[i] - m.core_ly) / m.size_y + 1, m.cnt_y);
    for (int a = lo_x; a < hi_x; a++) {
      for (int c = lo_y; c < hi_y; c++) {
        int rlx = std::max(bin_lo_x(a), m.ilx[i]), rly = std::max(bin_lo_y(c), m.ily[i]);
        int rux = std::min(bin_hi_x(a), m.iux[i]), ruy = std::min(bin_hi_y(c), m.iuy[i]);
        int64_t ov = (rlx >= rux || rly >= ruy) ? 0 : (int64_t)(rux - rlx) * (int64_t)(ruy - rly);
        // getOverlapArea * targetDensity: int64 * float evaluated in float
        m.bin_nonplace[(size_t)c * m.cnt_x + a] += (int64_t)(ov * p.target_density);
      }
    }
  }
  // density size and scale (src/nesterovBase.cpp:1033-1061); the comparison
  // and the size are evaluated in long double as in the reference
  m.gdlx = m.glx; m.gdly = m.gly; m.gdux = m.gux; m.gduy = m.guy;
  m.gscale.assign(m.n_g, 0.0f);
  // The long double terms depend on the bin size only, so they are formed
  // once (long double is a software type on some hosts).  For an integer d,
  // d < sqrt2 * size  <=>  d < ceil(sqrt2 * size).
  const long double thx = kSqrt2 * m.size_x, thy = kSqrt2 * m.size_y;
  const int64_t lim_x = (int64_t)ceill(thx), lim_y = (int64_t)ceill(thy);
  const float den_x = (float)thx, den_y = (float)thy;
  const float small_dsx = (float)(kSqrt2 * (float)m.size_x), small_dsy = (float)(kSqrt2 * (float)m.size_y);
  for (int g = 0; g < m.n_g; g++) {
    int dx = m.gux[g] - m.glx[g], dy = m.guy[g] - m.gly[g];
    float sx, sy, dsx, dsy;
    if (dx < lim_x) {
      sx = (float)dx / den_x;
      dsx = small_dsx;
    } else { sx = 1.0f; dsx = (float)dx; }
    if (dy < lim_y) {
      sy = (float)dy / den_y;
      dsy = small_dsy;
    } else { sy = 1.0f; dsy = (float)dy; }
    int ddx = (int)dsx, ddy = (int)dsy;   // GCell::setDensitySize(int, int)
    int cx = (m.gdux[g] + m.gdlx[g]) / 2, cy = (m.gduy[g] + m.gdly[g]) / 2;
    m.gdlx[g] = cx - ddx / 2; m.gdly[g] = cy - ddy / 2;
    m.gdux[g] = cx + ddx / 2; m.gduy[g] = cy + ddy / 2;
    m.gscale[g] = sx * sy;
  }
  return GPL_OK;
}

// The movable gcells' real and density rectangles at the instances' current
// positions (GCell(Instance*) and setDensityCenterLocation: the density
// rectangle keeps its size and the real rectangle's centre).
void place_gcells(HostModel& m) {
  for (int k = 0; k < m.n_place; k++) {
    const int i = m.place_insts[k];
    const int hx = (m.gdux[k] - m.gdlx[k]) / 2, hy = (m.gduy[k] - m.gdly[k]) / 2;
    m.glx[k] = m.ilx[i]; m.gly[k] = m.ily[i]; m.gux[k] = m.iux[i]; m.guy[k] = m.iuy[i];
    const int cx = (m.gux[k] + m.glx[k]) / 2, cy = (m.guy[k] + m.gly[k]) / 2;
    m.gdlx[k] = cx - hx; m.gdly[k] = cy - hy;
    m.gdux[k] = cx + hx; m.gduy[k] = cy + hy;
  }
}

int build_nesterov_base(HostModel& m) {
  int rc = build_nesterov_static(m, place_rects(m));
  if (rc) return rc;
  place_gcells(m);
  return GPL_OK;
}

void make_twiddle(std::vector<float2>& tw) {
  tw.resize(kFftMax / 2);
  for (int k = 0; k < kFftMax / 2; k++) {
    double a = -2.0 * M_PI * (double)k / (double)kFftMax;
    tw[k] = make_float2((float)cos(a), (float)sin(a));
  }
}

// FFT::init (src/fft.cpp:78-90): wx[i] = pi*i/nx, wy[j] = pi*j/ny*bsy/bsx,
// evaluated in long double and stored as float.
void make_freq(int nx, int ny, int bsx, int bsy, std::vector<float>& wx, std::vector<float>& wy) {
  const long double kPi = 3.141592653589793238462L;
  wx.resize(nx);
  wy.resize(ny);
  for (int i = 0; i < nx; i++) wx[i] = (float)(kPi * (float)i / (float)nx);
  for (int j = 0; j < ny; j++) wy[j] = (float)(kPi * (float)j / (float)ny * (float)bsy / (float)bsx);
}

}  // namespace gpl
