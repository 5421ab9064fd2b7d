#include "placer_base.h"

#include <opendb/db.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <unordered_map>

#include "logger.h"

namespace replace {

GplJob::~GplJob() {
  if (job) gpl_destroy(job);
}

namespace {

bool is_fixed_status(odb::dbPlacementStatus s) {
  // Instance::isFixed (src/placerBase.cpp:72-91)
  switch (s) {
    case odb::dbPlacementStatus::LOCKED:
    case odb::dbPlacementStatus::FIRM:
    case odb::dbPlacementStatus::COVER:
      return true;
    default:
      return false;
  }
}

// Site index range [lo, hi) of the span [ll, uu) on a grid of `cnt` sites
// starting at c0: the lower index truncates, the upper rounds up
// (getMinMaxIdx, src/placerBase.cpp:984-993, C integer division).
void site_range(int ll, int uu, int c0, int site, int cnt, int& lo, int& hi) {
  lo = std::max(0, (ll - c0) / site);
  const int d = uu - c0;
  const int up = (d >= site ? d % site : d) == 0 ? d / site : d / site + 1;
  hi = std::min(cnt, up);
}

}  // namespace

PlacerBase::PlacerBase() { gpl_params_default(&base_params_); }

PlacerBase::PlacerBase(odb::dbDatabase* db, std::shared_ptr<Logger> log)
    : db_(db), log_(std::move(log)) {
  gpl_params_default(&base_params_);
  base_params_.verbose_level = log_ ? log_->verbose() : 0;
  init();
}

PlacerBase::~PlacerBase() = default;

void PlacerBase::init() {
  odb::dbBlock* block = db_->getChip()->getBlock();
  if (log_) log_->infoInt("DBU", db_->getTech()->getDbUnitsPerMicron());

  // core = bounding box of the rows; site size from the first row
  core_lx_ = core_ly_ = INT_MAX;
  core_ux_ = core_uy_ = INT_MIN;
  bool first = true;
  for (odb::dbRow* row : block->getRows()) {
    odb::Rect r;
    row->getBBox(r);
    core_lx_ = std::min(core_lx_, r.xMin());
    core_ly_ = std::min(core_ly_, r.yMin());
    core_ux_ = std::max(core_ux_, r.xMax());
    core_uy_ = std::max(core_uy_, r.yMax());
    if (first) {
      site_w_ = row->getSite()->getWidth();
      site_h_ = row->getSite()->getHeight();
      first = false;
    }
  }
  if (first && log_) log_->error("the block has no rows", 1);
  odb::dbBox* die = block->getBBox();
  die_lx_ = die->xMin(); die_ly_ = die->yMin(); die_ux_ = die->xMax(); die_uy_ = die->yMax();
  if (log_) {
    log_->infoIntPair("SiteSize", site_w_, site_h_);
    log_->infoIntPair("CoreAreaLxLy", core_lx_, core_ly_);
    log_->infoIntPair("CoreAreaUxUy", core_ux_, core_uy_);
  }

  // real instances
  std::unordered_map<const odb::dbInst*, int> inst_index;
  std::vector<int> fixed_boxes;   // lx ly ux uy of every fixed real instance
  for (odb::dbInst* inst : block->getInsts()) {
    int x = 0, y = 0;
    inst->getLocation(x, y);
    odb::dbBox* bb = inst->getBBox();
    const int k = (int)lx_.size();
    inst_index[inst] = k;
    db_insts_.push_back(inst);
    lx_.push_back(x);
    ly_.push_back(y);
    ux_.push_back(x + bb->getDX());
    uy_.push_back(y + bb->getDY());
    if (is_fixed_status(inst->getPlacementStatus())) {
      fixed_boxes.insert(fixed_boxes.end(), {lx_[k], ly_[k], ux_[k], uy_[k]});
      const int rlx = std::max(core_lx_, lx_[k]), rly = std::max(core_ly_, ly_[k]);
      const int rux = std::min(core_ux_, ux_[k]), ruy = std::min(core_uy_, uy_[k]);
      if (rlx < rux && rly < ruy) {
        kind_.push_back(GPL_INST_FIXED);
        n_fixed_++;
        non_place_area_ += (int64_t)(rux - rlx) * (int64_t)(ruy - rly);
      } else {
        kind_.push_back(GPL_INST_OUTSIDE);
      }
    } else {
      kind_.push_back(GPL_INST_PLACE);
      n_place_++;
      const int64_t a = (int64_t)(ux_[k] - lx_[k]) * (int64_t)(uy_[k] - ly_[k]);
      place_area_ += a;
      if (uy_[k] - ly_[k] > site_h_ * 6) macro_area_ += a;
      else std_area_ += a;
    }
  }
  addFragmentedRowDummies(fixed_boxes);

  // pins of the signal nets, net-major
  std::unordered_map<const void*, int> iterm_pin;
  net_start_.push_back(0);
  for (odb::dbNet* net : block->getNets()) {
    const odb::dbSigType t = net->getSigType();
    if (t == odb::dbSigType::GROUND || t == odb::dbSigType::POWER || t == odb::dbSigType::RESET)
      continue;
    for (odb::dbITerm* it : net->getITerms()) {
      odb::dbInst* inst = it->getInst();
      int lo_x = INT_MAX, lo_y = INT_MAX, hi_x = INT_MIN, hi_y = INT_MIN;
      for (odb::dbMPin* mp : it->getMTerm()->getMPins())
        for (odb::dbBox* b : mp->getGeometry()) {
          lo_x = std::min(lo_x, b->xMin());
          lo_y = std::min(lo_y, b->yMin());
          hi_x = std::max(hi_x, b->xMax());
          hi_y = std::max(hi_y, b->yMax());
        }
      const int hw = inst->getMaster()->getWidth() / 2, hh = inst->getMaster()->getHeight() / 2;
      int ox = 0, oy = 0;
      if (lo_x != INT_MAX && lo_y != INT_MAX && hi_x != INT_MIN && hi_y != INT_MIN) {
        ox = (lo_x + hi_x) / 2 - hw;
        oy = (lo_y + hi_y) / 2 - hh;
      }
      const auto f = inst_index.find(inst);
      const int k = f == inst_index.end() ? -1 : f->second;
      if (k < 0 && log_) log_->error("a net pin's instance is not in the block", 1);
      iterm_pin[it] = (int)pin_inst_.size();
      pin_inst_.push_back(k);
      pin_ox_.push_back(ox);
      pin_oy_.push_back(oy);
      pin_x_.push_back(inst->getBBox()->xMin() + hw + ox);
      pin_y_.push_back(inst->getBBox()->yMin() + hh + oy);
    }
    for (odb::dbBTerm* bt : net->getBTerms()) {
      int lo_x = INT_MAX, lo_y = INT_MAX, hi_x = INT_MIN, hi_y = INT_MIN;
      for (odb::dbBPin* bp : bt->getBPins()) {
        lo_x = std::min(lo_x, bp->getBox()->xMin());
        lo_y = std::min(lo_y, bp->getBox()->yMin());
        hi_x = std::max(hi_x, bp->getBox()->xMax());
        hi_y = std::max(hi_y, bp->getBox()->yMax());
      }
      if (lo_x == INT_MAX || lo_y == INT_MAX || hi_x == INT_MIN || hi_y == INT_MIN) {
        // Pin::updateCoordi(dbBTerm*): an unplaced port counts as (0, 0)
        if (log_)
          log_->warn(std::string(bt->getConstName()) + " toplevel port is not placed!\n" +
                     "       Replace will regard " + bt->getConstName() + " is placed in (0, 0)", 1);
        lo_x = hi_x = lo_y = hi_y = 0;
      }
      pin_inst_.push_back(-1);
      pin_ox_.push_back(0);
      pin_oy_.push_back(0);
      pin_x_.push_back((int)(((int64_t)lo_x + hi_x) / 2));
      pin_y_.push_back((int)(((int64_t)lo_y + hi_y) / 2));
    }
    net_start_.push_back((int32_t)pin_inst_.size());
  }

  // each instance's pins in dbInst::getITerms order (pins of skipped nets
  // are not the placer's)
  const int n = instCount();
  inst_pin_start_.assign(n + 1, 0);
  for (int k = 0; k < (int)db_insts_.size(); k++) {
    inst_pin_start_[k] = (int32_t)inst_pins_.size();
    for (odb::dbITerm* it : db_insts_[k]->getITerms()) {
      const auto f = iterm_pin.find(it);
      if (f != iterm_pin.end()) inst_pins_.push_back(f->second);
    }
  }
  for (int k = (int)db_insts_.size(); k <= n; k++) inst_pin_start_[k] = (int32_t)inst_pins_.size();
  refreshDesc();
  printInfo();
}

void PlacerBase::addFragmentedRowDummies(const std::vector<int>& fixed_boxes) {
  // initInstsForFragmentedRow (src/placerBase.cpp:761-846): a site grid
  // over the core, rows mark their sites, fixed instances theirs; each run
  // of unmarked sites in a site row becomes a fixed dummy instance.
  const int nx = (core_ux_ - core_lx_) / site_w_, ny = (core_uy_ - core_ly_) / site_h_;
  if (nx <= 0 || ny <= 0) return;
  std::vector<uint8_t> grid((size_t)nx * ny, 0);   // 0 empty, 1 row, 2 fixed
  auto mark = [&](int lx, int ly, int ux, int uy, uint8_t v) {
    int a, b, c, d;
    site_range(lx, ux, core_lx_, site_w_, nx, a, b);
    site_range(ly, uy, core_ly_, site_h_, ny, c, d);
    for (int j = c; j < d; j++)
      for (int i = a; i < b; i++) grid[(size_t)j * nx + i] = v;
  };
  for (odb::dbRow* row : db_->getChip()->getBlock()->getRows()) {
    odb::Rect r;
    row->getBBox(r);
    mark(r.xMin(), r.yMin(), r.xMax(), r.yMax(), 1);
  }
  for (size_t f = 0; f + 3 < fixed_boxes.size(); f += 4)
    mark(fixed_boxes[f], fixed_boxes[f + 1], fixed_boxes[f + 2], fixed_boxes[f + 3], 2);
  for (int j = 0; j < ny; j++) {
    for (int i = 0; i < nx; i++) {
      if (grid[(size_t)j * nx + i] != 0) continue;
      const int s = i;
      while (i < nx && grid[(size_t)j * nx + i] == 0) i++;
      lx_.push_back(core_lx_ + site_w_ * s);
      ly_.push_back(core_ly_ + site_h_ * j);
      ux_.push_back(core_lx_ + site_w_ * i);
      uy_.push_back(core_ly_ + site_h_ * (j + 1));
      kind_.push_back(GPL_INST_DUMMY);
      n_dummy_++;
      non_place_area_ += (int64_t)(ux_.back() - lx_.back()) * (int64_t)(uy_.back() - ly_.back());
    }
  }
}

void PlacerBase::refreshDesc() {
  gpl_netlist_desc& d = desc_;
  d.core_lx = core_lx_; d.core_ly = core_ly_; d.core_ux = core_ux_; d.core_uy = core_uy_;
  d.site_w = site_w_; d.site_h = site_h_;
  d.n_insts = instCount();
  d.inst_lx = lx_.data(); d.inst_ly = ly_.data(); d.inst_ux = ux_.data(); d.inst_uy = uy_.data();
  d.inst_kind = kind_.data();
  d.n_pins = pinCount();
  d.pin_inst = pin_inst_.data(); d.pin_ox = pin_ox_.data(); d.pin_oy = pin_oy_.data();
  d.pin_x = pin_x_.data(); d.pin_y = pin_y_.data();
  d.n_nets = netCount();
  d.net_start = net_start_.data();
  d.inst_pin_start = inst_pin_start_.data();
  d.inst_pins = inst_pins_.data();
}

void PlacerBase::printInfo() const {
  // PlacerBase::printInfo (src/placerBase.cpp:897-957)
  if (!log_) return;
  log_->infoInt("NumInstances", instCount());
  log_->infoInt("NumPlaceInstances", n_place_);
  log_->infoInt("NumFixedInstances", n_fixed_);
  log_->infoInt("NumDummyInstances", n_dummy_);
  log_->infoInt("NumNets", netCount());
  log_->infoInt("NumPins", pinCount());
  log_->infoIntPair("DieAreaLxLy", die_lx_, die_ly_);
  log_->infoIntPair("DieAreaUxUy", die_ux_, die_uy_);
  log_->infoIntPair("CoreAreaLxLy", core_lx_, core_ly_);
  log_->infoIntPair("CoreAreaUxUy", core_ux_, core_uy_);
  const int64_t core_area = (int64_t)(core_ux_ - core_lx_) * (int64_t)(core_uy_ - core_ly_);
  const float util = (float)place_area_ / (core_area - non_place_area_) * 100;
  log_->infoInt64("CoreArea", core_area);
  log_->infoInt64("NonPlaceInstsArea", non_place_area_);
  log_->infoInt64("PlaceInstsArea", place_area_);
  log_->infoFloat("Util(%)", util);
  log_->infoInt64("StdInstsArea", std_area_);
  log_->infoInt64("MacroInstsArea", macro_area_);
  if (util >= 100.1) {
    printf("Error: Util exceeds 100%%.\n       Please double-check your die/row size\n");
    fflush(stdout);
    exit(1);
  }
}

void PlacerBase::setInstCenterBoxes(const int32_t* lx, const int32_t* ly) {
  for (int k = 0; k < instCount(); k++) {
    if (kind_[k] != GPL_INST_PLACE) continue;
    const int hx = (ux_[k] - lx_[k]) / 2, hy = (uy_[k] - ly_[k]) / 2;
    lx_[k] = lx[k];
    ly_[k] = ly[k];
    ux_[k] = lx[k] + 2 * hx;
    uy_[k] = ly[k] + 2 * hy;
  }
  // Pin::updateLocation: instance centre + offset
  for (int q = 0; q < pinCount(); q++) {
    const int k = pin_inst_[q];
    if (k < 0 || kind_[k] != GPL_INST_PLACE) continue;
    pin_x_[q] = (lx_[k] + ux_[k]) / 2 + pin_ox_[q];
    pin_y_[q] = (ly_[k] + uy_[k]) / 2 + pin_oy_[q];
  }
}

void PlacerBase::writeDb(const int32_t* lx, const int32_t* ly) const {
  for (int k = 0; k < (int)db_insts_.size(); k++) {
    if (kind_[k] != GPL_INST_PLACE) continue;
    db_insts_[k]->setLocation(lx[k], ly[k]);
    db_insts_[k]->setPlacementStatus(odb::dbPlacementStatus::PLACED);
  }
}

}  // namespace replace
