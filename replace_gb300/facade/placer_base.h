// replace::PlacerBase - the design as the placer sees it, read from OpenDB.
//
// Follows PlacerBase::init (src/placerBase.cpp:606-758): the core is the
// rows' bounding box, instances are movable (status NONE / UNPLACED /
// SUGGESTED / PLACED) or fixed (LOCKED / FIRM / COVER; fixed instances
// outside the core are ignored by the placer), the empty sites between rows
// become fixed dummy instances (initInstsForFragmentedRow, :761-846), and the
// pins are those of the signal nets (power, ground and reset nets skipped),
// net by net: component pins in dbNet::getITerms order, then IO pins in
// dbNet::getBTerms order.  A component pin sits at the centre of its master
// pin's shapes, unrotated (Pin::updateCoordi, :336-375); an IO pin at the
// centre of its port boxes.
//
// The result is held as the flat arrays of gpl_netlist_desc (gpl.h) that the
// GPU core takes, plus the map back to the database's instances for the
// final write-back.  One GPU job per placement is kept here so that the
// initial place and the Nesterov place, built on the same PlacerBase, run on
// one device copy of the netlist when their parameters allow.
#ifndef REPLACE_GB300_FACADE_PLACER_BASE_H
#define REPLACE_GB300_FACADE_PLACER_BASE_H

#include <cstdint>
#include <memory>
#include <vector>

#include "gpl.h"

namespace odb {
class dbDatabase;
class dbInst;
}  // namespace odb

namespace replace {

class Logger;

// A GPU job and the parameters it was created with.
struct GplJob {
  gpl_job* job = nullptr;
  gpl_params params{};
  bool initial_placed = false;
  bool nesterov_ready = false;
  ~GplJob();
};

class PlacerBase {
 public:
  PlacerBase();
  PlacerBase(odb::dbDatabase* db, std::shared_ptr<Logger> log);
  ~PlacerBase();

  odb::dbDatabase* db() const { return db_; }
  const gpl_netlist_desc& netlist() const { return desc_; }

  int instCount() const { return (int)lx_.size(); }
  int placeInstCount() const { return n_place_; }
  int netCount() const { return (int)net_start_.size() - 1; }
  int pinCount() const { return (int)pin_inst_.size(); }
  int64_t placeInstsArea() const { return place_area_; }
  int64_t nonPlaceInstsArea() const { return non_place_area_; }
  int64_t stdInstsArea() const { return std_area_; }
  int64_t macroInstsArea() const { return macro_area_; }

  // Instance boxes after a placement step (all instances, lower-left
  // corners): movable instances move to (lx, ly) and keep the width and
  // height of Instance::setCenterLocation, 2 * (dx / 2) by 2 * (dy / 2)
  // (src/placerBase.cpp:127-140); their pins follow (Pin::updateLocation).
  void setInstCenterBoxes(const int32_t* lx, const int32_t* ly);

  // NesterovPlace::updateDb (src/nesterovPlace.cpp:585-595): the movable
  // database instances get (lx, ly) and status PLACED.
  void writeDb(const int32_t* lx, const int32_t* ly) const;

  // gpl_params every job of this placement starts from (device, verbose
  // level, defaults); a Replace sets its whole parameter set here so that
  // its initial place creates a job the Nesterov place can continue.
  gpl_params& baseParams() { return base_params_; }
  void setNetWeights(std::vector<float> w) { net_weights_ = std::move(w); }
  const std::vector<float>& netWeights() const { return net_weights_; }

  std::shared_ptr<GplJob>& job() { return job_; }

 private:
  void init();
  void addFragmentedRowDummies(const std::vector<int>& fixed_boxes);
  void refreshDesc();
  void printInfo() const;

  odb::dbDatabase* db_ = nullptr;
  std::shared_ptr<Logger> log_;

  int core_lx_ = 0, core_ly_ = 0, core_ux_ = 0, core_uy_ = 0;
  int die_lx_ = 0, die_ly_ = 0, die_ux_ = 0, die_uy_ = 0;
  int site_w_ = 0, site_h_ = 0;
  std::vector<int32_t> lx_, ly_, ux_, uy_;
  std::vector<uint8_t> kind_;
  std::vector<odb::dbInst*> db_insts_;     // real instances, in database order
  std::vector<int32_t> pin_inst_, pin_ox_, pin_oy_, pin_x_, pin_y_;
  std::vector<int32_t> net_start_;
  std::vector<int32_t> inst_pin_start_, inst_pins_;
  int n_place_ = 0, n_fixed_ = 0, n_dummy_ = 0;
  int64_t place_area_ = 0, non_place_area_ = 0, std_area_ = 0, macro_area_ = 0;
  gpl_netlist_desc desc_{};

  gpl_params base_params_{};
  std::vector<float> net_weights_;
  std::shared_ptr<GplJob> job_;
};

}  // namespace replace

#endif
