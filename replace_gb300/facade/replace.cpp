// replace::Replace over the GB300 core: the flow of src/replace.cpp:73-128
// (a PlacerBase from the database, the initial place on it, then
// NesterovBase / NesterovPlace on the same PlacerBase).
#include "replace/Replace.h"

#include "initial_place.h"
#include "logger.h"
#include "nesterov.h"
#include "placer_base.h"

namespace replace {

// Replace::Replace() defaults (src/replace.cpp:13-33)
Replace::Replace()
    : db_(nullptr), sta_(nullptr), pb_(nullptr), nb_(nullptr), ip_(nullptr), np_(nullptr),
      log_(nullptr), initialPlaceMaxIter_(20), initialPlaceMinDiffLength_(1500),
      initialPlaceMaxSolverIter_(100), initialPlaceMaxFanout_(200),
      initialPlaceNetWeightScale_(800), nesterovPlaceMaxIter_(2000), binGridCntX_(0),
      binGridCntY_(0), overflow_(0.1f), density_(1.0f), initDensityPenalityFactor_(0.00008f),
      initWireLengthCoef_(0.25f), minPhiCoef_(0.95f), maxPhiCoef_(1.05f),
      referenceHpwl_(446000000), incrementalPlaceMode_(false), verbose_(0), device_(0) {}

Replace::~Replace() { reset(); }

void Replace::init() {}

// Replace::reset (src/replace.cpp:39-65): the values it sets differ from the
// constructor's, and are kept as the reference has them.
void Replace::reset() {
  np_.reset();
  ip_.reset();
  nb_.reset();
  pb_.reset();
  db_ = nullptr;
  sta_ = nullptr;
  initialPlaceMaxIter_ = 20;
  initialPlaceMinDiffLength_ = 1500;
  initialPlaceMaxSolverIter_ = 100;
  initialPlaceMaxFanout_ = 200;
  initialPlaceNetWeightScale_ = 800;
  nesterovPlaceMaxIter_ = 2000;
  binGridCntX_ = binGridCntY_ = 0;
  overflow_ = 0;
  density_ = 0;
  initDensityPenalityFactor_ = 0.0001f;
  initWireLengthCoef_ = 1.0f;
  minPhiCoef_ = 0.95f;
  maxPhiCoef_ = 1.05f;
  referenceHpwl_ = 446000000;
  incrementalPlaceMode_ = false;
  verbose_ = 0;
  netWeights_.clear();
}

void Replace::setDb(odb::dbDatabase* db) { db_ = db; }
void Replace::setSta(sta::dbSta* sta) { sta_ = sta; }

namespace {

// The whole parameter set of one placement, so that the job the initial
// place creates can also run the Nesterov loop.
void fill_params(gpl_params& p, int ip_iter, int min_diff, int solver_iter, int fanout,
                 float weight_scale, bool incremental, float density, int bx, int by,
                 int np_iter, float idp, float iwc, float ovf, float minphi, float maxphi,
                 float ref_hpwl, int verbose, int device) {
  gpl_params_default(&p);
  p.initial_place_max_iter = ip_iter;
  p.initial_place_min_diff_length = min_diff;
  p.initial_place_max_solver_iter = solver_iter;
  p.initial_place_max_fanout = fanout;
  p.initial_place_net_weight_scale = weight_scale;
  p.incremental_place_mode = incremental ? 1 : 0;
  p.target_density = density;
  p.bin_grid_cnt_x = bx;
  p.bin_grid_cnt_y = by;
  p.nesterov_place_max_iter = np_iter;
  p.init_density_penalty = idp;
  p.init_wire_length_coef = iwc;
  p.target_overflow = ovf;
  p.min_phi_coef = minphi;
  p.max_phi_coef = maxphi;
  p.reference_hpwl = ref_hpwl;
  p.verbose_level = verbose;
  p.device = device;
}

}  // namespace

void Replace::doInitialPlace() {
  log_ = std::make_shared<Logger>("REPL", verbose_);
  pb_ = std::make_shared<PlacerBase>(db_, log_);
  fill_params(pb_->baseParams(), initialPlaceMaxIter_, initialPlaceMinDiffLength_,
              initialPlaceMaxSolverIter_, initialPlaceMaxFanout_, initialPlaceNetWeightScale_,
              incrementalPlaceMode_, density_, binGridCntX_, binGridCntY_, nesterovPlaceMaxIter_,
              initDensityPenalityFactor_, initWireLengthCoef_, overflow_, minPhiCoef_, maxPhiCoef_,
              referenceHpwl_, verbose_, device_);
  pb_->setNetWeights(netWeights_);

  InitialPlaceVars ipVars;
  ipVars.maxIter = initialPlaceMaxIter_;
  ipVars.minDiffLength = initialPlaceMinDiffLength_;
  ipVars.maxSolverIter = initialPlaceMaxSolverIter_;
  ipVars.maxFanout = initialPlaceMaxFanout_;
  ipVars.netWeightScale = initialPlaceNetWeightScale_;
  ipVars.incrementalPlaceMode = incrementalPlaceMode_;
  ip_.reset(new InitialPlace(ipVars, pb_, log_));
  ip_->doBicgstabPlace();
}

void Replace::doNesterovPlace() {
  if (!log_) log_ = std::make_shared<Logger>("REPL", verbose_);
  if (!pb_) {
    pb_ = std::make_shared<PlacerBase>(db_, log_);
    pb_->baseParams().device = device_;
    pb_->setNetWeights(netWeights_);
  }

  NesterovBaseVars nbVars;
  nbVars.targetDensity = density_;
  if (binGridCntX_ != 0) {
    nbVars.isSetBinCntX = 1;
    nbVars.binCntX = binGridCntX_;
  }
  if (binGridCntY_ != 0) {
    nbVars.isSetBinCntY = 1;
    nbVars.binCntY = binGridCntY_;
  }
  nb_ = std::make_shared<NesterovBase>(nbVars, pb_, log_);

  NesterovPlaceVars npVars;
  npVars.minPhiCoef = minPhiCoef_;
  npVars.maxPhiCoef = maxPhiCoef_;
  npVars.referenceHpwl = referenceHpwl_;
  npVars.initDensityPenalty = initDensityPenalityFactor_;
  npVars.initWireLengthCoef = initWireLengthCoef_;
  npVars.targetOverflow = overflow_;
  npVars.maxNesterovIter = nesterovPlaceMaxIter_;
  np_.reset(new NesterovPlace(npVars, pb_, nb_, log_));
  np_->doNesterovPlace();
}

void Replace::setInitialPlaceMaxIter(int iter) { initialPlaceMaxIter_ = iter; }
void Replace::setInitialPlaceMinDiffLength(int length) { initialPlaceMinDiffLength_ = length; }
void Replace::setInitialPlaceMaxSolverIter(int iter) { initialPlaceMaxSolverIter_ = iter; }
void Replace::setInitialPlaceMaxFanout(int fanout) { initialPlaceMaxFanout_ = fanout; }
void Replace::setInitialPlaceNetWeightScale(float scale) { initialPlaceNetWeightScale_ = scale; }
void Replace::setNesterovPlaceMaxIter(int iter) { nesterovPlaceMaxIter_ = iter; }
void Replace::setBinGridCntX(int n) { binGridCntX_ = n; }
void Replace::setBinGridCntY(int n) { binGridCntY_ = n; }
void Replace::setTargetDensity(float density) { density_ = density; }
void Replace::setTargetOverflow(float overflow) { overflow_ = overflow; }
void Replace::setInitDensityPenalityFactor(float f) { initDensityPenalityFactor_ = f; }
void Replace::setInitWireLengthCoef(float coef) { initWireLengthCoef_ = coef; }
void Replace::setMinPhiCoef(float c) { minPhiCoef_ = c; }
void Replace::setMaxPhiCoef(float c) { maxPhiCoef_ = c; }
void Replace::setReferenceHpwl(float h) { referenceHpwl_ = h; }
void Replace::setIncrementalPlaceMode(bool mode) { incrementalPlaceMode_ = mode; }
void Replace::setVerboseLevel(int verbose) { verbose_ = verbose; }
void Replace::setDevice(int device) { device_ = device; }
void Replace::setNetWeights(const std::vector<float>& w) { netWeights_ = w; }

}  // namespace replace
