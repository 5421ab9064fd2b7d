#include "nesterov.h"

#include <vector>

#include "logger.h"
#include "placer_base.h"

namespace replace {

// NesterovBaseVars (src/nesterovBase.cpp:875-895)
NesterovBaseVars::NesterovBaseVars() { reset(); }

void NesterovBaseVars::reset() {
  targetDensity = 1.0f;
  minAvgCut = 0.1f;
  maxAvgCut = 0.9f;
  binCntX = binCntY = 0;
  minWireLengthForceBar = -300;
  isSetBinCntX = isSetBinCntY = 0;
}

NesterovBase::NesterovBase() = default;

NesterovBase::NesterovBase(NesterovBaseVars nbVars, std::shared_ptr<PlacerBase> pb,
                           std::shared_ptr<Logger> log)
    : nbVars_(nbVars), pb_(std::move(pb)), log_(std::move(log)) {}

NesterovBase::~NesterovBase() = default;

// NesterovPlaceVars (src/nesterovPlace.cpp:19-29)
NesterovPlaceVars::NesterovPlaceVars()
    : maxNesterovIter(2000), maxBackTrack(10), initDensityPenalty(0.00008f),
      initWireLengthCoef(0.25f), targetOverflow(0.1f), minPhiCoef(0.95f), maxPhiCoef(1.05f),
      minPreconditioner(1.0f), initialPrevCoordiUpdateCoef(100), referenceHpwl(446000000) {}

NesterovPlace::NesterovPlace() = default;

NesterovPlace::NesterovPlace(NesterovPlaceVars npVars, std::shared_ptr<PlacerBase> pb,
                             std::shared_ptr<NesterovBase> nb, std::shared_ptr<Logger> log)
    : pb_(std::move(pb)), nb_(std::move(nb)), log_(std::move(log)), npVars_(npVars) {
  init();
}

NesterovPlace::~NesterovPlace() = default;

namespace {

// The Nesterov-side members of two parameter sets agree (a job made for the
// initial place can then run the loop as well).
bool same_nesterov_params(const gpl_params& a, const gpl_params& b) {
  return a.target_density == b.target_density && a.bin_grid_cnt_x == b.bin_grid_cnt_x &&
         a.bin_grid_cnt_y == b.bin_grid_cnt_y &&
         a.min_wire_length_force_bar == b.min_wire_length_force_bar &&
         a.nesterov_place_max_iter == b.nesterov_place_max_iter &&
         a.max_back_track == b.max_back_track && a.init_density_penalty == b.init_density_penalty &&
         a.init_wire_length_coef == b.init_wire_length_coef &&
         a.target_overflow == b.target_overflow && a.min_phi_coef == b.min_phi_coef &&
         a.max_phi_coef == b.max_phi_coef && a.min_preconditioner == b.min_preconditioner &&
         a.initial_prev_coordi_update_coef == b.initial_prev_coordi_update_coef &&
         a.reference_hpwl == b.reference_hpwl && a.device == b.device &&
         a.poisson_path == b.poisson_path && a.use_graph == b.use_graph &&
         a.device_loop == b.device_loop && a.scatter_tile == b.scatter_tile &&
         a.scatter_chunk == b.scatter_chunk;
}

}  // namespace

void NesterovPlace::init() {
  const NesterovBaseVars& nv = nb_->vars();
  gpl_params p = pb_->baseParams();
  p.target_density = nv.targetDensity;
  p.bin_grid_cnt_x = nv.isSetBinCntX ? nv.binCntX : 0;
  p.bin_grid_cnt_y = nv.isSetBinCntY ? nv.binCntY : 0;
  p.min_wire_length_force_bar = nv.minWireLengthForceBar;
  p.nesterov_place_max_iter = npVars_.maxNesterovIter;
  p.max_back_track = npVars_.maxBackTrack;
  p.init_density_penalty = npVars_.initDensityPenalty;
  p.init_wire_length_coef = npVars_.initWireLengthCoef;
  p.target_overflow = npVars_.targetOverflow;
  p.min_phi_coef = npVars_.minPhiCoef;
  p.max_phi_coef = npVars_.maxPhiCoef;
  p.min_preconditioner = npVars_.minPreconditioner;
  p.initial_prev_coordi_update_coef = npVars_.initialPrevCoordiUpdateCoef;
  p.reference_hpwl = npVars_.referenceHpwl;
  if (log_) p.verbose_level = log_->verbose();

  std::shared_ptr<GplJob>& held = pb_->job();
  if (held && held->job && held->initial_placed && !held->nesterov_ready &&
      same_nesterov_params(held->params, p)) {
    job_ = held;            // continue on the initial place's device copy
  } else {
    // a new job from the PlacerBase's current locations: no centring and no
    // initial-place rounds (the locations are the caller's)
    p.initial_place_max_iter = 0;
    p.incremental_place_mode = 1;
    auto job = std::make_shared<GplJob>();
    job->params = p;
    gpl_status st = gpl_create(&pb_->netlist(), &p, &job->job);
    if (st != GPL_OK) log_->error(gpl_last_error(), st == GPL_ERR_UTIL ? 1 : (int)st);
    gpl_ip_stats s{};
    st = gpl_initial_place(job->job, &s);
    if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
    job->initial_placed = true;
    held = job;
    job_ = job;
  }
  const std::vector<float>& w = pb_->netWeights();
  if (!w.empty()) {
    gpl_status st = gpl_set_net_weights(job_->job, w.data(), (int64_t)w.size());
    if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
  }
  gpl_job_info& info = nb_->info();
  gpl_status st = gpl_nesterov_init(job_->job, &info);
  if (st != GPL_OK) {
    // NesterovPlace::init reports a NaN start with code 2; the filler-area
    // failure of NesterovBase::initFillerGCells is code 1
    log_->error(gpl_last_error(), (int)st);
  }
  job_->nesterov_ready = true;
  if (log_) {
    log_->infoIntPair("BinCnt", info.bin_cnt_x, info.bin_cnt_y, 1);
    log_->infoIntPair("BinSize", info.bin_size_x, info.bin_size_y, 1);
    log_->infoInt("FillerInit: NumGCells", info.n_gcells, 1);
    log_->infoInt("FillerInit: NumGNets", pb_->netCount(), 1);
    log_->infoInt("FillerInit: NumGPins", pb_->pinCount(), 1);
  }
}

void NesterovPlace::doNesterovPlace() {
  const gpl_status st = gpl_nesterov_run(job_->job, 0, &stats_, nullptr);
  // in every case, divergence included, the database gets the locations
  updateDb();
  if (st == GPL_ERR_DIVERGED_BACKTRACK || st == GPL_ERR_DIVERGED_PHI)
    log_->error(gpl_last_error(), (int)st);
  if (st == GPL_ERR_DIVERGED_NAN) log_->error(gpl_last_error(), 0);
  if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
}

void NesterovPlace::updateDb() {
  std::vector<int32_t> lx(pb_->instCount()), ly(pb_->instCount());
  const gpl_status st = gpl_get_inst_locations(job_->job, lx.data(), ly.data());
  if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
  pb_->writeDb(lx.data(), ly.data());
}

}  // namespace replace
