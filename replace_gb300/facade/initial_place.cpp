#include "initial_place.h"

#include <vector>

#include "gpl.h"
#include "logger.h"
#include "placer_base.h"

namespace replace {

// InitialPlaceVars::InitialPlaceVars / reset (src/initialPlace.cpp:18-33)
InitialPlaceVars::InitialPlaceVars() { reset(); }

void InitialPlaceVars::reset() {
  maxIter = 20;
  minDiffLength = 1500;
  maxSolverIter = 100;
  maxFanout = 200;
  netWeightScale = 800;
  incrementalPlaceMode = false;
}

InitialPlace::InitialPlace() = default;

InitialPlace::InitialPlace(InitialPlaceVars ipVars, std::shared_ptr<PlacerBase> pb,
                           std::shared_ptr<Logger> log)
    : ipVars_(ipVars), pb_(std::move(pb)), log_(std::move(log)) {}

InitialPlace::~InitialPlace() = default;

void InitialPlace::doBicgstabPlace() {
  gpl_params p = pb_->baseParams();
  p.initial_place_max_iter = ipVars_.maxIter;
  p.initial_place_min_diff_length = ipVars_.minDiffLength;
  p.initial_place_max_solver_iter = ipVars_.maxSolverIter;
  p.initial_place_max_fanout = ipVars_.maxFanout;
  p.initial_place_net_weight_scale = ipVars_.netWeightScale;
  p.incremental_place_mode = ipVars_.incrementalPlaceMode ? 1 : 0;
  if (log_) p.verbose_level = log_->verbose();

  auto job = std::make_shared<GplJob>();
  job->params = p;
  gpl_status st = gpl_create(&pb_->netlist(), &p, &job->job);
  if (st != GPL_OK) log_->error(gpl_last_error(), st == GPL_ERR_UTIL ? 1 : (int)st);
  gpl_ip_stats s{};
  st = gpl_initial_place(job->job, &s);
  if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
  job->initial_placed = true;

  // updateCoordi: the PlacerBase's instances take the solved locations
  std::vector<int32_t> lx(pb_->instCount()), ly(pb_->instCount());
  st = gpl_get_inst_locations(job->job, lx.data(), ly.data());
  if (st != GPL_OK) log_->error(gpl_last_error(), (int)st);
  pb_->setInstCenterBoxes(lx.data(), ly.data());
  // the Nesterov place may continue on this job (same device copy)
  pb_->job() = job;
}

}  // namespace replace
