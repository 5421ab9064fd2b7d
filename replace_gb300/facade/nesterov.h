// replace::NesterovBase and replace::NesterovPlace on the GB300 core.
//
// Same constructors and entry points as RePlAce's (src/nesterovBase.h:695-714,
// src/nesterovPlace.h:16-40).  NesterovBase carries the bin-grid and density
// settings; NesterovPlace's constructor does NesterovPlace::init (the first
// gradients, step length and penalty; code 2 on NaN) and doNesterovPlace
// runs the loop to its stop rule (src/nesterovPlace.cpp:64-175, 275-472), all
// on the GPU (gpl_nesterov_init, gpl_nesterov_run).  updateDb writes the
// final locations into OpenDB (src/nesterovPlace.cpp:585-595); divergence
// codes 3 and 4 are reported after the write-back, as the reference does.
#ifndef REPLACE_GB300_FACADE_NESTEROV_H
#define REPLACE_GB300_FACADE_NESTEROV_H

#include <memory>

#include "gpl.h"

namespace replace {

class PlacerBase;
class Logger;
struct GplJob;

class NesterovBaseVars {
 public:
  float targetDensity;
  float minAvgCut;
  float maxAvgCut;
  int binCntX;
  int binCntY;
  float minWireLengthForceBar;
  unsigned char isSetBinCntX : 1;
  unsigned char isSetBinCntY : 1;

  NesterovBaseVars();
  void reset();
};

class NesterovBase {
 public:
  NesterovBase();
  NesterovBase(NesterovBaseVars nbVars, std::shared_ptr<PlacerBase> pb, std::shared_ptr<Logger> log);
  ~NesterovBase();

  const NesterovBaseVars& vars() const { return nbVars_; }
  // the bin grid and gcell counts the job chose (valid once a NesterovPlace
  // was built on this base)
  const gpl_job_info& info() const { return info_; }
  gpl_job_info& info() { return info_; }

 private:
  NesterovBaseVars nbVars_;
  std::shared_ptr<PlacerBase> pb_;
  std::shared_ptr<Logger> log_;
  gpl_job_info info_{};
};

class NesterovPlaceVars {
 public:
  int maxNesterovIter;
  int maxBackTrack;
  float initDensityPenalty;
  float initWireLengthCoef;
  float targetOverflow;
  float minPhiCoef;
  float maxPhiCoef;
  float minPreconditioner;
  float initialPrevCoordiUpdateCoef;
  float referenceHpwl;
  NesterovPlaceVars();
};

class NesterovPlace {
 public:
  NesterovPlace();
  NesterovPlace(NesterovPlaceVars npVars, std::shared_ptr<PlacerBase> pb,
                std::shared_ptr<NesterovBase> nb, std::shared_ptr<Logger> log);
  ~NesterovPlace();

  void doNesterovPlace();
  void updateDb();

  // progress of the last doNesterovPlace (iterations, overflow, HPWL)
  const gpl_nesterov_stats& stats() const { return stats_; }

 private:
  void init();

  std::shared_ptr<PlacerBase> pb_;
  std::shared_ptr<NesterovBase> nb_;
  std::shared_ptr<Logger> log_;
  NesterovPlaceVars npVars_;
  std::shared_ptr<GplJob> job_;
  gpl_nesterov_stats stats_{};
};

}  // namespace replace

#endif
