// replace::InitialPlace on the GB300 core.
//
// Same constructor and entry point as RePlAce's InitialPlace
// (src/initialPlace.h:27-35): doBicgstabPlace centres the movable instances
// (unless incremental) and runs up to maxIter bound-to-bound rounds, each a
// BiCGSTAB solve of the x and y systems (src/initialPlace.cpp:56-105), on
// the GPU (gpl_initial_place).  The new locations are written into the
// PlacerBase, as the reference's updateCoordi does.
#ifndef REPLACE_GB300_FACADE_INITIAL_PLACE_H
#define REPLACE_GB300_FACADE_INITIAL_PLACE_H

#include <memory>

namespace replace {

class PlacerBase;
class Logger;

class InitialPlaceVars {
 public:
  int maxIter;
  int minDiffLength;
  int maxSolverIter;
  int maxFanout;
  float netWeightScale;
  bool incrementalPlaceMode;

  InitialPlaceVars();
  void reset();
};

class InitialPlace {
 public:
  InitialPlace();
  InitialPlace(InitialPlaceVars ipVars, std::shared_ptr<PlacerBase> pb, std::shared_ptr<Logger> log);
  ~InitialPlace();

  void doBicgstabPlace();

 private:
  InitialPlaceVars ipVars_;
  std::shared_ptr<PlacerBase> pb_;
  std::shared_ptr<Logger> log_;
};

}  // namespace replace

#endif
