/*
 * replace/Replace.h - the replace::Replace placement object on the GB300 core.
 *
 * Same class, methods and argument meaning as RePlAce's public header
 * (include/replace/Replace.h:23-94 of the reference), so that OpenROAD's
 * SWIG layer (src/replace.i) and its ord::makeReplace / initReplace hooks
 * (src/MakeReplace.cpp:16-34) compile against it unchanged.  The work runs in
 * libgpl_gb300.so (gpl.h): doInitialPlace is the B2B/BiCGSTAB initial place
 * on the GPU, doNesterovPlace the Nesterov loop on the GPU, and the final
 * locations are written back into OpenDB as NesterovPlace::updateDb does.
 *
 * Behaviour kept from the reference:
 *  - the defaults of Replace::Replace() (src/replace.cpp:13-33);
 *  - doInitialPlace builds a new PlacerBase from the database and runs the
 *    initial place; doNesterovPlace builds NesterovBase / NesterovPlace on the
 *    same PlacerBase (src/replace.cpp:73-128);
 *  - errors go through Logger::error, which prints the reference's message
 *    and code and exits the process with that code (src/logger.cpp:31-36).
 *    Callers that want status codes instead use gpl.h directly.
 * Added: setDevice (CUDA device ordinal) and setNetWeights (GNet custom
 * weights, gpl_set_net_weights).
 */
#ifndef REPLACE_GB300_REPLACE_H
#define REPLACE_GB300_REPLACE_H

#include <memory>
#include <vector>

namespace odb {
class dbDatabase;
}
namespace sta {
class dbSta;
}

namespace replace {

class PlacerBase;
class NesterovBase;
class InitialPlace;
class NesterovPlace;
class Logger;

class Replace {
 public:
  Replace();
  ~Replace();

  void init();
  void reset();

  void setDb(odb::dbDatabase* odb);
  void setSta(sta::dbSta* dbSta);

  void doInitialPlace();
  void doNesterovPlace();

  // initial place
  void setInitialPlaceMaxIter(int iter);
  void setInitialPlaceMinDiffLength(int length);
  void setInitialPlaceMaxSolverIter(int iter);
  void setInitialPlaceMaxFanout(int fanout);
  void setInitialPlaceNetWeightScale(float scale);

  // Nesterov place
  void setNesterovPlaceMaxIter(int iter);
  void setBinGridCntX(int binGridCntX);
  void setBinGridCntY(int binGridCntY);
  void setTargetDensity(float density);
  void setTargetOverflow(float overflow);
  void setInitDensityPenalityFactor(float penaltyFactor);
  void setInitWireLengthCoef(float coef);
  void setMinPhiCoef(float minPhiCoef);
  void setMaxPhiCoef(float maxPhiCoef);
  void setReferenceHpwl(float deltaHpwl);

  void setIncrementalPlaceMode(bool mode);
  void setVerboseLevel(int verbose);

  // GB300 additions
  void setDevice(int device);
  // one weight per signal net, in the order PlacerBase lists them (the
  // database's net order without power, ground and reset nets); empty = none
  void setNetWeights(const std::vector<float>& weights);

 private:
  odb::dbDatabase* db_;
  sta::dbSta* sta_;

  std::shared_ptr<PlacerBase> pb_;
  std::shared_ptr<NesterovBase> nb_;
  std::unique_ptr<InitialPlace> ip_;
  std::unique_ptr<NesterovPlace> np_;
  std::shared_ptr<Logger> log_;

  int initialPlaceMaxIter_;
  int initialPlaceMinDiffLength_;
  int initialPlaceMaxSolverIter_;
  int initialPlaceMaxFanout_;
  float initialPlaceNetWeightScale_;

  int nesterovPlaceMaxIter_;
  int binGridCntX_;
  int binGridCntY_;
  float overflow_;
  float density_;
  float initDensityPenalityFactor_;
  float initWireLengthCoef_;
  float minPhiCoef_;
  float maxPhiCoef_;
  float referenceHpwl_;

  bool incrementalPlaceMode_;
  int verbose_;
  int device_;
  std::vector<float> netWeights_;
};

}  // namespace replace

#endif
