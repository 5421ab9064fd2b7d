// Driver of the replace::Replace facade tests.
//
// TEST INFRASTRUCTURE: links the facade sources (replace_gb300/facade) with
// the in-memory OpenDB stand-in that the reference build also uses, reads a
// netlist in refnet.py's text format into it, and runs one of:
//
//   flatten <net.txt> <out.bin>           PlacerBase only: the flat netlist
//                                         it hands to the GPU core
//   place <net.txt> <out.txt> [options]   Replace: setters, doInitialPlace,
//                                         doNesterovPlace; the database's
//                                         instance locations and statuses
//   components <net.txt> <out.txt> [opt]  the same flow through InitialPlace,
//                                         NesterovBase and NesterovPlace built
//                                         directly from their Vars
//
// Options: --density d --bins n --idp p --overflow o --maxphi m --minphi m
//          --ip-iter n --incremental --verbose v --maxiter n
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "initial_place.h"
#include "logger.h"
#include "nesterov.h"
#include "opendb/db.h"
#include "placer_base.h"
#include "refnet_db.h"
#include "replace/Replace.h"

namespace {

struct Opts {
  float density = 0.7f;
  int bins = 0;
  float idp = 0.00008f;
  float overflow = 0.1f;
  float maxphi = 1.05f, minphi = 0.95f;
  int ip_iter = 20;
  bool incremental = false;
  int verbose = 0;
  int maxiter = 2000;
};

Opts parse(int argc, char** argv, int start) {
  Opts o;
  for (int i = start; i < argc; i++) {
    std::string a = argv[i];
    auto nxt = [&]() { return std::string(argv[++i]); };
    if (a == "--density") o.density = std::stof(nxt());
    else if (a == "--bins") o.bins = std::stoi(nxt());
    else if (a == "--idp") o.idp = std::stof(nxt());
    else if (a == "--overflow") o.overflow = std::stof(nxt());
    else if (a == "--maxphi") o.maxphi = std::stof(nxt());
    else if (a == "--minphi") o.minphi = std::stof(nxt());
    else if (a == "--ip-iter") o.ip_iter = std::stoi(nxt());
    else if (a == "--incremental") o.incremental = true;
    else if (a == "--verbose") o.verbose = std::stoi(nxt());
    else if (a == "--maxiter") o.maxiter = std::stoi(nxt());
    else { fprintf(stderr, "unknown option %s\n", a.c_str()); exit(2); }
  }
  return o;
}

template <class T>
void put(FILE* f, const char* name, const char* dt, const T* v, size_t n) {
  fprintf(f, "%s %s %zu\n", name, dt, n);
  fwrite(v, sizeof(T), n, f);
  fprintf(f, "\n");
}

void write_locations(odb::dbDatabase* db, const char* path) {
  FILE* f = fopen(path, "w");
  for (odb::dbInst* inst : db->getChip()->getBlock()->getInsts())
    fprintf(f, "%d %d %d\n", inst->x, inst->y, (int)(odb::dbPlacementStatus::Value)inst->getPlacementStatus());
  fclose(f);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: facade_driver flatten|place|components net.txt out [options]\n");
    return 2;
  }
  const std::string mode = argv[1];
  odb::dbDatabase* db = read_net(argv[2]);
  const Opts o = parse(argc, argv, 4);
  if (mode == "flatten") {
    auto log = std::make_shared<replace::Logger>("REPL", o.verbose);
    replace::PlacerBase pb(db, log);
    const gpl_netlist_desc& d = pb.netlist();
    const int32_t geo[6] = {d.core_lx, d.core_ly, d.core_ux, d.core_uy, d.site_w, d.site_h};
    FILE* f = fopen(argv[3], "wb");
    put(f, "geometry", "i4", geo, 6);
    put(f, "inst_lx", "i4", d.inst_lx, d.n_insts);
    put(f, "inst_ly", "i4", d.inst_ly, d.n_insts);
    put(f, "inst_ux", "i4", d.inst_ux, d.n_insts);
    put(f, "inst_uy", "i4", d.inst_uy, d.n_insts);
    put(f, "inst_kind", "u1", d.inst_kind, d.n_insts);
    put(f, "pin_inst", "i4", d.pin_inst, d.n_pins);
    put(f, "pin_ox", "i4", d.pin_ox, d.n_pins);
    put(f, "pin_oy", "i4", d.pin_oy, d.n_pins);
    put(f, "pin_x", "i4", d.pin_x, d.n_pins);
    put(f, "pin_y", "i4", d.pin_y, d.n_pins);
    put(f, "net_start", "i4", d.net_start, d.n_nets + 1);
    put(f, "inst_pin_start", "i4", d.inst_pin_start, d.n_insts + 1);
    put(f, "inst_pins", "i4", d.inst_pins, d.inst_pin_start[d.n_insts]);
    const int64_t areas[4] = {pb.placeInstsArea(), pb.nonPlaceInstsArea(), pb.stdInstsArea(),
                              pb.macroInstsArea()};
    put(f, "areas", "i8", areas, 4);
    fclose(f);
    return 0;
  }
  if (mode == "place") {
    replace::Replace r;
    r.setDb(db);
    r.setTargetDensity(o.density);
    r.setInitDensityPenalityFactor(o.idp);
    r.setTargetOverflow(o.overflow);
    r.setMaxPhiCoef(o.maxphi);
    r.setMinPhiCoef(o.minphi);
    r.setInitialPlaceMaxIter(o.incremental ? 0 : o.ip_iter);
    r.setIncrementalPlaceMode(o.incremental);
    r.setNesterovPlaceMaxIter(o.maxiter);
    r.setVerboseLevel(o.verbose);
    if (o.bins) {
      r.setBinGridCntX(o.bins);
      r.setBinGridCntY(o.bins);
    }
    r.doInitialPlace();
    r.doNesterovPlace();
    write_locations(db, argv[3]);
    return 0;
  }
  if (mode == "components") {
    auto log = std::make_shared<replace::Logger>("REPL", o.verbose);
    auto pb = std::make_shared<replace::PlacerBase>(db, log);
    replace::InitialPlaceVars ipv;
    ipv.maxIter = o.incremental ? 0 : o.ip_iter;
    ipv.incrementalPlaceMode = o.incremental;
    replace::InitialPlace ip(ipv, pb, log);
    ip.doBicgstabPlace();
    replace::NesterovBaseVars nbv;
    nbv.targetDensity = o.density;
    if (o.bins) {
      nbv.isSetBinCntX = nbv.isSetBinCntY = 1;
      nbv.binCntX = nbv.binCntY = o.bins;
    }
    auto nb = std::make_shared<replace::NesterovBase>(nbv, pb, log);
    replace::NesterovPlaceVars npv;
    npv.initDensityPenalty = o.idp;
    npv.targetOverflow = o.overflow;
    npv.maxPhiCoef = o.maxphi;
    npv.minPhiCoef = o.minphi;
    npv.maxNesterovIter = o.maxiter;
    replace::NesterovPlace np(npv, pb, nb, log);
    np.doNesterovPlace();
    write_locations(db, argv[3]);
    printf("[FACADE] iterations %d overflow %g hpwl %lld\n", np.stats().iterations,
           np.stats().overflow, (long long)np.stats().hpwl);
    return 0;
  }
  fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
