// Driver around the reference's own global-placement sources.
//
// TEST INFRASTRUCTURE ONLY (never shipped, never linked into the product).
// It is compiled together with the reference's unchanged
// src/placerBase.cpp, src/nesterovBase.cpp, src/nesterovPlace.cpp,
// src/fft.cpp, src/fftsg.cpp, src/fftsg2d.cpp, src/logger.cpp and
// src/point.cpp (see Makefile) and an in-memory OpenDB stand-in (opendb/db.h).
//
// Modes
//   place <net.txt> [options]          Replace::doNesterovPlace after the
//                                      centre placement that
//                                      InitialPlace::placeInstsCenter does
//                                      (src/initialPlace.cpp:108-115) when the
//                                      initial place runs zero iterations.
//   eval  <net.txt> <out.bin> [opts]   one NesterovBase evaluation at seeded
//                                      random gcell centres (or the initial
//                                      density centres with --init-coords):
//                                      bin areas, density, phi, field, per-gcell
//                                      WA and density gradients, HPWL.
//                                      --coords <file> reads the centres
//                                      instead (raw float32 x, y per gcell).
//
// Options: --density d  --bins n  --idp p (init density penalty)  --iwc c
//          --minphi m --maxphi m --overflow o --maxiter n --incremental
//          --verbose v --seed s --init-coords --wlcoef c --out-pos file
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "opendb/db.h"
#include "refnet_db.h"
#include "placerBase.h"
#include "nesterovBase.h"
#include "nesterovPlace.h"
#include "logger.h"
#include "point.h"

using namespace replace;

struct Opts {
  float density = 0.7f;
  int bins = 0;
  float idp = 0.00008f;
  float iwc = 0.25f;
  float minphi = 0.95f, maxphi = 1.05f;
  float overflow = 0.1f;
  int maxiter = 2000;
  bool incremental = false;
  int verbose = 0;
  unsigned seed = 1;
  bool init_coords = false;
  float wlcoef = -1.0f;
  std::string out_pos;
  std::string coords;
};

static void parse_opts(int argc, char** argv, int start, Opts& o) {
  for (int i = start; i < argc; i++) {
    std::string a = argv[i];
    auto nxt = [&]() { return std::string(argv[++i]); };
    if (a == "--density") o.density = std::stof(nxt());
    else if (a == "--bins") o.bins = std::stoi(nxt());
    else if (a == "--idp") o.idp = std::stof(nxt());
    else if (a == "--iwc") o.iwc = std::stof(nxt());
    else if (a == "--minphi") o.minphi = std::stof(nxt());
    else if (a == "--maxphi") o.maxphi = std::stof(nxt());
    else if (a == "--overflow") o.overflow = std::stof(nxt());
    else if (a == "--maxiter") o.maxiter = std::stoi(nxt());
    else if (a == "--incremental") o.incremental = true;
    else if (a == "--verbose") o.verbose = std::stoi(nxt());
    else if (a == "--seed") o.seed = (unsigned)std::stoul(nxt());
    else if (a == "--init-coords") o.init_coords = true;
    else if (a == "--wlcoef") o.wlcoef = std::stof(nxt());
    else if (a == "--out-pos") o.out_pos = nxt();
    else if (a == "--coords") o.coords = nxt();
    else { fprintf(stderr, "unknown option %s\n", a.c_str()); exit(2); }
  }
}

// InitialPlace::placeInstsCenter (src/initialPlace.cpp:108-115)
static void place_center(PlacerBase& pb) {
  const int cx = pb.die().coreCx();
  const int cy = pb.die().coreCy();
  for (auto& inst : pb.placeInsts()) inst->setCenterLocation(cx, cy);
}

static NesterovBaseVars nb_vars(const Opts& o) {
  NesterovBaseVars v;
  v.targetDensity = o.density;
  if (o.bins) { v.isSetBinCntX = 1; v.binCntX = o.bins; v.isSetBinCntY = 1; v.binCntY = o.bins; }
  return v;
}

template <class T>
static void put(FILE* f, const char* name, const char* dt, const std::vector<T>& v) {
  fprintf(f, "%s %s %zu\n", name, dt, v.size());
  fwrite(v.data(), sizeof(T), v.size(), f);
  fprintf(f, "\n");
}

int main(int argc, char** argv) {
  if (argc < 3) { fprintf(stderr, "usage: ref_driver place|eval net.txt ...\n"); return 2; }
  std::string mode = argv[1];
  odb::dbDatabase* db = read_net(argv[2]);
  Opts o;
  if (mode == "place") {
    parse_opts(argc, argv, 3, o);
    auto log = std::make_shared<Logger>("REPL", o.verbose);
    auto pb = std::make_shared<PlacerBase>(db, log);
    if (!o.incremental) place_center(*pb);
    auto nb = std::make_shared<NesterovBase>(nb_vars(o), pb, log);
    NesterovPlaceVars npv;
    npv.minPhiCoef = o.minphi;
    npv.maxPhiCoef = o.maxphi;
    npv.initDensityPenalty = o.idp;
    npv.initWireLengthCoef = o.iwc;
    npv.targetOverflow = o.overflow;
    npv.maxNesterovIter = o.maxiter;
    NesterovPlace np(npv, pb, nb, log);
    np.doNesterovPlace();
    printf("[REF] FinalHPWL %lld\n", (long long)nb->getHpwl());
    fflush(stdout);
    if (!o.out_pos.empty()) {
      FILE* f = fopen(o.out_pos.c_str(), "w");
      for (auto* inst : db->chip->block->insts) fprintf(f, "%d %d\n", inst->x, inst->y);
      fclose(f);
    }
    return 0;
  }
  if (mode == "eval") {
    const char* out = argv[3];
    parse_opts(argc, argv, 4, o);
    auto log = std::make_shared<Logger>("REPL", o.verbose);
    auto pb = std::make_shared<PlacerBase>(db, log);
    if (!o.incremental) place_center(*pb);
    auto nb = std::make_shared<NesterovBase>(nb_vars(o), pb, log);
    const auto& gcells = nb->gCells();
    const int ng = (int)gcells.size();
    std::vector<FloatPoint> coords(ng);
    std::vector<float> given;
    if (!o.coords.empty()) {
      given.resize(2 * (size_t)ng);
      FILE* cf = fopen(o.coords.c_str(), "rb");
      if (!cf || fread(given.data(), sizeof(float), given.size(), cf) != given.size()) {
        fprintf(stderr, "cannot read %d coordinate pairs from %s\n", ng, o.coords.c_str());
        return 2;
      }
      fclose(cf);
    }
    std::mt19937 rng(o.seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<int32_t> ginfo;   // per gcell: lx ly ux uy dLx dLy dUx dUy kind
    std::vector<float> gscale;
    for (int i = 0; i < ng; i++) {
      GCell* g = gcells[i];
      nb->updateDensityCoordiLayoutInside(g);
      ginfo.insert(ginfo.end(), {g->lx(), g->ly(), g->ux(), g->uy(),
                                 g->dLx(), g->dLy(), g->dUx(), g->dUy(),
                                 g->isFiller() ? 2 : (g->isMacroInstance() ? 1 : 0)});
      gscale.push_back(g->densityScale());
      if (!given.empty()) {
        coords[i] = FloatPoint(given[2 * i], given[2 * i + 1]);
      } else if (o.init_coords) {
        coords[i] = FloatPoint(g->dCx(), g->dCy());
      } else {
        const Die& die = pb->die();
        double ddx = g->dDx(), ddy = g->dDy();
        double x = die.coreLx() + ddx / 2 + U(rng) * (die.coreDx() - ddx);
        double y = die.coreLy() + ddy / 2 + U(rng) * (die.coreDy() - ddy);
        coords[i] = FloatPoint((float)x, (float)y);
      }
    }
    nb->updateGCellDensityCenterLocation(coords);
    nb->updateDensityForceBin();
    float wl = o.wlcoef > 0 ? o.wlcoef : 1.0f / (0.5f * (nb->binSizeX() + nb->binSizeY()));
    nb->updateWireLengthForceWA(wl, wl);
    std::vector<float> xy(2 * ng), wlg(2 * ng), dg(2 * ng);
    std::vector<int32_t> drect;
    for (int i = 0; i < ng; i++) {
      GCell* g = gcells[i];
      xy[2 * i] = coords[i].x; xy[2 * i + 1] = coords[i].y;
      FloatPoint a = nb->getWireLengthGradientWA(g, wl, wl);
      FloatPoint b = nb->getDensityGradient(g);
      wlg[2 * i] = a.x; wlg[2 * i + 1] = a.y;
      dg[2 * i] = b.x; dg[2 * i + 1] = b.y;
      drect.insert(drect.end(), {g->dLx(), g->dLy(), g->dUx(), g->dUy()});
    }
    std::vector<int64_t> inst_a, fill_a, np_a;
    std::vector<float> dens, phi, ex, ey;
    for (auto* bin : nb->bins()) {
      inst_a.push_back(bin->instPlacedArea());
      fill_a.push_back(bin->fillerArea());
      np_a.push_back(bin->nonPlaceArea());
      dens.push_back(bin->density());
      phi.push_back(bin->electroPhi());
      ex.push_back(bin->electroForceX());
      ey.push_back(bin->electroForceY());
    }
    std::vector<int32_t> grid = {nb->binCntX(), nb->binCntY(), nb->binSizeX(), nb->binSizeY()};
    std::vector<int64_t> scal = {nb->overflowArea(), nb->getHpwl(), pb->stdInstsArea(),
                                 pb->macroInstsArea(), pb->nonPlaceInstsArea(),
                                 (int64_t)gcells.size(), (int64_t)nb->gCellFillers().size()};
    std::vector<float> fscal = {nb->sumPhi(), wl};
    FILE* f = fopen(out, "wb");
    put(f, "grid", "i4", grid);
    put(f, "scalars", "i8", scal);
    put(f, "fscalars", "f4", fscal);
    put(f, "ginfo", "i4", ginfo);
    put(f, "gscale", "f4", gscale);
    put(f, "coords", "f4", xy);
    put(f, "drect", "i4", drect);
    put(f, "wl_grad", "f4", wlg);
    put(f, "density_grad", "f4", dg);
    put(f, "inst_area", "i8", inst_a);
    put(f, "filler_area", "i8", fill_a);
    put(f, "nonplace_area", "i8", np_a);
    put(f, "density", "f4", dens);
    put(f, "phi", "f4", phi);
    put(f, "ex", "f4", ex);
    put(f, "ey", "f4", ey);
    fclose(f);
    return 0;
  }
  fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
