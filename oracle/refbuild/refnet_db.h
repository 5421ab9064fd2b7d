// Reads the plain-text netlist format of refnet.py into the in-memory
// OpenDB stand-in (opendb/db.h).
//
// TEST INFRASTRUCTURE ONLY: shared by the reference-build driver
// (ref_driver.cpp) and the driver of the replace::Replace facade tests.
#ifndef GPL_REFBUILD_REFNET_DB_H
#define GPL_REFBUILD_REFNET_DB_H

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "opendb/db.h"

inline odb::dbDatabase* read_net(const char* path) {
  std::ifstream in(path);
  if (!in) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  std::string tag;
  auto db = new odb::dbDatabase();
  db->tech = new odb::dbTech();
  db->chip = new odb::dbChip();
  auto blk = new odb::dbBlock();
  db->chip->block = blk;
  auto site = new odb::dbSite();
  int nrows = 0, ninst = 0, nnet = 0;
  in >> tag;  // REFNET
  int ver; in >> ver;
  in >> tag >> db->tech->dbu;                       // DBU
  in >> tag >> site->w >> site->h;                  // SITE
  in >> tag >> blk->bbox.xl >> blk->bbox.yl >> blk->bbox.xh >> blk->bbox.yh;  // DIE
  in >> tag >> nrows;                               // ROWS
  for (int i = 0; i < nrows; i++) {
    auto r = new odb::dbRow();
    in >> r->box.xl_ >> r->box.yl_ >> r->box.xh_ >> r->box.yh_;
    r->site = site;
    blk->rows.push_back(r);
  }
  in >> tag >> ninst;                               // INSTS
  std::vector<std::vector<std::pair<int, odb::dbITerm*>>> inst_terms(ninst);
  for (int i = 0; i < ninst; i++) {
    auto inst = new odb::dbInst();
    int st;
    inst->master = new odb::dbMaster();
    in >> inst->x >> inst->y >> inst->w >> inst->h >> inst->master->w >> inst->master->h >> st;
    inst->status = st ? odb::dbPlacementStatus::FIRM : odb::dbPlacementStatus::NONE;
    inst->bbox = odb::dbBox(inst->x, inst->y, inst->x + inst->w, inst->y + inst->h);
    blk->insts.push_back(inst);
  }
  in >> tag >> nnet;                                // NETS
  for (int n = 0; n < nnet; n++) {
    auto net = new odb::dbNet();
    int sig, ni, nb;
    in >> sig >> ni >> nb;
    net->sig = (odb::dbSigType::Value)sig;
    for (int k = 0; k < ni; k++) {
      int inst, key, has, xl, yl, xh, yh;
      in >> inst >> key >> has >> xl >> yl >> xh >> yh;
      auto it = new odb::dbITerm();
      it->inst = blk->insts[inst];
      it->mterm = new odb::dbMTerm();
      if (has) {
        auto mp = new odb::dbMPin();
        mp->boxes.push_back(new odb::dbBox(xl, yl, xh, yh));
        it->mterm->mpins.push_back(mp);
      }
      net->iterms.push_back(it);
      inst_terms[inst].push_back({key, it});
    }
    for (int k = 0; k < nb; k++) {
      int has, xl, yl, xh, yh;
      in >> has >> xl >> yl >> xh >> yh;
      auto bt = new odb::dbBTerm();
      bt->name = "io" + std::to_string(n) + "_" + std::to_string(k);
      if (has) {
        auto bp = new odb::dbBPin();
        bp->box = odb::dbBox(xl, yl, xh, yh);
        bt->bpins.push_back(bp);
      }
      net->bterms.push_back(bt);
    }
    blk->nets.push_back(net);
  }
  // instance iterm order = master pin order (stable by key)
  for (int i = 0; i < ninst; i++) {
    auto& v = inst_terms[i];
    std::stable_sort(v.begin(), v.end(),
                     [](const std::pair<int, odb::dbITerm*>& a,
                        const std::pair<int, odb::dbITerm*>& b) { return a.first < b.first; });
    for (auto& p : v) blk->insts[i]->iterms.push_back(p.second);
  }
  return db;
}

#endif
