// In-memory stand-in for the slice of the OpenDB API that RePlAce's
// placerBase.cpp / nesterovBase.cpp / nesterovPlace.cpp call.
//
// TEST INFRASTRUCTURE ONLY.  This header lets the reference's own placement
// sources compile unchanged (from the reference tree, into oracle/_ref/) so
// that its outputs can pin the oracle restatement.  Nothing in the product
// includes it.  The object model is populated by ref_driver.cpp from a plain
// text netlist.
#ifndef GPL_REFBUILD_OPENDB_STUB_H
#define GPL_REFBUILD_OPENDB_STUB_H

#include <climits>
#include <cstdint>
#include <string>
#include <vector>

namespace odb {

class Rect {
 public:
  Rect() : xl_(0), yl_(0), xh_(0), yh_(0) {}
  Rect(int xl, int yl, int xh, int yh) : xl_(xl), yl_(yl), xh_(xh), yh_(yh) {}
  int xMin() const { return xl_; }
  int yMin() const { return yl_; }
  int xMax() const { return xh_; }
  int yMax() const { return yh_; }
  int xl_, yl_, xh_, yh_;
};

class dbBox {
 public:
  dbBox() : xl(0), yl(0), xh(0), yh(0) {}
  dbBox(int a, int b, int c, int d) : xl(a), yl(b), xh(c), yh(d) {}
  int xMin() const { return xl; }
  int yMin() const { return yl; }
  int xMax() const { return xh; }
  int yMax() const { return yh; }
  int getDX() const { return xh - xl; }
  int getDY() const { return yh - yl; }
  int xl, yl, xh, yh;
};

template <class T>
class dbSet {
 public:
  typedef typename std::vector<T*>::const_iterator iterator;
  dbSet() : v_(nullptr) {}
  explicit dbSet(const std::vector<T*>* v) : v_(v) {}
  iterator begin() const { return v_->begin(); }
  iterator end() const { return v_->end(); }
  unsigned size() const { return (unsigned)v_->size(); }
 private:
  const std::vector<T*>* v_;
};

class dbPlacementStatus {
 public:
  enum Value { NONE, UNPLACED, SUGGESTED, PLACED, LOCKED, FIRM, COVER };
  dbPlacementStatus() : v_(NONE) {}
  dbPlacementStatus(Value v) : v_(v) {}
  operator Value() const { return v_; }
 private:
  Value v_;
};

class dbSigType {
 public:
  enum Value { SIGNAL, POWER, GROUND, CLOCK, ANALOG, RESET, SCAN, TIEOFF };
  dbSigType() : v_(SIGNAL) {}
  dbSigType(Value v) : v_(v) {}
  operator Value() const { return v_; }
 private:
  Value v_;
};

class dbSite {
 public:
  int w = 0, h = 0;
  int getWidth() const { return w; }
  int getHeight() const { return h; }
};

class dbRow {
 public:
  Rect box;
  dbSite* site = nullptr;
  void getBBox(Rect& r) const { r = box; }
  dbSite* getSite() const { return site; }
};

class dbMaster {
 public:
  int w = 0, h = 0;
  int getWidth() const { return w; }
  int getHeight() const { return h; }
};

class dbMPin {
 public:
  std::vector<dbBox*> boxes;
  dbSet<dbBox> getGeometry() const { return dbSet<dbBox>(&boxes); }
};

class dbMTerm {
 public:
  std::vector<dbMPin*> mpins;
  dbSet<dbMPin> getMPins() const { return dbSet<dbMPin>(&mpins); }
};

class dbInst;
class dbNet;

class dbITerm {
 public:
  dbInst* inst = nullptr;
  dbMTerm* mterm = nullptr;
  dbInst* getInst() const { return inst; }
  dbMTerm* getMTerm() const { return mterm; }
};

class dbInst {
 public:
  int x = 0, y = 0, w = 0, h = 0;
  dbBox bbox;
  dbMaster* master = nullptr;
  dbPlacementStatus status;
  std::vector<dbITerm*> iterms;
  void getLocation(int& ox, int& oy) const { ox = x; oy = y; }
  dbBox* getBBox() { bbox = dbBox(x, y, x + w, y + h); return &bbox; }
  dbPlacementStatus getPlacementStatus() const { return status; }
  void setPlacementStatus(dbPlacementStatus s) { status = s; }
  void setLocation(int nx, int ny) { x = nx; y = ny; bbox = dbBox(x, y, x + w, y + h); }
  dbMaster* getMaster() const { return master; }
  dbSet<dbITerm> getITerms() const { return dbSet<dbITerm>(&iterms); }
};

class dbBPin {
 public:
  dbBox box;
  dbBox* getBox() { return &box; }
};

class dbBTerm {
 public:
  std::string name;
  std::vector<dbBPin*> bpins;
  dbSet<dbBPin> getBPins() const { return dbSet<dbBPin>(&bpins); }
  const char* getConstName() const { return name.c_str(); }
};

class dbNet {
 public:
  dbSigType sig;
  std::vector<dbITerm*> iterms;
  std::vector<dbBTerm*> bterms;
  dbSigType getSigType() const { return sig; }
  dbSet<dbITerm> getITerms() const { return dbSet<dbITerm>(&iterms); }
  dbSet<dbBTerm> getBTerms() const { return dbSet<dbBTerm>(&bterms); }
};

class dbBlock {
 public:
  std::vector<dbInst*> insts;
  std::vector<dbRow*> rows;
  std::vector<dbNet*> nets;
  dbBox bbox;
  dbSet<dbInst> getInsts() const { return dbSet<dbInst>(&insts); }
  dbSet<dbRow> getRows() const { return dbSet<dbRow>(&rows); }
  dbSet<dbNet> getNets() const { return dbSet<dbNet>(&nets); }
  dbBox* getBBox() { return &bbox; }
};

class dbChip {
 public:
  dbBlock* block = nullptr;
  dbBlock* getBlock() const { return block; }
};

class dbTech {
 public:
  int dbu = 2000;
  int getDbUnitsPerMicron() const { return dbu; }
};

class dbDatabase {
 public:
  dbTech* tech = nullptr;
  dbChip* chip = nullptr;
  dbTech* getTech() const { return tech; }
  dbChip* getChip() const { return chip; }
};

}  // namespace odb

#endif
