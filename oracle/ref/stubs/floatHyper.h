// Stand-in for sepVector's floatHyper (test infrastructure only): a float
// array over a hypercube with the arithmetic the reference calls.
#pragma once
#include <algorithm>
#include <cassert>
#include <functional>
#include <iostream>
#include <numeric>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <sstream>
#include "SEPException.h"
#include "Vector.h"
#include "hypercube.h"
namespace SEP {
class floatHyper : public Vector {
 public:
  floatHyper() {}
  float* getVals() { return _vals; }
  const float* getCVals() const { return _vals; }
  std::shared_ptr<hypercube> getHyper() const { return _hyper; }
  void setHyper(std::shared_ptr<hypercube> h) { _hyper = h; }
  void setData(float* p) {
    _vals = p;
    setNotSpace();
  }
  bool getSpaceOnly() const { return _spaceOnly; }
  virtual void add(std::shared_ptr<floatHyper> v) {
    for (long long i = 0; i < _hyper->getN123(); ++i) _vals[i] += v->_vals[i];
  }
  virtual void scale(const double s) {
    for (long long i = 0; i < _hyper->getN123(); ++i) _vals[i] = _vals[i] * s;
  }
  virtual void scaleAdd(std::shared_ptr<floatHyper> v, const double s1, const double s2) {
    for (long long i = 0; i < _hyper->getN123(); ++i) _vals[i] = _vals[i] * s1 + s2 * v->_vals[i];
  }
  virtual void set(const float v) {
    for (long long i = 0; i < _hyper->getN123(); ++i) _vals[i] = v;
  }
  virtual void zero() { set(0.f); }
  virtual void random() {
    for (long long i = 0; i < _hyper->getN123(); ++i) _vals[i] = ((double)rand() / RAND_MAX) - .5;
  }
  virtual double dot(std::shared_ptr<floatHyper> v) const {
    double d = 0.;
    for (long long i = 0; i < _hyper->getN123(); ++i) d += (double)_vals[i] * (double)v->_vals[i];
    return d;
  }
  virtual float absMax() const {
    float m = 0.f;
    for (long long i = 0; i < _hyper->getN123(); ++i) m = std::max(m, std::fabs(_vals[i]));
    return m;
  }
  bool checkSame(const std::shared_ptr<floatHyper> v) const { return (bool)v; }
  void calcCheckSum() {}

 private:
  std::shared_ptr<hypercube> _hyper;
  float* _vals = nullptr;
};
}  // namespace SEP

