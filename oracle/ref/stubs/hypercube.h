// Stand-in for SEP hypercube (test infrastructure only): axes 1..ndim, the
// first axis fastest.
#pragma once
#include <algorithm>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <vector>
#include "SEPException.h"
#include "axis.h"
namespace SEP {
class hypercube {
 public:
  hypercube() {}
  explicit hypercube(const std::vector<axis>& a) : _axes(a) {}
  hypercube(const axis& a1) : _axes{a1} {}
  hypercube(const axis& a1, const axis& a2) : _axes{a1, a2} {}
  hypercube(const axis& a1, const axis& a2, const axis& a3) : _axes{a1, a2, a3} {}
  hypercube(const axis& a1, const axis& a2, const axis& a3, const axis& a4) : _axes{a1, a2, a3, a4} {}
  // 1-based, as SEP; axes past ndim are of length 1
  axis getAxis(int i) const {
    if (i < 1) throw std::out_of_range("hypercube::getAxis");
    return i <= (int)_axes.size() ? _axes[i - 1] : axis(1);
  }
  void setAxis(int i, const axis& a) {
    if ((int)_axes.size() < i) _axes.resize(i);
    _axes[i - 1] = a;
  }
  std::vector<axis> getAxes() const { return _axes; }
  std::vector<axis> getAxes(int n) const {
    std::vector<axis> a = _axes;
    a.resize(n);
    return a;
  }
  std::vector<int> getNs() const {
    std::vector<int> n;
    for (const auto& a : _axes) n.push_back(a.n);
    return n;
  }
  long long getN123() const {
    long long n = 1;
    for (const auto& a : _axes) n *= a.n;
    return n;
  }
  int getNdim() const { return (int)_axes.size(); }
  int getNdimG1() const {
    int n = (int)_axes.size();
    while (n > 1 && _axes[n - 1].n == 1) --n;
    return n;
  }
  bool checkSame(const std::shared_ptr<hypercube>& o) const {
    if (!o || o->_axes.size() != _axes.size()) return false;
    for (size_t i = 0; i < _axes.size(); ++i)
      if (o->_axes[i].n != _axes[i].n) return false;
    return true;
  }
  void infoStream(std::stringstream& x) const {
    for (size_t i = 0; i < _axes.size(); ++i) x << "axis " << i + 1 << " n=" << _axes[i].n << "\n";
  }

 private:
  std::vector<axis> _axes;
};
}  // namespace SEP
