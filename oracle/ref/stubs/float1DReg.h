// Stand-in for sepVector's float1DReg (test infrastructure only).
#pragma once
#include <vector>
#include "floatHyper.h"
#include "boost/multi_array.hpp"
typedef boost::multi_array<float, 1> float1D;
namespace SEP {
class float1DReg : public floatHyper {
 public:
  float1DReg() {}
  float1DReg(std::shared_ptr<hypercube> h) { init(h); }
  float1DReg(const int n1) {
    std::vector<axis> a;
    a.push_back(axis(n1));
    init(std::make_shared<hypercube>(a));
  }
  float1DReg(const axis& a1) {
    std::vector<axis> a;
    a.push_back(a1);
    init(std::make_shared<hypercube>(a));
  }
  float1DReg(std::shared_ptr<hypercube> h, const float1D& vals) {
    init(h);
    std::copy(vals.data(), vals.data() + vals.num_elements(), _mat->data());
  }
  std::shared_ptr<float1DReg> clone() const {
    auto x = std::make_shared<float1DReg>(getHyper());
    if (!getSpaceOnly()) std::copy(_mat->data(), _mat->data() + _mat->num_elements(), x->_mat->data());
    return x;
  }
  std::shared_ptr<float1DReg> cloneSpace() const {
    auto x = std::make_shared<float1DReg>(getHyper());
    x->setSpace();
    return x;
  }
  void allocate() { init(getHyper()); }
  virtual void cleanMemory() { setSpace(); }
  std::shared_ptr<float1D> _mat;

 private:
  void init(std::shared_ptr<hypercube> h) {
    setHyper(h);
    std::vector<axis> ax = h->getAxes();
    ax.resize(1, axis(1));
    _mat.reset(new float1D(boost::extents[ax[0].n]));
    setData(_mat->data());
  }
};
}  // namespace SEP
#include "sep_all.h"
