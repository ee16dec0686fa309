// Stand-in for sepVector's float2DReg (test infrastructure only).
#pragma once
#include <vector>
#include "floatHyper.h"
#include "boost/multi_array.hpp"
typedef boost::multi_array<float, 2> float2D;
namespace SEP {
class float2DReg : public floatHyper {
 public:
  float2DReg() {}
  float2DReg(std::shared_ptr<hypercube> h) { init(h); }
  float2DReg(const int n1, const int n2) {
    std::vector<axis> a;
    a.push_back(axis(n1));
    a.push_back(axis(n2));
    init(std::make_shared<hypercube>(a));
  }
  float2DReg(const axis& a1, const axis& a2) {
    std::vector<axis> a;
    a.push_back(a1);
    a.push_back(a2);
    init(std::make_shared<hypercube>(a));
  }
  float2DReg(std::shared_ptr<hypercube> h, const float2D& vals) {
    init(h);
    std::copy(vals.data(), vals.data() + vals.num_elements(), _mat->data());
  }
  std::shared_ptr<float2DReg> clone() const {
    auto x = std::make_shared<float2DReg>(getHyper());
    if (!getSpaceOnly()) std::copy(_mat->data(), _mat->data() + _mat->num_elements(), x->_mat->data());
    return x;
  }
  std::shared_ptr<float2DReg> cloneSpace() const {
    auto x = std::make_shared<float2DReg>(getHyper());
    x->setSpace();
    return x;
  }
  void allocate() { init(getHyper()); }
  virtual void cleanMemory() { setSpace(); }
  std::shared_ptr<float2D> _mat;

 private:
  void init(std::shared_ptr<hypercube> h) {
    setHyper(h);
    std::vector<axis> ax = h->getAxes();
    ax.resize(2, axis(1));
    _mat.reset(new float2D(boost::extents[ax[1].n][ax[0].n]));
    setData(_mat->data());
  }
};
}  // namespace SEP
#include "sep_all.h"
