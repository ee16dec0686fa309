// Stand-in for sepVector's float4DReg (test infrastructure only).
#pragma once
#include <vector>
#include "floatHyper.h"
#include "boost/multi_array.hpp"
typedef boost::multi_array<float, 4> float4D;
namespace SEP {
class float4DReg : public floatHyper {
 public:
  float4DReg() {}
  float4DReg(std::shared_ptr<hypercube> h) { init(h); }
  float4DReg(const int n1, const int n2, const int n3, const int n4) {
    std::vector<axis> a;
    a.push_back(axis(n1));
    a.push_back(axis(n2));
    a.push_back(axis(n3));
    a.push_back(axis(n4));
    init(std::make_shared<hypercube>(a));
  }
  float4DReg(const axis& a1, const axis& a2, const axis& a3, const axis& a4) {
    std::vector<axis> a;
    a.push_back(a1);
    a.push_back(a2);
    a.push_back(a3);
    a.push_back(a4);
    init(std::make_shared<hypercube>(a));
  }
  float4DReg(std::shared_ptr<hypercube> h, const float4D& vals) {
    init(h);
    std::copy(vals.data(), vals.data() + vals.num_elements(), _mat->data());
  }
  std::shared_ptr<float4DReg> clone() const {
    auto x = std::make_shared<float4DReg>(getHyper());
    if (!getSpaceOnly()) std::copy(_mat->data(), _mat->data() + _mat->num_elements(), x->_mat->data());
    return x;
  }
  std::shared_ptr<float4DReg> cloneSpace() const {
    auto x = std::make_shared<float4DReg>(getHyper());
    x->setSpace();
    return x;
  }
  void allocate() { init(getHyper()); }
  virtual void cleanMemory() { setSpace(); }
  std::shared_ptr<float4D> _mat;

 private:
  void init(std::shared_ptr<hypercube> h) {
    setHyper(h);
    std::vector<axis> ax = h->getAxes();
    ax.resize(4, axis(1));
    _mat.reset(new float4D(boost::extents[ax[3].n][ax[2].n][ax[1].n][ax[0].n]));
    setData(_mat->data());
  }
};
}  // namespace SEP
#include "sep_all.h"
