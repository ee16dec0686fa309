// ORACLE — test infrastructure only.  Construction of the conformal maps
// restated in cmap_oracle.hpp (conformal/src: ShiftAndScale.h, ComplexLog.h,
// Rotation.h; propagator/src/PropParam.h:88-137).  Compiled with
// -ffp-contract=off: float coordinates are truncated to grid cells, so the
// rounding must not change with the machine.  PARITY PINNED to the reference
// run (tests/test_ref_pin.py).
#include "cmap_oracle.hpp"

namespace wo {
namespace cm {
namespace {
const float kPiMap = 4 * std::atan(1.f);  // ConformalMap.h:119
}  // namespace

std::vector<cf> regular_coord(const Hyper& h) {
  std::vector<cf> c(h.n());
  for (int i2 = 0; i2 < h.n2; ++i2) {
    const float z = h.o2 + i2 * h.d2;
    for (int i1 = 0; i1 < h.n1; ++i1) {
      const float x = h.o1 + i1 * h.d1;
      c[(size_t)i1 + (size_t)i2 * h.n1] = cf(z, x);
    }
  }
  return c;
}

// ConformalMap.h:86-94
void Map::complexify() {
  zcoord = regular_coord(in);
  ucoord = regular_coord(out);
  zmap.assign(in.n(), cf(0));
  umap.assign(in.n(), cf(0));
  jacob.assign(in.n(), 1.f);
}

// ShiftAndScale.h:12-58: f(z) = a (z - b)
std::unique_ptr<Map> shift_and_scale(const Hyper& h, cf a, cf b) {
  auto m = std::make_unique<Map>();
  m->in = h;
  cf mn(h.o2, h.o1), mx(h.o2 + (h.n2 - 1) * h.d2, h.o1 + (h.n1 - 1) * h.d1);
  mn = a * (mn - b);
  mx = a * (mx - b);
  m->out = Hyper{h.n1, h.n2, mn.imag(), (mx - mn).imag() / (h.n1 - 1), mn.real(), (mx - mn).real() / (h.n2 - 1)};
  m->complexify();
  for (size_t i = 0; i < m->zcoord.size(); ++i) {
    m->zmap[i] = m->ucoord[i] / a + b;
    m->umap[i] = a * (m->zcoord[i] - b);
  }
  for (size_t i = 0; i < m->zcoord.size(); ++i) m->jacob[i] = std::abs(1.f / a);
  return m;
}

// ComplexLog.h:12-71: w = log z on the annulus eps <= |z| <= 1
std::unique_ptr<Map> complex_log(const Hyper& h, float eps) {
  auto m = std::make_unique<Map>();
  m->in = h;
  m->is_log = true;
  m->leps = std::log(eps);
  m->out = Hyper{h.n1, h.n2, 0.f, 2 * kPiMap / (h.n1 - 1), m->leps, -m->leps / (h.n2 - 1)};
  m->complexify();
  const cf ip(0, kPiMap);
  for (size_t i = 0; i < m->zcoord.size(); ++i) {
    m->zmap[i] = std::exp(m->ucoord[i]);
    const cf zz = m->zcoord[i];
    if (std::abs(zz) < std::exp(m->leps)) m->umap[i] = cf(m->leps, std::arg(zz));
    else m->umap[i] = std::log(zz);
    if (m->umap[i].imag() < 0) m->umap[i] += 2.f * ip;
  }
  for (size_t i = 0; i < m->zcoord.size(); ++i) m->jacob[i] = std::exp(m->ucoord[i].real());
  return m;
}

// Rotation.h:12-100: rotation by exp(-i rad) into the bounding box of the
// rotated corners and the origin
std::unique_ptr<Map> rotation(const Hyper& h, float rad) {
  auto m = std::make_unique<Map>();
  m->in = h;
  const cf I(0, 1);
  const cf rot = std::exp(-I * rad), irot = std::exp(I * rad);
  cf v[4] = {cf(h.o2, h.o1), cf(h.o2, h.o1 + (h.n1 - 1) * h.d1), cf(h.o2 + (h.n2 - 1) * h.d2, h.o1),
             cf(h.o2 + (h.n2 - 1) * h.d2, h.o1 + (h.n1 - 1) * h.d1)};
  float o1 = 0, o2 = 0, max1 = 0, max2 = 0;
  for (int i = 0; i < 4; ++i) {
    const cf u = v[i] * rot;
    o1 = std::min(o1, u.imag());
    o2 = std::min(o2, u.real());
    max1 = std::max(max1, u.imag());
    max2 = std::max(max2, u.real());
  }
  m->out = Hyper{h.n1, h.n2, o1, (max1 - o1) / (h.n1 - 1), o2, (max2 - o2) / (h.n2 - 1)};
  m->complexify();
  const float m1 = (h.n1 - 1) * h.d1 + h.o1, m2 = (h.n2 - 1) * h.d2 + h.o2;
  for (size_t i = 0; i < m->zcoord.size(); ++i) {
    cf z = m->ucoord[i] * irot;
    const int i1 = (int)((z.imag() - h.o1) / h.d1);
    const int i2 = (int)((z.real() - h.o2) / h.d2);
    float x;
    if (i1 < 0) {
      x = -(z.imag() - h.o1) / std::tan(rad);
      x = std::min(z.real() + x, m2);
      z = cf(x, h.o1);
    }
    if (i2 < 0) {
      x = -(z.real() - h.o2) * std::tan(rad);
      x = std::min(z.imag() + x, m1);
      z = cf(h.o2, x);
    }
    if (i1 >= h.n1) {
      x = (z.imag() - m1) / std::tan(rad);
      x = std::max(z.real() - x, h.o1);
      z = cf(x, m1);
    }
    if (i2 >= h.n2) {
      x = (z.real() - m2) * std::tan(rad);
      x = std::min(z.imag() - x, h.o1);
      z = cf(m2, x);
    }
    m->zmap[i] = z;
    m->umap[i] = m->zcoord[i] * rot;
  }
  return m;
}

// PropParam.h:88-137 for shot is: the source at grid (sz, sx) of the model
ShotChain shot_chain(int cmap, const Hyper& model, int sz, int sx, float eps_log, float angle) {
  ShotChain c;
  if (cmap == 1) {
    cf a = 0, b;
    const float z = model.o2 + sz * model.d2, x = model.o1 + sx * model.d1;
    b = cf(z, x);
    for (int i2 = 0; i2 < model.n2; i2 += model.n2 - 1)
      for (int i1 = 0; i1 < model.n1; i1 += model.n1 - 1) {
        const cf corner(model.o2 + i2 * model.d2, model.o1 + i1 * model.d1);
        a = std::max(a.real(), std::abs(corner - b));
      }
    a = 1.f / a;
    c.maps.push_back(shift_and_scale(model, a, b));
    c.maps.push_back(complex_log(c.maps[0]->out, eps_log));
  } else {
    c.maps.push_back(rotation(model, angle));
  }
  return c;
}

}  // namespace cm
}  // namespace wo
