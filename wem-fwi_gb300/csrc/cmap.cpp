// Conformal-map geometry (cmap.h).  Every map is built on the host in the
// reference's float complex arithmetic (std::complex<float>, the same
// library calls), and reduced to what the GPU needs: two gather tables
// (model -> mapped grid, mapped grid -> model), the Jacobian and the mapped
// devices.  Grid coordinates are z + i x (real part depth, imaginary part
// lateral), as in the reference; a coordinate becomes a grid index by the
// reference's truncating int conversion.
//
//   cmap 1: ShiftAndScale(a, b) then ComplexLog(eps_log)  (PropParam.h:89-111)
//     b = the source position, a = 1 / (largest distance from b to a corner):
//     the model maps into the unit disc around the source, then
//     w = log(z): depth = log radius in [log eps_log, 0], x = angle in
//     [0, 2 pi].  Model samples reach the log grid by nearest neighbour
//     (ConformalMap.cpp:59-79 for the shift and scale, ComplexLog.cpp:103-137
//     for the log, whose points outside the disc repeat the last value met in
//     their column); images come back through the annulus
//     eps_log < |z| < 0.99 (ComplexLog.cpp:139-160) and the shift and scale
//     (ConformalMap.cpp:81-101).  The source becomes the whole first mapped
//     depth (ComplexLog.cpp:203-227), each receiver its log image with the
//     depth index clamped at 0 (ComplexLog.cpp:162-201).
//   cmap 2: Rotation(angle of the shot)  (PropParam.h:113-130, Rotation.h):
//     the grid rotated by exp(-i angle) into its bounding box (which always
//     holds the origin); preimages that leave the model are moved back to
//     its edges by the reference's rules (Rotation.h:55-86).  Jacobian 1.
//
// Mapped points whose preimage falls outside the model get zero, and model
// points whose image falls outside the mapped grid get a zero image.  The
// reference leaves those points of its per-task buffers untouched instead
// (ConformalMap.cpp:73-77, 95-99), so there they hold what the task's
// previous shot left, or zero for its first shot.
#include "cmap.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <string>

namespace wg {
namespace {

using cf = std::complex<float>;

struct Grid {
  int n1 = 0, n2 = 0;
  float o1 = 0, d1 = 1, o2 = 0, d2 = 1;
  size_t size() const { return (size_t)n1 * n2; }
  // coordinate of sample (i1, i2) (ConformalMap.h:96-108)
  cf at(int i1, int i2) const { return cf(o2 + i2 * d2, o1 + i1 * d1); }
  cf at(size_t k) const { return at((int)(k % n1), (int)(k / n1)); }
  bool inside(int i1, int i2) const { return i1 >= 0 && i1 < n1 && i2 >= 0 && i2 < n2; }
  // truncating index of a coordinate along each axis
  int c1(const cf& z) const { return (int)((z.imag() - o1) / d1); }
  int c2(const cf& z) const { return (int)((z.real() - o2) / d2); }
};

// pi as the conformal maps hold it (ConformalMap.h:119)
const float kPiF = 4 * std::atan(1.f);

// nearest-neighbour source table of a gather: out point i takes the in point
// its coordinate map[i] lands on, -1 outside
std::vector<int> nearest(const Grid& in, const std::vector<cf>& map) {
  std::vector<int> idx(map.size(), -1);
  for (size_t i = 0; i < map.size(); ++i) {
    const int i1 = in.c1(map[i]), i2 = in.c2(map[i]);
    if (in.inside(i1, i2)) idx[i] = i2 * in.n1 + i1;
  }
  return idx;
}

void shift_log_map(const wem_params& p, const Geometry& g, const Grid& model, int is, ShotMap& sm) {
  const int n1 = model.n1, n2 = model.n2;
  // a = 1 / max |corner - b|, b = source (PropParam.h:89-105)
  const cf b(model.o2 + g.sz[is] * model.d2, model.o1 + g.sx[is] * model.d1);
  float amax = 0;
  for (int i2 : {0, n2 - 1})
    for (int i1 : {0, n1 - 1}) amax = std::max(amax, std::abs(model.at(i1, i2) - b));
  const cf a = 1.f / cf(amax, 0.f);
  // shift and scale: f(z) = a (z - b) onto the box of the model's image
  // (ShiftAndScale.h:29-53)
  Grid sg;
  {
    cf lo(model.o2, model.o1), hi(model.o2 + (n2 - 1) * model.d2, model.o1 + (n1 - 1) * model.d1);
    lo = a * (lo - b);
    hi = a * (hi - b);
    sg = Grid{n1, n2, lo.imag(), (hi - lo).imag() / (n1 - 1), lo.real(), (hi - lo).real() / (n2 - 1)};
  }
  std::vector<cf> s_pre(sg.size()), s_img(model.size());
  for (size_t k = 0; k < sg.size(); ++k) s_pre[k] = sg.at(k) / a + b;
  for (size_t k = 0; k < model.size(); ++k) s_img[k] = a * (model.at(k) - b);
  // complex log with inner radius eps_log (ComplexLog.h:37-67)
  const float leps = std::log(p.eps_log);
  const Grid lg{n1, n2, 0.f, 2 * kPiF / (n1 - 1), leps, -leps / (n2 - 1)};
  std::vector<cf> l_pre(lg.size()), l_img(sg.size());
  for (size_t k = 0; k < lg.size(); ++k) l_pre[k] = std::exp(lg.at(k));
  const float rmin = std::exp(leps);
  for (size_t k = 0; k < sg.size(); ++k) {
    const cf zz = sg.at(k);
    cf u = std::abs(zz) < rmin ? cf(leps, std::arg(zz)) : std::log(zz);
    if (u.imag() < 0) u += 2.f * cf(0, kPiF);
    l_img[k] = u;
  }
  sm.o1 = lg.o1;
  sm.d1 = lg.d1;
  sm.o2 = lg.o2;
  sm.d2 = lg.d2;
  // model -> log grid: the shift and scale's nearest neighbour, then the
  // log's, whose misses repeat the column's last hit
  const std::vector<int> s_fwd = nearest(model, s_pre);
  sm.fwd.assign(lg.size(), -1);
  std::vector<int> column(n1, -1);
  for (int i2 = 0; i2 < n2; ++i2)
    for (int i1 = 0; i1 < n1; ++i1) {
      const cf z = l_pre[(size_t)i2 * n1 + i1];
      const int j1 = sg.c1(z), j2 = sg.c2(z);
      if (sg.inside(j1, j2)) column[i1] = j2 * n1 + j1;
      sm.fwd[(size_t)i2 * n1 + i1] = column[i1] >= 0 ? s_fwd[column[i1]] : -1;
    }
  // log grid -> model: through the annulus, then the shift and scale
  std::vector<int> l_inv(sg.size(), -1);
  for (size_t k = 0; k < sg.size(); ++k) {
    const float r = std::abs(sg.at(k));
    if (r > rmin && r < .99f) {
      const int j1 = lg.c1(l_img[k]), j2 = lg.c2(l_img[k]);
      if (lg.inside(j1, j2)) l_inv[k] = j2 * n1 + j1;
    }
  }
  sm.inv.assign(model.size(), -1);
  for (size_t m = 0; m < model.size(); ++m) {
    const int j1 = sg.c1(s_img[m]), j2 = sg.c2(s_img[m]);
    if (sg.inside(j1, j2)) sm.inv[m] = l_inv[(size_t)j2 * n1 + j1];
  }
  // Jacobians: |1 / a| of the shift and scale, exp(Re w) of the log
  // (ShiftAndScale.h:47-52, ComplexLog.h:61-65)
  sm.js = std::abs(1.f / a);
  sm.jl.resize(lg.size());
  for (size_t k = 0; k < lg.size(); ++k) sm.jl[k] = std::exp(lg.at(k).real());
  // the source: the first log depth across the grid
  sm.src_z = 0;
  sm.src_x.resize(n1);
  for (int i = 0; i < n1; ++i) sm.src_x[i] = i;
  // receivers: shift-and-scale cell, then its log image, depth clamped at 0
  require(g.nr >= 2, "cmap 1 needs at least 2 receivers (one receiver becomes a line, ComplexLog.cpp:203-227)");
  for (int r = 0; r < g.nr; ++r) {
    require(g.rx[r] < n1 && g.rz[r] < n2, "cmap: a receiver lies outside the model");
    const cf u = s_img[(size_t)g.rz[r] * n1 + g.rx[r]];
    const int j1 = sg.c1(u), j2 = sg.c2(u);
    require(sg.inside(j1, j2), "cmap: a receiver maps outside the scaled grid");
    const cf w = l_img[(size_t)j2 * n1 + j1];
    const int iz = std::max(0, lg.c2(w)), ix = lg.c1(w);
    require(lg.inside(ix, iz), "cmap: a receiver maps outside the log grid");
    sm.rec_x.push_back(ix);
    sm.rec_z.push_back(iz);
  }
}

void rotation_map(const Geometry& g, const Grid& model, float rad, ShotMap& sm) {
  const int n1 = model.n1, n2 = model.n2;
  const cf I(0, 1);
  const cf rot = std::exp(-I * rad), irot = std::exp(I * rad);
  // bounding box of the rotated corners and the origin (Rotation.h:32-46)
  const cf v[4] = {cf(model.o2, model.o1), cf(model.o2, model.o1 + (n1 - 1) * model.d1),
                   cf(model.o2 + (n2 - 1) * model.d2, model.o1),
                   cf(model.o2 + (n2 - 1) * model.d2, model.o1 + (n1 - 1) * model.d1)};
  float lo1 = 0, lo2 = 0, hi1 = 0, hi2 = 0;
  for (const cf& c : v) {
    const cf u = c * rot;
    lo1 = std::min(lo1, u.imag());
    lo2 = std::min(lo2, u.real());
    hi1 = std::max(hi1, u.imag());
    hi2 = std::max(hi2, u.real());
  }
  const Grid rg{n1, n2, lo1, (hi1 - lo1) / (n1 - 1), lo2, (hi2 - lo2) / (n2 - 1)};
  // preimages, moved back onto the model's edges when they leave it
  // (Rotation.h:55-86; the conditions use the indices before any move)
  const float m1 = (n1 - 1) * model.d1 + model.o1, m2 = (n2 - 1) * model.d2 + model.o2;
  const float t = std::tan(rad);
  std::vector<cf> pre(rg.size()), img(model.size());
  for (size_t k = 0; k < rg.size(); ++k) {
    cf z = rg.at(k) * irot;
    const int i1 = model.c1(z), i2 = model.c2(z);
    float x;
    if (i1 < 0) {
      x = -(z.imag() - model.o1) / t;
      x = std::min(z.real() + x, m2);
      z = cf(x, model.o1);
    }
    if (i2 < 0) {
      x = -(z.real() - model.o2) * t;
      x = std::min(z.imag() + x, m1);
      z = cf(model.o2, x);
    }
    if (i1 >= n1) {
      x = (z.imag() - m1) / t;
      x = std::max(z.real() - x, model.o1);
      z = cf(x, m1);
    }
    if (i2 >= n2) {
      x = (z.real() - m2) * t;
      x = std::min(z.imag() - x, model.o1);
      z = cf(m2, x);
    }
    pre[k] = z;
  }
  for (size_t k = 0; k < model.size(); ++k) img[k] = model.at(k) * rot;
  sm.o1 = rg.o1;
  sm.d1 = rg.d1;
  sm.o2 = rg.o2;
  sm.d2 = rg.d2;
  sm.fwd = nearest(model, pre);
  sm.inv = nearest(rg, img);
  // devices: the cells of their images (ConformalMap.h:32-65)
  auto place = [&](int x, int z, int& ix, int& iz) {
    require(x < n1 && z < n2, "cmap: a device lies outside the model");
    const cf u = img[(size_t)z * n1 + x];
    ix = rg.c1(u);
    iz = rg.c2(u);
    require(rg.inside(ix, iz), "cmap: a device maps outside the rotated grid");
  };
  int ix, iz;
  place(g.sx[0], g.sz[0], ix, iz);
  sm.src_z = iz;
  sm.src_x = {ix};
  for (int r = 0; r < g.nr; ++r) {
    place(g.rx[r], g.rz[r], ix, iz);
    sm.rec_x.push_back(ix);
    sm.rec_z.push_back(iz);
  }
}

}  // namespace

std::vector<ShotMap> make_shot_maps(const wem_params& p, const Geometry& g) {
  require(p.cmap == WEM_CMAP_LOG || p.cmap == WEM_CMAP_ROT, "cmap must be 0, 1 or 2");
  require(p.nx >= 2 && p.nz >= 2, "cmap needs at least 2 samples on each model axis");
  const Grid model{p.nx, p.nz, p.ox, p.dx, p.oz, p.dz};
  std::vector<ShotMap> maps(g.ns);
  for (int is = 0; is < g.ns; ++is) {
    if (p.cmap == WEM_CMAP_LOG) {
      require(p.eps_log > 0 && p.eps_log < 1, "eps_log must be in (0, 1)");
      shift_log_map(p, g, model, is, maps[is]);
    } else {
      require(p.cmap_angles != nullptr, "cmap 2 needs one angle per shot (cmap_angles)");
      Geometry one = g;
      one.sx = {g.sx[is]};
      one.sz = {g.sz[is]};
      rotation_map(one, model, p.cmap_angles[is], maps[is]);
    }
    const ShotMap& m = maps[is];
    require(std::isfinite(m.d1) && std::isfinite(m.d2) && m.d1 > 0 && m.d2 > 0,
            "cmap: the mapped grid of shot " + std::to_string(is) + " is degenerate");
  }
  return maps;
}

}  // namespace wg
