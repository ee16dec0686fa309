// Test infrastructure only: C entry points over the reference's own operator
// classes (propagator/src WEM, BornFull, BornRefl, BornTomo, extWEM,
// extBornFull), compiled unchanged against oracle/ref/stubs.  Each call
// builds the operator the way the reference's Python wrappers do
// (propagator/src/python/WEM.py:36-130, pyWEM.cpp), runs one forward or
// adjoint and copies the result out.  Parameters arrive as "key=value;..."
// with the reference's own parameter names (ns, osx, dsx, nr, orx, drx,
// prop, nref, tap, pad, tpad, eps, fmin, fmax, nfreq, ntaylor, ...).
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "BornFull.h"
#include "Injection.h"
#include "LanczosInterpolation2D.h"
#include "Spline2D.h"
#include "BornRefl.h"
#include "BornTomo.h"
#include "WEM.h"
#include "extBornFull.h"
#include "extWEM.h"

using namespace SEP;

namespace {

thread_local std::string g_err;

std::shared_ptr<paramObj> params(const char* kv) {
  std::map<std::string, std::string> m;
  std::stringstream ss(kv ? kv : "");
  std::string item;
  while (std::getline(ss, item, ';')) {
    const auto e = item.find('=');
    if (e == std::string::npos || e == 0) continue;
    m[item.substr(0, e)] = item.substr(e + 1);
  }
  return std::make_shared<paramObj>(m);
}

struct Grid {
  int nx, nz;
  float ox, oz, dx, dz;
  std::shared_ptr<hypercube> hyp() const {
    return std::make_shared<hypercube>(axis(nx, ox, dx), axis(nz, oz, dz));
  }
};

struct Time {
  int nt;
  float ot, dt;
};

std::shared_ptr<float1DReg> wavelet(const Time& t, const float* w) {
  auto v = std::make_shared<float1DReg>(std::make_shared<hypercube>(axis(t.nt, t.ot, t.dt)));
  std::memcpy(v->getVals(), w, sizeof(float) * t.nt);
  return v;
}

std::shared_ptr<complex2DReg> plane(const Grid& g, const float* c) {
  auto v = std::make_shared<complex2DReg>(g.hyp());
  if (c) std::memcpy(v->getVals(), c, sizeof(std::complex<float>) * (size_t)g.nx * g.nz);
  else v->scale(0.f);
  return v;
}

std::shared_ptr<complex3DReg> cube(const Grid& g, int n3, const float* c) {
  auto v = std::make_shared<complex3DReg>(std::make_shared<hypercube>(axis(g.nx, g.ox, g.dx), axis(g.nz, g.oz, g.dz),
                                                                      axis(n3, 0.f, 1.f)));
  if (c) std::memcpy(v->getVals(), c, sizeof(std::complex<float>) * (size_t)g.nx * g.nz * n3);
  else v->scale(0.f);
  return v;
}

std::shared_ptr<float3DReg> traces(const Time& t, int nr, int ns, const float* d) {
  auto v = std::make_shared<float3DReg>(
      std::make_shared<hypercube>(axis(t.nt, t.ot, t.dt), axis(nr, 0.f, 1.f), axis(ns, 0.f, 1.f)));
  if (d) std::memcpy(v->getVals(), d, sizeof(float) * (size_t)t.nt * nr * ns);
  else v->scale(0.);
  return v;
}

template <class F>
int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
  } catch (...) {
    g_err = "unknown exception";
  }
  return 1;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// number of frequencies the reference propagates (PropParam.h:45-85)
int ref_nfreq(const char* kv, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox, float oz,
              float dx, float dz, int* nfreq) {
  return guarded([&] {
    WEM op(wavelet({nt, ot, dt}, wave), Grid{nx, nz, ox, oz, dx, dz}.hyp(), params(kv));
    *nfreq = op.get_nfreq();
  });
}

// WEM.forward: slowness and density planes [nz][nx] -> data [ns][nr][nt]
int ref_wem_forward(const char* kv, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                    float oz, float dx, float dz, const float* slow, const float* den, int ns, int nr, float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    WEM op(wavelet({nt, ot, dt}, wave), g.hyp(), params(kv));
    std::vector<std::shared_ptr<complex2DReg>> m{plane(g, slow), plane(g, den)};
    auto d = traces({nt, ot, dt}, nr, ns, nullptr);
    op.forward(m, d, false);
    std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
  });
}

// Born.forward at background (slow, den): perturbations -> data
int ref_born_forward(const char* kv, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                     float oz, float dx, float dz, const float* slow, const float* den, const float* dslow,
                     const float* dden, int ns, int nr, float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    std::vector<std::shared_ptr<complex2DReg>> bg{plane(g, slow), plane(g, den)};
    BornFull op(wavelet({nt, ot, dt}, wave), bg, params(kv));
    std::vector<std::shared_ptr<complex2DReg>> m{plane(g, dslow), plane(g, dden)};
    auto d = traces({nt, ot, dt}, nr, ns, nullptr);
    op.forward(m, d, false);
    std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
  });
}

// Born.adjoint at background (slow, den): data -> gradients of slowness, density
int ref_born_adjoint(const char* kv, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                     float oz, float dx, float dz, const float* slow, const float* den, const float* data, int ns,
                     int nr, float* gslow, float* gden) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    std::vector<std::shared_ptr<complex2DReg>> bg{plane(g, slow), plane(g, den)};
    BornFull op(wavelet({nt, ot, dt}, wave), bg, params(kv));
    std::vector<std::shared_ptr<complex2DReg>> m{plane(g, nullptr), plane(g, nullptr)};
    auto d = traces({nt, ot, dt}, nr, ns, data);
    op.adjoint(m, d, false);
    const size_t n = sizeof(std::complex<float>) * (size_t)nx * nz;
    std::memcpy(gslow, m[0]->getVals(), n);
    std::memcpy(gden, m[1]->getVals(), n);
  });
}

// BornRefl (frequency-extended reflectivity [nf][nz][nx]) at background slowness
int ref_bornrefl(const char* kv, int adj, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                 float oz, float dx, float dz, const float* slow, int nf, float* refl, int ns, int nr, float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    BornRefl op(wavelet({nt, ot, dt}, wave), plane(g, slow), params(kv));
    auto r = cube(g, nf, adj ? nullptr : refl);
    auto d = traces({nt, ot, dt}, nr, ns, adj ? data : nullptr);
    if (adj) {
      op.adjoint(r, d, false);
      std::memcpy(refl, r->getVals(), sizeof(std::complex<float>) * (size_t)nx * nz * nf);
    } else {
      op.forward(r, d, false);
      std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
    }
  });
}

// BornTomo (slowness perturbation [nz][nx]) at background slowness and
// frequency-extended reflectivity [nf][nz][nx]
int ref_borntomo(const char* kv, int adj, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                 float oz, float dx, float dz, const float* slow, int nf, const float* bgrefl, float* dslow, int ns,
                 int nr, float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    BornTomo op(wavelet({nt, ot, dt}, wave), plane(g, slow), params(kv));
    op.setBgRefl(cube(g, nf, bgrefl));
    auto m = plane(g, adj ? nullptr : dslow);
    auto d = traces({nt, ot, dt}, nr, ns, adj ? data : nullptr);
    if (adj) {
      op.adjoint(m, d, false);
      std::memcpy(dslow, m->getVals(), sizeof(std::complex<float>) * (size_t)nx * nz);
    } else {
      op.forward(m, d, false);
      std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
    }
  });
}

// extWEM.forward: per-frequency slowness and density cubes [nf][nz][nx]
int ref_extwem_forward(const char* kv, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                       float oz, float dx, float dz, int nf, const float* slow, const float* den, int ns, int nr,
                       float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    auto s = cube(g, nf, slow);
    extWEM op(wavelet({nt, ot, dt}, wave), s->getHyper(), params(kv));
    std::vector<std::shared_ptr<complex3DReg>> m{s, cube(g, nf, den)};
    auto d = traces({nt, ot, dt}, nr, ns, nullptr);
    op.forward(m, d, false);
    std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
  });
}

// extBornFull forward / adjoint at per-frequency backgrounds
int ref_extborn(const char* kv, int adj, int nt, float ot, float dt, const float* wave, int nx, int nz, float ox,
                float oz, float dx, float dz, int nf, const float* slow, const float* den, float* dslow, float* dden,
                int ns, int nr, float* data) {
  return guarded([&] {
    const Grid g{nx, nz, ox, oz, dx, dz};
    std::vector<std::shared_ptr<complex3DReg>> bg{cube(g, nf, slow), cube(g, nf, den)};
    extBornFull op(wavelet({nt, ot, dt}, wave), bg, params(kv));
    std::vector<std::shared_ptr<complex3DReg>> m{cube(g, nf, adj ? nullptr : dslow),
                                                 cube(g, nf, adj ? nullptr : dden)};
    auto d = traces({nt, ot, dt}, nr, ns, adj ? data : nullptr);
    if (adj) {
      op.adjoint(m, d, false);
      const size_t n = sizeof(std::complex<float>) * (size_t)nx * nz * nf;
      std::memcpy(dslow, m[0]->getVals(), n);
      std::memcpy(dden, m[1]->getVals(), n);
    } else {
      op.forward(m, d, false);
      std::memcpy(data, d->getVals(), sizeof(float) * (size_t)nt * nr * ns);
    }
  });
}

// LanczosInterpolation2D (kind 0; p0, p1 the half widths in coarse cells)
// or Spline2D (kind 1; p0, p1 = a, b) from the coarse model grid
// (mn1 x mn2, spacings md1, md2) to the fine one (dn1 x dn2): forward reads
// model and writes data, adjoint the reverse (operator/src/
// LanczosInterpolation2D.h:14-90, Spline2D.h:14-90)
int ref_interp2d(int kind, int adj, int mn1, float md1, int mn2, float md2, int dn1, float dd1, int dn2, float dd2,
                 float p0, float p1, float* model, float* data) {
  return guarded([&] {
    auto m = std::make_shared<complex2DReg>(std::make_shared<hypercube>(axis(mn1, 0.f, md1), axis(mn2, 0.f, md2)));
    auto d = std::make_shared<complex2DReg>(std::make_shared<hypercube>(axis(dn1, 0.f, dd1), axis(dn2, 0.f, dd2)));
    const size_t nm = sizeof(std::complex<float>) * (size_t)mn1 * mn2, nd = sizeof(std::complex<float>) * (size_t)dn1 * dn2;
    std::unique_ptr<Operator<complex2DReg, complex2DReg>> op;
    if (kind == 0) op.reset(new LanczosInterpolation2D(m, d, std::vector<float>{p0, p1}));
    else op.reset(new Spline2D(m, d, p0, p1));
    if (adj) {
      std::memcpy(d->getVals(), data, nd);
      op->adjoint(m, d, false);
      std::memcpy(model, m->getVals(), nm);
    } else {
      std::memcpy(m->getVals(), model, nm);
      op->forward(m, d, false);
      std::memcpy(data, d->getVals(), nd);
    }
  });
}

// Injection (propagator/src/Injection.h:19-65, Injection.cpp:8-33, 52-75)
// between a model [nt] (nshot = 0) or [nshot][npt][nt] and rows [nz][nx]:
// forward reads model and writes data, adjoint the reverse (neither adds)
int ref_inject(const int* iz, const int* ix, int npt, int ng, int tap, int nx, int nz, int nt, int nshot, int step,
               int shot, int adj, float* model, float* data) {
  return guarded([&] {
    Injection op(std::vector<int>(iz, iz + npt), std::vector<int>(ix, ix + npt), ng, tap);
    op.setStep(step);
    op.setShot(shot);
    auto d = std::make_shared<complex2DReg>(std::make_shared<hypercube>(axis(nx, 0.f, 1.f), axis(nz, 0.f, 1.f)));
    const size_t nd = sizeof(std::complex<float>) * (size_t)nx * nz;
    auto run = [&](auto m, size_t nm) {
      if (adj) {
        std::memcpy(d->getVals(), data, nd);
        op.adjoint(m, d, false);
        std::memcpy(model, m->getVals(), nm);
      } else {
        std::memcpy(m->getVals(), model, nm);
        op.forward(m, d, false);
        std::memcpy(data, d->getVals(), nd);
      }
    };
    if (nshot == 0) {
      run(std::make_shared<complex1DReg>(std::make_shared<hypercube>(axis(nt, 0.f, 1.f))),
          sizeof(std::complex<float>) * (size_t)nt);
    } else {
      run(std::make_shared<complex3DReg>(
              std::make_shared<hypercube>(axis(nt, 0.f, 1.f), axis(npt, 0.f, 1.f), axis(nshot, 0.f, 1.f))),
          sizeof(std::complex<float>) * (size_t)nshot * npt * nt);
    }
  });
}

}  // extern "C"
