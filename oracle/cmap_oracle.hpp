// ORACLE — test infrastructure only.  CPU restatement of the reference's
// conformal maps (conformal/src: ConformalMap.h/.cpp, ShiftAndScale.h,
// ComplexLog.h/.cpp, Rotation.h, MapChain.h) and of their use per shot
// (propagator/src/PropParam.h:88-137, wem_prop.cpp:19-45,
// born_prop.cpp:28-70, 138-232).  Only the oracle drivers include it.
//
// PARITY PINNED: WEM and Born through both maps (and with explicit device
// coordinates) are held to the reference's own sources, compiled unchanged
// by oracle/ref/Makefile (fixtures tests/golden/ref_cmap_*.npz,
// tests/test_ref_pin.py).  The maps follow
// the reference class by class: each holds its coordinate tables zmap (the
// preimage of every output sample), umap (the image of every input sample)
// and its Jacobian, in float complex arithmetic, and a chain applies its two
// maps in turn.  One deliberate difference: samples the reference leaves
// untouched in its per-task buffers (a preimage or image outside the grid)
// are zero here, as for the first shot of a task.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <memory>
#include <vector>

namespace wo {
namespace cm {

using cf = std::complex<float>;

// 2D axes: 1 = x (fast), 2 = z
struct Hyper {
  int n1 = 0, n2 = 0;
  float o1 = 0, d1 = 1, o2 = 0, d2 = 1;
  size_t n() const { return (size_t)n1 * n2; }
};

// coordinates z + i x of every sample (ConformalMap.h:96-108)
std::vector<cf> regular_coord(const Hyper& h);


// Base map (ConformalMap.h:14-123): g maps the input grid Z onto the output
// grid U.  zmap[i] = preimage of output sample i, umap[i] = image of input
// sample i.
struct Map {
  Hyper in, out;
  std::vector<cf> zmap, umap, zcoord, ucoord;
  std::vector<float> jacob;
  bool is_log = false;
  float leps = 0;
  virtual ~Map() = default;

  void complexify();

  // field on `in` -> field on `out` (ConformalMap.cpp:59-79); `o` must hold
  // zeros where nothing is written
  template <class T>
  void forward(const std::vector<T>& f, std::vector<T>& o) const {
    if (is_log) return log_forward(f, o);
    for (int i2 = 0; i2 < in.n2; ++i2)
      for (int i1 = 0; i1 < in.n1; ++i1) {
        const cf z = zmap[(size_t)i1 + (size_t)i2 * in.n1];
        const int iz = (int)((z.real() - in.o2) / in.d2);
        const int ix = (int)((z.imag() - in.o1) / in.d1);
        if (iz >= 0 && iz < in.n2 && ix >= 0 && ix < in.n1)
          o[(size_t)i2 * in.n1 + i1] = f[(size_t)iz * in.n1 + ix];
      }
  }

  // field on `out` -> field on `in` (ConformalMap.cpp:81-101)
  template <class T>
  void inverse(std::vector<T>& f, const std::vector<T>& o) const {
    if (is_log) return log_inverse(f, o);
    for (int i2 = 0; i2 < out.n2; ++i2)
      for (int i1 = 0; i1 < out.n1; ++i1) {
        const cf u = umap[(size_t)i1 + (size_t)i2 * out.n1];
        const int iz = (int)((u.real() - out.o2) / out.d2);
        const int ix = (int)((u.imag() - out.o1) / out.d1);
        if (iz >= 0 && iz < out.n2 && ix >= 0 && ix < out.n1)
          f[(size_t)i2 * out.n1 + i1] = o[(size_t)iz * out.n1 + ix];
      }
  }

  // devices (ConformalMap.h:32-65; ComplexLog.cpp:162-227 for the log)
  void points(const std::vector<int>& re, const std::vector<int>& im, std::vector<int>& oz,
              std::vector<int>& ox) const {
    oz.clear();
    ox.clear();
    if (is_log && re.size() == 1) {
      // one point becomes the whole first depth
      for (int i = 0; i < out.n1; ++i) {
        oz.push_back(0);
        ox.push_back(i);
      }
      return;
    }
    for (size_t i = 0; i < re.size(); ++i) {
      const cf c = umap[(size_t)im[i] + (size_t)re[i] * in.n1];
      int iz = (int)((c.real() - out.o2) / out.d2);
      if (is_log) iz = std::max(0, iz);
      const int ix = (int)((c.imag() - out.o1) / out.d1);
      oz.push_back(iz);
      ox.push_back(ix);
    }
  }

  template <class T>
  void scale_by_jacobian(T* v) const {
    for (size_t i = 0; i < jacob.size(); ++i) v[i] *= jacob[i];
  }

 private:
  // ComplexLog.cpp:103-137: nearest neighbour; a sample whose preimage
  // misses the grid repeats the last hit of its column
  template <class T>
  void log_forward(const std::vector<T>& f, std::vector<T>& o) const {
    std::vector<T> buffer(out.n1, T(0));
    for (int i2 = 0; i2 < in.n2; ++i2)
      for (int i1 = 0; i1 < in.n1; ++i1) {
        const cf z = zmap[(size_t)i1 + (size_t)i2 * in.n1];
        const int iz = (int)((z.real() - in.o2) / in.d2);
        const int ix = (int)((z.imag() - in.o1) / in.d1);
        if (iz >= 0 && iz < in.n2 && ix >= 0 && ix < in.n1) buffer[i1] = f[(size_t)iz * in.n1 + ix];
        o[(size_t)i2 * in.n1 + i1] = buffer[i1];
      }
  }
  // ComplexLog.cpp:139-160: only the annulus eps < |z| < 0.99 comes back
  template <class T>
  void log_inverse(std::vector<T>& f, const std::vector<T>& o) const {
    for (int i2 = 0; i2 < out.n2; ++i2)
      for (int i1 = 0; i1 < out.n1; ++i1) {
        const size_t i = (size_t)i1 + (size_t)i2 * out.n1;
        const float amp = std::abs(zcoord[i]);
        if (amp > std::exp(leps) && amp < .99f) {
          const int iz = (int)((umap[i].real() - out.o2) / out.d2);
          const int ix = (int)((umap[i].imag() - out.o1) / out.d1);
          if (iz >= 0 && iz < out.n2 && ix >= 0 && ix < out.n1) f[i] = o[(size_t)iz * out.n1 + ix];
        }
      }
  }
};

// The maps' construction lives in cmap_oracle.cpp, compiled without fused
// multiply-adds so that its float coordinates, and the grid cells they
// truncate to, are the same on every machine.
// ShiftAndScale.h:12-58: f(z) = a (z - b)
std::unique_ptr<Map> shift_and_scale(const Hyper& h, cf a, cf b);
// ComplexLog.h:12-71: w = log z on the annulus eps <= |z| <= 1
std::unique_ptr<Map> complex_log(const Hyper& h, float eps);
// Rotation.h:12-100: rotation by exp(-i rad) into the bounding box of the
// rotated corners and the origin
std::unique_ptr<Map> rotation(const Hyper& h, float rad);

// the map of one shot: one map or a chain of two (MapChain.h:12-63)
struct ShotChain {
  std::vector<std::unique_ptr<Map>> maps;
  const Hyper& out() const { return maps.back()->out; }

  template <class T>
  std::vector<T> forward(const std::vector<T>& f) const {
    std::vector<T> cur = f;
    for (const auto& m : maps) {
      std::vector<T> o(m->out.n(), T(0));
      m->forward(cur, o);
      cur.swap(o);
    }
    return cur;
  }
  template <class T>
  std::vector<T> inverse(const std::vector<T>& o) const {
    std::vector<T> cur = o;
    for (size_t k = maps.size(); k-- > 0;) {
      std::vector<T> f(maps[k]->in.n(), T(0));
      maps[k]->inverse(f, cur);
      cur.swap(f);
    }
    return cur;
  }
  void points(std::vector<int> re, std::vector<int> im, std::vector<int>& oz, std::vector<int>& ox) const {
    for (const auto& m : maps) {
      m->points(re, im, oz, ox);
      re = oz;
      im = ox;
    }
  }
  template <class T>
  void scale_by_jacobian(T* v) const {
    for (const auto& m : maps) m->scale_by_jacobian(v);
  }
};

// PropParam.h:88-137 for shot is: the source at grid (sz, sx) of the model
ShotChain shot_chain(int cmap, const Hyper& model, int sz, int sx, float eps_log, float angle);

}  // namespace cm
}  // namespace wo
