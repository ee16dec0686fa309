// Conformal-map geometry of the one-way operators (cmap = 1, 2): per shot,
// the grid the shot propagates on and the gathers between it and the model
// grid (propagator/src/PropParam.h:88-137, conformal/src).
#pragma once
#include <vector>

#include "planner.h"

namespace wg {

struct ShotMap {
  // mapped grid: axis 1 (x) and axis 2 (z) samplings; n as the model's
  float o1 = 0, d1 = 1, o2 = 0, d2 = 1;
  // model -> mapped grid: mapped point i takes model point fwd[i] (-1: zero)
  std::vector<int> fwd;
  // mapped grid -> model grid (the image's way back): model point m takes
  // mapped point inv[m] (-1: zero)
  std::vector<int> inv;
  // Jacobian of the map, applied twice to the padded slowness^2 by flat
  // index k < nx nz: s *= js, s *= jl[k] (jl empty: 1), then again
  float js = 1;
  std::vector<float> jl;
  // devices on the mapped grid: the shot's source points (one depth) and
  // its receivers
  int src_z = 0;
  std::vector<int> src_x;
  std::vector<int> rec_x, rec_z;
};

// one map per shot of the geometry g (model grid and devices of p)
std::vector<ShotMap> make_shot_maps(const wem_params& p, const Geometry& g);

}  // namespace wg
