// Stand-in for SEP hypercube's axis (test infrastructure only).
#pragma once
#include <string>
namespace SEP {
class axis {
 public:
  axis() : n(1), o(0.f), d(1.f) {}
  explicit axis(int n_) : n(n_), o(0.f), d(1.f) {}
  axis(int n_, float o_, float d_, const std::string& l = "", const std::string& u = "")
      : n(n_), o(o_), d(d_), label(l), unit(u) {}
  int n;
  float o, d;
  std::string label, unit;
};
}  // namespace SEP
