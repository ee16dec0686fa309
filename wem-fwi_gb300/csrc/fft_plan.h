// FFT plan: the radix sequence of one transform length (host and device).
#pragma once

namespace wg {

constexpr int kMaxStages = 24;

struct FftPlan {
  int n;
  int nstage;
  int radix[kMaxStages];
};

}  // namespace wg
