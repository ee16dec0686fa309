// Stand-in for TBB (test infrastructure only).
#pragma once
#include "blocked_range.h"
namespace tbb {
template <class R, class C = R>
class blocked_range2d {
 public:
  blocked_range2d(R rb, R re, C cb, C ce) : _r(rb, re), _c(cb, ce) {}
  blocked_range2d(R rb, R re, std::size_t, C cb, C ce, std::size_t) : _r(rb, re), _c(cb, ce) {}
  const blocked_range<R>& rows() const { return _r; }
  const blocked_range<C>& cols() const { return _c; }

 private:
  blocked_range<R> _r;
  blocked_range<C> _c;
};
}  // namespace tbb
