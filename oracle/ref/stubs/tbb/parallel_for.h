// Stand-in for TBB (test infrastructure only): serial, in order.
#pragma once
#include "blocked_range.h"
namespace tbb {
struct static_partitioner {};
struct auto_partitioner {};
struct simple_partitioner {};
template <class Range, class Body>
void parallel_for(const Range& r, const Body& body) {
  body(r);
}
template <class Range, class Body, class P>
void parallel_for(const Range& r, const Body& body, const P&) {
  body(r);
}
template <class Index, class Func>
void parallel_for(Index first, Index last, const Func& f) {
  for (Index i = first; i < last; ++i) f(i);
}
template <class Index, class Func>
void parallel_for(Index first, Index last, Index step, const Func& f) {
  for (Index i = first; i < last; i += step) f(i);
}
}  // namespace tbb
