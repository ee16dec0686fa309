// Stand-in for TBB (test infrastructure only): serial.
#pragma once
#include "blocked_range.h"
namespace tbb {
template <class Range, class Value, class Body, class Reduction>
Value parallel_reduce(const Range& r, const Value& identity, const Body& body, const Reduction&) {
  return body(r, identity);
}
}  // namespace tbb
