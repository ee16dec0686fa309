// Stand-in for TBB (test infrastructure only): every loop runs serially,
// in order, on the calling thread.
#pragma once
#include <cstddef>
namespace tbb {
template <class V>
class blocked_range {
 public:
  typedef V const_iterator;
  blocked_range() : _b(), _e() {}
  blocked_range(V b, V e, std::size_t = 1) : _b(b), _e(e) {}
  V begin() const { return _b; }
  V end() const { return _e; }
  std::size_t size() const { return (std::size_t)(_e - _b); }
  bool empty() const { return !(_b < _e); }

 private:
  V _b, _e;
};
}  // namespace tbb
