// Stand-in for boost::progress_display (test infrastructure only): silent.
#pragma once
#include <iostream>
namespace boost {
class progress_display {
 public:
  progress_display(unsigned long, std::ostream& = std::cout) {}
  unsigned long operator++() { return ++_n; }
  unsigned long operator+=(unsigned long k) { return _n += k; }

 private:
  unsigned long _n = 0;
};
}  // namespace boost
