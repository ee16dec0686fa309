// Stand-in for boost::irange (test infrastructure only).
#pragma once
namespace boost {
template <class I>
struct integer_range {
  struct iterator {
    I v;
    I operator*() const { return v; }
    iterator& operator++() { ++v; return *this; }
    bool operator!=(const iterator& o) const { return v != o.v; }
    bool operator==(const iterator& o) const { return v == o.v; }
  };
  I b, e;
  iterator begin() const { return {b}; }
  iterator end() const { return {e}; }
};
template <class I>
integer_range<I> irange(I b, I e) { return {b, e}; }
}  // namespace boost
