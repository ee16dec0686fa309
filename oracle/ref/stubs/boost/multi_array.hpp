// Stand-in for boost::multi_array (test infrastructure only): row-major
// (C order) storage, extents via boost::extents[n0][n1]..., element access by
// chained operator[], data(), shape(), size(), num_elements(), resize().
#pragma once
#include <array>
#include <cstddef>
#include <vector>

namespace boost {

template <std::size_t N>
struct extent_gen {
  std::array<std::size_t, N> n{};
  extent_gen<N + 1> operator[](std::ptrdiff_t e) const {
    extent_gen<N + 1> g;
    for (std::size_t i = 0; i < N; ++i) g.n[i] = n[i];
    g.n[N] = (std::size_t)e;
    return g;
  }
};
static const extent_gen<0> extents{};

namespace detail {
template <class T, std::size_t N>
struct view {
  T* p;
  const std::size_t* shape;
  const std::size_t* stride;
  const std::ptrdiff_t* base;
  view<T, N - 1> operator[](std::ptrdiff_t i) const {
    return view<T, N - 1>{p + (i - base[0]) * (std::ptrdiff_t)stride[0], shape + 1, stride + 1, base + 1};
  }
  std::size_t size() const { return shape[0]; }
};
template <class T>
struct view<T, 1> {
  T* p;
  const std::size_t* shape;
  const std::size_t* stride;
  const std::ptrdiff_t* base;
  T& operator[](std::ptrdiff_t i) const { return p[i - base[0]]; }
  std::size_t size() const { return shape[0]; }
};
}  // namespace detail

namespace multi_array_types {
struct index_range {};
}

template <class T, std::size_t N>
class multi_array {
 public:
  typedef T element;
  template <std::size_t K>
  struct array_view {
    typedef detail::view<T, K> type;
  };
  multi_array() {
    _shape.fill(0);
    _stride.fill(0);
    _base.fill(0);
  }
  multi_array(const extent_gen<N>& e) { resize(e); }
  multi_array(const multi_array& o) = default;
  multi_array& operator=(const multi_array& o) = default;
  multi_array& resize(const extent_gen<N>& e) {
    _shape = e.n;
    _base.fill(0);
    std::size_t s = 1;
    for (std::size_t i = N; i-- > 0;) {
      _stride[i] = s;
      s *= _shape[i];
    }
    _v.assign(s, T());
    return *this;
  }
  // index bases (boost's reindex): element i of a dimension is at i - base
  void reindex(std::ptrdiff_t b) { _base.fill(b); }
  const std::ptrdiff_t* index_bases() const { return _base.data(); }
  T* data() { return _v.data(); }
  const T* data() const { return _v.data(); }
  T* origin() { return _v.data(); }
  const std::size_t* shape() const { return _shape.data(); }
  std::size_t size() const { return _shape[0]; }
  std::size_t num_elements() const { return _v.size(); }
  decltype(auto) operator[](std::ptrdiff_t i) {
    if constexpr (N == 1) return (_v[i - _base[0]]);
    else
      return detail::view<T, N - 1>{_v.data() + (i - _base[0]) * (std::ptrdiff_t)_stride[0], _shape.data() + 1,
                                    _stride.data() + 1, _base.data() + 1};
  }
  decltype(auto) operator[](std::ptrdiff_t i) const {
    if constexpr (N == 1) return (_v[i - _base[0]]);
    else
      return detail::view<const T, N - 1>{_v.data() + (i - _base[0]) * (std::ptrdiff_t)_stride[0], _shape.data() + 1,
                                          _stride.data() + 1, _base.data() + 1};
  }

 private:
  std::vector<T> _v;
  std::array<std::size_t, N> _shape{};
  std::array<std::size_t, N> _stride{};
  std::array<std::ptrdiff_t, N> _base{};
};

}  // namespace boost
