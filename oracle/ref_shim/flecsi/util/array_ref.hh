// Stand-in declaration for compiling flecsolve's serial (seq_vec / mat::csr)
// Krylov path without FleCSI or Boost.  Only the names the reference
// headers mention are declared; nothing here executes FleCSI behaviour.
#pragma once
#include <cstddef>
#include <array>
#include <vector>
namespace flecsi::util {
using id = std::size_t; using gid = std::size_t;
template<class T> struct span {
  using element_type = T; using value_type = std::remove_cv_t<T>;
  T* p = nullptr; std::size_t n = 0;
  span() = default; span(T* p, std::size_t n) : p(p), n(n) {}
  template<class U> span(std::vector<U>& v) : p(v.data()), n(v.size()) {}
  T* data() const { return p; } std::size_t size() const { return n; }
  T& operator[](std::size_t i) const { return p[i]; }
  T* begin() const { return p; } T* end() const { return p + n; }
  T& front() const { return p[0]; } T& back() const { return p[n-1]; }
  bool operator==(const span& o) const { return p == o.p && n == o.n; }
  bool operator!=(const span& o) const { return !(*this == o); }
};
template<class T, std::size_t D> struct mdcolex {
  T* p; std::array<std::size_t, D> s;
  mdcolex(T* p, std::array<std::size_t, D> s) : p(p), s(s) {}
  T& operator()(std::size_t i, std::size_t j) const { return p[i + s[0]*j]; }
};
template<class T> struct iota_view {
  T b, e; iota_view(T b, T e):b(b),e(e){}
  struct iterator { T v; T operator*() const { return v; } iterator& operator++() { ++v; return *this; }
    bool operator!=(const iterator& o) const { return v != o.v; } };
  iterator begin() const { return {b}; } iterator end() const { return {e}; }
  std::size_t size() const { return e - b; } T front() const { return b; } T back() const { return e - 1; }
};
template<class R, class F> struct transform_view { transform_view(R, F) {} };
// 2-D view used by NKA's normal-equation matrix (solvers/nka.hh:468-484):
// h[i] is row i, h[i][j] an element; only read back through the same view
template<class T, std::size_t D> struct mdspan;
template<class T> struct mdspan<T, 2> {
  using size_type = std::size_t;
  mdspan(T* p, std::array<size_type, 2> e) : p(p), e(e) {}
  T* operator[](size_type i) const { return p + i * e[1]; }
  T* p; std::array<size_type, 2> e;
};
}
