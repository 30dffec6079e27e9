// Minimal stand-in for SpaceLand's <sl/fixed_size_point.hpp> (test
// infrastructure for the oracle build only; see cstdint.hpp).
#pragma once

#include <sl/fixed_size_vector.hpp>

namespace sl {

template <std::size_t N, class T>
class fixed_size_point {
 public:
  typedef T value_t;
  typedef fixed_size_vector<N, T> vector_t;
  T v_[N];

  fixed_size_point() { for (std::size_t i = 0; i < N; ++i) v_[i] = T(0); }
  template <class A, class B, class C>
  fixed_size_point(A a, B b, C c) { v_[0] = T(a); v_[1] = T(b); v_[2] = T(c); }

  T& operator[](std::size_t i) { return v_[i]; }
  const T& operator[](std::size_t i) const { return v_[i]; }
  T* to_pointer() { return v_; }
  const T* to_pointer() const { return v_; }

  vector_t as_vector() const { vector_t r; for (std::size_t i = 0; i < N; ++i) r[i] = v_[i]; return r; }
  fixed_size_point operator+(const vector_t& o) const { fixed_size_point r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] + o[i]; return r; }
  fixed_size_point operator-(const vector_t& o) const { fixed_size_point r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] - o[i]; return r; }
  vector_t operator-(const fixed_size_point& o) const { vector_t r; for (std::size_t i = 0; i < N; ++i) r[i] = v_[i] - o.v_[i]; return r; }
  fixed_size_point& operator+=(const vector_t& o) { for (std::size_t i = 0; i < N; ++i) v_[i] += o[i]; return *this; }
  bool operator==(const fixed_size_point& o) const { for (std::size_t i = 0; i < N; ++i) if (v_[i] != o.v_[i]) return false; return true; }

  T distance_to(const fixed_size_point& o) const { return ((*this) - o).two_norm(); }
};

template <std::size_t N, class T>
inline std::ostream& operator<<(std::ostream& os, const fixed_size_point<N, T>& p) {
  os << "(";
  for (std::size_t i = 0; i < N; ++i) os << (i ? " " : "") << p[i];
  return os << ")";
}

typedef fixed_size_point<3, float> point3f;
typedef fixed_size_point<3, double> point3d;

}  // namespace sl
