// Minimal stand-in for SpaceLand's <sl/fixed_size_vector.hpp> (test
// infrastructure for the oracle build only; see cstdint.hpp).
//
// Arithmetic order is fixed here because the reference's fp64 triangle/box
// test calls dot() and cross():
//   dot(a,b)   = (a0*b0 + a1*b1) + a2*b2            (left to right)
//   cross(a,b) = (a1*b2 - a2*b1, a2*b0 - a0*b2, a0*b1 - a1*b0)
// The CUDA kernel uses the same order.  SpaceLand's own order is not
// published with the reference, so this is the pinned assumption.
#pragma once

#include <sl/cstdint.hpp>
// The symvox sources reach the pathname / human-readable helpers through the
// geometry headers, so they are made visible from here too.
#include <sl/clock.hpp>

namespace sl {

template <std::size_t N, class T>
class fixed_size_vector {
 public:
  typedef T value_t;
  T v_[N];

  fixed_size_vector() { for (std::size_t i = 0; i < N; ++i) v_[i] = T(0); }
  template <class A, class B, class C>
  fixed_size_vector(A a, B b, C c) { v_[0] = T(a); v_[1] = T(b); v_[2] = T(c); }

  T& operator[](std::size_t i) { return v_[i]; }
  const T& operator[](std::size_t i) const { return v_[i]; }
  T* to_pointer() { return v_; }
  const T* to_pointer() const { return v_; }

  fixed_size_vector operator+(const fixed_size_vector& o) const { fixed_size_vector r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] + o.v_[i]; return r; }
  fixed_size_vector operator-(const fixed_size_vector& o) const { fixed_size_vector r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] - o.v_[i]; return r; }
  fixed_size_vector operator-() const { fixed_size_vector r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = -v_[i]; return r; }
  fixed_size_vector operator*(T s) const { fixed_size_vector r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] * s; return r; }
  fixed_size_vector operator/(T s) const { fixed_size_vector r; for (std::size_t i = 0; i < N; ++i) r.v_[i] = v_[i] / s; return r; }
  fixed_size_vector& operator+=(const fixed_size_vector& o) { for (std::size_t i = 0; i < N; ++i) v_[i] += o.v_[i]; return *this; }
  fixed_size_vector& operator-=(const fixed_size_vector& o) { for (std::size_t i = 0; i < N; ++i) v_[i] -= o.v_[i]; return *this; }

  T dot(const fixed_size_vector& o) const {
    T r = v_[0] * o.v_[0];
    for (std::size_t i = 1; i < N; ++i) r = r + v_[i] * o.v_[i];
    return r;
  }
  fixed_size_vector cross(const fixed_size_vector& o) const {
    return fixed_size_vector(v_[1] * o.v_[2] - v_[2] * o.v_[1],
                             v_[2] * o.v_[0] - v_[0] * o.v_[2],
                             v_[0] * o.v_[1] - v_[1] * o.v_[0]);
  }
  T two_norm() const { return std::sqrt(dot(*this)); }
  fixed_size_vector ok_normalized() const {
    T n = two_norm();
    return (n > T(0)) ? (*this) / n : *this;
  }
};

template <std::size_t N, class T>
inline fixed_size_vector<N, T> operator*(T s, const fixed_size_vector<N, T>& v) { return v * s; }

template <std::size_t N, class T>
inline std::ostream& operator<<(std::ostream& os, const fixed_size_vector<N, T>& v) {
  os << "[";
  for (std::size_t i = 0; i < N; ++i) os << (i ? " " : "") << v[i];
  return os << "]";
}

typedef fixed_size_vector<3, float> vector3f;
typedef fixed_size_vector<3, double> vector3d;
typedef fixed_size_vector<3, float> color3f;

}  // namespace sl
