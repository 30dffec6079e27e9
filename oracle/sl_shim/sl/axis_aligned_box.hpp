// Minimal stand-in for SpaceLand's <sl/axis_aligned_box.hpp> (test
// infrastructure for the oracle build only; see cstdint.hpp).
//
// center() is (min + max) * 0.5 per axis and half_side_lengths() is
// (max - min) * 0.5.  For the unit-cube-pinned scenes used by the tests both
// are exact, so they agree with any SpaceLand formula.
#pragma once

#include <sl/fixed_size_point.hpp>

namespace sl {

template <std::size_t N, class T>
class axis_aligned_box {
 public:
  typedef fixed_size_point<N, T> point_t;
  typedef fixed_size_vector<N, T> vector_t;
  point_t b_[2];

  axis_aligned_box() { to_empty(); }
  axis_aligned_box(const point_t& lo, const point_t& hi) { b_[0] = lo; b_[1] = hi; }

  point_t& operator[](std::size_t i) { return b_[i]; }
  const point_t& operator[](std::size_t i) const { return b_[i]; }

  void to_empty() {
    for (std::size_t i = 0; i < N; ++i) {
      b_[0][i] = std::numeric_limits<T>::max();
      b_[1][i] = -std::numeric_limits<T>::max();
    }
  }
  bool is_empty() const { for (std::size_t i = 0; i < N; ++i) if (b_[0][i] > b_[1][i]) return true; return false; }
  void merge(const point_t& p) {
    for (std::size_t i = 0; i < N; ++i) {
      if (p[i] < b_[0][i]) b_[0][i] = p[i];
      if (p[i] > b_[1][i]) b_[1][i] = p[i];
    }
  }
  point_t center() const { point_t c; for (std::size_t i = 0; i < N; ++i) c[i] = (b_[0][i] + b_[1][i]) * T(0.5); return c; }
  vector_t half_side_lengths() const { vector_t v; for (std::size_t i = 0; i < N; ++i) v[i] = (b_[1][i] - b_[0][i]) * T(0.5); return v; }
  vector_t diagonal() const { return b_[1] - b_[0]; }
  bool contains(const point_t& p) const {
    for (std::size_t i = 0; i < N; ++i) if (p[i] < b_[0][i] || p[i] > b_[1][i]) return false;
    return true;
  }
};

template <std::size_t N, class T>
inline std::ostream& operator<<(std::ostream& os, const axis_aligned_box<N, T>& b) {
  return os << "{" << b[0] << " " << b[1] << "}";
}

typedef axis_aligned_box<3, float> aabox3f;
typedef axis_aligned_box<3, double> aabox3d;

}  // namespace sl
