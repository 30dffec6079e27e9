// Minimal stand-in for SpaceLand's <sl/clock.hpp> plus the pathname and
// human-readable helpers the symvox sources call (test infrastructure for the
// oracle build only; see cstdint.hpp).
#pragma once

#include <sl/cstdint.hpp>
#include <chrono>

namespace sl {

class time_duration {
 public:
  std::int64_t ns_;
  time_duration() : ns_(0) {}
  explicit time_duration(std::int64_t ns) : ns_(ns) {}
  std::size_t as_microseconds() const { return std::size_t(ns_ / 1000); }
  std::size_t as_milliseconds() const { return std::size_t(ns_ / 1000000); }
  double as_seconds() const { return double(ns_) * 1e-9; }
  time_duration operator+(const time_duration& o) const { return time_duration(ns_ + o.ns_); }
  time_duration operator-(const time_duration& o) const { return time_duration(ns_ - o.ns_); }
  time_duration& operator+=(const time_duration& o) { ns_ += o.ns_; return *this; }
  time_duration operator*(double s) const { return time_duration(std::int64_t(double(ns_) * s)); }
};

class time_point {
 public:
  std::int64_t ns_;
  time_point() : ns_(0) {}
  explicit time_point(std::int64_t ns) : ns_(ns) {}
  time_duration operator-(const time_point& o) const { return time_duration(ns_ - o.ns_); }
};

class real_time_clock {
 public:
  time_point start_;
  real_time_clock() { restart(); }
  static time_point now() {
    return time_point(std::chrono::duration_cast<std::chrono::nanoseconds>(
                          std::chrono::steady_clock::now().time_since_epoch()).count());
  }
  void restart() { start_ = now(); }
  time_duration elapsed() const { return now() - start_; }
};

inline std::string human_readable_duration(const time_duration& d) {
  char b[64];
  double s = d.as_seconds();
  if (s < 1e-3) std::snprintf(b, sizeof(b), "%.1fus", s * 1e6);
  else if (s < 1.0) std::snprintf(b, sizeof(b), "%.2fms", s * 1e3);
  else std::snprintf(b, sizeof(b), "%.2fs", s);
  return b;
}
inline std::string human_readable_size(std::size_t n) {
  char b[64];
  if (n < 1024) std::snprintf(b, sizeof(b), "%zuB", n);
  else if (n < 1024 * 1024) std::snprintf(b, sizeof(b), "%.2fKB", n / 1024.0);
  else if (n < 1024ull * 1024 * 1024) std::snprintf(b, sizeof(b), "%.2fMB", n / (1024.0 * 1024.0));
  else std::snprintf(b, sizeof(b), "%.2fGB", n / (1024.0 * 1024.0 * 1024.0));
  return b;
}
inline std::string human_readable_quantity(std::size_t n) {
  char b[64];
  if (n < 1000) std::snprintf(b, sizeof(b), "%zu", n);
  else if (n < 1000000) std::snprintf(b, sizeof(b), "%.2fK", n / 1e3);
  else if (n < 1000000000) std::snprintf(b, sizeof(b), "%.2fM", n / 1e6);
  else std::snprintf(b, sizeof(b), "%.2fG", n / 1e9);
  return b;
}

inline std::string pathname_directory_separators() { return "/"; }
inline std::string pathname_directory(const std::string& p) {
  std::size_t k = p.find_last_of('/');
  return (k == std::string::npos) ? std::string(".") : p.substr(0, k);
}
inline std::string pathname_base(const std::string& p) {
  std::size_t k = p.find_last_of('/');
  return (k == std::string::npos) ? p : p.substr(k + 1);
}
inline std::string pathname_without_extension(const std::string& p) {
  std::size_t k = p.find_last_of('.');
  std::size_t s = p.find_last_of('/');
  if (k == std::string::npos || (s != std::string::npos && k < s)) return p;
  return p.substr(0, k);
}

}  // namespace sl
