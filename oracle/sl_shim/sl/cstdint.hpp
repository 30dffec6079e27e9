// Minimal stand-in for the SpaceLand (SL 7.8.2) header <sl/cstdint.hpp>.
//
// Test infrastructure only: the oracle build compiles the reference's own
// symvox sources against these headers.  SpaceLand itself is not vendored
// with the reference (its .gitignore lists sl-7.8.2-*), so this shim supplies
// exactly the API surface the symvox sources use, written from that usage.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <algorithm>
#include <vector>
#include <map>
#include <set>
#include <string>
#include <iostream>
#include <sstream>
#include <fstream>
#include <tuple>
#include <functional>
#include <unordered_map>
#include <stdexcept>

namespace sl {
typedef std::uint8_t uint8_t;
typedef std::uint16_t uint16_t;
typedef std::uint32_t uint32_t;
typedef std::uint64_t uint64_t;
typedef std::int32_t int32_t;

template <class T> inline const T& min(const T& a, const T& b) { return (b < a) ? b : a; }
template <class T> inline const T& max(const T& a, const T& b) { return (a < b) ? b : a; }
using std::tie;
}  // namespace sl
