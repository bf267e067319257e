// Compatibility shim (test infrastructure, not product code).
//
// The reference simulator includes headers from two git submodules
// (altlib, altmath) that are not vendored with it.  This directory provides
// the small surface the simulator's call sites use, written from those call
// sites only, so that the unmodified simulator sources compile for the
// oracle.  Semantics chosen here are fixed by the call sites:
//   aml::clamp(v, lo, hi) = min(max(v, lo), hi)
//   aml::min / aml::max   = the usual two-argument forms (ties return `a`)
//   aml::sgn(x)           = -1, 0 or +1
// None of this arithmetic is pinned by tests of the reference (it has none),
// so parity at this boundary is unpinned.
#pragma once
#include <cmath>
#include <cstdlib>
#include <stdlib.h>
#include <cstring>
#include <cstdint>
#include <cassert>
#include <cstdio>

namespace aml {

template <typename T> inline T max(T a, T b) { return (a < b) ? b : a; }
template <typename T> inline T min(T a, T b) { return (b < a) ? b : a; }
template <typename T> inline T clamp(T v, T lo, T hi) { return min<T>(max<T>(v, lo), hi); }
template <typename T> inline T sgn(T x) { return (T)((T(0) < x) - (x < T(0))); }

}  // namespace aml
