// Compatibility shim (test infrastructure): 2-component vectors used by the
// reference simulator (vec2d particles and velocities, vec2i grid indices).
// Operators evaluate component-wise in the obvious order; scalar * vector
// multiplies each component by the scalar.
#pragma once
#include <cmath>
#include "math_utils.h"

template <typename T>
struct vec2 {
    T x;
    T y;

    vec2& operator+=(const vec2& o) { x += o.x; y += o.y; return *this; }
    vec2& operator-=(const vec2& o) { x -= o.x; y -= o.y; return *this; }
    vec2& operator*=(T s) { x *= s; y *= s; return *this; }
    vec2& operator/=(T s) { x /= s; y /= s; return *this; }
};

template <typename T> inline vec2<T> operator+(vec2<T> a, vec2<T> b) { return vec2<T>{a.x + b.x, a.y + b.y}; }
template <typename T> inline vec2<T> operator-(vec2<T> a, vec2<T> b) { return vec2<T>{a.x - b.x, a.y - b.y}; }
template <typename T> inline vec2<T> operator-(vec2<T> a) { return vec2<T>{-a.x, -a.y}; }
template <typename T> inline vec2<T> operator*(vec2<T> a, T s) { return vec2<T>{a.x * s, a.y * s}; }
template <typename T> inline vec2<T> operator*(T s, vec2<T> a) { return vec2<T>{s * a.x, s * a.y}; }
template <typename T> inline vec2<T> operator/(vec2<T> a, T s) { return vec2<T>{a.x / s, a.y / s}; }

using vec2d = vec2<double>;
using vec2f = vec2<float>;
using vec2i = vec2<int>;

namespace aml {
template <typename T> inline T normsq(vec2<T> a) { return a.x * a.x + a.y * a.y; }
template <typename T> inline T norm(vec2<T> a) { return std::sqrt(normsq(a)); }
inline vec2f toFloat(vec2d a) { return vec2f{(float)a.x, (float)a.y}; }
}  // namespace aml
