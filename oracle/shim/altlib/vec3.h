// Compatibility shim (test infrastructure): 3-component vectors used by the
// reference's 3D containers (include/Array3D.h, include/MACGrid3D.h):
// aggregate vec3<T>{x, y, z}, component assignment (`pos.y -= 0.5`) and
// scalar * vector, which multiplies each component by the scalar.
#pragma once
#include "math_utils.h"

template <typename T>
struct vec3 {
    T x;
    T y;
    T z;
};

template <typename T> inline vec3<T> operator*(T s, vec3<T> a) { return vec3<T>{s * a.x, s * a.y, s * a.z}; }

using vec3d = vec3<double>;
