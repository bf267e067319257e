/*
 * MACGrid3D_gb300.hpp — the reference's 3D containers (include/Array3D.h,
 * include/MACGrid3D.h) for C++ programs that use this library.
 *
 * `Array3D<T>` and `MACGrid3D` keep the reference's names, public fields
 * ({data, NX, NY, NZ}; {u, v, w, sizeX, sizeY, sizeZ}), layout (element
 * (i, j, k) at data[k*NY*NX + j*NX + i]) and methods, on host memory, so a
 * program written against the reference's headers compiles against this one.
 * The methods follow the reference's arithmetic in its operation order, with
 * the two corrections include/fs3d.h states: the bulk loops (+=,
 * setMultiplyAdd, innerProduct, infiniteNorm) cover the array's own
 * NX*NY*NZ elements once each, and triCubic reads element (xp, yp, zp).
 *
 * The same structs whose `data` point to DEVICE memory are what the C ABI of
 * include/fs3d.h takes (the layouts are identical); namespace fs3d_device
 * wraps those calls, one bulk GPU launch per method: a whole array, every
 * cell, every face of an axis, or a batch of points.
 *
 * Define FS3D_GB300_NO_VEC_TYPES when the program already has the
 * reference's vec3<T> / vec3d (altmath); otherwise this header provides a
 * minimal version with the members the containers use.
 */
#ifndef MACGRID3D_GB300_HPP
#define MACGRID3D_GB300_HPP

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "fs2d.h"
#include "fs3d.h"

#ifndef FS3D_GB300_NO_VEC_TYPES
template <typename T>
struct vec3 {
    T x, y, z;
};
template <typename T>
inline vec3<T> operator*(T s, vec3<T> a) {
    return vec3<T>{s * a.x, s * a.y, s * a.z};
}
using vec3d = vec3<double>;
#endif

// Array3D<T> (include/Array3D.h:15-128), host storage.
template <typename T>
struct Array3D {
    T* data;
    int NX, NY, NZ;

    static Array3D create(int nx, int ny, int nz) {
        const size_t n = (size_t)nx * ny * nz;
        T* p = new (std::nothrow) T[n ? n : 1]();
        if (!p) {
            std::fprintf(stderr, "fs3d: out of host memory\n");
            std::exit(EXIT_FAILURE);
        }
        return {p, nx, ny, nz};
    }
    void free() {
        delete[] data;
        data = nullptr;
    }
    size_t count() const { return (size_t)NX * NY * NZ; }
    void copyFrom(const Array3D& arr) { std::memcpy(static_cast<void*>(data), arr.data, sizeof(T) * count()); }

    T& operator()(int i, int j, int k) { return data[((size_t)k * NY + j) * NX + i]; }
    const T& operator()(int i, int j, int k) const { return data[((size_t)k * NY + j) * NX + i]; }

    Array3D& operator+=(const Array3D& rhs) {
        for (size_t e = 0; e < count(); e++) data[e] += rhs.data[e];
        return *this;
    }
    void setMultiplyAdd(Array3D& a, T b, const Array3D& c) {
        for (size_t e = 0; e < count(); e++) data[e] = a.data[e] + b * c.data[e];
    }
    T innerProduct(const Array3D& rhs) const {
        T result = {};
        for (size_t e = 0; e < count(); e++) result += data[e] * rhs.data[e];
        return result;
    }
    T infiniteNorm() const {
        T result = {};
        for (size_t e = 0; e < count(); e++)
            if (std::abs(data[e]) > result) result = std::abs(data[e]);
        return result;
    }

    // Catmull-Rom sample at grid coordinates p: 4x4x4 neighbours with
    // clamped indices, rows then planes accumulated in the reference's
    // order; 0 outside the array (or where a coordinate's truncation is no
    // int); negative results replaced by 0.
    T triCubic(vec3<T> p) const {
        if (!inRange(p.x) || !inRange(p.y) || !inRange(p.z)) return T(0);
        const int x = (int)p.x, y = (int)p.y, z = (int)p.z;
        if (x < 0 || x >= NX || y < 0 || y >= NY || z < 0 || z >= NZ) return T(0);
        T u[4], v[4], w[4];
        weights(p.x - (T)x, u);
        weights(p.y - (T)y, v);
        weights(p.z - (T)z, w);
        T vox = 0;
        for (int k = 0; k < 4; k++) {
            const int zp = clampi(z + k - 1, 0, NZ - 1);
            T q = 0;
            for (int j = 0; j < 4; j++) {
                const int yp = clampi(y + j - 1, 0, NY - 1);
                T r = 0;
                for (int i = 0; i < 4; i++) r += u[i] * (*this)(clampi(x + i - 1, 0, NX - 1), yp, zp);
                q += v[j] * r;
            }
            vox += w[k] * q;
        }
        return (T)(vox < 0 ? 0.0 : vox);
    }

  private:
    static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
    static bool inRange(T p) { return p > T(-2147483649.0) && p < T(2147483648.0); }
    static void weights(T t, T* c) {
        const T t3 = t * t * t, t2 = t * t;
        c[0] = T(-0.5) * t3 + t2 - T(0.5) * t;
        c[1] = T(1.5) * t3 - T(2.5) * t2 + 1;
        c[2] = T(-1.5) * t3 + 2 * t2 + T(0.5) * t;
        c[3] = T(0.5) * t3 - T(0.5) * t2;
    }
};

// MACGrid3D (include/MACGrid3D.h:12-168), host storage.
struct MACGrid3D {
    Array3D<double> u, v, w;
    int sizeX, sizeY, sizeZ;

    static MACGrid3D create(int nx, int ny, int nz) {
        return {Array3D<double>::create(nx + 1, ny, nz), Array3D<double>::create(nx, ny + 1, nz),
                Array3D<double>::create(nx, ny, nz + 1), nx, ny, nz};
    }
    void free() {
        u.free();
        v.free();
        w.free();
    }

    template <typename Fun>
    void iterateU(Fun f) {
        for (int k = 0; k < sizeZ; k++)
            for (int j = 0; j < sizeY; j++)
                for (int i = 0; i < sizeX + 1; i++) f(i, j, k);
    }
    template <typename Fun>
    void iterateV(Fun f) {
        for (int k = 0; k < sizeZ; k++)
            for (int j = 0; j < sizeY + 1; j++)
                for (int i = 0; i < sizeX; i++) f(i, j, k);
    }
    template <typename Fun>
    void iterateW(Fun f) {
        for (int k = 0; k < sizeZ + 1; k++)
            for (int j = 0; j < sizeY; j++)
                for (int i = 0; i < sizeX; i++) f(i, j, k);
    }
    template <typename Fun>
    void iterate(Fun f) {
        for (int k = 0; k < sizeZ; k++)
            for (int j = 0; j < sizeY; j++)
                for (int i = 0; i < sizeX; i++) f(i, j, k);
    }
    template <typename Fun>
    void iterateBackwards(Fun f) {
        for (int k = sizeZ; k-- > 0;)
            for (int j = sizeY; j-- > 0;)
                for (int i = sizeX; i-- > 0;) f(i, j, k);
    }

    // cell-centre velocity
    vec3d vel(int i, int j, int k) {
        return vec3d{0.5 * (u(i + 1, j, k) + u(i, j, k)), 0.5 * (v(i, j + 1, k) + v(i, j, k)),
                     0.5 * (w(i, j, k + 1) + w(i, j, k))};
    }
    // velocity at a u face: v and w averaged over the adjacent faces
    vec3d velU(int i, int j, int k) {
        if (i > 0 && i < sizeX)
            return vec3d{u(i, j, k), 0.25 * (v(i - 1, j, k) + v(i - 1, j + 1, k) + v(i, j, k) + v(i, j + 1, k)),
                         0.25 * (w(i - 1, j, k) + w(i - 1, j, k + 1) + w(i, j, k) + w(i, j, k + 1))};
        if (i == 0) return vec3d{u(i, j, k), 0.25 * (v(i, j, k) + v(i, j + 1, k)), 0.25 * (w(i, j, k) + w(i, j, k + 1))};
        return vec3d{u(i, j, k), 0.25 * (v(i - 1, j, k) + v(i - 1, j + 1, k)),
                     0.25 * (w(i - 1, j, k) + w(i - 1, j, k + 1))};
    }
    vec3d velV(int i, int j, int k) {
        if (j > 0 && j < sizeY)
            return vec3d{0.25 * (u(i, j - 1, k) + u(i, j, k) + u(i + 1, j - 1, k) + u(i + 1, j, k)), v(i, j, k),
                         0.25 * (w(i, j - 1, k) + w(i, j - 1, k + 1) + w(i, j, k) + w(i, j, k + 1))};
        if (j == 0) return vec3d{0.25 * (u(i, j, k) + u(i + 1, j, k)), v(i, j, k), 0.25 * (w(i, j, k) + w(i, j, k + 1))};
        return vec3d{0.25 * (u(i, j - 1, k) + u(i + 1, j - 1, k)), v(i, j, k),
                     0.25 * (w(i, j - 1, k) + w(i, j - 1, k + 1))};
    }
    vec3d velW(int i, int j, int k) {
        if (k > 0 && k < sizeZ)
            return vec3d{0.25 * (u(i, j, k - 1) + u(i + 1, j, k - 1) + u(i, j, k) + u(i + 1, j, k)),
                         0.25 * (v(i, j, k - 1) + v(i, j + 1, k - 1) + v(i, j, k) + v(i, j + 1, k)), w(i, j, k)};
        if (k == 0) return vec3d{0.25 * (u(i, j, k) + u(i + 1, j, k)), 0.25 * (v(i, j, k) + v(i, j + 1, k)), w(i, j, k)};
        return vec3d{0.25 * (u(i, j, k - 1) + u(i + 1, j, k - 1)), 0.25 * (v(i, j, k - 1) + v(i, j + 1, k - 1)),
                     w(i, j, k)};
    }
    // tricubic velocity at grid coordinates (each component sampled at its
    // face positions: half a cell off in the two other axes)
    double velInterpU(vec3d pos) {
        pos.y -= 0.5;
        pos.z -= 0.5;
        return u.triCubic(pos);
    }
    double velInterpV(vec3d pos) {
        pos.z -= 0.5;
        pos.x -= 0.5;
        return v.triCubic(pos);
    }
    double velInterpW(vec3d pos) {
        pos.x -= 0.5;
        pos.y -= 0.5;
        return w.triCubic(pos);
    }
    vec3d velInterp(vec3d pos) { return vec3d{velInterpU(pos), velInterpV(pos), velInterpW(pos)}; }
    double velDiv(int i, int j, int k) {
        return (u(i + 1, j, k) - u(i, j, k) + v(i, j + 1, k) - v(i, j, k) + w(i, j, k + 1) - w(i, j, k));
    }
};

static_assert(sizeof(Array3D<double>) == sizeof(fs3d_array), "Array3D<double> is laid out as fs3d_array");
static_assert(sizeof(MACGrid3D) == sizeof(fs3d_mac), "MACGrid3D is laid out as fs3d_mac");

// Bulk device versions of the methods (include/fs3d.h): the structs' data
// point to device memory; each returns the library's status (FS2D_OK = 0,
// message in fs2d_last_error()).
namespace fs3d_device {

inline fs3d_array view(const Array3D<double>& a) {
    fs3d_array r;
    std::memcpy(&r, &a, sizeof r);
    return r;
}
inline fs3d_mac view(const MACGrid3D& g) {
    fs3d_mac r;
    std::memcpy(&r, &g, sizeof r);
    return r;
}

// a += b
inline int add(Array3D<double>& a, const Array3D<double>& b, void* stream = nullptr) {
    const fs3d_array x = view(a), y = view(b);
    return fs3d_add(&x, &y, stream);
}
// out.setMultiplyAdd(a, s, c)
inline int setMultiplyAdd(Array3D<double>& out, const Array3D<double>& a, double s, const Array3D<double>& c,
                          void* stream = nullptr) {
    const fs3d_array o = view(out), x = view(a), y = view(c);
    return fs3d_set_multiply_add(&o, &x, s, &y, stream);
}
inline int innerProduct(const Array3D<double>& a, const Array3D<double>& b, double* result, void* stream = nullptr) {
    const fs3d_array x = view(a), y = view(b);
    return fs3d_inner_product(&x, &y, result, stream);
}
inline int infiniteNorm(const Array3D<double>& a, double* result, void* stream = nullptr) {
    const fs3d_array x = view(a);
    return fs3d_infinite_norm(&x, result, stream);
}
// out[n] = a.triCubic(points[n]); points and out in device memory
inline int triCubic(const Array3D<double>& a, const vec3d* points, size_t n, double* out, void* stream = nullptr) {
    const fs3d_array x = view(a);
    return fs3d_tricubic(&x, reinterpret_cast<const double*>(points), n, out, stream);
}
inline int vel(const MACGrid3D& g, vec3d* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_vel(&m, reinterpret_cast<double*>(out), stream);
}
inline int velU(const MACGrid3D& g, vec3d* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_face_vel(&m, FS3D_U, reinterpret_cast<double*>(out), stream);
}
inline int velV(const MACGrid3D& g, vec3d* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_face_vel(&m, FS3D_V, reinterpret_cast<double*>(out), stream);
}
inline int velW(const MACGrid3D& g, vec3d* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_face_vel(&m, FS3D_W, reinterpret_cast<double*>(out), stream);
}
inline int velInterp(const MACGrid3D& g, const vec3d* points, size_t n, vec3d* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_vel_interp(&m, FS3D_UVW, reinterpret_cast<const double*>(points), n,
                               reinterpret_cast<double*>(out), stream);
}
inline int velDiv(const MACGrid3D& g, double* out, void* stream = nullptr) {
    const fs3d_mac m = view(g);
    return fs3d_mac_vel_div(&m, out, stream);
}

}  // namespace fs3d_device

#endif  // MACGRID3D_GB300_HPP
