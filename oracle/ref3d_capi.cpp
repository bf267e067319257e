// ref3d_capi.cpp — C wrapper around the reference's UNMODIFIED 3D containers
// (test infrastructure: the oracle, never part of the product).
//
// include/Array3D.h and include/MACGrid3D.h are header-only; this file
// includes them in place from the reference checkout (with the oracle shim
// for altlib/altmath) and is compiled into oracle/_ref/libfs3d_ref.so.  Each
// function wraps caller-owned buffers in the reference's own structs and
// calls the reference's method, so that tests can compare the restatement
// (oracle/restate/fs3d_oracle.c) with the reference's code.
//
// The reference's bulk loops run j up to NY inclusive and therefore touch NX
// elements past the end of an array: callers pass buffers with at least NX
// spare elements after the NX*NY*NZ of the array.  Its triCubic reads
// element (zp, yp, xp), which stays inside the array only when NX == NZ.
#include <cstddef>
#include <cstring>
#include "Array3D.h"
#include "MACGrid3D.h"
#include "../include/fs3d.h"

static_assert(sizeof(vec3d) == 3 * sizeof(double), "vec3d layout");
// the C ABI's structs are the reference's, byte for byte
static_assert(sizeof(fs3d_array) == sizeof(Array3D<double>), "Array3D layout");
static_assert(offsetof(fs3d_array, NX) == offsetof(Array3D<double>, NX), "Array3D layout");
static_assert(offsetof(fs3d_array, NZ) == offsetof(Array3D<double>, NZ), "Array3D layout");
static_assert(sizeof(fs3d_mac) == sizeof(MACGrid3D), "MACGrid3D layout");
static_assert(offsetof(fs3d_mac, v) == offsetof(MACGrid3D, v), "MACGrid3D layout");
static_assert(offsetof(fs3d_mac, w) == offsetof(MACGrid3D, w), "MACGrid3D layout");
static_assert(offsetof(fs3d_mac, sizeX) == offsetof(MACGrid3D, sizeX), "MACGrid3D layout");
static_assert(offsetof(fs3d_mac, sizeZ) == offsetof(MACGrid3D, sizeZ), "MACGrid3D layout");

static Array3D<double> wrap(double* d, int nx, int ny, int nz) { return Array3D<double>{d, nx, ny, nz}; }

static MACGrid3D mac(double* u, double* v, double* w, int sx, int sy, int sz) {
    return MACGrid3D{wrap(u, sx + 1, sy, sz), wrap(v, sx, sy + 1, sz), wrap(w, sx, sy, sz + 1), sx, sy, sz};
}

extern "C" {

// Array3D::operator+= (include/Array3D.h:39-45)
void r3_add(double* a, double* b, int nx, int ny, int nz) {
    Array3D<double> A = wrap(a, nx, ny, nz), B = wrap(b, nx, ny, nz);
    A += B;
}

// Array3D::setMultiplyAdd (include/Array3D.h:48-53)
void r3_set_multiply_add(double* out, double* a, double s, double* c, int nx, int ny, int nz) {
    Array3D<double> O = wrap(out, nx, ny, nz), A = wrap(a, nx, ny, nz), Cc = wrap(c, nx, ny, nz);
    O.setMultiplyAdd(A, s, Cc);
}

// Array3D::innerProduct (include/Array3D.h:55-62)
double r3_inner_product(double* a, double* b, int nx, int ny, int nz) {
    const Array3D<double> A = wrap(a, nx, ny, nz), B = wrap(b, nx, ny, nz);
    return A.innerProduct(B);
}

// Array3D::infiniteNorm (include/Array3D.h:64-73)
double r3_infinite_norm(double* a, int nx, int ny, int nz) {
    const Array3D<double> A = wrap(a, nx, ny, nz);
    return A.infiniteNorm();
}

// Array3D::triCubic (include/Array3D.h:75-124) at n points
void r3_tricubic(double* a, int nx, int ny, int nz, const double* pts, size_t n, double* out) {
    Array3D<double> A = wrap(a, nx, ny, nz);
    for (size_t e = 0; e < n; e++) out[e] = A.triCubic(vec3d{pts[3 * e], pts[3 * e + 1], pts[3 * e + 2]});
}

// MACGrid3D::vel (include/MACGrid3D.h:73-78) at every cell
void r3_mac_vel(double* u, double* v, double* w, int sx, int sy, int sz, double* out) {
    MACGrid3D g = mac(u, v, w, sx, sy, sz);
    size_t c = 0;
    g.iterate([&](int i, int j, int k) {
        const vec3d r = g.vel(i, j, k);
        out[3 * c] = r.x;
        out[3 * c + 1] = r.y;
        out[3 * c + 2] = r.z;
        c++;
    });
}

// MACGrid3D::velU / velV / velW (include/MACGrid3D.h:80-141) at every face of one axis
void r3_mac_face_vel(double* u, double* v, double* w, int sx, int sy, int sz, int axis, double* out) {
    MACGrid3D g = mac(u, v, w, sx, sy, sz);
    size_t c = 0;
    auto put = [&](vec3d r) {
        out[3 * c] = r.x;
        out[3 * c + 1] = r.y;
        out[3 * c + 2] = r.z;
        c++;
    };
    if (axis == 0) g.iterateU([&](int i, int j, int k) { put(g.velU(i, j, k)); });
    else if (axis == 1) g.iterateV([&](int i, int j, int k) { put(g.velV(i, j, k)); });
    else g.iterateW([&](int i, int j, int k) { put(g.velW(i, j, k)); });
}

// MACGrid3D::velDiv (include/MACGrid3D.h:165-167) at every cell
void r3_mac_vel_div(double* u, double* v, double* w, int sx, int sy, int sz, double* out) {
    MACGrid3D g = mac(u, v, w, sx, sy, sz);
    size_t c = 0;
    g.iterate([&](int i, int j, int k) { out[c++] = g.velDiv(i, j, k); });
}

// MACGrid3D::velInterpU / V / W / velInterp (include/MACGrid3D.h:143-163) on
// a grid whose three component arrays are all n x n x n cubes, the only
// shape on which the reference's triCubic stays inside its array.
void r3_mac_vel_interp_cubes(double* u, double* v, double* w, int n, int component, const double* pts, size_t np,
                             double* out) {
    MACGrid3D g{wrap(u, n, n, n), wrap(v, n, n, n), wrap(w, n, n, n), n, n, n};
    for (size_t e = 0; e < np; e++) {
        const vec3d p{pts[3 * e], pts[3 * e + 1], pts[3 * e + 2]};
        if (component == 0) out[e] = g.velInterpU(p);
        else if (component == 1) out[e] = g.velInterpV(p);
        else if (component == 2) out[e] = g.velInterpW(p);
        else {
            const vec3d r = g.velInterp(p);
            out[3 * e] = r.x;
            out[3 * e + 1] = r.y;
            out[3 * e + 2] = r.z;
        }
    }
}

}  // extern "C"
