/*
 * fs3d.h — C ABI of the GB300 3D grid containers.
 *
 * The reference ships two 3D containers that no simulation step uses yet:
 * `Array3D<T>` (include/Array3D.h:15-128) and the staggered `MACGrid3D`
 * (include/MACGrid3D.h:12-168).  This header gives every method of both a
 * bulk device counterpart: one call applies the method to a whole array,
 * every cell, every face of one axis or a batch of sample points, as CUDA
 * kernels on one GPU.  They live in the same library as fs2d.h (libfs2d.so),
 * return the same status codes and report through fs2d_last_error().
 *
 * Structs are byte-compatible with the reference's: `fs3d_array` with
 * Array3D<double> {data, NX, NY, NZ} and `fs3d_mac` with MACGrid3D
 * {u, v, w, sizeX, sizeY, sizeZ}, so a caller that fills a reference struct
 * with DEVICE pointers can pass it as it is.  Element (i, j, k) is
 * data[k*NY*NX + j*NX + i] (Array3D::operator(), include/Array3D.h:32-37);
 * u has (sizeX+1) x sizeY x sizeZ faces, v sizeX x (sizeY+1) x sizeZ and w
 * sizeX x sizeY x (sizeZ+1) (MACGrid3D::create, include/MACGrid3D.h:16-23).
 * Vectors (points, velocities) are interleaved (x, y, z) doubles, one vec3d
 * each.
 *
 * Every data pointer must be device memory (or managed memory) of the
 * current device: each call checks this with cudaPointerGetAttributes and
 * refuses host pointers with FS2D_ERR_INVALID before any kernel runs.
 * Work is queued on `stream` (NULL: the legacy default stream); the calls
 * that return a scalar (inner product, infinite norm) wait for it.
 *
 * Two places where the reference's own code cannot be followed literally
 * (its arithmetic is followed everywhere else, bit for bit):
 *   - the bulk loops of operator+=, setMultiplyAdd, innerProduct and
 *     infiniteNorm (include/Array3D.h:39-73) run j up to NY inclusive, so
 *     they visit row 0 of every slab k+1 a second time and, in the last
 *     slab, NX elements past the end of the array.  Here they cover the
 *     array's own NX*NY*NZ elements once each;
 *   - triCubic (include/Array3D.h:75-124) reads the sample as
 *     (*this)(zp, yp, xp), the x and z indices swapped, which for NX != NZ
 *     (every face array of a MAC grid) reads outside the array.  Here it
 *     reads (xp, yp, zp), matching its own bounds test and clamping; on a
 *     cube the reference's result equals this one on the array with its x
 *     and z axes exchanged.
 */
#ifndef FS3D_H
#define FS3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Array3D<double> (include/Array3D.h:15-18): device data, NX x NY x NZ. */
typedef struct fs3d_array {
    double* data;
    int NX;
    int NY;
    int NZ;
} fs3d_array;

/* MACGrid3D (include/MACGrid3D.h:12-14). */
typedef struct fs3d_mac {
    fs3d_array u;
    fs3d_array v;
    fs3d_array w;
    int sizeX;
    int sizeY;
    int sizeZ;
} fs3d_mac;

/* which velocity component(s) fs3d_mac_vel_interp samples */
#define FS3D_U   0  /* velInterpU: one double per point */
#define FS3D_V   1  /* velInterpV */
#define FS3D_W   2  /* velInterpW */
#define FS3D_UVW 3  /* velInterp: one vec3d per point */

/* a = a + b, element by element (Array3D::operator+=, include/Array3D.h:39-45).
 * b has a's extents. */
int fs3d_add(const fs3d_array* a, const fs3d_array* b, void* stream);

/* out = a + s * c (Array3D::setMultiplyAdd, include/Array3D.h:48-53; the
 * product rounded before the sum).  a, c and out have the same extents; out
 * may be a or c. */
int fs3d_set_multiply_add(const fs3d_array* out, const fs3d_array* a, double s, const fs3d_array* c,
                          void* stream);

/* *result (host) = sum of a*b over all elements (Array3D::innerProduct,
 * include/Array3D.h:55-62).  The sum is taken as a fixed tree (the same
 * result on every run), not in the serial loop's order, each product added
 * with a fused multiply-add; it differs from the serial sum by at most
 * 2 n 2^-53 sum |a*b|. */
int fs3d_inner_product(const fs3d_array* a, const fs3d_array* b, double* result, void* stream);

/* *result (host) = max |a| over all elements, 0 for an empty array; NaN
 * elements are passed over, as the reference's `abs(x) > result` test does
 * (Array3D::infiniteNorm, include/Array3D.h:64-73). */
int fs3d_infinite_norm(const fs3d_array* a, double* result, void* stream);

/* out[n] = a.triCubic(points[n]) for n points in grid coordinates
 * (include/Array3D.h:75-124): Catmull-Rom weights of the fractional parts,
 * 4x4x4 neighbours with clamped indices, rows then planes accumulated in
 * the reference's order, 0 where (int)x, (int)y or (int)z lies outside the
 * array, negative results replaced by 0. */
int fs3d_tricubic(const fs3d_array* a, const double* points, size_t n, double* out, void* stream);

/* out[c] = vel(i, j, k) at every cell c = k*sizeY*sizeX + j*sizeX + i, one
 * vec3d each (MACGrid3D::vel, include/MACGrid3D.h:73-78). */
int fs3d_mac_vel(const fs3d_mac* g, double* out, void* stream);

/* velU / velV / velW (include/MACGrid3D.h:80-141) at every face of the axis
 * given by `axis` (FS3D_U, FS3D_V or FS3D_W), one vec3d per face, faces in
 * the layout of that component's array. */
int fs3d_mac_face_vel(const fs3d_mac* g, int axis, double* out, void* stream);

/* velInterpU / V / W or velInterp (include/MACGrid3D.h:143-163) at n points
 * in grid coordinates: `component` FS3D_U, FS3D_V, FS3D_W writes one double
 * per point, FS3D_UVW one vec3d per point. */
int fs3d_mac_vel_interp(const fs3d_mac* g, int component, const double* points, size_t n, double* out,
                        void* stream);

/* out[c] = velDiv(i, j, k) at every cell (include/MACGrid3D.h:165-167). */
int fs3d_mac_vel_div(const fs3d_mac* g, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FS3D_H */
