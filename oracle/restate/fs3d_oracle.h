/*
 * fs3d_oracle.h — CPU restatement of the reference's 3D grid containers
 * (include/Array3D.h, include/MACGrid3D.h of lasagnaphil/fluid-sim).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the device kernels behind
 * include/fs3d.h, called by tests/, never by the product.  Layouts are the
 * reference's: element (i, j, k) at k*NY*NX + j*NX + i; face arrays of a
 * sx x sy x sz MAC grid are (sx+1) x sy x sz (u), sx x (sy+1) x sz (v),
 * sx x sy x (sz+1) (w); points and vectors are interleaved (x, y, z).
 * `component` / `axis`: 0 u, 1 v, 2 w, 3 all three (velInterp).
 */
#ifndef FS3D_ORACLE_H
#define FS3D_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

void or3_add(double* a, const double* b, int nx, int ny, int nz);
void or3_set_multiply_add(double* out, const double* a, double s, const double* c, int nx, int ny, int nz);
double or3_inner_product(const double* a, const double* b, int nx, int ny, int nz);
double or3_infinite_norm(const double* a, int nx, int ny, int nz);
double or3_tricubic_at(const double* a, int nx, int ny, int nz, double px, double py, double pz);
void or3_tricubic(const double* a, int nx, int ny, int nz, const double* pts, size_t n, double* out);
void or3_mac_vel(const double* u, const double* v, const double* w, int sx, int sy, int sz, double* out);
void or3_mac_vel_div(const double* u, const double* v, const double* w, int sx, int sy, int sz, double* out);
void or3_mac_face_vel(const double* u, const double* v, const double* w, int sx, int sy, int sz, int axis,
                      double* out);
void or3_mac_vel_interp(const double* u, const double* v, const double* w, int sx, int sy, int sz, int component,
                        const double* pts, size_t n, double* out);

#ifdef __cplusplus
}
#endif

#endif
