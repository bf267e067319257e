/*
 * fs3d_oracle.c — CPU restatement of the reference's 3D grid containers.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Called by tests/ as the checker of
 * the device kernels behind include/fs3d.h, never by the product.
 *
 * Restates, in C and in the reference's floating-point operation order,
 *   include/Array3D.h   — operator+= (:39-45), setMultiplyAdd (:48-53),
 *                         innerProduct (:55-62), infiniteNorm (:64-73),
 *                         triCubic (:75-124);
 *   include/MACGrid3D.h — vel (:73-78), velU (:80-99), velV (:101-120),
 *                         velW (:122-141), velInterpU/V/W (:143-159),
 *                         velDiv (:165-167).
 * Build with -ffp-contract=off: every result then equals the reference's
 * scalar C++ bit for bit where the reference's code is well defined.  Two
 * rules differ from the literal code, as include/fs3d.h states: the bulk
 * loops cover the array's own NX*NY*NZ elements (the reference runs j up
 * to NY inclusive), and triCubic reads element (xp, yp, zp) (the reference
 * reads (zp, yp, xp)).  tests/test_grid3d_oracle.py pins both against the
 * reference's own headers compiled with the oracle shim, on inputs where
 * the literal code stays inside its arrays.
 */
#include <math.h>
#include <stddef.h>
#include "fs3d_oracle.h"

static size_t count3(int nx, int ny, int nz) { return (size_t)nx * ny * nz; }

void or3_add(double* a, const double* b, int nx, int ny, int nz) {
    const size_t n = count3(nx, ny, nz);
    for (size_t e = 0; e < n; e++) a[e] += b[e];
}

void or3_set_multiply_add(double* out, const double* a, double s, const double* c, int nx, int ny, int nz) {
    const size_t n = count3(nx, ny, nz);
    for (size_t e = 0; e < n; e++) out[e] = a[e] + s * c[e];
}

double or3_inner_product(const double* a, const double* b, int nx, int ny, int nz) {
    const size_t n = count3(nx, ny, nz);
    double r = 0.0;
    for (size_t e = 0; e < n; e++) r += a[e] * b[e];
    return r;
}

double or3_infinite_norm(const double* a, int nx, int ny, int nz) {
    const size_t n = count3(nx, ny, nz);
    double r = 0.0;
    for (size_t e = 0; e < n; e++)
        if (fabs(a[e]) > r) r = fabs(a[e]);
    return r;
}

static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* A coordinate whose truncation is no int (NaN, infinities, |p| >= 2^31)
 * counts as outside, which is what the reference gives on x86-64, where such
 * a conversion yields INT_MIN. */
static int int_range(double p) { return p > -2147483649.0 && p < 2147483648.0; }

#define CUBE(x) ((x) * (x) * (x))
#define SQR(x) ((x) * (x))

double or3_tricubic_at(const double* a, int NX, int NY, int NZ, double px, double py, double pz) {
    if (!int_range(px) || !int_range(py) || !int_range(pz)) return 0.0;
    const int x = (int)px, y = (int)py, z = (int)pz;
    if (x < 0 || x >= NX || y < 0 || y >= NY || z < 0 || z >= NZ) return 0.0;
    const double dx = px - (double)x, dy = py - (double)y, dz = pz - (double)z;
    double u[4], v[4], w[4], r[4], q[4];
    double vox = 0;
    u[0] = -0.5 * CUBE(dx) + SQR(dx) - 0.5 * dx;
    u[1] = 1.5 * CUBE(dx) - 2.5 * SQR(dx) + 1;
    u[2] = -1.5 * CUBE(dx) + 2 * SQR(dx) + 0.5f * dx;
    u[3] = 0.5 * CUBE(dx) - 0.5 * SQR(dx);
    v[0] = -0.5 * CUBE(dy) + SQR(dy) - 0.5 * dy;
    v[1] = 1.5 * CUBE(dy) - 2.5 * SQR(dy) + 1;
    v[2] = -1.5 * CUBE(dy) + 2 * SQR(dy) + 0.5 * dy;
    v[3] = 0.5 * CUBE(dy) - 0.5 * SQR(dy);
    w[0] = -0.5 * CUBE(dz) + SQR(dz) - 0.5 * dz;
    w[1] = 1.5 * CUBE(dz) - 2.5 * SQR(dz) + 1;
    w[2] = -1.5 * CUBE(dz) + 2 * SQR(dz) + 0.5 * dz;
    w[3] = 0.5 * CUBE(dz) - 0.5 * SQR(dz);
    for (int k = 0; k < 4; k++) {
        const int zp = clampi(z + k - 1, 0, NZ - 1);
        q[k] = 0;
        for (int j = 0; j < 4; j++) {
            const int yp = clampi(y + j - 1, 0, NY - 1);
            r[j] = 0;
            for (int i = 0; i < 4; i++) {
                const int xp = clampi(x + i - 1, 0, NX - 1);
                r[j] += u[i] * a[((size_t)zp * NY + yp) * NX + xp];
            }
            q[k] += v[j] * r[j];
        }
        vox += w[k] * q[k];
    }
    return vox < 0 ? 0.0 : vox;
}

void or3_tricubic(const double* a, int nx, int ny, int nz, const double* pts, size_t n, double* out) {
    for (size_t e = 0; e < n; e++) out[e] = or3_tricubic_at(a, nx, ny, nz, pts[3 * e], pts[3 * e + 1], pts[3 * e + 2]);
}

/* element (i, j, k) of the u, v, w face arrays of a sx x sy x sz grid */
#define U(i, j, k) u[((size_t)(k) * sy + (j)) * (sx + 1) + (i)]
#define V(i, j, k) v[((size_t)(k) * (sy + 1) + (j)) * sx + (i)]
#define W(i, j, k) w[((size_t)(k) * sy + (j)) * sx + (i)]

void or3_mac_vel(const double* u, const double* v, const double* w, int sx, int sy, int sz, double* out) {
    for (int k = 0; k < sz; k++)
        for (int j = 0; j < sy; j++)
            for (int i = 0; i < sx; i++) {
                double* o = out + 3 * (((size_t)k * sy + j) * sx + i);
                o[0] = 0.5 * (U(i + 1, j, k) + U(i, j, k));
                o[1] = 0.5 * (V(i, j + 1, k) + V(i, j, k));
                o[2] = 0.5 * (W(i, j, k + 1) + W(i, j, k));
            }
}

void or3_mac_vel_div(const double* u, const double* v, const double* w, int sx, int sy, int sz, double* out) {
    for (int k = 0; k < sz; k++)
        for (int j = 0; j < sy; j++)
            for (int i = 0; i < sx; i++)
                out[((size_t)k * sy + j) * sx + i] =
                    (U(i + 1, j, k) - U(i, j, k) + V(i, j + 1, k) - V(i, j, k) + W(i, j, k + 1) - W(i, j, k));
}

void or3_mac_face_vel(const double* u, const double* v, const double* w, int sx, int sy, int sz, int axis,
                      double* out) {
    const int fx = sx + (axis == 0), fy = sy + (axis == 1), fz = sz + (axis == 2);
    for (int k = 0; k < fz; k++)
        for (int j = 0; j < fy; j++)
            for (int i = 0; i < fx; i++) {
                double* o = out + 3 * (((size_t)k * fy + j) * fx + i);
                if (axis == 0) {            /* velU */
                    o[0] = U(i, j, k);
                    if (i > 0 && i < sx) {
                        o[1] = 0.25 * (V(i - 1, j, k) + V(i - 1, j + 1, k) + V(i, j, k) + V(i, j + 1, k));
                        o[2] = 0.25 * (W(i - 1, j, k) + W(i - 1, j, k + 1) + W(i, j, k) + W(i, j, k + 1));
                    } else if (i == 0) {
                        o[1] = 0.25 * (V(i, j, k) + V(i, j + 1, k));
                        o[2] = 0.25 * (W(i, j, k) + W(i, j, k + 1));
                    } else {
                        o[1] = 0.25 * (V(i - 1, j, k) + V(i - 1, j + 1, k));
                        o[2] = 0.25 * (W(i - 1, j, k) + W(i - 1, j, k + 1));
                    }
                } else if (axis == 1) {     /* velV */
                    o[1] = V(i, j, k);
                    if (j > 0 && j < sy) {
                        o[0] = 0.25 * (U(i, j - 1, k) + U(i, j, k) + U(i + 1, j - 1, k) + U(i + 1, j, k));
                        o[2] = 0.25 * (W(i, j - 1, k) + W(i, j - 1, k + 1) + W(i, j, k) + W(i, j, k + 1));
                    } else if (j == 0) {
                        o[0] = 0.25 * (U(i, j, k) + U(i + 1, j, k));
                        o[2] = 0.25 * (W(i, j, k) + W(i, j, k + 1));
                    } else {
                        o[0] = 0.25 * (U(i, j - 1, k) + U(i + 1, j - 1, k));
                        o[2] = 0.25 * (W(i, j - 1, k) + W(i, j - 1, k + 1));
                    }
                } else {                    /* velW */
                    o[2] = W(i, j, k);
                    if (k > 0 && k < sz) {
                        o[0] = 0.25 * (U(i, j, k - 1) + U(i + 1, j, k - 1) + U(i, j, k) + U(i + 1, j, k));
                        o[1] = 0.25 * (V(i, j, k - 1) + V(i, j + 1, k - 1) + V(i, j, k) + V(i, j + 1, k));
                    } else if (k == 0) {
                        o[0] = 0.25 * (U(i, j, k) + U(i + 1, j, k));
                        o[1] = 0.25 * (V(i, j, k) + V(i, j + 1, k));
                    } else {
                        o[0] = 0.25 * (U(i, j, k - 1) + U(i + 1, j, k - 1));
                        o[1] = 0.25 * (V(i, j, k - 1) + V(i, j + 1, k - 1));
                    }
                }
            }
}

void or3_mac_vel_interp(const double* u, const double* v, const double* w, int sx, int sy, int sz, int component,
                        const double* pts, size_t n, double* out) {
    for (size_t e = 0; e < n; e++) {
        const double x = pts[3 * e], y = pts[3 * e + 1], z = pts[3 * e + 2];
        const double ru = or3_tricubic_at(u, sx + 1, sy, sz, x, y - 0.5, z - 0.5);
        const double rv = or3_tricubic_at(v, sx, sy + 1, sz, x - 0.5, y, z - 0.5);
        const double rw = or3_tricubic_at(w, sx, sy, sz + 1, x - 0.5, y - 0.5, z);
        if (component == 0) out[e] = ru;
        else if (component == 1) out[e] = rv;
        else if (component == 2) out[e] = rw;
        else {
            out[3 * e] = ru;
            out[3 * e + 1] = rv;
            out[3 * e + 2] = rw;
        }
    }
}
