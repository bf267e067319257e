/*
 * fs2d_oracle.c — CPU restatement of the reference FluidSim2D time step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Restates, in C and in the same
 * floating-point operation order as the reference's scalar build,
 *   src/FluidSim2D.cpp  (lasagnaphil/fluid-sim)  — every stage of runFrame,
 *   include/Array2D.h   — triCubic, linearDistribute, linearExtract,
 *                         extrapolate, innerProduct, infiniteNorm,
 *   include/MACGrid2D.h — velInterpU / velInterpV,
 *   include/FluidSim2D.h — fastSweepIterate.
 * Build with -ffp-contract=off so that no multiply-add is fused: the
 * reference's scalar build with the same flag is then reproduced bit for bit.
 *
 * OpenMP pragmas sit on the loops the reference parallelises, except the
 * three whose parallel form races in the reference (MIC(0) factorisation,
 * particle seeding of the level set, in-place semi-Lagrangian advection);
 * those stay serial.  Without -fopenmp the pragmas are ignored.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "fs2d_oracle.h"

#define CELL_EMPTY 0
#define CELL_FLUID 1
#define CELL_SOLID 2
#define MASK_UNKNOWN 0xFFFFFFFFu

struct or_sim {
    int NX, NY, ppcSqrt, ppc;
    double dt, dx, dr, rho, gx, gy, alpha;
    int mode;
    or_options opt;
    uint8_t* cell;
    double* phi;
    double* p;
    double *u, *v, *nu, *nv;   /* mac.u, mac.v, newMac.u, newMac.v */
    double* pos;               /* 2*np interleaved */
    double* vel;
    size_t np;
    double waterVolume, origWaterVolume, totalEnergy, particleTotalEnergy, currentTime;
    int lastIters;
    double lastRelRes;
};

/* aml::max / aml::min / aml::clamp with the shim's tie and NaN behaviour */
static inline double maxd(double a, double b) { return (a < b) ? b : a; }
static inline double mind(double a, double b) { return (b < a) ? b : a; }
static inline double clampd(double v, double lo, double hi) { return mind(maxd(v, lo), hi); }
static inline int clampi(int v, int lo, int hi) {
    int m = (v < lo) ? lo : v;
    return (hi < m) ? hi : m;
}

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

/* ------------------------------------------------------------------ */
/* Array2D<double> numerics (include/Array2D.h)                       */
/* ------------------------------------------------------------------ */

#define CUBE(x) ((x) * (x) * (x))
#define SQR(x) ((x) * (x))

/* Array2D::triCubic, scalar branch (include/Array2D.h:244-249,328-355):
 * Catmull-Rom weights, indices clamped to the array. */
double or_tricubic(const double* data, int NX, int NY, double px, double py) {
    int x = (int)px, y = (int)py;
    if (x < 0 || x >= NX || y < 0 || y >= NY) return 0;
    double dx = px - (double)x, dy = py - (double)y;
    double u[4], v[4], r[4];
    double vox = 0;
    u[0] = -0.5 * CUBE(dx) + SQR(dx) - 0.5 * dx;
    u[1] = 1.5 * CUBE(dx) - 2.5 * SQR(dx) + 1;
    u[2] = -1.5 * CUBE(dx) + 2 * SQR(dx) + 0.5 * dx;
    u[3] = 0.5 * CUBE(dx) - 0.5 * SQR(dx);
    v[0] = -0.5 * CUBE(dy) + SQR(dy) - 0.5 * dy;
    v[1] = 1.5 * CUBE(dy) - 2.5 * SQR(dy) + 1;
    v[2] = -1.5 * CUBE(dy) + 2 * SQR(dy) + 0.5 * dy;
    v[3] = 0.5 * CUBE(dy) - 0.5 * SQR(dy);
    for (int j = 0; j < 4; j++) {
        int yp = clampi(y + j - 1, 0, NY - 1);
        r[j] = 0;
        for (int i = 0; i < 4; i++) {
            int xp = clampi(x + i - 1, 0, NX - 1);
            r[j] += u[i] * data[yp * NX + xp];
        }
        vox += v[j] * r[j];
    }
    return vox;
}

/* Array2D::linearDistribute (include/Array2D.h:361-376) */
static void linear_distribute(double* a, int NX, int NY, double px, double py, double value) {
    int ui = (int)px, uj = (int)py;
    double dispx = px - ui, dispy = py - uj;
    int x1 = clampi(ui, 0, NX - 1), x2 = clampi(ui + 1, 0, NX - 1);
    int y1 = clampi(uj, 0, NY - 1), y2 = clampi(uj + 1, 0, NY - 1);
    a[y1 * NX + x1] += (1 - dispx) * (1 - dispy) * value;
    a[y1 * NX + x2] += dispx * (1 - dispy) * value;
    a[y2 * NX + x1] += (1 - dispx) * dispy * value;
    a[y2 * NX + x2] += dispx * dispy * value;
}

/* Array2D::linearExtract (include/Array2D.h:402-420) */
static double linear_extract(const double* a, int NX, int NY, double px, double py) {
    int ui = (int)px, uj = (int)py;
    double dispx = px - ui, dispy = py - uj;
    double value = 0.0;
    int x1 = clampi(ui, 0, NX - 1), x2 = clampi(ui + 1, 0, NX - 1);
    int y1 = clampi(uj, 0, NY - 1), y2 = clampi(uj + 1, 0, NY - 1);
    value += a[y1 * NX + x1] * (1 - dispx) * (1 - dispy);
    value += a[y1 * NX + x2] * dispx * (1 - dispy);
    value += a[y2 * NX + x1] * (1 - dispx) * dispy;
    value += a[y2 * NX + x2] * dispx * dispy;
    return value;
}

/* Array2D::extrapolate (include/Array2D.h:552-591): breadth-first layers
 * from the known faces (mask 0); each unknown face takes the mean of its
 * 4-neighbours of strictly lower layer, summed in the order x-1, x+1, y-1,
 * y+1.  `band` > 0 stops after that many layers (not in the reference). */
void or_extrapolate(double* a, int NX, int NY, uint32_t* mask, int band) {
    size_t cap = (size_t)NX * NY;
    int* qx = (int*)xcalloc(cap, sizeof(int));
    int* qy = (int*)xcalloc(cap, sizeof(int));
    size_t head = 0, tail = 0;
    for (int j = 0; j < NY; j++) {
        for (int i = 0; i < NX; i++) {
            if (mask[j * NX + i] != 0 &&
                ((i > 0 && mask[j * NX + i - 1] == 0) || (i < NX - 1 && mask[j * NX + i + 1] == 0) ||
                 (j > 0 && mask[(j - 1) * NX + i] == 0) || (j < NY - 1 && mask[(j + 1) * NX + i] == 0))) {
                mask[j * NX + i] = 1;
                qx[tail] = i; qy[tail] = j; tail++;
            }
        }
    }
    static const int ox[4] = {-1, 1, 0, 0};
    static const int oy[4] = {0, 0, -1, 1};
    while (tail > head) {
        int x = qx[head], y = qy[head];
        head++;
        uint32_t m = mask[y * NX + x];
        double sum = 0.0;
        int count = 0;
        for (int k = 0; k < 4; k++) {
            int nx = x + ox[k], ny = y + oy[k];
            if (nx < 0 || nx >= NX || ny < 0 || ny >= NY) continue;
            if (mask[ny * NX + nx] < m) { sum += a[ny * NX + nx]; count++; }
        }
        a[y * NX + x] = count == 0 ? 0 : sum / count;
        if (band > 0 && m >= (uint32_t)band) continue;
        for (int k = 0; k < 4; k++) {
            int nx = x + ox[k], ny = y + oy[k];
            if (nx < 0 || nx >= NX || ny < 0 || ny >= NY) continue;
            if (mask[ny * NX + nx] == MASK_UNKNOWN) {
                mask[ny * NX + nx] = m + 1;
                qx[tail] = nx; qy[tail] = ny; tail++;
            }
        }
    }
    free(qx);
    free(qy);
}

/* Array2D::innerProduct and infiniteNorm, scalar branch (include/Array2D.h:211-216,235-240) */
static double inner_product(const double* a, const double* b, size_t n) {
    double result = 0;
    for (size_t k = 0; k < n; k++) result += a[k] * b[k];
    return result;
}
static double infinite_norm(const double* a, size_t n) {
    double result = 0;
    for (size_t k = 0; k < n; k++)
        if (fabs(a[k]) > result) result = fabs(a[k]);
    return result;
}

/* ------------------------------------------------------------------ */
/* MACGrid2D sampling (include/MACGrid2D.h:80-97)                     */
/* ------------------------------------------------------------------ */

static double vel_interp_u(const or_sim* s, const double* u, double x, double y) {
    double px = x / s->dx, py = y / s->dx;
    py -= 0.5;
    px = clampd(px, 1e-6, (double)(s->NX - 1) - 1e-6);
    py = clampd(py, 1e-6, (double)(s->NY - 1) - 1e-6);
    return or_tricubic(u, s->NX + 1, s->NY, px, py);
}
static double vel_interp_v(const or_sim* s, const double* v, double x, double y) {
    double px = x / s->dx, py = y / s->dx;
    px -= 0.5;
    px = clampd(px, 1e-6, (double)(s->NX - 1) - 1e-6);
    py = clampd(py, 1e-6, (double)(s->NY - 1) - 1e-6);
    return or_tricubic(v, s->NX, s->NY + 1, px, py);
}

/* FluidSim2D::clampPos (src/FluidSim2D.cpp:645-651) */
static void clamp_pos(const or_sim* s, double* x, double* y) {
    const double offset = 1e-3;
    *x = clampd(*x, (1.0 + offset) * s->dx, (s->NX - 1.0 - offset) * s->dx);
    *y = clampd(*y, (1.0 + offset) * s->dx, (s->NY - 1.0 - offset) * s->dx);
}

/* ------------------------------------------------------------------ */
/* create (src/FluidSim2D.cpp:19-76)                                  */
/* ------------------------------------------------------------------ */

static double randf(float max) { return ((double)rand() / (double)RAND_MAX) * max; }

void or_default_options(or_options* o) {
    o->mic_tau = 0.999;
    o->mic_sigma = 0.25;
    o->pcg_tol = 1e-12;
    o->pcg_max_iters = 200;
    o->sl_inplace = 1;
    o->extrapolate_band = 0;
    o->volume_rate = 0.0;
}

or_sim* or_create(const fs2d_config* cfg, const or_options* opt, int use_seed, unsigned seed) {
    or_sim* s = (or_sim*)xcalloc(1, sizeof(or_sim));
    if (opt) s->opt = *opt; else or_default_options(&s->opt);
    s->NX = cfg->sizeX;
    s->NY = cfg->sizeY;
    s->ppcSqrt = cfg->particlesPerCellSqrt;
    s->ppc = s->ppcSqrt * s->ppcSqrt;
    s->dt = cfg->dt;
    s->dx = cfg->dx;
    s->dr = 0.9 * cfg->dx;
    s->rho = cfg->rho;
    s->gx = cfg->gravityX;
    s->gy = cfg->gravityY;
    s->mode = cfg->mode;
    s->alpha = cfg->picFlipAlpha;
    size_t N = (size_t)s->NX * s->NY;
    size_t NU = (size_t)(s->NX + 1) * s->NY, NV = (size_t)s->NX * (s->NY + 1);
    s->cell = (uint8_t*)xcalloc(N, 1);
    s->phi = (double*)xcalloc(N, sizeof(double));
    s->p = (double*)xcalloc(N, sizeof(double));
    s->u = (double*)xcalloc(NU, sizeof(double));
    s->nu = (double*)xcalloc(NU, sizeof(double));
    s->v = (double*)xcalloc(NV, sizeof(double));
    s->nv = (double*)xcalloc(NV, sizeof(double));
    memcpy(s->cell, cfg->initialValues, N);

    if (use_seed) srand(seed);
    size_t fluidCount = 0;
    for (size_t k = 0; k < N; k++) fluidCount += s->cell[k] == CELL_FLUID;
    s->pos = (double*)xcalloc(2 * fluidCount * s->ppc, sizeof(double));
    s->vel = (double*)xcalloc(2 * fluidCount * s->ppc, sizeof(double));
    float dist = 1.0f / s->ppcSqrt;
    size_t e = 0;
    for (int j = 0; j < s->NY; j++) {
        for (int i = 0; i < s->NX; i++) {
            if (s->cell[j * s->NX + i] == CELL_FLUID) {
                for (int k = 0; k < s->ppc; k++) {
                    int x = k % s->ppcSqrt;
                    int y = k / s->ppcSqrt;
                    double px = ((double)i + dist * x + randf(dist)) * s->dx;
                    double py = ((double)j + dist * y + randf(dist)) * s->dx;
                    s->pos[2 * e] = px;
                    s->pos[2 * e + 1] = py;
                    e++;
                }
            }
        }
    }
    s->np = e;
    s->waterVolume = fluidCount * s->dx * s->dx;
    s->origWaterVolume = s->waterVolume;
    return s;
}

void or_destroy(or_sim* s) {
    if (!s) return;
    free(s->cell); free(s->phi); free(s->p);
    free(s->u); free(s->v); free(s->nu); free(s->nv);
    free(s->pos); free(s->vel);
    free(s);
}

void or_set_options(or_sim* s, const or_options* opt) { s->opt = *opt; }

void or_set_params(or_sim* s, double gx, double gy, double alpha, double dt) {
    s->gx = gx; s->gy = gy; s->alpha = alpha; s->dt = dt;
}

/* ------------------------------------------------------------------ */
/* Level set (src/FluidSim2D.cpp:653-732,752-920)                     */
/* ------------------------------------------------------------------ */

/* LevelSet::constructFromParticles closest-point update, the body of the
 * fastSweepIterate lambda (src/FluidSim2D.cpp:775-792). */
static void closest_point_update(or_sim* s, int64_t* t, int i, int j) {
    const int il[4] = {i - 1, i + 1, i, i};
    const int jl[4] = {j, j, j - 1, j + 1};
    int NX = s->NX, NY = s->NY;
    double dx = s->dx;
    for (int k = 0; k < 4; k++) {
        if (il[k] < 0 || il[k] >= NX || jl[k] < 0 || jl[k] >= NY) continue;
        int64_t e = t[jl[k] * NX + il[k]];
        if (e != -1) {
            double px = s->pos[2 * e], py = s->pos[2 * e + 1];
            double d = sqrt((px - i * dx) * (px - i * dx) + (py - j * dx) * (py - j * dx)) - s->dr;
            if (d < s->phi[j * NX + i]) {
                s->phi[j * NX + i] = d;
                t[j * NX + i] = e;
            }
        }
    }
}

static void construct_from_particles(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    double dx = s->dx;
    int64_t* t = (int64_t*)xcalloc((size_t)NX * NY, sizeof(int64_t));
#pragma omp parallel for
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
            s->phi[j * NX + i] = HUGE_VAL;
            t[j * NX + i] = -1;
        }
    for (size_t e = 0; e < s->np; e++) {
        double px = s->pos[2 * e], py = s->pos[2 * e + 1];
        int x = (int)(px / dx), y = (int)(py / dx);
        double d = sqrt((px - x * dx) * (px - x * dx) + (py - y * dx) * (py - y * dx)) - s->dr;
        if (d < s->phi[y * NX + x]) {
            s->phi[y * NX + x] = d;
            t[y * NX + x] = (int64_t)e;
        }
    }
    /* LevelSet::fastSweepIterate (include/FluidSim2D.h:178-203) */
    for (int k = 0; k < 4; k++) {
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) closest_point_update(s, t, i, j);
        for (int j = 0; j < NY; j++)
            for (int i = NX; i-- > 0;) closest_point_update(s, t, i, j);
        for (int j = NY; j-- > 0;)
            for (int i = 0; i < NX; i++) closest_point_update(s, t, i, j);
        for (int j = NY; j-- > 0;)
            for (int i = NX; i-- > 0;) closest_point_update(s, t, i, j);
    }
    free(t);
}

/* One Eikonal update of LevelSet::redistance (src/FluidSim2D.cpp:848-857):
 * (ia, ja) and (ib, jb) are the two upwind neighbours of the sweep. */
static inline void eikonal_update(double* phi, int NX, double dx, int i, int j, int ia, int ja, int ib, int jb) {
    if (phi[j * NX + i] >= 0) return;
    double a = fabs(phi[ja * NX + ia]), b = fabs(phi[jb * NX + ib]);
    double phi0 = mind(a, b);
    double phi1 = maxd(a, b);
    double d = phi0 + dx;
    if (d > phi1) d = 0.5 * (phi0 + phi1 + sqrt(2 * dx * dx - (phi1 - phi0) * (phi1 - phi0)));
    if (d < -phi[j * NX + i]) phi[j * NX + i] = -d;
}

static void redistance(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    double dx = s->dx;
    double* phi = s->phi;
    uint8_t* isSurface = (uint8_t*)xcalloc((size_t)NX * NY, 1);
    double* oldPhi = (double*)xcalloc((size_t)NX * NY, sizeof(double));
    memcpy(oldPhi, phi, sizeof(double) * NX * NY);
    /* src/FluidSim2D.cpp:803-834.  The "correction" branches there assign
     * phi(i,j) its own old value, which changes nothing, so only the
     * surface flags are restated. */
    for (int j = 0; j < NY - 1; j++) {
        for (int i = 0; i < NX - 1; i++) {
            double phi0 = oldPhi[j * NX + i];
            double phi1 = oldPhi[j * NX + i + 1];
            double phi2 = oldPhi[(j + 1) * NX + i];
            if (phi0 * phi1 < 0) { isSurface[j * NX + i] = 1; isSurface[j * NX + i + 1] = 1; }
            if (phi0 * phi2 < 0) { isSurface[j * NX + i] = 1; isSurface[(j + 1) * NX + i] = 1; }
        }
    }
    for (int k = 0; k < NX * NY; k++)
        if (!isSurface[k] && phi[k] < 0) phi[k] = -HUGE_VAL;
    for (int k = 0; k < 4; k++) {
        for (int j = 1; j < NY; j++)
            for (int i = 1; i < NX; i++) eikonal_update(phi, NX, dx, i, j, i - 1, j, i, j - 1);
        for (int j = 1; j < NY; j++)
            for (int i = NX - 1; i-- > 0;) eikonal_update(phi, NX, dx, i, j, i + 1, j, i, j - 1);
        for (int j = NY - 1; j-- > 0;)
            for (int i = 1; i < NX; i++) eikonal_update(phi, NX, dx, i, j, i - 1, j, i, j + 1);
        for (int j = NY - 1; j-- > 0;)
            for (int i = NX - 1; i-- > 0;) eikonal_update(phi, NX, dx, i, j, i + 1, j, i, j + 1);
    }
    /* two min-smoothing passes (src/FluidSim2D.cpp:904-919) */
    for (int k = 0; k < 2; k++) {
        memcpy(oldPhi, phi, sizeof(double) * NX * NY);
#pragma omp parallel for
        for (int j = 1; j < NY - 1; j++) {
            for (int i = 1; i < NX - 1; i++) {
                double avg = 0.25 * (oldPhi[j * NX + i - 1] + oldPhi[j * NX + i + 1] + oldPhi[(j - 1) * NX + i] +
                                     oldPhi[(j + 1) * NX + i]);
                if (avg < oldPhi[j * NX + i]) phi[j * NX + i] = avg;
            }
        }
    }
    free(isSurface);
    free(oldPhi);
}

/* FluidSim2D::createWaterLevelSet with USE_LEVEL_SET (src/FluidSim2D.cpp:653-664,709-731) */
static void create_water_level_set(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    double dx = s->dx, rho = s->rho;
    construct_from_particles(s);
    redistance(s);
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++)
            if (s->cell[j * NX + i] != CELL_SOLID) s->cell[j * NX + i] = s->phi[j * NX + i] < 0.0 ? CELL_FLUID : CELL_EMPTY;
    s->waterVolume = 0.0;
    s->totalEnergy = 0.0;
    s->particleTotalEnergy = 0.0;
    for (int j = 0; j < NY; j++) {
        for (int i = 0; i < NX; i++) {
            if (s->cell[j * NX + i] == CELL_FLUID) {
                s->waterVolume += dx * dx;
                double vx = vel_interp_u(s, s->u, i * dx, j * dx);
                double vy = vel_interp_v(s, s->v, i * dx, j * dx);
                s->totalEnergy += 0.5 * (rho * dx * dx) * (vx * vx + vy * vy);
                s->totalEnergy -= (rho * dx * dx) * (s->gx * (i * dx) + s->gy * (j * dx));
            }
        }
    }
    for (size_t e = 0; e < s->np; e++) {
        double px = s->pos[2 * e], py = s->pos[2 * e + 1];
        double vx = s->vel[2 * e], vy = s->vel[2 * e + 1];
        s->particleTotalEnergy += 0.5 * (rho * dx * dx / (s->ppcSqrt * s->ppcSqrt)) * (vx * vx + vy * vy);
        s->particleTotalEnergy -= (rho * dx * dx / (s->ppcSqrt * s->ppcSqrt)) * (s->gx * px + s->gy * py);
    }
}

/* ------------------------------------------------------------------ */
/* Transfers and advection                                             */
/* ------------------------------------------------------------------ */

/* FluidSim2D::transferVelocityToGrid (src/FluidSim2D.cpp:144-204) */
static void transfer_velocity_to_grid(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    double dx = s->dx;
    size_t NU = (size_t)(NX + 1) * NY, NV = (size_t)NX * (NY + 1);
    memset(s->u, 0, NU * sizeof(double));
    memset(s->v, 0, NV * sizeof(double));
    double* udiv = (double*)xcalloc(NU, sizeof(double));
    double* vdiv = (double*)xcalloc(NV, sizeof(double));
    for (size_t e = 0; e < s->np; e++) {
        double xpx = s->pos[2 * e], xpy = s->pos[2 * e + 1];
        double upx = xpx / dx, upy = xpy / dx - 0.5;
        linear_distribute(s->u, NX + 1, NY, upx, upy, s->vel[2 * e]);
        linear_distribute(udiv, NX + 1, NY, upx, upy, 1.0);
        double vpx = xpx / dx - 0.5, vpy = xpy / dx;
        linear_distribute(s->v, NX, NY + 1, vpx, vpy, s->vel[2 * e + 1]);
        linear_distribute(vdiv, NX, NY + 1, vpx, vpy, 1.0);
    }
    for (size_t k = 0; k < NU; k++) if (udiv[k] > 0) s->u[k] /= udiv[k];
    for (size_t k = 0; k < NV; k++) if (vdiv[k] > 0) s->v[k] /= vdiv[k];
    uint32_t* uf = (uint32_t*)xcalloc(NU, sizeof(uint32_t));
    uint32_t* vf = (uint32_t*)xcalloc(NV, sizeof(uint32_t));
    for (size_t k = 0; k < NU; k++) uf[k] = s->u[k] == 0.0 ? MASK_UNKNOWN : 0;
    for (size_t k = 0; k < NV; k++) vf[k] = s->v[k] == 0.0 ? MASK_UNKNOWN : 0;
    or_extrapolate(s->u, NX + 1, NY, uf, s->opt.extrapolate_band);
    or_extrapolate(s->v, NX, NY + 1, vf, s->opt.extrapolate_band);
    free(udiv); free(vdiv); free(uf); free(vf);
}

/* One semi-Lagrangian backtrace (src/FluidSim2D.cpp:212-217): RK3 with
 * Ralston weights 2/9, 3/9, 4/9 through the velocity (su, sv). */
static void sl_backtrace(const or_sim* s, const double* su, const double* sv, double xpx, double xpy,
                         double* ox, double* oy) {
    double dt = s->dt;
    double k1x = vel_interp_u(s, su, xpx, xpy), k1y = vel_interp_v(s, sv, xpx, xpy);
    double ax = xpx - 0.5 * dt * k1x, ay = xpy - 0.5 * dt * k1y;
    double k2x = vel_interp_u(s, su, ax, ay), k2y = vel_interp_v(s, sv, ax, ay);
    double bx = xpx - 0.75 * dt * k2x, by = xpy - 0.75 * dt * k2y;
    double k3x = vel_interp_u(s, su, bx, by), k3y = vel_interp_v(s, sv, bx, by);
    double nx = xpx - ((2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x);
    double ny = xpy - ((2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y);
    clamp_pos(s, &nx, &ny);
    *ox = nx;
    *oy = ny;
}

/* FluidSim2D::applySemiLagrangianAdvection (src/FluidSim2D.cpp:206-235).
 * sl_inplace = 1 overwrites mac.u while later faces still read it, exactly
 * as the reference's serial loop does; sl_inplace = 0 reads the pre-step
 * velocity for every face (the GPU's semantics). */
static void apply_semi_lagrangian_advection(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    double dx = s->dx;
    size_t NU = (size_t)(NX + 1) * NY, NV = (size_t)NX * (NY + 1);
    if (s->opt.sl_inplace) {
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX + 1; i++) {
                double nx, ny;
                sl_backtrace(s, s->u, s->v, (double)i * dx, ((double)j + 0.5) * dx, &nx, &ny);
                s->u[j * (NX + 1) + i] = vel_interp_u(s, s->u, nx, ny);
            }
        for (int j = 0; j < NY + 1; j++)
            for (int i = 0; i < NX; i++) {
                double nx, ny;
                sl_backtrace(s, s->u, s->v, ((double)i + 0.5) * dx, (double)j * dx, &nx, &ny);
                s->v[j * NX + i] = vel_interp_v(s, s->v, nx, ny);
            }
        return;
    }
    double* u0 = (double*)xcalloc(NU, sizeof(double));
    double* v0 = (double*)xcalloc(NV, sizeof(double));
    memcpy(u0, s->u, NU * sizeof(double));
    memcpy(v0, s->v, NV * sizeof(double));
#pragma omp parallel for
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX + 1; i++) {
            double nx, ny;
            sl_backtrace(s, u0, v0, (double)i * dx, ((double)j + 0.5) * dx, &nx, &ny);
            s->u[j * (NX + 1) + i] = vel_interp_u(s, u0, nx, ny);
        }
#pragma omp parallel for
    for (int j = 0; j < NY + 1; j++)
        for (int i = 0; i < NX; i++) {
            double nx, ny;
            sl_backtrace(s, u0, v0, ((double)i + 0.5) * dx, (double)j * dx, &nx, &ny);
            s->v[j * NX + i] = vel_interp_v(s, v0, nx, ny);
        }
    free(u0);
    free(v0);
}

/* FluidSim2D::applyGravity (src/FluidSim2D.cpp:237-250) */
static void apply_gravity(or_sim* s) {
    int NX = s->NX, NY = s->NY;
#pragma omp parallel for
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX + 1; i++) s->u[j * (NX + 1) + i] += s->dt * s->gx;
#pragma omp parallel for
    for (int j = 0; j < NY + 1; j++)
        for (int i = 0; i < NX; i++) s->v[j * NX + i] += s->dt * s->gy;
}

/* ------------------------------------------------------------------ */
/* Pressure projection (src/FluidSim2D.cpp:252-467)                   */
/* ------------------------------------------------------------------ */

/* applyPreconditioner lambda (src/FluidSim2D.cpp:397-421): MIC(0) forward
 * substitution into q, then backward substitution into z. */
static void apply_preconditioner(int NX, int NY, const uint8_t* cell, const double* Ax, const double* Ay,
                                 const double* precon, const double* r, double* q, double* z) {
    memset(q, 0, sizeof(double) * NX * NY);
    for (int j = 1; j < NY; j++)
        for (int i = 1; i < NX; i++)
            if (cell[j * NX + i] == CELL_FLUID) {
                double t = r[j * NX + i] - Ax[j * NX + i - 1] * precon[j * NX + i - 1] * q[j * NX + i - 1] -
                           Ay[(j - 1) * NX + i] * precon[(j - 1) * NX + i] * q[(j - 1) * NX + i];
                q[j * NX + i] = t * precon[j * NX + i];
            }
    for (int j = NY - 1; j-- > 0;)
        for (int i = NX - 1; i-- > 0;)
            if (cell[j * NX + i] == CELL_FLUID) {
                double t = q[j * NX + i] - Ax[j * NX + i] * precon[j * NX + i] * z[j * NX + i + 1] -
                           Ay[j * NX + i] * precon[j * NX + i] * z[(j + 1) * NX + i];
                z[j * NX + i] = t * precon[j * NX + i];
            }
}

static void apply_projection(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    size_t N = (size_t)NX * NY;
    double dt = s->dt, dx = s->dx, rho = s->rho;
    const uint8_t* cell = s->cell;
    const double* phi = s->phi;
    double* Adiag = (double*)xcalloc(N, sizeof(double));
    double* Ax = (double*)xcalloc(N, sizeof(double));
    double* Ay = (double*)xcalloc(N, sizeof(double));
    double* rhs = (double*)xcalloc(N, sizeof(double));
    double* precon = (double*)xcalloc(N, sizeof(double));
    double* r = (double*)xcalloc(N, sizeof(double));
    double* z = (double*)xcalloc(N, sizeof(double));
    double* sv = (double*)xcalloc(N, sizeof(double));
    double* q = (double*)xcalloc(N, sizeof(double));

    /* matrix with ghost-fluid diagonal (USE_GHOST_PRESSURE, :261-303) */
    double scaleA = dt / (rho * dx * dx);
#pragma omp parallel for
    for (int j = 0; j < NY; j++) {
        for (int i = 0; i < NX; i++) {
            size_t c = (size_t)j * NX + i;
            if (cell[c] != CELL_FLUID) continue;
            double phi0 = phi[c];
            if (cell[c - 1] == CELL_FLUID) Adiag[c] += scaleA;
            else if (cell[c - 1] == CELL_EMPTY) Adiag[c] -= scaleA * maxd(phi[c - 1] / phi0, -1e3);
            if (cell[c + 1] == CELL_FLUID) { Adiag[c] += scaleA; Ax[c] = -scaleA; }
            else if (cell[c + 1] == CELL_EMPTY) Adiag[c] += scaleA * (1 - maxd(phi[c + 1] / phi0, -1e3));
            if (cell[c - NX] == CELL_FLUID) Adiag[c] += scaleA;
            else if (cell[c - NX] == CELL_EMPTY) Adiag[c] -= scaleA * maxd(phi[c - NX] / phi0, -1e3);
            if (cell[c + NX] == CELL_FLUID) { Adiag[c] += scaleA; Ay[c] = -scaleA; }
            else if (cell[c + NX] == CELL_EMPTY) Adiag[c] += scaleA * (1 - maxd(phi[c + NX] / phi0, -1e3));
        }
    }
    /* divergence right-hand side with solid-face terms (:337-362) */
    {
        double scale = 1.0 / dx;
        const double* u = s->u;
        const double* v = s->v;
#pragma omp parallel for
        for (int j = 0; j < NY; j++) {
            for (int i = 0; i < NX; i++) {
                size_t c = (size_t)j * NX + i;
                if (cell[c] != CELL_FLUID) continue;
                double u0 = u[j * (NX + 1) + i], u1 = u[j * (NX + 1) + i + 1];
                double v0 = v[j * NX + i], v1 = v[(j + 1) * NX + i];
                rhs[c] = -scale * (u1 - u0 + v1 - v0);
                if (cell[c - 1] == CELL_SOLID) rhs[c] -= scale * (u0 - 0);
                if (cell[c + 1] == CELL_SOLID) rhs[c] += scale * (u1 - 0);
                if (cell[c - NX] == CELL_SOLID) rhs[c] -= scale * (v0 - 0);
                if (cell[c + NX] == CELL_SOLID) rhs[c] += scale * (v1 - 0);
                /* volume correction (an option; not in the reference) */
                if (s->opt.volume_rate != 0.0 && s->waterVolume > 0.0)
                    rhs[c] += s->opt.volume_rate * ((s->origWaterVolume - s->waterVolume) / s->origWaterVolume) / s->dt;
            }
        }
    }
    /* MIC(0) factor (:364-387); the reference's OpenMP form of this loop races, so it stays serial */
    {
        double tau = s->opt.mic_tau, sigma = s->opt.mic_sigma;
        for (int j = 1; j < NY; j++)
            for (int i = 1; i < NX; i++) {
                size_t c = (size_t)j * NX + i;
                if (cell[c] != CELL_FLUID) continue;
                /* the reference's SQUARE(x) expands to (x)*(x) without outer
                 * parentheses, so a*b*SQUARE(p) associates as ((a*b)*p)*p */
                double e = Adiag[c] - (Ax[c - 1] * precon[c - 1]) * (Ax[c - 1] * precon[c - 1]) -
                           (Ay[c - NX] * precon[c - NX]) * (Ay[c - NX] * precon[c - NX]) -
                           tau * (Ax[c - 1] * Ay[c - 1] * precon[c - 1] * precon[c - 1] +
                                  Ay[c - NX] * Ax[c - NX] * precon[c - NX] * precon[c - NX]);
                if (e < sigma * Adiag[c]) e = Adiag[c];
                precon[c] = 1 / sqrt(e);
            }
    }
    /* PCG (:423-466) */
    memset(s->p, 0, N * sizeof(double));
    memcpy(r, rhs, N * sizeof(double));
    apply_preconditioner(NX, NY, cell, Ax, Ay, precon, r, q, z);
    memcpy(sv, z, N * sizeof(double));
    double sigma = inner_product(z, r, N);
    int maxIters = s->opt.pcg_max_iters;
    int iter = 0;
    double rhsNorm = infinite_norm(rhs, N);
    double rnorm = rhsNorm;
    while (iter < maxIters) {
#pragma omp parallel for
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) {
                size_t c = (size_t)j * NX + i;
                if (cell[c] == CELL_FLUID)
                    z[c] = Adiag[c] * sv[c] + Ax[c - 1] * sv[c - 1] + Ax[c] * sv[c + 1] + Ay[c - NX] * sv[c - NX] +
                           Ay[c] * sv[c + NX];
            }
        if (rhsNorm <= 1e-12) { rnorm = 0; break; }
        double alpha = sigma / inner_product(z, sv, N);
        for (size_t k = 0; k < N; k++) s->p[k] = s->p[k] + alpha * sv[k];
        for (size_t k = 0; k < N; k++) r[k] = r[k] + -alpha * z[k];
        rnorm = infinite_norm(r, N);
        if (rnorm <= s->opt.pcg_tol * rhsNorm) break;
        apply_preconditioner(NX, NY, cell, Ax, Ay, precon, r, q, z);
        double sigma_new = inner_product(z, r, N);
        double beta = sigma_new / sigma;
        for (size_t k = 0; k < N; k++) sv[k] = z[k] + beta * sv[k];
        sigma = sigma_new;
        iter++;
    }
    s->lastIters = iter;
    s->lastRelRes = rhsNorm > 0 ? rnorm / rhsNorm : 0;
    free(Adiag); free(Ax); free(Ay); free(rhs); free(precon);
    free(r); free(z); free(sv); free(q);
}

/* FluidSim2D::updateVelocity with USE_GHOST_PRESSURE (src/FluidSim2D.cpp:469-550) */
static void update_velocity(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    size_t NU = (size_t)(NX + 1) * NY, NV = (size_t)NX * (NY + 1);
    const uint8_t* cell = s->cell;
    const double* phi = s->phi;
    const double* p = s->p;
    uint32_t* du = (uint32_t*)xcalloc(NU, sizeof(uint32_t));
    uint32_t* dv = (uint32_t*)xcalloc(NV, sizeof(uint32_t));
    memcpy(s->nu, s->u, NU * sizeof(double));
    memcpy(s->nv, s->v, NV * sizeof(double));
    double scale = s->dt / (s->rho * s->dx);
#pragma omp parallel for
    for (int j = 0; j < NY; j++) {
        for (int i = 0; i < NX; i++) {
            size_t c = (size_t)j * NX + i;
            size_t fu = (size_t)j * (NX + 1) + i;
            size_t fv = c;
            if ((i > 0 && cell[c - 1] == CELL_FLUID) || cell[c] == CELL_FLUID) {
                if ((i == 0 || cell[c - 1] == CELL_SOLID) || cell[c] == CELL_SOLID) {
                    s->nu[fu] = 0;
                } else if (i > 0 && cell[c - 1] == CELL_EMPTY) {
                    double phi1 = phi[c - 1], phi0 = phi[c];
                    s->nu[fu] -= scale * (1 - maxd(phi1 / phi0, -1e3)) * p[c];
                } else if (cell[c] == CELL_EMPTY) {
                    double phi1 = phi[c], phi0 = phi[c - 1];
                    s->nu[fu] -= scale * (maxd(phi1 / phi0, -1e3) - 1) * p[c - 1];
                } else if (i > 0) {
                    s->nu[fu] -= scale * (p[c] - p[c - 1]);
                } else {
                    s->nu[fu] = 0;
                }
            } else {
                du[fu] = MASK_UNKNOWN;
            }
            if ((j > 0 && cell[c - NX] == CELL_FLUID) || cell[c] == CELL_FLUID) {
                if ((j == 0 || cell[c - NX] == CELL_SOLID) || cell[c] == CELL_SOLID) {
                    s->nv[fv] = 0;
                } else if (j > 0 && cell[c - NX] == CELL_EMPTY) {
                    double phi1 = phi[c - NX], phi0 = phi[c];
                    s->nv[fv] -= scale * (1 - maxd(phi1 / phi0, -1e3)) * p[c];
                } else if (cell[c] == CELL_EMPTY) {
                    double phi1 = phi[c], phi0 = phi[c - NX];
                    s->nv[fv] -= scale * (maxd(phi1 / phi0, -1e3) - 1) * p[c - NX];
                } else if (j > 0) {
                    s->nv[fv] -= scale * (p[c] - p[c - NX]);
                } else {
                    s->nv[fv] = 0;
                }
            } else {
                dv[fv] = MASK_UNKNOWN;
            }
        }
    }
    or_extrapolate(s->nu, NX + 1, NY, du, s->opt.extrapolate_band);
    or_extrapolate(s->nv, NX, NY + 1, dv, s->opt.extrapolate_band);
    if (s->mode == FS2D_SEMILAGRANGIAN) {
        memcpy(s->u, s->nu, NU * sizeof(double));
        memcpy(s->v, s->nv, NV * sizeof(double));
    }
    free(du);
    free(dv);
}

/* FluidSim2D::updateParticleVelocities (src/FluidSim2D.cpp:552-568) */
static void update_particle_velocities(or_sim* s) {
    int NX = s->NX, NY = s->NY;
    size_t NU = (size_t)(NX + 1) * NY, NV = (size_t)NX * (NY + 1);
    double dx = s->dx;
    double* uDiff = (double*)xcalloc(NU, sizeof(double));
    double* vDiff = (double*)xcalloc(NV, sizeof(double));
    for (size_t k = 0; k < NU; k++) uDiff[k] = s->nu[k] - s->u[k];
    for (size_t k = 0; k < NV; k++) vDiff[k] = s->nv[k] - s->v[k];
    double a = s->alpha;
#pragma omp parallel for
    for (long e = 0; e < (long)s->np; e++) {
        double px = s->pos[2 * e], py = s->pos[2 * e + 1];
        double upx = px / dx, upy = py / dx - 0.5;
        double vpx = px / dx - 0.5, vpy = py / dx;
        double picx = linear_extract(s->nu, NX + 1, NY, upx, upy);
        double picy = linear_extract(s->nv, NX, NY + 1, vpx, vpy);
        double flipx = s->vel[2 * e] + linear_extract(uDiff, NX + 1, NY, upx, upy);
        double flipy = s->vel[2 * e + 1] + linear_extract(vDiff, NX, NY + 1, vpx, vpy);
        s->vel[2 * e] = a * picx + (1 - a) * flipx;
        s->vel[2 * e + 1] = a * picy + (1 - a) * flipy;
    }
    memcpy(s->u, s->nu, NU * sizeof(double));
    memcpy(s->v, s->nv, NV * sizeof(double));
    free(uDiff);
    free(vDiff);
}

/* FluidSim2D::applyAdvection (src/FluidSim2D.cpp:570-604).  The reference
 * checks the pre-step position for NaN and exits; this returns 1 instead. */
static int apply_advection(or_sim* s) {
    double dt = s->dt;
    int bad = 0;
#pragma omp parallel for reduction(| : bad)
    for (long e = 0; e < (long)s->np; e++) {
        double px = s->pos[2 * e], py = s->pos[2 * e + 1];
        double k1x = vel_interp_u(s, s->u, px, py), k1y = vel_interp_v(s, s->v, px, py);
        double ax = px + 0.5 * dt * k1x, ay = py + 0.5 * dt * k1y;
        double k2x = vel_interp_u(s, s->u, ax, ay), k2y = vel_interp_v(s, s->v, ax, ay);
        double bx = px + 0.75 * dt * k2x, by = py + 0.75 * dt * k2y;
        double k3x = vel_interp_u(s, s->u, bx, by), k3y = vel_interp_v(s, s->v, bx, by);
        double nx = px + (2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x;
        double ny = py + (2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y;
        clamp_pos(s, &nx, &ny);
        if (isnan(px) || isnan(py)) bad |= 1;
        s->pos[2 * e] = nx;
        s->pos[2 * e + 1] = ny;
    }
    return bad;
}

/* ------------------------------------------------------------------ */
/* Frame / stage drivers                                              */
/* ------------------------------------------------------------------ */

/* ------------------------------------------------------------------ */
/* particle reseeding (an option; not in the reference)                */
/* ------------------------------------------------------------------ */

static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void or_reseed_jitter(unsigned seed, size_t c, unsigned m, double* jx, double* jy) {
    uint64_t key = (uint64_t)seed * 0x9E3779B97F4A7C15ull + (uint64_t)c * 0x100000001B3ull + (uint64_t)m;
    *jx = (double)(mix64(key) >> 11) * 0x1.0p-53;
    *jy = (double)(mix64(key ^ 0xD6E8FEB86659FD93ull) >> 11) * 0x1.0p-53;
}

static size_t particle_cell(const or_sim* s, double x, double y) {
    int i = clampi((int)(x / s->dx), 0, s->NX - 1), j = clampi((int)(y / s->dx), 0, s->NY - 1);
    return (size_t)j * s->NX + i;
}

void or_reseed(or_sim* s, int minPerCell, int maxPerCell, unsigned seed, size_t* out) {
    const int NX = s->NX, NY = s->NY;
    const size_t N = (size_t)NX * NY;
    uint32_t* cnt = (uint32_t*)xcalloc(N, sizeof(uint32_t));
    uint32_t* seen = (uint32_t*)xcalloc(N, sizeof(uint32_t));
    for (size_t e = 0; e < s->np; e++) cnt[particle_cell(s, s->pos[2 * e], s->pos[2 * e + 1])]++;
    size_t add = 0;
    for (size_t c = 0; c < N; c++)
        if (s->cell[c] == CELL_FLUID && cnt[c] < (uint32_t)minPerCell) add += (uint32_t)minPerCell - cnt[c];
    double* pos = (double*)xcalloc(2 * (s->np + add), sizeof(double));
    double* vel = (double*)xcalloc(2 * (s->np + add), sizeof(double));
    size_t n = 0, removed = 0;
    for (size_t e = 0; e < s->np; e++) {
        size_t c = particle_cell(s, s->pos[2 * e], s->pos[2 * e + 1]);
        if (maxPerCell > 0 && seen[c] >= (uint32_t)maxPerCell) {
            seen[c]++;
            removed++;
            continue;
        }
        seen[c]++;
        pos[2 * n] = s->pos[2 * e];
        pos[2 * n + 1] = s->pos[2 * e + 1];
        vel[2 * n] = s->vel[2 * e];
        vel[2 * n + 1] = s->vel[2 * e + 1];
        n++;
    }
    const double dx = s->dx;
    for (size_t c = 0; c < N; c++) {
        if (s->cell[c] != CELL_FLUID || cnt[c] >= (uint32_t)minPerCell) continue;
        const int i = (int)(c % NX), j = (int)(c / NX);
        for (unsigned m = 0; m < (uint32_t)minPerCell - cnt[c]; m++) {
            double jx, jy;
            or_reseed_jitter(seed, c, m, &jx, &jy);
            const double px = ((double)i + jx) * dx, py = ((double)j + jy) * dx;
            pos[2 * n] = px;
            pos[2 * n + 1] = py;
            vel[2 * n] = linear_extract(s->u, NX + 1, NY, px / dx, py / dx - 0.5);
            vel[2 * n + 1] = linear_extract(s->v, NX, NY + 1, px / dx - 0.5, py / dx);
            n++;
        }
    }
    free(s->pos);
    free(s->vel);
    s->pos = pos;
    s->vel = vel;
    s->np = n;
    free(cnt);
    free(seen);
    out[0] = removed;
    out[1] = add;
}

int or_run_stage(or_sim* s, int stage) {
    switch (stage) {
        case FS2D_STAGE_CREATE_WATER_LEVEL_SET: create_water_level_set(s); return 0;
        case FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID: transfer_velocity_to_grid(s); return 0;
        case FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION: apply_semi_lagrangian_advection(s); return 0;
        case FS2D_STAGE_APPLY_GRAVITY: apply_gravity(s); return 0;
        case FS2D_STAGE_CREATE_SOLID_LEVEL_SET: return 0; /* empty in the reference (:734-736) */
        case FS2D_STAGE_APPLY_PROJECTION: apply_projection(s); return 0;
        case FS2D_STAGE_UPDATE_VELOCITY: update_velocity(s); return 0;
        case FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES: update_particle_velocities(s); return 0;
        case FS2D_STAGE_APPLY_ADVECTION: return apply_advection(s) ? FS2D_ERR_NONFINITE : 0;
        default: return FS2D_ERR_INVALID;
    }
}

/* FluidSim2D::runFrame (src/FluidSim2D.cpp:94-138) */
int or_run_frame(or_sim* s) {
    static const int sl[] = {1, 3, 4, 5, 6, 7, 9};
    static const int pic[] = {1, 2, 4, 5, 6, 7, 8, 9};
    const int* st = s->mode == FS2D_SEMILAGRANGIAN ? sl : pic;
    int n = s->mode == FS2D_SEMILAGRANGIAN ? 7 : 8;
    int rc = 0;
    for (int k = 0; k < n; k++) {
        int r = or_run_stage(s, st[k]);
        if (r) rc = r;
    }
    s->currentTime += s->dt;
    return rc;
}

size_t or_num_particles(or_sim* s) { return s->np; }

int or_get_state(or_sim* s, fs2d_state* st) {
    size_t N = (size_t)s->NX * s->NY;
    size_t NU = (size_t)(s->NX + 1) * s->NY, NV = (size_t)s->NX * (s->NY + 1);
    if (st->cell) memcpy(st->cell, s->cell, N);
    if (st->phi) memcpy(st->phi, s->phi, N * sizeof(double));
    if (st->p) memcpy(st->p, s->p, N * sizeof(double));
    if (st->u) memcpy(st->u, s->u, NU * sizeof(double));
    if (st->v) memcpy(st->v, s->v, NV * sizeof(double));
    if (st->newU) memcpy(st->newU, s->nu, NU * sizeof(double));
    if (st->newV) memcpy(st->newV, s->nv, NV * sizeof(double));
    if (st->particles || st->particleVels) {
        if (st->numParticles < s->np) return FS2D_ERR_INVALID;
        if (st->particles) memcpy(st->particles, s->pos, 2 * s->np * sizeof(double));
        if (st->particleVels) memcpy(st->particleVels, s->vel, 2 * s->np * sizeof(double));
    }
    st->numParticles = s->np;
    return 0;
}

int or_set_state(or_sim* s, const fs2d_state* st) {
    size_t N = (size_t)s->NX * s->NY;
    size_t NU = (size_t)(s->NX + 1) * s->NY, NV = (size_t)s->NX * (s->NY + 1);
    if (st->cell) memcpy(s->cell, st->cell, N);
    if (st->phi) memcpy(s->phi, st->phi, N * sizeof(double));
    if (st->p) memcpy(s->p, st->p, N * sizeof(double));
    if (st->u) memcpy(s->u, st->u, NU * sizeof(double));
    if (st->v) memcpy(s->v, st->v, NV * sizeof(double));
    if (st->newU) memcpy(s->nu, st->newU, NU * sizeof(double));
    if (st->newV) memcpy(s->nv, st->newV, NV * sizeof(double));
    if (st->particles && st->particleVels) {
        free(s->pos);
        free(s->vel);
        s->np = st->numParticles;
        s->pos = (double*)xcalloc(2 * s->np, sizeof(double));
        s->vel = (double*)xcalloc(2 * s->np, sizeof(double));
        memcpy(s->pos, st->particles, 2 * s->np * sizeof(double));
        memcpy(s->vel, st->particleVels, 2 * s->np * sizeof(double));
    }
    return 0;
}

/* out: waterVolume, totalEnergy, particleTotalEnergy, avgPressure,
 * avgPressureInFluid, maxVelocity (src/FluidSim2D.cpp:607-638) */
void or_stats(or_sim* s, double* out) {
    int NX = s->NX, NY = s->NY;
    out[0] = s->waterVolume;
    out[1] = s->totalEnergy;
    out[2] = s->particleTotalEnergy;
    double avgP = 0.0;
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) avgP += s->p[j * NX + i];
    avgP /= (NX * NY);
    out[3] = avgP;
    double avgF = 0.0;
    size_t count = 0;
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++)
            if (s->cell[j * NX + i] == CELL_FLUID) { avgF += s->p[j * NX + i]; count++; }
    avgF /= count;
    out[4] = avgF;
    double maxVel = 0.0;
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++)
            if (s->cell[j * NX + i] == CELL_FLUID) {
                double x = (double)i * s->dx, y = (double)j * s->dx;
                double vx = vel_interp_u(s, s->u, x, y), vy = vel_interp_v(s, s->v, x, y);
                double vel = sqrt(vx * vx + vy * vy);
                if (vel > maxVel) maxVel = vel;
            }
    out[5] = maxVel;
}

void or_solver_info(or_sim* s, double* out) {
    out[0] = s->lastIters;
    out[1] = s->lastRelRes;
}
