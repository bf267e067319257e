/* The C ABI from plain C (include/fs2d.h): a closed-box rollout and its
 * gradient against a central difference, a batch of dam breaks against the
 * same scenes run alone (bit-identical states), and the batched rollout.
 * Prints "OK ..." and exits 0 when every check holds. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fs2d.h"

#define CHECK(call)                                                                     \
    do {                                                                                \
        int rc_ = (call);                                                               \
        if (rc_ != FS2D_OK) {                                                           \
            fprintf(stderr, "%s:%d %s -> %d: %s\n", __FILE__, __LINE__, #call, rc_,    \
                    fs2d_last_error());                                                 \
            return 1;                                                                   \
        }                                                                               \
    } while (0)

static uint8_t* labels(int n, double ex, double ey, int closed) {
    uint8_t* c = (uint8_t*)malloc((size_t)n * n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const double x = (i + 0.5) / n, y = (j + 0.5) / n;
            uint8_t v = (closed || (x < ex && y < ey)) ? FS2D_FLUID : FS2D_EMPTY;
            if (i == 0 || j == 0 || i == n - 1 || j == n - 1) v = FS2D_SOLID;
            c[(size_t)j * n + i] = v;
        }
    return c;
}

static fs2d_config config(int n, int mode, const uint8_t* cells) {
    fs2d_config cfg;
    cfg.sizeX = n;
    cfg.sizeY = n;
    cfg.particlesPerCellSqrt = 2;
    cfg.dt = mode == FS2D_PICFLIP ? (1.0 / 240) * (256.0 / n) : 1.0 / 60;
    cfg.dx = 1.0 / n;
    cfg.rho = 997.0;
    cfg.gravityX = 0.0;
    cfg.gravityY = mode == FS2D_PICFLIP ? -9.8 : 0.0;
    cfg.mode = mode;
    cfg.picFlipAlpha = 0.05;
    cfg.initialValues = cells;
    return cfg;
}

/* smooth seeded face field: a few plane waves */
static void field(double* a, int w, int h, double ox, double oy, double dx, unsigned seed) {
    srand(seed);
    double k[4][4];
    for (int m = 0; m < 4; m++)
        for (int q = 0; q < 4; q++) k[m][q] = (double)rand() / RAND_MAX;
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            const double x = (i + ox) * dx, y = (j + oy) * dx;
            double s = 0;
            for (int m = 0; m < 4; m++)
                s += (k[m][0] - 0.5) * sin(2 * M_PI * ((1 + m) * x + (1 + (m % 3)) * y) + 6.28 * k[m][1]);
            a[(size_t)j * w + i] = s;
        }
}

int main(void) {
    fs2d_options opt;
    fs2d_default_options(&opt);
    opt.use_seed = 1;
    opt.seed = 7;

    /* ---- rollout on a closed box ---- */
    const int n = 32, T = 6;
    const size_t NU = (size_t)(n + 1) * n, NV = (size_t)n * (n + 1);
    uint8_t* box = labels(n, 0, 0, 1);
    fs2d_config bc = config(n, FS2D_SEMILAGRANGIAN, box);
    fs2d_sim* sim = NULL;
    opt.pcg_tol = 1e-12;
    opt.pcg_max_iters = 1000;
    CHECK(fs2d_create(&bc, &opt, &sim));
    double *u0 = malloc(NU * 8), *v0 = malloc(NV * 8), *ut = malloc(NU * 8), *vt = malloc(NV * 8);
    double *gu = malloc(NU * 8), *gv = malloc(NV * 8), *du = malloc(NU * 8), *dv = malloc(NV * 8);
    double *up = malloc(NU * 8), *vp = malloc(NV * 8);
    field(u0, n + 1, n, 0.0, 0.5, 1.0 / n, 1);
    field(v0, n, n + 1, 0.5, 0.0, 1.0 / n, 2);
    field(ut, n + 1, n, 0.0, 0.5, 1.0 / n, 3);
    field(vt, n, n + 1, 0.5, 0.0, 1.0 / n, 4);
    double loss = 0;
    CHECK(fs2d_forward(sim, T, 0, u0, v0, ut, vt, &loss));
    CHECK(fs2d_backward(sim, gu, gv));
    srand(11);
    for (size_t k = 0; k < NU; k++) du[k] = (double)rand() / RAND_MAX - 0.5;
    for (size_t k = 0; k < NV; k++) dv[k] = (double)rand() / RAND_MAX - 0.5;
    const double eps = 1e-4;
    double lp = 0, lm = 0, ad = 0;
    for (size_t k = 0; k < NU; k++) up[k] = u0[k] + eps * du[k];
    for (size_t k = 0; k < NV; k++) vp[k] = v0[k] + eps * dv[k];
    CHECK(fs2d_forward(sim, T, 0, up, vp, ut, vt, &lp));
    for (size_t k = 0; k < NU; k++) up[k] = u0[k] - eps * du[k];
    for (size_t k = 0; k < NV; k++) vp[k] = v0[k] - eps * dv[k];
    CHECK(fs2d_forward(sim, T, 0, up, vp, ut, vt, &lm));
    for (size_t k = 0; k < NU; k++) ad += gu[k] * du[k];
    for (size_t k = 0; k < NV; k++) ad += gv[k] * dv[k];
    const double fd = (lp - lm) / (2 * eps);
    if (!(fabs(fd - ad) <= 1e-4 * fabs(ad))) {
        fprintf(stderr, "adjoint %.12g vs central difference %.12g\n", ad, fd);
        return 1;
    }
    CHECK(fs2d_destroy(sim));

    /* ---- batch of dam breaks vs the same scenes alone ---- */
    enum { NB = 3 };
    const int sides[NB] = {40, 56, 72};
    uint8_t* cells[NB];
    fs2d_config cfgs[NB];
    for (int k = 0; k < NB; k++) {
        cells[k] = labels(sides[k], 0.3 + 0.1 * k, 0.5, 0);
        cfgs[k] = config(sides[k], FS2D_PICFLIP, cells[k]);
    }
    fs2d_options bo;
    fs2d_default_options(&bo);
    bo.precision = FS2D_PRECISION_MIXED;
    bo.pcg_tol = 1e-6;
    bo.use_seed = 1;
    bo.seed = 100;
    fs2d_batch* b = NULL;
    CHECK(fs2d_batch_create(cfgs, NB, &bo, 2, &b));
    int rc = fs2d_batch_step(b, 3);
    if (rc != FS2D_OK && rc != FS2D_ERR_NOT_CONVERGED) {
        fprintf(stderr, "fs2d_batch_step -> %d: %s\n", rc, fs2d_last_error());
        return 1;
    }
    for (int k = 0; k < NB; k++) {
        const int s = sides[k];
        const size_t nu = (size_t)(s + 1) * s;
        fs2d_sim* in_batch = NULL;
        CHECK(fs2d_batch_scene(b, k, &in_batch));
        fs2d_options ok = bo;
        ok.seed = bo.seed + (unsigned)k;
        fs2d_sim* alone = NULL;
        CHECK(fs2d_create(&cfgs[k], &ok, &alone));
        rc = fs2d_step(alone, 3);
        if (rc != FS2D_OK && rc != FS2D_ERR_NOT_CONVERGED) return 1;
        double *ua = malloc(nu * 8), *ub = malloc(nu * 8);
        fs2d_state sa, sb;
        memset(&sa, 0, sizeof(sa));
        memset(&sb, 0, sizeof(sb));
        sa.u = ua;
        sb.u = ub;
        CHECK(fs2d_download_state(alone, &sa));
        CHECK(fs2d_download_state(in_batch, &sb));
        if (memcmp(ua, ub, nu * 8) != 0) {
            fprintf(stderr, "scene %d differs from the same scene run alone\n", k);
            return 1;
        }
        free(ua);
        free(ub);
        CHECK(fs2d_destroy(alone));
    }
    CHECK(fs2d_batch_destroy(b));

    printf("OK loss %.6f adjoint %.9g central difference %.9g\n", loss, ad, fd);
    return 0;
}
