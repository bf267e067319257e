/*
 * fs2d_oracle.h — CPU restatement of the reference FluidSim2D time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is checked
 * against: it is called by tests/, by __graft_entry__.smoke() as the checker
 * and by bench.py's CPU-baseline leg, never by the product.
 *
 * It restates src/FluidSim2D.cpp and include/Array2D.h of
 * lasagnaphil/fluid-sim in plain C, loop by loop and in the same floating
 * point operation order as the reference's scalar build (USE_AVX off),
 * so that, compiled with -ffp-contract=off, it reproduces the reference
 * bit for bit.  That equality is checked by tests/test_oracle_vs_reference.py
 * against the reference compiled from its own sources (oracle/_ref) and
 * against committed golden vectors made by that build (tests/golden/).
 *
 * It adds, as options, what the reference hard-codes: MIC(0) tau/sigma,
 * the PCG tolerance and iteration cap, and a double-buffered variant of the
 * in-place semi-Lagrangian advection (the order-independent semantics the
 * GPU implements).
 */
#ifndef FS2D_ORACLE_H
#define FS2D_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../../include/fs2d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_options {
    double mic_tau;        /* reference 0.999 */
    double mic_sigma;      /* reference 0.25 */
    double pcg_tol;        /* reference 1e-12 */
    int pcg_max_iters;     /* reference 200 */
    int sl_inplace;        /* 1: the reference's in-place advection; 0: double-buffered */
    int extrapolate_band;  /* 0: all BFS layers (reference); k > 0: layers <= k only */
    double volume_rate;    /* volume correction (not in the reference, which lists it as a TODO): 0 off;
                              r > 0 adds r * ((V0 - V) / V0) / dt to the projection's right-hand side of
                              every fluid cell (V the frame's waterVolume, V0 origWaterVolume) */
} or_options;

typedef struct or_sim or_sim;

void or_default_options(or_options* o);
or_sim* or_create(const fs2d_config* cfg, const or_options* opt, int use_seed, unsigned seed);
void or_destroy(or_sim* s);
void or_set_options(or_sim* s, const or_options* opt);
int or_run_frame(or_sim* s);
int or_run_stage(or_sim* s, int stage);
size_t or_num_particles(or_sim* s);
int or_get_state(or_sim* s, fs2d_state* st);
int or_set_state(or_sim* s, const fs2d_state* st);
/* out[0..5] = waterVolume, totalEnergy, particleTotalEnergy, avgPressure,
 *             avgPressureInFluid, maxVelocity */
void or_stats(or_sim* s, double* out);
/* out[0] = PCG iterations of the last solve, out[1] = ||r||inf/||b||inf at exit */
void or_solver_info(or_sim* s, double* out);
void or_set_params(or_sim* s, double gx, double gy, double alpha, double dt);

/* Particle reseeding (not in the reference, which lists it as a TODO):
 * particles counted per cell at (int)(x/dx), (int)(y/dx) clamped into the
 * grid; in every cell with more than maxPerCell (> 0) particles those after
 * the first maxPerCell in index order are removed; every FLUID cell with
 * fewer than minPerCell gets new particles up to minPerCell, in row-major
 * cell order, at ((i + jx) dx, (j + jy) dx) with jx, jy in [0, 1) from
 * or_reseed_jitter, and the bilinear grid velocity there (the PIC part of
 * updateParticleVelocities).  Survivors keep their order, new particles
 * follow.  out[0] = removed, out[1] = added. */
void or_reseed(or_sim* s, int minPerCell, int maxPerCell, unsigned seed, size_t* out);
/* the jitter of new particle m of cell c: bits of a 64-bit mix (splitmix64's
 * finaliser) of (seed, c, m), 53 of them scaled into [0, 1) */
void or_reseed_jitter(unsigned seed, size_t c, unsigned m, double* jx, double* jy);

/* Building blocks, exposed for unit tests. */
double or_tricubic(const double* data, int NX, int NY, double px, double py);
void or_extrapolate(double* data, int NX, int NY, uint32_t* mask, int band);

#ifdef __cplusplus
}
#endif

#endif
