// ref_capi.cpp — C wrapper around the UNMODIFIED reference simulator
// (test infrastructure: the oracle, never part of the product).
//
// Compiled together with the reference's own src/FluidSim2D.cpp and
// src/PerformanceCounter.cpp (read in place, never copied) and the
// altlib/altmath compatibility shim in oracle/shim/, into
// oracle/_ref/libfs2d_ref*.so.  It lets the tests create a reference
// FluidSim2D, overwrite or read its public fields, and run single stage
// methods or whole frames, so that every GPU stage can be compared with the
// reference on identical input state.
#include <cstring>
#include <cstdlib>
#include <new>
#include "FluidSim2D.h"
#include "../include/fs2d.h"

static_assert(sizeof(FluidSim2DConfig) == sizeof(fs2d_config), "config layout");
static_assert(sizeof(vec2d) == 2 * sizeof(double), "vec2d layout");

extern "C" {

// FluidSim2D::create (src/FluidSim2D.cpp:23-76); `use_seed` calls srand(seed)
// first so that libc rand() particle jitter is reproducible.
void* ref_create(const fs2d_config* cfg, int use_seed, unsigned seed) {
    FluidSim2DConfig c;
    std::memcpy(&c, cfg, sizeof(c));
    if (use_seed) srand(seed);
    FluidSim2D* sim = new (std::nothrow) FluidSim2D();
    if (!sim) return nullptr;
    *sim = FluidSim2D::create(c);
    return sim;
}

void ref_destroy(void* h) {
    FluidSim2D* sim = (FluidSim2D*)h;
    sim->free();
    delete sim;
}

void ref_run_frame(void* h) { ((FluidSim2D*)h)->runFrame(); }

// One stage method, by FluidSim2D::StageType value (include/FluidSim2D.h:93-97).
int ref_run_stage(void* h, int stage) {
    FluidSim2D* s = (FluidSim2D*)h;
    switch (stage) {
        case FS2D_STAGE_CREATE_WATER_LEVEL_SET: s->createWaterLevelSet(); return 0;
        case FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID: s->transferVelocityToGrid(); return 0;
        case FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION: s->applySemiLagrangianAdvection(); return 0;
        case FS2D_STAGE_APPLY_GRAVITY: s->applyGravity(); return 0;
        case FS2D_STAGE_CREATE_SOLID_LEVEL_SET: s->createSolidLevelSet(); return 0;
        case FS2D_STAGE_APPLY_PROJECTION: s->applyProjection(); return 0;
        case FS2D_STAGE_UPDATE_VELOCITY: s->updateVelocity(); return 0;
        case FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES: s->updateParticleVelocities(); return 0;
        case FS2D_STAGE_APPLY_ADVECTION: s->applyAdvection(); return 0;
        default: return 1;
    }
}

size_t ref_num_particles(void* h) { return ((FluidSim2D*)h)->particles.size; }

static void copy_out(double* dst, const Array2D<double>& a) {
    if (dst) std::memcpy(dst, a.data, sizeof(double) * (size_t)a.NX * a.NY);
}
static void copy_in(Array2D<double>& a, const double* src) {
    if (src) std::memcpy(a.data, src, sizeof(double) * (size_t)a.NX * a.NY);
}

int ref_get_state(void* h, fs2d_state* st) {
    FluidSim2D* s = (FluidSim2D*)h;
    size_t n = (size_t)s->sizeX * s->sizeY;
    if (st->cell) std::memcpy(st->cell, s->cell.data, n);
    copy_out(st->phi, s->waterLevelSet.phi);
    copy_out(st->p, s->p);
    copy_out(st->u, s->mac.u);
    copy_out(st->v, s->mac.v);
    copy_out(st->newU, s->newMac.u);
    copy_out(st->newV, s->newMac.v);
    if (st->particles || st->particleVels) {
        if (st->numParticles < s->particles.size) return 1;
        if (st->particles) std::memcpy(st->particles, s->particles.data, sizeof(vec2d) * s->particles.size);
        if (st->particleVels) std::memcpy(st->particleVels, s->particleVels.data, sizeof(vec2d) * s->particles.size);
    }
    st->numParticles = s->particles.size;
    return 0;
}

int ref_set_state(void* h, const fs2d_state* st) {
    FluidSim2D* s = (FluidSim2D*)h;
    size_t n = (size_t)s->sizeX * s->sizeY;
    if (st->cell) std::memcpy(s->cell.data, st->cell, n);
    copy_in(s->waterLevelSet.phi, st->phi);
    copy_in(s->p, st->p);
    copy_in(s->mac.u, st->u);
    copy_in(s->mac.v, st->v);
    copy_in(s->newMac.u, st->newU);
    copy_in(s->newMac.v, st->newV);
    if (st->particles && st->particleVels) {
        s->particles.resize(st->numParticles);
        s->particleVels.resize(st->numParticles);
        std::memcpy(s->particles.data, st->particles, sizeof(vec2d) * st->numParticles);
        std::memcpy(s->particleVels.data, st->particleVels, sizeof(vec2d) * st->numParticles);
    }
    return 0;
}

// out[0..5] = waterVolume, totalEnergy, particleTotalEnergy, avgPressure,
//             avgPressureInFluid, maxVelocity (src/FluidSim2D.cpp:607-638,709-731)
void ref_stats(void* h, double* out) {
    FluidSim2D* s = (FluidSim2D*)h;
    out[0] = s->waterVolume;
    out[1] = s->totalEnergy;
    out[2] = s->particleTotalEnergy;
    out[3] = s->avgPressure();
    out[4] = s->avgPressureInFluid();
    out[5] = s->maxVelocity();
}

void ref_set_gravity(void* h, double gx, double gy) { ((FluidSim2D*)h)->gravity = vec2d{gx, gy}; }

void ref_save_stats(void* h) { ((FluidSim2D*)h)->saveStats(); }

// Feeds given series through the reference's own statistics code: each of
// `nframes` rows of stage times goes into perfCounter.samples for the
// current frame followed by PerformanceCounter::endFrame
// (src/PerformanceCounter.cpp:39-56), and the conservation series are
// appended to waterVolumeData / totalEnergyData / particleTotalEnergyData,
// so that ref_save_stats then writes what the reference writes for them.
void ref_feed_stats(void* h, const float* stage_ms, int nframes, const double* vol, const double* en,
                    const double* pen, int n) {
    FluidSim2D* s = (FluidSim2D*)h;
    PerformanceCounter& pc = s->perfCounter;
    const int ns = (int)pc.samples.size;
    for (int f = 0; f < nframes; f++) {
        for (int k = 0; k < ns; k++) pc.samples[k][pc.currentFrame] = stage_ms[(size_t)f * ns + k];
        pc.endFrame();
    }
    for (int k = 0; k < n; k++) {
        s->waterVolumeData.push(vol[k]);
        s->totalEnergyData.push(en[k]);
        s->particleTotalEnergyData.push(pen[k]);
    }
}

int ref_num_stages(void* h) { return (int)((FluidSim2D*)h)->perfCounter.samples.size; }

}  // extern "C"
