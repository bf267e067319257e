/*
 * fs2d.h — C ABI of the GB300 FluidSim2D time step.
 *
 * This is the drop-in boundary for the reference simulator's per-frame step
 * (lasagnaphil/fluid-sim, `FluidSim2D` in include/FluidSim2D.h and
 * src/FluidSim2D.cpp).  Every entry point is `extern "C"`, takes plain
 * pointers and sizes, never throws, and returns an `int` status (FS2D_OK = 0).
 * All simulation work runs as CUDA kernels on one GPU, on the stream the
 * handle owns (or the one given to fs2d_set_stream).  There is no CPU
 * fallback: if no CUDA device is usable, fs2d_create fails with
 * FS2D_ERR_CUDA.
 *
 * Threading: a handle is used by one host thread at a time; different
 * handles may be used from different threads at once.  The library starts
 * host threads only inside fs2d_batch_step and joins them before returning.
 *
 * Layout conventions follow the reference exactly:
 *   - grids are row-major, element (i, j) at index j*NX + i
 *     (Array2D::operator(), include/Array2D.h:41-49);
 *   - the MAC grid stores u with (sizeX+1) x sizeY faces and v with
 *     sizeX x (sizeY+1) faces (MACGrid2D::create, include/MACGrid2D.h:19-25);
 *   - particles are interleaved (x, y) doubles, one vec2d per particle
 *     (FluidSim2D::particles, include/FluidSim2D.h:75-76);
 *   - cell labels are one byte: 0 EMPTY, 1 FLUID, 2 SOLID
 *     (FluidCellType, include/FluidSim2D.h:44-46).
 */
#ifndef FS2D_H
#define FS2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference exits or logs instead, src/FluidSim2D.cpp:464-466,598-601) ---- */
#define FS2D_OK                 0
#define FS2D_ERR_INVALID        1  /* bad argument or configuration */
#define FS2D_ERR_ALLOC          2  /* device or pinned-host allocation failed */
#define FS2D_ERR_CUDA           3  /* a CUDA runtime call or kernel launch failed */
#define FS2D_ERR_NOT_CONVERGED  4  /* PCG hit its iteration cap (the frame still completes) */
#define FS2D_ERR_NONFINITE      5  /* a NaN/Inf particle position was produced */
#define FS2D_ERR_TIMEOUT        6  /* a wavefront kernel gave up waiting on a neighbour tile */

/* ---- cell labels: FluidCellType, include/FluidSim2D.h:44-46 ---- */
#define FS2D_EMPTY 0
#define FS2D_FLUID 1
#define FS2D_SOLID 2

/* ---- modes: FluidSimMode, include/FluidSim2D.h:40-42 ---- */
#define FS2D_SEMILAGRANGIAN 0
#define FS2D_PICFLIP        1

/* ---- stage ids: FluidSim2D::StageType, include/FluidSim2D.h:93-97 ---- */
#define FS2D_STAGE_INIT                            0
#define FS2D_STAGE_CREATE_WATER_LEVEL_SET          1
#define FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID       2
#define FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION 3
#define FS2D_STAGE_APPLY_GRAVITY                   4
#define FS2D_STAGE_CREATE_SOLID_LEVEL_SET          5
#define FS2D_STAGE_APPLY_PROJECTION                6
#define FS2D_STAGE_UPDATE_VELOCITY                 7
#define FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES      8
#define FS2D_STAGE_APPLY_ADVECTION                 9

/* ---- precision of the device path ---- */
#define FS2D_PRECISION_FP64  0  /* every stage in FP64 with the reference's operation order */
#define FS2D_PRECISION_MIXED 1  /* FP32 SpMV/preconditioner/vector updates, FP64-accurate dot
                                   products, FP64 outer iterative-refinement residual and
                                   stopping test */
#define FS2D_PRECISION_FP32  2  /* plain FP32 PCG: FP32 SpMV, preconditioner, vector updates and
                                   dot products, one solve to pcg_tol on the FP32 residual, no
                                   refinement; the FP64 residual is reported */

/* ---- P2G accumulation ---- */
#define FS2D_P2G_ORDERED 0  /* per-face sums in particle-index order: reproducible, matches the reference */
#define FS2D_P2G_ATOMIC  1  /* warp-aggregated atomics: fastest, order not reproducible */

/*
 * Scene configuration.  Byte-compatible with FluidSim2DConfig
 * (include/FluidSim2D.h:48-63): same fields, same order, same types
 * (`mode` is the FluidSimMode enum, an int; `initialValues` is the
 * caller-owned FluidCellType array, copied at create time as the reference
 * does at src/FluidSim2D.cpp:47).
 */
typedef struct fs2d_config {
    int sizeX;
    int sizeY;
    int particlesPerCellSqrt;
    double dt;
    double dx;
    double rho;
    double gravityX;
    double gravityY;
    int mode;
    double picFlipAlpha;   /* weight of the PIC velocity: v = a*pic + (1-a)*flip (src/FluidSim2D.cpp:564) */
    const uint8_t* initialValues;
} fs2d_config;

/*
 * Options the reference hard-codes (src/FluidSim2D.cpp:369-370,429,447-453).
 * fs2d_default_options fills in the reference's values.
 */
typedef struct fs2d_options {
    int precision;          /* FS2D_PRECISION_*; default FP64 */
    double mic_tau;         /* MIC(0) modification parameter; reference 0.999 */
    double mic_sigma;       /* MIC(0) safety parameter; reference 0.25 */
    double pcg_tol;         /* stop when ||r||inf <= tol * ||b||inf; reference 1e-12 */
    int pcg_max_iters;      /* reference 200 */
    double ir_inner_tol;    /* MIXED only: tightest relative tolerance of an FP32 inner solve (a sweep that
                               only needs a smaller reduction stops earlier); default 1e-4 */
    int ir_max_outer;       /* MIXED only: cap on refinement sweeps; default 30 */
    int p2g_mode;           /* FS2D_P2G_*; default ORDERED */
    int extrapolate_band;   /* 0 = every BFS layer (the reference); k > 0 = layers <= k only */
    int use_seed;           /* 1: srand(seed) before seeding particles; 0: use libc rand() as it stands,
                               exactly like the reference's create (src/FluidSim2D.cpp:19-21,52-64) */
    unsigned int seed;
    int device;             /* CUDA device ordinal; default 0 */
} fs2d_options;

/*
 * A view of caller-owned host buffers holding the full simulation state.
 * Any pointer may be NULL, in which case that field is skipped.
 */
typedef struct fs2d_state {
    uint8_t* cell;          /* sizeX*sizeY labels */
    double* phi;            /* sizeX*sizeY water level set (negative inside) */
    double* p;              /* sizeX*sizeY pressure */
    double* u;              /* (sizeX+1)*sizeY  mac.u */
    double* v;              /* sizeX*(sizeY+1)  mac.v */
    double* newU;           /* (sizeX+1)*sizeY  newMac.u */
    double* newV;           /* sizeX*(sizeY+1)  newMac.v */
    double* particles;      /* 2*numParticles interleaved (x, y) */
    double* particleVels;   /* 2*numParticles interleaved (vx, vy) */
    size_t numParticles;    /* on upload: particle count to install; on download: capacity check */
} fs2d_state;

/* Per-frame conservation statistics and solver diagnostics. */
typedef struct fs2d_stats {
    double waterVolume;          /* src/FluidSim2D.cpp:709-716 */
    double totalEnergy;          /* src/FluidSim2D.cpp:717-719 */
    double particleTotalEnergy;  /* src/FluidSim2D.cpp:723-728 */
    double origWaterVolume;      /* src/FluidSim2D.cpp:71-72 */
    double currentTime;          /* src/FluidSim2D.cpp:135 */
    long long frames;            /* frames run so far */
    int pcgIterations;           /* iterations of the last pressure solve (sum over refinement sweeps) */
    int irOuterIterations;       /* MIXED: refinement sweeps of the last solve; FP64: 0 */
    double pcgRelResidual;       /* ||r||inf / ||b||inf at exit of the last solve (FP64 residual) */
    int lastStatus;              /* status of the last frame or standalone pressure solve */
} fs2d_stats;

typedef struct fs2d_sim fs2d_sim;

/* Fills `opt` with the reference's hard-coded values (FP64, tau 0.999, sigma 0.25,
 * tol 1e-12, 200 iterations, ordered P2G, exact extrapolation). */
void fs2d_default_options(fs2d_options* opt);

/* FluidSim2D::create (include/FluidSim2D.h:116, src/FluidSim2D.cpp:23-76).
 * Seeds particles on the host with libc rand() exactly as the reference does,
 * then uploads the state.  The border cells of initialValues must be SOLID
 * (the reference reads outside its arrays otherwise).  `opt` may be NULL. */
int fs2d_create(const fs2d_config* cfg, const fs2d_options* opt, fs2d_sim** out);

/* FluidSim2D::free (include/FluidSim2D.h:118, src/FluidSim2D.cpp:78-92). */
int fs2d_destroy(fs2d_sim* sim);

/* FluidSim2D::runFrame / update (include/FluidSim2D.h:120-122, src/FluidSim2D.cpp:94-142).
 * Enqueues the frame's kernels; returns after the frame's device work
 * completed.  Returns FS2D_ERR_NOT_CONVERGED if the pressure solve hit its
 * cap (the reference logs and continues; so does this call). */
int fs2d_run_frame(fs2d_sim* sim);

/* The pressure solve alone (applyProjection, src/FluidSim2D.cpp:252-467) on
 * caller-supplied host arrays: labels `cell` and level set `phi`
 * (sizeX*sizeY), face velocities `u` ((sizeX+1)*sizeY) and `v`
 * (sizeX*(sizeY+1)).  They replace the handle's fields; the matrix and
 * right-hand side are built as the reference builds them, the system is
 * solved with the handle's precision and stopping rule, and the pressure is
 * written to `pressure` (sizeX*sizeY).  `stats` (may be NULL) receives the
 * iteration count and final relative residual.  Returns
 * FS2D_ERR_NOT_CONVERGED (with the last iterate in `pressure`) when the
 * iteration cap was reached. */
int fs2d_solve_pressure(fs2d_sim* sim, const uint8_t* cell, const double* phi, const double* u, const double* v,
                        double* pressure, fs2d_stats* stats);

/* Differentiable rollout.  No reference counterpart: the reference has no
 * derivatives.  The forward pass is the semi-Lagrangian frame's velocity
 * stages (applySemiLagrangianAdvection, applyGravity, applyProjection with
 * the handle's precision and tolerance, updateVelocity;
 * src/FluidSim2D.cpp:100-113) repeated `steps` times
 * from the face velocities (u0, v0), on the handle's fixed labels, which may
 * hold no EMPTY cell (a closed box: the projection is then a fixed linear
 * map).  The loss is the L2 distance sqrt(sum (u_T - uTarget)^2 +
 * sum (v_T - vTarget)^2) over all faces.  The state before every
 * `checkpointEvery`-th step is kept (0: ceil(sqrt(steps))).
 *
 * fs2d_backward then writes dL/du_0 and dL/dv_0 (reverse mode, hand-written
 * adjoint kernels), recomputing each segment from its checkpoint.  The
 * handle's u and v afterwards hold an intermediate state.  All pointers may
 * be host or device memory; sizes are the handle's face grids.
 * FS2D_ERR_INVALID for a mode other than FS2D_SEMILAGRANGIAN or a scene with
 * an EMPTY cell; FS2D_ERR_NOT_CONVERGED if a pressure solve hit its cap. */
int fs2d_forward(fs2d_sim* sim, int steps, int checkpointEvery, const double* u0, const double* v0,
                 const double* uTarget, const double* vTarget, double* loss);
int fs2d_backward(fs2d_sim* sim, double* gradU0, double* gradV0);

/* Transposes of the particle transfers, for reverse-mode use with the
 * particle positions held fixed (no reference counterpart).  Both act at the
 * handle's current particle positions.
 *
 * fs2d_p2g_adjoint: transferVelocityToGrid (src/FluidSim2D.cpp:144-204) maps
 * the particle velocities linearly to the face velocities (bilinear splat,
 * division by the summed weights, extrapolation of the unknown faces).  Call
 * it after that stage ran on the current positions (it uses the stage's
 * known/unknown masks); (uBar, vBar), adjoints of the face grids, give
 * particleVelsBar (2 per particle, interleaved).
 *
 * fs2d_g2p_adjoint: updateParticleVelocities (:552-568) maps (newMac, mac,
 * particle velocities) linearly to the new particle velocities; the adjoint
 * of the new velocities gives the adjoints of newMac (newUBar, newVBar), of
 * mac (uBar, vBar) and of the old velocities (particleVelsInBar).
 *
 * Pointers may be host or device memory; scratch is allocated with
 * cudaMalloc for the duration of the call. */
int fs2d_p2g_adjoint(fs2d_sim* sim, const double* uBar, const double* vBar, double* particleVelsBar);
int fs2d_g2p_adjoint(fs2d_sim* sim, const double* particleVelsBar, double* newUBar, double* newVBar, double* uBar,
                     double* vBar, double* particleVelsInBar);

/* Batches of independent scenes.  No reference counterpart (the reference
 * runs one scene per process).  fs2d_batch_create makes one handle per
 * scene (cfgs[k], all with the options `opt`, which may be NULL; with
 * use_seed, scene k is seeded with seed + k) in order, each on its own CUDA
 * stream.  fs2d_batch_step advances every scene by `nframes` frames
 * (fs2d_run_frame each) with `workers` host threads issuing the scenes'
 * frames concurrently, scenes assigned longest-first to the least-loaded
 * thread; workers = 0 lets the first frames choose the count (one frame
 * timed per candidate; those are ordinary frames of the run).  A scene's
 * results do not depend on the worker count.  fs2d_batch_step starts and
 * joins its threads within the call; it returns the first error, or
 * FS2D_ERR_NOT_CONVERGED if a scene's last pressure solve hit its cap.
 * At most min(scenes, 64) workers are used.
 * fs2d_batch_scene gives scene k's handle for the per-scene calls (state,
 * statistics); do not destroy it or use it during fs2d_batch_step. */
typedef struct fs2d_batch fs2d_batch;
int fs2d_batch_create(const fs2d_config* cfgs, int n, const fs2d_options* opt, int workers, fs2d_batch** out);
int fs2d_batch_step(fs2d_batch* batch, int nframes);
int fs2d_batch_size(fs2d_batch* batch, int* n);
int fs2d_batch_scene(fs2d_batch* batch, int k, fs2d_sim** sim);
int fs2d_batch_workers(fs2d_batch* batch, int* workers);   /* 0 until chosen */
int fs2d_batch_set_workers(fs2d_batch* batch, int workers); /* 0: choose again on the next frames */
int fs2d_batch_destroy(fs2d_batch* batch);
/* Kernels launched so far by the batch and its scenes. */
int fs2d_batch_launch_count(fs2d_batch* batch, unsigned long long* out);
/* Mixed precision: the batch solves every scene's pressure system together
 * (one launch per kernel of the inner solve for all scenes; the FP32 MIC(0)
 * sweeps as persistent CTAs over work items of one strip of 128 columns of
 * one scene).  fs2d_batch_create times candidate schedules and CTA counts
 * on forward sweeps and keeps the fastest (schedules 0-2 list whole scenes:
 * as given, by decreasing rows, by decreasing cells; schedule 3 lists every
 * scene's first strip, then every second strip, ...); this reports the
 * choice, the number of work items and the chosen sweep's time (schedule -1
 * for an FP64 batch).  Any pointer may be NULL. */
int fs2d_batch_sweep_schedule(fs2d_batch* batch, int* schedule, int* ctas, int* items, double* sweepUs);
/* Overrides the autotuner: schedule 0..4 and, ctas > 0, the number of
 * persistent CTAs (at most the SM count).  A scene's results do not depend on
 * either. */
int fs2d_batch_set_schedule(fs2d_batch* batch, int schedule, int ctas);
/* Milliseconds of the frames of the last fs2d_batch_step of a
 * mixed-precision batch, summed over its frames (zeros for an FP64 batch),
 * four values: host wall clock of ms[0] the scenes' stages up to their
 * pressure solves, ms[1] the batch's joint pressure solve, ms[2] the
 * remaining stages; ms[3] the device time of the level-set sweeps of all
 * scenes (part of ms[0]). */
int fs2d_batch_phase_ms(fs2d_batch* batch, double* ms);
/* Per-scene work between the batch's joint steps (a mixed-precision batch):
 * on (default), each scene's three phases of a frame are captured into CUDA
 * graphs on their second frame and replayed after (captured again when the
 * scene's state or parameters change); off, launched directly.  Results do
 * not depend on it. */
int fs2d_batch_set_graphs(fs2d_batch* batch, int on);
/* fs2d_forward / fs2d_backward for every scene of a batch (each a closed box:
 * no EMPTY cell, semi-Lagrangian mode), scenes issued concurrently by the
 * batch's workers (all hardware threads up to 16 while the count is not
 * chosen).  Arrays of per-scene pointers (host or device memory, scene k's
 * face grids); losses[k] receives scene k's loss.  Returns the first error. */
int fs2d_batch_forward(fs2d_batch* batch, int steps, int checkpointEvery, const double* const* u0,
                       const double* const* v0, const double* const* uTarget, const double* const* vTarget,
                       double* losses);
int fs2d_batch_backward(fs2d_batch* batch, double* const* gradU0, double* const* gradV0);

/* Runs `nframes` frames back to back without host synchronisation between them
 * (except the pressure solver's convergence polls). */
int fs2d_step(fs2d_sim* sim, int nframes);

/* Runs one stage method (createWaterLevelSet, transferVelocityToGrid, ...;
 * include/FluidSim2D.h:124-140) on the current device state. */
int fs2d_run_stage(fs2d_sim* sim, int stage);

/* Array2D::extrapolate (include/Array2D.h:552-591) on caller-owned DEVICE
 * buffers: `values` holds width*height doubles, `mask` width*height uint32
 * (0 = known, nonzero = unknown).  Every unknown face at breadth-first layer
 * L (its 4-connected grid distance to the nearest known face) becomes the
 * mean of its neighbours of lower layer, as in the reference; `mask` is left
 * holding the layers, as the reference leaves its intMask.  band > 0 stops
 * after that many layers.  Runs on `stream` (NULL: the default stream) and
 * returns after the work completed.  Allocates 4 bytes of scratch per face
 * with cudaMalloc for the duration of the call. */
int fs2d_extrapolate(double* values, uint32_t* mask, int width, int height, int band, void* stream);

/* fs2d_extrapolate for callers that cannot allocate device memory — code
 * that must run on the buffers it is handed, such as a plugin living inside
 * a host application's own memory pool.  No reference counterpart: the
 * reference allocates its BFS queue on the host per call.  Same arguments
 * and results as fs2d_extrapolate, but no cudaMalloc, cudaFree or other
 * allocating call: the scratch is one static device array of 8 MiB + 24 KiB
 * (FS2D_NOALLOC_MAX_FACES faces, each side at most FS2D_NOALLOC_MAX_SIDE),
 * which every GPU that loads the library holds until the process exits.
 * Larger grids are rejected with FS2D_ERR_INVALID.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.
 * Every call shares the one array, so calls that overlap on the GPU (other
 * streams, other host threads) race; each call initialises what it reads
 * and returns after its work completed. */
#define FS2D_NOALLOC_MAX_FACES 2097152
#define FS2D_NOALLOC_MAX_SIDE 8192
int fs2d_extrapolate_noalloc(double* values, uint32_t* mask, int width, int height, int band, void* stream);

/* Host <-> device state transfer (the reference's public fields). */
int fs2d_upload_state(fs2d_sim* sim, const fs2d_state* st);
int fs2d_download_state(fs2d_sim* sim, fs2d_state* st);
int fs2d_num_particles(fs2d_sim* sim, size_t* n);

/* The fields a caller may change between frames (FluidSim2D::gravity,
 * picFlipAlpha, dt; written by demo/FluidRenderer2D.cpp:322,388). */
int fs2d_set_params(fs2d_sim* sim, double gravityX, double gravityY, double picFlipAlpha, double dt);

/* Statistics of the last frame, and the per-frame conservation series
 * (waterVolumeData, totalEnergyData, particleTotalEnergyData;
 * include/FluidSim2D.h:106-114).  `history` copies up to `cap` frames into
 * each non-NULL array and stores the frame count in *n. */
int fs2d_get_stats(fs2d_sim* sim, fs2d_stats* out);
int fs2d_get_history(fs2d_sim* sim, double* volume, double* energy, double* particleEnergy,
                     size_t cap, size_t* n);

/* Diagnostics (src/FluidSim2D.cpp:607-638): device reductions. */
int fs2d_avg_pressure(fs2d_sim* sim, double* out);
int fs2d_avg_pressure_in_fluid(fs2d_sim* sim, double* out);
int fs2d_max_velocity(fs2d_sim* sim, double* out);
/* The CFL check of applyAdvection (src/FluidSim2D.cpp:571-585), which the
 * reference only logs when it exceeds 5: over the particles, the largest
 * c = (vx + vy) * dt / dx above 0 (the reference's expression, without
 * absolute values; NaN never counts) and the first particle reaching it;
 * *cfl = 0 and *particle = -1 when no particle has c > 0.  Either pointer
 * may be NULL. */
int fs2d_cfl(fs2d_sim* sim, double* cfl, long long* particle);

/* Checkpoint and resume (no reference counterpart: the reference keeps no
 * state on disk).  fs2d_save_checkpoint writes the handle's whole state to
 * one binary file: a header (magic "FS2DCKP1", version, grid, mode,
 * particle count, frame count, time, dt, dx, rho, gravity, picFlipAlpha,
 * the volume at creation and the current water volume, the volume
 * correction rate), then cell, phi, p, u, v, newU, newV, particles and
 * particleVels in the layouts of fs2d_state, in host byte order.
 * fs2d_load_checkpoint restores it into a handle of the same grid, mode, dx
 * and rho (FS2D_ERR_INVALID otherwise, or for a file that is not a complete
 * checkpoint); frames after a resume are the frames the saved handle would
 * have run, bit for bit on the reproducible paths.  The statistics history
 * (fs2d_get_history) is not part of the file. */
int fs2d_save_checkpoint(fs2d_sim* sim, const char* path);
int fs2d_load_checkpoint(fs2d_sim* sim, const char* path);

/* Per-stage device times (ms, CUDA events) of the last frame, in the
 * reference's stage order (src/FluidSim2D.cpp:100-133); *n = stage count
 * (7 semi-Lagrangian, 8 PIC/FLIP). */
int fs2d_get_stage_times(fs2d_sim* sim, float* ms, int cap, int* n);

/* FluidSim2D::saveStats (src/FluidSim2D.cpp:738-750,
 * src/PerformanceCounter.cpp:58-74): writes perf and conservation CSV files
 * in the reference's formats.  Either path may be NULL to skip that file. */
int fs2d_save_stats(fs2d_sim* sim, const char* perfPath, const char* conservationPath);

/* The formatting of fs2d_save_stats applied to caller-supplied series, on
 * the host only (no device work; usable without a GPU): `stageMs` holds
 * `frames` rows of `numStages` stage times (ms), fed through the
 * reference's 30-frame PerformanceCounter averaging
 * (src/PerformanceCounter.cpp:39-56) into perfPath; `volume`, `energy`,
 * `particleEnergy` hold `n` frames of the conservation series
 * (src/FluidSim2D.cpp:709-731), written to conservationPath.  Either path
 * may be NULL. */
int fs2d_write_stats(const float* stageMs, int numStages, size_t frames, const double* volume, const double* energy,
                     const double* particleEnergy, size_t n, const char* perfPath, const char* conservationPath);

/* Headless render data: what the reference's renderer gathers each frame
 * (FluidRenderer2D::updateBuffers, demo/FluidRenderer2D.cpp:435-486),
 * computed on the device into caller-owned DEVICE buffers (float pairs).
 * NULL buffers are skipped; list counts are written to the host size_t's.
 * Lists keep the reference's row-major cell order; at most `*Cap` entries
 * are written, the count is the full one. */
typedef struct fs2d_render {
    float* waterCells;      /* corner (i dx, j dx) of each FLUID cell: 2 floats per cell */
    size_t waterCap;
    size_t* waterCount;
    float* solidCells;      /* corner of each SOLID cell */
    size_t solidCap;
    size_t* solidCount;
    float* pressureCells;   /* corner of each cell with p != 0 */
    float* pressureValues;  /* sigmoid(0.01 p) of those cells */
    size_t pressureCap;
    size_t* pressureCount;
    float* cellVels;        /* (sizeX-1)*(sizeY-1) segments: centre, centre + dt*velInterp(centre): 4 floats each */
    float* particleLines;   /* one segment per particle: position, position + dt*velInterp(position) */
    float* phiValues;       /* sizeX*sizeY values sigmoid(100 phi) */
} fs2d_render;
int fs2d_render_export(fs2d_sim* sim, fs2d_render* r);

/* Particle reseeding and volume correction.  The reference lists both as
 * features it needs and does not have (README.md:13-18: "the fluid
 * simulation doesn't conserve volume very well"); it records the water
 * volume at creation (origWaterVolume, src/FluidSim2D.cpp:71-72) but never
 * uses it.  Both are off unless called, and then deterministic: the same
 * state and arguments give the same bits on every run.
 *
 * fs2d_reseed: call between frames.  Particles are counted per cell at
 * (int)(x/dx), (int)(y/dx), clamped into the grid.  In every cell holding
 * more than maxPerCell particles (maxPerCell > 0), those after the first
 * maxPerCell in particle order are removed; every FLUID cell (labels of the
 * last createWaterLevelSet) holding fewer than minPerCell gets new particles
 * up to minPerCell, at ((i + jx) dx, (j + jy) dx) with jx, jy in [0, 1)
 * drawn from a 64-bit mix of (seed, cell, k), moving with the bilinear grid
 * velocity there (the PIC part of updateParticleVelocities).  Survivors
 * keep their order; new particles follow in row-major cell order.  0 <=
 * minPerCell <= 64, maxPerCell == 0 (no removal) or minPerCell <=
 * maxPerCell.  `out` (may be NULL) receives the counts.  A cell over
 * maxPerCell is ordered by one thread, in time that grows with the square
 * of its particle count (a few to a few dozen in a simulation). */
typedef struct fs2d_reseed_stats {
    size_t removed;
    size_t added;
    size_t numParticles;   /* after reseeding */
} fs2d_reseed_stats;
int fs2d_reseed(fs2d_sim* sim, int minPerCell, int maxPerCell, unsigned int seed, fs2d_reseed_stats* out);

/* fs2d_set_volume_correction: from the next applyProjection on, every FLUID
 * cell's right-hand side gets rate * ((V0 - V) / V0) / dt added, V the
 * waterVolume of the frame's createWaterLevelSet (the volume at creation
 * before the first one) and V0 origWaterVolume: the pressure solve then
 * targets a uniform divergence that gives back the fraction `rate` of the
 * relative volume error per step.  rate 0 (the default) turns it off and
 * leaves every stage as the reference's; 0 <= rate <= 1. */
int fs2d_set_volume_correction(fs2d_sim* sim, double rate);

/* Test hook of the failure path of the wavefront sweeps (no reference
 * counterpart).  Every wait of a sweep on its neighbour strip is bounded: it
 * gives up after `polls` polls (<= 0: the default, about half a second),
 * the kernel then finishes without the value and the call returns
 * FS2D_ERR_TIMEOUT.  With holdKinds != 0, strip `holdStrip` of every sweep
 * of those kinds withholds its hand-off to the next strip, so that strip's
 * wait runs out (kinds: 1 closest-point sweeps, 2 Eikonal sweeps, 4 FP64
 * MIC(0) factor and solves, counted in blocks of their launch, 8 FP32
 * MIC(0) factor and solves); 0 turns the hold off.  Results of a frame that timed out
 * are invalid; the handle stays usable. */
#define FS2D_WAVE_CLOSEST_POINT 1
#define FS2D_WAVE_EIKONAL       2
#define FS2D_WAVE_MIC_FP64      4
#define FS2D_WAVE_MIC_FP32      8
int fs2d_debug_wavefront(fs2d_sim* sim, long long polls, int holdKinds, int holdStrip);

/* Test hook of the allocation failure path (no reference counterpart; the
 * reference exits when an allocation fails, include/Array2D.h:69-72): after
 * `after` more device allocations of a handle's arrays succeed, every
 * further one fails with FS2D_ERR_ALLOC as if the device were out of
 * memory, until the hook is turned off with a negative value.  Process-wide;
 * a create that fails this way frees what it had allocated. */
int fs2d_debug_fail_alloc(long long after);

/* Use `stream` (a cudaStream_t) for all subsequent work of this handle;
 * NULL restores the handle's own stream. */
int fs2d_set_stream(fs2d_sim* sim, void* stream);

/* Number of kernels this handle has launched so far. */
int fs2d_launch_count(fs2d_sim* sim, unsigned long long* out);

/* Per-kernel device timing, the kernel-level analogue of the reference's
 * PerformanceCounter stage timers (src/PerformanceCounter.cpp:16-50): CUDA
 * events are recorded on the handle's stream around every launch whose
 * kernel name contains one of the comma-separated `patterns` ("" or NULL
 * turns timing off).  fs2d_get_kernel_times writes one line per timed
 * kernel, "name launches total_ms\n", covering the launches since the
 * previous call, and resets the counts. */
int fs2d_set_kernel_timing(fs2d_sim* sim, const char* patterns);
int fs2d_get_kernel_times(fs2d_sim* sim, char* buf, size_t cap);

/* Message of the last error on the calling thread ("" if none). */
const char* fs2d_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* FS2D_H */
