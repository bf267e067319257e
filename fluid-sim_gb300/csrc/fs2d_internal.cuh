// fs2d_internal.cuh — device state and shared helpers of the GB300 FluidSim2D step.
//
// One simulation handle owns all of its device memory.  Grids are row-major
// (element (i, j) at j*width + i) exactly as the reference's Array2D
// (include/Array2D.h:41-49); u faces are (NX+1) x NY, v faces NX x (NY+1)
// (include/MACGrid2D.h:19-25); particles are interleaved (x, y) pairs.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <atomic>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "fs2d.h"

namespace fs2d {

constexpr uint8_t kEmpty = FS2D_EMPTY;
constexpr uint8_t kFluid = FS2D_FLUID;
constexpr uint8_t kSolid = FS2D_SOLID;
constexpr uint32_t kUnknown = 0xFFFFFFFFu;   // extrapolation mask of an unknown face

// The device error word and the controls of the wavefront waits share one
// allocation of kErrWords ints (Sim::err):
//   err[0]      error bits: 1 a wait between strips gave up (timeout), 2 a
//               non-finite particle position, 4 a particle outside the grid,
//               8 a wait between extrapolation bands gave up (timeout);
//               with bit 0, the sweep kind (kWaveKind* << 4) and the wait
//               (256 previous strip, 512 own tile loads, 1024 other warp);
//   err[1]      kinds of sweep (kWaveKind*) in which strip err[2] withholds
//               its hand-off to the next strip (0: none).  A test hook
//               (fs2d_debug_wavefront): the next strip's wait then runs out
//               and the sweep reports a timeout without any fault;
//   err[4..5]   polls before a wait between strips gives up (a long long;
//               kWaveSpinLimit unless a test shortened it).
// Waits for a sweep's own TMA copies always use kWaveSpinLimit: those
// copies complete whatever the other strips do.
constexpr int kErrWords = 8;
constexpr long long kWaveSpinLimit = 1ll << 22;   // polls before a wait gives up (~0.5 s), by default
constexpr int kWaveKindCp = 1, kWaveKindEik = 2, kWaveKindWave2 = 4, kWaveKindMic32 = 8;
// A wait that gave up sets bit 0 of err[0] together with what it waited for
// (which sweep: kWaveKind* << 4; which wait: kWait*), for the message.
constexpr int kWaitStrip = 1 | 256;    // the previous strip's hand-off
constexpr int kWaitTile = 1 | 512;     // the strip's own TMA tile loads
constexpr int kWaitWarp = 1 | 1024;    // the other warp of the strip's CTA

// Scalars of one pressure solve, kept in device memory so that the PCG loop
// runs without host round trips.  Finalised by the last block of each
// reduction kernel.
struct PcgScalars {
    double sigma;       // z . r
    double alpha;
    double beta;
    double rhs_norm;    // ||b||inf
    double r_norm;      // ||r||inf after the last update
    double tol_abs;     // tol * ||b||inf
    int iter;           // completed iterations (reference's `iter`)
    int done;           // 1 once the solve stopped
    int first;          // 1 until the first search direction was formed
    unsigned int ticket[4];  // last-block-done counters, one per reduction kernel
    // mixed precision: the FP64 refinement around the FP32 inner solves
    // (kept in the handle's FP64 scalars) and whether an inner solve runs in
    // the current refinement sweep (kept in the FP32 scalars)
    int outer_iters;    // refinement sweeps done
    int outer_done;     // 1 once the refinement stopped (converged, nothing to solve, or the sweep cap)
    int inner_total;    // inner iterations summed over the sweeps
    int active;         // FP32 scalars: 1 while this sweep solves the scene
};

// Scalars of the per-frame statistics (createWaterLevelSet, src/FluidSim2D.cpp:709-731).
struct FrameStats {
    double volume;
    double energy;
    double particle_energy;
    double avg_p;
    double avg_p_fluid;
    double max_vel;
    unsigned int ticket;
    unsigned int pad;
};

// FP32 arrays of the mixed-precision inner solver (projection_mixed.cu),
// each P32 x NY32: the row pitch P32 is NX rounded up to 128 floats and the
// rows NY rounded up to 32, so that the FP32 MIC(0) sweeps work on whole
// strips of 128 columns and tiles of 32 rows; padding holds zeros.
struct Mixed32 {
    float *a0 = nullptr, *ax = nullptr, *ay = nullptr;             // matrix
    float *pc = nullptr, *fa = nullptr, *fb = nullptr, *fc = nullptr, *fd = nullptr;  // MIC(0), folded
    float *r = nullptr, *rp = nullptr, *q = nullptr, *z = nullptr, *w = nullptr;
    float *s0 = nullptr, *s1 = nullptr, *e = nullptr;
};
// One scene of a pack (below): where its padded FP32 region lies in the
// pack's arrays, its block ranges in the pack's reduction launches, and the
// handle arrays the FP64 refinement works on.
struct PackScene {
    int NX, NY;              // cells
    int P32, NY32;           // padded extent (multiples of 128 columns and 32 rows)
    long long off;           // pack offset of the scene's cell (0, 0): y0 * pitch + x0
    int x0, y0;              // pack column and row of that cell
    int nb32, blk0;          // FP32 kernels: nb32 blocks over the padded P32 x NY region, from block blk0
    int nb64, blk64;         // FP64 refinement kernels: nb64 blocks of 256 cells, from block blk64
    const uint8_t* cell;     // labels (NX x NY)
    const double *A0, *Ax, *Ay, *rhs;
    double *p, *r;           // FP64 pressure and residual
    PcgScalars *outer;       // the handle's FP64 scalars (refinement)
    PcgScalars *inner;       // the handle's FP32 scalars (inner solve)
    float2* part;            // FP32 reduction partials (nb32), in the pack's buffer
    double* part64;          // FP64 residual partials (nb64), in the pack's buffer
};

// Work item of a sweep over several scenes: one strip of 128 columns of one
// scene.  Any order of the work list is valid in which each strip comes after
// the strip before it in its scene.
struct Mic32Item {
    int scene;               // index in the pack's scene table
    int strip;               // strip of the scene (0: first in sweep order)
    int nstrips;             // strips of the scene
    int x0, P32;             // the scene's pack column and padded width
    int y0, NY32;            // the scene's pack row and padded rows
    int pidx;                // progress counter of this strip (the scene's strips have consecutive counters)
};

// TMA descriptors of the two FP32 MIC(0) sweeps (see mic32_tma.cuh).
struct Mic32MapsHost {
    alignas(64) unsigned char fwd[4 * 128];
    alignas(64) unsigned char bwd[4 * 128];
    alignas(64) unsigned char fac[4 * 128];   // the FP32 MIC(0) factor
};

// TMA descriptors of the closest-point sweeps (see cp_sweep.cuh).
struct CpMapsHost {
    alignas(64) unsigned char b[3 * 128];
};
// Constants of the FP32 closest-point decision (computed on the device per
// level-set build, see cp_sweep.cuh).
struct CpConst {
    float A42;       // 2^-42 A, A >= every |coordinate| of particles and cell corners
    float C0;        // 2^-80 A^2 + 2^-120
    float tiny_q;    // >= 2^-20 dr^2
    unsigned amax;   // bits of max |h| over particle coordinates (non-negative float)
    int fast;        // 0: dr or A not finite/representable, every decision is exact
};

// A pack: the FP32 solver arrays of one scene, or of several scenes side by
// side in one set of pitched arrays (a batch), with everything one launch
// per kernel of the inner solve needs: the scene table, the map from block to
// scene of the reduction launches, the sweep work items and the counters the
// host polls.  A mixed-precision handle owns a pack of its own scene; a batch
// owns a pack of all its scenes, and each scene's handle then works on its
// region of the batch's arrays (projection_mixed.cu).
struct Pack {
    int n = 0;                            // scenes
    int pitch = 0, rows = 0;              // array extent: rows x pitch floats
    Mixed32 m;                            // the arrays
    bool owns_arrays = false;             // freed with the pack (a batch); else the handle's
    bool plain = false;                   // plain FP32 PCG (FP32 dot products, no FP64 refinement)
    std::vector<PackScene> scenes;        // scene table (host copy)
    PackScene* d_scenes = nullptr;
    float2* part = nullptr;               // FP32 reduction partials, one per block of nblk
    double* part64 = nullptr;             // FP64 residual partials, one per block of nblk64
    int* d_blk = nullptr;                 // scene of each block of the FP32 reduction launches
    int nblk = 0;
    int* d_blk64 = nullptr;               // scene of each block of the FP64 refinement launches
    int nblk64 = 0;
    Mic32Item* d_items = nullptr;         // sweep work items (several scenes only)
    int nitems = 0;
    // counters in device memory: [0] scenes whose inner solve is running,
    // [1] scenes still refining, [2..5] work and exit counters of the two
    // persistent sweeps; h_ctl is a pinned mirror for polling
    int* d_ctl = nullptr;
    int* h_ctl = nullptr;
    unsigned long long* progress = nullptr;    // sweep progress (items), direct launches
    unsigned long long* gprogress = nullptr;   // ... graph-replayed launches
    unsigned long long* gbase = nullptr;       // device progress base of graph-replayed sweeps
    int progress_cap = 0;
    Mic32MapsHost* maps = nullptr;             // tensor maps of the pack's arrays
    int cluster = 0;                           // cluster size of single-scene sweeps (0: not chosen)
    int sweep_ctas = 0;                        // CTAs of persistent sweeps (several scenes)
    int schedule = 0;                          // order of the scenes in the sweep's work list (pack_tune)
    unsigned long long wave_launch = 0;        // progress bases of direct sweeps
    cudaGraphExec_t graph = nullptr;           // inner iterations captured as a graph
    const void* graph_key = nullptr;
    unsigned long long graph_launches = 0;
    int graph_state = 0;                       // 0 not tried, 1 ready, -1 unavailable (direct launches)
};

struct Sim {
    // configuration
    int NX = 0, NY = 0, ppc_sqrt = 0, mode = 0;
    double dt = 0, dx = 0, dr = 0, rho = 0, gx = 0, gy = 0, alpha = 0;
    fs2d_options opt{};
    size_t N = 0, NU = 0, NV = 0;

    // state (FluidSim2D public fields)
    uint8_t* cell = nullptr;
    double* phi = nullptr;
    double* p = nullptr;
    double *u = nullptr, *v = nullptr, *nu = nullptr, *nv = nullptr;
    double2* pos = nullptr;
    double2* vel = nullptr;
    size_t np = 0, np_cap = 0;

    // level-set scratch
    int* t = nullptr;                 // closest particle of each cell (-1 = none), row pitch P
    float4* pos_df = nullptr;         // float-pair particle positions (np_cap)
    float2* cp_tab = nullptr;         // float-pair corner coordinates: P columns, then NY rows
    CpConst* cpc = nullptr;           // constants of the FP32 closest-point decision
    uint2* eik_rng = nullptr;         // per strip: column range of the current Eikonal sweep (see k_eik_check)
    int* cp_hb_t = nullptr;           // closest-point strip hand-off rows (progress_cap x P)
    float4* cp_hb_p = nullptr;
    CpMapsHost* cpmaps = nullptr;
    double* phi_p = nullptr;          // pitched level set of the Eikonal sweeps (P x NY)
    uint8_t* emask = nullptr;         // Eikonal: cells whose update changes them (P x NY)
    CpMapsHost* ekmaps = nullptr;     // TMA descriptors of the Eikonal sweeps
    int ek_cluster = 0;               // cluster size of the Eikonal sweeps (0: not chosen)
    unsigned long long* seed_key = nullptr;
    double* phi_tmp = nullptr;
    uint8_t* surface = nullptr;

    // transfer scratch
    double *u0 = nullptr, *v0 = nullptr;    // pre-advection copy / uDiff source
    double *udiv = nullptr, *vdiv = nullptr;
    uint32_t *mask_u = nullptr, *mask_v = nullptr;
    uint32_t *cnt_u = nullptr, *cnt_v = nullptr;     // P2G contributions per face (then offsets)
    uint32_t *fill_u = nullptr, *fill_v = nullptr;
    uint32_t *ent_u = nullptr, *ent_v = nullptr;     // P2G contribution keys, 4 per particle
    size_t ent_cap = 0;
    uint32_t* scan_tmp = nullptr;
    size_t scan_tmp_n = 0;
    int2* tile_range = nullptr;                      // extrapolation: per 32x32 tile [min,max] layer
    unsigned int* max_layer = nullptr;

    // projection scratch
    double *Adiag = nullptr, *Ax = nullptr, *Ay = nullptr, *rhs = nullptr, *precon = nullptr;
    // MIC(0) triangular-solve coefficients: forward Ax(i-1,j)*pc(i-1,j), Ay(i,j-1)*pc(i,j-1);
    // backward Ax(i,j)*pc(i,j), Ay(i,j)*pc(i,j)
    double *cfx = nullptr, *cfy = nullptr, *cbx = nullptr, *cby = nullptr;
    double *r = nullptr, *z = nullptr, *q = nullptr, *w = nullptr;
    double *s0 = nullptr, *s1 = nullptr;             // ping-pong search direction
    double* partial = nullptr;                       // per-block reduction partials
    size_t partial_cap = 0;
    PcgScalars* pcg = nullptr;
    PcgScalars* pcg_host = nullptr;                  // pinned mirror for polling
    Mixed32 m32;                                     // MIXED precision only: views into pack->m
    int P = 0;                                       // row pitch of the pitched arrays (NX rounded up to 32)
    int P32 = 0, NY32 = 0;                           // pitch of the FP32 solver arrays, padded rows of the scene
    PcgScalars* pcg32 = nullptr;                     // inner FP32 solve scalars
    PcgScalars* pcg32_host = nullptr;
    Pack* pack = nullptr;                            // MIXED: the pack of this scene alone
    bool m32_owned = true;                           // m32 arrays allocated by this handle (not a batch's views)

    // wavefront progress flags (monotonic, 64-bit, never reset)
    unsigned long long* progress = nullptr;
    int progress_cap = 0;
    unsigned long long wave_launch = 0;
    // wavefront sweeps captured into a CUDA graph (a batch's per-scene
    // phases): their own progress flags and a device-side base that a
    // one-thread kernel before each such sweep advances, so every replay
    // starts from fresh bases
    bool capturing = false;
    unsigned long long* gprogress = nullptr;
    unsigned long long* gbase = nullptr;
    // bumped whenever buffers, parameters or options change: a captured
    // phase of an older generation is captured again
    unsigned long long generation = 0;

    // frame statistics and errors
    FrameStats* stats = nullptr;
    FrameStats* stats_host = nullptr;
    int* err = nullptr;            // device error word and wait controls (kErrWords ints)
    int* err_host = nullptr;

    // history of per-frame conservation values (host)
    double* hist = nullptr;        // 3 per frame
    size_t hist_n = 0, hist_cap = 0;

    // bookkeeping
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[20] = {};
    float stage_ms[10] = {};
    int n_stage_times = 0;
    unsigned long long launches = 0;
    long long frames = 0;
    double current_time = 0;
    double orig_volume = 0;
    double volume_rate = 0;   // fs2d_set_volume_correction (0: off)
    int last_iters = 0;
    int last_outer = 0;
    double last_rel_res = 0;
    int last_status = 0;
    int device = 0;

    // differentiable rollout (fs2d_forward / fs2d_backward), allocated on first use
    struct Rollout* ro = nullptr;

    // opt-in per-kernel event timing (fs2d_set_kernel_timing)
    std::string kt_patterns;
    std::map<const char*, bool> kt_match;
    std::vector<cudaEvent_t> kt_pool;
    size_t kt_used = 0;
    std::vector<std::pair<const char*, size_t>> kt_pending;  // name, index of the start event
    std::map<std::string, std::pair<long long, double>> kt_acc;
};

// ---- error reporting (thread-local message, see fs2d_last_error) ----
void set_error(const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
#define FS2D_CUDA(call)                                   \
    do {                                                  \
        int _rc = ::fs2d::check_cuda((call), #call);      \
        if (_rc) return _rc;                              \
    } while (0)

// Kernel timing hooks: returns the start-event index, or -1 when `name` is
// not being timed.
long long ktimer_begin(Sim* s, const char* name);
void ktimer_end(Sim* s, long long slot);
void ktimer_collect(Sim* s);  // after the stream drained

// Launch helper: counts the launch, optionally times it, reports launch errors.
#define FS2D_LAUNCH(sim, kernel, grid, block, smem, ...)                               \
    do {                                                                              \
        (sim)->launches++;                                                            \
        long long _kt = ::fs2d::ktimer_begin((sim), #kernel);                         \
        kernel<<<(grid), (block), (smem), (sim)->stream>>>(__VA_ARGS__);             \
        ::fs2d::ktimer_end((sim), _kt);                                              \
        int _rc = ::fs2d::check_cuda(cudaGetLastError(), #kernel);                   \
        if (_rc) return _rc;                                                          \
    } while (0)

// 2D tensor map (TMA descriptor) of a pitched row-major array.
int make_tensor_map_2d(CUtensorMap* map, void* base, CUtensorMapDataType dtype, int elem_bytes, int width,
                       int height, int pitch_elems, int box_w, int box_h);

// Cooperative launch of `nblocks` blocks (rounded up to whole clusters of
// `cluster` blocks when cluster > 1).
cudaError_t launch_clustered(const void* kernel, int nblocks, int cluster, int threads, size_t smem,
                             cudaStream_t stream, void** args);
// Largest cluster size (<= 8) with which every cluster of a grid of
// `nblocks` blocks can be co-resident; 1 when clusters are not usable.
int choose_cluster(const void* kernel, int nblocks, int threads, size_t smem);

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per kernel and
// device; `done` is the kernel's own bit set of configured devices.  Safe
// from several host threads (batches drive their scenes concurrently).
inline int ensure_smem_attr(std::atomic<unsigned long long>& done, int device, const void* fn, int bytes) {
    const unsigned long long bit = 1ull << (device & 63);
    if (done.load(std::memory_order_acquire) & bit) return 0;
    int rc = check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                        "cudaFuncSetAttribute");
    if (!rc) done.fetch_or(bit, std::memory_order_acq_rel);
    return rc;
}

// Waits for the work queued on `st` (the handle's stream) to finish.
inline int wait_stream(Sim*, cudaStream_t st) { return check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize"); }

inline unsigned int blocks_for(size_t n, int threads) { return (unsigned int)((n + threads - 1) / threads); }

// ---- stage entry points (implemented in the per-stage .cu files) ----
int levelset_create(Sim* s);              // createWaterLevelSet
// createWaterLevelSet of a batch of scenes: levelset_seed per scene, then
// ls_batch_sweeps (every scene's sweeps, one launch per sweep for all of
// them), then levelset_finish per scene.
int levelset_seed(Sim* s);
int levelset_finish(Sim* s);
struct LsBatch;
LsBatch* ls_batch_create(Sim* const* sims, int n, int device, int* rc);
void ls_batch_free(LsBatch* b);
int ls_batch_sweeps(LsBatch* b, cudaStream_t stream, int* err, unsigned long long* launches);
int p2g(Sim* s);                          // transferVelocityToGrid
int sl_advect(Sim* s);                    // applySemiLagrangianAdvection
int apply_gravity(Sim* s);                // applyGravity
int projection(Sim* s, int* status);      // applyProjection, FP64
int projection_mixed(Sim* s, int* status);  // applyProjection, FP32 PCG in FP64 refinement
int projection_build(Sim* s);             // FP64 matrix, rhs, p = 0, r = rhs, ||rhs||
int projection_set_rhs(Sim* s, const double* b);   // after projection_build: rhs = r = b, p = 0
int projection_solve_custom(Sim* s, const double* b, int* status);  // A p = b (device b), handle's precision
int projection_mixed_rhs(Sim* s, const double* b, int* status);     // mixed solve; b == nullptr: physical rhs
// ---- packs of FP32 solver arrays (projection_mixed.cu) ----
// The pack of a handle's own scene (its FP32 arrays at pitch s->P32).
int pack_create_single(Sim* s);
// A pack of several handles' scenes in new arrays; each scene's FP32 arrays
// become views into them (their pitch becomes the pack's).
int pack_create_batch(Sim* const* sims, int n, Pack** out);
void pack_free(Pack* pk);
// Device state of the handle's FP32 setup for a solve (matrix, MIC(0) factor,
// folded coefficients) after projection_build / projection_set_rhs.
int mixed_setup(Sim* s);
// The refinement loop of every scene of the pack (each after mixed_setup),
// on `stream`; returns after the work completed.
// Kernels go on `stream`, count into *launches and report waits that gave up
// in `err` (an error word with its wait controls); `timer` (may be null)
// times the launches as fs2d_set_kernel_timing asks.
int pack_solve(Pack* pk, const fs2d_options& opt, cudaStream_t stream, unsigned long long* launches, int* err,
               int device, Sim* timer);
// Chooses the persistent sweep's schedule and CTA count of a pack of several
// scenes by timing forward sweeps of each candidate; *best_us (may be null)
// receives the chosen sweep's time.
int pack_tune(Pack* pk, cudaStream_t stream, int* err, int device, unsigned long long* launches, double* best_us);
// Sets the persistent sweep's schedule (0..3, see pack_tune) and, ctas > 0,
// its CTA count.
int pack_set_schedule(Pack* pk, int schedule, int ctas, cudaStream_t stream);
// Statistics of the handle's last mixed solve (from its scalars); *status =
// FS2D_ERR_NOT_CONVERGED when it stopped short of its tolerance.
int mixed_finish(Sim* s, int* status);
// mixed_finish in two halves (a batch frame reads the scalars at frame close)
int mixed_finish_queue(Sim* s);
void mixed_finish_read(Sim* s, int* status);
int cp_setup_maps(Sim* s);                // TMA descriptors of the closest-point sweeps
int update_velocity(Sim* s);              // updateVelocity
int g2p(Sim* s);                          // updateParticleVelocities
int render_export(Sim* s, fs2d_render* r);    // headless render data (render.cu)
int advect_particles(Sim* s);             // applyAdvection
int diagnostics(Sim* s);                  // avgPressure, avgPressureInFluid, maxVelocity
int extrapolate(Sim* s, double* a, uint32_t* mask, int W, int H, double* b, uint32_t* mask_b, int Wb, int Hb);

// Scratch of one extrapolation call over up to two face grids.
struct ExtrapScratch {
    int* dist[2];              // W*H ints per grid (distance transform)
    int2* tile_range;          // per 32x32 tile [min, max] layer, grid 1 after grid 0
    unsigned int* max_layer;   // 2 counters
};
size_t extrap_tiles(int W, int H);
int extrapolate_core(Sim* s, cudaStream_t stream, const ExtrapScratch& x, double* const a[2], uint32_t* const m[2],
                     const int W[2], const int H[2], int band);
int exclusive_scan_u32(Sim* s, uint32_t* data, size_t n);

// applyAdvection's CFL check (fs2d_cfl): the largest c > 0 and its first particle.
int cfl_check(Sim* s, double* cfl, long long* particle);

// Particle reseeding (fs2d_reseed): scratch of N + 1 (cells) or np + 1
// (particles) words each.
struct ReseedScratch {
    uint32_t *cnt, *start, *fill, *spawn;   // per cell
    uint32_t *bucket, *keep;                // per particle
};
// Counts and plans on the handle's stream, then waits: *n_keep survivors,
// *n_add new particles.
int reseed_plan(Sim* s, const ReseedScratch& x, int min_per_cell, int max_per_cell, size_t* n_keep, size_t* n_add);
// Writes the survivors and the new particles into npos / nvel (n_keep + n_add entries).
int reseed_write(Sim* s, const ReseedScratch& x, unsigned seed, double2* npos, double2* nvel);

// ---- transposes of the particle transfers (transfer.cu) ----
int p2g_adjoint(Sim* s, double* ubar, double* vbar, double* wu, double* wv, double2* velbar);
int g2p_adjoint(Sim* s, const double2* velbar, double* nub, double* nvb, double* ub, double* vb, double2* vinb);

// ---- differentiable rollout (adjoint.cu) ----
int rollout_forward(Sim* s, int steps, int every, const double* u0, const double* v0, const double* ut,
                    const double* vt, double* loss);
int rollout_backward(Sim* s, double* gu, double* gv);
void rollout_free(Sim* s);

// ---- frames in parts (capi.cu), for batches that solve their scenes together ----
int frame_stages(fs2d_sim* p, int k0, int k1, int* status, int solve_part = 0);
int frame_levelset(fs2d_sim* p, int part);
void frame_mark(fs2d_sim* p, int what);
int frame_solve_stage(fs2d_sim* p);   // index of applyProjection in the frame's stage order
int frame_close(fs2d_sim* p, int rc, int status);
Sim* sim_of(fs2d_sim* p);

// ---- wavefront plumbing ----
// Reserves `n` progress counters and returns the base value for this launch.
unsigned long long wave_begin(Sim* s);

}  // namespace fs2d
