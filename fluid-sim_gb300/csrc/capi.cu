// capi.cu — the C ABI (include/fs2d.h): handle lifetime, frame and stage
// drivers, host <-> device state transfer, statistics and CSV output,
// checkpoint / resume, and the host side of reseeding, volume correction,
// the CFL check and the allocation-failure test hook.
//
// Mirrors FluidSim2D (include/FluidSim2D.h:65-176, src/FluidSim2D.cpp):
// create seeds particles on the host with libc rand() in the reference's
// loop order, so the same rand() state gives the same particles; every
// stage then runs on the device.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <new>
#include <string>
#include <vector>

#include "fs2d_internal.cuh"

namespace fs2d {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FS2D_ERR_ALLOC : FS2D_ERR_CUDA;
}

long long ktimer_begin(Sim* s, const char* name) {
    if (s->kt_patterns.empty()) return -1;
    auto it = s->kt_match.find(name);
    bool hit;
    if (it == s->kt_match.end()) {
        hit = false;
        size_t a = 0;
        const std::string& pat = s->kt_patterns;
        while (a <= pat.size()) {
            size_t b = pat.find(',', a);
            if (b == std::string::npos) b = pat.size();
            std::string tok = pat.substr(a, b - a);
            if (!tok.empty() && strstr(name, tok.c_str())) hit = true;
            a = b + 1;
        }
        s->kt_match[name] = hit;
    } else {
        hit = it->second;
    }
    if (!hit) return -1;
    if (s->kt_used + 2 > s->kt_pool.size()) {
        for (int k = 0; k < 64; k++) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            s->kt_pool.push_back(e);
        }
    }
    size_t slot = s->kt_used;
    s->kt_used += 2;
    cudaEventRecord(s->kt_pool[slot], s->stream);
    s->kt_pending.push_back(std::make_pair(name, slot));
    return (long long)slot;
}

void ktimer_end(Sim* s, long long slot) {
    if (slot < 0) return;
    cudaEventRecord(s->kt_pool[(size_t)slot + 1], s->stream);
}

void ktimer_collect(Sim* s) {
    for (auto& pr : s->kt_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, s->kt_pool[pr.second], s->kt_pool[pr.second + 1]) == cudaSuccess) {
            auto& acc = s->kt_acc[pr.first];
            acc.first += 1;
            acc.second += ms;
        } else {
            (void)cudaGetLastError();
        }
    }
    s->kt_pending.clear();
    s->kt_used = 0;
}

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    // looked up once per process (thread-safe static initialisation)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000)p;
        return nullptr;
    }();
    return fn;
}

int make_tensor_map_2d(CUtensorMap* map, void* base, CUtensorMapDataType dtype, int elem_bytes, int width,
                       int height, int pitch_elems, int box_w, int box_h) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return FS2D_ERR_CUDA;
    }
    cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    cuuint64_t strides[1] = {(cuuint64_t)pitch_elems * (cuuint64_t)elem_bytes};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, dtype, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return FS2D_ERR_CUDA;
    }
    return 0;
}

cudaError_t launch_clustered(const void* kernel, int nblocks, int cluster, int threads, size_t smem,
                             cudaStream_t stream, void** args) {
    if (cluster < 1) cluster = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((nblocks + cluster - 1) / cluster * cluster));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    at[1].id = cudaLaunchAttributeClusterDimension;
    at[1].val.clusterDim.x = (unsigned)cluster;
    at[1].val.clusterDim.y = 1;
    at[1].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = cluster > 1 ? 2 : 1;
    return cudaLaunchKernelExC(&cfg, kernel, args);
}

int choose_cluster(const void* kernel, int nblocks, int threads, size_t smem) {
    for (int cs = nblocks < 8 ? nblocks : 8; cs > 1; cs--) {
        const int grid = (nblocks + cs - 1) / cs * cs;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) == cudaSuccess && n * cs >= grid) return cs;
        (void)cudaGetLastError();
    }
    return 1;
}

unsigned long long wave_begin(Sim* s) {
    // progress values are base + (columns done); columns < 2^24
    s->wave_launch++;
    return s->wave_launch << 24;
}

namespace {

struct Host {
    Sim sim;
    std::vector<float> frame_stage_ms;  // numStages per frame
    bool stats_pending = false;
    bool solve_pending = false;   // a batch frame's solve scalars are on their way to pcg_host
};

// fs2d_debug_fail_alloc: < 0 no injection; otherwise the number of device
// allocations that still succeed before every further one fails.
std::atomic<long long> g_alloc_budget{-1};

bool injected_alloc_failure() {
    long long b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) return true;
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) return false;
    }
    return false;
}

template <typename T>
int dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    if (injected_alloc_failure()) {
        set_error("cudaMalloc of %zu bytes failed: injected by fs2d_debug_fail_alloc", n * sizeof(T));
        return FS2D_ERR_ALLOC;
    }
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        set_error("cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
        return FS2D_ERR_ALLOC;
    }
    e = cudaMemset(*p, 0, n * sizeof(T));
    return check_cuda(e, "cudaMemset");
}

int num_stages(const Sim* s) { return s->mode == FS2D_SEMILAGRANGIAN ? 7 : 8; }

const int kSlStages[7] = {FS2D_STAGE_CREATE_WATER_LEVEL_SET, FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION,
                          FS2D_STAGE_APPLY_GRAVITY,          FS2D_STAGE_CREATE_SOLID_LEVEL_SET,
                          FS2D_STAGE_APPLY_PROJECTION,       FS2D_STAGE_UPDATE_VELOCITY,
                          FS2D_STAGE_APPLY_ADVECTION};
const int kPicStages[8] = {FS2D_STAGE_CREATE_WATER_LEVEL_SET, FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID,
                           FS2D_STAGE_APPLY_GRAVITY,          FS2D_STAGE_CREATE_SOLID_LEVEL_SET,
                           FS2D_STAGE_APPLY_PROJECTION,       FS2D_STAGE_UPDATE_VELOCITY,
                           FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES, FS2D_STAGE_APPLY_ADVECTION};

int alloc_particles(Sim* s, size_t cap) {
    s->generation++;
    cudaFree(s->pos);
    cudaFree(s->vel);
    cudaFree(s->ent_u);
    cudaFree(s->ent_v);
    s->pos = nullptr;
    s->vel = nullptr;
    s->ent_u = s->ent_v = nullptr;
    int rc;
    if ((rc = dalloc(&s->pos, cap))) return rc;
    if ((rc = dalloc(&s->vel, cap))) return rc;
    if ((rc = dalloc(&s->ent_u, 4 * cap))) return rc;
    if ((rc = dalloc(&s->ent_v, 4 * cap))) return rc;
    cudaFree(s->pos_df);
    s->pos_df = nullptr;
    if ((rc = dalloc(&s->pos_df, std::max<size_t>(cap, 1)))) return rc;
    s->np_cap = cap;
    size_t need = std::max(std::max(s->N, std::max(s->NU, s->NV)), cap) / 32 + 4096;
    if (4 * need > s->partial_cap) {
        cudaFree(s->partial);
        s->partial = nullptr;
        if ((rc = dalloc(&s->partial, 4 * need))) return rc;
        s->partial_cap = 4 * need;
    }
    return 0;
}

// Writes the wait controls that follow the device error word (kErrWords).
int set_wave_controls(Sim* s, long long polls, int kinds, int strip) {
    int w[kErrWords] = {0};
    w[1] = kinds;
    w[2] = strip;
    memcpy(&w[4], &polls, sizeof(polls));
    FS2D_CUDA(cudaMemcpyAsync(s->err + 1, w + 1, (kErrWords - 1) * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    return wait_stream(s, s->stream);
}

int alloc_all(Sim* s) {
    int rc;
    const size_t N = s->N, NU = s->NU, NV = s->NV;
#define A(ptr, n) \
    if ((rc = dalloc(&s->ptr, (n)))) return rc
    A(cell, N);
    A(phi, N);
    A(p, N);
    A(u, NU);
    A(v, NV);
    A(nu, NU);
    A(nv, NV);
    s->P = (s->NX + 31) / 32 * 32;
    A(t, (size_t)s->P * s->NY);
    A(seed_key, N);
    A(phi_tmp, N);
    A(u0, NU);
    A(v0, NV);
    A(udiv, NU);
    A(vdiv, NV);
    A(mask_u, NU);
    A(mask_v, NV);
    A(cnt_u, NU + 1);
    A(cnt_v, NV + 1);
    A(fill_u, NU);
    A(fill_v, NV);
    s->scan_tmp_n = std::max(NU, NV) / 4096 + 4;
    A(scan_tmp, s->scan_tmp_n);
    size_t tiles = (size_t)((s->NX + 1 + 31) / 32) * ((s->NY + 31) / 32) + (size_t)((s->NX + 31) / 32) * ((s->NY + 1 + 31) / 32);
    A(tile_range, tiles);
    A(max_layer, 16);
    A(Adiag, N);
    A(Ax, N);
    A(Ay, N);
    A(rhs, N);
    A(precon, N);
    A(cfx, N);
    A(cfy, N);
    A(cbx, N);
    A(cby, N);
    A(r, N);
    A(z, N);
    A(q, N);
    A(w, N);
    A(s0, N);
    A(s1, N);
    A(pcg, 1);
    s->progress_cap = std::max(s->NX, s->NY) / 32 + 2;
    A(progress, (size_t)s->progress_cap);
    A(gprogress, (size_t)s->progress_cap);
    A(gbase, 1);
    A(cp_tab, (size_t)s->P + s->NY);
    A(cpc, 1);
    A(eik_rng, (size_t)s->progress_cap);
    A(cp_hb_t, (size_t)s->progress_cap * s->P);
    A(cp_hb_p, (size_t)s->progress_cap * s->P);
    A(phi_p, (size_t)s->P * s->NY);
    A(emask, (size_t)s->P * s->NY);
    s->cpmaps = new (std::nothrow) CpMapsHost();
    s->ekmaps = new (std::nothrow) CpMapsHost();
    if (!s->cpmaps || !s->ekmaps) {
        set_error("out of host memory");
        return FS2D_ERR_ALLOC;
    }
    if ((rc = cp_setup_maps(s))) return rc;
    A(stats, 1);
    A(err, kErrWords);
    if ((rc = set_wave_controls(s, kWaveSpinLimit, 0, -1))) return rc;
    if (s->opt.precision != FS2D_PRECISION_FP64) {
        Mixed32& m = s->m32;
        s->P32 = (s->NX + 127) / 128 * 128;
        s->NY32 = (s->NY + 31) / 32 * 32;
        const size_t N = (size_t)s->P32 * s->NY32;  // pitched, padded FP32 arrays
        A(m32.a0, N);
        A(m32.ax, N);
        A(m32.ay, N);
        A(m32.pc, N);
        A(m32.fa, N);
        A(m32.fb, N);
        A(m32.fc, N);
        A(m32.fd, N);
        A(m32.r, N);
        A(m32.rp, N);
        A(m32.q, N);
        A(m32.z, N);
        A(m32.w, N);
        A(m32.s0, N);
        A(m32.s1, N);
        A(m32.e, N);
        A(pcg32, 1);
        (void)m;
        s->m32_owned = true;
        if ((rc = pack_create_single(s))) return rc;
    }
#undef A
    if ((rc = check_cuda(cudaMallocHost((void**)&s->pcg_host, sizeof(PcgScalars)), "cudaMallocHost"))) return rc;
    if ((rc = check_cuda(cudaMallocHost((void**)&s->stats_host, sizeof(FrameStats)), "cudaMallocHost"))) return rc;
    if ((rc = check_cuda(cudaMallocHost((void**)&s->err_host, sizeof(int)), "cudaMallocHost"))) return rc;
    if ((rc = check_cuda(cudaMallocHost((void**)&s->pcg32_host, sizeof(PcgScalars)), "cudaMallocHost"))) return rc;
    memset(s->pcg32_host, 0, sizeof(PcgScalars));
    memset(s->pcg_host, 0, sizeof(PcgScalars));
    memset(s->stats_host, 0, sizeof(FrameStats));
    *s->err_host = 0;
    return 0;
}

void free_all(Sim* s) {
    rollout_free(s);
    pack_free(s->pack);
    s->pack = nullptr;
    if (!s->m32_owned) s->m32 = Mixed32();   // views into a batch's arrays, freed with the batch
    void* ptrs[] = {s->cell, s->phi, s->p, s->u, s->v, s->nu, s->nv, s->pos, s->vel, s->t, s->seed_key,
                    s->phi_tmp, s->surface, s->u0, s->v0, s->udiv, s->vdiv, s->mask_u, s->mask_v, s->cnt_u,
                    s->cnt_v, s->fill_u, s->fill_v, s->ent_u, s->ent_v, s->scan_tmp, s->tile_range, s->max_layer,
                    s->Adiag, s->Ax, s->Ay, s->rhs, s->precon, s->cfx, s->cfy, s->cbx, s->cby, s->r, s->z, s->q, s->w, s->s0,
                    s->s1, s->partial, s->pcg, s->progress, s->stats, s->err, s->m32.a0, s->m32.ax, s->m32.ay,
                    s->m32.pc, s->m32.fa, s->m32.fb, s->m32.fc, s->m32.fd, s->m32.r, s->m32.rp, s->m32.q,
                    s->m32.z, s->m32.w, s->m32.s0, s->m32.s1, s->m32.e, s->pcg32,
                    s->pos_df,
                    s->cp_tab, s->cpc, s->cp_hb_t, s->cp_hb_p, s->phi_p, s->emask, s->gprogress, s->gbase,
                    s->eik_rng};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->pcg_host) cudaFreeHost(s->pcg_host);
    if (s->pcg32_host) cudaFreeHost(s->pcg32_host);
    delete s->cpmaps;
    delete s->ekmaps;
    if (s->stats_host) cudaFreeHost(s->stats_host);
    if (s->err_host) cudaFreeHost(s->err_host);
    for (auto& e : s->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : s->kt_pool) cudaEventDestroy(e);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    free(s->hist);
}

// libc rand() jitter exactly as src/FluidSim2D.cpp:19-21,52-64.
double randf(float max) { return ((double)rand() / (double)RAND_MAX) * max; }

int run_stage_impl(Sim* s, int stage, int* status) {
    switch (stage) {
        case FS2D_STAGE_CREATE_WATER_LEVEL_SET: return levelset_create(s);
        case FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID: return p2g(s);
        case FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION: return sl_advect(s);
        case FS2D_STAGE_APPLY_GRAVITY: return apply_gravity(s);
        case FS2D_STAGE_CREATE_SOLID_LEVEL_SET: return 0;  // empty in the reference (:734-736)
        case FS2D_STAGE_APPLY_PROJECTION:
            return s->opt.precision != FS2D_PRECISION_FP64 ? projection_mixed(s, status) : projection(s, status);
        case FS2D_STAGE_UPDATE_VELOCITY: return update_velocity(s);
        case FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES: return g2p(s);
        case FS2D_STAGE_APPLY_ADVECTION: return advect_particles(s);
        default:
            set_error("unknown stage %d", stage);
            return FS2D_ERR_INVALID;
    }
}

// Reads the device error word and the level-set statistics after the stream
// drained; appends a history entry when the level-set stage ran.
int finish(Host* h) {
    Sim* s = &h->sim;
    FS2D_CUDA(cudaMemcpyAsync(s->err_host, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(s->stats_host, s->stats, sizeof(FrameStats), cudaMemcpyDeviceToHost, s->stream));
    if (int rcw = wait_stream(s, s->stream)) return rcw;
    ktimer_collect(s);
    if (h->stats_pending) {
        if (s->hist_n == s->hist_cap) {
            size_t cap = s->hist_cap ? 2 * s->hist_cap : 64;
            double* nh = (double*)realloc(s->hist, cap * 3 * sizeof(double));
            if (!nh) {
                set_error("out of host memory");
                return FS2D_ERR_ALLOC;
            }
            s->hist = nh;
            s->hist_cap = cap;
        }
        s->hist[3 * s->hist_n] = s->stats_host->volume;
        s->hist[3 * s->hist_n + 1] = s->stats_host->energy;
        s->hist[3 * s->hist_n + 2] = s->stats_host->particle_energy;
        s->hist_n++;
        h->stats_pending = false;
    }
    int e = *s->err_host;
    if (e) {
        FS2D_CUDA(cudaMemsetAsync(s->err, 0, sizeof(int), s->stream));
        if (e & 1) {
            const char* kind = (e & (kWaveKindCp << 4))      ? "closest-point"
                               : (e & (kWaveKindEik << 4))   ? "Eikonal"
                               : (e & (kWaveKindWave2 << 4)) ? "FP64 MIC(0)"
                               : (e & (kWaveKindMic32 << 4)) ? "FP32 MIC(0)"
                                                             : "wavefront";
            const char* what = (e & 256) ? "its neighbour strip" : (e & 512) ? "its own tile loads" : (e & 1024) ? "its other warp" : "a neighbour";
            set_error("a %s sweep timed out waiting for %s", kind, what);
            return FS2D_ERR_TIMEOUT;
        }
        if (e & 8) {
            set_error("the extrapolation timed out waiting between bands");
            return FS2D_ERR_TIMEOUT;
        }
        set_error("non-finite or out-of-domain particle position");
        return FS2D_ERR_NONFINITE;
    }
    return 0;
}

// Device scratch of the transfer transposes, freed when the call returns.
struct DevScratch {
    std::vector<void*> ptrs;
    ~DevScratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* get(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

Host* H(fs2d_sim* p) { return reinterpret_cast<Host*>(p); }

}  // namespace

// Stages k0 .. k1-1 of runFrame's order (k1 < 0: to the end), each between
// its two timing events.  With a pack solve in between (a batch), the
// projection stage is split: `solve_part` 1 runs its FP64 build and FP32
// setup and stops, 2 takes the finished solve's statistics and goes on.
// Records a stage-timing event on the handle's stream; inside a stream
// capture as an event node of the graph, so every replay records it.
static cudaError_t stage_event(Sim* s, cudaEvent_t e) {
    return s->capturing ? cudaEventRecordWithFlags(e, s->stream, cudaEventRecordExternal) : cudaEventRecord(e, s->stream);
}

int frame_stages(fs2d_sim* p, int k0, int k1, int* status, int solve_part) {
    Host* h = H(p);
    Sim* s = &h->sim;
    const int n = num_stages(s);
    const int* st = s->mode == FS2D_SEMILAGRANGIAN ? kSlStages : kPicStages;
    if (k1 < 0) k1 = n;
    for (int k = k0; k < k1; k++) {
        const bool split = solve_part != 0 && st[k] == FS2D_STAGE_APPLY_PROJECTION;
        if (!(split && solve_part == 2)) FS2D_CUDA(stage_event(s, s->ev[2 * k]));
        int sst = 0;
        int rc;
        if (split && solve_part == 1) {
            rc = projection_build(s);
            if (!rc) rc = mixed_setup(s);
            if (rc) return rc;
            return 0;   // the pack solve follows
        } else if (split) {
            // the solve's scalars are read when the frame closes (no wait here;
            // frame_mark(p, 2) flags them)
            rc = mixed_finish_queue(s);
        } else {
            rc = run_stage_impl(s, st[k], &sst);
        }
        if (rc) return rc;
        if (sst) *status = sst;
        FS2D_CUDA(stage_event(s, s->ev[2 * k + 1]));
        if (st[k] == FS2D_STAGE_CREATE_WATER_LEVEL_SET) h->stats_pending = true;
    }
    return 0;
}

// createWaterLevelSet (stage 0 in both modes) of a batch frame, around the
// batch's sweeps: part 1 records the stage's start and queues the seeds,
// part 2 the rest of the stage.
int frame_levelset(fs2d_sim* p, int part) {
    Host* h = H(p);
    Sim* s = &h->sim;
    if (part == 1) {
        FS2D_CUDA(stage_event(s, s->ev[0]));
        return levelset_seed(s);
    }
    int rc = levelset_finish(s);
    if (rc) return rc;
    FS2D_CUDA(stage_event(s, s->ev[1]));
    return 0;
}

// Host bookkeeping of a batch frame's phases (done on every frame, also when
// the phase's device work was replayed from a graph): 1 the level set's
// statistics are due at frame close, 2 so are the solve's scalars.
void frame_mark(fs2d_sim* p, int what) {
    Host* h = H(p);
    if (what == 1) h->stats_pending = true;
    if (what == 2) h->solve_pending = true;
}

int frame_solve_stage(fs2d_sim* p) {
    Sim* s = &H(p)->sim;
    const int* st = s->mode == FS2D_SEMILAGRANGIAN ? kSlStages : kPicStages;
    for (int k = 0; k < num_stages(s); k++)
        if (st[k] == FS2D_STAGE_APPLY_PROJECTION) return k;
    return -1;
}

// End of a frame: device error word, statistics, stage times, counters.
int frame_close(fs2d_sim* p, int rc, int status) {
    Host* h = H(p);
    Sim* s = &h->sim;
    if (rc) {
        h->solve_pending = false;
        return rc;
    }
    rc = finish(h);
    if (h->solve_pending) {   // the frame's solve scalars arrived with finish's wait
        int sst = 0;
        mixed_finish_read(s, &sst);
        if (!status) status = sst;
        h->solve_pending = false;
    }
    const int n = num_stages(s);
    for (int k = 0; k < n; k++) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, s->ev[2 * k], s->ev[2 * k + 1]) != cudaSuccess) {
            ms = 0;
            (void)cudaGetLastError();   // no stale error for the next call to pick up
        }
        s->stage_ms[k] = ms;
        h->frame_stage_ms.push_back(ms);
    }
    s->n_stage_times = n;
    s->current_time += s->dt;
    s->frames++;
    s->last_status = rc ? rc : status;
    return s->last_status;
}

Sim* sim_of(fs2d_sim* p) { return &H(p)->sim; }

}  // namespace fs2d

using namespace fs2d;

extern "C" {

void fs2d_default_options(fs2d_options* o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->precision = FS2D_PRECISION_FP64;
    o->mic_tau = 0.999;
    o->mic_sigma = 0.25;
    o->pcg_tol = 1e-12;
    o->pcg_max_iters = 200;
    o->ir_inner_tol = 1e-4;
    o->ir_max_outer = 30;
    o->p2g_mode = FS2D_P2G_ORDERED;
    o->extrapolate_band = 0;
    o->use_seed = 0;
    o->seed = 0;
    o->device = 0;
}

const char* fs2d_last_error(void) { return g_err; }

int fs2d_create(const fs2d_config* cfg, const fs2d_options* opt, fs2d_sim** out) {
    if (!cfg || !out) {
        set_error("fs2d_create: null argument");
        return FS2D_ERR_INVALID;
    }
    *out = nullptr;
    const int NX = cfg->sizeX, NY = cfg->sizeY;
    if (NX < 3 || NY < 3 || cfg->particlesPerCellSqrt < 1 || !(cfg->dx > 0) || !cfg->initialValues ||
        (cfg->mode != FS2D_SEMILAGRANGIAN && cfg->mode != FS2D_PICFLIP)) {
        set_error("fs2d_create: invalid configuration");
        return FS2D_ERR_INVALID;
    }
    if ((long long)NX * NY > (1ll << 28)) {
        set_error("fs2d_create: grid of %d x %d cells is too large", NX, NY);
        return FS2D_ERR_INVALID;
    }
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
            bool border = i == 0 || j == 0 || i == NX - 1 || j == NY - 1;
            uint8_t c = cfg->initialValues[(size_t)j * NX + i];
            if (c > FS2D_SOLID || (border && c != FS2D_SOLID)) {
                set_error("fs2d_create: label %d at (%d, %d): labels must be 0..2 and border cells SOLID", c, i, j);
                return FS2D_ERR_INVALID;
            }
        }
    fs2d_options o;
    if (opt) o = *opt; else fs2d_default_options(&o);
    if (o.precision != FS2D_PRECISION_FP64 && o.precision != FS2D_PRECISION_MIXED &&
        o.precision != FS2D_PRECISION_FP32) {
        set_error("fs2d_create: unknown precision mode %d", o.precision);
        return FS2D_ERR_INVALID;
    }
    if (!(o.pcg_tol >= 0) || o.pcg_max_iters < 0 || !(o.ir_inner_tol > 0) || o.ir_max_outer < 1) {
        set_error("fs2d_create: invalid solver options");
        return FS2D_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device) {
        set_error("fs2d_create: no CUDA device %d", o.device);
        return FS2D_ERR_CUDA;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, o.device) != cudaSuccess || !prop.cooperativeLaunch) {
        set_error("fs2d_create: device %d does not support cooperative launches", o.device);
        return FS2D_ERR_CUDA;
    }
    if (cudaSetDevice(o.device) != cudaSuccess) {
        set_error("fs2d_create: cudaSetDevice(%d) failed", o.device);
        return FS2D_ERR_CUDA;
    }
    Host* h = new (std::nothrow) Host();
    if (!h) {
        set_error("out of host memory");
        return FS2D_ERR_ALLOC;
    }
    Sim* s = &h->sim;
    s->device = o.device;
    s->opt = o;
    s->NX = NX;
    s->NY = NY;
    s->ppc_sqrt = cfg->particlesPerCellSqrt;
    s->mode = cfg->mode;
    s->dt = cfg->dt;
    s->dx = cfg->dx;
    s->dr = 0.9 * cfg->dx;
    s->rho = cfg->rho;
    s->gx = cfg->gravityX;
    s->gy = cfg->gravityY;
    s->alpha = cfg->picFlipAlpha;
    s->N = (size_t)NX * NY;
    s->NU = (size_t)(NX + 1) * NY;
    s->NV = (size_t)NX * (NY + 1);

    // particle seeding (src/FluidSim2D.cpp:49-69)
    if (o.use_seed) srand(o.seed);
    const int ppc = s->ppc_sqrt * s->ppc_sqrt;
    std::vector<double> pos;
    size_t fluid = 0;
    const float dist = 1.0f / s->ppc_sqrt;
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++)
            if (cfg->initialValues[(size_t)j * NX + i] == FS2D_FLUID) {
                fluid++;
                for (int k = 0; k < ppc; k++) {
                    int x = k % s->ppc_sqrt;
                    int y = k / s->ppc_sqrt;
                    double px = ((double)i + dist * x + randf(dist)) * s->dx;
                    double py = ((double)j + dist * y + randf(dist)) * s->dx;
                    pos.push_back(px);
                    pos.push_back(py);
                }
            }
    s->np = pos.size() / 2;
    s->orig_volume = fluid * s->dx * s->dx;

    int rc = check_cuda(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!rc) {
        s->stream = s->own_stream;
        for (auto& e : s->ev)
            if (!rc) rc = check_cuda(cudaEventCreate(&e), "cudaEventCreate");
    }
    if (!rc) rc = alloc_all(s);
    if (!rc) rc = alloc_particles(s, std::max<size_t>(s->np, 1024));
    if (!rc) rc = check_cuda(cudaMemcpy(s->cell, cfg->initialValues, s->N, cudaMemcpyHostToDevice), "upload cell");
    if (!rc && s->np)
        rc = check_cuda(cudaMemcpy(s->pos, pos.data(), s->np * sizeof(double2), cudaMemcpyHostToDevice), "upload pos");
    if (rc) {
        free_all(s);
        delete h;
        return rc;
    }
    s->stats_host->volume = s->orig_volume;
    // waterVolume before the first createWaterLevelSet is origWaterVolume (src/FluidSim2D.cpp:71-72)
    rc = check_cuda(cudaMemcpy(&s->stats->volume, &s->orig_volume, sizeof(double), cudaMemcpyHostToDevice),
                    "upload volume");
    if (rc) {
        free_all(s);
        delete h;
        return rc;
    }
    *out = reinterpret_cast<fs2d_sim*>(h);
    return FS2D_OK;
}

int fs2d_destroy(fs2d_sim* p) {
    if (!p) return FS2D_OK;
    Host* h = H(p);
    cudaSetDevice(h->sim.device);
    if (h->sim.stream) cudaStreamSynchronize(h->sim.stream);
    free_all(&h->sim);
    delete h;
    return FS2D_OK;
}

int fs2d_run_stage(fs2d_sim* p, int stage) {
    if (!p) return FS2D_ERR_INVALID;
    Host* h = H(p);
    Sim* s = &h->sim;
    int status = 0;
    int rc = run_stage_impl(s, stage, &status);
    if (rc) return rc;
    if (stage == FS2D_STAGE_CREATE_WATER_LEVEL_SET) h->stats_pending = true;
    rc = finish(h);
    return rc ? rc : status;
}

int fs2d_render_export(fs2d_sim* p, fs2d_render* r) {
    if (!p || !r) return FS2D_ERR_INVALID;
    return render_export(&H(p)->sim, r);
}

// Particle reseeding (include/fs2d.h): plan on the device (counts, removals,
// requests), one wait for the two totals, the new arrays written into
// scratch and copied over the handle's (grown first when they do not fit).
int fs2d_reseed(fs2d_sim* p, int minPerCell, int maxPerCell, unsigned int seed, fs2d_reseed_stats* out) {
    if (!p || minPerCell < 0 || minPerCell > 64 || maxPerCell < 0 || (maxPerCell > 0 && maxPerCell < minPerCell)) {
        set_error("fs2d_reseed: need 0 <= minPerCell <= 64 and maxPerCell == 0 or >= minPerCell");
        return FS2D_ERR_INVALID;
    }
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    const size_t N = s->N, np = s->np;
    // the scans below run over np + 1 particle words
    const size_t scan_need = std::max(N, np) / 4096 + 4;
    if (scan_need > s->scan_tmp_n) {
        cudaFree(s->scan_tmp);
        s->scan_tmp = nullptr;
        s->scan_tmp_n = 0;
        int rc = dalloc(&s->scan_tmp, scan_need);
        if (rc) return rc;
        s->scan_tmp_n = scan_need;
    }
    s->generation++;
    DevScratch mem;
    ReseedScratch x{mem.get<uint32_t>(N + 1), mem.get<uint32_t>(N + 1), mem.get<uint32_t>(N + 1),
                    mem.get<uint32_t>(N + 1), mem.get<uint32_t>(np + 1), mem.get<uint32_t>(np + 1)};
    if (!x.cnt || !x.start || !x.fill || !x.spawn || !x.bucket || !x.keep) {
        set_error("fs2d_reseed: out of device memory for scratch");
        return FS2D_ERR_ALLOC;
    }
    size_t n_keep = 0, n_add = 0;
    int rc = reseed_plan(s, x, minPerCell, maxPerCell, &n_keep, &n_add);
    if (rc) return rc;
    const size_t n = n_keep + n_add;
    double2* npos = mem.get<double2>(n);
    double2* nvel = mem.get<double2>(n);
    if (!npos || !nvel) {
        set_error("fs2d_reseed: out of device memory for %zu particles", n);
        return FS2D_ERR_ALLOC;
    }
    if ((rc = reseed_write(s, x, seed, npos, nvel))) return rc;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    if (n > s->np_cap && (rc = alloc_particles(s, n + n / 4))) return rc;
    if (n) {
        FS2D_CUDA(cudaMemcpyAsync(s->pos, npos, n * sizeof(double2), cudaMemcpyDeviceToDevice, s->stream));
        FS2D_CUDA(cudaMemcpyAsync(s->vel, nvel, n * sizeof(double2), cudaMemcpyDeviceToDevice, s->stream));
    }
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    s->np = n;
    if (out) {
        out->removed = np - n_keep;
        out->added = n_add;
        out->numParticles = n;
    }
    return FS2D_OK;
}

int fs2d_set_volume_correction(fs2d_sim* p, double rate) {
    if (!p || !(rate >= 0.0 && rate <= 1.0)) {
        set_error("fs2d_set_volume_correction: need 0 <= rate <= 1");
        return FS2D_ERR_INVALID;
    }
    Sim* s = &H(p)->sim;
    s->volume_rate = rate;
    s->generation++;   // captured phases take the rate by value
    return FS2D_OK;
}

int fs2d_solve_pressure(fs2d_sim* p, const uint8_t* cell, const double* phi, const double* u, const double* v,
                        double* pressure, fs2d_stats* stats) {
    if (!p || !cell || !phi || !u || !v || !pressure) {
        set_error("fs2d_solve_pressure: cell, phi, u, v and pressure are required");
        return FS2D_ERR_INVALID;
    }
    fs2d_state in{};
    in.cell = const_cast<uint8_t*>(cell);
    in.phi = const_cast<double*>(phi);
    in.u = const_cast<double*>(u);
    in.v = const_cast<double*>(v);
    int rc = fs2d_upload_state(p, &in);
    if (rc) return rc;
    const int status = fs2d_run_stage(p, FS2D_STAGE_APPLY_PROJECTION);
    H(p)->sim.last_status = status;
    if (status && status != FS2D_ERR_NOT_CONVERGED) return status;
    fs2d_state out{};
    out.p = pressure;
    rc = fs2d_download_state(p, &out);
    if (rc) return rc;
    if (stats) {
        rc = fs2d_get_stats(p, stats);
        if (rc) return rc;
    }
    return status;
}

int fs2d_forward(fs2d_sim* p, int steps, int checkpointEvery, const double* u0, const double* v0,
                 const double* uTarget, const double* vTarget, double* loss) {
    if (!p || !loss) {
        set_error("fs2d_forward: handle and loss are required");
        return FS2D_ERR_INVALID;
    }
    Host* h = H(p);
    int rc = rollout_forward(&h->sim, steps, checkpointEvery, u0, v0, uTarget, vTarget, loss);
    int rc2 = finish(h);
    return rc ? rc : rc2;
}


int fs2d_p2g_adjoint(fs2d_sim* p, const double* uBar, const double* vBar, double* particleVelsBar) {
    if (!p || !uBar || !vBar || !particleVelsBar) {
        set_error("fs2d_p2g_adjoint: uBar, vBar and particleVelsBar are required");
        return FS2D_ERR_INVALID;
    }
    Host* h = H(p);
    Sim* s = &h->sim;
    DevScratch sc;
    double *mu = sc.get<double>(s->NU), *mv = sc.get<double>(s->NV), *wu = sc.get<double>(s->NU),
           *wv = sc.get<double>(s->NV);
    double2* vb = sc.get<double2>(s->np);
    if (!mu || !mv || !wu || !wv || !vb) {
        set_error("fs2d_p2g_adjoint: device scratch allocation failed");
        return FS2D_ERR_ALLOC;
    }
    FS2D_CUDA(cudaMemcpyAsync(mu, uBar, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(mv, vBar, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    int rc = p2g_adjoint(s, mu, mv, wu, wv, vb);
    if (rc) return rc;
    if (s->np > 0)
        FS2D_CUDA(cudaMemcpyAsync(particleVelsBar, vb, s->np * sizeof(double2), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return finish(h);
}

int fs2d_g2p_adjoint(fs2d_sim* p, const double* particleVelsBar, double* newUBar, double* newVBar, double* uBar,
                     double* vBar, double* particleVelsInBar) {
    if (!p || !particleVelsBar || !newUBar || !newVBar || !uBar || !vBar || !particleVelsInBar) {
        set_error("fs2d_g2p_adjoint: every array is required");
        return FS2D_ERR_INVALID;
    }
    Host* h = H(p);
    Sim* s = &h->sim;
    DevScratch sc;
    double *nub = sc.get<double>(s->NU), *nvb = sc.get<double>(s->NV), *ub = sc.get<double>(s->NU),
           *vb = sc.get<double>(s->NV);
    double2 *gb = sc.get<double2>(s->np), *ib = sc.get<double2>(s->np);
    if (!nub || !nvb || !ub || !vb || !gb || !ib) {
        set_error("fs2d_g2p_adjoint: device scratch allocation failed");
        return FS2D_ERR_ALLOC;
    }
    if (s->np > 0)
        FS2D_CUDA(cudaMemcpyAsync(gb, particleVelsBar, s->np * sizeof(double2), cudaMemcpyDefault, s->stream));
    int rc = g2p_adjoint(s, gb, nub, nvb, ub, vb, ib);
    if (rc) return rc;
    FS2D_CUDA(cudaMemcpyAsync(newUBar, nub, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(newVBar, nvb, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(uBar, ub, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(vBar, vb, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    if (s->np > 0)
        FS2D_CUDA(cudaMemcpyAsync(particleVelsInBar, ib, s->np * sizeof(double2), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return finish(h);
}

int fs2d_backward(fs2d_sim* p, double* gradU0, double* gradV0) {
    if (!p) return FS2D_ERR_INVALID;
    Host* h = H(p);
    int rc = rollout_backward(&h->sim, gradU0, gradV0);
    int rc2 = finish(h);
    return rc ? rc : rc2;
}

int fs2d_run_frame(fs2d_sim* p) {
    if (!p) return FS2D_ERR_INVALID;
    int status = 0;
    int rc = frame_stages(p, 0, -1, &status);
    return frame_close(p, rc, status);
}

int fs2d_step(fs2d_sim* p, int nframes) {
    int last = 0;
    for (int k = 0; k < nframes; k++) {
        int rc = fs2d_run_frame(p);
        if (rc && rc != FS2D_ERR_NOT_CONVERGED) return rc;
        if (rc) last = rc;
    }
    return last;
}

int fs2d_num_particles(fs2d_sim* p, size_t* n) {
    if (!p || !n) return FS2D_ERR_INVALID;
    *n = H(p)->sim.np;
    return FS2D_OK;
}

int fs2d_upload_state(fs2d_sim* p, const fs2d_state* st) {
    if (!p || !st) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    s->generation++;
    auto up = [&](void* d, const void* src, size_t bytes) -> int {
        if (!src) return 0;
        return check_cuda(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, s->stream), "upload");
    };
    int rc = 0;
    if (st->cell) {
        for (int j = 0; j < s->NY && !rc; j++)
            for (int i = 0; i < s->NX; i++) {
                bool border = i == 0 || j == 0 || i == s->NX - 1 || j == s->NY - 1;
                uint8_t c = st->cell[(size_t)j * s->NX + i];
                if (c > FS2D_SOLID || (border && c != FS2D_SOLID)) {
                    set_error("fs2d_upload_state: label %d at (%d, %d)", c, i, j);
                    return FS2D_ERR_INVALID;
                }
            }
    }
    rc = rc ? rc : up(s->cell, st->cell, s->N);
    rc = rc ? rc : up(s->phi, st->phi, s->N * sizeof(double));
    rc = rc ? rc : up(s->p, st->p, s->N * sizeof(double));
    rc = rc ? rc : up(s->u, st->u, s->NU * sizeof(double));
    rc = rc ? rc : up(s->v, st->v, s->NV * sizeof(double));
    rc = rc ? rc : up(s->nu, st->newU, s->NU * sizeof(double));
    rc = rc ? rc : up(s->nv, st->newV, s->NV * sizeof(double));
    if (rc) return rc;
    if (st->particles && st->particleVels) {
        size_t n = st->numParticles;
        if (n > s->np_cap) {
            FS2D_CUDA(cudaStreamSynchronize(s->stream));
            rc = alloc_particles(s, n + n / 4);
            if (rc) return rc;
        }
        s->np = n;
        if (n) {
            rc = up(s->pos, st->particles, n * sizeof(double2));
            rc = rc ? rc : up(s->vel, st->particleVels, n * sizeof(double2));
        }
    } else if (st->particles || st->particleVels) {
        set_error("fs2d_upload_state: particles and particleVels must be given together");
        return FS2D_ERR_INVALID;
    }
    if (rc) return rc;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return FS2D_OK;
}

int fs2d_download_state(fs2d_sim* p, fs2d_state* st) {
    if (!p || !st) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    if ((st->particles || st->particleVels) && st->numParticles < s->np) {
        set_error("fs2d_download_state: particle buffers hold %zu, need %zu", st->numParticles, s->np);
        st->numParticles = s->np;
        return FS2D_ERR_INVALID;
    }
    auto dn = [&](void* dst, const void* d, size_t bytes) -> int {
        if (!dst || !bytes) return 0;
        return check_cuda(cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, s->stream), "download");
    };
    int rc = dn(st->cell, s->cell, s->N);
    rc = rc ? rc : dn(st->phi, s->phi, s->N * sizeof(double));
    rc = rc ? rc : dn(st->p, s->p, s->N * sizeof(double));
    rc = rc ? rc : dn(st->u, s->u, s->NU * sizeof(double));
    rc = rc ? rc : dn(st->v, s->v, s->NV * sizeof(double));
    rc = rc ? rc : dn(st->newU, s->nu, s->NU * sizeof(double));
    rc = rc ? rc : dn(st->newV, s->nv, s->NV * sizeof(double));
    rc = rc ? rc : dn(st->particles, s->pos, s->np * sizeof(double2));
    rc = rc ? rc : dn(st->particleVels, s->vel, s->np * sizeof(double2));
    if (rc) return rc;
    st->numParticles = s->np;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return FS2D_OK;
}

int fs2d_set_params(fs2d_sim* p, double gx, double gy, double alpha, double dt) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    s->gx = gx;
    s->gy = gy;
    s->alpha = alpha;
    s->dt = dt;
    s->generation++;
    return FS2D_OK;
}

int fs2d_get_stats(fs2d_sim* p, fs2d_stats* out) {
    if (!p || !out) return FS2D_ERR_INVALID;
    Host* h = H(p);
    Sim* s = &h->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    out->waterVolume = s->stats_host->volume;
    out->totalEnergy = s->stats_host->energy;
    out->particleTotalEnergy = s->stats_host->particle_energy;
    out->origWaterVolume = s->orig_volume;
    out->currentTime = s->current_time;
    out->frames = s->frames;
    out->pcgIterations = s->last_iters;
    out->irOuterIterations = s->last_outer;
    out->pcgRelResidual = s->last_rel_res;
    out->lastStatus = s->last_status;
    return FS2D_OK;
}

int fs2d_get_history(fs2d_sim* p, double* vol, double* en, double* pen, size_t cap, size_t* n) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    size_t m = std::min(cap, s->hist_n);
    for (size_t k = 0; k < m; k++) {
        if (vol) vol[k] = s->hist[3 * k];
        if (en) en[k] = s->hist[3 * k + 1];
        if (pen) pen[k] = s->hist[3 * k + 2];
    }
    if (n) *n = s->hist_n;
    return FS2D_OK;
}

static int run_diag(fs2d_sim* p) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    int rc = diagnostics(s);
    if (rc) return rc;
    FS2D_CUDA(cudaMemcpyAsync(s->stats_host, s->stats, sizeof(FrameStats), cudaMemcpyDeviceToHost, s->stream));
    if (int rcw = wait_stream(s, s->stream)) return rcw;
    return FS2D_OK;
}

int fs2d_avg_pressure(fs2d_sim* p, double* out) {
    int rc = run_diag(p);
    if (!rc && out) *out = H(p)->sim.stats_host->avg_p;
    return rc;
}
int fs2d_avg_pressure_in_fluid(fs2d_sim* p, double* out) {
    int rc = run_diag(p);
    if (!rc && out) *out = H(p)->sim.stats_host->avg_p_fluid;
    return rc;
}
int fs2d_max_velocity(fs2d_sim* p, double* out) {
    int rc = run_diag(p);
    if (!rc && out) *out = H(p)->sim.stats_host->max_vel;
    return rc;
}

int fs2d_cfl(fs2d_sim* p, double* cfl, long long* particle) {
    if (!p) return FS2D_ERR_INVALID;
    double c = 0;
    long long e = -1;
    int rc = cfl_check(&H(p)->sim, &c, &e);
    if (rc) return rc;
    if (cfl) *cfl = c;
    if (particle) *particle = e;
    return FS2D_OK;
}

int fs2d_debug_fail_alloc(long long after) {
    g_alloc_budget.store(after < 0 ? -1 : after);
    return FS2D_OK;
}

// ---- checkpoint and resume ----

}  // extern "C"

namespace {

struct CheckpointHeader {
    char magic[8];            // "FS2DCKP1"
    uint32_t version;         // 1
    uint32_t header_bytes;    // sizeof(CheckpointHeader)
    int32_t NX, NY, mode, pad;
    uint64_t num_particles;
    int64_t frames;
    double dt, dx, rho, gx, gy, alpha, current_time, orig_volume, water_volume, volume_rate;
};
constexpr char kCheckpointMagic[8] = {'F', 'S', '2', 'D', 'C', 'K', 'P', '1'};

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

// The arrays of a checkpoint after its header, in order: cell (padded to 8
// bytes), phi, p, u, v, newU, newV, particles, particleVels.
struct CheckpointArrays {
    std::vector<uint8_t> cell;
    std::vector<double> phi, p, u, v, nu, nv, pos, vel;
    CheckpointArrays(const Sim* s, size_t np)
        : cell((s->N + 7) / 8 * 8), phi(s->N), p(s->N), u(s->NU), v(s->NV), nu(s->NU), nv(s->NV), pos(2 * np),
          vel(2 * np) {}
    fs2d_state view(size_t np) {
        fs2d_state st{};
        st.cell = cell.data();
        st.phi = phi.data();
        st.p = p.data();
        st.u = u.data();
        st.v = v.data();
        st.newU = nu.data();
        st.newV = nv.data();
        st.particles = np ? pos.data() : nullptr;
        st.particleVels = np ? vel.data() : nullptr;
        st.numParticles = np;
        return st;
    }
    template <typename Fn>
    bool each(Fn fn) {
        return fn(cell.data(), cell.size()) && fn(phi.data(), phi.size() * 8) && fn(p.data(), p.size() * 8) &&
               fn(u.data(), u.size() * 8) && fn(v.data(), v.size() * 8) && fn(nu.data(), nu.size() * 8) &&
               fn(nv.data(), nv.size() * 8) && fn(pos.data(), pos.size() * 8) && fn(vel.data(), vel.size() * 8);
    }
};

// Bytes after the header: exactly what CheckpointArrays::each reads or writes.
size_t checkpoint_payload_bytes(const Sim* s, size_t np) {
    return (s->N + 7) / 8 * 8 + sizeof(double) * (2 * s->N + 2 * s->NU + 2 * s->NV + 4 * np);
}

}  // namespace

extern "C" {

int fs2d_save_checkpoint(fs2d_sim* p, const char* path) try {
    if (!p || !path) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    const size_t np = s->np;
    CheckpointArrays a(s, np);
    fs2d_state st = a.view(np);
    int rc = fs2d_download_state(p, &st);
    if (rc) return rc;
    FrameStats fs;
    FS2D_CUDA(cudaMemcpyAsync(&fs, s->stats, sizeof(fs), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    CheckpointHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCheckpointMagic, 8);
    h.version = 1;
    h.header_bytes = sizeof(h);
    h.NX = s->NX;
    h.NY = s->NY;
    h.mode = s->mode;
    h.num_particles = np;
    h.frames = s->frames;
    h.dt = s->dt;
    h.dx = s->dx;
    h.rho = s->rho;
    h.gx = s->gx;
    h.gy = s->gy;
    h.alpha = s->alpha;
    h.current_time = s->current_time;
    h.orig_volume = s->orig_volume;
    h.water_volume = fs.volume;
    h.volume_rate = s->volume_rate;
    File f;
    f.f = fopen(path, "wb");
    if (!f.f) {
        set_error("fs2d_save_checkpoint: cannot open %s for writing", path);
        return FS2D_ERR_INVALID;
    }
    bool ok = fwrite(&h, sizeof(h), 1, f.f) == 1 &&
              a.each([&](const void* d, size_t n) { return n == 0 || fwrite(d, 1, n, f.f) == n; });
    ok = (fclose(f.f) == 0) && ok;
    f.f = nullptr;
    if (!ok) {
        set_error("fs2d_save_checkpoint: writing %s failed", path);
        return FS2D_ERR_INVALID;
    }
    return FS2D_OK;
} catch (const std::bad_alloc&) {
    set_error("fs2d_save_checkpoint: out of host memory");
    return FS2D_ERR_ALLOC;
}

int fs2d_load_checkpoint(fs2d_sim* p, const char* path) try {
    if (!p || !path) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    File f;
    f.f = fopen(path, "rb");
    if (!f.f) {
        set_error("fs2d_load_checkpoint: cannot open %s", path);
        return FS2D_ERR_INVALID;
    }
    CheckpointHeader h;
    if (fread(&h, sizeof(h), 1, f.f) != 1 || memcmp(h.magic, kCheckpointMagic, 8) != 0 || h.version != 1 ||
        h.header_bytes != sizeof(h)) {
        set_error("fs2d_load_checkpoint: %s is not a version-1 checkpoint", path);
        return FS2D_ERR_INVALID;
    }
    if (h.NX != s->NX || h.NY != s->NY || h.mode != s->mode || h.dx != s->dx || h.rho != s->rho) {
        set_error("fs2d_load_checkpoint: %s holds a %d x %d grid (mode %d, dx %g, rho %g); the handle's is %d x %d "
                  "(mode %d, dx %g, rho %g)",
                  path, h.NX, h.NY, h.mode, h.dx, h.rho, s->NX, s->NY, s->mode, s->dx, s->rho);
        return FS2D_ERR_INVALID;
    }
    if (h.num_particles > ((size_t)1 << 40)) {
        set_error("fs2d_load_checkpoint: %s: implausible particle count", path);
        return FS2D_ERR_INVALID;
    }
    const size_t np = (size_t)h.num_particles;
    // the file holds exactly the header and the arrays it announces: checked
    // before any buffer is sized from the header
    long long file_bytes = -1;
    if (fseek(f.f, 0, SEEK_END) == 0) file_bytes = (long long)ftell(f.f);
    if (file_bytes != (long long)(sizeof(h) + checkpoint_payload_bytes(s, np)) ||
        fseek(f.f, (long)sizeof(h), SEEK_SET) != 0) {
        set_error("fs2d_load_checkpoint: %s is truncated or too long for %zu particles", path, np);
        return FS2D_ERR_INVALID;
    }
    CheckpointArrays a(s, np);
    bool ok = a.each([&](void* d, size_t n) { return n == 0 || fread(d, 1, n, f.f) == n; });
    if (!ok || fgetc(f.f) != EOF) {
        set_error("fs2d_load_checkpoint: %s is truncated or too long", path);
        return FS2D_ERR_INVALID;
    }
    fs2d_state st = a.view(np);
    int rc = fs2d_upload_state(p, &st);
    if (rc) return rc;
    if (!np) s->np = 0;   // fs2d_upload_state leaves the particles when none are given
    s->gx = h.gx;
    s->gy = h.gy;
    s->alpha = h.alpha;
    s->dt = h.dt;
    s->current_time = h.current_time;
    s->frames = h.frames;
    s->orig_volume = h.orig_volume;
    s->volume_rate = h.volume_rate;
    s->generation++;
    s->stats_host->volume = h.water_volume;
    FS2D_CUDA(cudaMemcpyAsync(&s->stats->volume, &s->stats_host->volume, sizeof(double), cudaMemcpyHostToDevice,
                              s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return FS2D_OK;
} catch (const std::bad_alloc&) {
    set_error("fs2d_load_checkpoint: out of host memory");
    return FS2D_ERR_ALLOC;
}

int fs2d_get_stage_times(fs2d_sim* p, float* ms, int cap, int* n) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    for (int k = 0; k < std::min(cap, s->n_stage_times); k++) ms[k] = s->stage_ms[k];
    if (n) *n = s->n_stage_times;
    return FS2D_OK;
}

// PerformanceCounter (src/PerformanceCounter.cpp:16-74): a 30-frame ring of
// stage times, averaged once the ring is full; saveToFile writes one row per
// frame from frame 30 on, each stage's average followed by ','.  The
// conservation file follows FluidSim2D::saveStats (src/FluidSim2D.cpp:738-750).
int fs2d_write_stats(const float* stage_ms, int ns, size_t frames, const double* vol, const double* en,
                     const double* pen, size_t n, const char* perf_path, const char* cons_path) {
    if ((perf_path && (ns < 1 || (frames > 0 && !stage_ms))) || (cons_path && n > 0 && (!vol || !en || !pen))) {
        set_error("fs2d_write_stats: missing series");
        return FS2D_ERR_INVALID;
    }
    if (perf_path) {
        const int kSamples = 30;
        std::vector<float> ring((size_t)ns * kSamples, 0.0f), avg(ns, 0.0f);
        std::string buf;
        bool finished = false;
        for (size_t f = 0; f < frames; f++) {
            int slot = (int)(f % kSamples);
            for (int k = 0; k < ns; k++) ring[(size_t)k * kSamples + slot] = stage_ms[f * ns + k];
            if (finished) {
                for (int k = 0; k < ns; k++) {
                    float a = 0.0f;
                    for (int m = 0; m < kSamples; m++) a += ring[(size_t)k * kSamples + m];
                    avg[k] = a / kSamples;
                }
            }
            if (slot == kSamples - 1) finished = true;
            if (f >= (size_t)kSamples) {
                for (int k = 0; k < ns; k++) {
                    buf += std::to_string(avg[k]);
                    buf += ',';
                }
                buf += '\n';
            }
        }
        FILE* fp = fopen(perf_path, "w+");
        if (!fp) {
            set_error("cannot open %s", perf_path);
            return FS2D_ERR_INVALID;
        }
        fputs(buf.c_str(), fp);
        fclose(fp);
    }
    if (cons_path) {
        FILE* fp = fopen(cons_path, "w+");
        if (!fp) {
            set_error("cannot open %s", cons_path);
            return FS2D_ERR_INVALID;
        }
        fputs("Total Volume, Total Energy, Total Energy (Particle) \n", fp);
        for (size_t k = 0; k < n; k++) fprintf(fp, "%f, %f, %f\n", vol[k], en[k], pen[k]);
        fclose(fp);
    }
    return FS2D_OK;
}

int fs2d_save_stats(fs2d_sim* p, const char* perf_path, const char* cons_path) {
    if (!p) return FS2D_ERR_INVALID;
    Host* h = H(p);
    Sim* s = &h->sim;
    const int ns = num_stages(s);
    std::vector<double> vol(s->hist_n), en(s->hist_n), pen(s->hist_n);
    for (size_t k = 0; k < s->hist_n; k++) {
        vol[k] = s->hist[3 * k];
        en[k] = s->hist[3 * k + 1];
        pen[k] = s->hist[3 * k + 2];
    }
    return fs2d_write_stats(h->frame_stage_ms.data(), ns, h->frame_stage_ms.size() / ns, vol.data(), en.data(),
                            pen.data(), s->hist_n, perf_path, cons_path);
}

int fs2d_debug_wavefront(fs2d_sim* p, long long polls, int holdKinds, int holdStrip) {
    if (!p || holdKinds < 0 || holdKinds > 15) {
        set_error("fs2d_debug_wavefront: invalid arguments");
        return FS2D_ERR_INVALID;
    }
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return set_wave_controls(s, polls > 0 ? polls : kWaveSpinLimit, holdKinds, holdKinds ? holdStrip : -1);
}

int fs2d_set_stream(fs2d_sim* p, void* stream) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    s->stream = stream ? (cudaStream_t)stream : s->own_stream;
    return FS2D_OK;
}

int fs2d_launch_count(fs2d_sim* p, unsigned long long* out) {
    if (!p || !out) return FS2D_ERR_INVALID;
    *out = H(p)->sim.launches;
    return FS2D_OK;
}

int fs2d_set_kernel_timing(fs2d_sim* p, const char* patterns) {
    if (!p) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    ktimer_collect(s);
    s->kt_patterns = patterns ? patterns : "";
    s->generation++;
    s->kt_match.clear();
    s->kt_acc.clear();
    return FS2D_OK;
}

int fs2d_get_kernel_times(fs2d_sim* p, char* buf, size_t cap) {
    if (!p || !buf || cap == 0) return FS2D_ERR_INVALID;
    Sim* s = &H(p)->sim;
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    ktimer_collect(s);
    std::string out;
    for (auto& kv : s->kt_acc) {
        char line[256];
        snprintf(line, sizeof(line), "%s %lld %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
        out += line;
    }
    s->kt_acc.clear();
    if (out.size() + 1 > cap) {
        set_error("fs2d_get_kernel_times: buffer of %zu bytes too small", cap);
        return FS2D_ERR_INVALID;
    }
    memcpy(buf, out.c_str(), out.size() + 1);
    return FS2D_OK;
}

}  // extern "C"
