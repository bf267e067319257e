// levelset.cu — FluidSim2D::createWaterLevelSet on the GPU (FP64, exact).
//
// Restates, kernel by kernel:
//   LevelSet::constructFromParticles   src/FluidSim2D.cpp:752-794
//   LevelSet::fastSweepIterate         include/FluidSim2D.h:178-203
//   LevelSet::redistance               src/FluidSim2D.cpp:796-920
//   labels + conservation statistics   src/FluidSim2D.cpp:653-664,709-731
// Compiled with --fmad=false; the result (phi, labels) is bit-identical to
// the reference's serial loops:
//   * the per-cell seed minimum is an atomic minimum on an order-preserving
//     integer image of d, then an atomic minimum of the particle index among
//     the particles that reach it — the same (smallest d, then first index)
//     winner as the reference's "if (d < phi)" loop;
//   * every Gauss-Seidel sweep runs as a strip wavefront, which visits each
//     cell after exactly the neighbours the serial loop visits before it;
//   * the closest-point sweeps carry the particle index alone and decide
//     each "d(e) < phi" from FP32 squared distances with a rigorous error
//     bound, falling back to the FP64 expression when the bound cannot
//     decide (cp_sweep.cuh); phi = d(t) is evaluated once at the end;
//   * a sweep that would change no cell is skipped: a parallel check first
//     evaluates every cell's update against the current values, and if none
//     would change, the serial sweep would not change anything either.
#include <cuda_runtime.h>
#include <math.h>
#include <limits.h>
#include <string.h>
#include <algorithm>
#include "fs2d_device.cuh"
#include "wave2.cuh"
#include "cp_sweep.cuh"
#include "eik_sweep.cuh"

namespace fs2d {
namespace {

__device__ __forceinline__ unsigned long long order_key(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
// Seeds (src/FluidSim2D.cpp:763-773).  t is pitched (row pitch P); the
// padding columns stay -1.
__global__ void k_seed_init(int* t, unsigned long long* key, int NX, int NY, int P) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= (size_t)P * NY) return;
    t[c] = INT_MAX;
    if (c < (size_t)NX * NY) key[c] = ~0ull;
}

__global__ void k_seed_min(const double2* __restrict__ pos, size_t np, unsigned long long* key, int NX, int NY,
                           double dx, double dr, int* err) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    int x = (int)(p.x / dx), y = (int)(p.y / dx);
    if (x < 0 || x >= NX || y < 0 || y >= NY) { atomicOr(err, 4); return; }
    atomicMin(key + (size_t)y * NX + x, order_key(corner_dist(p, x, y, dx, dr)));
}

__global__ void k_seed_idx(const double2* __restrict__ pos, size_t np, const unsigned long long* __restrict__ key,
                           int* t, int NX, int NY, int P, double dx, double dr) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    int x = (int)(p.x / dx), y = (int)(p.y / dx);
    if (x < 0 || x >= NX || y < 0 || y >= NY) return;
    if (order_key(corner_dist(p, x, y, dx, dr)) == key[(size_t)y * NX + x]) atomicMin(t + (size_t)y * P + x, (int)e);
}

__global__ void k_seed_write(int* t, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n) return;
    if (t[c] == INT_MAX) t[c] = -1;
}

// ---- closest-point propagation (the fastSweepIterate lambda) ----

// Float-pair positions (h = nearest float, l = nearest float of the rest)
// and the largest |h| over all particles.
__device__ __forceinline__ float2 split_f2(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
}

__global__ void k_posdf(const double2* __restrict__ pos, size_t np, float4* pos_df, CpConst* kc) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    float m = 0.f;
    if (e < np) {
        const double2 p = pos[e];
        const float2 x = split_f2(p.x), y = split_f2(p.y);
        pos_df[e] = make_float4(x.x, x.y, y.x, y.y);
        m = fmaxf(fabsf(x.x), fabsf(y.x));
        if (!(m <= 3.0e38f)) m = INFINITY;   // NaN or overflow: no fast decisions
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(&kc->amax, __float_as_uint(m));
}

// Corner coordinate tables and the constants of the FP32 decision.
__global__ void k_cp_tabs(float2* xtab, float2* ytab, int P, int NY, double dx) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < P) xtab[k] = split_f2(k * dx);
    if (k < NY) ytab[k] = split_f2(k * dx);
}

__global__ void k_cp_const(CpConst* kc, int NX, int NY, double dx, double dr) {
    const double grid = (double)(NX > NY ? NX : NY) * dx;
    double A = fmax((double)__uint_as_float(kc->amax), grid) * (1.0 + 0x1p-20);
    const bool ok = isfinite(dr) && isfinite(A) && A < 0x1p60;
    kc->fast = ok ? 1 : 0;
    if (!ok) A = 1.0;
    kc->A42 = __double2float_ru(A * 0x1p-42);
    kc->C0 = __double2float_ru(A * A * 0x1p-80 + 0x1p-120);
    kc->tiny_q = ok ? __double2float_ru(dr * dr * 0x1p-20) : INFINITY;
}

// Would any cell change under one closest-point update with the current
// values?  (Every candidate in the reference's order, against the cell's own.)
__global__ void k_cp_check(const int* __restrict__ t, const float4* __restrict__ pos_df,
                           const double2* __restrict__ pos, const float2* __restrict__ xtab,
                           const float2* __restrict__ ytab, const CpConst* __restrict__ kcp, int NX, int NY, int P,
                           double dx, double dr, int* noop) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    const CpConst kc = *kcp;
    const size_t c = (size_t)j * P + i;
    const float2 xc = xtab[i], yc = ytab[j];
    CpCur cur;
    cur.t = t[c];
    const int own = cur.t;
    cur.q = cur.E = 0.f;
    cur.p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (own >= 0) {
        cur.p = pos_df[own];
        cp_q32(cur.p, xc, yc, kc, cur.q, cur.E);
    }
    const int nb[4] = {i > 0 ? t[c - 1] : -1, i < NX - 1 ? t[c + 1] : -1, j > 0 ? t[c - P] : -1,
                       j < NY - 1 ? t[c + P] : -1};
    float4 np4[4];
#pragma unroll
    for (int k = 0; k < 4; k++) np4[k] = nb[k] >= 0 ? pos_df[nb[k]] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 own_p = cur.p;
    bool und = false;
#pragma unroll
    for (int k = 0; k < 4; k++) cp_offer_fast(nb[k], np4[k], true, cur, xc, yc, kc, und);
    if (und) {
        float4 sp;
        cur.t = cp_cell_slow(own, own_p, nb[0], np4[0], true, nb[1], np4[1], true, nb[2], np4[2], true, nb[3], np4[3],
                             true, xc, yc, kc, pos, i, j, dx, dr, &sp);
    }
    if (cur.t != own) *noop = 0;
}

// phi = d(t) of every cell (HUGE_VAL without a particle), as the reference
// stores it with t.
__global__ void k_cp_phi(const int* __restrict__ t, const double2* __restrict__ pos, size_t np, double* phi, int NX,
                         int NY, int P, double dx, double dr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    const int e = t[(size_t)j * P + i];
    phi[(size_t)j * NX + i] = (e < 0 || (size_t)e >= np) ? HUGE_VAL : corner_dist(pos[e], i, j, dx, dr);
}

// ---- redistance ----

// Surface flags from the sign changes the reference tests
// (src/FluidSim2D.cpp:803-834: pairs with the base cell in [0,NX-2]x[0,NY-2]),
// then non-surface negative cells -> -inf (:836-842).  Reads phi, writes out.
__global__ void k_surface(const double* __restrict__ phi, double* out, int NX, int NY, int P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    size_t c = (size_t)j * NX + i;
    double p = phi[c];
    bool surf = false;
    if (i <= NX - 2 && j <= NY - 2 && p * phi[c + 1] < 0) surf = true;
    if (i >= 1 && j <= NY - 2 && phi[c - 1] * p < 0) surf = true;
    if (i <= NX - 2 && j <= NY - 2 && p * phi[c + NX] < 0) surf = true;
    if (i <= NX - 2 && j >= 1 && phi[c - NX] * p < 0) surf = true;
    out[(size_t)j * P + i] = (!surf && p < 0) ? -HUGE_VAL : p;
}

// One Eikonal update (src/FluidSim2D.cpp:848-857); a = upwind x neighbour,
// b = upwind y neighbour.  Returns the cell's (possibly new) value.
__device__ __forceinline__ double eikonal(double own, double a, double b, double dx) {
    if (own >= 0) return own;
    double fa = fabs(a), fb = fabs(b);
    double phi0 = dmin(fa, fb);
    double phi1 = dmax(fa, fb);
    double d = phi0 + dx;
    if (d > phi1) d = 0.5 * (phi0 + phi1 + sqrt(2 * dx * dx - (phi1 - phi0) * (phi1 - phi0)));
    return (d < -own) ? -d : own;
}


__global__ void k_eik_check(const double* __restrict__ phi, uint8_t* mask, int NX, int NY, int P, int i_lo,
                            int i_hi, int j_lo, int j_hi, int sx, int sy, double dx, int* noop) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    size_t c = (size_t)j * P + i;
    bool ch = false;
    if (i >= i_lo && i <= i_hi && j >= j_lo && j <= j_hi) {
        double own = phi[c];
        if (own < 0) {
            double nv = eikonal(own, phi[c - sx], phi[(size_t)(j - sy) * P + i], dx);
            ch = nv != own;
        }
    }
    mask[c] = ch ? 1 : 0;
    if (ch) *noop = 0;
}

// Min-smoothing pass (src/FluidSim2D.cpp:904-919): Jacobi, interior cells.
__global__ void k_smooth(const double* __restrict__ oldp, int pin, double* out, int NX, int NY) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    size_t c = (size_t)j * pin + i;
    double o = oldp[c];
    if (i >= 1 && i <= NX - 2 && j >= 1 && j <= NY - 2) {
        double avg = 0.25 * (oldp[c - 1] + oldp[c + 1] + oldp[c - pin] + oldp[c + pin]);
        if (avg < o) o = avg;
    }
    out[(size_t)j * NX + i] = o;
}

// Labels (src/FluidSim2D.cpp:657-664) and grid statistics (:709-722).
// Copies the final level set into phi.
__global__ void k_labels_stats(const double* __restrict__ phis, double* phi, uint8_t* cell,
                               const double* __restrict__ u, const double* __restrict__ v, int NX, int NY,
                               double dx, double rho, double gx, double gy, double* partial, FrameStats* st) {
    __shared__ double sh[32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    double vol = 0, en = 0;
    if (i < NX) {
        size_t c = (size_t)j * NX + i;
        double p = phis[c];
        phi[c] = p;
        uint8_t lab = cell[c];
        if (lab != kSolid) {
            lab = p < 0.0 ? kFluid : kEmpty;
            cell[c] = lab;
        }
        if (lab == kFluid) {
            vol = dx * dx;
            double x = i * dx, y = j * dx;
            double vx = vel_interp_u(u, NX, NY, dx, x, y);
            double vy = vel_interp_v(v, NX, NY, dx, x, y);
            en = 0.5 * (rho * dx * dx) * (vx * vx + vy * vy) - (rho * dx * dx) * (gx * (i * dx) + gy * (j * dx));
        }
    }
    double a = block_sum(vol, sh);
    double b = block_sum(en, sh);
    size_t blk = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
        partial[2 * blk] = a;
        partial[2 * blk + 1] = b;
    }
    if (last_block(&st->ticket)) {
        size_t nb = (size_t)gridDim.x * gridDim.y;
        double sa = 0, sb = 0;
        for (size_t k = threadIdx.x; k < nb; k += blockDim.x) {
            sa += partial[2 * k];
            sb += partial[2 * k + 1];
        }
        sa = block_sum(sa, sh);
        sb = block_sum(sb, sh);
        if (threadIdx.x == 0) {
            st->volume = sa;
            st->energy = sb;
        }
    }
}

// Particle energy (src/FluidSim2D.cpp:723-728).
__global__ void k_particle_energy(const double2* __restrict__ pos, const double2* __restrict__ vel, size_t np,
                                  double m, double gx, double gy, double* partial, FrameStats* st) {
    __shared__ double sh[32];
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double en = 0;
    if (e < np) {
        double2 p = pos[e], w = vel[e];
        en = 0.5 * m * (w.x * w.x + w.y * w.y) - m * (gx * p.x + gy * p.y);
    }
    double a = block_sum(en, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    if (last_block(&st->ticket)) {
        double sa = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) sa += partial[k];
        sa = block_sum(sa, sh);
        if (threadIdx.x == 0) st->particle_energy = sa;
    }
}

}  // namespace

template <int SX, int SY>
static int launch_cp_sweep_dir(Sim* s, const int* skip) {
    const int nstrips = (s->NY + 31) / 32;
    if (nstrips > s->progress_cap) {
        set_error("closest-point sweep: %d strips exceed the %d progress counters", nstrips, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    static std::atomic<unsigned long long> configured{0};
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)cp_sweep_kernel<SX, SY>, (int)kCpSmem)) return rc0;
    CpArgs a;
    a.pos_df = s->pos_df;
    a.pos = s->pos;
    a.xtab = s->cp_tab;
    a.ytab = s->cp_tab + s->P;
    a.kc = s->cpc;
    a.hb_t = s->cp_hb_t;
    a.hb_p = s->cp_hb_p;
    a.progress = s->progress;
    a.base = wave_begin(s);
    a.err = s->err;
    a.skip = skip;
    a.np = (int)s->np;
    a.NX = s->NX;
    a.NY = s->NY;
    a.P = s->P;
    a.dx = s->dx;
    a.dr = s->dr;
    const CpMaps* maps = reinterpret_cast<const CpMaps*>(s->cpmaps->b);
    void* args[] = {(void*)maps, (void*)&a};
    s->launches++;
    long long kt = ktimer_begin(s, "cp_sweep");
    int rc = check_cuda(cudaLaunchCooperativeKernel((const void*)cp_sweep_kernel<SX, SY>, dim3(nstrips), dim3(64),
                                                    args, kCpSmem, s->stream),
                        "cp_sweep");
    ktimer_end(s, kt);
    return rc;
}

template <int SX, int SY>
static int launch_eik_sweep_dir(Sim* s, const WaveGeom& g, const int* skip) {
    const int nstrips = (s->NY + kEkRows - 1) / kEkRows;
    if (nstrips > s->progress_cap) {
        set_error("Eikonal sweep: %d strips exceed the %d progress counters", nstrips, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    static std::atomic<unsigned long long> configured{0};
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)eik_sweep_kernel<SX, SY>, (int)kEkSmem)) return rc0;
    EkArgs a;
    a.hb = reinterpret_cast<double2*>(s->cp_hb_p);
    a.progress = s->progress;
    a.base = wave_begin(s);
    a.err = s->err;
    a.skip = skip;
    a.NX = s->NX;
    a.NY = s->NY;
    a.P = s->P;
    a.i_lo = g.i_lo;
    a.i_hi = g.i_hi;
    a.j_lo = g.j_lo;
    a.j_hi = g.j_hi;
    a.dx = s->dx;
    a.c2 = 2 * s->dx * s->dx;
    const EkMaps* maps = reinterpret_cast<const EkMaps*>(s->ekmaps->b);
    void* args[] = {(void*)maps, (void*)&a};
    s->launches++;
    long long kt = ktimer_begin(s, "eik_sweep");
    int& cs = s->ek_cluster;   // 0: not chosen yet
    if (cs == 0) cs = choose_cluster((const void*)eik_sweep_kernel<SX, SY>, nstrips, 64, kEkSmem);
    cudaError_t e = launch_clustered((const void*)eik_sweep_kernel<SX, SY>, nstrips, cs, 64, kEkSmem, s->stream, args);
    if (e != cudaSuccess && cs > 1) {   // clusters refused: plain cooperative launch
        (void)cudaGetLastError();
        cs = 1;
        e = launch_clustered((const void*)eik_sweep_kernel<SX, SY>, nstrips, 1, 64, kEkSmem, s->stream, args);
    }
    int rc = check_cuda(e, "eik_sweep");
    ktimer_end(s, kt);
    return rc;
}

static int launch_eik_sweep(Sim* s, const WaveGeom& g, const int* skip) {
    if (g.sx > 0) return g.sy > 0 ? launch_eik_sweep_dir<1, 1>(s, g, skip) : launch_eik_sweep_dir<1, -1>(s, g, skip);
    return g.sy > 0 ? launch_eik_sweep_dir<-1, 1>(s, g, skip) : launch_eik_sweep_dir<-1, -1>(s, g, skip);
}

static int launch_cp_sweep(Sim* s, int sx, int sy, const int* skip) {
    if (sx > 0) return sy > 0 ? launch_cp_sweep_dir<1, 1>(s, skip) : launch_cp_sweep_dir<1, -1>(s, skip);
    return sy > 0 ? launch_cp_sweep_dir<-1, 1>(s, skip) : launch_cp_sweep_dir<-1, -1>(s, skip);
}

// TMA descriptors of the closest-point sweeps over the pitched index array.
int cp_setup_maps(Sim* s) {
    static_assert(sizeof(CpMaps) <= sizeof(CpMapsHost::b), "tensor map storage");
    CpMaps m{};
    const int tail = s->NY % 32;
    int rc = make_tensor_map_2d(&m.ld, s->t, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, s->P, s->NY, s->P, kCpCols, kCpBoxRows);
    if (!rc) rc = make_tensor_map_2d(&m.st, s->t, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, s->P, s->NY, s->P, kCpCols, 32);
    if (!rc)
        rc = make_tensor_map_2d(&m.st_tail, s->t, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, s->P, s->NY, s->P, kCpCols,
                                tail > 0 ? tail : 32);
    if (rc) return rc;
    memcpy(s->cpmaps->b, &m, sizeof(m));
    static_assert(sizeof(EkMaps) <= sizeof(CpMapsHost::b), "tensor map storage");
    EkMaps e{};
    rc = make_tensor_map_2d(&e.ld, s->phi_p, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, s->P, s->NY, s->P, kEkCols, kEkRows);
    if (!rc)
        rc = make_tensor_map_2d(&e.st_tail, s->phi_p, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, s->P, s->NY, s->P, kEkCols,
                                tail > 0 ? tail : kEkRows);
    if (!rc)
        rc = make_tensor_map_2d(&e.mask, s->emask, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, s->P, s->NY, s->P, kEkCols,
                                kEkRows);
    if (rc) return rc;
    memcpy(s->ekmaps->b, &e, sizeof(e));
    return 0;
}

int levelset_create(Sim* s) {
    const int NX = s->NX, NY = s->NY;
    const int T = 256;
    // one extra int per sweep for the no-op flags, at the end of `partial`'s
    // companion: reuse the err-adjacent scratch in `max_layer`
    int* noop = (int*)s->max_layer + 4;

    const int P = s->P;
    const size_t NP = (size_t)P * NY;
    // constructFromParticles: seed (pitched t)
    FS2D_LAUNCH(s, k_seed_init, blocks_for(NP, T), T, 0, s->t, s->seed_key, NX, NY, P);
    if (s->np > 0) {
        FS2D_LAUNCH(s, k_seed_min, blocks_for(s->np, T), T, 0, s->pos, s->np, s->seed_key, NX, NY, s->dx, s->dr,
                    s->err);
        FS2D_LAUNCH(s, k_seed_idx, blocks_for(s->np, T), T, 0, s->pos, s->np, s->seed_key, s->t, NX, NY, P, s->dx,
                    s->dr);
    }
    FS2D_LAUNCH(s, k_seed_write, blocks_for(NP, T), T, 0, s->t, NP);

    // decision constants, float-pair positions and corner tables
    FS2D_CUDA(cudaMemsetAsync(s->cpc, 0, sizeof(CpConst), s->stream));
    if (s->np > 0) FS2D_LAUNCH(s, k_posdf, blocks_for(s->np, T), T, 0, s->pos, s->np, s->pos_df, s->cpc);
    FS2D_LAUNCH(s, k_cp_tabs, blocks_for(std::max(P, NY), T), T, 0, s->cp_tab, s->cp_tab + P, P, NY, s->dx);
    FS2D_LAUNCH(s, k_cp_const, 1, 1, 0, s->cpc, NX, NY, s->dx, s->dr);

    // fastSweepIterate: 4 x {(+,+), (-,+), (+,-), (-,-)}
    const int dirs[4][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
    dim3 g2(blocks_for(NX, 128), NY);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));  // -1 -> nonzero = no-op
            FS2D_LAUNCH(s, k_cp_check, g2, 128, 0, s->t, s->pos_df, s->pos, s->cp_tab, s->cp_tab + P, s->cpc, NX, NY,
                        P, s->dx, s->dr, noop);
            int rc = launch_cp_sweep(s, dirs[d][0], dirs[d][1], noop);
            if (rc) return rc;
        }
    }
    FS2D_LAUNCH(s, k_cp_phi, g2, 128, 0, s->t, s->pos, s->np, s->phi, NX, NY, P, s->dx, s->dr);

    // redistance on the pitched copy phi_p
    FS2D_LAUNCH(s, k_surface, g2, 128, 0, s->phi, s->phi_p, NX, NY, P);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            int sx = dirs[d][0], sy = dirs[d][1];
            int i_lo = sx > 0 ? 1 : 0, i_hi = sx > 0 ? NX - 1 : NX - 2;
            int j_lo = sy > 0 ? 1 : 0, j_hi = sy > 0 ? NY - 1 : NY - 2;
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));
            FS2D_LAUNCH(s, k_eik_check, g2, 128, 0, s->phi_p, s->emask, NX, NY, P, i_lo, i_hi, j_lo, j_hi, sx, sy,
                        s->dx, noop);
            WaveGeom g{sx, sy, i_lo, i_hi, j_lo, j_hi};
            int rc = launch_eik_sweep(s, g, noop);
            if (rc) return rc;
        }
    }
    FS2D_LAUNCH(s, k_smooth, g2, 128, 0, s->phi_p, P, s->phi, NX, NY);
    FS2D_LAUNCH(s, k_smooth, g2, 128, 0, s->phi, NX, s->phi_tmp, NX, NY);

    // labels + statistics (phi_tmp -> phi)
    FS2D_LAUNCH(s, k_labels_stats, g2, 128, 0, s->phi_tmp, s->phi, s->cell, s->u, s->v, NX, NY, s->dx, s->rho, s->gx,
                s->gy, s->partial, s->stats);
    if (s->np > 0) {
        double m = s->rho * s->dx * s->dx / (s->ppc_sqrt * s->ppc_sqrt);
        FS2D_LAUNCH(s, k_particle_energy, blocks_for(s->np, T), T, 0, s->pos, s->vel, s->np, m, s->gx, s->gy,
                    s->partial, s->stats);
    } else {
        FS2D_CUDA(cudaMemsetAsync(&s->stats->particle_energy, 0, sizeof(double), s->stream));
    }
    return 0;
}

}  // namespace fs2d
