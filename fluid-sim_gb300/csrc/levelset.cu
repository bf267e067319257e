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
__device__ __forceinline__ bool cp_check_cell(const int* __restrict__ t, const float4* __restrict__ pos_df,
                                              const double2* __restrict__ pos, const float2* __restrict__ xtab,
                                              const float2* __restrict__ ytab, const CpConst& kc, int NX, int NY,
                                              int P, double dx, double dr, int i, int j) {
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
    return cur.t != own;
}

__global__ void k_cp_check(const int* __restrict__ t, const float4* __restrict__ pos_df,
                           const double2* __restrict__ pos, const float2* __restrict__ xtab,
                           const float2* __restrict__ ytab, const CpConst* __restrict__ kcp, int NX, int NY, int P,
                           double dx, double dr, int* noop) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    const CpConst kc = *kcp;
    if (cp_check_cell(t, pos_df, pos, xtab, ytab, kc, NX, NY, P, dx, dr, i, j)) *noop = 0;
}

// phi = d(t) of every cell (HUGE_VAL without a particle), as the reference
// stores it with t.
__device__ __forceinline__ void cp_phi_cell(const int* __restrict__ t, const double2* __restrict__ pos, size_t np,
                                            double* phi, int NX, int P, double dx, double dr, int i, int j) {
    const int e = t[(size_t)j * P + i];
    phi[(size_t)j * NX + i] = (e < 0 || (size_t)e >= np) ? HUGE_VAL : corner_dist(pos[e], i, j, dx, dr);
}
__global__ void k_cp_phi(const int* __restrict__ t, const double2* __restrict__ pos, size_t np, double* phi, int NX,
                         int NY, int P, double dx, double dr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    cp_phi_cell(t, pos, np, phi, NX, P, dx, dr, i, j);
}

// ---- redistance ----

// Surface flags from the sign changes the reference tests
// (src/FluidSim2D.cpp:803-834: pairs with the base cell in [0,NX-2]x[0,NY-2]),
// then non-surface negative cells -> -inf (:836-842).  Reads phi, writes out.
__device__ __forceinline__ void surface_cell(const double* __restrict__ phi, double* out, int NX, int NY, int P, int i,
                                             int j) {
    size_t c = (size_t)j * NX + i;
    double p = phi[c];
    bool surf = false;
    if (i <= NX - 2 && j <= NY - 2 && p * phi[c + 1] < 0) surf = true;
    if (i >= 1 && j <= NY - 2 && phi[c - 1] * p < 0) surf = true;
    if (i <= NX - 2 && j <= NY - 2 && p * phi[c + NX] < 0) surf = true;
    if (i <= NX - 2 && j >= 1 && phi[c - NX] * p < 0) surf = true;
    out[(size_t)j * P + i] = (!surf && p < 0) ? -HUGE_VAL : p;
}
__global__ void k_surface(const double* __restrict__ phi, double* out, int NX, int NY, int P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    surface_cell(phi, out, NX, NY, P, i, j);
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


__device__ __forceinline__ bool eik_check_cell(const double* __restrict__ phi, uint8_t* mask, int P, int i_lo,
                                               int i_hi, int j_lo, int j_hi, int sx, int sy, double dx, int i, int j) {
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
    return ch;
}
// Range of an Eikonal sweep strip (rows of one 32-row strip in sweep order):
// x = the first sweep column whose cell the check marked, y = P - 1 - the last
// sweep column holding a negative cell the sweep may update (both 0xffffffff
// when there is none).  One row per block: a block minimum, then one atomic.
__device__ __forceinline__ void eik_range_add(uint2* rng, int strip, unsigned first_marked, unsigned last_neg_rev) {
    __shared__ unsigned sm[2][4];
    const unsigned fm = __reduce_min_sync(0xffffffffu, first_marked);
    const unsigned ln = __reduce_min_sync(0xffffffffu, last_neg_rev);
    const int wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        sm[0][wid] = fm;
        sm[1][wid] = ln;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned a = 0xffffffffu, b = 0xffffffffu;
        for (int k = 0; k < nw; k++) {
            a = min(a, sm[0][k]);
            b = min(b, sm[1][k]);
        }
        if (a != 0xffffffffu) atomicMin(&rng[strip].x, a);
        if (b != 0xffffffffu) atomicMin(&rng[strip].y, b);
    }
}

// The range terms of cell (i, j) for eik_range_add (i >= NX: none).
__device__ __forceinline__ void eik_range_terms(const double* __restrict__ phi, bool marked, int NX, int P, int i_lo,
                                                int i_hi, int j_lo, int j_hi, int sx, int i, int j, unsigned& fm,
                                                unsigned& ln) {
    fm = ln = 0xffffffffu;
    if (i >= NX || i < i_lo || i > i_hi || j < j_lo || j > j_hi) return;
    const unsigned c = (unsigned)(sx > 0 ? i : P - 1 - i);   // sweep column
    if (marked) fm = c;
    if (phi[(size_t)j * P + i] < 0) ln = (unsigned)(P - 1) - c;
}

__global__ void __launch_bounds__(128) k_eik_check(const double* __restrict__ phi, uint8_t* mask, int NX, int NY,
                                                   int P, int i_lo, int i_hi, int j_lo, int j_hi, int sx, int sy,
                                                   double dx, int* noop, uint2* rng) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    bool marked = false;
    if (i < NX) {
        marked = eik_check_cell(phi, mask, P, i_lo, i_hi, j_lo, j_hi, sx, sy, dx, i, j);
        if (marked) *noop = 0;
    }
    unsigned fm, ln;
    eik_range_terms(phi, marked, NX, P, i_lo, i_hi, j_lo, j_hi, sx, i, j, fm, ln);
    eik_range_add(rng, (sy > 0 ? j : NY - 1 - j) / 32, fm, ln);
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
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)cp_sweep_kernel<SX, SY, false>, (int)kCpSmem)) return rc0;
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
    WaveWork w{};
    void* args[] = {(void*)maps, (void*)&a, (void*)&w};
    s->launches++;
    long long kt = ktimer_begin(s, "cp_sweep");
    int rc = check_cuda(cudaLaunchCooperativeKernel((const void*)cp_sweep_kernel<SX, SY, false>, dim3(nstrips), dim3(64),
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
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)eik_sweep_kernel<SX, SY, false>, (int)kEkSmem)) return rc0;
    EkArgs a;
    a.hb = reinterpret_cast<double2*>(s->cp_hb_p);
    a.phi = s->phi_p;
    a.rng = s->eik_rng;
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
    WaveWork w{};
    void* args[] = {(void*)maps, (void*)&a, (void*)&w};
    s->launches++;
    long long kt = ktimer_begin(s, "eik_sweep");
    int& cs = s->ek_cluster;   // 0: not chosen yet
    if (cs == 0) cs = choose_cluster((const void*)eik_sweep_kernel<SX, SY, false>, nstrips, 64, kEkSmem);
    cudaError_t e = launch_clustered((const void*)eik_sweep_kernel<SX, SY, false>, nstrips, cs, 64, kEkSmem, s->stream, args);
    if (e != cudaSuccess && cs > 1) {   // clusters refused: plain cooperative launch
        (void)cudaGetLastError();
        cs = 1;
        e = launch_clustered((const void*)eik_sweep_kernel<SX, SY, false>, nstrips, 1, 64, kEkSmem, s->stream, args);
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

// createWaterLevelSet in parts around its two groups of sweeps (a batch of
// scenes runs each sweep of all its scenes in one launch, ls_batch_sweeps).
// Seeds (constructFromParticles), float-pair positions, corner tables and
// the constants of the closest-point decisions.
int levelset_seed(Sim* s) {
    const int NX = s->NX, NY = s->NY;
    const int T = 256;
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
    return 0;
}

// The reference's sweep directions, in its order: 4 x {(+,+), (-,+), (+,-), (-,-)}.
static const int kDirs[4][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}};

// Smoothing, labels and statistics (after the Eikonal sweeps).
int levelset_finish(Sim* s) {
    const int NX = s->NX, NY = s->NY;
    const int T = 256;
    dim3 g2(blocks_for(NX, 128), NY);
    FS2D_LAUNCH(s, k_smooth, g2, 128, 0, s->phi_p, s->P, s->phi, NX, NY);
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

int levelset_create(Sim* s) {
    const int NX = s->NX, NY = s->NY;
    const int P = s->P;
    // the no-op flag of the current sweep, in the err-adjacent scratch of `max_layer`
    int* noop = (int*)s->max_layer + 4;
    int rc = levelset_seed(s);
    if (rc) return rc;

    // fastSweepIterate: 4 x 4 directions
    dim3 g2(blocks_for(NX, 128), NY);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));  // -1 -> nonzero = no-op
            FS2D_LAUNCH(s, k_cp_check, g2, 128, 0, s->t, s->pos_df, s->pos, s->cp_tab, s->cp_tab + P, s->cpc, NX, NY,
                        P, s->dx, s->dr, noop);
            if ((rc = launch_cp_sweep(s, kDirs[d][0], kDirs[d][1], noop))) return rc;
        }
    }
    FS2D_LAUNCH(s, k_cp_phi, g2, 128, 0, s->t, s->pos, s->np, s->phi, NX, NY, P, s->dx, s->dr);

    // redistance on the pitched copy phi_p
    FS2D_LAUNCH(s, k_surface, g2, 128, 0, s->phi, s->phi_p, NX, NY, P);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            int sx = kDirs[d][0], sy = kDirs[d][1];
            int i_lo = sx > 0 ? 1 : 0, i_hi = sx > 0 ? NX - 1 : NX - 2;
            int j_lo = sy > 0 ? 1 : 0, j_hi = sy > 0 ? NY - 1 : NY - 2;
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));
            FS2D_CUDA(cudaMemsetAsync(s->eik_rng, 0xff, (size_t)((NY + 31) / 32) * sizeof(uint2), s->stream));
            FS2D_LAUNCH(s, k_eik_check, g2, 128, 0, s->phi_p, s->emask, NX, NY, P, i_lo, i_hi, j_lo, j_hi, sx, sy,
                        s->dx, noop, s->eik_rng);
            WaveGeom g{sx, sy, i_lo, i_hi, j_lo, j_hi};
            if ((rc = launch_eik_sweep(s, g, noop))) return rc;
        }
    }
    return levelset_finish(s);
}

// ---- the level-set sweeps of a batch of scenes ----

namespace {

// One scene of the batched per-cell kernels (128-thread blocks, one row
// segment each: block blk0 + j * gx + bx covers columns 128 bx .. of row j).
struct LsCells {
    int* t;
    const float4* pos_df;
    const double2* pos;
    const float2* xtab;
    const float2* ytab;
    const CpConst* kc;
    double* phi;
    double* phi_p;
    uint8_t* emask;
    size_t np;
    int NX, NY, P;
    int blk0, gx;
    int pidx0;    // the scene's first strip in the work list's counters (also no padding: tables are compared byte by byte)
    double dx, dr;
};

static_assert(sizeof(LsCells) == 9 * 8 + 8 + 6 * 4 + 2 * 8, "LsCells has no padding");

__device__ __forceinline__ const LsCells& ls_cell(const LsCells* __restrict__ sc, const int* __restrict__ blk, int& k,
                                                  int& i, int& j) {
    k = blk[blockIdx.x];
    const LsCells& S = sc[k];
    const int local = blockIdx.x - S.blk0;
    j = local / S.gx;
    i = (local % S.gx) * 128 + threadIdx.x;
    return S;
}

__global__ void k_cp_check_all(const LsCells* __restrict__ sc, const int* __restrict__ blk, int* noop) {
    int k, i, j;
    const LsCells& S = ls_cell(sc, blk, k, i, j);
    if (i >= S.NX) return;
    const CpConst kc = *S.kc;
    if (cp_check_cell(S.t, S.pos_df, S.pos, S.xtab, S.ytab, kc, S.NX, S.NY, S.P, S.dx, S.dr, i, j)) noop[k] = 0;
}

__global__ void k_cp_phi_all(const LsCells* __restrict__ sc, const int* __restrict__ blk) {
    int k, i, j;
    const LsCells& S = ls_cell(sc, blk, k, i, j);
    if (i >= S.NX) return;
    cp_phi_cell(S.t, S.pos, S.np, S.phi, S.NX, S.P, S.dx, S.dr, i, j);
}

__global__ void k_surface_all(const LsCells* __restrict__ sc, const int* __restrict__ blk) {
    int k, i, j;
    const LsCells& S = ls_cell(sc, blk, k, i, j);
    if (i >= S.NX) return;
    surface_cell(S.phi, S.phi_p, S.NX, S.NY, S.P, i, j);
}

__global__ void __launch_bounds__(128) k_eik_check_all(const LsCells* __restrict__ sc, const int* __restrict__ blk,
                                                       int sx, int sy, int* noop, uint2* rng) {
    int k, i, j;
    const LsCells& S = ls_cell(sc, blk, k, i, j);
    const int i_lo = sx > 0 ? 1 : 0, i_hi = sx > 0 ? S.NX - 1 : S.NX - 2;
    const int j_lo = sy > 0 ? 1 : 0, j_hi = sy > 0 ? S.NY - 1 : S.NY - 2;
    bool marked = false;
    if (i < S.NX) {
        marked = eik_check_cell(S.phi_p, S.emask, S.P, i_lo, i_hi, j_lo, j_hi, sx, sy, S.dx, i, j);
        if (marked) noop[k] = 0;
    }
    unsigned fm, ln;
    eik_range_terms(S.phi_p, marked, S.NX, S.P, i_lo, i_hi, j_lo, j_hi, sx, i, j, fm, ln);
    eik_range_add(rng, S.pidx0 + (sy > 0 ? j : S.NY - 1 - j) / 32, fm, ln);
}

template <typename T>
int ls_alloc(T** p, size_t n) {
    return check_cuda(cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)), "cudaMalloc");
}

}  // namespace

struct LsBatch {
    std::vector<Sim*> sims;
    std::vector<int> first;      // per scene: its first strip's counter (progress, ranges)
    std::vector<CpScene> cp;     // host copies of the device tables
    std::vector<EkScene> ek;
    std::vector<LsCells> cells;
    CpScene* d_cp = nullptr;
    EkScene* d_ek = nullptr;
    LsCells* d_cells = nullptr;
    int* d_blk = nullptr;
    int nblk = 0;
    WaveItem* d_items = nullptr;
    int nitems = 0;
    int* d_noop = nullptr;               // per scene: nonzero = no cell would change in this sweep
    uint2* d_rng = nullptr;              // per strip (counter order): the Eikonal sweep's column range
    int* d_work = nullptr;               // persistent-CTA counters of the cp and Eikonal sweeps
    unsigned long long* progress = nullptr;
    unsigned long long launch = 0;       // progress base of the next sweep
    int cp_ctas = 0, ek_ctas = 0;
};

void ls_batch_free(LsBatch* b) {
    if (!b) return;
    void* ptrs[] = {b->d_cp, b->d_ek, b->d_cells, b->d_blk, b->d_items, b->d_noop, b->d_work, b->progress, b->d_rng};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete b;
}

// The tables of every scene from its current buffers (particle arrays may
// have been replaced since the last frame); uploaded when they changed.
static int ls_batch_refresh(LsBatch* b, cudaStream_t stream) {
    const int n = (int)b->sims.size();
    std::vector<CpScene> cp(n);
    std::vector<EkScene> ek(n);
    std::vector<LsCells> cells(n);
    int blk = 0;
    for (int k = 0; k < n; k++) {
        Sim* s = b->sims[k];
        memset((void*)&cp[k], 0, sizeof(CpScene));
        memset((void*)&ek[k], 0, sizeof(EkScene));
        memcpy((void*)&cp[k].maps, s->cpmaps->b, sizeof(CpMaps));
        memcpy((void*)&ek[k].maps, s->ekmaps->b, sizeof(EkMaps));
        CpArgs& a = cp[k].a;
        a.pos_df = s->pos_df;
        a.pos = s->pos;
        a.xtab = s->cp_tab;
        a.ytab = s->cp_tab + s->P;
        a.kc = s->cpc;
        a.hb_t = s->cp_hb_t;
        a.hb_p = s->cp_hb_p;
        a.np = (int)s->np;
        a.NX = s->NX;
        a.NY = s->NY;
        a.P = s->P;
        a.dx = s->dx;
        a.dr = s->dr;
        EkArgs& e = ek[k].a;
        e.hb = reinterpret_cast<double2*>(s->cp_hb_p);
        e.phi = s->phi_p;
        e.NX = s->NX;
        e.NY = s->NY;
        e.P = s->P;
        e.dx = s->dx;
        e.c2 = 2 * s->dx * s->dx;
        LsCells& c = cells[k];
        c = LsCells{s->t, s->pos_df, s->pos, s->cp_tab, s->cp_tab + s->P, s->cpc, s->phi, s->phi_p, s->emask,
                    s->np, s->NX, s->NY, s->P, blk, (s->NX + 127) / 128, b->first[k], s->dx, s->dr};
        blk += c.gx * s->NY;
    }
    if (memcmp((const void*)cp.data(), (const void*)b->cp.data(), n * sizeof(CpScene)) != 0 ||
        memcmp((const void*)ek.data(), (const void*)b->ek.data(), n * sizeof(EkScene)) != 0 ||
        memcmp((const void*)cells.data(), (const void*)b->cells.data(), n * sizeof(LsCells)) != 0) {
        FS2D_CUDA(cudaMemcpyAsync(b->d_cp, cp.data(), n * sizeof(CpScene), cudaMemcpyHostToDevice, stream));
        FS2D_CUDA(cudaMemcpyAsync(b->d_ek, ek.data(), n * sizeof(EkScene), cudaMemcpyHostToDevice, stream));
        FS2D_CUDA(cudaMemcpyAsync(b->d_cells, cells.data(), n * sizeof(LsCells), cudaMemcpyHostToDevice, stream));
        FS2D_CUDA(cudaStreamSynchronize(stream));   // the host vectors are replaced below
        b->cp.swap(cp);
        b->ek.swap(ek);
        b->cells.swap(cells);
    }
    return 0;
}

LsBatch* ls_batch_create(Sim* const* sims, int n, int device, int* rc_out) {
    int rc = 0;
    LsBatch* b = new (std::nothrow) LsBatch();
    if (!b) {
        set_error("out of host memory");
        *rc_out = FS2D_ERR_ALLOC;
        return nullptr;
    }
    b->sims.assign(sims, sims + n);
    b->cp.resize(n);
    b->ek.resize(n);
    b->cells.resize(n);
    for (int k = 0; k < n; k++) {   // nothing matches: the first refresh uploads
        memset((void*)&b->cp[k], 0xff, sizeof(CpScene));
        memset((void*)&b->ek[k], 0xff, sizeof(EkScene));
        memset((void*)&b->cells[k], 0xff, sizeof(LsCells));
    }
    // block map of the per-cell kernels and the work list, critical path
    // first: a strip's rank is (strips after it) x the strip-to-strip lag
    // (~45 column steps measured) + its own steps; progress counters are
    // numbered scene by scene
    std::vector<int> blk;
    std::vector<int>& first = b->first;
    first.assign(n, 0);
    int pidx = 0;
    for (int k = 0; k < n; k++) {
        const Sim* s = sims[k];
        blk.insert(blk.end(), (size_t)((s->NX + 127) / 128) * s->NY, k);
        first[k] = pidx;
        pidx += (s->NY + 31) / 32;
    }
    std::vector<std::pair<long long, WaveItem>> ranked;
    for (int k = 0; k < n; k++) {
        const int ns = (sims[k]->NY + 31) / 32;
        for (int st = 0; st < ns; st++)
            ranked.push_back({(long long)(ns - 1 - st) * 45 + sims[k]->P + 31, WaveItem{k, st, first[k] + st}});
    }
    std::stable_sort(ranked.begin(), ranked.end(), [](const std::pair<long long, WaveItem>& a,
                                                      const std::pair<long long, WaveItem>& b) { return a.first > b.first; });
    std::vector<WaveItem> items;
    for (const auto& r : ranked) items.push_back(r.second);
    b->nblk = (int)blk.size();
    b->nitems = (int)items.size();
    if (!rc) rc = ls_alloc(&b->d_cp, n);
    if (!rc) rc = ls_alloc(&b->d_ek, n);
    if (!rc) rc = ls_alloc(&b->d_cells, n);
    if (!rc) rc = ls_alloc(&b->d_blk, blk.size());
    if (!rc) rc = ls_alloc(&b->d_items, items.size());
    if (!rc) rc = ls_alloc(&b->d_noop, n);
    if (!rc) rc = ls_alloc(&b->d_work, 4);
    if (!rc) rc = ls_alloc(&b->progress, items.size());
    if (!rc) rc = ls_alloc(&b->d_rng, items.size());
    if (!rc && ((uintptr_t)b->d_cp % alignof(CpScene) != 0 || (uintptr_t)b->d_ek % alignof(EkScene) != 0)) {
        set_error("level-set batch: the tensor map tables are not aligned");
        rc = FS2D_ERR_CUDA;
    }
    if (!rc) rc = check_cuda(cudaMemset(b->d_work, 0, 4 * sizeof(int)), "cudaMemset");
    if (!rc) rc = check_cuda(cudaMemset(b->progress, 0, items.size() * sizeof(unsigned long long)), "cudaMemset");
    if (!rc) rc = check_cuda(cudaMemcpy(b->d_blk, blk.data(), blk.size() * sizeof(int), cudaMemcpyHostToDevice),
                             "cudaMemcpy");
    if (!rc)
        rc = check_cuda(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(WaveItem), cudaMemcpyHostToDevice),
                        "cudaMemcpy");
    // persistent CTAs: as many as the SMs hold at once, at most one per item
    int sms = 1, per_cp = 0, per_ek = 0;
    if (!rc) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        const void* cps[] = {(const void*)cp_sweep_kernel<1, 1, true>, (const void*)cp_sweep_kernel<-1, 1, true>,
                             (const void*)cp_sweep_kernel<1, -1, true>, (const void*)cp_sweep_kernel<-1, -1, true>};
        const void* eks[] = {(const void*)eik_sweep_kernel<1, 1, true>, (const void*)eik_sweep_kernel<-1, 1, true>,
                             (const void*)eik_sweep_kernel<1, -1, true>, (const void*)eik_sweep_kernel<-1, -1, true>};
        static std::atomic<unsigned long long> cfg_cp[4] = {{0}, {0}, {0}, {0}}, cfg_ek[4] = {{0}, {0}, {0}, {0}};
        for (int k = 0; k < 4 && !rc; k++) rc = ensure_smem_attr(cfg_cp[k], device, cps[k], (int)kCpSmem);
        for (int k = 0; k < 4 && !rc; k++) rc = ensure_smem_attr(cfg_ek[k], device, eks[k], (int)kEkSmem);
        // every direction's instance must fit the CTA count (a cooperative launch is refused otherwise)
        per_cp = per_ek = 1 << 30;
        for (int k = 0; k < 4 && !rc; k++) {
            int a = 0, e = 0;
            rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, cps[k], 64, kCpSmem),
                            "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
            if (!rc)
                rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e, eks[k], 64, kEkSmem),
                                "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
            per_cp = std::min(per_cp, a);
            per_ek = std::min(per_ek, e);
        }
    }
    if (!rc && (per_cp < 1 || per_ek < 1)) {
        set_error("level-set batch: the sweep kernels do not fit on an SM");
        rc = FS2D_ERR_CUDA;
    }
    if (rc) {
        ls_batch_free(b);
        *rc_out = rc;
        return nullptr;
    }
    b->cp_ctas = std::max(1, std::min(per_cp * sms, b->nitems));
    b->ek_ctas = std::max(1, std::min(per_ek * sms, b->nitems));
    *rc_out = 0;
    return b;
}

template <int SX, int SY>
static int ls_launch_cp(LsBatch* b, cudaStream_t stream, int* err) {
    WaveWork w{b->d_cp, b->d_items, b->nitems, b->d_work, b->progress, (++b->launch) << 24, err, b->d_noop,
               nullptr};
    CpMaps m{};
    CpArgs a{};
    void* args[] = {(void*)&m, (void*)&a, (void*)&w};
    return check_cuda(
        launch_clustered((const void*)cp_sweep_kernel<SX, SY, true>, b->cp_ctas, 1, 64, kCpSmem, stream, args),
        "cp_sweep (batch)");
}

template <int SX, int SY>
static int ls_launch_ek(LsBatch* b, cudaStream_t stream, int* err) {
    WaveWork w{b->d_ek, b->d_items, b->nitems, b->d_work + 2, b->progress, (++b->launch) << 24, err, b->d_noop,
               b->d_rng};
    EkMaps m{};
    EkArgs a{};
    void* args[] = {(void*)&m, (void*)&a, (void*)&w};
    return check_cuda(
        launch_clustered((const void*)eik_sweep_kernel<SX, SY, true>, b->ek_ctas, 1, 64, kEkSmem, stream, args),
        "eik_sweep (batch)");
}

// Between levelset_seed and levelset_finish of every scene: the 16
// closest-point sweeps, phi and the surface, the 16 Eikonal sweeps, each
// step one launch for all scenes on `stream`.  Every scene computes what
// levelset_create computes for it alone (the same cells, strips and order).
int ls_batch_sweeps(LsBatch* b, cudaStream_t stream, int* err, unsigned long long* launches) {
    int rc = ls_batch_refresh(b, stream);
    if (rc) return rc;
    const int n = (int)b->sims.size();
    const unsigned nblk = (unsigned)b->nblk;
    auto count = [&](int k) { if (launches) *launches += (unsigned long long)k; };
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            FS2D_CUDA(cudaMemsetAsync(b->d_noop, 0xff, n * sizeof(int), stream));
            k_cp_check_all<<<nblk, 128, 0, stream>>>(b->d_cells, b->d_blk, b->d_noop);
            if ((rc = check_cuda(cudaGetLastError(), "k_cp_check_all"))) return rc;
            const int sx = kDirs[d][0], sy = kDirs[d][1];
            rc = sx > 0 ? (sy > 0 ? ls_launch_cp<1, 1>(b, stream, err) : ls_launch_cp<1, -1>(b, stream, err))
                        : (sy > 0 ? ls_launch_cp<-1, 1>(b, stream, err) : ls_launch_cp<-1, -1>(b, stream, err));
            if (rc) return rc;
            count(2);
        }
    }
    k_cp_phi_all<<<nblk, 128, 0, stream>>>(b->d_cells, b->d_blk);
    if ((rc = check_cuda(cudaGetLastError(), "k_cp_phi_all"))) return rc;
    k_surface_all<<<nblk, 128, 0, stream>>>(b->d_cells, b->d_blk);
    if ((rc = check_cuda(cudaGetLastError(), "k_surface_all"))) return rc;
    count(2);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            const int sx = kDirs[d][0], sy = kDirs[d][1];
            FS2D_CUDA(cudaMemsetAsync(b->d_noop, 0xff, n * sizeof(int), stream));
            FS2D_CUDA(cudaMemsetAsync(b->d_rng, 0xff, (size_t)b->nitems * sizeof(uint2), stream));
            k_eik_check_all<<<nblk, 128, 0, stream>>>(b->d_cells, b->d_blk, sx, sy, b->d_noop, b->d_rng);
            if ((rc = check_cuda(cudaGetLastError(), "k_eik_check_all"))) return rc;
            rc = sx > 0 ? (sy > 0 ? ls_launch_ek<1, 1>(b, stream, err) : ls_launch_ek<1, -1>(b, stream, err))
                        : (sy > 0 ? ls_launch_ek<-1, 1>(b, stream, err) : ls_launch_ek<-1, -1>(b, stream, err));
            if (rc) return rc;
            count(2);
        }
    }
    return 0;
}

}  // namespace fs2d
