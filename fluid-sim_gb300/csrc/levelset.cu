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
//   * every Gauss-Seidel sweep runs as a strip wavefront (wave_kernel),
//     which visits each cell after exactly the neighbours the serial loop
//     visits before it;
//   * a sweep that would change no cell is skipped: a parallel check first
//     evaluates every cell's update against the current values, and if none
//     would change, the serial sweep would not change anything either.
#include <cuda_runtime.h>
#include <math.h>
#include <limits.h>
#include "fs2d_device.cuh"
#include "wave2.cuh"

namespace fs2d {
namespace {

__device__ __forceinline__ unsigned long long order_key(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double order_key_inv(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

// d = |particle - cell corner (i dx, j dx)| - dr  (src/FluidSim2D.cpp:768,785)
__device__ __forceinline__ double corner_dist(double2 p, int i, int j, double dx, double dr) {
    double ax = p.x - i * dx, ay = p.y - j * dx;
    return sqrt(ax * ax + ay * ay) - dr;
}

__global__ void k_seed_init(double* phi, int* t, unsigned long long* key, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n) return;
    phi[c] = HUGE_VAL;
    t[c] = INT_MAX;
    key[c] = ~0ull;
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
                           int* t, int NX, int NY, double dx, double dr) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    int x = (int)(p.x / dx), y = (int)(p.y / dx);
    if (x < 0 || x >= NX || y < 0 || y >= NY) return;
    size_t c = (size_t)y * NX + x;
    if (order_key(corner_dist(p, x, y, dx, dr)) == key[c]) atomicMin(t + c, (int)e);
}

__global__ void k_seed_write(double* phi, int* t, const unsigned long long* __restrict__ key, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n) return;
    if (t[c] == INT_MAX) {
        t[c] = -1;
        phi[c] = HUGE_VAL;
    } else {
        phi[c] = order_key_inv(key[c]);
    }
}

// ---- closest-point propagation (the fastSweepIterate lambda) ----

struct CPCarry {
    int t;
};

// Candidate order of the reference: (i-1,j), (i+1,j), (i,j-1), (i,j+1); each
// replaces the current value when strictly smaller.  A candidate equal to the
// current particle gives the same d and never wins, so it is skipped.
__device__ __forceinline__ void cp_candidate(int e, const double2* __restrict__ pos, int i, int j, double dx,
                                             double dr, double& cur, int& ct) {
    if (e != -1 && e != ct) {
        double d = corner_dist(pos[e], i, j, dx, dr);
        if (d < cur) {
            cur = d;
            ct = e;
        }
    }
}

struct ClosestPointOp {
    static constexpr const char* kName = "wave_ClosestPointOp";
    typedef CPCarry Carry;
    double* phi;
    int* t;
    const double2* pos;
    int NX, NY, sx, sy;
    double dx, dr;

    __device__ void prefetch(int i, int j) const {
        size_t c = (size_t)j * NX + i;
        prefetch_l1(phi + c);
        prefetch_l1(t + c);
        if (j + sy >= 0 && j + sy < NY) prefetch_l1(t + (size_t)(j + sy) * NX + i);
    }
    __device__ Carry fetch(int i, int j, bool l2) const {
        if (i < 0 || i >= NX || j < 0 || j >= NY) return Carry{-1};
        const int* a = t + (size_t)j * NX + i;
        return Carry{l2 ? __ldcg(a) : *a};
    }
    __device__ Carry update(int i, int j, Carry left, Carry below) const {
        size_t c = (size_t)j * NX + i;
        double cur = phi[c];
        int ct = t[c];
        const int cur_t0 = ct;
        int tx_next = (i + sx >= 0 && i + sx < NX) ? t[c + sx] : -1;
        int ty_next = (j + sy >= 0 && j + sy < NY) ? t[(size_t)(j + sy) * NX + i] : -1;
        int tm = sx > 0 ? left.t : tx_next;
        int tp = sx > 0 ? tx_next : left.t;
        int td = sy > 0 ? below.t : ty_next;
        int tu = sy > 0 ? ty_next : below.t;
        cp_candidate(tm, pos, i, j, dx, dr, cur, ct);
        cp_candidate(tp, pos, i, j, dx, dr, cur, ct);
        cp_candidate(td, pos, i, j, dx, dr, cur, ct);
        cp_candidate(tu, pos, i, j, dx, dr, cur, ct);
        if (ct != cur_t0) {
            phi[c] = cur;
            t[c] = ct;
        }
        return Carry{ct};
    }
    static __device__ Carry shfl_up(Carry v) { return Carry{__shfl_up_sync(0xffffffffu, v.t, 1)}; }
};

// Would any cell change under one closest-point update with the current values?
__global__ void k_cp_check(const double* __restrict__ phi, const int* __restrict__ t,
                           const double2* __restrict__ pos, int NX, int NY, double dx, double dr, int* noop) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    size_t c = (size_t)j * NX + i;
    double cur = phi[c];
    int ct = t[c];
    const int t0 = ct;
    cp_candidate(i > 0 ? t[c - 1] : -1, pos, i, j, dx, dr, cur, ct);
    cp_candidate(i < NX - 1 ? t[c + 1] : -1, pos, i, j, dx, dr, cur, ct);
    cp_candidate(j > 0 ? t[c - NX] : -1, pos, i, j, dx, dr, cur, ct);
    cp_candidate(j < NY - 1 ? t[c + NX] : -1, pos, i, j, dx, dr, cur, ct);
    if (ct != t0) *noop = 0;
}

// ---- redistance ----

// Surface flags from the sign changes the reference tests
// (src/FluidSim2D.cpp:803-834: pairs with the base cell in [0,NX-2]x[0,NY-2]),
// then non-surface negative cells -> -inf (:836-842).  Reads phi, writes out.
__global__ void k_surface(const double* __restrict__ phi, double* out, int NX, int NY) {
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
    out[c] = (!surf && p < 0) ? -HUGE_VAL : p;
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

struct Eikonal64 {
    static constexpr const char* kName = "wave2_Eikonal64";
    typedef double T;
    static constexpr int NA = 1;
    const double* in[1];  // phi before the sweep (the output array itself)
    double* out;
    int pitch;
    double dx;
    __device__ double stored(const double*, double r) const { return r; }
    __device__ double border(int i, int j) const { return out[(size_t)j * pitch + i]; }
    __device__ double compute(const double* v, double left, double below, int, int) const {
        return eikonal(v[0], left, below, dx);
    }
};

__global__ void k_eik_check(const double* __restrict__ phi, int NX, int i_lo, int i_hi, int j_lo, int j_hi, int sx,
                            int sy, double dx, int* noop) {
    int i = i_lo + blockIdx.x * blockDim.x + threadIdx.x;
    int j = j_lo + blockIdx.y;
    if (i > i_hi || j > j_hi) return;
    size_t c = (size_t)j * NX + i;
    double own = phi[c];
    if (own >= 0) return;
    double nv = eikonal(own, phi[c - sx], phi[(size_t)(j - sy) * NX + i], dx);
    if (nv != own) *noop = 0;
}

// Min-smoothing pass (src/FluidSim2D.cpp:904-919): Jacobi, interior cells.
__global__ void k_smooth(const double* __restrict__ oldp, double* out, int NX, int NY) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= NX) return;
    size_t c = (size_t)j * NX + i;
    double o = oldp[c];
    if (i >= 1 && i <= NX - 2 && j >= 1 && j <= NY - 2) {
        double avg = 0.25 * (oldp[c - 1] + oldp[c + 1] + oldp[c - NX] + oldp[c + NX]);
        if (avg < o) o = avg;
    }
    out[c] = o;
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

int levelset_create(Sim* s) {
    const int NX = s->NX, NY = s->NY;
    const size_t N = s->N;
    const int T = 256;
    // one extra int per sweep for the no-op flags, at the end of `partial`'s
    // companion: reuse the err-adjacent scratch in `max_layer`
    int* noop = (int*)s->max_layer + 4;

    // constructFromParticles: seed
    FS2D_LAUNCH(s, k_seed_init, blocks_for(N, T), T, 0, s->phi, s->t, s->seed_key, N);
    if (s->np > 0) {
        FS2D_LAUNCH(s, k_seed_min, blocks_for(s->np, T), T, 0, s->pos, s->np, s->seed_key, NX, NY, s->dx, s->dr,
                    s->err);
        FS2D_LAUNCH(s, k_seed_idx, blocks_for(s->np, T), T, 0, s->pos, s->np, s->seed_key, s->t, NX, NY, s->dx,
                    s->dr);
    }
    FS2D_LAUNCH(s, k_seed_write, blocks_for(N, T), T, 0, s->phi, s->t, s->seed_key, N);

    // fastSweepIterate: 4 x {(+,+), (-,+), (+,-), (-,-)}
    const int dirs[4][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
    dim3 g2(blocks_for(NX, 128), NY);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));  // -1 -> nonzero = no-op
            FS2D_LAUNCH(s, k_cp_check, g2, 128, 0, s->phi, s->t, s->pos, NX, NY, s->dx, s->dr, noop);
            ClosestPointOp op{s->phi, s->t, s->pos, NX, NY, dirs[d][0], dirs[d][1], s->dx, s->dr};
            WaveGeom g{dirs[d][0], dirs[d][1], 0, NX - 1, 0, NY - 1};
            int rc = launch_wave(s, op, g, noop);
            if (rc) return rc;
        }
    }

    // redistance
    FS2D_LAUNCH(s, k_surface, g2, 128, 0, s->phi, s->phi_tmp, NX, NY);
    for (int rep = 0; rep < 4; rep++) {
        for (int d = 0; d < 4; d++) {
            int sx = dirs[d][0], sy = dirs[d][1];
            int i_lo = sx > 0 ? 1 : 0, i_hi = sx > 0 ? NX - 1 : NX - 2;
            int j_lo = sy > 0 ? 1 : 0, j_hi = sy > 0 ? NY - 1 : NY - 2;
            FS2D_CUDA(cudaMemsetAsync(noop, 0xff, sizeof(int), s->stream));
            dim3 gc(blocks_for(i_hi - i_lo + 1, 128), j_hi - j_lo + 1);
            FS2D_LAUNCH(s, k_eik_check, gc, 128, 0, s->phi_tmp, NX, i_lo, i_hi, j_lo, j_hi, sx, sy, s->dx, noop);
            Eikonal64 op{{s->phi_tmp}, s->phi_tmp, NX, s->dx};
            WaveGeom g{sx, sy, i_lo, i_hi, j_lo, j_hi};
            int rc = launch_wave2<Eikonal64, 2, 8>(s, op, g, noop);
            if (rc) return rc;
        }
    }
    FS2D_LAUNCH(s, k_smooth, g2, 128, 0, s->phi_tmp, s->phi, NX, NY);
    FS2D_LAUNCH(s, k_smooth, g2, 128, 0, s->phi, s->phi_tmp, NX, NY);

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
