// projection.cu — pressure projection and velocity update (FP64).
//
//   FluidSim2D::applyProjection   src/FluidSim2D.cpp:252-467
//   FluidSim2D::updateVelocity    src/FluidSim2D.cpp:469-550
//   diagnostics                   src/FluidSim2D.cpp:607-638
// Compiled with --fmad=false.
//
// The matrix (ghost-fluid diagonal), right-hand side, MIC(0) factor and the
// two triangular solves per iteration round exactly like the reference's
// serial loops: the factor and the solves are Gauss-Seidel-ordered
// recurrences and run as strip wavefronts (wave2.cuh) that keep the
// reference's dependency order.  Dot products and norms are tree reductions
// (a different summation order than the reference's serial loop), so the
// iterates agree with the reference to rounding, not bit for bit.
//
// The PCG loop runs without host round trips: alpha, beta, sigma, the
// residual norm and the stop flag live in device memory (PcgScalars), each
// reduction's last block finalises them, and every kernel of an iteration
// returns at once when the stop flag is set.  The host enqueues iterations
// in batches and polls the flag between batches.
#include <cuda_runtime.h>
#include <math.h>
#include "fs2d_device.cuh"
#include "wave2.cuh"

namespace fs2d {
namespace {

constexpr int kT = 256;

// Matrix with ghost-fluid diagonal (USE_GHOST_PRESSURE, :261-303) and the
// divergence right-hand side with solid faces (:337-362).  Also p = 0 and
// r = rhs (:424-425), and ||rhs||inf finalised into the solver scalars.
__global__ void k_build(const uint8_t* __restrict__ cell, const double* __restrict__ phi,
                        const double* __restrict__ u, const double* __restrict__ v, int NX, int NY, double scaleA,
                        double scale, double* Adiag, double* Ax, double* Ay, double* rhs, double* r, double* p,
                        double* partial, PcgScalars* pcg, double tol, const FrameStats* __restrict__ stats,
                        double vol0, double vol_rate, double dt) {
    __shared__ double sh[32];
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t N = (size_t)NX * NY;
    double bn = 0;
    if (c < N) {
        int i = (int)(c % NX), j = (int)(c / NX);
        double ad = 0, ax = 0, ay = 0, b = 0;
        if (cell[c] == kFluid) {
            double phi0 = phi[c];
            uint8_t l = cell[c - 1], rgt = cell[c + 1], d = cell[c - NX], up = cell[c + NX];
            if (l == kFluid) ad += scaleA;
            else if (l == kEmpty) ad -= scaleA * dmax(phi[c - 1] / phi0, -1e3);
            if (rgt == kFluid) { ad += scaleA; ax = -scaleA; }
            else if (rgt == kEmpty) ad += scaleA * (1 - dmax(phi[c + 1] / phi0, -1e3));
            if (d == kFluid) ad += scaleA;
            else if (d == kEmpty) ad -= scaleA * dmax(phi[c - NX] / phi0, -1e3);
            if (up == kFluid) { ad += scaleA; ay = -scaleA; }
            else if (up == kEmpty) ad += scaleA * (1 - dmax(phi[c + NX] / phi0, -1e3));
            double u0 = u[(size_t)j * (NX + 1) + i], u1 = u[(size_t)j * (NX + 1) + i + 1];
            double v0 = v[c], v1 = v[c + NX];
            b = -scale * (u1 - u0 + v1 - v0);
            if (l == kSolid) b -= scale * (u0 - 0);
            if (rgt == kSolid) b += scale * (u1 - 0);
            if (d == kSolid) b -= scale * (v0 - 0);
            if (up == kSolid) b += scale * (v1 - 0);
            // volume correction (fs2d_set_volume_correction; not in the reference)
            if (vol_rate != 0.0) {
                const double vol = stats->volume;
                if (vol > 0.0) b += vol_rate * ((vol0 - vol) / vol0) / dt;
            }
        }
        // non-fluid cells carry -0.0: a marker the MIC(0) factor reads from its
        // staged operands (fluid cells hold the reference's value, >= +0.0)
        Adiag[c] = (cell[c] == kFluid) ? ad : -0.0;
        Ax[c] = ax;
        Ay[c] = ay;
        rhs[c] = b;
        r[c] = b;
        p[c] = 0.0;
        bn = fabs(b);
    }
    double m = block_max(bn, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
    if (last_block(&pcg->ticket[0])) {
        double mm = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) mm = fmax(mm, partial[k]);
        mm = block_max(mm, sh);
        if (threadIdx.x == 0) {
            pcg->rhs_norm = mm;
            pcg->tol_abs = tol * mm;
            pcg->r_norm = mm;
            pcg->iter = 0;
            pcg->done = 0;
            pcg->first = 1;
            pcg->sigma = 0;
            pcg->alpha = 0;
            pcg->beta = 0;
        }
    }
}

// MIC(0) factor (:364-387): precon(i,j) from precon(i-1,j) and precon(i,j-1),
// staged operands Adiag(i,j), Ax(i-1,j), Ay(i-1,j), Ay(i,j-1), Ax(i,j-1).
// The reference's SQUARE(x) is (x)*(x) without outer parentheses, so
// a*b*SQUARE(p) associates as ((a*b)*p)*p.
struct MicFactor64 {
    static constexpr const char* kName = "wave2_MicFactor64";
    typedef double T;
    static constexpr int NA = 5;
    const double* in[5];
    double* out;
    int pitch;
    double tau, sigma;
    __device__ double stored(const double*, double r) const { return r; }
    __device__ double border(int i, int j) const { return out[(size_t)j * pitch + i]; }
    __device__ double compute(const double* v, double pl, double pd, int, int) const {
        const double ad = v[0];
        if (signbit(ad)) return 0.0;  // not a fluid cell
        const double axl = v[1], ayl = v[2], ayd = v[3], axd = v[4];
        double e = ad - (axl * pl) * (axl * pl) - (ayd * pd) * (ayd * pd) -
                   tau * (axl * ayl * pl * pl + ayd * axd * pd * pd);
        if (e < sigma * ad) e = ad;
        return 1 / sqrt(e);
    }
};

// Triangular-solve coefficients: forward uses Ax(i-1,j)*precon(i-1,j) and
// Ay(i,j-1)*precon(i,j-1), backward Ax(i,j)*precon(i,j) and Ay(i,j)*precon(i,j)
// (:403-405,413-415), each product rounded exactly as the reference rounds it.
__global__ void k_coef(const double* __restrict__ Ax, const double* __restrict__ Ay, const double* __restrict__ pc,
                       double* cfx, double* cfy, double* cbx, double* cby, int NX, int NY) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= (size_t)NX * NY) return;
    int i = (int)(c % NX), j = (int)(c / NX);
    cfx[c] = i > 0 ? Ax[c - 1] * pc[c - 1] : 0.0;
    cfy[c] = j > 0 ? Ay[c - NX] * pc[c - NX] : 0.0;
    cbx[c] = Ax[c] * pc[c];
    cby[c] = Ay[c] * pc[c];
}

// applyPreconditioner, forward substitution (:400-409): q = L^-1 r.  Fluid
// cells are exactly those with precon != 0 (precon = 1/sqrt(e) with e finite).
struct MicForward64 {
    static constexpr const char* kName = "wave2_MicForward64";
    typedef double T;
    static constexpr int NA = 4;
    const double* in[4];  // r, cfx, cfy, precon
    double* out;          // q
    int pitch;
    __device__ double stored(const double*, double r) const { return r; }
    __device__ double border(int i, int j) const { return out[(size_t)j * pitch + i]; }
    __device__ double compute(const double* v, double ql, double qd, int, int) const {
        if (__double_as_longlong(v[3]) == 0) return 0.0;
        double t = v[0] - v[1] * ql - v[2] * qd;
        return t * v[3];
    }
};

// applyPreconditioner, backward substitution (:410-419): z = L^-T q.
struct MicBackward64 {
    static constexpr const char* kName = "wave2_MicBackward64";
    typedef double T;
    static constexpr int NA = 4;
    const double* in[4];  // q, cbx, cby, precon
    double* out;          // z
    int pitch;
    __device__ double stored(const double*, double r) const { return r; }
    __device__ double border(int i, int j) const { return out[(size_t)j * pitch + i]; }
    __device__ double compute(const double* v, double zr, double zu, int, int) const {
        if (__double_as_longlong(v[3]) == 0) return 0.0;
        double t = v[0] - v[1] * zr - v[2] * zu;
        return t * v[3];
    }
};

// sigma = z.r (:428 before the loop; :457-460 in it).  In the loop the last
// block also forms beta, counts the iteration and stops at the cap.
__global__ void k_dot_zr(const double* __restrict__ z, const double* __restrict__ r, size_t N, double* partial,
                         PcgScalars* pcg, int init, int max_iters) {
    __shared__ double sh[32];
    if (pcg->done) return;
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double a = c < N ? z[c] * r[c] : 0.0;
    a = block_sum(a, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    if (last_block(&pcg->ticket[1])) {
        double s = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) s += partial[k];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) {
            if (init) {
                pcg->sigma = s;
            } else {
                pcg->beta = s / pcg->sigma;
                pcg->sigma = s;
                pcg->iter += 1;
                pcg->first = 0;
                if (pcg->iter >= max_iters) pcg->done = 2;
            }
        }
    }
}

// Search direction s_new = z + beta * s_old (s_new = z on the first
// iteration, :427,459), w = A s_new on fluid cells (:433-444), z.s
// partials; the last block forms alpha (:450) or stops when ||b||inf <= 1e-12
// (:447-448).  s_new at the neighbours is recomputed from z and s_old, which
// rounds identically to reading it back.
__global__ void k_spmv(const uint8_t* __restrict__ cell, const double* __restrict__ Adiag,
                       const double* __restrict__ Ax, const double* __restrict__ Ay, const double* __restrict__ z,
                       const double* __restrict__ s_old, double* s_new, double* w, int NX, size_t N, double* partial,
                       PcgScalars* pcg) {
    __shared__ double sh[32];
    if (pcg->done) return;
    const bool first = pcg->first != 0;
    const double beta = pcg->beta;
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double a = 0;
    if (c < N) {
        double sc = first ? z[c] : z[c] + beta * s_old[c];
        s_new[c] = sc;
        double out = 0.0;
        if (cell[c] == kFluid) {
            double sl = first ? z[c - 1] : z[c - 1] + beta * s_old[c - 1];
            double sr = first ? z[c + 1] : z[c + 1] + beta * s_old[c + 1];
            double sd = first ? z[c - NX] : z[c - NX] + beta * s_old[c - NX];
            double su = first ? z[c + NX] : z[c + NX] + beta * s_old[c + NX];
            out = Adiag[c] * sc + Ax[c - 1] * sl + Ax[c] * sr + Ay[c - NX] * sd + Ay[c] * su;
        }
        w[c] = out;
        a = out * sc;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = a;
    if (last_block(&pcg->ticket[2])) {
        double s = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) s += partial[k];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) {
            if (pcg->rhs_norm <= 1e-12) {
                pcg->done = 1;
                pcg->r_norm = pcg->rhs_norm;
            } else {
                pcg->alpha = pcg->sigma / s;
            }
        }
    }
}

// p += alpha s, r -= alpha w (:451-452), ||r||inf; stop at tol (:453).
__global__ void k_axpy(double* p, double* r, const double* __restrict__ s, const double* __restrict__ w, size_t N,
                       double* partial, PcgScalars* pcg) {
    __shared__ double sh[32];
    if (pcg->done) return;
    const double alpha = pcg->alpha;
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double m = 0;
    if (c < N) {
        p[c] = p[c] + alpha * s[c];
        double rv = r[c] + -alpha * w[c];
        r[c] = rv;
        m = fabs(rv);
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
    if (last_block(&pcg->ticket[3])) {
        double mm = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) mm = fmax(mm, partial[k]);
        mm = block_max(mm, sh);
        if (threadIdx.x == 0) {
            pcg->r_norm = mm;
            if (mm <= pcg->tol_abs) pcg->done = 1;
        }
    }
}

// updateVelocity (:476-541): newMac = mac, then the pressure gradient on faces
// with a fluid side (ghost pressure at EMPTY sides, zero at SOLID sides and at
// the i=0 / j=0 boundary); faces with no fluid side are marked unknown.
// Faces i = NX (u) and j = NY (v) are never visited by the reference.
__global__ void k_update_velocity(const uint8_t* __restrict__ cell, const double* __restrict__ phi,
                                  const double* __restrict__ p, const double* __restrict__ u,
                                  const double* __restrict__ v, double* nu, double* nv, uint32_t* mu, uint32_t* mv,
                                  int NX, int NY, double scale) {
    int comp = blockIdx.z;
    int W = comp == 0 ? NX + 1 : NX;
    int H = comp == 0 ? NY : NY + 1;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= W || j >= H) return;
    size_t f = (size_t)j * W + i;
    if (comp == 0) {
        double val = u[f];
        uint32_t m = 0;
        if (i < NX) {
            size_t c = (size_t)j * NX + i;
            uint8_t cc = cell[c];
            uint8_t cl = i > 0 ? cell[c - 1] : kSolid;
            if ((i > 0 && cl == kFluid) || cc == kFluid) {
                if ((i == 0 || cl == kSolid) || cc == kSolid) {
                    val = 0;
                } else if (i > 0 && cl == kEmpty) {
                    double phi1 = phi[c - 1], phi0 = phi[c];
                    val -= scale * (1 - dmax(phi1 / phi0, -1e3)) * p[c];
                } else if (cc == kEmpty) {
                    double phi1 = phi[c], phi0 = phi[c - 1];
                    val -= scale * (dmax(phi1 / phi0, -1e3) - 1) * p[c - 1];
                } else if (i > 0) {
                    val -= scale * (p[c] - p[c - 1]);
                } else {
                    val = 0;
                }
            } else {
                m = kUnknown;
            }
        }
        nu[f] = val;
        mu[f] = m;
    } else {
        double val = v[f];
        uint32_t m = 0;
        if (j < NY) {
            size_t c = (size_t)j * NX + i;
            uint8_t cc = cell[c];
            uint8_t cd = j > 0 ? cell[c - NX] : kSolid;
            if ((j > 0 && cd == kFluid) || cc == kFluid) {
                if ((j == 0 || cd == kSolid) || cc == kSolid) {
                    val = 0;
                } else if (j > 0 && cd == kEmpty) {
                    double phi1 = phi[c - NX], phi0 = phi[c];
                    val -= scale * (1 - dmax(phi1 / phi0, -1e3)) * p[c];
                } else if (cc == kEmpty) {
                    double phi1 = phi[c], phi0 = phi[c - NX];
                    val -= scale * (dmax(phi1 / phi0, -1e3) - 1) * p[c - NX];
                } else if (j > 0) {
                    val -= scale * (p[c] - p[c - NX]);
                } else {
                    val = 0;
                }
            } else {
                m = kUnknown;
            }
        }
        nv[f] = val;
        mv[f] = m;
    }
}

// avgPressure, avgPressureInFluid, maxVelocity (src/FluidSim2D.cpp:607-638).
__global__ void k_diag(const uint8_t* __restrict__ cell, const double* __restrict__ p, const double* __restrict__ u,
                       const double* __restrict__ v, int NX, int NY, double dx, double* partial, FrameStats* st) {
    __shared__ double sh[32];
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t N = (size_t)NX * NY;
    double sp = 0, sf = 0, nf = 0, mv = 0;
    if (c < N) {
        sp = p[c];
        if (cell[c] == kFluid) {
            int i = (int)(c % NX), j = (int)(c / NX);
            sf = p[c];
            nf = 1;
            double x = (double)i * dx, y = (double)j * dx;
            double vx = vel_interp_u(u, NX, NY, dx, x, y), vy = vel_interp_v(v, NX, NY, dx, x, y);
            mv = sqrt(vx * vx + vy * vy);
        }
    }
    double a = block_sum(sp, sh), b = block_sum(sf, sh), d = block_sum(nf, sh), e = block_max(mv, sh);
    if (threadIdx.x == 0) {
        partial[4 * blockIdx.x] = a;
        partial[4 * blockIdx.x + 1] = b;
        partial[4 * blockIdx.x + 2] = d;
        partial[4 * blockIdx.x + 3] = e;
    }
    if (last_block(&st->ticket)) {
        double A = 0, B = 0, D = 0, E = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) {
            A += partial[4 * k];
            B += partial[4 * k + 1];
            D += partial[4 * k + 2];
            E = fmax(E, partial[4 * k + 3]);
        }
        A = block_sum(A, sh);
        B = block_sum(B, sh);
        D = block_sum(D, sh);
        E = block_max(E, sh);
        if (threadIdx.x == 0) {
            st->avg_p = A / (double)N;
            st->avg_p_fluid = B / D;
            st->max_vel = E;
        }
    }
}

// A caller-supplied right-hand side b on the fluid cells (0 elsewhere): r = b,
// p = 0 and the solver scalars reset as k_build does for the physical one.
__global__ void k_custom_rhs(const uint8_t* __restrict__ cell, const double* __restrict__ b, double* rhs, double* r,
                             double* p, size_t N, double* partial, PcgScalars* pcg, double tol) {
    __shared__ double sh[32];
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double bn = 0.0;
    if (c < N) {
        const double v = cell[c] == kFluid ? b[c] : 0.0;
        rhs[c] = v;
        r[c] = v;
        p[c] = 0.0;
        bn = fabs(v);
    }
    double m = block_max(bn, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
    if (last_block(&pcg->ticket[0])) {
        double mm = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) mm = fmax(mm, partial[k]);
        mm = block_max(mm, sh);
        if (threadIdx.x == 0) {
            pcg->rhs_norm = mm;
            pcg->tol_abs = tol * mm;
            pcg->r_norm = mm;
            pcg->iter = 0;
            pcg->done = 0;
            pcg->first = 1;
            pcg->sigma = 0;
            pcg->alpha = 0;
            pcg->beta = 0;
        }
    }
}

}  // namespace

static int projection_pcg(Sim* s, int* status);

int projection_build(Sim* s) {
    const double scaleA = s->dt / (s->rho * s->dx * s->dx);
    FS2D_LAUNCH(s, k_build, blocks_for(s->N, kT), kT, 0, s->cell, s->phi, s->u, s->v, s->NX, s->NY, scaleA,
                1.0 / s->dx, s->Adiag, s->Ax, s->Ay, s->rhs, s->r, s->p, s->partial, s->pcg, s->opt.pcg_tol,
                s->stats, s->orig_volume, s->volume_rate, s->dt);
    return 0;
}

int projection(Sim* s, int* status) {
    int rc0 = projection_build(s);
    if (rc0) return rc0;
    return projection_pcg(s, status);
}

// Replaces the built right-hand side by a caller-supplied device array b
// (fluid cells; 0 elsewhere), with r = b, p = 0 and the solver scalars reset.
int projection_set_rhs(Sim* s, const double* b) {
    FS2D_LAUNCH(s, k_custom_rhs, blocks_for(s->N, kT), kT, 0, s->cell, b, s->rhs, s->r, s->p, s->N, s->partial,
                s->pcg, s->opt.pcg_tol);
    return 0;
}

// A p = b for a caller-supplied device array b (the matrix of the current
// labels and level set), with the handle's precision; the solution is left
// in s->p.
int projection_solve_custom(Sim* s, const double* b, int* status) {
    if (s->opt.precision != FS2D_PRECISION_FP64) return projection_mixed_rhs(s, b, status);
    int rc0 = projection_build(s);
    if (rc0) return rc0;
    if ((rc0 = projection_set_rhs(s, b))) return rc0;
    return projection_pcg(s, status);
}

// MIC(0) factor and the PCG loop on the built system (rhs, r, p = 0).
static int projection_pcg(Sim* s, int* status) {
    const int NX = s->NX, NY = s->NY;
    const size_t N = s->N;
    const unsigned nb = blocks_for(N, kT);
    {
        MicFactor64 op{{s->Adiag, s->Ax - 1, s->Ay - 1, s->Ay - NX, s->Ax - NX}, s->precon, NX, s->opt.mic_tau,
                       s->opt.mic_sigma};
        int rc = launch_wave2<MicFactor64, 1, 8>(s, op, WaveGeom{1, 1, 1, NX - 1, 1, NY - 1}, nullptr);
        if (rc) return rc;
    }
    FS2D_LAUNCH(s, k_coef, nb, kT, 0, s->Ax, s->Ay, s->precon, s->cfx, s->cfy, s->cbx, s->cby, NX, NY);
    const int* done = &s->pcg->done;
    MicForward64 fwd{{s->r, s->cfx, s->cfy, s->precon}, s->q, NX};
    MicBackward64 bwd{{s->q, s->cbx, s->cby, s->precon}, s->z, NX};
    const WaveGeom gf{1, 1, 1, NX - 1, 1, NY - 1};
    const WaveGeom gb{-1, -1, 0, NX - 2, 0, NY - 2};
    int rc = launch_wave2<MicForward64, 2, 8>(s, fwd, gf, done);
    if (rc) return rc;
    rc = launch_wave2<MicBackward64, 2, 8>(s, bwd, gb, done);
    if (rc) return rc;
    FS2D_LAUNCH(s, k_dot_zr, nb, kT, 0, s->z, s->r, N, s->partial, s->pcg, 1, s->opt.pcg_max_iters);

    const int max_iters = s->opt.pcg_max_iters;
    const int batch = 4;
    double* sbuf[2] = {s->s0, s->s1};
    int it = 0;
    for (; it < max_iters; it++) {
        double* s_old = sbuf[it & 1];
        double* s_new = sbuf[(it + 1) & 1];
        FS2D_LAUNCH(s, k_spmv, nb, kT, 0, s->cell, s->Adiag, s->Ax, s->Ay, s->z, s_old, s_new, s->w, NX, N, s->partial,
                    s->pcg);
        FS2D_LAUNCH(s, k_axpy, nb, kT, 0, s->p, s->r, s_new, s->w, N, s->partial, s->pcg);
        rc = launch_wave2<MicForward64, 2, 8>(s, fwd, gf, done);
        if (rc) return rc;
        rc = launch_wave2<MicBackward64, 2, 8>(s, bwd, gb, done);
        if (rc) return rc;
        FS2D_LAUNCH(s, k_dot_zr, nb, kT, 0, s->z, s->r, N, s->partial, s->pcg, 0, max_iters);
        if ((it + 1) % batch == 0 || it + 1 == max_iters) {
            FS2D_CUDA(cudaMemcpyAsync(s->pcg_host, s->pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
            if (int rcw = wait_stream(s, s->stream)) return rcw;
            if (s->pcg_host->done) break;
        }
    }
    FS2D_CUDA(cudaMemcpyAsync(s->pcg_host, s->pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
    if (int rcw = wait_stream(s, s->stream)) return rcw;
    const PcgScalars& h = *s->pcg_host;
    s->last_iters = h.iter;
    s->last_outer = 0;
    s->last_rel_res = h.rhs_norm > 0 ? h.r_norm / h.rhs_norm : 0.0;
    if (status) *status = (h.iter >= max_iters && h.done != 1) ? FS2D_ERR_NOT_CONVERGED : 0;
    return 0;
}

int update_velocity(Sim* s) {
    dim3 grid(blocks_for(s->NX + 1, 128), s->NY + 1, 2);
    FS2D_LAUNCH(s, k_update_velocity, grid, 128, 0, s->cell, s->phi, s->p, s->u, s->v, s->nu, s->nv, s->mask_u,
                s->mask_v, s->NX, s->NY, s->dt / (s->rho * s->dx));
    int rc = extrapolate(s, s->nu, s->mask_u, s->NX + 1, s->NY, s->nv, s->mask_v, s->NX, s->NY + 1);
    if (rc) return rc;
    if (s->mode == FS2D_SEMILAGRANGIAN) {
        FS2D_CUDA(cudaMemcpyAsync(s->u, s->nu, s->NU * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
        FS2D_CUDA(cudaMemcpyAsync(s->v, s->nv, s->NV * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    }
    return 0;
}

int diagnostics(Sim* s) {
    FS2D_LAUNCH(s, k_diag, blocks_for(s->N, kT), kT, 0, s->cell, s->p, s->u, s->v, s->NX, s->NY, s->dx, s->partial,
                s->stats);
    return 0;
}

}  // namespace fs2d
