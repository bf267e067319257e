// projection_mixed.cu — mixed-precision pressure solve (FS2D_PRECISION_MIXED).
//
// The reference's MIC(0)-PCG (src/FluidSim2D.cpp:252-467) with the inner
// iteration in FP32 and the accuracy owned by FP64:
//   * iterative refinement: the FP64 residual r = b - A p is recomputed from
//     the FP64 matrix (built exactly as the reference builds it, projection.cu)
//     after each inner solve, and the stop test is the reference's
//     ||r||inf <= tol * ||b||inf on that FP64 residual;
//   * each inner solve runs MIC(0)-PCG on A e = r / ||r||inf in FP32: matrix,
//     preconditioner factor and both triangular solves (strip wavefronts in the
//     reference's dependency order; the forward solve runs on q~ = q*precon,
//     so both solves have the form out = v0 - v1*left - v2*below with three
//     operand arrays, TMA-staged, see mic32_tma.cuh), SpMV and vector updates;
//   * inner dot products use exact FP32 products (p + e, e from an FMA),
//     double-float (FP32 pair) accumulation inside a warp and FP64 across
//     warps and blocks; norms are maxima (exact in any precision); the
//     scalars alpha, beta, sigma are FP64.
// Compiled with the default FMA contraction.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <cudaTypedefs.h>
#include "fs2d_device.cuh"
#include "wave2.cuh"
#include "mic32_tma.cuh"

namespace fs2d {
namespace {

constexpr int kT = 256;

// ---- double-float accumulation of exact products ----
struct DF {
    float hi, lo;
};
__device__ __forceinline__ void df_add(DF& a, float b) {  // TwoSum
    float s = a.hi + b;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b - bb);
    a.hi = s;
    a.lo += err;
}
__device__ __forceinline__ DF df_prod(float x, float y) {  // exact: x*y = hi + lo
    float p = x * y;
    return DF{p, fmaf(x, y, -p)};
}
__device__ __forceinline__ void df_add(DF& a, DF b) {
    df_add(a, b.hi);
    a.lo += b.lo;
}
__device__ __forceinline__ DF df_warp_sum(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DF t{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
        df_add(v, t);
    }
    return v;
}
// Block sum of per-thread products as FP64 (valid in thread 0).

// FP32 copies of the FP64 matrix in the pitched layout (Adiag keeps its
// -0.0 non-fluid marker).
__global__ void k_mixed_matrix(const double* __restrict__ A0, const double* __restrict__ Ax,
                               const double* __restrict__ Ay, float* a0, float* ax, float* ay, int NX, int P,
                               size_t N) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= N) return;
    size_t k = (c / NX) * (size_t)P + (c % NX);
    a0[k] = (float)A0[c];
    ax[k] = (float)Ax[c];
    ay[k] = (float)Ay[c];
}

struct MicFactor32 {
    static constexpr const char* kName = "wave2_MicFactor32";
    typedef float T;
    static constexpr int NA = 5;
    const float* in[5];  // Adiag(i,j), Ax(i-1,j), Ay(i-1,j), Ay(i,j-1), Ax(i,j-1)
    float* out;          // precon
    int pitch;
    float tau, sigma;
    __device__ float border(int i, int j) const { return out[(size_t)j * pitch + i]; }
    __device__ float stored(const float*, float r) const { return r; }
    __device__ float compute(const float* v, float pl, float pd, int, int) const {
        const float ad = v[0];
        if (signbit(ad)) return 0.0f;
        const float axl = v[1], ayl = v[2], ayd = v[3], axd = v[4];
        float e = ad - (axl * pl) * (axl * pl) - (ayd * pd) * (ayd * pd) -
                  tau * (axl * ayl * pl * pl + ayd * axd * pd * pd);
        if (e < sigma * ad) e = ad;
        return 1.0f / sqrtf(e);
    }
};

// Folded MIC(0) coefficients.  With q~ = q*pc the reference's forward
// substitution q = (r - Ax(i-1,j)pc(i-1,j)q(i-1,j) - Ay(i,j-1)pc(i,j-1)q(i,j-1))*pc
// becomes q~ = r*pc^2 - fa*q~(i-1,j) - fb*q~(i,j-1) with fa = Ax(i-1,j)*pc^2,
// fb = Ay(i,j-1)*pc^2, and the backward substitution
// z = (q - Ax pc z(i+1,j) - Ay pc z(i,j+1))*pc becomes z = q~ - fc*z(i+1,j) - fd*z(i,j+1)
// with fc = Ax*pc^2, fd = Ay*pc^2 (pc taken at (i,j)).
__global__ void k_mixed_coef(const float* __restrict__ ax, const float* __restrict__ ay,
                             const float* __restrict__ pc, float* fa, float* fb, float* fc, float* fd, int NX, int NY,
                             int P) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= (size_t)NX * NY) return;
    int i = (int)(c % NX), j = (int)(c / NX);
    size_t k = (size_t)j * P + i;
    float p = pc[k];
    float p2 = p * p;
    fa[k] = i > 0 ? ax[k - 1] * p2 : 0.0f;
    fb[k] = j > 0 ? ay[k - P] * p2 : 0.0f;
    fc[k] = ax[k] * p2;
    fd[k] = ay[k] * p2;
}

// FP64 residual r = b - A p on fluid cells (the SpMV of :433-444 in FP64),
// ||r||inf into the outer scalars.
__global__ void k_resid64(const uint8_t* __restrict__ cell, const double* __restrict__ A0,
                          const double* __restrict__ Ax, const double* __restrict__ Ay, const double* __restrict__ rhs,
                          const double* __restrict__ p, double* r, int NX, size_t N, double* partial,
                          PcgScalars* outer) {
    __shared__ double sh[32];
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double m = 0;
    if (c < N) {
        double v = 0.0;
        if (cell[c] == kFluid) {
            double ap = A0[c] * p[c] + Ax[c - 1] * p[c - 1] + Ax[c] * p[c + 1] + Ay[c - NX] * p[c - NX] +
                        Ay[c] * p[c + NX];
            v = rhs[c] - ap;
        }
        r[c] = v;
        m = fabs(v);
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
    if (last_block(&outer->ticket[0])) {
        double mm = 0;
        for (size_t k = threadIdx.x; k < gridDim.x; k += blockDim.x) mm = fmax(mm, partial[k]);
        mm = block_max(mm, sh);
        if (threadIdx.x == 0) outer->r_norm = mm;
    }
}

// Start of an inner solve: r32 = r64 / ||r64||inf, r*pc^2, e = 0, scalars reset.
__global__ void k_inner_init(const double* __restrict__ r64, const PcgScalars* __restrict__ outer,
                             const float* __restrict__ pc, float* r32, float* rp32, float* e32, int NX, int P,
                             size_t N, PcgScalars* inner, double inner_tol) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const double rn = outer->r_norm;
    const double scale = rn > 0 ? 1.0 / rn : 0.0;
    if (c < N) {
        size_t k = (c / NX) * (size_t)P + (c % NX);
        float rv = (float)(r64[c] * scale);
        float p = pc[k];
        r32[k] = rv;
        rp32[k] = rv * (p * p);
        e32[k] = 0.0f;
    }
    if (c == 0) {
        inner->iter = 0;
        inner->done = (rn > 0) ? 0 : 1;
        inner->first = 1;
        inner->sigma = inner->alpha = inner->beta = 0;
        inner->rhs_norm = 1.0;
        inner->r_norm = 1.0;
        inner->tol_abs = inner_tol;   // read by k_axpy32 (device memory, so a captured loop can replay it)
    }
}

// ---- inner FP32 PCG kernels ----
// Row-segment layout: block (bx, by) covers columns bx*kRT .. bx*kRT+kRT-1
// of rows by, by + gridDim.y, ...; sums are accumulated and reduced in
// double-float (FP32 pairs), in a fixed order (deterministic), and the
// last block finishes the scalar.
constexpr int kRT = 256;

__device__ __forceinline__ void df_block_partial(DF v, float2* partial, float2* sh) {
    v = df_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = make_float2(v.hi, v.lo);
    __syncthreads();
    if (wid == 0) {
        DF t = lane < nw ? DF{sh[lane].x, sh[lane].y} : DF{0.f, 0.f};
        t = df_warp_sum(t);
        if (lane == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = make_float2(t.hi, t.lo);
    }
}

// Sum of the partials of every block (called by the last block).
__device__ __forceinline__ double df_final(const float2* partial, int n, float2* sh) {
    DF acc{0.f, 0.f};
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float2 v = partial[k];
        df_add(acc, DF{v.x, v.y});
    }
    acc = df_warp_sum(acc);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = make_float2(acc.hi, acc.lo);
    __syncthreads();
    DF t = (wid == 0 && lane < nw) ? DF{sh[lane].x, sh[lane].y} : DF{0.f, 0.f};
    if (wid == 0) t = df_warp_sum(t);
    return (double)t.hi + (double)t.lo;
}

__device__ __forceinline__ float block_max_f(float v, float* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = lane < nw ? sh[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(kRT) k_dot32(const float* __restrict__ z, const float* __restrict__ r, int NX,
                                               int NY, int P, float2* partial, PcgScalars* pcg, int init,
                                               int max_iters) {
    __shared__ float2 sh[32];
    if (pcg->done) return;
    const int i = blockIdx.x * kRT + threadIdx.x;
    DF a{0.f, 0.f};
    if (i < NX) {
#pragma unroll 4
        for (int j = blockIdx.y; j < NY; j += gridDim.y) {
            const size_t k = (size_t)j * P + i;
            df_add(a, df_prod(z[k], r[k]));
        }
    }
    df_block_partial(a, partial, sh);
    if (last_block(&pcg->ticket[1])) {
        const double s = df_final(partial, gridDim.x * gridDim.y, sh);
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

// s_new = z + beta s_old (z on the first iteration), w = A s_new on fluid
// cells, alpha = sigma / (w . s_new).
__global__ void __launch_bounds__(kRT) k_spmv32(const uint8_t* __restrict__ cell, const float* __restrict__ a0,
                                                const float* __restrict__ ax, const float* __restrict__ ay,
                                                const float* __restrict__ z, const float* __restrict__ s_old,
                                                float* s_new, float* w, int NX, int NY, int P, float2* partial,
                                                PcgScalars* pcg) {
    __shared__ float2 sh[32];
    if (pcg->done) return;
    const bool first = pcg->first != 0;
    const float beta = (float)pcg->beta;
    const int i = blockIdx.x * kRT + threadIdx.x;
    DF a{0.f, 0.f};
    if (i < NX) {
        for (int j = blockIdx.y; j < NY; j += gridDim.y) {
            const size_t k = (size_t)j * P + i;
            const float sc = first ? z[k] : fmaf(beta, s_old[k], z[k]);
            s_new[k] = sc;
            float out = 0.0f;
            if (cell[(size_t)j * NX + i] == kFluid) {
                const float sl = first ? z[k - 1] : fmaf(beta, s_old[k - 1], z[k - 1]);
                const float sr = first ? z[k + 1] : fmaf(beta, s_old[k + 1], z[k + 1]);
                const float sd = first ? z[k - P] : fmaf(beta, s_old[k - P], z[k - P]);
                const float su = first ? z[k + P] : fmaf(beta, s_old[k + P], z[k + P]);
                out = a0[k] * sc + ax[k - 1] * sl + ax[k] * sr + ay[k - P] * sd + ay[k] * su;
            }
            w[k] = out;
            df_add(a, df_prod(out, sc));
        }
    }
    df_block_partial(a, partial, sh);
    if (last_block(&pcg->ticket[2])) {
        const double sum = df_final(partial, gridDim.x * gridDim.y, sh);
        if (threadIdx.x == 0) {
            if (sum == 0.0) pcg->done = 1;
            else pcg->alpha = pcg->sigma / sum;
        }
    }
}

// e += alpha s, r -= alpha w, rp = r pc^2, ||r||inf (stop when below the
// inner tolerance, pcg->tol_abs).
__global__ void __launch_bounds__(kRT) k_axpy32(float* e, float* r, float* rp, const float* __restrict__ pc,
                                                const float* __restrict__ s, const float* __restrict__ w, int NX,
                                                int NY, int P, float* partial, PcgScalars* pcg) {
    __shared__ float sh[32];
    if (pcg->done) return;
    const float alpha = (float)pcg->alpha;
    const int i = blockIdx.x * kRT + threadIdx.x;
    float m = 0.f;
    if (i < NX) {
#pragma unroll 2
        for (int j = blockIdx.y; j < NY; j += gridDim.y) {
            const size_t k = (size_t)j * P + i;
            e[k] = fmaf(alpha, s[k], e[k]);
            const float rv = fmaf(-alpha, w[k], r[k]);
            r[k] = rv;
            const float p = pc[k];
            rp[k] = rv * (p * p);
            m = fmaxf(m, fabsf(rv));
        }
    }
    m = block_max_f(m, sh);
    if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = m;
    if (last_block(&pcg->ticket[3])) {
        float mm = 0.f;
        for (int k = threadIdx.x; k < (int)(gridDim.x * gridDim.y); k += blockDim.x) mm = fmaxf(mm, partial[k]);
        mm = block_max_f(mm, sh);
        if (threadIdx.x == 0) {
            pcg->r_norm = mm;
            if (mm <= pcg->tol_abs) pcg->done = 1;
        }
    }
}

// p += e * ||r||inf (undo the inner scaling) in FP64.
__global__ void k_update64(double* p, const float* __restrict__ e, const PcgScalars* __restrict__ outer, int NX, int P,
                           size_t N) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < N) p[c] = p[c] + (double)e[(c / NX) * (size_t)P + (c % NX)] * outer->r_norm;
}

}  // namespace

int mic32_make_map(CUtensorMap* map, float* base, int P, int NR) {
    return make_tensor_map_2d(map, base, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, P, kM32Cols, kM32Rows);
}

static_assert(sizeof(Mic32Maps) <= sizeof(Mic32MapsHost::fwd), "tensor map storage");

// Tensor maps of the FP32 MIC(0) sweeps, built once per handle.
int mixed_setup_maps(Sim* s) {
    Mixed32& m = s->m32;
    Mic32Maps f{}, b{};
    int rc = 0;
    float* fin[3] = {m.rp, m.fa, m.fb};
    float* bin[3] = {m.q, m.fc, m.fd};
    for (int a = 0; a < 3 && !rc; a++) rc = mic32_make_map(&f.in[a], fin[a], s->P32, s->NY32);
    for (int a = 0; a < 3 && !rc; a++) rc = mic32_make_map(&b.in[a], bin[a], s->P32, s->NY32);
    if (!rc) rc = mic32_make_map(&f.out, m.q, s->P32, s->NY32);
    if (!rc) rc = mic32_make_map(&b.out, m.z, s->P32, s->NY32);
    if (rc) return rc;
    memcpy(s->m32maps->fwd, &f, sizeof(f));
    memcpy(s->m32maps->bwd, &b, sizeof(b));
    return 0;
}

constexpr int kM32GraphIters = 8;   // inner iterations per graph replay (even: the search-direction ping-pong)

int projection_mixed(Sim* s, int* status) { return projection_mixed_rhs(s, nullptr, status); }

// b == nullptr: the physical right-hand side; otherwise A p = b for a device
// array b on the fluid cells.
int projection_mixed_rhs(Sim* s, const double* b, int* status) {
    const int NX = s->NX, NY = s->NY, P = s->P32;   // FP32 arrays: pitch P32
    const size_t N = s->N;
    const unsigned nb = blocks_for(N, kT);
    Mixed32& m = s->m32;
    // the FP64 matrix, rhs, ||b||inf, p = 0, r = b (exactly the reference's)
    int rc = projection_build(s);
    if (rc) return rc;
    if (b && (rc = projection_set_rhs(s, b))) return rc;
    FS2D_LAUNCH(s, k_mixed_matrix, nb, kT, 0, s->Adiag, s->Ax, s->Ay, m.a0, m.ax, m.ay, NX, P, N);
    {
        MicFactor32 op{{m.a0, m.ax - 1, m.ay - 1, m.ay - P, m.ax - P}, m.pc, P, (float)s->opt.mic_tau,
                       (float)s->opt.mic_sigma};
        rc = launch_wave2<MicFactor32, 2, 16>(s, op, WaveGeom{1, 1, 1, NX - 1, 1, NY - 1}, nullptr);
        if (rc) return rc;
    }
    FS2D_LAUNCH(s, k_mixed_coef, nb, kT, 0, m.ax, m.ay, m.pc, m.fa, m.fb, m.fc, m.fd, NX, NY, P);

    PcgScalars* outer = s->pcg;     // rhs_norm, tol_abs from projection_build; r_norm = ||r64||
    PcgScalars* inner = s->pcg32;
    const int* done = &inner->done;
    const Mic32Maps& fmaps = *reinterpret_cast<const Mic32Maps*>(s->m32maps->fwd);
    const Mic32Maps& bmaps = *reinterpret_cast<const Mic32Maps*>(s->m32maps->bwd);
    const int max_iters = s->opt.pcg_max_iters;
    const int batch = 4;
    // inner kernels: ~8 blocks per SM of row segments
    const int gx = (NX + kRT - 1) / kRT;
    const dim3 rg(gx, std::max(1, std::min(NY, 1216 / gx)));
    float2* part2 = reinterpret_cast<float2*>(s->partial);
    float* partf = reinterpret_cast<float*>(s->partial);
    int total_iters = 0, outer_iters = 0, status_out = 0;

    FS2D_CUDA(cudaMemcpyAsync(s->pcg_host, outer, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
    if (int rcw = wait_stream(s, s->stream)) return rcw;
    const double rhs_norm = s->pcg_host->rhs_norm;
    const double tol_abs = s->pcg_host->tol_abs;
    double r_norm = rhs_norm;
    if (rhs_norm > 1e-12) {
        for (outer_iters = 0; outer_iters < s->opt.ir_max_outer; outer_iters++) {
            if (r_norm <= tol_abs) break;
            // each inner solve works on r / ||r||inf: it has to reduce that
            // by tol_abs / ||r||inf (with a factor 2 of margin for the FP32
            // recurrence), but never asks for more than ir_inner_tol
            const double inner_tol = std::max(s->opt.ir_inner_tol, 0.5 * tol_abs / r_norm);
            FS2D_LAUNCH(s, k_inner_init, nb, kT, 0, s->r, outer, m.pc, m.r, m.rp, m.e, NX, P, N, inner, inner_tol);
            rc = launch_mic32<true>(s, fmaps, m.q, done);
            if (rc) return rc;
            rc = launch_mic32<false>(s, bmaps, m.z, done);
            if (rc) return rc;
            FS2D_LAUNCH(s, k_dot32, rg, kRT, 0, m.z, m.r, NX, NY, P, part2, inner, 1, max_iters);
            // one inner iteration; graph = true inside a stream capture
            auto iteration = [&](int it, bool graph) -> int {
                float* sbuf[2] = {m.s0, m.s1};
                float* s_old = sbuf[it & 1];
                float* s_new = sbuf[(it + 1) & 1];
                FS2D_LAUNCH(s, k_spmv32, rg, kRT, 0, s->cell, m.a0, m.ax, m.ay, m.z, s_old, s_new, m.w, NX, NY, P,
                            part2, inner);
                FS2D_LAUNCH(s, k_axpy32, rg, kRT, 0, m.e, m.r, m.rp, m.pc, s_new, m.w, NX, NY, P, partf, inner);
                const int slot = graph ? 2 * (it % kM32GraphIters) : -1;   // sweeps of one replay
                int rc1 = launch_mic32<true>(s, fmaps, m.q, done, slot, 2 * kM32GraphIters);
                if (rc1) return rc1;
                rc1 = launch_mic32<false>(s, bmaps, m.z, done, graph ? slot + 1 : -1, 2 * kM32GraphIters);
                if (rc1) return rc1;
                FS2D_LAUNCH(s, k_dot32, rg, kRT, 0, m.z, m.r, NX, NY, P, part2, inner, 0, max_iters);
                return 0;
            };
            // true once the inner solve stopped; a failed copy or wait also
            // stops it and leaves its status in rc_poll
            int rc_poll = 0;
            auto poll_done = [&]() -> bool {
                rc_poll = check_cuda(cudaMemcpyAsync(s->pcg32_host, inner, sizeof(PcgScalars),
                                                     cudaMemcpyDeviceToHost, s->stream),
                                     "cudaMemcpyAsync");
                if (!rc_poll) rc_poll = wait_stream(s, s->stream);
                return rc_poll != 0 || s->pcg32_host->done != 0;
            };
            // Captures kM32GraphIters iterations as a CUDA graph (once per handle,
            // again whenever the reduction scratch moved); false: launch directly
            // (per-kernel timing is on, or capture is not available here).
            auto ensure_graph = [&]() -> bool {
                if (!s->kt_patterns.empty() || s->m32_graph_state < 0) return false;
                if (s->m32_graph_state == 1 && s->m32_graph_key == (const void*)s->partial) return true;
                if (s->m32_graph) {
                    cudaGraphExecDestroy(s->m32_graph);
                    s->m32_graph = nullptr;
                }
                s->m32_graph_state = -1;   // until the capture below succeeds
                const unsigned long long l0 = s->launches;
                if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    (void)cudaGetLastError();
                    return false;
                }
                int rc1 = 0;
                for (int k = 0; k < kM32GraphIters && !rc1; k++) rc1 = iteration(k, true);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(s->stream, &g);
                s->m32_graph_launches = s->launches - l0;
                s->launches = l0;   // captured, not run
                if (rc1 || e != cudaSuccess || g == nullptr) {
                    if (g) cudaGraphDestroy(g);
                    (void)cudaGetLastError();
                    return false;
                }
                e = cudaGraphInstantiate(&s->m32_graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    (void)cudaGetLastError();
                    s->m32_graph = nullptr;
                    return false;
                }
                s->m32_graph_key = s->partial;
                s->m32_graph_state = 1;
                return true;
            };
            int it = 0;
            if (ensure_graph()) {
                // whole batches of iterations from the captured graph (kernels
                // after convergence return at once on the done flag)
                for (; it + kM32GraphIters <= max_iters; it += kM32GraphIters) {
                    FS2D_CUDA(cudaGraphLaunch(s->m32_graph, s->stream));
                    s->launches += s->m32_graph_launches;
                    if (poll_done()) {
                        it = max_iters;
                        break;
                    }
                }
            }
            for (; it < max_iters; it++) {
                if ((rc = iteration(it, false))) return rc;
                if ((it + 1) % batch == 0 || it + 1 == max_iters) {
                    if (poll_done()) break;
                }
            }
            if (rc_poll) return rc_poll;
            FS2D_LAUNCH(s, k_update64, nb, kT, 0, s->p, m.e, outer, NX, P, N);
            FS2D_LAUNCH(s, k_resid64, nb, kT, 0, s->cell, s->Adiag, s->Ax, s->Ay, s->rhs, s->p, s->r, NX, N,
                        s->partial, outer);
            FS2D_CUDA(cudaMemcpyAsync(s->pcg32_host, inner, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
            FS2D_CUDA(cudaMemcpyAsync(s->pcg_host, outer, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
            if (int rcw = wait_stream(s, s->stream)) return rcw;
            total_iters += s->pcg32_host->iter;
            r_norm = s->pcg_host->r_norm;
        }
        if (r_norm > tol_abs) status_out = FS2D_ERR_NOT_CONVERGED;
    } else {
        r_norm = rhs_norm;
    }
    s->last_iters = total_iters;
    s->last_outer = outer_iters;
    s->last_rel_res = rhs_norm > 0 ? r_norm / rhs_norm : 0.0;
    if (status) *status = status_out;
    return 0;
}

}  // namespace fs2d
