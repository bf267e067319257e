// projection_mixed.cu — mixed-precision pressure solve (FS2D_PRECISION_MIXED)
// and the plain FP32 solve (FS2D_PRECISION_FP32).
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
//     operand arrays, and the factor the form pc = 1/sqrt(v0 - v1*left^2 -
//     v2*below^2), TMA-staged, see mic32_tma.cuh), SpMV and vector updates;
//   * inner dot products use exact FP32 products (p + e, e from an FMA),
//     double-float (FP32 pair) accumulation inside a warp and FP64 across
//     warps and blocks; norms are maxima (exact in any precision); the
//     scalars alpha, beta, sigma are FP64.
// Compiled with the default FMA contraction.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <numeric>
#include <vector>
#include <cudaTypedefs.h>
#include "fs2d_device.cuh"
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

// Operands of the FP32 MIC(0) factor sweep (kM32Factor in mic32_tma.cuh),
// on the reference's loop range (cells 1..NX-1 x 1..NY-1): the left term
// Ax(i-1,j) (Ax(i-1,j) + tau Ay(i-1,j)) into fa and the lower term
// Ay(i,j-1) (Ay(i,j-1) + tau Ax(i,j-1)) into fb (both are free until the
// folded coefficients replace them); 0 on the first row and column.
__global__ void k_factor_prep(const float* __restrict__ ax, const float* __restrict__ ay, float* fa, float* fb,
                              float tau, int NX, int NY, int P) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= (size_t)NX * NY) return;
    int i = (int)(c % NX), j = (int)(c / NX);
    size_t k = (size_t)j * P + i;
    float l = 0.f, d = 0.f;
    if (i > 0) {
        const float x = ax[k - 1], y = ay[k - 1];
        l = x * fmaf(tau, y, x);
    }
    if (j > 0) {
        const float x = ax[k - P], y = ay[k - P];
        d = y * fmaf(tau, x, y);
    }
    fa[k] = l;
    fb[k] = d;
}

// Folded MIC(0) coefficients of every scene of a pack (its FP32 blocks).
// With q~ = q*pc the reference's forward substitution
// q = (r - Ax(i-1,j)pc(i-1,j)q(i-1,j) - Ay(i,j-1)pc(i,j-1)q(i,j-1))*pc
// becomes q~ = r*pc^2 - fa*q~(i-1,j) - fb*q~(i,j-1) with fa = Ax(i-1,j)*pc^2,
// fb = Ay(i,j-1)*pc^2, and the backward substitution
// z = (q - Ax pc z(i+1,j) - Ay pc z(i,j+1))*pc becomes z = q~ - fc*z(i+1,j) - fd*z(i,j+1)
// with fc = Ax*pc^2, fd = Ay*pc^2 (pc taken at (i,j)).  Padding cells (pc 0)
// get zeros.
__global__ void __launch_bounds__(256) k_mixed_coef(const PackScene* __restrict__ sc, const int* __restrict__ blk,
                                                    int pitch, const float* __restrict__ ax,
                                                    const float* __restrict__ ay, const float* __restrict__ pc,
                                                    float* fa, float* fb, float* fc, float* fd) {
    const PackScene& S = sc[blk[blockIdx.x]];
    const int lb = blockIdx.x - S.blk0;
    const unsigned n = (unsigned)S.P32 * (unsigned)S.NY;
    for (unsigned c = (unsigned)lb * 256 + threadIdx.x; c < n; c += (unsigned)S.nb32 * 256) {
        const int j = (int)(c / (unsigned)S.P32), i = (int)(c - (unsigned)j * (unsigned)S.P32);
        const size_t k = (size_t)S.off + (size_t)j * pitch + i;
        const float p = pc[k];
        const float p2 = p * p;
        fa[k] = i > 0 ? ax[k - 1] * p2 : 0.0f;
        fb[k] = j > 0 ? ay[k - pitch] * p2 : 0.0f;
        fc[k] = ax[k] * p2;
        fd[k] = ay[k] * p2;
    }
}

// Every padding cell's Adiag (and the gaps between a batch's scenes) carries
// the -0.0 non-fluid marker, so the factor sweep leaves pc = 0 there and
// the SpMV skips them; k_mixed_matrix rewrites the scenes' cells each frame.
__global__ void k_fill_marker(float* a, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n) a[c] = -0.0f;
}

// ---- the refinement loop over the scenes of a pack ----
// Every kernel below covers every scene of a pack in one launch: block b
// belongs to scene blk[b] and is block b - blk0 (FP32 reductions) or
// b - blk64 (FP64 refinement) of that scene.  A scene's blocks and their
// order are those of the scene alone, so a scene's results do not depend on
// the other scenes of the pack.

// Start of a solve: per scene, the refinement stops at once when there is
// nothing to solve (||b||inf <= 1e-12) or the zero start already meets the
// tolerance; ctl[1] counts the scenes still refining.  One thread per scene.
__global__ void k_outer_start(const PackScene* __restrict__ sc, int n, int* ctl) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    PcgScalars* o = sc[k].outer;
    o->outer_iters = 0;
    o->inner_total = 0;
    o->outer_done = (o->rhs_norm > 1e-12 && o->r_norm > o->tol_abs) ? 0 : 1;
    sc[k].inner->done = 1;
    sc[k].inner->active = 0;
    if (!o->outer_done) atomicAdd(&ctl[1], 1);
}

// Start of an inner solve: r32 = r64 / ||r64||inf, r*pc^2, e = 0, scalars
// reset; the inner tolerance is the reduction the FP64 target still needs
// (with a factor 2 of margin for the FP32 recurrence), never tighter than
// inner_tol_min.  Scenes whose refinement stopped are marked inactive.
__global__ void k_inner_init(const PackScene* __restrict__ sc, const int* __restrict__ blk, int pitch,
                             const float* __restrict__ pc, float* r32, float* rp32, float* e32, double inner_tol_min,
                             int* ctl) {
    const PackScene& S = sc[blk[blockIdx.x]];
    const PcgScalars* outer = S.outer;
    if (outer->outer_done) return;
    const int lb = blockIdx.x - S.blk64;
    const size_t N = (size_t)S.NX * S.NY;
    const size_t c = (size_t)lb * blockDim.x + threadIdx.x;
    const double rn = outer->r_norm;
    const double scale = rn > 0 ? 1.0 / rn : 0.0;
    if (c < N) {
        const size_t k = (size_t)S.off + (c / S.NX) * (size_t)pitch + (c % S.NX);
        const float rv = (float)(S.r[c] * scale);
        const float p = pc[k];
        r32[k] = rv;
        rp32[k] = rv * (p * p);
        e32[k] = 0.0f;
    }
    if (lb == 0 && threadIdx.x == 0) {
        PcgScalars* inner = S.inner;
        inner->iter = 0;
        inner->done = (rn > 0) ? 0 : 1;
        inner->first = 1;
        inner->sigma = inner->alpha = inner->beta = 0;
        inner->rhs_norm = 1.0;
        inner->r_norm = 1.0;
        inner->tol_abs = fmax(inner_tol_min, 0.5 * outer->tol_abs / rn);   // read by k_axpy32
        inner->active = 1;
        if (!inner->done) atomicAdd(&ctl[0], 1);
    }
}

// Inner solve stops (first time only): one scene fewer running.
__device__ __forceinline__ void inner_stop(PcgScalars* pcg, int how, int* ctl) {
    if (pcg->done == 0) {
        pcg->done = how;
        atomicSub(&ctl[0], 1);
    }
}

// Last-block-done over the `nblocks` blocks of one scene.
__device__ __forceinline__ bool last_block_of(unsigned int* ticket, unsigned nblocks) {
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        is_last = (t == nblocks - 1);
        if (is_last) *ticket = 0;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// ---- inner FP32 PCG kernels ----
// Row-segment layout: block (bx, by) of a scene covers columns
// bx*kRT .. bx*kRT+kRT-1 of rows by, by + gy, ...; sums are accumulated and
// reduced in double-float (FP32 pairs), in a fixed order (deterministic), and
// the scene's last block finishes its scalar.
constexpr int kRT = 256;   // threads per block of the inner kernels
constexpr int kRV = 4;     // columns per thread
constexpr int kRC = kRT * kRV;

__device__ __forceinline__ float f_warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <bool PLAIN>
__device__ __forceinline__ void df_block_partial(DF v, float2* partial, int slot, float2* sh) {
    if (PLAIN) {   // FP32 tree sum
        float f = f_warp_sum(v.hi);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        __syncthreads();
        if (lane == 0) sh[wid] = make_float2(f, 0.f);
        __syncthreads();
        if (wid == 0) {
            float t = f_warp_sum(lane < nw ? sh[lane].x : 0.f);
            if (lane == 0) partial[slot] = make_float2(t, 0.f);
        }
        return;
    }
    v = df_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = make_float2(v.hi, v.lo);
    __syncthreads();
    if (wid == 0) {
        DF t = lane < nw ? DF{sh[lane].x, sh[lane].y} : DF{0.f, 0.f};
        t = df_warp_sum(t);
        if (lane == 0) partial[slot] = make_float2(t.hi, t.lo);
    }
}

// Sum of the partials of every block of a scene (called by its last block).
template <bool PLAIN>
__device__ __forceinline__ double df_final(const float2* partial, int n, float2* sh) {
    if (PLAIN) {   // FP32 tree sum of the block partials
        float f = 0.f;
        for (int k = threadIdx.x; k < n; k += blockDim.x) f += partial[k].x;
        f = f_warp_sum(f);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        __syncthreads();
        if (lane == 0) sh[wid] = make_float2(f, 0.f);
        __syncthreads();
        float t = 0.f;
        if (wid == 0) t = f_warp_sum(lane < nw ? sh[lane].x : 0.f);
        return (double)t;
    }
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

// Products accumulated exactly in double-float (FP64-accurate dots), or, for
// the plain FP32 solve (PLAIN), in FP32 arithmetic (the low part stays 0).
template <bool PLAIN>
__device__ __forceinline__ void acc_prod(DF& a, float x, float y) {
    if (PLAIN) a.hi = fmaf(x, y, a.hi);
    else df_add(a, df_prod(x, y));
}

// The inner kernels see a scene's padded region (P32 x NY, row-major, the
// pack's pitch between rows) as a run of float4s: thread t of the scene's
// block b takes the four adjacent cells 4q .. 4q+3 for q = b*kRT + t,
// b*kRT + t + nb32*kRT, ... (128-bit accesses: the pack's pitch and every
// scene's column origin are multiples of 128 floats, and P32 of 4, so a
// float4 never crosses a row).  The padding holds zeros.
__device__ __forceinline__ void cell_of(unsigned q, int P32, int& i, int& j) {
    const unsigned c = 4u * q;   // a region holds fewer than 2^31 cells (checked by pack_check)
    j = (int)(c / (unsigned)P32);
    i = (int)(c - (unsigned)j * (unsigned)P32);
}
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 fma4(float a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}

template <bool PLAIN>
__global__ void __launch_bounds__(kRT) k_dot32(const PackScene* __restrict__ sc, const int* __restrict__ blk,
                                               int pitch, const float* __restrict__ z, const float* __restrict__ r,
                                               int init, int max_iters, int* ctl) {
    __shared__ float2 sh[32];
    const PackScene& S = sc[blk[blockIdx.x]];
    PcgScalars* pcg = S.inner;
    if (pcg->done) return;
    const int lb = blockIdx.x - S.blk0;
    const unsigned n4 = (unsigned)S.P32 * (unsigned)S.NY / kRV;
    DF a{0.f, 0.f};
#pragma unroll 2
    for (unsigned q = (unsigned)lb * kRT + threadIdx.x; q < n4; q += (unsigned)S.nb32 * kRT) {
        int i, j;
        cell_of(q, S.P32, i, j);
        const size_t k = (size_t)S.off + (size_t)j * pitch + i;
        const float4 zz = ld4(z + k), rr = ld4(r + k);
        acc_prod<PLAIN>(a, zz.x, rr.x);
        acc_prod<PLAIN>(a, zz.y, rr.y);
        acc_prod<PLAIN>(a, zz.z, rr.z);
        acc_prod<PLAIN>(a, zz.w, rr.w);
    }
    df_block_partial<PLAIN>(a, S.part, lb, sh);
    if (last_block_of(&pcg->ticket[1], S.nb32)) {
        const double s = df_final<PLAIN>(S.part, S.nb32, sh);
        if (threadIdx.x == 0) {
            if (init) {
                pcg->sigma = s;
            } else {
                pcg->beta = s / pcg->sigma;
                pcg->sigma = s;
                pcg->iter += 1;
                pcg->first = 0;
                if (pcg->iter >= max_iters) inner_stop(pcg, 2, ctl);
            }
        }
    }
}

// s_new = z + beta s_old (z on the first iteration), w = A s_new on fluid
// cells, alpha = sigma / (w . s_new).  A cell is fluid unless its FP32
// diagonal carries the -0.0 marker of non-fluid cells; the first and last
// rows and the first column are solid borders, so the neighbour reads stay
// inside the scene's region.
template <bool PLAIN>
__global__ void __launch_bounds__(kRT) k_spmv32(const PackScene* __restrict__ sc, const int* __restrict__ blk,
                                                int pitch, const float* __restrict__ a0, const float* __restrict__ ax,
                                                const float* __restrict__ ay, const float* __restrict__ z,
                                                const float* __restrict__ s_old, float* s_new, float* w, int* ctl) {
    __shared__ float2 sh[32];
    const PackScene& S = sc[blk[blockIdx.x]];
    PcgScalars* pcg = S.inner;
    if (pcg->done) return;
    const bool first = pcg->first != 0;
    const float beta = first ? 0.0f : (float)pcg->beta;
    const int lb = blockIdx.x - S.blk0;
    const unsigned n4 = (unsigned)S.P32 * (unsigned)S.NY / kRV;
    const int P = pitch;
    // s of one cell or four, from z and s_old (the first iteration: z alone)
    auto s1 = [&](size_t k) { return first ? z[k] : fmaf(beta, s_old[k], z[k]); };
    auto s4 = [&](size_t k) { return first ? ld4(z + k) : fma4(beta, ld4(s_old + k), ld4(z + k)); };
    DF a{0.f, 0.f};
    {
        for (unsigned q = (unsigned)lb * kRT + threadIdx.x; q < n4; q += (unsigned)S.nb32 * kRT) {
            int i, j;
            cell_of(q, S.P32, i, j);
            const size_t k = (size_t)S.off + (size_t)j * P + i;
            const float4 sc0 = s4(k);
            st4(s_new + k, sc0);
            float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j > 0 && j < S.NY - 1) {
                const float4 d = ld4(a0 + k);
                if (!(signbit(d.x) && signbit(d.y) && signbit(d.z) && signbit(d.w))) {
                    const float sl = i > 0 ? s1(k - 1) : 0.0f;
                    const float sr = i + kRV < S.P32 ? s1(k + kRV) : 0.0f;
                    const float axl = i > 0 ? ax[k - 1] : 0.0f;
                    const float4 axv = ld4(ax + k), ayd = ld4(ay + k - P), ayv = ld4(ay + k);
                    const float4 sd = s4(k - P), su = s4(k + P);
                    if (!signbit(d.x)) out.x = d.x * sc0.x + axl * sl + axv.x * sc0.y + ayd.x * sd.x + ayv.x * su.x;
                    if (!signbit(d.y)) out.y = d.y * sc0.y + axv.x * sc0.x + axv.y * sc0.z + ayd.y * sd.y + ayv.y * su.y;
                    if (!signbit(d.z)) out.z = d.z * sc0.z + axv.y * sc0.y + axv.z * sc0.w + ayd.z * sd.z + ayv.z * su.z;
                    if (!signbit(d.w)) out.w = d.w * sc0.w + axv.z * sc0.z + axv.w * sr + ayd.w * sd.w + ayv.w * su.w;
                }
            }
            st4(w + k, out);
            acc_prod<PLAIN>(a, out.x, sc0.x);
            acc_prod<PLAIN>(a, out.y, sc0.y);
            acc_prod<PLAIN>(a, out.z, sc0.z);
            acc_prod<PLAIN>(a, out.w, sc0.w);
        }
    }
    df_block_partial<PLAIN>(a, S.part, lb, sh);
    if (last_block_of(&pcg->ticket[2], S.nb32)) {
        const double sum = df_final<PLAIN>(S.part, S.nb32, sh);
        if (threadIdx.x == 0) {
            if (sum == 0.0) inner_stop(pcg, 1, ctl);
            else pcg->alpha = pcg->sigma / sum;
        }
    }
}

// e += alpha s, r -= alpha w, rp = r pc^2, ||r||inf (stop when below the
// inner tolerance, pcg->tol_abs).
__global__ void __launch_bounds__(kRT) k_axpy32(const PackScene* __restrict__ sc, const int* __restrict__ blk,
                                                int pitch, float* e, float* r, float* rp, const float* __restrict__ pc,
                                                const float* __restrict__ s, const float* __restrict__ w, int* ctl) {
    __shared__ float sh[32];
    const PackScene& S = sc[blk[blockIdx.x]];
    PcgScalars* pcg = S.inner;
    if (pcg->done) return;
    const float alpha = (float)pcg->alpha;
    const int lb = blockIdx.x - S.blk0;
    const unsigned n4 = (unsigned)S.P32 * (unsigned)S.NY / kRV;
    float m = 0.f;
    {
#pragma unroll 2
        for (unsigned q = (unsigned)lb * kRT + threadIdx.x; q < n4; q += (unsigned)S.nb32 * kRT) {
            int i, j;
            cell_of(q, S.P32, i, j);
            const size_t k = (size_t)S.off + (size_t)j * pitch + i;
            st4(e + k, fma4(alpha, ld4(s + k), ld4(e + k)));
            const float4 rv = fma4(-alpha, ld4(w + k), ld4(r + k));
            st4(r + k, rv);
            const float4 p = ld4(pc + k);
            st4(rp + k, make_float4(rv.x * (p.x * p.x), rv.y * (p.y * p.y), rv.z * (p.z * p.z), rv.w * (p.w * p.w)));
            m = fmaxf(m, fmaxf(fmaxf(fabsf(rv.x), fabsf(rv.y)), fmaxf(fabsf(rv.z), fabsf(rv.w))));
        }
    }
    m = block_max_f(m, sh);
    float* partf = reinterpret_cast<float*>(S.part);
    if (threadIdx.x == 0) partf[lb] = m;
    if (last_block_of(&pcg->ticket[3], S.nb32)) {
        float mm = 0.f;
        for (int k = threadIdx.x; k < S.nb32; k += blockDim.x) mm = fmaxf(mm, partf[k]);
        mm = block_max_f(mm, sh);
        if (threadIdx.x == 0) {
            pcg->r_norm = mm;
            if (mm <= pcg->tol_abs) inner_stop(pcg, 1, ctl);
        }
    }
}

// End of an inner solve: p += e * ||r||inf (undo the inner scaling) in FP64.
__global__ void k_update64(const PackScene* __restrict__ sc, const int* __restrict__ blk, int pitch,
                           const float* __restrict__ e) {
    const PackScene& S = sc[blk[blockIdx.x]];
    if (!S.inner->active) return;
    const size_t N = (size_t)S.NX * S.NY;
    const size_t c = (size_t)(blockIdx.x - S.blk64) * blockDim.x + threadIdx.x;
    if (c < N) S.p[c] = S.p[c] + (double)e[(size_t)S.off + (c / S.NX) * (size_t)pitch + (c % S.NX)] * S.outer->r_norm;
}

// FP64 residual r = b - A p on fluid cells (the SpMV of :433-444 in FP64) and
// its norm; the scene's last block counts the sweep and ends the refinement
// when the reference's test ||r||inf <= tol * ||b||inf holds or the sweep cap
// is reached.
__global__ void k_resid64(const PackScene* __restrict__ sc, const int* __restrict__ blk, int max_outer, int* ctl) {
    __shared__ double sh[32];
    const PackScene& S = sc[blk[blockIdx.x]];
    PcgScalars* inner = S.inner;
    if (!inner->active) return;
    const int NX = S.NX;
    const size_t N = (size_t)NX * S.NY;
    const int lb = blockIdx.x - S.blk64;
    const size_t c = (size_t)lb * blockDim.x + threadIdx.x;
    double m = 0;
    if (c < N) {
        double v = 0.0;
        if (S.cell[c] == kFluid) {
            const double* A0 = S.A0;
            const double* Ax = S.Ax;
            const double* Ay = S.Ay;
            const double* p = S.p;
            double ap = A0[c] * p[c] + Ax[c - 1] * p[c - 1] + Ax[c] * p[c + 1] + Ay[c - NX] * p[c - NX] +
                        Ay[c] * p[c + NX];
            v = S.rhs[c] - ap;
        }
        S.r[c] = v;
        m = fabs(v);
    }
    m = block_max(m, sh);
    if (threadIdx.x == 0) S.part64[lb] = m;
    PcgScalars* outer = S.outer;
    if (last_block_of(&outer->ticket[0], S.nb64)) {
        double mm = 0;
        for (int k = threadIdx.x; k < S.nb64; k += blockDim.x) mm = fmax(mm, S.part64[k]);
        mm = block_max(mm, sh);
        if (threadIdx.x == 0) {
            outer->r_norm = mm;
            outer->outer_iters += 1;
            outer->inner_total += inner->iter;
            inner->active = 0;
            if (mm <= outer->tol_abs || outer->outer_iters >= max_outer) {
                outer->outer_done = 1;
                atomicSub(&ctl[1], 1);
            }
        }
    }
}

#define PK_LAUNCH_PLAIN(stream, kernel, grid, block, ...)                      \
    do {                                                                        \
        kernel<<<(grid), (block), 0, (stream)>>>(__VA_ARGS__);                  \
        int _rc = ::fs2d::check_cuda(cudaGetLastError(), #kernel);              \
        if (_rc) return _rc;                                                    \
    } while (0)

// A launch of a pack's kernel: counted, timed when asked, errors reported.
#define PK_LAUNCH(L, kernel, grid, block, ...)                                  \
    do {                                                                        \
        (*(L).launches)++;                                                      \
        long long _kt = (L).timer ? ::fs2d::ktimer_begin((L).timer, #kernel) : -1; \
        kernel<<<(grid), (block), 0, (L).stream>>>(__VA_ARGS__);               \
        if ((L).timer) ::fs2d::ktimer_end((L).timer, _kt);                      \
        int _rc = ::fs2d::check_cuda(cudaGetLastError(), #kernel);              \
        if (_rc) return _rc;                                                    \
    } while (0)

}  // namespace

int mic32_make_map(CUtensorMap* map, float* base, int P, int NR) {
    return make_tensor_map_2d(map, base, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, P, kM32Cols, kM32Rows);
}

static_assert(sizeof(Mic32Maps) <= sizeof(Mic32MapsHost::fwd), "tensor map storage");

namespace {

// Tensor maps of the FP32 MIC(0) sweeps over the pack's arrays.
int pack_setup_maps(Pack* pk) {
    Mixed32& m = pk->m;
    Mic32Maps f{}, b{}, c{};
    int rc = 0;
    float* fin[3] = {m.rp, m.fa, m.fb};
    float* bin[3] = {m.q, m.fc, m.fd};
    float* cin[3] = {m.a0, m.fa, m.fb};   // the factor: Adiag and the left / lower terms (prepared in fa, fb)
    for (int a = 0; a < 3 && !rc; a++) rc = mic32_make_map(&f.in[a], fin[a], pk->pitch, pk->rows);
    for (int a = 0; a < 3 && !rc; a++) rc = mic32_make_map(&b.in[a], bin[a], pk->pitch, pk->rows);
    for (int a = 0; a < 3 && !rc; a++) rc = mic32_make_map(&c.in[a], cin[a], pk->pitch, pk->rows);
    if (!rc) rc = mic32_make_map(&f.out, m.q, pk->pitch, pk->rows);
    if (!rc) rc = mic32_make_map(&b.out, m.z, pk->pitch, pk->rows);
    if (!rc) rc = mic32_make_map(&c.out, m.pc, pk->pitch, pk->rows);
    if (rc) return rc;
    memcpy(pk->maps->fwd, &f, sizeof(f));
    memcpy(pk->maps->bwd, &b, sizeof(b));
    memcpy(pk->maps->fac, &c, sizeof(c));
    return 0;
}

template <typename T>
int dev_alloc(T** p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) {
        set_error("cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
        return FS2D_ERR_ALLOC;
    }
    return check_cuda(cudaMemset(*p, 0, (n ? n : 1) * sizeof(T)), "cudaMemset");
}

// The sixteen FP32 arrays of a Mixed32.
void mixed_array_slots(Mixed32& m, float** f[16]) {
    float** g[16] = {&m.a0, &m.ax, &m.ay, &m.pc, &m.fa, &m.fb, &m.fc, &m.fd,
                     &m.r,  &m.rp, &m.q,  &m.z,  &m.w,  &m.s0, &m.s1, &m.e};
    for (int k = 0; k < 16; k++) f[k] = g[k];
}

// Scene table entry of a handle placed at pack column x0, row y0.
PackScene scene_entry(Sim* s, int pitch, int x0, int y0) {
    PackScene e{};
    e.NX = s->NX;
    e.NY = s->NY;
    e.P32 = (s->NX + kM32Cols - 1) / kM32Cols * kM32Cols;
    e.NY32 = (s->NY + kM32Rows - 1) / kM32Rows * kM32Rows;
    e.x0 = x0;
    e.y0 = y0;
    e.off = (long long)y0 * pitch + x0;
    // blocks of the FP32 kernels: one per kRC cells of the padded region, at
    // most 8 per SM of a GB300
    e.nb32 = (int)std::max(1LL, std::min((long long)e.P32 * s->NY / kRC, 1216LL));
    e.nb64 = (int)blocks_for(s->N, kT);
    e.cell = s->cell;
    e.A0 = s->Adiag;
    e.Ax = s->Ax;
    e.Ay = s->Ay;
    e.rhs = s->rhs;
    e.p = s->p;
    e.r = s->r;
    e.outer = s->pcg;
    e.inner = s->pcg32;
    e.part = nullptr;     // the pack's own partials, placed by pack_finish
    e.part64 = nullptr;
    return e;
}

// Every scene's region lies inside the pack's arrays and every pointer the
// kernels follow is set (checked on the host before anything is launched).
int pack_check(const Pack* pk) {
    if (pk->pitch % kM32Cols || pk->rows % kM32Rows || pk->n != (int)pk->scenes.size()) {
        set_error("pack: pitch %d / rows %d not whole strips and tiles", pk->pitch, pk->rows);
        return FS2D_ERR_INVALID;
    }
    for (int k = 0; k < pk->n; k++) {
        const PackScene& e = pk->scenes[k];
        const bool inside = e.x0 >= 0 && e.y0 >= 0 && e.x0 % kM32Cols == 0 && e.P32 >= e.NX && e.NY32 >= e.NY &&
                            e.P32 % kM32Cols == 0 && e.NY32 % kM32Rows == 0 && e.x0 + e.P32 <= pk->pitch &&
                            e.y0 + e.NY32 <= pk->rows && e.off == (long long)e.y0 * pk->pitch + e.x0 &&
                            (long long)e.P32 * e.NY32 < (1LL << 31);
        const bool set = e.cell && e.A0 && e.Ax && e.Ay && e.rhs && e.p && e.r && e.outer && e.inner && e.part &&
                         e.part64 && e.nb32 >= 1 && e.nb64 >= 1;
        if (!inside || !set) {
            set_error("pack: scene %d (%d x %d at %d, %d) does not fit the %d x %d arrays or lacks an array", k,
                      e.NX, e.NY, e.x0, e.y0, pk->pitch, pk->rows);
            return FS2D_ERR_INVALID;
        }
    }
    const Mixed32& m = pk->m;
    const float* arr[16] = {m.a0, m.ax, m.ay, m.pc, m.fa, m.fb, m.fc, m.fd, m.r, m.rp, m.q, m.z, m.w, m.s0, m.s1, m.e};
    for (const float* a : arr)
        if (!a) {
            set_error("pack: FP32 array missing");
            return FS2D_ERR_INVALID;
        }
    return 0;
}

// Block maps, work items and device copies of a pack's scene table.
int pack_finish(Pack* pk) {
    std::vector<int> blk, blk64;
    std::vector<Mic32Item> items;
    for (int k = 0; k < pk->n; k++) {
        PackScene& e = pk->scenes[k];
        e.blk0 = (int)blk.size();
        blk.insert(blk.end(), (size_t)e.nb32, k);
        e.blk64 = (int)blk64.size();
        blk64.insert(blk64.end(), (size_t)e.nb64, k);
        const int ns = e.P32 / kM32Cols;
        const int p0 = (int)items.size();
        for (int st = 0; st < ns; st++) items.push_back(Mic32Item{k, st, ns, e.x0, e.P32, e.y0, e.NY32, p0 + st});
    }
    pk->nblk = (int)blk.size();
    pk->nblk64 = (int)blk64.size();
    pk->nitems = (int)items.size();
    pk->progress_cap = std::max(pk->nitems, 1);
    int rc = 0;
    // reduction partials of every scene: its FP32 blocks' slots from blk0, its
    // FP64 blocks' from blk64, in buffers the pack owns
    if (!rc) rc = dev_alloc(&pk->part, (size_t)pk->nblk);
    if (!rc) rc = dev_alloc(&pk->part64, (size_t)pk->nblk64);
    if (rc) return rc;
    for (PackScene& e : pk->scenes) {
        e.part = pk->part + e.blk0;
        e.part64 = pk->part64 + e.blk64;
    }
    if ((rc = pack_check(pk))) return rc;
    if (!rc) rc = dev_alloc(&pk->d_scenes, pk->scenes.size());
    if (!rc) rc = dev_alloc(&pk->d_blk, blk.size());
    if (!rc) rc = dev_alloc(&pk->d_blk64, blk64.size());
    if (!rc) rc = dev_alloc(&pk->d_items, items.size());
    if (!rc) rc = dev_alloc(&pk->d_ctl, 8);
    if (!rc) rc = dev_alloc(&pk->progress, (size_t)pk->progress_cap);
    if (!rc) rc = dev_alloc(&pk->gprogress, (size_t)pk->progress_cap);
    if (!rc) rc = dev_alloc(&pk->gbase, 1);
    if (rc) return rc;
    FS2D_CUDA(cudaMemcpy(pk->d_scenes, pk->scenes.data(), pk->scenes.size() * sizeof(PackScene),
                         cudaMemcpyHostToDevice));
    FS2D_CUDA(cudaMemcpy(pk->d_blk, blk.data(), blk.size() * sizeof(int), cudaMemcpyHostToDevice));
    FS2D_CUDA(cudaMemcpy(pk->d_blk64, blk64.data(), blk64.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!items.empty())
        FS2D_CUDA(cudaMemcpy(pk->d_items, items.data(), items.size() * sizeof(Mic32Item), cudaMemcpyHostToDevice));
    FS2D_CUDA(cudaMallocHost((void**)&pk->h_ctl, 8 * sizeof(int)));
    memset(pk->h_ctl, 0, 8 * sizeof(int));
    pk->maps = new (std::nothrow) Mic32MapsHost();
    if (!pk->maps) {
        set_error("out of host memory");
        return FS2D_ERR_ALLOC;
    }
    if (int rcm = pack_setup_maps(pk)) return rcm;
    const size_t cells = (size_t)pk->pitch * pk->rows;
    k_fill_marker<<<blocks_for(cells, 256), 256>>>(pk->m.a0, cells);
    return check_cuda(cudaDeviceSynchronize(), "k_fill_marker");
}

}  // namespace

void pack_free(Pack* pk) {
    if (!pk) return;
    if (pk->graph) cudaGraphExecDestroy(pk->graph);
    if (pk->owns_arrays) {
        float** f[16];
        mixed_array_slots(pk->m, f);
        for (int k = 0; k < 16; k++)
            if (*f[k]) cudaFree(*f[k]);
    }
    void* ptrs[] = {pk->d_scenes, pk->d_blk, pk->d_blk64, pk->d_items, pk->d_ctl, pk->progress, pk->gprogress,
                    pk->gbase, pk->part, pk->part64};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (pk->h_ctl) cudaFreeHost(pk->h_ctl);
    delete pk->maps;
    delete pk;
}

int pack_create_single(Sim* s) {
    Pack* pk = new (std::nothrow) Pack();
    if (!pk) {
        set_error("out of host memory");
        return FS2D_ERR_ALLOC;
    }
    pk->n = 1;
    pk->pitch = s->P32;
    pk->rows = s->NY32;
    pk->m = s->m32;
    pk->owns_arrays = false;
    pk->plain = s->opt.precision == FS2D_PRECISION_FP32;
    pk->scenes.push_back(scene_entry(s, s->P32, 0, 0));
    int rc = pack_finish(pk);
    if (rc) {
        pack_free(pk);
        return rc;
    }
    s->pack = pk;
    return 0;
}

// Shelf packing: scenes by decreasing padded height, left to right on
// shelves of a common width (a multiple of 128 columns, at least the widest
// scene and about the square root of the total area), a new shelf when the
// next scene does not fit.
int pack_create_batch(Sim* const* sims, int n, Pack** out) {
    *out = nullptr;
    std::vector<int> order(n);
    long long area = 0;
    int wmax = 0;
    for (int k = 0; k < n; k++) {
        order[k] = k;
        const int w = (sims[k]->NX + kM32Cols - 1) / kM32Cols * kM32Cols;
        const int h = (sims[k]->NY + kM32Rows - 1) / kM32Rows * kM32Rows;
        area += (long long)w * h;
        wmax = std::max(wmax, w);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sims[a]->NY > sims[b]->NY; });
    int width = (int)std::sqrt((double)area);
    width = std::max(wmax, (width + kM32Cols - 1) / kM32Cols * kM32Cols);
    std::vector<int> x0(n), y0(n);
    int x = 0, y = 0, shelf_h = 0;
    for (int k : order) {
        const int w = (sims[k]->NX + kM32Cols - 1) / kM32Cols * kM32Cols;
        const int h = (sims[k]->NY + kM32Rows - 1) / kM32Rows * kM32Rows;
        if (x + w > width) {
            y += shelf_h;
            x = 0;
            shelf_h = 0;
        }
        x0[k] = x;
        y0[k] = y;
        x += w;
        shelf_h = std::max(shelf_h, h);
    }
    const int rows = y + shelf_h;
    Pack* pk = new (std::nothrow) Pack();
    if (!pk) {
        set_error("out of host memory");
        return FS2D_ERR_ALLOC;
    }
    pk->n = n;
    pk->pitch = width;
    pk->rows = rows;
    pk->owns_arrays = true;
    pk->plain = sims[0]->opt.precision == FS2D_PRECISION_FP32;
    float** f[16];
    mixed_array_slots(pk->m, f);
    int rc = 0;
    for (int k = 0; k < 16 && !rc; k++) rc = dev_alloc(f[k], (size_t)width * rows);
    for (int k = 0; k < n && !rc; k++) {
        // the scene's FP32 arrays become views into the pack at its place (its
        // own arrays are released), and its own pack is rebuilt on them
        Sim* s = sims[k];
        const long long off = (long long)y0[k] * width + x0[k];
        float** g[16];
        mixed_array_slots(s->m32, g);
        for (int a = 0; a < 16; a++) {
            if (s->m32_owned && *g[a]) cudaFree(*g[a]);
            *g[a] = *f[a] + off;
        }
        s->m32_owned = false;
        s->P32 = width;
        pack_free(s->pack);
        s->pack = nullptr;
        rc = pack_create_single(s);
        if (!rc) pk->scenes.push_back(scene_entry(s, width, x0[k], y0[k]));
    }
    if (!rc) rc = pack_finish(pk);
    if (rc) {
        pack_free(pk);
        return rc;
    }
    // persistent sweep CTAs: one per SM (a sweep CTA takes most of an SM's
    // shared memory), at most one per work item
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    pk->sweep_ctas = std::max(1, std::min(sms, pk->nitems));
    *out = pk;
    return 0;
}

// FP32 copies of the matrix, the MIC(0) factor and the folded coefficients of
// the handle's built system (its region of its pack's arrays).
int mixed_setup(Sim* s) {
    const int NX = s->NX, NY = s->NY, P = s->P32;
    const size_t N = s->N;
    const unsigned nb = blocks_for(N, kT);
    Mixed32& m = s->m32;
    FS2D_LAUNCH(s, k_mixed_matrix, nb, kT, 0, s->Adiag, s->Ax, s->Ay, m.a0, m.ax, m.ay, NX, P, N);
    // the factor itself runs for every scene of the pack at the start of its solve
    FS2D_LAUNCH(s, k_factor_prep, nb, kT, 0, m.ax, m.ay, m.fa, m.fb, (float)s->opt.mic_tau, NX, NY, P);
    return 0;
}

constexpr int kM32GraphIters = 8;   // inner iterations per graph replay (even: the search-direction ping-pong)

// One inner iteration of every scene of the pack; graph = inside a stream capture.
static int pack_iteration(Pack* pk, PackLaunch& L, int it, bool graph, int max_iters) {
    Mixed32& m = pk->m;
    float* sbuf[2] = {m.s0, m.s1};
    float* s_old = sbuf[it & 1];
    float* s_new = sbuf[(it + 1) & 1];
    if (pk->plain)
        PK_LAUNCH(L, k_spmv32<true>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.a0, m.ax, m.ay, m.z, s_old,
                  s_new, m.w, pk->d_ctl);
    else
        PK_LAUNCH(L, k_spmv32<false>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.a0, m.ax, m.ay, m.z, s_old,
                  s_new, m.w, pk->d_ctl);
    PK_LAUNCH(L, k_axpy32, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.e, m.r, m.rp, m.pc, s_new, m.w,
              pk->d_ctl);
    const int slot = graph ? 2 * (it % kM32GraphIters) : -1;   // sweeps of one replay
    int rc = launch_mic32<true>(pk, L, m.q, slot, 2 * kM32GraphIters);
    if (rc) return rc;
    rc = launch_mic32<false>(pk, L, m.z, graph ? slot + 1 : -1, 2 * kM32GraphIters);
    if (rc) return rc;
    if (pk->plain)
        PK_LAUNCH(L, k_dot32<true>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.z, m.r, 0, max_iters, pk->d_ctl);
    else
        PK_LAUNCH(L, k_dot32<false>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.z, m.r, 0, max_iters,
                  pk->d_ctl);
    return 0;
}

// Captures kM32GraphIters inner iterations as a CUDA graph (once per pack);
// false: launch directly (per-kernel timing is on, or capture is not
// available here).
static bool pack_graph(Pack* pk, PackLaunch& L, int max_iters) {
    if ((L.timer && !L.timer->kt_patterns.empty()) || pk->graph_state < 0) return false;
    if (pk->graph_state == 1) return true;
    pk->graph_state = -1;   // until the capture below succeeds
    const unsigned long long l0 = *L.launches;
    if (cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    int rc1 = 0;
    for (int k = 0; k < kM32GraphIters && !rc1; k++) rc1 = pack_iteration(pk, L, k, true, max_iters);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(L.stream, &g);
    pk->graph_launches = *L.launches - l0;
    *L.launches = l0;   // captured, not run
    if (rc1 || e != cudaSuccess || g == nullptr) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return false;
    }
    e = cudaGraphInstantiate(&pk->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        pk->graph = nullptr;
        return false;
    }
    pk->graph_state = 1;
    return true;
}

// The refinement loop of every scene of the pack: FP32 inner solves of
// A e = r / ||r||inf (batches of iterations replayed from a CUDA graph until
// every scene's inner solve stopped), p += e ||r||inf and the FP64 residual,
// until every scene met the reference's stopping test or the sweep cap.  The
// host polls one counter per graph replay and one per sweep for the whole pack.
static int pack_solve_impl(Pack* pk, const fs2d_options& opt_in, PackLaunch& L) {
    Mixed32& m = pk->m;
    fs2d_options opt = opt_in;
    if (pk->plain) {
        // plain FP32 PCG: one FP32 solve to the solve's own tolerance (the FP64
        // residual is still computed once, for the statistics and the status)
        opt.ir_max_outer = 1;
        opt.ir_inner_tol = opt.pcg_tol;
    }
    const int max_iters = opt.pcg_max_iters;
    const int batch = 4;
    // MIC(0) factor of every scene (one forward sweep of the pack), then the
    // folded coefficients of the triangular solves
    if (int rcf = launch_mic32<true, kM32Factor>(pk, L, m.pc, -1, 0, (float)opt.mic_sigma)) return rcf;
    PK_LAUNCH(L, k_mixed_coef, pk->nblk, 256, pk->d_scenes, pk->d_blk, pk->pitch, m.ax, m.ay, m.pc, m.fa, m.fb,
              m.fc, m.fd);
    FS2D_CUDA(cudaMemsetAsync(pk->d_ctl, 0, 2 * sizeof(int), L.stream));
    PK_LAUNCH(L, k_outer_start, blocks_for(pk->n, 128), 128, pk->d_scenes, pk->n, pk->d_ctl);
    auto poll = [&](int which, int* value) -> int {
        FS2D_CUDA(cudaMemcpyAsync(pk->h_ctl + which, pk->d_ctl + which, sizeof(int), cudaMemcpyDeviceToHost, L.stream));
        FS2D_CUDA(cudaStreamSynchronize(L.stream));
        *value = pk->h_ctl[which];
        return 0;
    };
    int refining = 0;
    if (int rc = poll(1, &refining)) return rc;
    for (int outer = 0; outer < opt.ir_max_outer && refining > 0; outer++) {
        PK_LAUNCH(L, k_inner_init, pk->nblk64, kT, pk->d_scenes, pk->d_blk64, pk->pitch, m.pc, m.r, m.rp, m.e,
                  opt.ir_inner_tol, pk->d_ctl);
        int rc = launch_mic32<true>(pk, L, m.q);
        if (rc) return rc;
        rc = launch_mic32<false>(pk, L, m.z);
        if (rc) return rc;
        if (pk->plain)
            PK_LAUNCH(L, k_dot32<true>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.z, m.r, 1, max_iters,
                      pk->d_ctl);
        else
            PK_LAUNCH(L, k_dot32<false>, pk->nblk, kRT, pk->d_scenes, pk->d_blk, pk->pitch, m.z, m.r, 1, max_iters,
                      pk->d_ctl);
        int it = 0, running = 1;
        if (pack_graph(pk, L, max_iters)) {
            // whole batches of iterations from the captured graph (kernels of a
            // scene whose inner solve stopped return at once)
            for (; it + kM32GraphIters <= max_iters + kM32GraphIters && running > 0; it += kM32GraphIters) {
                FS2D_CUDA(cudaGraphLaunch(pk->graph, L.stream));
                *L.launches += pk->graph_launches;
                if ((rc = poll(0, &running))) return rc;
            }
        }
        for (; it < max_iters && running > 0; it++) {
            if ((rc = pack_iteration(pk, L, it, false, max_iters))) return rc;
            if ((it + 1) % batch == 0 || it + 1 == max_iters) {
                if ((rc = poll(0, &running))) return rc;
            }
        }
        PK_LAUNCH(L, k_update64, pk->nblk64, kT, pk->d_scenes, pk->d_blk64, pk->pitch, m.e);
        PK_LAUNCH(L, k_resid64, pk->nblk64, kT, pk->d_scenes, pk->d_blk64, opt.ir_max_outer, pk->d_ctl);
        if ((rc = poll(1, &refining))) return rc;
    }
    return 0;
}

int pack_solve(Pack* pk, const fs2d_options& opt, cudaStream_t stream, unsigned long long* launches, int* err,
               int device, Sim* timer) {
    PackLaunch L{stream, err, device, launches, pk->wave_launch, timer};
    int rc = pack_solve_impl(pk, opt, L);
    pk->wave_launch = L.wave_launch;
    return rc;
}

namespace {
// Sets the inner-solve stop flag of every scene of the pack (one thread per scene).
__global__ void k_set_done(const PackScene* __restrict__ sc, int n, int done) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) sc[k].inner->done = done;
}
}  // namespace

// Autotuner of the persistent sweep of several scenes: the schedule (the
// order of the work list: whole scenes as given, by decreasing rows or by
// decreasing cells, strip-major, or critical path first) and the number of persistent CTAs
// (all SMs, three quarters, half) are each timed on forward sweeps of the
// pack (CUDA events, after a warm-up sweep), and the fastest pair is kept.
// A scene's results do not depend on either choice: its strips are computed
// in the same order by the same step code whichever CTA takes them.
// The work list of schedule `variant` (see pack_tune).
static std::vector<Mic32Item> pack_schedule(const Pack* pk, int variant) {
    std::vector<int> order(pk->n);
    std::vector<int> strip0(pk->n);   // progress counter of each scene's first strip (as pack_finish numbers them)
    for (int k = 0, c = 0; k < pk->n; k++) {
        strip0[k] = c;
        c += pk->scenes[k].P32 / kM32Cols;
    }
    std::iota(order.begin(), order.end(), 0);
    if (variant == 1)
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return pk->scenes[a].NY32 > pk->scenes[b].NY32; });
    if (variant == 2)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return (long long)pk->scenes[a].NY32 * pk->scenes[a].P32 > (long long)pk->scenes[b].NY32 * pk->scenes[b].P32;
        });
    std::vector<Mic32Item> items;
    if (variant == 4) {
        // critical path first: a strip's rank is the time from its start to
        // the end of its scene's last strip if nothing waits, (strips after
        // it) x the strip-to-strip lag + its own steps, in column steps (lag
        // ~66 steps measured); a scene's strips keep their order because the
        // rank falls along the scene
        struct Ranked {
            long long rank;
            Mic32Item item;
        };
        std::vector<Ranked> all;
        for (int k = 0; k < pk->n; k++) {
            const PackScene& e = pk->scenes[k];
            const int ns = e.P32 / kM32Cols;
            for (int st = 0; st < ns; st++)
                all.push_back(Ranked{(long long)(ns - 1 - st) * 66 + e.NY32 + 31,
                                     Mic32Item{k, st, ns, e.x0, e.P32, e.y0, e.NY32, strip0[k] + st}});
        }
        std::stable_sort(all.begin(), all.end(), [](const Ranked& a, const Ranked& b) { return a.rank > b.rank; });
        for (const Ranked& r : all) items.push_back(r.item);
        return items;
    }
    if (variant < 3) {
        for (int k : order) {
            const PackScene& e = pk->scenes[k];
            const int ns = e.P32 / kM32Cols;
            for (int st = 0; st < ns; st++)
                items.push_back(Mic32Item{k, st, ns, e.x0, e.P32, e.y0, e.NY32, strip0[k] + st});
        }
    } else {
        // strip-major: every scene's first strip (scenes by decreasing rows),
        // then every second strip, ...: a strip is taken long after the strip
        // it waits for, so its left column is usually there already
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return pk->scenes[a].NY32 > pk->scenes[b].NY32; });
        for (int st = 0;; st++) {
            bool any = false;
            for (int k : order) {
                const PackScene& e = pk->scenes[k];
                const int ns = e.P32 / kM32Cols;
                if (st < ns) {
                    items.push_back(Mic32Item{k, st, ns, e.x0, e.P32, e.y0, e.NY32, strip0[k] + st});
                    any = true;
                }
            }
            if (!any) break;
        }
    }
    return items;
}

int pack_set_schedule(Pack* pk, int schedule, int ctas, cudaStream_t stream) {
    if (pk->n < 2 || schedule < 0 || schedule > 4 || ctas < 0) {
        set_error("schedule %d / %d CTAs: a batch's schedule is 0..4 and its CTA count >= 0", schedule, ctas);
        return FS2D_ERR_INVALID;
    }
    const std::vector<Mic32Item> items = pack_schedule(pk, schedule);
    FS2D_CUDA(cudaMemcpyAsync(pk->d_items, items.data(), items.size() * sizeof(Mic32Item), cudaMemcpyHostToDevice,
                              stream));
    FS2D_CUDA(cudaStreamSynchronize(stream));
    pk->schedule = schedule;
    if (ctas > 0) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        pk->sweep_ctas = std::max(1, std::min({ctas, sms, pk->nitems}));
    }
    return 0;
}

int pack_tune(Pack* pk, cudaStream_t stream, int* err, int device, unsigned long long* launches, double* best_us) {
    if (pk->n < 2) return 0;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    std::vector<std::vector<Mic32Item>> schedules;
    for (int variant = 0; variant < 5; variant++) schedules.push_back(pack_schedule(pk, variant));
    const int ctas[3] = {sms, sms * 3 / 4, sms / 2};
    cudaEvent_t e0, e1;
    FS2D_CUDA(cudaEventCreate(&e0));
    FS2D_CUDA(cudaEventCreate(&e1));
    PK_LAUNCH_PLAIN(stream, k_set_done, blocks_for(pk->n, 128), 128, pk->d_scenes, pk->n, 0);
    PackLaunch L{stream, err, device, launches, pk->wave_launch, nullptr};
    double best = 1e300;
    int best_s = 0, best_c = sms;
    int rc = 0;
    for (int si = 0; si < (int)schedules.size() && !rc; si++) {
        rc = check_cuda(cudaMemcpyAsync(pk->d_items, schedules[si].data(), schedules[si].size() * sizeof(Mic32Item),
                                        cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync");
        for (int ci = 0; ci < 3 && !rc; ci++) {
            pk->sweep_ctas = std::max(1, std::min(ctas[ci], pk->nitems));
            rc = launch_mic32<true>(pk, L, pk->m.q);   // warm-up
            if (!rc) rc = check_cuda(cudaEventRecord(e0, stream), "cudaEventRecord");
            for (int r = 0; r < 3 && !rc; r++) rc = launch_mic32<true>(pk, L, pk->m.q);
            if (!rc) rc = check_cuda(cudaEventRecord(e1, stream), "cudaEventRecord");
            if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0;
            if (!rc) cudaEventElapsedTime(&ms, e0, e1);
            if (!rc && ms < best) {
                best = ms;
                best_s = si;
                best_c = pk->sweep_ctas;
            }
        }
    }
    if (!rc) rc = check_cuda(cudaMemcpyAsync(pk->d_items, schedules[best_s].data(),
                                             schedules[best_s].size() * sizeof(Mic32Item), cudaMemcpyHostToDevice,
                                             stream), "cudaMemcpyAsync");
    pk->sweep_ctas = best_c;
    pk->schedule = best_s;
    pk->wave_launch = L.wave_launch;
    if (!rc) {
        k_set_done<<<blocks_for(pk->n, 128), 128, 0, stream>>>(pk->d_scenes, pk->n, 1);
        rc = check_cuda(cudaGetLastError(), "k_set_done");
    }
    if (!rc) rc = check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_us) *best_us = best * 1000.0 / 3;
    return rc;
}

int mixed_finish(Sim* s, int* status) {
    if (int rc = mixed_finish_queue(s)) return rc;
    if (int rcw = wait_stream(s, s->stream)) return rcw;
    mixed_finish_read(s, status);
    return 0;
}

// The solver's scalars to the host, queued on the handle's stream.
int mixed_finish_queue(Sim* s) {
    FS2D_CUDA(cudaMemcpyAsync(s->pcg_host, s->pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
    return 0;
}

// Statistics and status of the solve, once the copy queued by
// mixed_finish_queue has arrived.
void mixed_finish_read(Sim* s, int* status) {
    const PcgScalars& o = *s->pcg_host;
    s->last_iters = o.inner_total;
    s->last_outer = o.outer_iters;
    const bool solved = o.rhs_norm > 1e-12;
    s->last_rel_res = o.rhs_norm > 0 ? (solved ? o.r_norm : o.rhs_norm) / o.rhs_norm : 0.0;
    if (status) *status = (solved && o.r_norm > o.tol_abs) ? FS2D_ERR_NOT_CONVERGED : 0;
}

int projection_mixed(Sim* s, int* status) { return projection_mixed_rhs(s, nullptr, status); }

// b == nullptr: the physical right-hand side; otherwise A p = b for a device
// array b on the fluid cells.
int projection_mixed_rhs(Sim* s, const double* b, int* status) {
    // the FP64 matrix, rhs, ||b||inf, p = 0, r = b (exactly the reference's)
    int rc = projection_build(s);
    if (rc) return rc;
    if (b && (rc = projection_set_rhs(s, b))) return rc;
    if ((rc = mixed_setup(s))) return rc;
    if ((rc = pack_solve(s->pack, s->opt, s->stream, &s->launches, s->err, s->device, s))) return rc;
    return mixed_finish(s, status);
}

}  // namespace fs2d
