// fs2d_device.cuh — device helpers shared by the stage kernels.
//
// Files that include this header and implement FP64 stages are compiled with
// --fmad=false: no multiply-add is fused, so every expression below rounds
// exactly like the reference's scalar C++ build (-ffp-contract=off).  The
// order of operations in each helper follows the reference expression it
// cites; changing it changes results in the last bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "fs2d_internal.cuh"

namespace fs2d {

// aml::max / aml::min / aml::clamp semantics (first argument wins ties).
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dclamp(double v, double lo, double hi) { return dmin(dmax(v, lo), hi); }
__device__ __forceinline__ int iclamp(int v, int lo, int hi) {
    int m = (v < lo) ? lo : v;
    return (hi < m) ? hi : m;
}

// Array2D::triCubic, scalar branch (include/Array2D.h:244-249,328-355):
// Catmull-Rom weights and a row-by-row weighted sum with clamped indices.
template <typename T>
__device__ __forceinline__ T tricubic(const T* __restrict__ data, int W, int H, T px, T py) {
    int x = (int)px, y = (int)py;
    if (x < 0 || x >= W || y < 0 || y >= H) return T(0);
    T dx = px - (T)x, dy = py - (T)y;
    T u[4], v[4];
    u[0] = T(-0.5) * (dx * dx * dx) + (dx * dx) - T(0.5) * dx;
    u[1] = T(1.5) * (dx * dx * dx) - T(2.5) * (dx * dx) + T(1);
    u[2] = T(-1.5) * (dx * dx * dx) + T(2) * (dx * dx) + T(0.5) * dx;
    u[3] = T(0.5) * (dx * dx * dx) - T(0.5) * (dx * dx);
    v[0] = T(-0.5) * (dy * dy * dy) + (dy * dy) - T(0.5) * dy;
    v[1] = T(1.5) * (dy * dy * dy) - T(2.5) * (dy * dy) + T(1);
    v[2] = T(-1.5) * (dy * dy * dy) + T(2) * (dy * dy) + T(0.5) * dy;
    v[3] = T(0.5) * (dy * dy * dy) - T(0.5) * (dy * dy);
    int xs[4];
#pragma unroll
    for (int i = 0; i < 4; i++) xs[i] = iclamp(x + i - 1, 0, W - 1);
    T vox = T(0);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const T* row = data + (size_t)iclamp(y + j - 1, 0, H - 1) * W;
        T r = T(0);
#pragma unroll
        for (int i = 0; i < 4; i++) r += u[i] * row[xs[i]];
        vox += v[j] * r;
    }
    return vox;
}

// MACGrid2D::velInterpU / velInterpV (include/MACGrid2D.h:80-97): world
// position -> face-grid coordinates, clamped to [1e-6, N-1-1e-6] in cell
// units (NX for x, NY for y, for both components), then triCubic.
__device__ __forceinline__ double vel_interp_u(const double* __restrict__ u, int NX, int NY, double dx, double x,
                                               double y) {
    double px = x / dx, py = y / dx;
    py -= 0.5;
    px = dclamp(px, 1e-6, (double)(NX - 1) - 1e-6);
    py = dclamp(py, 1e-6, (double)(NY - 1) - 1e-6);
    return tricubic<double>(u, NX + 1, NY, px, py);
}
__device__ __forceinline__ double vel_interp_v(const double* __restrict__ v, int NX, int NY, double dx, double x,
                                               double y) {
    double px = x / dx, py = y / dx;
    px -= 0.5;
    px = dclamp(px, 1e-6, (double)(NX - 1) - 1e-6);
    py = dclamp(py, 1e-6, (double)(NY - 1) - 1e-6);
    return tricubic<double>(v, NX, NY + 1, px, py);
}

// FluidSim2D::clampPos (src/FluidSim2D.cpp:645-651)
__device__ __forceinline__ void clamp_pos(int NX, int NY, double dx, double& x, double& y) {
    const double offset = 1e-3;
    x = dclamp(x, (1.0 + offset) * dx, (NX - 1.0 - offset) * dx);
    y = dclamp(y, (1.0 + offset) * dx, (NY - 1.0 - offset) * dx);
}

// ---- reductions ----
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
// Block-wide sum / max; result valid in thread 0.  `sh` holds >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    return v;
}
__device__ __forceinline__ double block_max(double v, double* sh) {
    v = warp_max(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_max(v);
    return v;
}

// Last-block-done: thread 0 of each block calls after writing its partial;
// returns true in exactly one block (the last), which may then read every
// partial.  The ticket is reset for the next launch.
__device__ __forceinline__ bool last_block(unsigned int* ticket) {
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x * gridDim.y - 1);
        if (is_last) *ticket = 0;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// ---- acquire / release flags for the wavefront ----
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Geometry of one Gauss-Seidel sweep: cells i in [i_lo, i_hi], j in
// [j_lo, j_hi] (inclusive), visited in the reference's loop order for
// direction (sx, sy): rows in order of sy, and within a row columns in order
// of sx.  Cell (i, j) then depends only on (i - sx, j) and (i, j - sy) of
// the same sweep, so anti-diagonals of the (sx, sy)-oriented grid can run
// in parallel and reproduce the serial result exactly.
struct WaveGeom {
    int sx, sy;
    int i_lo, i_hi, j_lo, j_hi;
};

constexpr int kWavePublish = 8;                 // columns per progress publication
constexpr long long kWaveSpinLimit = 1ll << 22; // polls before giving up (~0.5 s)
constexpr int kWavePrefetch = 32;               // columns of look-ahead for the L1 prefetch
constexpr int kWaveQueue = 4;                   // lane 0: below-row values loaded ahead

__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Strip wavefront: block k (32 threads) owns rows 32k .. 32k+31 in sweep
// order, lane l one row.  At step s lane l visits column c = s - l, so the
// warp forms a diagonal front; the value of the cell below (previous row in
// sweep order) arrives by shuffle from lane l-1, the value of the previous
// column stays in the lane's register.  Lane 0 reads the last row of strip
// k-1 from L2 after waiting on that strip's progress counter, which lane 31
// of strip k-1 publishes (release) every kWavePublish columns; it loads
// those values kWaveQueue columns ahead of use so the L2 round trip stays
// off the critical path.  Every lane prefetches its own row's operands into
// L1 kWavePrefetch columns ahead.  The wait is bounded: on timeout bit 0 of
// *err is set and the strip carries on (results are then invalid, but
// nothing hangs).
//
// Op interface:
//   typename Op::Carry;                       value handed to the next column / row
//   Carry op.fetch(int i, int j, bool l2)     value of a cell outside this strip
//   Carry op.update(int i, int j, Carry prev_x, Carry prev_y)
//   void op.prefetch(int i, int j)            L1 prefetch of what update(i, j) reads
//   static Carry Op::shfl_up(Carry c)         __shfl_up_sync by one lane
template <class Op>
__global__ void __launch_bounds__(32) wave_kernel(Op op, WaveGeom g, unsigned long long* progress,
                                                  unsigned long long base, int* err, const int* skip) {
    typedef typename Op::Carry Carry;
    if (skip != nullptr && *skip) return;
    const int lane = threadIdx.x;
    const int k = blockIdx.x;
    const int ncols = g.i_hi - g.i_lo + 1;
    const int nrows = g.j_hi - g.j_lo + 1;
    const int row = k * 32 + lane;
    const bool valid = row < nrows;
    const int j = g.sy > 0 ? g.j_lo + row : g.j_hi - row;
    Carry out{};
    const unsigned long long* prev = (k > 0) ? progress + (k - 1) : nullptr;
    unsigned long long avail = 0;
    bool gave_up = false;
    const bool publisher = (lane == 31) && valid && (k * 32 + 32 < nrows);
    auto col = [&](int c) { return g.sx > 0 ? g.i_lo + c : g.i_hi - c; };
    // lane 0: below-row value of column cc, waiting for its publication first
    auto below_of = [&](int cc) -> Carry {
        if (prev != nullptr && !gave_up) {
            unsigned long long need = base + (unsigned long long)min(((cc / kWavePublish) + 1) * kWavePublish, ncols);
            if (avail < need) {
                long long polls = 0;
                unsigned long long v;
                while ((v = ld_acquire(prev)) < need) {
                    if (++polls > kWaveSpinLimit || *(volatile int*)err) {
                        atomicOr(err, 1);
                        gave_up = true;
                        break;
                    }
                    __nanosleep(32);
                }
                avail = v;
            }
        }
        return op.fetch(col(cc), j - g.sy, prev != nullptr);
    };
    Carry bq[kWaveQueue];
    if (lane == 0 && valid) {
#pragma unroll
        for (int q = 0; q < kWaveQueue; q++) bq[q] = (q < ncols) ? below_of(q) : Carry{};
    }
    if (valid) {
        for (int c = 0; c < min(kWavePrefetch, ncols); c += 8) op.prefetch(col(c), j);
    }
    for (int s = 0; s < ncols + 31; ++s) {
        const int c = s - lane;
        Carry below = Op::shfl_up(out);
        if (valid && c >= 0 && c < ncols) {
            const int i = col(c);
            if ((c & 7) == 0 && c + kWavePrefetch < ncols) op.prefetch(col(c + kWavePrefetch), j);
            if (lane == 0) {
                below = bq[0];
#pragma unroll
                for (int q = 0; q < kWaveQueue - 1; q++) bq[q] = bq[q + 1];
                if (c + kWaveQueue < ncols) bq[kWaveQueue - 1] = below_of(c + kWaveQueue);
            }
            Carry left = (c > 0) ? out : op.fetch(i - g.sx, j, false);
            out = op.update(i, j, left, below);
            if (publisher && (((c + 1) % kWavePublish) == 0 || c == ncols - 1)) {
                st_release(progress + k, base + (unsigned long long)(c + 1));
            }
        }
        __syncwarp();
    }
}

// Launches a wavefront sweep; blocks are co-resident (cooperative launch) so
// the waits between strips always make progress.
template <class Op>
int launch_wave(Sim* s, const Op& op, WaveGeom g, const int* skip) {
    int nrows = g.j_hi - g.j_lo + 1;
    int ncols = g.i_hi - g.i_lo + 1;
    if (nrows <= 0 || ncols <= 0) return 0;
    int nstrips = (nrows + 31) / 32;
    if (nstrips > s->progress_cap) {
        set_error("wavefront: %d strips exceed the %d progress counters", nstrips, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    // One strip per SM: the strips of a sweep run concurrently and, on GB300,
    // strips sharing an SM contend for its small FP64 pipe.  Reserving more
    // than half of the SM's shared memory keeps every strip on its own SM.
    const int kReserve = 120 * 1024;
    static std::atomic<unsigned long long> configured{0};
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)wave_kernel<Op>, kReserve)) return rc0;
    unsigned long long base = wave_begin(s);
    void* args[] = {(void*)&op, (void*)&g, (void*)&s->progress, (void*)&base, (void*)&s->err, (void*)&skip};
    s->launches++;
    long long kt = ktimer_begin(s, Op::kName);
    int rc = check_cuda(cudaLaunchCooperativeKernel((const void*)wave_kernel<Op>, dim3(nstrips), dim3(32), args,
                                                    kReserve, s->stream),
                        Op::kName);
    ktimer_end(s, kt);
    return rc;
}

}  // namespace fs2d
