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
__device__ __forceinline__ int ld_acquire_int(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_int(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
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

// Controls of the bounded waits (see kErrWords): polls before a wait between
// strips gives up, and whether the test hook holds back `strip`'s hand-off
// in sweeps of `kind`.
__device__ __forceinline__ long long wave_spin(const int* err) {
    return *reinterpret_cast<const volatile long long*>(err + 4);
}
// A wait of some sweep already gave up (other waits then give up early).
__device__ __forceinline__ bool wave_failed(const int* err) { return (*(const volatile int*)err & 1) != 0; }
__device__ __forceinline__ bool wave_held(const int* err, int kind, int strip) {
    return (err[1] & kind) != 0 && err[2] == strip;
}

// Level-set sweeps of several scenes in one launch: persistent CTAs take
// work items (one strip of one scene each) in list order from work[0];
// work[1] counts the CTAs that finished, and the last one resets both for
// the next launch.  A strip's previous strip comes earlier in the list, so
// the CTA it waits for took its item earlier and is running.  Progress
// counter pidx belongs to the item's strip, pidx - 1 to the scene's previous
// strip; an item of a scene whose skip flag is set is passed over.
struct WaveItem {
    int scene, strip, pidx;
};
struct WaveWork {
    const void* scenes;                  // CpScene[] or EkScene[]
    const WaveItem* items;
    int nitems;
    int* work;
    unsigned long long* progress;
    unsigned long long base;
    int* err;
    const int* skip;                     // per scene
    const uint2* rng;                    // Eikonal sweeps: per strip (counter order), its column range
};

}  // namespace fs2d
