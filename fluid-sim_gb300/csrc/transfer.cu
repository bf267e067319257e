// transfer.cu — particle/grid transfers and velocity extrapolation (FP64, exact).
//
//   FluidSim2D::transferVelocityToGrid   src/FluidSim2D.cpp:144-204   (P2G)
//   FluidSim2D::updateParticleVelocities src/FluidSim2D.cpp:552-568   (G2P)
//   Array2D::linearDistribute / linearExtract  include/Array2D.h:361-420
//   Array2D::extrapolate                 include/Array2D.h:552-591
// Compiled with --fmad=false.
//
// P2G, ordered mode: the reference adds each particle's four bilinear
// contributions into the face grid in particle order.  Here every
// contribution becomes a key (4*e + corner) in its face's bucket (counting
// sort: count, exclusive scan, scatter); each face then sorts its few keys
// and adds them in key order — the reference's order — so the sums are
// bit-identical and independent of thread scheduling.  Atomic mode sums
// each warp's contributions per face and adds them with FP64 atomics (fast,
// order not reproducible).
//
// Extrapolation: the reference's breadth-first search assigns every unknown
// face a layer L = its 4-connected (L1) grid distance to the nearest known
// face and sets it to the mean of its neighbours with layer < L, which are
// all final before any layer-L face is visited.  So the result depends only
// on the layers, not on the queue order.  Layers come from an exact
// separable L1 distance transform; values are then propagated in bands of
// kBand layers, each 32x32 output tile recomputing its band inside a halo of
// kBand cells (every dependency of a layer in the band lies within kBand
// cells), so one launch per band replaces one launch per layer.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <mutex>
#include "fs2d_device.cuh"

namespace fs2d {
namespace {

constexpr int kBand = 16;
constexpr int kTile = 32;
constexpr int kReg = kTile + 2 * kBand;
constexpr int kInf = 1 << 29;

// Bilinear corner k (0: (x1,y1), 1: (x2,y1), 2: (x1,y2), 3: (x2,y2)) of a
// position, with clamped indices and unclamped weights (include/Array2D.h:361-376).
struct Bilinear {
    int x1, x2, y1, y2;
    double dxp, dyp;
    __device__ Bilinear(double px, double py, int W, int H) {
        int ui = (int)px, uj = (int)py;
        dxp = px - ui;
        dyp = py - uj;
        x1 = iclamp(ui, 0, W - 1);
        x2 = iclamp(ui + 1, 0, W - 1);
        y1 = iclamp(uj, 0, H - 1);
        y2 = iclamp(uj + 1, 0, H - 1);
    }
    __device__ int face(int k, int W) const {
        int x = (k & 1) ? x2 : x1, y = (k & 2) ? y2 : y1;
        return y * W + x;
    }
    // linearDistribute's contribution: weight * value, evaluated as the
    // reference does ((wx * wy) * value).
    __device__ double contrib(int k, double value) const {
        double wx = (k & 1) ? dxp : (1 - dxp);
        double wy = (k & 2) ? dyp : (1 - dyp);
        return wx * wy * value;
    }
};

__device__ __forceinline__ void upos(double2 p, double dx, double& x, double& y) { x = p.x / dx; y = p.y / dx - 0.5; }
__device__ __forceinline__ void vpos(double2 p, double dx, double& x, double& y) { x = p.x / dx - 0.5; y = p.y / dx; }

__global__ void k_p2g_count(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY, uint32_t* cnt_u,
                            uint32_t* cnt_v) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        atomicAdd(cnt_u + bu.face(k, NX + 1), 1u);
        atomicAdd(cnt_v + bv.face(k, NX), 1u);
    }
}

__global__ void k_p2g_fill(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY,
                           const uint32_t* __restrict__ off_u, const uint32_t* __restrict__ off_v, uint32_t* fill_u,
                           uint32_t* fill_v, uint32_t* ent_u, uint32_t* ent_v) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int fu = bu.face(k, NX + 1);
        ent_u[off_u[fu] + atomicAdd(fill_u + fu, 1u)] = (uint32_t)(4 * e + k);
        int fv = bv.face(k, NX);
        ent_v[off_v[fv] + atomicAdd(fill_v + fv, 1u)] = (uint32_t)(4 * e + k);
    }
}

// Per face: sort the bucket's keys, then accumulate value and weight in key
// order from 0.0, divide where the weight is positive, and mark faces whose
// value is exactly 0.0 unknown (src/FluidSim2D.cpp:175-201).
template <int COMP>
__global__ void k_p2g_sum(const double2* __restrict__ pos, const double2* __restrict__ vel, double dx, int NX, int NY,
                          int W, int H, const uint32_t* __restrict__ off, uint32_t* ent, size_t nfaces, double* out,
                          uint32_t* mask) {
    size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (f >= nfaces) return;
    uint32_t b = off[f], e_ = off[f + 1];
    // insertion sort of the bucket (buckets hold a few keys per particle nearby)
    for (uint32_t a = b + 1; a < e_; a++) {
        uint32_t key = ent[a];
        uint32_t c = a;
        while (c > b && ent[c - 1] > key) {
            ent[c] = ent[c - 1];
            c--;
        }
        ent[c] = key;
    }
    double sum = 0.0, wsum = 0.0;
    for (uint32_t a = b; a < e_; a++) {
        uint32_t key = ent[a];
        size_t e = key >> 2;
        int k = key & 3;
        double2 p = pos[e];
        double x, y;
        if (COMP == 0) upos(p, dx, x, y); else vpos(p, dx, x, y);
        Bilinear bl(x, y, W, H);
        double value = COMP == 0 ? vel[e].x : vel[e].y;
        sum += bl.contrib(k, value);
        wsum += bl.contrib(k, 1.0);
    }
    if (wsum > 0) sum /= wsum;
    out[f] = sum;
    mask[f] = (sum == 0.0) ? kUnknown : 0u;
}

// Warp-aggregated add: the lanes of a warp that add to the same face (f >= 0)
// first sum their (value, weight) pairs — each lane adds its successor's
// partial sum along the list of lanes with that face, jumping pointers, so
// after five rounds the first lane of the list holds the list's sum — and
// only that lane issues the two atomics.  Particles stored near each other
// (the particle array keeps the cell order of FluidSim2D::create) share faces,
// so a warp issues a few atomics per face instead of one per particle.
__device__ __forceinline__ void agg_add(int f, double val, double wt, double* a, double* w) {
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(0xffffffffu, f);
    const unsigned above = lane == 31 ? 0u : peers & (0xffffffffu << (lane + 1));
    int nxt = above ? __ffs(above) - 1 : -1;
#pragma unroll
    for (int d = 0; d < 5; d++) {
        const int src = nxt < 0 ? lane : nxt;
        const double v2 = __shfl_sync(0xffffffffu, val, src);
        const double w2 = __shfl_sync(0xffffffffu, wt, src);
        const int n2 = __shfl_sync(0xffffffffu, nxt, src);
        if (nxt >= 0) {
            val += v2;
            wt += w2;
            nxt = n2;
        }
    }
    if (f >= 0 && lane == __ffs(peers) - 1) {
        atomicAdd(a + f, val);
        atomicAdd(w + f, wt);
    }
}

// P2G, fast mode: bilinear splats summed per warp and face, then FP64 atomics
// (sums are not in particle order: not reproducible bit for bit).  Whole
// warps run the aggregation; lanes past the last particle add nothing.
__global__ void k_p2g_atomic(const double2* __restrict__ pos, const double2* __restrict__ vel, size_t np, double dx,
                             int NX, int NY, double* u, double* udiv, double* v, double* vdiv) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const bool live = e < np;
    double2 p = live ? pos[e] : make_double2(0.0, 0.0), w = live ? vel[e] : make_double2(0.0, 0.0);
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        agg_add(live ? bu.face(k, NX + 1) : -1, bu.contrib(k, w.x), bu.contrib(k, 1.0), u, udiv);
        agg_add(live ? bv.face(k, NX) : -1, bv.contrib(k, w.y), bv.contrib(k, 1.0), v, vdiv);
    }
}

__global__ void k_p2g_normalize(double* a, const double* __restrict__ div, uint32_t* mask, size_t n) {
    size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (f >= n) return;
    double s = a[f], w = div[f];
    if (w > 0) s /= w;
    a[f] = s;
    mask[f] = (s == 0.0) ? kUnknown : 0u;
}

// ---- G2P (src/FluidSim2D.cpp:552-568) ----

// linearExtract (include/Array2D.h:402-420) of a face grid, or of the
// difference of two face grids (uDiff = newMac.u - mac.u, rounded per face).
__device__ __forceinline__ double extract(const double* __restrict__ a, const double* __restrict__ b, double px,
                                          double py, int W, int H) {
    Bilinear bl(px, py, W, H);
    int f0 = bl.y1 * W + bl.x1, f1 = bl.y1 * W + bl.x2, f2 = bl.y2 * W + bl.x1, f3 = bl.y2 * W + bl.x2;
    double a0 = a[f0], a1 = a[f1], a2 = a[f2], a3 = a[f3];
    if (b != nullptr) {
        a0 = a0 - b[f0];
        a1 = a1 - b[f1];
        a2 = a2 - b[f2];
        a3 = a3 - b[f3];
    }
    double value = 0.0;
    value += a0 * (1 - bl.dxp) * (1 - bl.dyp);
    value += a1 * bl.dxp * (1 - bl.dyp);
    value += a2 * (1 - bl.dxp) * bl.dyp;
    value += a3 * bl.dxp * bl.dyp;
    return value;
}

__global__ void k_g2p(const double2* __restrict__ pos, double2* vel, size_t np, const double* __restrict__ nu,
                      const double* __restrict__ nv, const double* __restrict__ u, const double* __restrict__ v,
                      double dx, int NX, int NY, double alpha) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double ux, uy, vx, vy;
    upos(p, dx, ux, uy);
    vpos(p, dx, vx, vy);
    double picx = extract(nu, nullptr, ux, uy, NX + 1, NY);
    double picy = extract(nv, nullptr, vx, vy, NX, NY + 1);
    double2 w = vel[e];
    double flipx = w.x + extract(nu, u, ux, uy, NX + 1, NY);
    double flipy = w.y + extract(nv, v, vx, vy, NX, NY + 1);
    vel[e] = make_double2(alpha * picx + (1 - alpha) * flipx, alpha * picy + (1 - alpha) * flipy);
}

// ---- transposes of the particle transfers (fixed particle positions) ----

// Sum of the bilinear weights per face (linearDistribute's weight splat).
__global__ void k_p2g_weights(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY, double* wu,
                              double* wv) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        atomicAdd(wu + bu.face(k, NX + 1), bu.contrib(k, 1.0));
        atomicAdd(wv + bv.face(k, NX), bv.contrib(k, 1.0));
    }
}

// P2G^T after E^T: a particle's velocity adjoint gathers, over its corners
// whose face kept its splatted value (mask 0), weight * mu / (sum of weights).
__global__ void k_p2g_adjoint(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY,
                              const double* __restrict__ mu, const double* __restrict__ mv,
                              const double* __restrict__ wu, const double* __restrict__ wv,
                              const uint32_t* __restrict__ mask_u, const uint32_t* __restrict__ mask_v,
                              double2* velbar) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
    double gx = 0.0, gy = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int fu = bu.face(k, NX + 1), fv = bv.face(k, NX);
        if (mask_u[fu] == 0 && wu[fu] > 0) gx += bu.contrib(k, 1.0) * mu[fu] / wu[fu];
        if (mask_v[fv] == 0 && wv[fv] > 0) gy += bv.contrib(k, 1.0) * mv[fv] / wv[fv];
    }
    velbar[e] = make_double2(gx, gy);
}

// G2P^T: v_new = alpha pic + (1 - alpha)(v + flip delta), pic = G newMac,
// delta = G (newMac - mac), so newMac^bar += G^T vbar, mac^bar -= (1 - alpha)
// G^T vbar, v^bar = (1 - alpha) vbar.
__global__ void k_g2p_adjoint(const double2* __restrict__ pos, const double2* __restrict__ vbar, size_t np, double dx,
                              int NX, int NY, double alpha, double* nub, double* nvb, double* ub, double* vb,
                              double2* vinb) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e], g = vbar[e];
    double x, y;
    upos(p, dx, x, y);
    Bilinear bu(x, y, NX + 1, NY);
    vpos(p, dx, x, y);
    Bilinear bv(x, y, NX, NY + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int fu = bu.face(k, NX + 1), fv = bv.face(k, NX);
        const double au = bu.contrib(k, 1.0) * g.x, av = bv.contrib(k, 1.0) * g.y;
        atomicAdd(nub + fu, au);
        atomicAdd(ub + fu, -(1 - alpha) * au);
        atomicAdd(nvb + fv, av);
        atomicAdd(vb + fv, -(1 - alpha) * av);
    }
    vinb[e] = make_double2((1 - alpha) * g.x, (1 - alpha) * g.y);
}

// ---- extrapolation ----

// Column pass of the L1 distance transform: vertical distance to the nearest
// known face (mask 0) of the same column, kInf if none.  Written into d.
// Column pass: d(x, y) = distance along the column to the nearest known
// face (mask 0), kInf if the column has none: the reference's order-free
// BFS distance restricted to one column.  Block = 32 columns x 32 row
// segments; each thread finds the last and the first known face of its
// segment, the segments of a column exchange them through shared memory
// (the last known face above the segment, the first known face below it),
// and each thread writes min(y - above, below - y) for its rows.
constexpr int kDtSeg = 32;
__global__ void __launch_bounds__(32 * kDtSeg) k_dt_cols(const uint32_t* __restrict__ mask, int* d, int W, int H) {
    __shared__ int last_k[kDtSeg][32], first_k[kDtSeg][32];
    const int cx = threadIdx.x, sg = threadIdx.y;
    const int x = blockIdx.x * 32 + cx;
    const int rows = (H + kDtSeg - 1) / kDtSeg;
    const int y0 = sg * rows, y1 = min(H, y0 + rows);
    int last = -1, first = -1;
    if (x < W) {
        for (int y = y0; y < y1; y++) {
            if (mask[(size_t)y * W + x] == 0) {
                if (first < 0) first = y;
                last = y;
            }
        }
    }
    last_k[sg][cx] = last;
    first_k[sg][cx] = first;
    __syncthreads();
    if (x >= W) return;
    int above = -1;   // last known face before this segment
    for (int k = sg - 1; k >= 0 && above < 0; k--) above = last_k[k][cx];
    int below = -1;   // first known face after this segment
    for (int k = sg + 1; k < kDtSeg && below < 0; k++) below = first_k[k][cx];
    // forward: the last known face at or above y; backward: the first at or below
    int a = above;
    for (int y = y0; y < y1; y++) {
        const size_t c = (size_t)y * W + x;
        if (mask[c] == 0) a = y;
        d[c] = a >= 0 ? y - a : kInf;
    }
    int bb = below;
    for (int y = y1 - 1; y >= y0; y--) {
        const size_t c = (size_t)y * W + x;
        if (mask[c] == 0) bb = y;
        if (bb >= 0) d[c] = min(d[c], bb - y);
    }
}

// Row pass: D(x) = min_x' (col(x') + |x - x'|) via a block-wide prefix-min of
// col(x') - x' (forward) and suffix-min of col(x') + x' (backward).  Writes
// layers into mask (0 known, >= 1 unknown, kUnknown unreachable) and
// per-32x32-tile layer ranges of the unknown faces.
__global__ void __launch_bounds__(1024) k_dt_rows(const int* __restrict__ d, uint32_t* mask, int W, int H,
                                                  int2* tile_range, int tiles_x) {
    __shared__ int fwd_carry[32], bwd_carry[32];
    int y = blockIdx.x;
    int T = blockDim.x;
    int chunk = (W + T - 1) / T;
    int x0 = threadIdx.x * chunk, x1 = min(W, x0 + chunk);
    const int* row = d + (size_t)y * W;
    // local scans
    int fm = kInf * 2, bm = kInf * 2;
    for (int x = x0; x < x1; x++) fm = min(fm, row[x] - x);
    for (int x = x0; x < x1; x++) bm = min(bm, row[x] + x);
    // exclusive prefix-min over threads (fm) and suffix-min (bm)
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (T + 31) >> 5;
    int f_inc = fm, b_inc = bm;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, f_inc, o);
        if (lane >= o) f_inc = min(f_inc, t);
        int u = __shfl_down_sync(0xffffffffu, b_inc, o);
        if (lane + o < 32) b_inc = min(b_inc, u);
    }
    if (lane == 31) fwd_carry[wid] = f_inc;
    if (lane == 0) bwd_carry[wid] = b_inc;
    __syncthreads();
    if (wid == 0) {
        int fv = lane < nw ? fwd_carry[lane] : kInf * 2;
        int bv = lane < nw ? bwd_carry[lane] : kInf * 2;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, fv, o);
            if (lane >= o) fv = min(fv, t);
            int u = __shfl_down_sync(0xffffffffu, bv, o);
            if (lane + o < 32) bv = min(bv, u);
        }
        __syncwarp();
        if (lane < nw) {
            fwd_carry[lane] = fv;
            bwd_carry[lane] = bv;
        }
    }
    __syncthreads();
    int f_prev = __shfl_up_sync(0xffffffffu, f_inc, 1);
    if (lane == 0) f_prev = kInf * 2;
    if (wid > 0) f_prev = min(f_prev, fwd_carry[wid - 1]);
    int b_next = __shfl_down_sync(0xffffffffu, b_inc, 1);
    if (lane == 31) b_next = kInf * 2;
    if (wid + 1 < nw) b_next = min(b_next, bwd_carry[wid + 1]);
    // apply: forward running min from the left, backward from the right
    int run = f_prev;
    int tmin = kInf * 2, tmax = -1;
    int tx_cur = -1;
    for (int x = x0; x < x1; x++) {
        run = min(run, row[x] - x);
        mask[(size_t)y * W + x] = (uint32_t)(run + x);  // provisional forward value
    }
    run = b_next;
    for (int x = x1 - 1; x >= x0; x--) {
        run = min(run, row[x] + x);
        int L = min((int)mask[(size_t)y * W + x], run - x);
        uint32_t out = (L >= kInf) ? kUnknown : (uint32_t)L;
        mask[(size_t)y * W + x] = out;
        int tx = x / kTile;
        if (tx != tx_cur) {
            if (tx_cur >= 0 && tmax >= 0) {
                int2* tr = tile_range + (size_t)(y / kTile) * tiles_x + tx_cur;
                atomicMin(&tr->x, tmin);
                atomicMax(&tr->y, tmax);
            }
            tx_cur = tx;
            tmin = kInf * 2;
            tmax = -1;
        }
        if (out != 0 && out != kUnknown) {
            tmin = min(tmin, (int)out);
            tmax = max(tmax, (int)out);
        }
    }
    if (tx_cur >= 0 && tmax >= 0) {
        int2* tr = tile_range + (size_t)(y / kTile) * tiles_x + tx_cur;
        atomicMin(&tr->x, tmin);
        atomicMax(&tr->y, tmax);
    }
}

__global__ void k_tile_init(int2* tr, size_t n) {
    size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k < n) tr[k] = make_int2(kInf * 2, -1);
}

__global__ void k_tile_max(const int2* __restrict__ tr, size_t n, unsigned int* max_layer) {
    size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k < n && tr[k].y >= 0) atomicMax(max_layer, (unsigned int)tr[k].y);
}

// One extrapolation of up to two face grids: every band of kBand layers of
// every 32x32 tile in one launch.  The deepest layer of each grid
// (max_layer, written by k_tile_max) is read on the device, so the host
// neither waits for it nor launches per band.  Work items are (band, tile)
// pairs in band-major order, taken by the CTAs from an atomic counter; a
// tile's band needs the previous band of the tile and of its eight
// neighbours (the halo), whose items come earlier in the list and were taken
// earlier by running CTAs, so every wait makes progress whatever the grid
// size and whatever else runs on the GPU.  Only items of bands a tile works
// in wait or report (done[t] = 1 + the last working band finished).
struct ExtrapJob {
    double* a[2];
    const uint32_t* layer[2];
    int W[2], H[2];
    const int2* tile_range[2];
    int tiles_x[2], tiles_y[2];
    int ntiles[2];              // tiles of grid 0, of grid 1 (0: no grid 1)
    const unsigned int* max_layer;
    unsigned int* work;         // item counter (zero before the launch)
    int* done;                  // per tile: bands finished (zero before the launch)
    int* err;                   // bit 3 (8): a wait for a neighbour tile gave up
    unsigned int band_limit;    // deepest layer to fill
    long long spin;             // polls before a wait gives up
};

// Layers [lo, hi] of one 32x32 tile, recomputed in shared memory inside a
// halo of kBand cells.  Only region cells that can still reach the tile
// within the band are recomputed: a cell of layer l at L1 distance d from the
// tile feeds tile cells of layer >= l + d, so it is kept iff lo <= l <= hi and
// d <= hi - l.  Every kept cell's lower-layer neighbours are either kept too
// (their distance is at most d + 1 and their layer l - 1) or have a layer
// below lo and are final in global memory; all of them lie inside the region
// (d <= kBand - 1).  Kept cells are bucketed by layer, so each layer step
// visits only its own front.  Layers are held relative to the band in one
// byte: 0 below lo, 1 + (l - lo) inside, kBand + 1 above hi or unreachable.
// Face values are read through L2 (other CTAs wrote them in earlier bands).
//
// The mean divides by the neighbour count as the reference does; for counts
// 1, 2 and 4 the quotient equals the product with the exact reciprocal (both
// are the correctly rounded value of the same real number), so only a count
// of 3 needs a division.
__global__ void __launch_bounds__(256) k_extrap_bands(const ExtrapJob job) {
    __shared__ double val[kReg * kReg];
    __shared__ unsigned char rel[kReg * kReg];
    __shared__ unsigned short list[kReg * kReg];
    __shared__ int cnt[kBand + 1], cur[kBand];
    __shared__ unsigned int item_sh;
    __shared__ int failed_sh;
    const int ng = job.ntiles[1] > 0 ? 2 : 1;
    unsigned int depth[2] = {0u, 0u};
    unsigned int deepest = 0u;
    for (int g = 0; g < ng; g++) {
        depth[g] = min(job.max_layer[g], job.band_limit);
        deepest = max(deepest, depth[g]);
    }
    const unsigned int total = (unsigned int)(job.ntiles[0] + job.ntiles[1]);
    const unsigned int nbands = (deepest + kBand - 1) / kBand;
    const unsigned long long nitems = (unsigned long long)nbands * total;
    // L1 distance from region cell (rx, ry) to the output tile
    auto tile_dist = [](int rx, int ry) {
        int dx = rx < kBand ? kBand - rx : (rx >= kBand + kTile ? rx - (kBand + kTile - 1) : 0);
        int dy = ry < kBand ? kBand - ry : (ry >= kBand + kTile ? ry - (kBand + kTile - 1) : 0);
        return dx + dy;
    };
    if (threadIdx.x == 0) failed_sh = 0;
    for (;;) {
        __syncthreads();   // the previous item's shared arrays are no longer read
        if (threadIdx.x == 0) item_sh = atomicAdd(job.work, 1u);
        __syncthreads();
        const unsigned long long item = item_sh;
        if (item >= nitems || failed_sh) break;
        const int band = (int)(item / total);
        const int tile = (int)(item % total);
        const int g = tile < job.ntiles[0] ? 0 : 1;
        const int t = tile - (g ? job.ntiles[0] : 0);
        const int tx = t % job.tiles_x[g], ty = t / job.tiles_x[g];
        const unsigned int lo_u = 1u + (unsigned int)band * kBand;
        const unsigned int hi_u = min(lo_u + kBand - 1, depth[g]);
        const int2 tr = job.tile_range[g][t];
        const bool work = lo_u <= depth[g] && tr.y >= (int)lo_u && tr.x <= (int)hi_u;
        // A tile works only in the bands its layer range [tr.x, tr.y] (up to
        // the depth) spans; an item without work neither waits nor reports.
        // A working item needs, of itself and each neighbour (the halo), every
        // working band before its own: it waits until that tile's done count
        // covers min(band - 1, its last working band), when that is one of its
        // working bands (thread k < 9 watches tile (tx + k % 3 - 1, ty + k / 3 - 1)).
        if (!work) continue;
        if (band > 0 && threadIdx.x < 9) {
            const int nx = tx + (int)(threadIdx.x % 3) - 1, ny = ty + (int)(threadIdx.x / 3) - 1;
            if (nx >= 0 && ny >= 0 && nx < job.tiles_x[g] && ny < job.tiles_y[g]) {
                const int n = ny * job.tiles_x[g] + nx;
                const int2 trn = job.tile_range[g][n];
                const int top = min(trn.y, (int)depth[g]);   // the neighbour's last layer to fill
                if (trn.y >= 1 && trn.x <= top) {
                    const int b_lo = (trn.x - 1) / kBand, b_hi = (top - 1) / kBand;
                    const int need = min(band - 1, b_hi);
                    if (need >= b_lo) {
                        const int* d = job.done + (g ? job.ntiles[0] : 0) + n;
                        long long polls = 0;
                        while (ld_acquire_int(d) < need + 1) {
                            if (++polls > job.spin) {
                                atomicOr(job.err, 8);
                                failed_sh = 1;
                                break;
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        if (failed_sh) break;   // results are invalid; this CTA takes no further item
        if (work) {
            const int lo = (int)lo_u, hi = (int)hi_u;
            const int W = job.W[g], H = job.H[g];
            double* a = job.a[g];
            const uint32_t* __restrict__ layer = job.layer[g];
            const int ox = tx * kTile - kBand, oy = ty * kTile - kBand;
            if (threadIdx.x <= kBand) cnt[threadIdx.x] = 0;
            if (threadIdx.x < kBand) cur[threadIdx.x] = 0;
            __syncthreads();
            for (int k = threadIdx.x; k < kReg * kReg; k += blockDim.x) {
                int rx = k % kReg, ry = k / kReg;
                int gx = ox + rx, gy = oy + ry;
                uint32_t l = kUnknown;
                double v = 0.0;
                if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                    size_t c = (size_t)gy * W + gx;
                    l = layer[c];
                    v = __ldcg(a + c);
                }
                const int r = l < (uint32_t)lo ? 0 : (l <= (uint32_t)hi ? 1 + (int)(l - lo) : kBand + 1);
                rel[k] = (unsigned char)r;
                val[k] = v;
                if (r >= 1 && r <= kBand && tile_dist(rx, ry) <= hi - lo + 1 - r) atomicAdd(&cnt[r], 1);
            }
            __syncthreads();
            if (threadIdx.x == 0)
                for (int b = 1; b <= kBand; b++) cnt[b] += cnt[b - 1];   // cnt[b] = first slot of layer lo + b
            __syncthreads();
            for (int k = threadIdx.x; k < kReg * kReg; k += blockDim.x) {
                const int r = rel[k];
                if (r >= 1 && r <= kBand && tile_dist(k % kReg, k / kReg) <= hi - lo + 1 - r)
                    list[cnt[r - 1] + atomicAdd(&cur[r - 1], 1)] = (unsigned short)k;
            }
            for (int L = lo; L <= hi; L++) {
                __syncthreads();
                const int b = L - lo;
                const int rl = b + 1;   // relative layer of L
                for (int i = cnt[b] + threadIdx.x; i < cnt[b + 1]; i += blockDim.x) {
                    const int k = list[i];
                    double sum = 0.0;
                    int count = 0;
                    // neighbours in the reference's order: x-1, x+1, y-1, y+1
                    if (rel[k - 1] < rl) { sum += val[k - 1]; count++; }
                    if (rel[k + 1] < rl) { sum += val[k + 1]; count++; }
                    if (rel[k - kReg] < rl) { sum += val[k - kReg]; count++; }
                    if (rel[k + kReg] < rl) { sum += val[k + kReg]; count++; }
                    double r;
                    if (count == 3) r = sum / 3.0;
                    else r = sum * (count == 1 ? 1.0 : (count == 2 ? 0.5 : (count == 4 ? 0.25 : 0.0)));
                    val[k] = r;
                }
            }
            __syncthreads();
            for (int k = threadIdx.x; k < kTile * kTile; k += blockDim.x) {
                int rx = kBand + k % kTile, ry = kBand + k / kTile;
                int gx = ox + rx, gy = oy + ry;
                if (gx >= W || gy >= H) continue;
                const int r = rel[ry * kReg + rx];
                if (r >= 1 && r <= kBand) a[(size_t)gy * W + gx] = val[ry * kReg + rx];
            }
        }
        __syncthreads();   // every store of this item is issued
        if (threadIdx.x == 0) {
            __threadfence();
            st_release_int(job.done + tile, band + 1);
        }
    }
}

// ---- exclusive scan of uint32 (counts -> offsets), n+1 outputs ----
constexpr int kScanBlock = 1024;

__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* out, size_t n, uint32_t* block_sums) {
    __shared__ uint32_t sh[32];
    size_t base = (size_t)blockIdx.x * kScanBlock * 4;
    uint32_t v[4];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        size_t idx = base + threadIdx.x * 4 + k;
        v[k] = idx < n ? in[idx] : 0u;
        local += v[k];
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = sh[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        sh[lane] = s;
    }
    __syncthreads();
    uint32_t excl = inc - local + (wid > 0 ? sh[wid - 1] : 0u);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        size_t idx = base + threadIdx.x * 4 + k;
        if (idx < n) out[idx] = excl;
        excl += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) block_sums[blockIdx.x] = sh[31];
}

__global__ void k_scan_sums(uint32_t* block_sums, int nb, uint32_t* total_out) {
    // single block: sequential over chunks, parallel within
    __shared__ uint32_t sh[32];
    uint32_t carry = 0;
    for (int base = 0; base < nb; base += blockDim.x) {
        int k = base + threadIdx.x;
        uint32_t v = k < nb ? block_sums[k] : 0u;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        __syncthreads();
        if (lane == 31) sh[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            uint32_t s = sh[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            sh[lane] = s;
        }
        __syncthreads();
        uint32_t excl = inc - v + (wid > 0 ? sh[wid - 1] : 0u) + carry;
        if (k < nb) block_sums[k] = excl;
        carry += sh[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_add(uint32_t* out, size_t n, const uint32_t* __restrict__ block_sums) {
    size_t base = (size_t)blockIdx.x * kScanBlock * 4;
    uint32_t add = block_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        size_t idx = base + threadIdx.x * 4 + k;
        if (idx < n) out[idx] += add;
    }
}

// ---- particle reseeding (fs2d_reseed; the reference lists it as a TODO, README.md:13-18) ----

// The cell a particle is counted in: (int)(x/dx), (int)(y/dx) clamped into the grid.
__device__ __forceinline__ size_t rs_cell(double2 p, double dx, int NX, int NY) {
    const int i = iclamp((int)(p.x / dx), 0, NX - 1), j = iclamp((int)(p.y / dx), 0, NY - 1);
    return (size_t)j * NX + i;
}

// splitmix64's finaliser; the jitter of new particle m of cell c takes 53
// bits of it for each axis, scaled into [0, 1)
__device__ __forceinline__ unsigned long long rs_mix(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_rs_count(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY, uint32_t* cnt,
                           uint32_t* keep) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    atomicAdd(&cnt[rs_cell(pos[e], dx, NX, NY)], 1u);
    keep[e] = 1u;
}

// Buckets of particle indices per cell (in arbitrary order within a bucket).
__global__ void k_rs_fill(const double2* __restrict__ pos, size_t np, double dx, int NX, int NY,
                          const uint32_t* __restrict__ start, uint32_t* fill, uint32_t* bucket) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    const size_t c = rs_cell(pos[e], dx, NX, NY);
    bucket[start[c] + atomicAdd(&fill[c], 1u)] = (uint32_t)e;
}

// Per cell: where it holds more than maxPC particles, its bucket is sorted
// by particle index and all but the first maxPC are dropped; a FLUID cell
// with fewer than minPC asks for the difference.
__global__ void k_rs_cells(const uint8_t* __restrict__ cell, const uint32_t* __restrict__ cnt,
                           const uint32_t* __restrict__ start, uint32_t* bucket, size_t N, int minPC, int maxPC,
                           uint32_t* keep, uint32_t* spawn) {
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const uint32_t k = cnt[c];
    if (maxPC > 0 && k > (uint32_t)maxPC) {
        uint32_t* b = bucket + start[c];
        for (uint32_t m = 1; m < k; m++) {   // insertion sort: buckets hold a few particles
            const uint32_t key = b[m];
            uint32_t q = m;
            while (q > 0 && b[q - 1] > key) {
                b[q] = b[q - 1];
                q--;
            }
            b[q] = key;
        }
        for (uint32_t m = (uint32_t)maxPC; m < k; m++) keep[b[m]] = 0u;
    }
    spawn[c] = (cell[c] == kFluid && k < (uint32_t)minPC) ? (uint32_t)minPC - k : 0u;
}

// Survivors, in particle order, to the start of the new arrays (keep holds
// the exclusive scan of the keep flags, np + 1 entries).
__global__ void k_rs_compact(const double2* __restrict__ pos, const double2* __restrict__ vel, size_t np,
                             const uint32_t* __restrict__ keep, double2* npos, double2* nvel) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np || keep[e + 1] == keep[e]) return;
    npos[keep[e]] = pos[e];
    nvel[keep[e]] = vel[e];
}

// New particles of each cell after the survivors (spawn holds the exclusive
// scan of the per-cell requests, N + 1 entries), moving with the bilinear
// grid velocity at their position.
__global__ void k_rs_spawn(const uint32_t* __restrict__ spawn, size_t N, int NX, int NY, double dx, size_t n_keep,
                           unsigned seed, const double* __restrict__ u, const double* __restrict__ v, double2* npos,
                           double2* nvel) {
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const uint32_t first = spawn[c], n = spawn[c + 1] - first;
    const int i = (int)(c % NX), j = (int)(c / NX);
    for (uint32_t m = 0; m < n; m++) {
        const unsigned long long key =
            (unsigned long long)seed * 0x9E3779B97F4A7C15ull + (unsigned long long)c * 0x100000001B3ull + m;
        const double jx = (double)(rs_mix(key) >> 11) * 0x1.0p-53;
        const double jy = (double)(rs_mix(key ^ 0xD6E8FEB86659FD93ull) >> 11) * 0x1.0p-53;
        const double px = ((double)i + jx) * dx, py = ((double)j + jy) * dx;
        const size_t d = n_keep + first + m;
        npos[d] = make_double2(px, py);
        nvel[d] = make_double2(extract(u, nullptr, px / dx, py / dx - 0.5, NX + 1, NY),
                               extract(v, nullptr, px / dx - 0.5, py / dx, NX, NY + 1));
    }
}

}  // namespace

// In-place exclusive scan of data[0..n); data[n] receives the total.
int exclusive_scan_u32(Sim* s, uint32_t* data, size_t n) {
    size_t nb = (n + kScanBlock * 4 - 1) / (kScanBlock * 4);
    if (nb + 1 > s->scan_tmp_n) {
        set_error("scan: %zu elements exceed scratch", n);
        return FS2D_ERR_INVALID;
    }
    FS2D_LAUNCH(s, k_scan_blocks, (unsigned)nb, kScanBlock, 0, data, data, n, s->scan_tmp);
    FS2D_LAUNCH(s, k_scan_sums, 1, 1024, 0, s->scan_tmp, (int)nb, data + n);
    FS2D_LAUNCH(s, k_scan_add, (unsigned)nb, kScanBlock, 0, data, n, s->scan_tmp);
    return 0;
}

int reseed_plan(Sim* s, const ReseedScratch& x, int min_per_cell, int max_per_cell, size_t* n_keep, size_t* n_add) {
    const size_t N = s->N, np = s->np;
    const int T = 256;
    FS2D_CUDA(cudaMemsetAsync(x.cnt, 0, (N + 1) * sizeof(uint32_t), s->stream));
    FS2D_CUDA(cudaMemsetAsync(x.fill, 0, (N + 1) * sizeof(uint32_t), s->stream));
    FS2D_CUDA(cudaMemsetAsync(x.keep, 0, (np + 1) * sizeof(uint32_t), s->stream));
    if (np) FS2D_LAUNCH(s, k_rs_count, blocks_for(np, T), T, 0, s->pos, np, s->dx, s->NX, s->NY, x.cnt, x.keep);
    FS2D_CUDA(cudaMemcpyAsync(x.start, x.cnt, (N + 1) * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s->stream));
    int rc = exclusive_scan_u32(s, x.start, N);
    if (rc) return rc;
    if (np)
        FS2D_LAUNCH(s, k_rs_fill, blocks_for(np, T), T, 0, s->pos, np, s->dx, s->NX, s->NY, x.start, x.fill,
                    x.bucket);
    FS2D_LAUNCH(s, k_rs_cells, blocks_for(N, T), T, 0, s->cell, x.cnt, x.start, x.bucket, N, min_per_cell,
                max_per_cell, x.keep, x.spawn);
    if (np && (rc = exclusive_scan_u32(s, x.keep, np))) return rc;   // np == 0: keep[0] = 0 from the memset
    if ((rc = exclusive_scan_u32(s, x.spawn, N))) return rc;
    uint32_t totals[2] = {0, 0};
    FS2D_CUDA(cudaMemcpyAsync(&totals[0], x.keep + np, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(&totals[1], x.spawn + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    *n_keep = totals[0];
    *n_add = totals[1];
    return 0;
}

int reseed_write(Sim* s, const ReseedScratch& x, unsigned seed, double2* npos, double2* nvel) {
    const size_t N = s->N, np = s->np;
    const int T = 256;
    size_t n_keep = 0;
    {
        uint32_t t = 0;
        FS2D_CUDA(cudaMemcpyAsync(&t, x.keep + np, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
        FS2D_CUDA(cudaStreamSynchronize(s->stream));
        n_keep = t;
    }
    if (np) FS2D_LAUNCH(s, k_rs_compact, blocks_for(np, T), T, 0, s->pos, s->vel, np, x.keep, npos, nvel);
    FS2D_LAUNCH(s, k_rs_spawn, blocks_for(N, T), T, 0, x.spawn, N, s->NX, s->NY, s->dx, n_keep, seed, s->u, s->v,
                npos, nvel);
    return 0;
}

// Launch inside the extrapolation core: counted and timed when a handle is given.
#define XLAUNCH(kernel, grid, block, ...)                                           \
    do {                                                                          \
        long long _kt = -1;                                                       \
        if (s) {                                                                  \
            s->launches++;                                                        \
            _kt = ktimer_begin(s, #kernel);                                       \
        }                                                                         \
        kernel<<<(grid), (block), 0, stream>>>(__VA_ARGS__);                      \
        if (s) ktimer_end(s, _kt);                                                \
        int _rc = check_cuda(cudaGetLastError(), #kernel);                        \
        if (_rc) return _rc;                                                      \
    } while (0)


size_t extrap_tiles(int W, int H) { return (size_t)((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile); }

// Array2D::extrapolate on one or two face grids (grid 1 may be absent,
// a[1] == nullptr).  Scratch: dist[g] holds W*H ints per grid, tile_range
// extrap_tiles(W,H) entries per grid (grid 1's after grid 0's), max_layer 16
// words (0-1 the deepest layers, 8 the band kernel's item counter, 12 the
// error word when there is no handle).  Queues work on `stream` only: the
// depth is read on the device by the band kernel, one launch.
int extrapolate_core(Sim* s, cudaStream_t stream, const ExtrapScratch& x, double* const a[2], uint32_t* const m[2],
                     const int W[2], const int H[2], int band) {
    int ng = a[1] ? 2 : 1;
    FS2D_CUDA(cudaMemsetAsync(x.max_layer, 0, 16 * sizeof(unsigned int), stream));
    int tiles_x[2] = {0, 0}, tiles_y[2] = {0, 0};
    size_t tile_off[2] = {0, 0};
    for (int gi = 0; gi < ng; gi++) {
        tiles_x[gi] = (W[gi] + kTile - 1) / kTile;
        tiles_y[gi] = (H[gi] + kTile - 1) / kTile;
        if (gi == 1) tile_off[1] = extrap_tiles(W[0], H[0]);
        size_t nt = (size_t)tiles_x[gi] * tiles_y[gi];
        int2* tr = x.tile_range + tile_off[gi];
        XLAUNCH(k_tile_init, blocks_for(nt, 256), 256, tr, nt);
        XLAUNCH(k_dt_cols, (W[gi] + 31) / 32, dim3(32, kDtSeg), m[gi], x.dist[gi], W[gi], H[gi]);
        XLAUNCH(k_dt_rows, H[gi], 1024, x.dist[gi], m[gi], W[gi], H[gi], tr, tiles_x[gi]);
        XLAUNCH(k_tile_max, blocks_for(nt, 256), 256, tr, nt, x.max_layer + gi);
    }
    ExtrapJob job{};
    for (int gi = 0; gi < ng; gi++) {
        job.a[gi] = a[gi];
        job.layer[gi] = m[gi];
        job.W[gi] = W[gi];
        job.H[gi] = H[gi];
        job.tile_range[gi] = x.tile_range + tile_off[gi];
        job.tiles_x[gi] = tiles_x[gi];
        job.tiles_y[gi] = tiles_y[gi];
        job.ntiles[gi] = tiles_x[gi] * tiles_y[gi];
    }
    const int total = job.ntiles[0] + job.ntiles[1];
    // the per-tile band counters live in grid 0's distance map, which the
    // layers no longer need (every tile count is below W * H)
    if ((size_t)total > (size_t)W[0] * H[0]) {
        set_error("extrapolation: %d tiles do not fit the scratch", total);
        return FS2D_ERR_INVALID;
    }
    job.max_layer = x.max_layer;
    job.work = x.max_layer + 8;
    job.done = x.dist[0];
    job.err = s ? s->err : reinterpret_cast<int*>(x.max_layer + 12);
    job.band_limit = band > 0 ? (unsigned int)band : (1u << 28);
    job.spin = kWaveSpinLimit;
    FS2D_CUDA(cudaMemsetAsync(job.done, 0, (size_t)total * sizeof(int), stream));
    // CTAs: as many as the SMs hold at once, at most one per tile (items
    // beyond what runs at once are taken by whichever CTA is free)
    int dev = 0;
    FS2D_CUDA(cudaGetDevice(&dev));
    static std::atomic<int> per_dev[64];
    int occ = (dev >= 0 && dev < 64) ? per_dev[dev].load() : 0;
    if (occ <= 0) {
        int sms = 1, per = 0;
        FS2D_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FS2D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_extrap_bands, 256, 0));
        occ = std::max(1, per * sms);
        if (dev >= 0 && dev < 64) per_dev[dev].store(occ);
    }
    XLAUNCH(k_extrap_bands, std::max(1, std::min(occ, total)), 256, job);
    return 0;
}
#undef XLAUNCH

// Array2D::extrapolate on one or two face grids of the handle (b may be null).
int extrapolate(Sim* s, double* a, uint32_t* mask_a, int Wa, int Ha, double* b, uint32_t* mask_b, int Wb, int Hb) {
    // scratch: the P2G weight arrays are free whenever extrapolation runs
    ExtrapScratch x{{(int*)s->udiv, (int*)s->vdiv}, s->tile_range, s->max_layer};
    double* const aa[2] = {a, b};
    uint32_t* const mm[2] = {mask_a, mask_b};
    const int W[2] = {Wa, Wb}, H[2] = {Ha, Hb};
    return extrapolate_core(s, s->stream, x, aa, mm, W, H, s->opt.extrapolate_band);
}

int p2g(Sim* s) {
    const int NX = s->NX, NY = s->NY, T = 256;
    const size_t NU = s->NU, NV = s->NV;
    if (s->opt.p2g_mode == FS2D_P2G_ATOMIC) {
        FS2D_CUDA(cudaMemsetAsync(s->u, 0, NU * sizeof(double), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->v, 0, NV * sizeof(double), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->udiv, 0, NU * sizeof(double), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->vdiv, 0, NV * sizeof(double), s->stream));
        if (s->np > 0)
            FS2D_LAUNCH(s, k_p2g_atomic, blocks_for(s->np, T), T, 0, s->pos, s->vel, s->np, s->dx, NX, NY, s->u, s->udiv,
                        s->v, s->vdiv);
        FS2D_LAUNCH(s, k_p2g_normalize, blocks_for(NU, T), T, 0, s->u, s->udiv, s->mask_u, NU);
        FS2D_LAUNCH(s, k_p2g_normalize, blocks_for(NV, T), T, 0, s->v, s->vdiv, s->mask_v, NV);
    } else {
        FS2D_CUDA(cudaMemsetAsync(s->cnt_u, 0, (NU + 1) * sizeof(uint32_t), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->cnt_v, 0, (NV + 1) * sizeof(uint32_t), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->fill_u, 0, NU * sizeof(uint32_t), s->stream));
        FS2D_CUDA(cudaMemsetAsync(s->fill_v, 0, NV * sizeof(uint32_t), s->stream));
        if (s->np > 0)
            FS2D_LAUNCH(s, k_p2g_count, blocks_for(s->np, T), T, 0, s->pos, s->np, s->dx, NX, NY, s->cnt_u, s->cnt_v);
        int rc = exclusive_scan_u32(s, s->cnt_u, NU);
        if (rc) return rc;
        rc = exclusive_scan_u32(s, s->cnt_v, NV);
        if (rc) return rc;
        if (s->np > 0)
            FS2D_LAUNCH(s, k_p2g_fill, blocks_for(s->np, T), T, 0, s->pos, s->np, s->dx, NX, NY, s->cnt_u, s->cnt_v,
                        s->fill_u, s->fill_v, s->ent_u, s->ent_v);
        FS2D_LAUNCH(s, k_p2g_sum<0>, blocks_for(NU, T), T, 0, s->pos, s->vel, s->dx, NX, NY, NX + 1, NY, s->cnt_u,
                    s->ent_u, NU, s->u, s->mask_u);
        FS2D_LAUNCH(s, k_p2g_sum<1>, blocks_for(NV, T), T, 0, s->pos, s->vel, s->dx, NX, NY, NX, NY + 1, s->cnt_v,
                    s->ent_v, NV, s->v, s->mask_v);
    }
    return extrapolate(s, s->u, s->mask_u, NX + 1, NY, s->v, s->mask_v, NX, NY + 1);
}

int extrap_adjoint(Sim* s, double* mu, const uint32_t* layer, int W, int H, uint32_t lim);

// P2G^T at the current particle positions and the masks of the last P2G:
// (ubar, vbar) face adjoints (device, overwritten by E^T) -> velbar.
int p2g_adjoint(Sim* s, double* ubar, double* vbar, double* wu, double* wv, double2* velbar) {
    const int NX = s->NX, NY = s->NY, T = 256;
    const uint32_t lim = s->opt.extrapolate_band > 0 ? (uint32_t)s->opt.extrapolate_band : 0xFFFFFFFEu;
    int rc = extrap_adjoint(s, ubar, s->mask_u, NX + 1, NY, lim);
    if (!rc) rc = extrap_adjoint(s, vbar, s->mask_v, NX, NY + 1, lim);
    if (rc) return rc;
    FS2D_CUDA(cudaMemsetAsync(wu, 0, s->NU * sizeof(double), s->stream));
    FS2D_CUDA(cudaMemsetAsync(wv, 0, s->NV * sizeof(double), s->stream));
    if (s->np == 0) return 0;
    FS2D_LAUNCH(s, k_p2g_weights, blocks_for(s->np, T), T, 0, s->pos, s->np, s->dx, NX, NY, wu, wv);
    FS2D_LAUNCH(s, k_p2g_adjoint, blocks_for(s->np, T), T, 0, s->pos, s->np, s->dx, NX, NY, ubar, vbar, wu, wv,
                s->mask_u, s->mask_v, velbar);
    return 0;
}

// G2P^T at the current particle positions: velbar -> (newMac, mac, vel) adjoints (zeroed first).
int g2p_adjoint(Sim* s, const double2* velbar, double* nub, double* nvb, double* ub, double* vb, double2* vinb) {
    const int T = 256;
    FS2D_CUDA(cudaMemsetAsync(nub, 0, s->NU * sizeof(double), s->stream));
    FS2D_CUDA(cudaMemsetAsync(nvb, 0, s->NV * sizeof(double), s->stream));
    FS2D_CUDA(cudaMemsetAsync(ub, 0, s->NU * sizeof(double), s->stream));
    FS2D_CUDA(cudaMemsetAsync(vb, 0, s->NV * sizeof(double), s->stream));
    if (s->np == 0) return 0;
    FS2D_LAUNCH(s, k_g2p_adjoint, blocks_for(s->np, T), T, 0, s->pos, velbar, s->np, s->dx, s->NX, s->NY, s->alpha,
                nub, nvb, ub, vb, vinb);
    return 0;
}

int g2p(Sim* s) {
    const int T = 256;
    if (s->np > 0)
        FS2D_LAUNCH(s, k_g2p, blocks_for(s->np, T), T, 0, s->pos, s->vel, s->np, s->nu, s->nv, s->u, s->v, s->dx, s->NX,
                    s->NY, s->alpha);
    FS2D_CUDA(cudaMemcpyAsync(s->u, s->nu, s->NU * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(s->v, s->nv, s->NV * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    return 0;
}

}  // namespace fs2d

using namespace fs2d;

// Status of a handle-less extrapolation from its error word (bit 3: a wait
// between the bands gave up).
static int extrap_wait_status(int werr) {
    if (werr & 8) {
        set_error("extrapolation: a wait between bands timed out");
        return FS2D_ERR_TIMEOUT;
    }
    return FS2D_OK;
}

// Array2D::extrapolate (include/Array2D.h:552-591) on caller-owned device
// buffers; scratch is allocated with cudaMalloc for the duration of the call.
extern "C" int fs2d_extrapolate(double* values, uint32_t* mask, int width, int height, int band, void* stream) {
    if (!values || !mask || width < 1 || height < 1) {
        set_error("fs2d_extrapolate: invalid arguments");
        return FS2D_ERR_INVALID;
    }
    const size_t n = (size_t)width * height;
    const size_t dist_bytes = (n * sizeof(int) + 255) / 256 * 256;
    const size_t tile_bytes = (extrap_tiles(width, height) * sizeof(int2) + 255) / 256 * 256;
    char* buf = nullptr;
    int rc = check_cuda(cudaMalloc((void**)&buf, dist_bytes + tile_bytes + 256), "cudaMalloc");
    if (rc) return rc;
    ExtrapScratch x{{(int*)buf, nullptr}, (int2*)(buf + dist_bytes), (unsigned int*)(buf + dist_bytes + tile_bytes)};
    double* const aa[2] = {values, nullptr};
    uint32_t* const mm[2] = {mask, nullptr};
    const int W[2] = {width, 0}, H[2] = {height, 0};
    cudaStream_t st = (cudaStream_t)stream;
    rc = extrapolate_core(nullptr, st, x, aa, mm, W, H, band);
    cudaError_t e = cudaStreamSynchronize(st);
    int werr = 0;
    if (!rc && e == cudaSuccess) e = cudaMemcpy(&werr, x.max_layer + 12, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (rc) return rc;
    if ((rc = check_cuda(e, "fs2d_extrapolate"))) return rc;
    return extrap_wait_status(werr);
}

// ---------------------------------------------------------------------------
// fs2d_extrapolate_noalloc: the same extrapolation for callers that cannot
// allocate device memory (for example code running under a memory pool or
// allocator it does not own, or a plugin that may only use the buffers it is
// handed).  Its scratch lives in this file-scope device array, sized for at
// most kNoAllocMaxFaces faces with each side at most kNoAllocMaxSide; every
// GPU that loads the library holds these bytes until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocMaxFaces = (size_t)1 << 21;  // 2,097,152 faces
constexpr int kNoAllocMaxSide = 8192;
constexpr size_t kNoAllocMaxTiles = kNoAllocMaxFaces / 1024 + 2 * (kNoAllocMaxSide / 32) + 1;
constexpr size_t kNoAllocDistBytes = kNoAllocMaxFaces * sizeof(int);
constexpr size_t kNoAllocTileBytes = (kNoAllocMaxTiles * sizeof(int2) + 255) / 256 * 256;
constexpr size_t kNoAllocBytes = kNoAllocDistBytes + kNoAllocTileBytes + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch, looked up once per device (with that
// device current) on the first call made on it.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

int noalloc_scratch(void** out) {
    int dev = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("fs2d_extrapolate_noalloc: device %d out of range", dev);
        return FS2D_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
        if (rc) return rc;
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return 0;
}

}  // namespace

// Same contract as fs2d_extrapolate, without allocating: see include/fs2d.h.
extern "C" int fs2d_extrapolate_noalloc(double* values, uint32_t* mask, int width, int height, int band,
                                        void* stream) {
    if (!values || !mask || width < 1 || height < 1) {
        set_error("fs2d_extrapolate_noalloc: invalid arguments");
        return FS2D_ERR_INVALID;
    }
    if (width > kNoAllocMaxSide || height > kNoAllocMaxSide || (size_t)width * height > kNoAllocMaxFaces) {
        set_error("fs2d_extrapolate_noalloc: %d x %d faces exceed the static scratch (at most %zu faces, "
                  "each side at most %d); use fs2d_extrapolate",
                  width, height, kNoAllocMaxFaces, kNoAllocMaxSide);
        return FS2D_ERR_INVALID;
    }
    void* base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    char* buf = (char*)base;
    // every part of the scratch is (re)initialised by the kernels of this call:
    // the distance map and tile ranges are written before they are read and
    // the layer counters are cleared by extrapolate_core
    ExtrapScratch x{{(int*)buf, nullptr}, (int2*)(buf + kNoAllocDistBytes),
                    (unsigned int*)(buf + kNoAllocDistBytes + kNoAllocTileBytes)};
    double* const aa[2] = {values, nullptr};
    uint32_t* const mm[2] = {mask, nullptr};
    const int W[2] = {width, 0}, H[2] = {height, 0};
    cudaStream_t st = (cudaStream_t)stream;
    rc = extrapolate_core(nullptr, st, x, aa, mm, W, H, band);
    cudaError_t e = cudaStreamSynchronize(st);
    int werr = 0;
    if (!rc && e == cudaSuccess) e = cudaMemcpy(&werr, x.max_layer + 12, sizeof(int), cudaMemcpyDeviceToHost);
    if (rc) return rc;
    if ((rc = check_cuda(e, "fs2d_extrapolate_noalloc"))) return rc;
    return extrap_wait_status(werr);
}
