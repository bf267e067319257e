// eik_sweep.cuh — the Eikonal sweeps of LevelSet::redistance
// (src/FluidSim2D.cpp:844-901) as a TMA-staged wavefront that skips cells
// whose value cannot change.
//
// One sweep visits cells in the reference's loop order and sets
// phi(i,j) = eik(phi(i,j), phi(i - sx, j), phi(i, j - sy)) from the upwind
// neighbours, which the sweep has already visited.  The update of a cell
// depends only on its own pre-sweep value and those two neighbours, so if
// neither neighbour changed during the sweep the result equals the update
// with pre-sweep values, which a parallel pass (k_eik_check) evaluated for
// every cell beforehand.  A cell is therefore recomputed only when that pass
// marked it (mask = 1) or an upwind neighbour changed; every other cell keeps
// its value without any arithmetic, and a step where no lane of the warp has
// such a cell issues no FP64 instruction.  The update itself is the
// reference's expression in FP64 with its comparisons done on the bit
// patterns of the non-negative operands (|a|, |b|, d, -phi), which order like
// the values when no operand is NaN; a NaN operand takes the plain FP64
// expression.
//
// Layout: phi is pitched (row pitch P), the mask is a byte per cell in the
// same pitch.  One 64-thread CTA per strip of 32 rows: warp 0 computes (lane
// l owns row l of the strip and works on column s - l at step s), warp 1
// moves data (tile stores, the strip's top row to the next strip, the row
// below in).
#pragma once

#include <cuda.h>
#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kEkCols = 32;
constexpr int kEkRows = 32;
constexpr int kEkSlots = 8;
constexpr int kEkAhead = 4;
constexpr int kEkCH = 16;
constexpr int kEkBndChunks = 8;
constexpr int kEkTopRing = 256;
constexpr unsigned kEkTileBytes = kEkCols * kEkRows * 8;
constexpr unsigned kEkMaskBytes = kEkCols * kEkRows;
constexpr size_t kEkSmem = (size_t)kEkSlots * (kEkTileBytes + kEkMaskBytes) + kEkBndChunks * kEkCH * 16 +
                           kEkTopRing * 16 + 16 * 4 + kEkSlots * 8;

struct EkMaps {
    CUtensorMap ld;       // phi, box 32 x 32 (load and store of full strips)
    CUtensorMap st_tail;  // phi, box 32 x (NY % 32) (store of the partial strip of a downward sweep)
    CUtensorMap mask;     // mask bytes, box 32 x 32
};

// One Eikonal update (src/FluidSim2D.cpp:848-857) with a = upwind x
// neighbour, b = upwind y neighbour; c2 = 2*dx*dx as the reference groups it.
__device__ __forceinline__ double eik_ref(double own, double a, double b, double dx, double c2) {
    if (own >= 0) return own;
    double fa = fabs(a), fb = fabs(b);
    double phi0 = (fb < fa) ? fb : fa;
    double phi1 = (fa < fb) ? fb : fa;
    double d = phi0 + dx;
    if (d > phi1) d = 0.5 * (phi0 + phi1 + sqrt(c2 - (phi1 - phi0) * (phi1 - phi0)));
    return (d < -own) ? -d : own;
}

__device__ __noinline__ double eik_ref_call(double own, double a, double b, double dx, double c2) {
    return eik_ref(own, a, b, dx, c2);
}

// The same update with bit-pattern comparisons (identical results).
__device__ __forceinline__ double eik_fast(double own, double a, double b, double dx, double c2) {
    const unsigned long long kSign = 0x8000000000000000ull, kInf = 0x7FF0000000000000ull;
    const unsigned long long ob = (unsigned long long)__double_as_longlong(own);
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a) & ~kSign;
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b) & ~kSign;
    if ((ob & ~kSign) > kInf || ab > kInf || bb > kInf) return eik_ref_call(own, a, b, dx, c2);
    if (!(ob >> 63) || ob == kSign) return own;   // own >= 0 (+0, -0, positive)
    const unsigned long long p0 = bb < ab ? bb : ab;   // min(|a|, |b|) as (y < x) ? y : x
    const unsigned long long p1 = ab < bb ? bb : ab;   // max(|a|, |b|) as (x < y) ? y : x
    const double phi0 = __longlong_as_double((long long)p0);
    const double phi1 = __longlong_as_double((long long)p1);
    double d = phi0 + dx;
    if ((unsigned long long)__double_as_longlong(d) > p1) {
        d = 0.5 * (phi0 + phi1 + sqrt(c2 - (phi1 - phi0) * (phi1 - phi0)));
    }
    // d >= 0 and -own > 0
    return ((unsigned long long)__double_as_longlong(d) < (ob & ~kSign)) ? -d : own;
}

__device__ __forceinline__ bool same_bits(double x, double y) {
    return __double_as_longlong(x) == __double_as_longlong(y);
}

struct EkArgs {
    double2* hb;          // strip hand-off rows: [strip][sweep column] = (value, changed)
    unsigned long long* progress;
    unsigned long long base;
    int* err;
    const int* skip;
    int NX, NY, P;
    int i_lo, i_hi, j_lo, j_hi;   // cells the sweep updates
    double dx, c2;
};

template <int SX, int SY>
__global__ void __launch_bounds__(64) eik_sweep_kernel(const __grid_constant__ EkMaps maps, const EkArgs a) {
    if (a.skip != nullptr && *a.skip) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    double* tiles = reinterpret_cast<double*>(smem_raw);
    unsigned char* mtiles = smem_raw + (size_t)kEkSlots * kEkTileBytes;
    double2* bnd = reinterpret_cast<double2*>(mtiles + (size_t)kEkSlots * kEkMaskBytes);
    double2* top = bnd + kEkBndChunks * kEkCH;
    volatile int* ctr = reinterpret_cast<volatile int*>(top + kEkTopRing);
    volatile int* bnd_ready = ctr + 0;
    volatile int* bnd_used = ctr + 1;
    volatile int* top_ready = ctr + 2;
    volatile int* top_done = ctr + 3;
    volatile int* quit = ctr + 4;
    volatile int* tiles_done = ctr + 5;
    volatile int* tiles_freed = ctr + 6;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 16);

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int strip = blockIdx.x;
    const int NX = a.NX, NY = a.NY, P = a.P;
    const int nstrips = (NY + kEkRows - 1) / kEkRows;
    const int nt = P / kEkCols;
    const int nchunks = P / kEkCH;
    const bool has_next = strip + 1 < nstrips;
    const bool below_in_grid = strip > 0;
    const int y0 = SY > 0 ? kEkRows * strip : NY - kEkRows - kEkRows * strip;   // memory row of box row 0

    if (threadIdx.x == 0) {
        for (int k = 0; k < kEkSlots; k++) mbar_init(bars + k, 1);
        fence_mbar_init();
        *bnd_ready = below_in_grid ? 0 : nchunks;
        *bnd_used = 0;
        *top_ready = 0;
        *top_done = 0;
        *quit = 0;
        *tiles_done = 0;
        *tiles_freed = 0;
    }
    if (!below_in_grid) {
        for (int k = threadIdx.x; k < kEkBndChunks * kEkCH; k += blockDim.x) bnd[k] = make_double2(0.0, 0.0);
    }
    __syncthreads();

    if (warp == 1) {
        // ---------------- I/O warp ----------------
        const unsigned long long* gprev = below_in_grid ? a.progress + (strip - 1) : nullptr;
        int hbk = below_in_grid ? 0 : nchunks;
        int tc = 0;
        const int tend = has_next ? P : 0;
        int ts = 0;
        unsigned long long gavail = 0;
        long long idle = 0;
        while (hbk < nchunks || tc < tend || ts < nt) {
            bool moved = false;
            if (ts < nt && *tiles_done > ts) {
                if (lane == 0) {
                    const double* src = tiles + (size_t)(ts % kEkSlots) * (kEkCols * kEkRows);
                    const int x = SX > 0 ? ts * kEkCols : P - (ts + 1) * kEkCols;
                    if (y0 >= 0) {
                        tma_store_2d(&maps.ld, x, y0, src);
                    } else {
                        const int tail = NY - kEkRows * strip;
                        tma_store_2d(&maps.st_tail, x, 0, src + (kEkRows - tail) * kEkCols);
                    }
                    bulk_commit();
                    bulk_wait_read<0>();
                    *tiles_freed = ts + 1;
                }
                __syncwarp();
                ts++;
                moved = true;
            }
            if (hbk < nchunks && hbk < *bnd_used + kEkBndChunks - 1) {
                const unsigned long long need = a.base + (unsigned long long)min((hbk + 1) * kEkCH, P);
                if (gavail < need) {
                    unsigned long long v = 0;
                    if (lane == 0) v = ld_acquire(gprev);
                    gavail = __shfl_sync(0xffffffffu, v, 0);
                }
                if (gavail >= need) {
                    if (lane < kEkCH)
                        bnd[(hbk % kEkBndChunks) * kEkCH + lane] =
                            __ldcg(a.hb + (size_t)(strip - 1) * P + hbk * kEkCH + lane);
                    __threadfence_block();
                    __syncwarp();
                    hbk++;
                    if (lane == 0) *bnd_ready = hbk;
                    moved = true;
                }
            }
            if (tc < tend) {
                const int tr = *top_ready;
                if (tr > tc) {
                    __threadfence_block();
                    for (int c = tc + lane; c < tr; c += 32) a.hb[(size_t)strip * P + c] = top[c % kEkTopRing];
                    __threadfence();
                    __syncwarp();
                    tc = tr;
                    if (lane == 0) {
                        st_release(a.progress + strip, a.base + (unsigned long long)tc);
                        *top_done = tc;
                    }
                    moved = true;
                }
            }
            if (moved) {
                idle = 0;
            } else if (++idle > 16 * kWaveSpinLimit || *quit || ((idle & 1023) == 0 && *(volatile int*)a.err)) {
                if (lane == 0) atomicOr(a.err, 1);
                break;
            }
        }
        if (lane == 0) bulk_wait_all();
        __syncwarp();
        return;
    }

    // ---------------- compute warp ----------------
    const bool rowvalid = kEkRows * strip + lane < NY;
    const int j = SY > 0 ? kEkRows * strip + lane : NY - 1 - kEkRows * strip - lane;
    const bool jupd = rowvalid && j >= a.j_lo && j <= a.j_hi;
    const int brow = SY > 0 ? lane : kEkRows - 1 - lane;    // box row of the lane's row
    auto tile_x = [&](int t) { return SX > 0 ? t * kEkCols : P - (t + 1) * kEkCols; };
    auto bc_of = [&](int c) { return SX > 0 ? (c & 31) : 31 - (c & 31); };
    auto issue = [&](int t) {
        if (lane == 0 && t < nt) {
            unsigned long long* bar = bars + (t % kEkSlots);
            mbar_expect_tx(bar, kEkTileBytes + kEkMaskBytes);
            tma_load_2d(tiles + (size_t)(t % kEkSlots) * (kEkCols * kEkRows), &maps.ld, tile_x(t), y0, bar);
            tma_load_2d(mtiles + (size_t)(t % kEkSlots) * kEkMaskBytes, &maps.mask, tile_x(t), y0, bar);
        }
    };
    bool failed = false;
    auto wait_tile = [&](int t) {
        unsigned long long* bar = bars + (t % kEkSlots);
        const unsigned parity = (unsigned)((t / kEkSlots) & 1);
        long long polls = 0;
        while (!mbar_try_wait(bar, parity)) {
            if (++polls > kWaveSpinLimit) {
                failed = true;
                atomicOr(a.err, 1);
                break;
            }
        }
    };
    auto spin_ge = [&](volatile int* flag, int need) {
        if (failed) return;
        long long polls = 0;
        while (*flag < need) {
            if (++polls > 16 * kWaveSpinLimit) {
                failed = true;
                atomicOr(a.err, 1);
                *quit = 1;
                return;
            }
        }
    };

    for (int t = 0; t < kEkAhead; t++) issue(t);

    double o_v = 0.0;     // output of the previous step (the left value)
    bool o_c = false;     // ... and whether the sweep changed it

    auto tile_steps = [&](int t, auto check_tag) {
        constexpr bool check = decltype(check_tag)::value;
#pragma unroll 4
        for (int u = 0; u < kEkCols; u++) {
            const int s = t * kEkCols + u;
            const int c = s - lane;
            if ((s % kEkCH) == 0 && s < P) {   // lane 0 enters a new chunk of the row below
                const int h = s / kEkCH;
                if (*bnd_ready <= h) spin_ge(bnd_ready, h + 1);
                __threadfence_block();
                if (lane == 0) *bnd_used = h;
                __syncwarp();
            }
            double b_v = __shfl_up_sync(0xffffffffu, o_v, 1);
            bool b_c = __shfl_up_sync(0xffffffffu, (int)o_c, 1) != 0;
            if (lane == 0) {
                const double2 e = bnd[((s / kEkCH) % kEkBndChunks) * kEkCH + (s % kEkCH)];
                b_v = e.x;
                b_c = e.y != 0.0;
            }
            const bool cin = !check || (c >= 0 && c < P);
            const int i = SX > 0 ? c : P - 1 - c;
            double own = 0.0;
            double* cell = nullptr;
            bool act = false;
            if (rowvalid && cin && i < NX) {
                const int slot = (c >> 5) % kEkSlots;   // c >= 0 here
                const int in_tile = brow * kEkCols + bc_of(c);
                cell = tiles + (size_t)slot * (kEkCols * kEkRows) + in_tile;
                own = *cell;
                const bool upd = jupd && i >= a.i_lo && i <= a.i_hi;
                act = upd && (o_c || b_c || mtiles[(size_t)slot * kEkMaskBytes + in_tile] != 0);
            }
            double out = own;
            bool chg = false;
            if (__any_sync(0xffffffffu, act)) {
                if (act) {
                    out = eik_fast(own, o_v, b_v, a.dx, a.c2);
                    chg = !same_bits(out, own);
                    if (chg) *cell = out;
                }
            }
            o_v = out;
            o_c = chg;
            if (has_next && lane == 31 && cin) {
                top[c % kEkTopRing] = make_double2(out, chg ? 1.0 : 0.0);
                if (((c + 1) % 8) == 0 || c == P - 1) {
                    __threadfence_block();
                    *top_ready = c + 1;
                }
            }
        }
    };

    const int nsteps = P + 31;
    for (int t = 0; t * kEkCols < nsteps; t++) {
        if (t < nt) wait_tile(t);
        if (has_next && t * kEkCols - 31 - *top_done > kEkTopRing / 2)
            spin_ge(top_done, t * kEkCols - 31 - kEkTopRing / 2);
        __syncwarp();
        if (t == 0 || t >= nt)
            tile_steps(t, BoolTag<true>{});
        else
            tile_steps(t, BoolTag<false>{});
        if (t >= 1 && t - 1 < nt) {
            fence_async_smem();
            __syncwarp();
            if (lane == 0) *tiles_done = t;
        }
        const int nx = t + kEkAhead;
        if (nx < nt) {
            if (nx >= kEkSlots && *tiles_freed < nx - kEkSlots + 1) spin_ge(tiles_freed, nx - kEkSlots + 1);
            __syncwarp();
            issue(nx);
        }
    }
    __syncwarp();
    if (lane == 0) *tiles_done = nt;
    (void)failed;
}

}  // namespace fs2d
