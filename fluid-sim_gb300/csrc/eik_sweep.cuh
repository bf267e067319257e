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
// below in).  Strips are launched in clusters; a boundary column travels as
// two 64-bit words (low and high half of the value), each tagged with its
// column (the high word's tag also carries the changed flag), so a column is
// valid once both tags match and no flag or fence orders the words.  Inside
// a cluster the I/O warp writes them into the next strip's shared ring;
// across clusters they go through global memory with a released progress
// counter.
#pragma once

#include <cuda.h>
#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kEkCols = 32;
constexpr int kEkRows = 32;
constexpr int kEkSlots = 8;
constexpr int kEkAhead = 4;
// Columns per arrival check / flow-control chunk.  A strip waits for whole
// chunks of the row below, so the chunk adds to the strip-to-strip lag; an
// Eikonal step is long (dependent FP64 updates), so a check every 4 columns
// costs little (measured at 1024^2: chunks of 16, 8, 4, 2 columns gave
// 14.8, 13.6, 13.2, 13.5 ms of sweeps per frame).
constexpr int kEkCH = 4;
constexpr int kEkRingChunks = 256 / kEkCH;
constexpr int kEkRing = kEkRingChunks * kEkCH;   // boundary ring, columns
constexpr int kEkTopRing = 256;
constexpr unsigned kEkTileBytes = kEkCols * kEkRows * 8;
constexpr unsigned kEkMaskBytes = kEkCols * kEkRows;
constexpr size_t kEkSmem = (size_t)kEkSlots * (kEkTileBytes + kEkMaskBytes) + (size_t)(kEkRing + kEkTopRing) * 16 +
                           16 * 4 + kEkSlots * 8;

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

// The same update with bit-pattern comparisons (identical results).
__device__ __forceinline__ double eik_fast(double own, double a, double b, double dx, double c2) {
    const unsigned long long kSign = 0x8000000000000000ull, kInf = 0x7FF0000000000000ull;
    const unsigned long long ob = (unsigned long long)__double_as_longlong(own);
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a) & ~kSign;
    const unsigned long long bb = (unsigned long long)__double_as_longlong(b) & ~kSign;
    if ((ob & ~kSign) > kInf || ab > kInf || bb > kInf) return eik_ref(own, a, b, dx, c2);
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
    const double* phi;    // the pitched level set the sweep updates (its unchanged columns are read directly)
    const uint2* rng;     // per strip: the check's column range (null: every strip marches every column)
    unsigned long long* progress;
    unsigned long long base;
    int* err;
    const int* skip;
    int NX, NY, P;
    int i_lo, i_hi, j_lo, j_hi;   // cells the sweep updates
    double dx, c2;
};

// Tagged boundary words of column c: value halves, tags 2c and 2c + changed.
__device__ __forceinline__ unsigned long long ek_w0(int c, double v) {
    return ((unsigned long long)(2u * (unsigned)c) << 32) | (unsigned)__double_as_longlong(v);
}
__device__ __forceinline__ unsigned long long ek_w1(int c, double v, bool chg) {
    return ((unsigned long long)(2u * (unsigned)c + (chg ? 1u : 0u)) << 32) |
           (unsigned)((unsigned long long)__double_as_longlong(v) >> 32);
}
__device__ __forceinline__ bool ek_w0_is(unsigned long long w, int c) { return (unsigned)(w >> 32) == 2u * (unsigned)c; }
__device__ __forceinline__ bool ek_w1_is(unsigned long long w, int c) { return (unsigned)(w >> 33) == (unsigned)c; }
__device__ __forceinline__ double ek_value(unsigned long long w0, unsigned long long w1) {
    return __longlong_as_double((long long)(((w1 & 0xffffffffull) << 32) | (w0 & 0xffffffffull)));
}
__device__ __forceinline__ bool ek_changed(unsigned long long w1) { return ((w1 >> 32) & 1ull) != 0; }

// One scene of a launch over several scenes: its tensor maps and arguments
// (progress, base, err and skip come from the launch's WaveWork; the
// update region i_lo .. j_hi from the direction).
struct EkScene {   // aligned as CUtensorMap
    EkMaps maps;
    EkArgs a;
};

// SEVERAL = false: one scene, CTA b = strip b, in clusters.  SEVERAL = true:
// persistent CTAs over w's work items (see WaveWork), no clusters.
template <int SX, int SY, bool SEVERAL>
__global__ void __launch_bounds__(64) eik_sweep_kernel(const __grid_constant__ EkMaps maps1, const EkArgs a1,
                                                       const WaveWork w) {
    if (!SEVERAL && a1.skip != nullptr && *a1.skip) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    double* tiles = reinterpret_cast<double*>(smem_raw);
    unsigned char* mtiles = smem_raw + (size_t)kEkSlots * kEkTileBytes;
    // row below the strip: 2 tagged words per column
    volatile unsigned long long* bnd =
        reinterpret_cast<volatile unsigned long long*>(mtiles + (size_t)kEkSlots * kEkMaskBytes);
    volatile unsigned long long* top = bnd + 2 * kEkRing;   // the strip's top row, 2 words per column
    volatile int* ctr = reinterpret_cast<volatile int*>(const_cast<unsigned long long*>(top + 2 * kEkTopRing));
    volatile int* bnd_used = ctr + 0;     // chunks of the row below the compute warp has finished
    volatile int* top_done = ctr + 1;     // top-row columns forwarded by the I/O warp
    volatile int* quit = ctr + 2;
    volatile int* tiles_done = ctr + 3;
    volatile int* tiles_freed = ctr + 4;
    volatile int* cur_item = ctr + 5;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 16);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // every CTA of the cluster (one scene) or of the block (several scenes)
    auto sync_all = [&]() {
        if (SEVERAL) __syncthreads();
        else cluster_sync_all();
    };

  // One strip of one scene (the whole grid of a launch per scene, or one
  // work item of a launch over several scenes).
  auto run_strip = [&](const EkMaps& maps, const EkArgs& a, const int strip) {
    const int NX = a.NX, NY = a.NY, P = a.P;
    const int nstrips = (NY + kEkRows - 1) / kEkRows;
    const bool has_next = strip + 1 < nstrips;
    // this strip hands its top row to the next one (unless the test hook holds it back)
    const bool publishes = has_next && !wave_held(a.err, kWaveKindEik, strip);
    const long long spin = wave_spin(a.err);
    const bool below_in_grid = strip > 0;
    const bool active = strip < nstrips;                       // the grid is rounded up to whole clusters
    const unsigned crank = SEVERAL ? 0u : cluster_ctarank(), csize = SEVERAL ? 1u : cluster_nctarank();
    const bool prev_local = below_in_grid && crank > 0;        // the previous strip fills this ring
    const bool next_local = publishes && crank + 1 < csize;    // this strip fills the next strip's ring
    const int y0 = SY > 0 ? kEkRows * strip : NY - kEkRows - kEkRows * strip;   // memory row of box row 0
    // Columns (sweep order) this strip can change: a cell changes only if the
    // check marked it or an upwind neighbour changed, changes travel right and
    // up, and cells >= 0 never change, so the strip's changes lie between the
    // first marked column of this and every earlier strip and its own last
    // negative column.  The strip marches whole tiles from the one holding
    // the column before that first column (whose unchanged value is the left
    // neighbour of the first cell that can change).  Its other columns keep
    // their values: the successor gets them straight from memory.
    int A = 0, Bm = P - 1;
    if (a.rng != nullptr && strip < nstrips) {   // (CTAs past the last strip exist only to round up clusters)
        unsigned c0 = 0xffffffffu;
        for (int k = 0; k <= strip; k++) c0 = min(c0, a.rng[k].x);
        const unsigned lr = a.rng[strip].y;
        const int last = lr == 0xffffffffu ? -1 : P - 1 - (int)lr;
        const int first = c0 == 0xffffffffu ? P : (int)c0;
        if (first <= last) {
            A = (max(first - 1, 0) / kEkCols) * kEkCols;
            Bm = last;
        } else {
            A = P;   // nothing to march
            Bm = P - 1;
        }
    }
    const bool march = A <= Bm;
    const int tA = A / kEkCols;                      // first marched tile
    const int tB = march ? Bm / kEkCols : tA - 1;    // last marched tile
    const int jtop = SY > 0 ? y0 + kEkRows - 1 : y0; // memory row of the strip's top row

    if (threadIdx.x == 0) {
        for (int k = 0; k < kEkSlots; k++) mbar_init(bars + k, 1);
        fence_mbar_init();
        *bnd_used = A / kEkCH;
        *top_done = 0;
        *quit = 0;
        *tiles_done = tA;
        *tiles_freed = tA;
    }
    for (int k = threadIdx.x; k < 2 * kEkRing; k += blockDim.x) bnd[k] = ~0ull;      // no column matches
    for (int k = threadIdx.x; k < 2 * kEkTopRing; k += blockDim.x) top[k] = ~0ull;
    sync_all();   // every ring and counter of the cluster is initialised

    if (warp == 1 && active) {
        // ---------------- I/O warp ----------------
        const unsigned long long* gprev = below_in_grid ? a.progress + (strip - 1) : nullptr;
        const int hb_end = march ? Bm + 1 : 0;            // the row below is needed on the marched columns
        int hb = (below_in_grid && !prev_local && march) ? A : hb_end;   // next column of the row below to fetch
        int tc = 0;                                        // top-row columns forwarded
        const int tend = publishes ? P : 0;
        int rused = 0;                                     // last seen chunk position of the consumer
        const unsigned r_bnd = next_local ? mapa_shared((const void*)bnd, crank + 1) : 0u;
        const unsigned r_used = next_local ? mapa_shared((const void*)bnd_used, crank + 1) : 0u;
        int ts = tA;
        unsigned long long gavail = 0;
        long long idle = 0;
        while (hb < hb_end || tc < tend || ts <= tB) {
            bool moved = false;
            // row below from global memory (the previous strip is in another cluster)
            const int hb_lim = (*bnd_used + kEkRingChunks - 2) * kEkCH;   // slots consumed two chunks ago
            if (hb < hb_end && hb < hb_lim) {
                const int n = min(min(32, hb_end - hb), hb_lim - hb);
                const unsigned long long need = a.base + (unsigned long long)(hb + n);
                if (gavail < need) {
                    unsigned long long v = 0;
                    if (lane == 0) v = ld_acquire(gprev);
                    gavail = __shfl_sync(0xffffffffu, v, 0);
                }
                const int avail = (int)min((unsigned long long)n, gavail > a.base + hb ? gavail - a.base - hb : 0ull);
                if (avail > 0) {
                    __syncwarp();   // lane 0's acquire orders the reads below
                    const int c = hb + lane;
                    if (lane < avail) {
                        const double2 e = __ldcg(a.hb + (size_t)(strip - 1) * P + c);
                        bnd[2 * (c % kEkRing)] = ek_w0(c, e.x);
                        bnd[2 * (c % kEkRing) + 1] = ek_w1(c, e.x, e.y != 0.0);
                    }
                    __syncwarp();
                    hb += avail;
                    moved = true;
                }
            }
            // top row out: to the next strip's ring (same cluster) or to global
            // memory, every complete run of up to 128 columns at once
            for (int rep = 0; rep < 4 && tc < tend; rep++) {
                const int c = tc + lane;
                unsigned long long w0 = 0ull, w1 = 0ull;
                if (c < P) {
                    if (c < A || c > Bm) {   // not marched: the unchanged value in memory
                        const double v = a.phi[(size_t)jtop * P + (SX > 0 ? c : P - 1 - c)];
                        w0 = ek_w0(c, v);
                        w1 = ek_w1(c, v, false);
                    } else {
                        w0 = top[2 * (c % kEkTopRing)];
                        w1 = top[2 * (c % kEkTopRing) + 1];
                    }
                }
                const bool ok = c >= P || (ek_w0_is(w0, c) && ek_w1_is(w1, c));
                const unsigned bad = __ballot_sync(0xffffffffu, !ok);
                int n = bad ? __ffs(bad) - 1 : 32;
                n = min(n, P - tc);
                if (n > 0 && next_local) {
                    if (tc + n > (rused + kEkRingChunks - 2) * kEkCH) {
                        int v = 0;
                        if (lane == 0) v = ld_volatile_cluster_remote(r_used);
                        rused = __shfl_sync(0xffffffffu, v, 0);
                    }
                    n = min(n, (rused + kEkRingChunks - 2) * kEkCH - tc);
                }
                if (n > 0) {
                    if (next_local) {
                        if (lane < n) {
                            const unsigned slot = 16u * (unsigned)(c % kEkRing);
                            st_cluster_u64(r_bnd + slot, w0);
                            st_cluster_u64(r_bnd + slot + 8u, w1);
                        }
                        __syncwarp();
                    } else {
                        if (lane < n)
                            a.hb[(size_t)strip * P + c] = make_double2(ek_value(w0, w1), ek_changed(w1) ? 1.0 : 0.0);
                        __threadfence();
                        __syncwarp();
                        if (lane == 0) st_release(a.progress + strip, a.base + (unsigned long long)(tc + n));
                    }
                    tc += n;
                    if (lane == 0) *top_done = tc;
                    moved = true;
                }
                if (n < 32) break;
            }
            if (ts <= tB && *tiles_done > ts) {
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
                    // no wait for this store's own read: once every store but the
                    // newest has read its tile, tiles < ts are free (the compute
                    // warp reuses a slot kEkSlots tiles later)
                    bulk_wait_read<1>();
                    *tiles_freed = ts;
                }
                __syncwarp();
                ts++;
                moved = true;
            }
            if (moved) {
                idle = 0;
            } else if (++idle > 16 * spin || *quit || ((idle & 1023) == 0 && wave_failed(a.err))) {
                if (lane == 0) {
                    atomicOr(a.err, kWaitStrip | (kWaveKindEik << 4));
                    *quit = 1;
                }
                break;
            }
        }
        if (lane == 0) bulk_wait_all();
        __syncwarp();
    } else if (warp == 0 && active) {
        // ---------------- compute warp ----------------
        const bool rowvalid = kEkRows * strip + lane < NY;
        const int j = SY > 0 ? kEkRows * strip + lane : NY - 1 - kEkRows * strip - lane;
        const bool jupd = rowvalid && j >= a.j_lo && j <= a.j_hi;
        const int brow = SY > 0 ? lane : kEkRows - 1 - lane;    // box row of the lane's row
        auto tile_x = [&](int t) { return SX > 0 ? t * kEkCols : P - (t + 1) * kEkCols; };
        auto bc_of = [&](int c) { return SX > 0 ? (c & 31) : 31 - (c & 31); };
        auto issue = [&](int t) {
            if (lane == 0 && t <= tB) {
                unsigned long long* bar = bars + (t % kEkSlots);
                mbar_expect_tx(bar, kEkTileBytes + kEkMaskBytes);
                tma_load_2d(tiles + (size_t)(t % kEkSlots) * (kEkCols * kEkRows), &maps.ld, tile_x(t), y0, bar);
                tma_load_2d(mtiles + (size_t)(t % kEkSlots) * kEkMaskBytes, &maps.mask, tile_x(t), y0, bar);
            }
        };
        bool failed = false;
        auto wait_tile = [&](int t) {
            unsigned long long* bar = bars + (t % kEkSlots);
            const unsigned parity = (unsigned)(((t - tA) / kEkSlots) & 1);   // slot phases count from tile tA
            long long polls = 0;
            while (!mbar_try_wait(bar, parity)) {
                if (++polls > kWaveSpinLimit) {
                    failed = true;
                    atomicOr(a.err, kWaitTile | (kWaveKindEik << 4));
                    *quit = 1;   // a copy may still be in flight: this CTA takes no further strip
                    break;
                }
            }
        };
        auto spin_ge = [&](volatile int* flag, int need) {
            if (failed) return;
            long long polls = 0;
            while (*flag < need) {
                if (++polls > 16 * spin) {
                    failed = true;
                    atomicOr(a.err, kWaitWarp | (kWaveKindEik << 4));
                    *quit = 1;
                    return;
                }
            }
        };
        // plain views of the rings for the per-step accesses (tags validate them)
        const unsigned long long* bnd_p = const_cast<const unsigned long long*>(bnd);
        unsigned long long* top_p = const_cast<unsigned long long*>(top);

        for (int t = tA; t < tA + kEkAhead; t++) issue(t);

        double o_v = 0.0;     // output of the previous step (the left value)
        bool o_c = false;     // ... and whether the sweep changed it
        unsigned long long bw0 = 0ull, bw1 = 0ull;   // row-below words of lane 0's column

        auto tile_steps = [&](int t, auto check_tag) {
            constexpr bool check = decltype(check_tag)::value;
#pragma unroll 4
            for (int u = 0; u < kEkCols; u++) {
                const int s = t * kEkCols + u;
                const int c = s - lane;
                if (below_in_grid && (u % kEkCH) == 0 && s >= A && s <= Bm) {
                    // lane 0 enters a chunk of the row below: every word of it
                    // must have arrived (one word per lane, one vote)
                    const int cc = s + (lane & (kEkCH - 1));
                    const int wi = 2 * (cc % kEkRing) + (lane >> 4);
                    bool ok = cc > Bm || ((lane >> 4) ? ek_w1_is(bnd_p[wi], cc) : ek_w0_is(bnd_p[wi], cc));
                    if (!__all_sync(0xffffffffu, ok)) {
                        // the whole warp polls in step until every word is there (lanes
                        // leaving a polling loop one by one would leave the warp diverged
                        // for the steps after it)
                        long long polls = 0;
                        while (!failed) {
                            const unsigned long long w = bnd[wi];
                            ok = cc > Bm || ((lane >> 4) ? ek_w1_is(w, cc) : ek_w0_is(w, cc));
                            if (__all_sync(0xffffffffu, ok)) break;
                            const bool give_up = ++polls > 16 * spin || ((polls & 1023) == 0 && wave_failed(a.err));
                            if (__any_sync(0xffffffffu, give_up)) {
                                failed = true;
                                if (lane == 0) {
                                    atomicOr(a.err, kWaitStrip | (kWaveKindEik << 4));
                                    *quit = 1;
                                }
                            }
                        }
                    }
                    __syncwarp();   // lane 0 reads the words its neighbours validated
                    if (lane == 0) *bnd_used = s / kEkCH;
                }
                if (below_in_grid && (!check || (s >= A && s <= Bm))) {
                    bw0 = bnd_p[2 * (s % kEkRing)];
                    bw1 = bnd_p[2 * (s % kEkRing) + 1];
                }
                double b_v = __shfl_up_sync(0xffffffffu, o_v, 1);
                bool b_c = __shfl_up_sync(0xffffffffu, (int)o_c, 1) != 0;
                if (lane == 0) {
                    b_v = below_in_grid ? ek_value(bw0, bw1) : 0.0;
                    b_c = below_in_grid && ek_changed(bw1);
                }
                const bool cin = !check || (c >= A && c <= Bm);
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
                if (publishes && lane == 31 && cin) {
                    top_p[2 * (c % kEkTopRing)] = ek_w0(c, out);
                    top_p[2 * (c % kEkTopRing) + 1] = ek_w1(c, out, chg);
                }
            }
        };

        const int tEnd = march ? (Bm + 31) / kEkCols : tA - 1;   // the last lane ends 31 columns behind
        for (int t = tA; t <= tEnd; t++) {
            if (t <= tB) wait_tile(t);
            if (publishes && t * kEkCols - 31 - *top_done > kEkTopRing / 2)
                spin_ge(top_done, t * kEkCols - 31 - kEkTopRing / 2);
            __syncwarp();
            if (t == tA || t >= tB)
                tile_steps(t, BoolTag<true>{});
            else
                tile_steps(t, BoolTag<false>{});
            if (t >= tA + 1 && t - 1 <= tB) {
                fence_async_smem();
                __syncwarp();
                if (lane == 0) *tiles_done = t;
            }
            const int nx = t + kEkAhead;
            if (nx <= tB) {
                if (nx - tA >= kEkSlots && *tiles_freed < nx - kEkSlots + 1) spin_ge(tiles_freed, nx - kEkSlots + 1);
                __syncwarp();
                issue(nx);
            }
        }
        __syncwarp();
        if (lane == 0) {
            *tiles_done = tB + 1;
            if (below_in_grid) *bnd_used = P / kEkCH + kEkRingChunks;
        }
        (void)failed;
    }
    sync_all();   // no CTA leaves while a neighbour may still touch its shared memory
  };

    if (!SEVERAL) {
        run_strip(maps1, a1, blockIdx.x);
        return;
    }
    const EkScene* scenes = static_cast<const EkScene*>(w.scenes);
    if (threadIdx.x == 0) *quit = 0;
    bool used = false;   // the ring barriers hold an earlier strip's phases
    for (;;) {
        __syncthreads();   // both warps are done with the previous item
        if (*quit) break;  // a wait of this CTA gave up: its rings and barriers stay as they are
        if (threadIdx.x == 0) *cur_item = atomicAdd(&w.work[0], 1);
        __syncthreads();
        const int it = *cur_item;
        if (it >= w.nitems) break;
        const WaveItem item = w.items[it];
        if (w.skip[item.scene]) continue;   // no cell of that scene would change in this sweep
        const EkScene* sc = scenes + item.scene;
        EkArgs a = sc->a;
        a.progress = w.progress + (item.pidx - item.strip);
        a.rng = w.rng != nullptr ? w.rng + (item.pidx - item.strip) : nullptr;
        a.base = w.base;
        a.err = w.err;
        a.skip = nullptr;
        if (used && threadIdx.x == 0)   // run_strip initialises them again (same thread, in order)
            for (int k = 0; k < kEkSlots; k++) mbar_inval(bars + k);
        used = true;
        a.i_lo = SX > 0 ? 1 : 0;
        a.i_hi = SX > 0 ? a.NX - 1 : a.NX - 2;
        a.j_lo = SY > 0 ? 1 : 0;
        a.j_hi = SY > 0 ? a.NY - 1 : a.NY - 2;
        run_strip(sc->maps, a, item.strip);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&w.work[1], 1) == (int)gridDim.x - 1) {   // the last CTA resets the counters
            w.work[0] = 0;
            w.work[1] = 0;
            __threadfence();
        }
    }
}

}  // namespace fs2d
