// mic32_tma.cuh — FP32 MIC(0) triangular solves as a TMA-staged wavefront
// over column strips.
//
// The forward and backward substitutions of applyPreconditioner
// (src/FluidSim2D.cpp:397-421) are recurrences over the grid in the
// reference's loop order: cell (i, j) needs its two upwind neighbours
// (i -+ 1, j) and (i, j -+ 1) of the same sweep.  This kernel keeps that
// dependency order and lays the work out as follows:
//   * one warp per CTA owns a strip of 128 columns; lane l owns the four
//     adjacent columns 4l .. 4l+3 (in sweep order) and at step s works on
//     row r = s - l, so the warp is a diagonal front.  Within a lane the
//     four cells of a row are computed left to right in the same step; the
//     cell left of the lane's first column arrives from lane l-1 by shuffle
//     (lane l-1 computed that row one step earlier), the row below stays in
//     the lane's registers.  The four operands of a lane lie side by side in
//     memory, so each operand array costs one 128-bit shared-memory load per
//     step and the result one 128-bit store;
//   * operand tiles of 128 columns x 32 rows come into shared memory by the
//     Tensor Memory Accelerator (cp.async.bulk.tensor, completion on an
//     mbarrier), into a ring of four tiles per operand array; results
//     overwrite operand 0 and each finished tile leaves by a TMA store, after
//     which the next tile's loads go into its ring tile (up to three tiles
//     ahead of the computing front);
//   * strips hand their last column to the next strip.  The grid is launched
//     as clusters of up to 8 CTAs: inside a cluster the column goes straight
//     into the next strip's shared ring (distributed shared memory), across
//     clusters through global memory with a published progress counter
//     (st.release / ld.acquire).  Every ring entry carries its row in the same
//     64-bit word as its value, so an entry is valid exactly when its tag
//     matches and no flag or fence orders the two.  A second warp per CTA
//     does all of that traffic and issues every tile load and store, so the
//     compute warp only touches its own shared memory and waits on the tiles'
//     mbarriers.  All CTAs of a cluster meet at a cluster barrier before any
//     of them exits.
// The arrays are padded to whole strips and tiles (pitch a multiple of 128
// columns, rows a multiple of 32) and the recurrence runs over the whole
// padded grid: cells outside the reference's loop ranges (border rows and
// columns, padding) have zero coefficients and a zero right-hand side, so
// they hold 0 exactly like the reference's untouched cells, and every TMA
// box lies inside the arrays.
//
// Every wait is bounded: a wait on another strip gives up after
// wave_spin(err) polls (times a fixed factor), sets bit 0 of *err and the
// kernel carries on with invalid values (nothing hangs); a wait on the
// strip's own TMA copies gives up after kWaveSpinLimit polls, and such a
// copy is waited for again (bounded) before the CTA exits.
#pragma once

#include <cuda.h>
#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kM32Lane = 4;                          // columns per lane
constexpr int kM32Cols = 32 * kM32Lane;              // columns per strip (pitch multiple)
constexpr int kM32Rows = 32;                         // rows per tile (row-count multiple)
constexpr int kM32Slots = 4;                         // tiles in each operand's ring
constexpr int kM32RingRows = kM32Slots * kM32Rows;
constexpr int kM32NA = 3;                            // operand arrays per sweep
constexpr int kM32CH = kM32Rows;                     // rows per arrival check of the left column (one per tile)
constexpr int kM32Unroll = 32;                       // steps per unrolled body of a tile's step loop
constexpr int kM32BndChunks = 16;
constexpr int kM32BndRing = kM32BndChunks * kM32CH;  // ring of the left column, rows
constexpr int kM32TopRing = 256;                     // ring of the strip's last column, rows
constexpr int kM32TileFloats = kM32Cols * kM32Rows;
constexpr unsigned kM32TileBytes = kM32TileFloats * 4;
constexpr int kM32ArrayFloats = kM32RingRows * kM32Cols;
static_assert((kM32BndRing & (kM32BndRing - 1)) == 0 && (kM32TopRing & (kM32TopRing - 1)) == 0 &&
                  (kM32Slots & (kM32Slots - 1)) == 0,
              "ring sizes are powers of two (indices are masked)");
constexpr size_t kM32Smem =
    (size_t)kM32NA * kM32ArrayFloats * 4 + (kM32BndRing + kM32TopRing) * 8 + 16 * 4 + 8 * kM32Slots;

// Tensor maps of one sweep: operands in[0..2] (results are written over
// in[0]'s tile in shared memory) and the output; box 128 x 32.
struct Mic32Maps {
    CUtensorMap in[kM32NA];
    CUtensorMap out;
};

// Ring entry of a strip boundary: the value and its sweep row in one 64-bit
// word, written and read with single 64-bit accesses.
__device__ __forceinline__ unsigned long long m32_entry(int r, float v) {
    return ((unsigned long long)(unsigned)r << 32) | (unsigned)__float_as_uint(v);
}
__device__ __forceinline__ bool m32_entry_is(unsigned long long e, int r) { return (unsigned)(e >> 32) == (unsigned)r; }
__device__ __forceinline__ float m32_entry_value(unsigned long long e) { return __uint_as_float((unsigned)e); }

// Components of a lane's float4 in sweep order (the backward sweep runs
// right to left, so its first column is the vector's last component).
template <bool FWD>
__device__ __forceinline__ float m32_get(const float4& v, int m) {
    const int c = FWD ? m : 3 - m;
    return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}
template <bool FWD>
__device__ __forceinline__ float4 m32_pack(const float (&o)[4]) {
    return FWD ? make_float4(o[0], o[1], o[2], o[3]) : make_float4(o[3], o[2], o[1], o[0]);
}

// Arguments of one sweep.  One scene (SEVERAL = false): strip = block, the
// scene's padded region is the whole pack (P32 x NY32 at the origin) and
// `skip` (may be null) cancels the launch.  Several scenes (SEVERAL = true):
// persistent CTAs take the work items in order from work[0] (work[1] counts
// the CTAs that finished; the last one resets both for the next launch); an
// item of a scene whose inner solve stopped is skipped.
struct Mic32Args {
    float* out;                          // result array (pack pitch)
    int pitch;                           // pack pitch
    int P32, NY32;                       // one scene: its padded extent
    const int* skip;                     // one scene: cancel flag
    const Mic32Item* items;              // several scenes
    int nitems;
    const PackScene* scenes;
    int* work;
    unsigned long long* progress;        // one counter per strip / item
    unsigned long long base_host;
    const unsigned long long* base_dev;  // graph-replayed launches: device-memory base (see launch_mic32)
    int* err;
    float sigma;                         // the factor: MIC(0) safety threshold
};

// What a sweep computes per cell from its operands v0, v1, v2, the cell on
// its left (in sweep order) and the cell below:
//   kM32Solve:  out = v0 - v1 * left - v2 * below   (the triangular solves);
//   kM32Factor: the FP32 MIC(0) factor pc = 1 / sqrt(e), with v0 = Adiag,
//               v1 = Ax(i-1,j) (Ax(i-1,j) + tau Ay(i-1,j)), v2 = Ay(i,j-1)
//               (Ay(i,j-1) + tau Ax(i,j-1)) and e = v0 - v1 left^2 - v2 below^2
//               (the reference's MIC(0) expression, regrouped), e replaced
//               by v0 when below sigma v0, and 0 where v0 carries the -0.0
//               non-fluid marker (also the padding's).
constexpr int kM32Solve = 0, kM32Factor = 1;

// out = v0 - v1 * left - v2 * below on the cells of sweep order: the forward
// sweep on q~ = q*pc (v0 = r*pc^2, v1 = fa, v2 = fb), the backward sweep on z
// (v0 = q~, v1 = fc, v2 = fd).  Blocks of 64 threads: warp 0 computes, warp 1
// moves the strip boundary and the tile stores.  One scene: P32 / 128
// strips, rounded up to whole clusters, neighbours in a cluster hand their
// columns over in shared memory; several scenes: a cooperative grid of
// persistent CTAs, hand-offs through global memory.
template <bool FWD, bool SEVERAL, int OP = kM32Solve>
__global__ void __launch_bounds__(64) mic32_kernel(const __grid_constant__ Mic32Maps maps, const Mic32Args a) {
    static_assert(OP == kM32Solve || FWD, "the factor runs forward");
    if (!SEVERAL && a.skip != nullptr && *a.skip) return;
    const unsigned long long base = a.base_dev != nullptr ? *a.base_dev + a.base_host : a.base_host;
    int* const err = a.err;
    float* const out = a.out;
    const int pitch = a.pitch;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);   // [kM32NA][kM32RingRows][kM32Cols]
    // the previous strip's last column (the cells left of this strip), tagged by row
    volatile unsigned long long* bnd = reinterpret_cast<volatile unsigned long long*>(ring + kM32NA * kM32ArrayFloats);
    // this strip's last column, tagged by row, before the I/O warp forwards it
    volatile unsigned long long* top = bnd + kM32BndRing;
    volatile int* ctr = reinterpret_cast<volatile int*>(const_cast<unsigned long long*>(top + kM32TopRing));
    volatile int* bnd_used = ctr + 0;       // chunks of the left column the compute warp has finished
    volatile int* top_done = ctr + 1;       // rows of the last column forwarded by the I/O warp
    volatile int* quit = ctr + 2;           // compute warp gave up (timeout)
    volatile int* tiles_done = ctr + 3;     // tiles whose results are complete in shared memory
    volatile int* cur_item = ctr + 5;       // several scenes: the CTA's current work item
    // loads issued into each ring tile since the launch (kept across work items):
    // load number m of ring tile k completes phase m of mbarrier k
    volatile int* slot_loads = ctr + 8;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 16);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long spin = wave_spin(err);
    const unsigned crank = SEVERAL ? 0u : cluster_ctarank(), csize = SEVERAL ? 1u : cluster_nctarank();
    if (threadIdx.x == 0) {
        for (int k = 0; k < kM32Slots; k++) {
            mbar_init(bars + k, 1);
            slot_loads[k] = 0;
        }
        fence_mbar_init();
    }
    // bit k: parity of the first load of ring tile k in the next strip
    auto slot_parities = [&]() {
        unsigned b = 0;
        for (int k = 0; k < kM32Slots; k++) b |= (unsigned)(slot_loads[k] & 1) << k;
        return b;
    };

    // One strip of one scene: `strip` of `nstrips`, the scene's padded region
    // at pack column x0, row y0, P32 x NR; progress counter `pidx` (the previous
    // strip's is pidx - 1); pbits: slot_parities() before the strip.
    auto run_strip = [&](int strip, int nstrips, int x0, int P32, int y0, int NR, int pidx, unsigned pbits) {
        const int nt = NR / kM32Rows;                           // tiles per strip
        const bool has_next = strip + 1 < nstrips;
        // this strip hands its last column to the next one (unless the test hook holds it back)
        const bool publishes = has_next && !wave_held(err, kWaveKindMic32, strip);
        const bool left_in_grid = strip > 0;
        const int xbox = x0 + (FWD ? strip * kM32Cols : P32 - (strip + 1) * kM32Cols);   // pack column of box column 0
        const int xlast = FWD ? xbox + kM32Cols - 1 : xbox;    // pack column of the strip's last sweep column
        const int xprev = FWD ? xbox - 1 : xbox + kM32Cols;    // ... and of the previous strip's
        const bool prev_local = !SEVERAL && left_in_grid && crank > 0;       // the previous strip fills this ring
        const bool next_local = !SEVERAL && publishes && crank + 1 < csize;  // this strip fills the next strip's ring
        auto mrow = [&](int r) { return y0 + (FWD ? r : NR - 1 - r); };   // pack row of sweep row r
        auto tile_y = [&](int t) { return y0 + (FWD ? t * kM32Rows : NR - (t + 1) * kM32Rows); };

        if (warp == 1) {
            // ---------------- I/O warp ----------------
            const unsigned long long* gprev = left_in_grid ? a.progress + (pidx - 1) : nullptr;
            int hb = (left_in_grid && !prev_local) ? 0 : NR;   // next row of the left column to fetch
            int tc = 0;                                        // rows of the last column forwarded
            const int tend = publishes ? NR : 0;
            int rused = 0;                                     // last seen chunk position of the consumer
            const unsigned r_bnd = next_local ? mapa_shared((const void*)bnd, crank + 1) : 0u;
            const unsigned r_used = next_local ? mapa_shared((const void*)bnd_used, crank + 1) : 0u;
            int ts = 0;                                        // next tile to store
            int rd = 0;                                        // stores that have read their ring tiles
            int tl = 0;                                        // next tile to load
            unsigned long long gavail = 0;
            long long idle = 0;
            while (hb < NR || tc < tend || ts < nt || tl < nt) {
                bool moved = false;
                // left column from global memory (the previous strip is in another cluster)
                const int hb_lim = (*bnd_used + kM32BndChunks - 2) * kM32CH;   // slots consumed two chunks ago
                if (hb < NR && hb < hb_lim) {
                    const int n = min(min(32, NR - hb), hb_lim - hb);
                    const unsigned long long need = base + (unsigned long long)(hb + n);
                    if (gavail < need) {
                        unsigned long long v = 0;
                        if (lane == 0) v = ld_acquire(gprev);
                        gavail = __shfl_sync(0xffffffffu, v, 0);
                    }
                    const int avail = (int)min((unsigned long long)n, gavail > base + hb ? gavail - base - hb : 0ull);
                    if (avail > 0) {
                        __syncwarp();   // lane 0's acquire orders the reads below
                        const int r = hb + lane;
                        if (lane < avail)
                            bnd[r & (kM32BndRing - 1)] = m32_entry(r, __ldcg(out + (size_t)mrow(r) * pitch + xprev));
                        __syncwarp();
                        hb += avail;
                        moved = true;
                    }
                }
                // last column out: to the next strip's ring (same cluster) or to global
                // memory, every complete run of up to 128 rows at once
                for (int rep = 0; rep < 4 && tc < tend; rep++) {
                    const int r = tc + lane;
                    const unsigned long long e = r < NR ? top[r & (kM32TopRing - 1)] : 0ull;
                    const bool ok = r >= NR || m32_entry_is(e, r);
                    const unsigned bad = __ballot_sync(0xffffffffu, !ok);
                    int n = bad ? __ffs(bad) - 1 : 32;
                    n = min(n, NR - tc);
                    if (n > 0 && next_local) {
                        // the consumer's ring slot of row r was last used by row r - kM32BndRing
                        if (tc + n > (rused + kM32BndChunks - 2) * kM32CH) {
                            int v = 0;
                            if (lane == 0) v = ld_volatile_cluster_remote(r_used);
                            rused = __shfl_sync(0xffffffffu, v, 0);
                        }
                        n = min(n, (rused + kM32BndChunks - 2) * kM32CH - tc);
                    }
                    if (n > 0) {
                        if (next_local) {
                            if (lane < n) st_cluster_u64(r_bnd + 8u * (unsigned)(r & (kM32BndRing - 1)), e);
                            __syncwarp();
                        } else {
                            if (lane < n) out[(size_t)mrow(r) * pitch + xlast] = m32_entry_value(e);
                            __threadfence();
                            __syncwarp();
                            if (lane == 0) st_release(a.progress + pidx, base + (unsigned long long)(tc + n));
                        }
                        tc += n;
                        if (lane == 0) *top_done = tc;
                        moved = true;
                    }
                    if (n < 32) break;
                }
                if (ts < nt && *tiles_done > ts) {
                    // results of tile ts are complete (the compute warp fenced them
                    // for the async proxy before publishing tiles_done).  The warp
                    // does not wait for this store to read its tile, only for the
                    // stores before it
                    if (lane == 0) {
                        tma_store_2d(&maps.out, xbox, tile_y(ts), ring + (size_t)(ts & (kM32Slots - 1)) * kM32TileFloats);
                        bulk_commit();
                        bulk_wait_read<1>();
                    }
                    __syncwarp();
                    ts++;
                    rd = ts - 1;
                    moved = true;
                }
                // operand tiles in: tile tl goes into the ring tile of tile
                // tl - kM32Slots, free once that tile's store has read it (the
                // store went out after the compute warp finished the tile)
                while (tl < nt && tl - kM32Slots < rd) {
                    if (lane == 0) {
                        const int k = tl & (kM32Slots - 1);
                        mbar_expect_tx(bars + k, kM32NA * kM32TileBytes);
                        float* dst = ring + (size_t)k * kM32TileFloats;
#pragma unroll
                        for (int q = 0; q < kM32NA; q++)
                            tma_load_2d(dst + (size_t)q * kM32ArrayFloats, &maps.in[q], xbox, tile_y(tl), bars + k);
                    }
                    __syncwarp();
                    tl++;
                    moved = true;
                }
                if (moved) {
                    idle = 0;
                } else if (rd < ts) {
                    // nothing else to do: wait for the newest store to read its
                    // tile, so that the next load into its ring tile goes out now
                    if (lane == 0) bulk_wait_read<0>();
                    __syncwarp();
                    rd = ts;
                } else if (++idle > 16 * spin || *quit || ((idle & 1023) == 0 && wave_failed(err))) {
                    if (lane == 0) {
                        atomicOr(err, kWaitStrip | (kWaveKindMic32 << 4));
                        *quit = 1;
                    }
                    break;
                }
            }
            if (lane == 0) {
                bulk_wait_all();
                // no load may still be writing into the ring when the CTA moves on or
                // exits: wait (bounded) for the newest load of every ring tile, then
                // count this strip's loads
                for (int k = 0; k < kM32Slots; k++) {
                    const int n = tl > k ? (tl - 1 - k) / kM32Slots + 1 : 0;
                    if (n > 0) {
                        const unsigned par = (unsigned)(slot_loads[k] + n - 1) & 1u;
                        long long polls = 0;
                        while (!mbar_try_wait(bars + k, par) && ++polls <= kWaveSpinLimit) {
                        }
                    }
                    slot_loads[k] += n;
                }
            }
            __syncwarp();
        } else {
            // ---------------- compute warp ----------------
            bool failed = false;
            // tile t of this strip is the (t / kM32Slots)-th load of its ring tile
            // in this strip, issued by the I/O warp once the ring tile is free (the
            // mbarrier's phase cannot complete before)
            auto wait_tile = [&](int t) {
                if (failed) return;   // after one timeout the results are invalid: do not wait again
                const int k = t & (kM32Slots - 1);
                const unsigned par = ((pbits >> k) ^ (unsigned)(t / kM32Slots)) & 1u;
                long long polls = 0;
                while (!mbar_try_wait(bars + k, par)) {
                    if (++polls > kWaveSpinLimit || ((polls & 1023) == 0 && *quit)) {
                        failed = true;
                        atomicOr(err, kWaitTile | (kWaveKindMic32 << 4));
                        *quit = 1;
                        return;
                    }
                }
            };
            auto spin_ge = [&](volatile int* flag, int need) {  // bounded wait on an I/O-warp counter
                if (failed) return;  // after one timeout the results are invalid: do not wait again
                long long polls = 0;
                while (*flag < need) {
                    if (++polls > 16 * spin) {
                        failed = true;
                        atomicOr(err, kWaitWarp | (kWaveKindMic32 << 4));
                        *quit = 1;
                        return;
                    }
                }
            };

            // the lane's float4 in every ring row: box columns 4l .. 4l+3 (the
            // backward sweep's box is mirrored: its sweep column 4l is box column
            // 127 - 4l); ring row of sweep row r: r (forward) or r ^ 31 (backward,
            // whose box rows run against the sweep), modulo the ring
            const int colbase = FWD ? kM32Lane * lane : kM32Cols - kM32Lane * (lane + 1);
            constexpr int kRowXor = FWD ? 0 : kM32Rows - 1;
            auto cell_ptr = [&](int r) {
                return ring + (size_t)((r ^ kRowXor) & (kM32RingRows - 1)) * kM32Cols + colbase;
            };
            // plain (non-volatile) views of the rings for the pipelined per-step
            // accesses; the row tags make stale reads harmless
            const unsigned long long* bnd_p = const_cast<const unsigned long long*>(bnd);
            unsigned long long* top_p = const_cast<unsigned long long*>(top);
            float o[4] = {0.f, 0.f, 0.f, 0.f};   // the lane's row r - 1 (the cells below)
            unsigned long long bn = 0ull;        // left-column entry of the next step (read one step ahead)
            float4 x_n, a_n, b_n;                // operands of the next step (loaded one step ahead)
            auto load_next = [&](const float* p) {
                x_n = *reinterpret_cast<const float4*>(p);
                a_n = *reinterpret_cast<const float4*>(p + kM32ArrayFloats);
                b_n = *reinterpret_cast<const float4*>(p + 2 * kM32ArrayFloats);
            };

            // One tile group of 32 steps.  CHECK: some lane's row may lie outside
            // [0, NR) (first and last groups); a compile-time flag, so that the
            // steady-state groups carry no per-step range tests (and the checking
            // groups only selects and predicated stores).
            auto tile_steps = [&](int t, auto check_tag) {
                constexpr bool check = decltype(check_tag)::value;
                const int s0 = t * kM32Rows;
                load_next(cell_ptr(s0 - lane));
                if (left_in_grid && (!check || s0 < NR)) {
                    // lane 0 enters the tile's chunk of the left column: every row of
                    // it must have arrived (one entry per lane, one vote)
                    const int rr = s0 + lane;
                    bool ok = rr >= NR || m32_entry_is(bnd_p[rr & (kM32BndRing - 1)], rr);
                    if (!__all_sync(0xffffffffu, ok)) {
                        // the whole warp polls in step until every entry is there:
                        // lanes leaving a polling loop one by one would leave the warp
                        // diverged for the steps after it (measured: a group of steps
                        // five times as long)
                        long long polls = 0;
                        while (!failed) {
                            ok = rr >= NR || m32_entry_is(bnd[rr & (kM32BndRing - 1)], rr);
                            if (__all_sync(0xffffffffu, ok)) break;
                            const bool give_up = ++polls > 16 * spin || ((polls & 1023) == 0 && wave_failed(err));
                            if (__any_sync(0xffffffffu, give_up)) {
                                failed = true;
                                if (lane == 0) {
                                    atomicOr(err, kWaitStrip | (kWaveKindMic32 << 4));
                                    *quit = 1;
                                }
                            }
                        }
                    }
                    __syncwarp();   // lane 0 reads the entries its neighbours validated
                    bn = bnd_p[s0 & (kM32BndRing - 1)];
                    // earlier chunks are read: their slots may be refilled (a plain
                    // store suffices, every value read from them was consumed by
                    // arithmetic before this store issues, and a refill lands at
                    // least two chunks behind it)
                    if (lane == 0) *bnd_used = s0 / kM32CH;
                }
#pragma unroll kM32Unroll
                for (int u = 0; u < kM32Rows; u++) {
                    {
                        const int s = s0 + u;
                        const int r = s - lane;
                        const float4 xv = x_n, av = a_n, bv = b_n;
                        // a row outside [0, NR) (first and last groups) is computed on
                        // whatever its ring row holds (the index wraps inside the ring),
                        // kept at 0 and not stored, so that no branch surrounds the step;
                        // it only feeds rows outside [0, NR) of the lanes to its right
                        const bool valid = !check || (r >= 0 && r < NR);
                        float* const p = cell_ptr(r);
                        // next step's operands (row r + 1), loaded before this step's store
                        load_next(cell_ptr(r + 1));
                        float left = __shfl_up_sync(0xffffffffu, o[3], 1);
                        const float l0 = left_in_grid ? m32_entry_value(bn) : 0.0f;
                        // next step's entry (after the tile's last step a stale one: the
                        // next tile reads its first entry again after its check)
                        bn = bnd_p[(s + 1) & (kM32BndRing - 1)];
                        if (lane == 0) left = l0;
                        {
                            float w[4];
                            if (OP == kM32Solve) {
#pragma unroll
                                for (int m = 0; m < 4; m++)
                                    w[m] = fmaf(-m32_get<FWD>(bv, m), o[m], m32_get<FWD>(xv, m));
#pragma unroll
                                for (int m = 0; m < 4; m++) {
                                    o[m] = fmaf(-m32_get<FWD>(av, m), left, w[m]);
                                    left = o[m];
                                }
                            } else {
#pragma unroll
                                for (int m = 0; m < 4; m++)
                                    w[m] = fmaf(-(m32_get<FWD>(bv, m) * o[m]), o[m], m32_get<FWD>(xv, m));
#pragma unroll
                                for (int m = 0; m < 4; m++) {
                                    const float ad = m32_get<FWD>(xv, m);
                                    const float e = fmaf(-(m32_get<FWD>(av, m) * left), left, w[m]);
                                    o[m] = signbit(ad) ? 0.0f : rsqrtf(e < a.sigma * ad ? ad : e);
                                    left = o[m];
                                }
                            }
                            if (check) {
#pragma unroll
                                for (int m = 0; m < 4; m++) o[m] = valid ? o[m] : 0.0f;
                            }
                            if (valid) *reinterpret_cast<float4*>(p) = m32_pack<FWD>(o);
                            if (publishes && lane == 31 && valid) top_p[r & (kM32TopRing - 1)] = m32_entry(r, o[3]);
                        }
                    }
                }
            };

            const int nsteps = NR + 31;
            for (int t = 0; t * kM32Rows < nsteps; t++) {
                if (t < nt) wait_tile(t);
                // last-column ring: do not run more than half a ring ahead of the I/O warp
                if (publishes && t * kM32Rows - 31 - *top_done > kM32TopRing / 2)
                    spin_ge(top_done, t * kM32Rows - 31 - kM32TopRing / 2);
                __syncwarp();
                if (t == 0 || t >= nt)
                    tile_steps(t, BoolTag<true>{});
                else
                    tile_steps(t, BoolTag<false>{});
                // tile t-1 is finished for every lane: hand it to the I/O warp for its
                // TMA store (after which its ring tile takes the loads of tile t+3)
                if (t >= 1 && t - 1 < nt) {
                    fence_async_smem();
                    __syncwarp();
                    if (lane == 0) *tiles_done = t;
                }
            }
            __syncwarp();
            if (lane == 0) {
                *tiles_done = nt;
                if (left_in_grid) *bnd_used = NR / kM32CH + kM32BndChunks;
            }
        }
    };
    // rings and counters of a strip: no row matches, nothing done
    auto reset_rings = [&]() {
        if (threadIdx.x == 0) {
            *bnd_used = 0;
            *top_done = 0;
            *quit = 0;
            *tiles_done = 0;
        }
        for (int k = threadIdx.x; k < kM32BndRing; k += blockDim.x) bnd[k] = ~0ull;
        for (int k = threadIdx.x; k < kM32TopRing; k += blockDim.x) top[k] = ~0ull;
    };

    if (!SEVERAL) {
        const int strip = blockIdx.x;
        const int nstrips = a.P32 / kM32Cols;
        reset_rings();
        cluster_sync_all();   // every ring and counter of the cluster is initialised
        if (strip < nstrips) run_strip(strip, nstrips, 0, a.P32, 0, a.NY32, strip, 0u);   // the grid is rounded up to whole clusters
        cluster_sync_all();   // no CTA leaves while a neighbour may still touch its shared memory
    } else {
        // persistent: items are taken in list order and a strip's previous strip
        // comes earlier in the list, so it was taken earlier by a co-resident CTA
        // and every wait makes progress
        for (;;) {
            __syncthreads();   // the previous item is finished by both warps
            if (threadIdx.x == 0) *cur_item = atomicAdd(&a.work[0], 1);
            reset_rings();
            // the previous item's loads are counted and this item's not yet issued
            const unsigned pbits = slot_parities();
            __syncthreads();
            const int it = *cur_item;
            if (it >= a.nitems) break;
            const Mic32Item item = a.items[it];
            if (OP == kM32Solve && a.scenes[item.scene].inner->done) continue;   // that scene's inner solve stopped
            run_strip(item.strip, item.nstrips, item.x0, item.P32, item.y0, item.NY32, item.pidx, pbits);
        }
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&a.work[1], 1) == (int)gridDim.x - 1) {   // the last CTA resets the counters
                a.work[0] = 0;
                a.work[1] = 0;
                __threadfence();
            }
        }
    }
}

// Host side: tensor map for one FP32 array of P x NR (row pitch P floats),
// box 128 x 32.
int mic32_make_map(CUtensorMap* map, float* base, int P, int NR);

// Advances the device-side progress base of graph-replayed sweeps by `n`
// sweeps' worth.
__global__ void k_wave_bump(unsigned long long* base, unsigned long long n) { *base += n << 24; }

// Where a pack's kernels go: stream, error word (with the wait controls),
// launch counter, progress bases, and the handle whose per-kernel timing
// applies (null: none).
struct PackLaunch {
    cudaStream_t stream;
    int* err;
    int device;
    unsigned long long* launches;
    unsigned long long wave_launch;   // progress base counter of direct sweeps
    Sim* timer;
};

// Launches one sweep of every scene of the pack.  One scene: cooperative
// (every strip co-resident, so the waits between strips always make
// progress) and, where the device can hold them, in clusters of up to 8
// strips that hand columns over in shared memory.  Several scenes: a
// cooperative grid of persistent CTAs (pk->sweep_ctas) over the work items.
// graph_slot >= 0: for stream capture; the sweep is number graph_slot of the
// graph_sweeps sweeps of one replay, uses the graph's progress counters and
// the device-memory base plus graph_slot sweeps; slot 0 first advances that
// base by graph_sweeps, so that every replay gets fresh bases.
template <bool FWD, int OP = kM32Solve>
int launch_mic32(Pack* pk, PackLaunch& L, float* out, int graph_slot = -1, int graph_sweeps = 0, float sigma = 0.f) {
    const bool graph = graph_slot >= 0;
    const bool several = pk->n > 1;
    const int nstrips = several ? pk->nitems : pk->scenes[0].P32 / kM32Cols;
    if (nstrips > pk->progress_cap) {
        set_error("mic32: %d strips exceed the %d progress counters", nstrips, pk->progress_cap);
        return FS2D_ERR_INVALID;
    }
    const void* fn =
        several ? (const void*)mic32_kernel<FWD, true, OP> : (const void*)mic32_kernel<FWD, false, OP>;
    static std::atomic<unsigned long long> configured[2] = {{0}, {0}};
    if (int rc0 = ensure_smem_attr(configured[several ? 1 : 0], L.device, fn, (int)kM32Smem)) return rc0;
    Mic32Args a{};
    a.out = out;
    a.pitch = pk->pitch;
    a.P32 = pk->scenes[0].P32;
    a.NY32 = pk->scenes[0].NY32;
    a.skip = (several || OP == kM32Factor) ? nullptr : &pk->scenes[0].inner->done;   // every scene needs its factor
    a.items = pk->d_items;
    a.nitems = pk->nitems;
    a.scenes = pk->d_scenes;
    a.work = pk->d_ctl + 2;
    a.err = L.err;
    a.sigma = sigma;
    if (graph) {
        if (graph_slot == 0) {
            (*L.launches)++;
            k_wave_bump<<<1, 1, 0, L.stream>>>(pk->gbase, (unsigned long long)graph_sweeps);
            if (int rc1 = check_cuda(cudaGetLastError(), "k_wave_bump")) return rc1;
        }
        a.base_host = (unsigned long long)graph_slot << 24;
        a.base_dev = pk->gbase;
        a.progress = pk->gprogress;
    } else {
        a.base_host = (++L.wave_launch) << 24;
        a.base_dev = nullptr;
        a.progress = pk->progress;
    }
    const Mic32Maps& maps =
        *reinterpret_cast<const Mic32Maps*>(OP == kM32Factor ? pk->maps->fac : (FWD ? pk->maps->fwd : pk->maps->bwd));
    void* args[] = {(void*)&maps, (void*)&a};
    (*L.launches)++;
    const char* name = OP == kM32Factor ? "mic32_factor" : (FWD ? "mic32_forward" : "mic32_backward");
    long long kt = L.timer ? ktimer_begin(L.timer, name) : -1;
    cudaError_t e;
    if (several) {
        e = launch_clustered(fn, pk->sweep_ctas, 1, 64, kM32Smem, L.stream, args);
    } else {
        int& cs = pk->cluster;   // 0: not chosen yet
        if (cs == 0) cs = choose_cluster(fn, nstrips, 64, kM32Smem);
        e = launch_clustered(fn, nstrips, cs, 64, kM32Smem, L.stream, args);
        if (e != cudaSuccess && cs > 1 && !graph) {   // clusters refused: plain cooperative launch
            (void)cudaGetLastError();
            cs = 1;
            e = launch_clustered(fn, nstrips, 1, 64, kM32Smem, L.stream, args);
        }
    }
    int rc = check_cuda(e, name);
    if (L.timer) ktimer_end(L.timer, kt);
    return rc;
}

}  // namespace fs2d
