// mic32_tma.cuh — FP32 MIC(0) triangular solves as a TMA-staged wavefront.
//
// The forward and backward substitutions of applyPreconditioner
// (src/FluidSim2D.cpp:397-421) are recurrences over the grid in the
// reference's loop order.  This kernel keeps that dependency order and
// spreads the work as follows:
//   * one warp per CTA owns a strip of 128 rows; lane l owns rows 4l..4l+3
//     (in sweep order) and at step s works on column c = s - l, so the warp
//     is a diagonal front; within a lane the four rows are computed bottom
//     to top in the same step, the row below lane l's first row arrives from
//     lane l-1 by shuffle, and the previous column stays in registers;
//   * operand tiles of 32 columns x 128 rows are brought into shared memory
//     by the Tensor Memory Accelerator (cp.async.bulk.tensor, completion on
//     an mbarrier), two tiles ahead, in a ring of four slots;
//   * results overwrite the operand they were computed from, and each
//     finished tile is written back with a TMA store (cp.async.bulk.tensor
//     ... bulk_group); the backward sweep's partial last strip uses a tensor
//     map with a shorter box so that no store starts at a negative row;
//   * strips hand their top row to the next strip.  The grid is launched as
//     clusters of up to 8 CTAs; inside a cluster the previous strip writes
//     each chunk of 16 columns straight into the next strip's shared ring
//     (distributed shared memory) and releases it with a cluster-scope add
//     to that strip's chunk counter.  Across clusters the top row goes
//     through global memory with a published progress counter (st.release /
//     ld.acquire).  A second warp per CTA does all of that traffic, so the
//     compute warp only touches its own shared memory (and issues the TMA
//     copies) and no remote write, release or L2 round trip sits on its
//     critical path.  All CTAs of a cluster meet at a cluster barrier before
//     any of them exits.
// The recurrence runs over the whole padded grid: cells outside the
// reference's loop ranges (border rows/columns, padding) have zero
// coefficients and a zero right-hand side, so they hold 0 exactly like the
// reference's untouched cells.  Every wait is bounded; on timeout bit 0 of
// *err is set and the kernel carries on (results invalid, nothing hangs), and
// before exiting it waits (bounded) for its own copies in flight.
#pragma once

#include <cuda.h>
#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kM32Rows = 128;   // rows per strip (4 per lane)
constexpr int kM32Cols = 32;    // tile width
constexpr int kM32Slots = 4;
constexpr int kM32NA = 3;       // operand arrays per sweep
constexpr int kM32CH = 16;      // flow-control chunk of the boundary rings (columns)
constexpr int kM32BndChunks = 16; // ring of the row below, in chunks
constexpr int kM32BndRing = kM32BndChunks * kM32CH;
constexpr int kM32TopRing = 256;  // ring of the strip's top row (columns)
constexpr int kM32TileFloats = kM32Rows * kM32Cols;
constexpr unsigned kM32TileBytes = kM32TileFloats * 4;
constexpr size_t kM32Smem =
    (size_t)kM32Slots * kM32NA * kM32TileBytes + (kM32BndRing + kM32TopRing) * 8 + 8 * 4 + 8 * kM32Slots;

// Tensor maps of one sweep: operands in[0..2] (in[0] is also where results
// are written in shared memory), the output, and the output with a box of
// `tail` rows (tail = NY % 128) for the backward sweep's partial strip.
struct Mic32Maps {
    CUtensorMap in[kM32NA];
    CUtensorMap out;
    CUtensorMap out_tail;
};

// Ring entries of the strip boundary: the value and its sweep column in one
// 64-bit word, written and read with single 64-bit accesses, so an entry is
// valid exactly when its column matches (no flag or fence is needed between
// the writer and the reader of the value).
__device__ __forceinline__ unsigned long long m32_entry(int c, float v) {
    return ((unsigned long long)(unsigned)c << 32) | (unsigned)__float_as_uint(v);
}
__device__ __forceinline__ bool m32_entry_is(unsigned long long e, int c) { return (unsigned)(e >> 32) == (unsigned)c; }
__device__ __forceinline__ float m32_entry_value(unsigned long long e) { return __uint_as_float((unsigned)e); }

// FWD: out = v0 - v1*left - v2*below  (forward, on q~ = q*pc)
// BWD: same form with the backward coefficients.
// Block of 64 threads: warp 0 computes, warp 1 moves the strip boundaries
// (so no remote write, release or L2 round trip stalls the compute warp).
template <bool FWD>
// base_dev: when non-null, the launch's progress base is the device-memory
// value plus `base_host` (launches replayed from a CUDA graph: one bump of
// that counter per replay, and a fixed offset per sweep of the replay);
// otherwise `base_host` alone.
__global__ void __launch_bounds__(64) mic32_kernel(const __grid_constant__ Mic32Maps maps, float* out, int P, int NY,
                                                   unsigned long long* progress, unsigned long long base_host,
                                                   const unsigned long long* base_dev, int* err, const int* skip) {
    if (skip != nullptr && *skip) return;
    const unsigned long long base = base_dev != nullptr ? *base_dev + base_host : base_host;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    // row below the strip, kM32BndRing columns of tagged entries
    volatile unsigned long long* bnd =
        reinterpret_cast<volatile unsigned long long*>(ring + (size_t)kM32Slots * kM32NA * kM32TileFloats);
    // the strip's top row, kM32TopRing columns of tagged entries
    volatile unsigned long long* top = bnd + kM32BndRing;
    volatile int* ctr = reinterpret_cast<volatile int*>(const_cast<unsigned long long*>(top + kM32TopRing));
    volatile int* bnd_used = ctr + 0;       // chunks of the row below the compute warp has finished
    volatile int* top_done = ctr + 1;       // top-row columns forwarded by the I/O warp
    volatile int* quit = ctr + 2;           // compute warp gave up (timeout)
    volatile int* tiles_done = ctr + 3;     // tiles whose results are complete in shared memory
    volatile int* tiles_freed = ctr + 4;    // tiles whose TMA store has finished reading shared memory
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 8);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int strip = blockIdx.x;
    const int nstrips = (NY + kM32Rows - 1) / kM32Rows;
    const int nt = P / kM32Cols;             // tiles per row (P is a multiple of 32)
    const int ncols = P;
    const int ybox = FWD ? strip * kM32Rows : NY - (strip + 1) * kM32Rows;  // first memory row of the box
    const bool has_next = strip + 1 < nstrips;
    const int ytop = FWD ? ybox + kM32Rows - 1 : ybox;       // the strip's last row in sweep order
    const int ybelow = FWD ? ybox - 1 : ybox + kM32Rows;     // the row below the strip
    const bool below_in_grid = strip > 0;
    const bool active = strip < nstrips;                       // the grid is rounded up to whole clusters
    const unsigned crank = cluster_ctarank(), csize = cluster_nctarank();
    const bool prev_local = below_in_grid && crank > 0;        // the previous strip fills this ring
    const bool next_local = has_next && crank + 1 < csize;     // this strip fills the next strip's ring
    auto mcol = [&](int c) { return FWD ? c : P - 1 - c; };  // memory column of sweep column c

    if (threadIdx.x == 0) {
        for (int k = 0; k < kM32Slots; k++) mbar_init(bars + k, 1);
        fence_mbar_init();
        *bnd_used = 0;
        *top_done = 0;
        *quit = 0;
        *tiles_done = 0;
        *tiles_freed = 0;
    }
    for (int k = threadIdx.x; k < kM32BndRing; k += blockDim.x) bnd[k] = ~0ull;   // no column matches
    for (int k = threadIdx.x; k < kM32TopRing; k += blockDim.x) top[k] = ~0ull;
    cluster_sync_all();   // every ring and counter of the cluster is initialised

    if (warp == 1 && active) {
        // ---------------- I/O warp ----------------
        const unsigned long long* gprev = below_in_grid ? progress + (strip - 1) : nullptr;
        int hb = (below_in_grid && !prev_local) ? 0 : ncols;   // next column of the row below to fetch
        int tc = 0;                                             // top-row columns forwarded
        const int tend = has_next ? ncols : 0;
        int rused = 0;                           // last seen chunk position of the consumer
        const unsigned r_bnd = next_local ? mapa_shared((const void*)bnd, crank + 1) : 0u;
        const unsigned r_used = next_local ? mapa_shared((const void*)bnd_used, crank + 1) : 0u;
        int ts = 0;                              // next tile to store
        unsigned long long gavail = 0;
        long long idle = 0;
        while (hb < ncols || tc < tend || ts < nt) {
            bool moved = false;
            // row below from global memory (the previous strip is in another cluster)
            const int hb_lim = (*bnd_used + kM32BndChunks - 2) * kM32CH;   // slots consumed two chunks ago
            if (hb < ncols && hb < hb_lim) {
                const int n = min(min(32, ncols - hb), hb_lim - hb);
                const unsigned long long need = base + (unsigned long long)(hb + n);
                if (gavail < need) {
                    unsigned long long v = 0;
                    if (lane == 0) v = ld_acquire(gprev);
                    gavail = __shfl_sync(0xffffffffu, v, 0);
                }
                const int avail = (int)min((unsigned long long)n, gavail > base + hb ? gavail - base - hb : 0ull);
                if (avail > 0) {
                    __syncwarp();   // lane 0's acquire orders the reads below
                    const int c = hb + lane;
                    if (lane < avail)
                        bnd[c % kM32BndRing] = m32_entry(c, __ldcg(out + (size_t)ybelow * P + mcol(c)));
                    __syncwarp();
                    hb += avail;
                    moved = true;
                }
            }
            // top row out: to the next strip's ring (same cluster) or to global memory
            if (tc < tend) {
                const int c = tc + lane;
                const unsigned long long e = c < ncols ? top[c % kM32TopRing] : 0ull;
                const bool ok = c >= ncols || m32_entry_is(e, c);
                const unsigned bad = __ballot_sync(0xffffffffu, !ok);
                int n = bad ? __ffs(bad) - 1 : 32;
                n = min(n, ncols - tc);
                if (n > 0 && next_local) {
                    // the consumer's ring slot of column c was last used by column c - kM32BndRing
                    if (tc + n > (rused + kM32BndChunks - 2) * kM32CH) {
                        int v = 0;
                        if (lane == 0) v = ld_volatile_cluster_remote(r_used);
                        rused = __shfl_sync(0xffffffffu, v, 0);
                    }
                    n = min(n, (rused + kM32BndChunks - 2) * kM32CH - tc);
                }
                if (n > 0) {
                    if (next_local) {
                        if (lane < n) st_cluster_u64(r_bnd + 8u * (unsigned)(c % kM32BndRing), e);
                        __syncwarp();
                    } else {
                        if (lane < n) out[(size_t)ytop * P + mcol(c)] = m32_entry_value(e);
                        __threadfence();
                        __syncwarp();
                        if (lane == 0) st_release(progress + strip, base + (unsigned long long)(tc + n));
                    }
                    tc += n;
                    if (lane == 0) *top_done = tc;
                    moved = true;
                }
            }
            if (ts < nt && *tiles_done > ts) {
                // results of tile ts are complete (the compute warp fenced them
                // for the async proxy before publishing tiles_done)
                if (lane == 0) {
                    const float* src = ring + (size_t)(ts & (kM32Slots - 1)) * kM32NA * kM32TileFloats;
                    const int x = FWD ? ts * kM32Cols : P - (ts + 1) * kM32Cols;
                    if (ybox >= 0) {
                        tma_store_2d(&maps.out, x, ybox, src);
                    } else {
                        const int tail = NY % kM32Rows;
                        tma_store_2d(&maps.out_tail, x, 0, src + (kM32Rows - tail) * kM32Cols);
                    }
                    bulk_commit();
                    bulk_wait_read<0>();
                    *tiles_freed = ts + 1;
                }
                __syncwarp();
                ts++;
                moved = true;
            }
            if (moved) {
                idle = 0;
            } else if (++idle > 16 * kWaveSpinLimit || *quit || ((idle & 1023) == 0 && *(volatile int*)err)) {
                if (lane == 0) atomicOr(err, 1);
                break;
            }
        }
        if (lane == 0) bulk_wait_all();
        __syncwarp();
    } else if (warp == 0 && active) {
        // ---------------- compute warp ----------------
        auto tile_x = [&](int t) { return FWD ? t * kM32Cols : P - (t + 1) * kM32Cols; };
        auto slot_ptr = [&](int t) { return ring + (size_t)(t & (kM32Slots - 1)) * kM32NA * kM32TileFloats; };
        auto issue = [&](int t) {
            if (lane == 0 && t < nt) {
                unsigned long long* bar = bars + (t & (kM32Slots - 1));
                mbar_expect_tx(bar, kM32NA * kM32TileBytes);
                float* dst = slot_ptr(t);
#pragma unroll
                for (int a = 0; a < kM32NA; a++)
                    tma_load_2d(dst + a * kM32TileFloats, &maps.in[a], tile_x(t), ybox, bar);
            }
        };
        bool failed = false;
        auto wait_tile = [&](int t) {
            unsigned long long* bar = bars + (t & (kM32Slots - 1));
            const unsigned parity = (unsigned)((t / kM32Slots) & 1);
            long long polls = 0;
            while (!mbar_try_wait(bar, parity)) {
                if (++polls > kWaveSpinLimit) {
                    failed = true;
                    atomicOr(err, 1);
                    break;
                }
            }
        };
        auto spin_ge = [&](volatile int* flag, int need) {  // bounded wait on an I/O-warp counter
            if (failed) return;  // after one timeout the results are invalid: do not wait again
            long long polls = 0;
            while (*flag < need) {
                if (++polls > 16 * kWaveSpinLimit) {
                    failed = true;
                    atomicOr(err, 1);
                    *quit = 1;
                    return;
                }
            }
        };
        issue(0);
        issue(1);

        const int row0 = FWD ? 4 * lane : kM32Rows - 1 - 4 * lane;   // box row of the lane's first row
        const int rstep = FWD ? kM32Cols : -kM32Cols;                 // box offset between the lane's rows
        const int cdir = FWD ? 1 : -1;                                // box-column step per column
        auto cell_ptr = [&](int c) {  // operand-0 address of (row0, c) in its ring slot (c >= 0)
            const int bc = FWD ? (c & 31) : 31 - (c & 31);
            return slot_ptr(c >> 5) + row0 * kM32Cols + bc;
        };
        // plain (non-volatile) views of the rings for the pipelined per-step
        // accesses; the column tags make stale reads harmless
        const unsigned long long* bnd_p = const_cast<const unsigned long long*>(bnd);
        unsigned long long* top_p = const_cast<unsigned long long*>(top);
        float o[4] = {0.f, 0.f, 0.f, 0.f};
        unsigned long long bn = 0ull;   // entry of the row below for the next step (read one step ahead)
        float vn[4][kM32NA];            // operands of the next step (loaded one step ahead)
        float* pn = nullptr;            // their address
        auto load_next = [&](float* p) {
#pragma unroll
            for (int k = 0; k < 4; k++)
#pragma unroll
                for (int a = 0; a < kM32NA; a++) vn[k][a] = p[k * rstep + a * kM32TileFloats];
        };

        // One tile of 32 steps.  CHECK: some lane's column may lie outside
        // [0, ncols) (first and last tiles); a compile-time flag, so that the
        // steady-state tiles carry no per-step range tests.
        auto tile_steps = [&](int t, auto check_tag) {
            constexpr bool check = decltype(check_tag)::value;
            {
                const int c0 = t * kM32Cols - lane;
                pn = cell_ptr(c0 < 0 ? 0 : c0);
                load_next(pn);
            }
            // one chunk of the row below per group: a rolled loop of two
            // groups with the chunk's steps unrolled measured 2-6 % faster
            // than the whole tile unrolled
#pragma unroll 1
            for (int g = 0; g < kM32Cols; g += kM32CH) {
#pragma unroll
            for (int u8 = 0; u8 < kM32CH; u8++) {
                const int u = g + u8;
                const int s = t * kM32Cols + u;
                const int c = s - lane;
                if (below_in_grid && u8 == 0 && (!check || s < ncols)) {
                    // lane 0 enters a chunk of the row below: every column of
                    // it must have arrived (one entry per lane, one vote)
                    const int cc = s + (lane & (kM32CH - 1));
                    bool ok = cc >= ncols || m32_entry_is(bnd_p[cc % kM32BndRing], cc);
                    if (!__all_sync(0xffffffffu, ok)) {
                        long long polls = 0;
                        while (!ok && !failed) {
                            ok = m32_entry_is(bnd[cc % kM32BndRing], cc);
                            if (!ok && ++polls > 16 * kWaveSpinLimit) {
                                failed = true;
                                atomicOr(err, 1);
                                *quit = 1;
                            }
                        }
                    }
                    __syncwarp();   // lane 0 reads the entries its neighbours validated
                    bn = bnd_p[s % kM32BndRing];
                    // chunks before this one are read: their slots may be
                    // refilled (a plain store suffices, every value read from
                    // them was consumed by arithmetic before this store issues,
                    // and a refill lands at least two chunks behind it)
                    if (lane == 0) *bnd_used = s / kM32CH;
                }
                float v[4][kM32NA];
#pragma unroll
                for (int k = 0; k < 4; k++)
#pragma unroll
                    for (int a = 0; a < kM32NA; a++) v[k][a] = vn[k][a];
                float* const p = pn;
                // next step's operands (column c+1), loaded before this step's stores
                pn = ((c + 1) & 31) ? p + cdir : cell_ptr(c + 1 < 0 ? 0 : c + 1);
                if (!check || (c + 1 >= 0 && c + 1 < ncols)) load_next(pn);
                float below = __shfl_up_sync(0xffffffffu, o[3], 1);
                const float b0 = below_in_grid ? m32_entry_value(bn) : 0.0f;
                // next step's entry (same chunk; a new chunk is read after its check)
                if (u8 + 1 != kM32CH) bn = bnd_p[(s + 1) % kM32BndRing];
                if (lane == 0) below = b0;
                if (!check || (c >= 0 && c < ncols)) {
                    float r[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        r[k] = fmaf(-v[k][2], below, fmaf(-v[k][1], o[k], v[k][0]));
                        below = r[k];
                    }
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        o[k] = r[k];
                        p[k * rstep] = r[k];
                    }
                    if (has_next && lane == 31) top_p[c % kM32TopRing] = m32_entry(c, o[3]);
                }
            }
            }
        };

        const int nsteps = ncols + 31;
        for (int t = 0; t * kM32Cols < nsteps; t++) {
            if (t < nt) wait_tile(t);
            // top ring: do not run more than half a ring ahead of the I/O warp
            if (has_next && t * kM32Cols - 31 - *top_done > kM32TopRing / 2)
                spin_ge(top_done, t * kM32Cols - 31 - kM32TopRing / 2);
            __syncwarp();
            if (t == 0 || t >= nt)
                tile_steps(t, BoolTag<true>{});
            else
                tile_steps(t, BoolTag<false>{});
            // tile t-1 is finished for every lane: hand it to the I/O warp for its
            // TMA store; the slot of tile t-2 is reused for tile t+2 once that
            // tile's store has read it
            if (t >= 1 && t - 1 < nt) {
                fence_async_smem();
                __syncwarp();
                if (lane == 0) *tiles_done = t;
            }
            if (t + 2 < nt) {
                if (t >= 2 && *tiles_freed < t - 1) spin_ge(tiles_freed, t - 1);
                __syncwarp();
                issue(t + 2);
            }
        }
        __syncwarp();
        if (lane == 0) {
            *tiles_done = nt;
            if (below_in_grid) *bnd_used = ncols / kM32CH + kM32BndChunks;
        }
        (void)failed;
    }
    cluster_sync_all();   // no CTA leaves while a neighbour may still touch its shared memory
}

// Host side: tensor maps for one FP32 array of P x NY (row pitch P floats).
int mic32_make_map(CUtensorMap* map, float* base, int P, int NY, int box_rows);

// Launches one sweep: cooperative (every strip co-resident, so the waits
// between strips always make progress) and, where the device can hold them,
// in clusters of up to 8 strips that hand rows over in shared memory.
// Advances the device-side progress base of graph-replayed sweeps by `n`
// sweeps' worth.
__global__ void k_wave_bump(unsigned long long* base, unsigned long long n) { *base += n << 24; }

// Launches one sweep: cooperative (every strip co-resident, so the waits
// between strips always make progress) and, where the device can hold them,
// in clusters of up to 8 strips that hand rows over in shared memory.
// graph_slot >= 0: for stream capture; the sweep is number graph_slot of the
// graph_sweeps sweeps of one replay, uses its own progress counters and the
// device-memory base plus graph_slot sweeps; slot 0 first advances that base
// by graph_sweeps, so that every replay gets fresh bases.
template <bool FWD>
int launch_mic32(Sim* s, const Mic32Maps& maps, float* out, const int* skip, int graph_slot = -1,
                 int graph_sweeps = 0) {
    const bool graph = graph_slot >= 0;
    const int nstrips = (s->NY + kM32Rows - 1) / kM32Rows;
    if (nstrips > s->progress_cap) {
        set_error("mic32: %d strips exceed the %d progress counters", nstrips, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    static std::atomic<unsigned long long> configured{0};
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)mic32_kernel<FWD>, (int)kM32Smem)) return rc0;
    unsigned long long base = 0;
    const unsigned long long* base_dev = nullptr;
    unsigned long long* progress = s->progress;
    if (graph) {
        if (graph_slot == 0) FS2D_LAUNCH(s, k_wave_bump, 1, 1, 0, s->m32_gbase, (unsigned long long)graph_sweeps);
        base = (unsigned long long)graph_slot << 24;
        base_dev = s->m32_gbase;
        progress = s->m32_gprogress;
    } else {
        base = wave_begin(s);
    }
    int P = s->P, NY = s->NY;
    void* args[] = {(void*)&maps, (void*)&out, (void*)&P, (void*)&NY, (void*)&progress, (void*)&base,
                    (void*)&base_dev, (void*)&s->err, (void*)&skip};
    s->launches++;
    const char* name = FWD ? "mic32_forward" : "mic32_backward";
    long long kt = ktimer_begin(s, name);
    int& cs = s->m32_cluster;   // 0: not chosen yet
    if (cs == 0) cs = choose_cluster((const void*)mic32_kernel<FWD>, nstrips, 64, kM32Smem);
    cudaError_t e = launch_clustered((const void*)mic32_kernel<FWD>, nstrips, cs, 64, kM32Smem, s->stream, args);
    if (e != cudaSuccess && cs > 1 && !graph) {   // clusters refused: plain cooperative launch
        (void)cudaGetLastError();
        cs = 1;
        e = launch_clustered((const void*)mic32_kernel<FWD>, nstrips, 1, 64, kM32Smem, s->stream, args);
    }
    int rc = check_cuda(e, name);
    ktimer_end(s, kt);
    return rc;
}

}  // namespace fs2d
