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
//   * strips hand their top row to the next CTA through global memory.  A
//     second warp per CTA does all of that traffic: it copies the compute
//     warp's top row from a shared ring to global memory and publishes
//     progress (st.release), and it polls the previous strip's progress and
//     brings the row below into a shared ring of chunks ahead of use.  The
//     compute warp itself only touches shared memory (and issues the TMA
//     copies), so no release or L2 round trip sits on the critical path.
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
constexpr int kM32CH = 16;      // boundary chunk (columns)
constexpr int kM32BndChunks = 8;  // ring of chunks of the row below
constexpr int kM32TopRing = 256;  // ring of the strip's top row (columns)
constexpr int kM32TileFloats = kM32Rows * kM32Cols;
constexpr unsigned kM32TileBytes = kM32TileFloats * 4;
constexpr size_t kM32Smem =
    (size_t)kM32Slots * kM32NA * kM32TileBytes + (kM32BndChunks * kM32CH + kM32TopRing) * 4 + 8 * 4 + 8 * kM32Slots;

// Tensor maps of one sweep: operands in[0..2] (in[0] is also where results
// are written in shared memory), the output, and the output with a box of
// `tail` rows (tail = NY % 128) for the backward sweep's partial strip.
struct Mic32Maps {
    CUtensorMap in[kM32NA];
    CUtensorMap out;
    CUtensorMap out_tail;
};

// FWD: out = v0 - v1*left - v2*below  (forward, on q~ = q*pc)
// BWD: same form with the backward coefficients.
// Block of 64 threads: warp 0 computes, warp 1 moves the strip boundaries
// between global and shared memory (so release/acquire round trips and L2
// latency never stall the compute warp).
template <bool FWD>
__global__ void __launch_bounds__(64) mic32_kernel(const __grid_constant__ Mic32Maps maps, float* out, int P, int NY,
                                                   unsigned long long* progress, unsigned long long base, int* err,
                                                   const int* skip) {
    if (skip != nullptr && *skip) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    float* bnd = ring + (size_t)kM32Slots * kM32NA * kM32TileFloats;   // kM32BndChunks chunks of kM32CH
    float* top = bnd + kM32BndChunks * kM32CH;                            // kM32TopRing columns
    volatile int* ctr = reinterpret_cast<volatile int*>(top + kM32TopRing);
    volatile int* bnd_ready = ctr + 0;      // chunks of the row below available in bnd
    volatile int* bnd_used = ctr + 1;       // chunk the compute warp works on
    volatile int* top_ready = ctr + 2;      // top-row columns written to `top`
    volatile int* top_done = ctr + 3;       // top-row columns copied out and published
    volatile int* quit = ctr + 4;           // compute warp gave up (timeout)
    volatile int* tiles_done = ctr + 5;     // tiles whose results are complete in shared memory
    volatile int* tiles_freed = ctr + 6;    // tiles whose TMA store has finished reading shared memory
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 8);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int strip = blockIdx.x;
    const int nstrips = (NY + kM32Rows - 1) / kM32Rows;
    const int nt = P / kM32Cols;             // tiles per row (P is a multiple of 32)
    const int ncols = P;
    const int nchunks = ncols / kM32CH;
    const int ybox = FWD ? strip * kM32Rows : NY - (strip + 1) * kM32Rows;  // first memory row of the box
    const bool has_next = strip + 1 < nstrips;
    const int ytop = FWD ? ybox + kM32Rows - 1 : ybox;       // the strip's last row in sweep order
    const int ybelow = FWD ? ybox - 1 : ybox + kM32Rows;     // the row below the strip
    const bool below_in_grid = strip > 0;
    auto mcol = [&](int c) { return FWD ? c : P - 1 - c; };  // memory column of sweep column c

    if (threadIdx.x == 0) {
        for (int k = 0; k < kM32Slots; k++) mbar_init(bars + k, 1);
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
        for (int k = threadIdx.x; k < kM32BndChunks * kM32CH; k += blockDim.x) bnd[k] = 0.0f;
    }
    __syncthreads();

    if (warp == 1) {
        // ---------------- I/O warp ----------------
        const unsigned long long* gprev = below_in_grid ? progress + (strip - 1) : nullptr;
        int hb = below_in_grid ? 0 : nchunks;    // next chunk of the row below to bring in
        int tc = 0;                              // top-row columns copied out
        const int tend = has_next ? ncols : 0;
        int ts = 0;                              // next tile to store
        unsigned long long gavail = 0;
        long long idle = 0;
        while (hb < nchunks || tc < tend || ts < nt) {
            bool moved = false;
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
            if (hb < nchunks && hb < *bnd_used + kM32BndChunks - 1) {
                const unsigned long long need = base + (unsigned long long)min((hb + 1) * kM32CH, ncols);
                if (gavail < need) {
                    unsigned long long v = 0;
                    if (lane == 0) v = ld_acquire(gprev);
                    gavail = __shfl_sync(0xffffffffu, v, 0);
                }
                if (gavail >= need) {
                    if (lane < kM32CH)
                        bnd[(hb % kM32BndChunks) * kM32CH + lane] =
                            __ldcg(out + (size_t)ybelow * P + mcol(hb * kM32CH + lane));
                    __threadfence_block();
                    __syncwarp();
                    hb++;
                    if (lane == 0) *bnd_ready = hb;
                    moved = true;
                }
            }
            if (tc < tend) {
                const int tr = *top_ready;
                if (tr > tc) {
                    __threadfence_block();  // acquire: the columns were written before top_ready
                    for (int c = tc + lane; c < tr; c += 32)
                        out[(size_t)ytop * P + mcol(c)] = top[c % kM32TopRing];
                    __threadfence();
                    __syncwarp();
                    tc = tr;
                    if (lane == 0) {
                        st_release(progress + strip, base + (unsigned long long)tc);
                        *top_done = tc;
                    }
                    moved = true;
                }
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
        return;
    }

    // ---------------- compute warp ----------------
    auto tile_x = [&](int t) { return FWD ? t * kM32Cols : P - (t + 1) * kM32Cols; };
    auto slot_ptr = [&](int t) { return ring + (size_t)(t & (kM32Slots - 1)) * kM32NA * kM32TileFloats; };
    auto issue = [&](int t) {
        if (lane == 0 && t < nt) {
            unsigned long long* bar = bars + (t & (kM32Slots - 1));
            mbar_expect_tx(bar, kM32NA * kM32TileBytes);
            float* dst = slot_ptr(t);
#pragma unroll
            for (int a = 0; a < kM32NA; a++) tma_load_2d(dst + a * kM32TileFloats, &maps.in[a], tile_x(t), ybox, bar);
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
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    float bn = 0.0f;         // lane 0's row-below value of the next step
    float vn[4][kM32NA];     // operands of the next step (loaded one step ahead)
    float* pn = nullptr;     // their address
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
            load_next(pn);   // a tile starts on a chunk boundary: bn is read there
        }
#pragma unroll
        for (int u = 0; u < kM32Cols; u++) {
            const int s = t * kM32Cols + u;
            const int c = s - lane;
            if ((s % kM32CH) == 0 && s < ncols) {   // lane 0 enters a new chunk of the row below
                const int h = s / kM32CH;
                if (*bnd_ready <= h) spin_ge(bnd_ready, h + 1);
                __threadfence_block();  // acquire: the chunk's values were written before bnd_ready
                if (lane == 0) *bnd_used = h;
                __syncwarp();
                bn = bnd[(h % kM32BndChunks) * kM32CH];
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
            const float b0 = bn;
            // next step's row-below value (same chunk; a new chunk is read at its boundary)
            if (((s + 1) % kM32CH) != 0) bn = bnd[((s / kM32CH) % kM32BndChunks) * kM32CH + ((s + 1) % kM32CH)];
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
                if (has_next && lane == 31) {
                    top[c % kM32TopRing] = o[3];
                    if ((((u + 2) & 7) == 0) || (check && c == ncols - 1)) {
                        __threadfence_block();
                        *top_ready = c + 1;
                    }
                }
            }
        }
    };

    const int nsteps = ncols + 31;
    for (int t = 0; t * kM32Cols < nsteps; t++) {
        if (t < nt) wait_tile(t);
        // top ring: do not run more than half a ring ahead of the I/O warp
        if (has_next && t * kM32Cols - 31 - *top_done > kM32TopRing / 2) spin_ge(top_done, t * kM32Cols - 31 - kM32TopRing / 2);
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
    if (lane == 0) *tiles_done = nt;
    (void)failed;
}

// Host side: tensor maps for one FP32 array of P x NY (row pitch P floats).
int mic32_make_map(CUtensorMap* map, float* base, int P, int NY, int box_rows);

template <bool FWD>
int launch_mic32(Sim* s, const Mic32Maps& maps, float* out, const int* skip) {
    const int nstrips = (s->NY + kM32Rows - 1) / kM32Rows;
    if (nstrips > s->progress_cap) {
        set_error("mic32: %d strips exceed the %d progress counters", nstrips, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    static bool configured = false;
    if (!configured) {
        int rc0 = check_cuda(cudaFuncSetAttribute((const void*)mic32_kernel<FWD>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kM32Smem),
                             "cudaFuncSetAttribute");
        if (rc0) return rc0;
        configured = true;
    }
    unsigned long long base = wave_begin(s);
    int P = s->P, NY = s->NY;
    void* args[] = {(void*)&maps, (void*)&out, (void*)&P, (void*)&NY, (void*)&s->progress, (void*)&base,
                    (void*)&s->err, (void*)&skip};
    s->launches++;
    const char* name = FWD ? "mic32_forward" : "mic32_backward";
    long long kt = ktimer_begin(s, name);
    int rc = check_cuda(cudaLaunchCooperativeKernel((const void*)mic32_kernel<FWD>, dim3(nstrips), dim3(64), args,
                                                    kM32Smem, s->stream),
                        name);
    ktimer_end(s, kt);
    return rc;
}

}  // namespace fs2d
