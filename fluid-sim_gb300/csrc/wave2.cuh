// wave2.cuh — staged strip wavefront for Gauss-Seidel-ordered recurrences.
//
// A recurrence out(i,j) = F(operands(i,j), out(i-sx,j), out(i,j-sy)) visited
// in the reference's loop order (rows in order of sy, columns in order of
// sx) is computed exactly when every cell runs after its two upwind
// neighbours; cells on one anti-diagonal are independent.  Layout of the
// work:
//   * a warp owns a strip of 32 rows (lane l: row 32*strip + l in sweep
//     order) and visits column c = s - l at step s, so the warp is a
//     diagonal front; out(i-sx, j) stays in the lane's register and
//     out(i, j-sy) arrives from lane l-1 by shuffle;
//   * the operands of each 32x32 tile are staged into shared memory with
//     cp.async one tile ahead (a ring of three tiles per warp) and the 32
//     steps of a tile are unrolled, so the critical path is shuffle +
//     arithmetic + shared-memory reads;
//   * W warps share a CTA; warp w's lane 31 hands its row to warp w+1 through
//     a shared-memory ring and a shared progress counter;
//   * the CTA's last warp publishes its row to the next CTA through global
//     memory (the output array plus a release/acquire progress counter);
//     warp 0 of the next CTA copies that row into shared memory in chunks of
//     CH columns, two chunks ahead of use, through registers and L2-only
//     loads (ld.global.cg), so the L2 round trip stays off the critical path.
// Every wait is bounded (wave_spin(err) polls, times a fixed factor): on
// timeout bit 0 of *err is set and the kernel carries on without the value
// (the result is then invalid, nothing hangs).  CTAs are co-resident
// (cooperative launch).
//
// Op interface:
//   typedef T;  static constexpr int NA;   operand element type and count
//   const T* in[NA];  T* out;  int pitch;  operand / output arrays, row pitch
//   __device__ T border(int i, int j) const     out() of a cell outside the sweep
//   __device__ T compute(const T* v, T left, T below, int i, int j) const
//              v[a] = in[a][j*pitch+i]; returns out(i,j), the value carried on
//   __device__ T stored(const T* v, T result) const  what is written to out[]
#pragma once

#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kW2Tile = 32;
constexpr int kW2Ring = 3;
constexpr int kW2EdgeRing = 1024;   // intra-CTA hand-off ring, columns
constexpr int kW2Publish = 8;       // columns per progress publication

__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}

template <typename T>
__device__ __forceinline__ T ldcg_t(const T* p) { return __ldcg(p); }

template <typename T>
__device__ __forceinline__ T shfl_up_t(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }

template <class Op>
__host__ __device__ constexpr size_t wave2_smem_per_warp() {
    return (size_t)kW2Ring * Op::NA * kW2Tile * kW2Tile * sizeof(typename Op::T);
}
template <class Op, int W, int CH>
__host__ __device__ constexpr size_t wave2_smem_bytes() {
    // staged tiles | boundary ring (4 chunks) | edge rings (W-1) | counters
    return W * wave2_smem_per_warp<Op>() + 4 * CH * sizeof(typename Op::T) +
           (size_t)(W > 1 ? W - 1 : 0) * kW2EdgeRing * sizeof(typename Op::T) + 2 * 32 * sizeof(int);
}

// Busy-wait on a shared-memory counter (no sleep: a consumer that slept
// past the moment its data arrived would fall further behind at every chunk).
__device__ __forceinline__ bool spin_until_smem(volatile int* flag, int need, int* err, long long spin) {
    long long polls = 0;
    while (*flag < need) {
        if (++polls > 64 * spin || ((polls & 1023) == 0 && wave_failed(err))) {
            atomicOr(err, kWaitWarp | (kWaveKindWave2 << 4));
            return false;
        }
    }
    return true;
}

template <class Op, int W, int CH>
__global__ void __launch_bounds__(32 * W) wave2_kernel(Op op, WaveGeom g, unsigned long long* progress,
                                                       unsigned long long base_host,
                                                       const unsigned long long* base_dev, int* err,
                                                       const int* skip) {
    // progress values of this launch are base + columns (base_dev: a
    // graph-replayed launch, its base advanced by the kernel before it)
    const unsigned long long base = base_dev != nullptr ? *base_dev + base_host : base_host;
    typedef typename Op::T T;
    constexpr int NA = Op::NA;
    constexpr int RC = kW2Ring * kW2Tile;  // ring columns per row
    static_assert(kW2Tile % CH == 0 && kW2Publish % CH == 0 || CH % kW2Publish == 0, "chunking");
    if (skip != nullptr && *skip) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int ncols = g.i_hi - g.i_lo + 1;
    const int nrows = g.j_hi - g.j_lo + 1;
    const int nstrips = (nrows + 31) / 32;
    const int strip = blockIdx.x * W + w;
    const bool strip_live = strip < nstrips;
    const bool last_in_cta = (w == W - 1) || (strip + 1 >= nstrips);

    // shared layout: per warp [NA][32 rows][RC ring columns] | bnd [4*CH] | edges [W-1][ring] | counters
    T* ring = reinterpret_cast<T*>(smem_raw) + (size_t)w * NA * 32 * RC;
    T* bnd = reinterpret_cast<T*>(smem_raw + W * wave2_smem_per_warp<Op>());
    T* edges = bnd + 4 * CH;
    volatile int* eprog = reinterpret_cast<volatile int*>(edges + (size_t)(W > 1 ? W - 1 : 0) * kW2EdgeRing);
    volatile int* eread = eprog + 32;
    if (threadIdx.x < 32) {
        eprog[threadIdx.x] = 0;
        eread[threadIdx.x] = 0;
    }
    __syncthreads();
    if (!strip_live) return;

    const int row = strip * 32 + lane;
    const bool valid = row < nrows;
    const int j = g.sy > 0 ? g.j_lo + row : g.j_hi - row;
    const int jbelow0 = g.sy > 0 ? g.j_lo + strip * 32 - 1 : g.j_hi - strip * 32 + 1;  // row below lane 0
    const int sx = g.sx;
    auto col = [&](int c) { return sx > 0 ? g.i_lo + c : g.i_hi - c; };
    T* const out_row = op.out + (size_t)(valid ? j : jbelow0 + g.sy) * op.pitch;

    const bool from_edge = (w > 0);
    const bool from_global = (w == 0) && (strip > 0);
    const unsigned long long* gprev = from_global ? progress + (blockIdx.x - 1) : nullptr;
    const T* edge_in = from_edge ? edges + (size_t)(w - 1) * kW2EdgeRing : nullptr;
    T* edge_out = (!last_in_cta) ? edges + (size_t)w * kW2EdgeRing : nullptr;
    // the CTA's last warp hands its row to the next CTA (unless the test hook
    // holds this CTA's hand-off back)
    const bool publish_global =
        last_in_cta && (strip + 1 < nstrips) && !wave_held(err, kWaveKindWave2, (int)blockIdx.x);
    const long long spin = wave_spin(err);

    // ---- staging: tile t (32 columns) -> ring columns (t%3)*32 .. +31 ----
    auto issue_tile = [&](int t) {
        const int c = t * kW2Tile + lane;
        if (c < ncols) {
            const int i = col(c);
            const int rc = (t % kW2Ring) * kW2Tile + lane;
            const int rows_here = min(32, nrows - strip * 32);
            for (int r = 0; r < rows_here; r++) {
                const int jr = g.sy > 0 ? g.j_lo + strip * 32 + r : g.j_hi - (strip * 32 + r);
                const size_t off = (size_t)jr * op.pitch + i;
#pragma unroll
                for (int a = 0; a < NA; a++) {
                    T* dst = ring + ((size_t)a * 32 + r) * RC + rc;
                    if (sizeof(T) == 8) cp_async8(dst, op.in[a] + off);
                    else cp_async4(dst, op.in[a] + off);
                }
            }
        }
        cp_async_commit();
    };

    // ---- lane 0's below row for warp 0: chunks of CH columns ----
    unsigned long long gavail = 0;
    auto gwait = [&](int cols_needed) {
        if (!from_global) return;
        unsigned long long need = base + (unsigned long long)min(cols_needed, ncols);
        if (gavail >= need) return;
        if (lane == 0) {
            long long polls = 0;
            unsigned long long v;
            while ((v = ld_acquire(gprev)) < need) {
                if (++polls > 16 * spin || ((polls & 255) == 0 && wave_failed(err))) {
                    atomicOr(err, kWaitStrip | (kWaveKindWave2 << 4));
                    v = need;
                    break;
                }
            }
            gavail = v;
        }
        gavail = __shfl_sync(0xffffffffu, gavail, 0);
    };
    auto load_chunk = [&](int h) -> T {  // lanes < CH: column h*CH + lane of the row below lane 0
        T v = T(0);
        const int c = h * CH + lane;
        if (lane < CH && c < ncols) {
            const int i = col(c);
            if (from_global) v = ldcg_t(op.out + (size_t)jbelow0 * op.pitch + i);
            else v = op.border(i, jbelow0);
        }
        return v;
    };
    // invariant at the start of chunk h: chunk h is in bnd (slot h&3), breg
    // holds chunk h+1 (loaded one chunk earlier, so its latency is hidden)
    T breg = T(0);
    const int nchunks = (ncols + CH - 1) / CH;
    if (!from_edge) {
        gwait(CH);
        T v = load_chunk(0);
        if (lane < CH) bnd[lane] = v;
        if (1 < nchunks) {
            gwait(2 * CH);
            breg = load_chunk(1);
        }
    }
    __syncwarp();

    issue_tile(0);
    issue_tile(1);

    T out = T(0);
    int edge_avail = 0;
    int p = (RC - lane) % RC;          // ring position of this lane's column c = s - lane
    int i_cur = col(-lane);            // memory column of c (valid once c >= 0)
    const int ntiles = (ncols + kW2Tile - 1) / kW2Tile;
    const int nsteps = ncols + 31;

    // Lane 0's row-below value of column cc, from the edge ring (warps > 0)
    // or the boundary chunks (warp 0).  Readable once the hand-off for cc's
    // chunk was done (see `handoff`).
    auto below_src = [&](int cc) -> T {
        return from_edge ? edge_in[cc & (kW2EdgeRing - 1)] : bnd[((cc / CH) & 3) * CH + (cc % CH)];
    };
    // Hand-off for the chunk starting at column s0 (warp-uniform): make
    // columns s0 .. s0+CH of the row below readable.
    auto handoff = [&](int s0) {
        const int h = s0 / CH;
        if (from_edge) {
            // two chunks of slack: in steady state the consumer never catches up
            const int need = min(s0 + 2 * CH, ncols);
            if (edge_avail < need) {
                if (lane == 0) spin_until_smem(eprog + (w - 1), need, err, spin);
                __syncwarp();
                __threadfence_block();
                edge_avail = need;
            }
            if (lane == 0) eread[w] = s0;
        } else {
            if (lane < CH && h + 1 < nchunks) bnd[((h + 1) & 3) * CH + lane] = breg;
            if (h + 2 < nchunks) {
                gwait((h + 4) * CH);
                breg = load_chunk(h + 2);
            }
            __syncwarp();
        }
    };
    handoff(0);

    // operands of the next step, loaded one step ahead (software pipeline)
    T vn[NA];
    T bn;

    // one step; CHECK: guard lanes outside [0, ncols) (first and last tiles)
    auto step = [&](const int s, const int u, const bool check) {
        T v[NA];
#pragma unroll
        for (int a = 0; a < NA; a++) v[a] = vn[a];
        const T b0 = bn;
        const int pn = (p + 1 == RC) ? 0 : p + 1;
#pragma unroll
        for (int a = 0; a < NA; a++) vn[a] = ring[((size_t)a * 32 + lane) * RC + pn];
        bn = below_src(s + 1);
        T below = shfl_up_t(out);
        if (lane == 0) below = b0;
        const int c = s - lane;
        if (!check || (valid && c >= 0 && c < ncols)) {
            const T left = (!check || c > 0) ? out : op.border(i_cur - sx, j);
            out = op.compute(v, left, below, i_cur, j);
            if (valid) out_row[i_cur] = op.stored(v, out);
            if (lane == 31) {
                if (edge_out != nullptr) {
                    edge_out[c & (kW2EdgeRing - 1)] = out;
                    if ((((u + 2) & (kW2Publish - 1)) == 0) || (check && c == ncols - 1)) {
                        __threadfence_block();
                        eprog[w] = c + 1;
                        if (c + 1 - eread[w + 1] > kW2EdgeRing - 64) {
                            long long polls = 0;
                            while (c + 1 - eread[w + 1] > kW2EdgeRing - 64) {
                                if (++polls > spin || wave_failed(err)) {
                                    atomicOr(err, kWaitWarp | (kWaveKindWave2 << 4));
                                    break;
                                }
                                __nanosleep(20);
                            }
                        }
                    }
                } else if (publish_global &&
                           ((((u + 2) & (kW2Publish - 1)) == 0) || (check && c == ncols - 1))) {
                    st_release(progress + blockIdx.x, base + (unsigned long long)(c + 1));
                }
            }
        }
        p = pn;
        i_cur += sx;
        // hand-off for the next chunk before its first column is prefetched
        if (((u + 1) % CH) == 0 && s + 1 < ncols) {
            handoff(s + 1);
            bn = below_src(s + 1);
        }
    };

    int t = 0;
    for (; t * kW2Tile < nsteps; t++) {
        cp_async_wait<1>();   // tile t staged (tile t-1 still in the ring)
        __syncwarp();
        // prime the pipeline with this step's operands
#pragma unroll
        for (int a = 0; a < NA; a++) vn[a] = ring[((size_t)a * 32 + lane) * RC + p];
        bn = below_src(t * kW2Tile);
        const bool full = t >= 1 && (t * kW2Tile + kW2Tile - 1) < ncols;
        if (full) {
#pragma unroll
            for (int u = 0; u < kW2Tile; u++) step(t * kW2Tile + u, u, false);
        } else {
#pragma unroll
            for (int u = 0; u < kW2Tile; u++) step(t * kW2Tile + u, u, true);
        }
        // stage tile t+2 into the ring slot of tile t-1 (no lane reads it any more)
        __syncwarp();
        if (t + 2 < ntiles) issue_tile(t + 2);
        else cp_async_commit();
    }
    cp_async_wait<0>();
}

// Advances the device base of graph-replayed sweeps by one sweep's worth
// (progress values are base + columns, columns < 2^24).
static __global__ void k_wave2_bump(unsigned long long* base) { *base += 1ull << 24; }

// Cooperative launch of the staged wavefront; W warps per CTA.
template <class Op, int W, int CH>
int launch_wave2(Sim* s, const Op& op, WaveGeom g, const int* skip) {
    const int nrows = g.j_hi - g.j_lo + 1;
    const int ncols = g.i_hi - g.i_lo + 1;
    if (nrows <= 0 || ncols <= 0) return 0;
    const int nstrips = (nrows + 31) / 32;
    const int nctas = (nstrips + W - 1) / W;
    if (nctas > s->progress_cap) {
        set_error("wavefront: %d CTAs exceed the %d progress counters", nctas, s->progress_cap);
        return FS2D_ERR_INVALID;
    }
    constexpr size_t smem = wave2_smem_bytes<Op, W, CH>();
    static std::atomic<unsigned long long> configured{0};
    if (int rc0 = ensure_smem_attr(configured, s->device, (const void*)wave2_kernel<Op, W, CH>, (int)smem)) return rc0;
    // direct launch: a host base and the handle's progress flags; inside a
    // stream capture: the graph's flags and device base, advanced first
    unsigned long long base = s->capturing ? 0ull : wave_begin(s);
    const unsigned long long* base_dev = s->capturing ? s->gbase : nullptr;
    unsigned long long* progress = s->capturing ? s->gprogress : s->progress;
    if (s->capturing) {
        s->launches++;
        k_wave2_bump<<<1, 1, 0, s->stream>>>(s->gbase);
        if (int rc1 = check_cuda(cudaGetLastError(), "k_wave2_bump")) return rc1;
    }
    void* args[] = {(void*)&op, (void*)&g, (void*)&progress, (void*)&base, (void*)&base_dev, (void*)&s->err,
                    (void*)&skip};
    s->launches++;
    long long kt = ktimer_begin(s, Op::kName);
    int rc = check_cuda(cudaLaunchCooperativeKernel((const void*)wave2_kernel<Op, W, CH>, dim3(nctas), dim3(32 * W),
                                                    args, smem, s->stream),
                        Op::kName);
    ktimer_end(s, kt);
    return rc;
}

}  // namespace fs2d
