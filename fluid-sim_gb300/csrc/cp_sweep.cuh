// cp_sweep.cuh — closest-point fast sweeps of LevelSet::constructFromParticles
// (the fastSweepIterate lambda, src/FluidSim2D.cpp:776-791, loop order
// include/FluidSim2D.h:178-203) as a TMA-staged wavefront over the
// closest-particle index alone.
//
// The reference keeps, per cell, phi = d(t) = |particle t - corner| - dr and
// replaces (phi, t) by a neighbour's particle e when d(e) < phi, in the
// candidate order (i-1,j), (i+1,j), (i,j-1), (i,j+1).  Since phi is always
// d(t) of the cell's own t, the sweep is carried out on t only and phi is
// evaluated once afterwards (k_cp_phi).  Each comparison d(e) < d(c) is
// decided from FP32 squared distances with a rigorous error bound:
//   * positions and corner coordinates are split into float pairs (h, l)
//     with h + l = value to ~2^-48; ex = (ph - xh) + (pl - xl) then differs
//     from the exact px - xi by at most 2^-23 |ex| + 2^-45 A, where A bounds
//     every coordinate; q32 = ex^2 + ey^2 differs from the reference's FP64
//     q by at most E = 2^-20 q32 + 2^-42 A (|ex| + |ey|) + C0 (factors of 2
//     to 4 above the derived bound);
//   * q(e) >= q(c) implies d(e) >= d(c) (sqrt and the subtraction of dr round
//     monotonically), so q32(e) - E(e) >= q32(c) + E(c) means "no";
//   * q(c) - q(e) >= 2^-40 q(c) with q(c) > 2^-20 dr^2 leaves a gap between
//     the two rounded distances larger than their rounding errors
//     (sqrt(q(c)) > 2^-10 dr, so the gap 2^-41 sqrt(q(c)) exceeds the
//     2^-52 max(sqrt(q), dr) the two roundings can take), so
//     q32(e) + E(e) < q32(c) - E(c) means "yes" (the slack in E covers the
//     2^-40 margin);
//   * otherwise both squared distances are recomputed as double-float pairs
//     (two-sum of the high parts, exact products by FMA), good to
//     2^-42.4 A (|ex| + |ey|) + 2^-44 q, and the same two tests are made with
//     that bound (cp_decide_df);
//   * anything still undecided (true ties, duplicates, particles on a
//     corner, NaN or overflow) is decided exactly in FP64 with the
//     reference's expression.
// The decision is therefore always the reference's.
//
// Layout: t is pitched (row pitch P = NX rounded up to 32; padding -1).  One
// 64-thread CTA per strip of 32 rows: warp 0 computes (lane l owns row l of
// the strip and works on column s - l at step s), warp 1 moves data (tile
// stores, the strip's top row out to the next strip, the row below in).
// Tiles of 32 columns x 33 rows (the strip and the next row in sweep order)
// arrive by TMA; the float-pair position of every cell's particle is
// gathered kCpD columns ahead with cp.async into a per-lane ring.
#pragma once

#include <cuda.h>
#include "fs2d_device.cuh"
#include "tma.cuh"

namespace fs2d {

constexpr int kCpCols = 32;
constexpr int kCpBoxRows = 33;
constexpr int kCpSlots = 8;
constexpr int kCpAhead = 4;        // tiles requested ahead
constexpr int kCpD = 8;            // gather distance (columns; 16 measured no faster at 1024^2)
constexpr int kCpR = 16;           // gather ring slots per row (power of two > kCpD + 1)
// Chunk of the row below (columns per arrival check): smaller chunks shorten
// the strip-to-strip lag (measured at 1024^2: 16 and 8 columns gave 9.8 and
// 8.9 ms of sweeps per frame, 4 columns no better than 8).
constexpr int kCpCH = 8;
// steps per unrolled body of a tile's step loop: one chunk of the row below
// for a scene per launch (the chunk check then falls on the body's first
// step); half of that in the persistent launches over many small scenes
template <bool SEVERAL>
__host__ __device__ constexpr int cp_unroll() { return SEVERAL ? kCpCH / 2 : kCpCH; }
constexpr int kCpBndChunks = 128 / kCpCH;
constexpr int kCpTopRing = 256;
constexpr int kCpTileInts = kCpBoxRows * kCpCols;
constexpr unsigned kCpTileBytes = kCpTileInts * 4;
constexpr size_t kCpSmem = (size_t)kCpSlots * kCpTileBytes + 33 * kCpR * 16 + kCpBndChunks * kCpCH * (16 + 4) +
                           kCpTopRing * (16 + 4) + 16 * 4 + kCpSlots * 8;

struct CpMaps {
    CUtensorMap ld;       // box 32 x 33 (load)
    CUtensorMap st;       // box 32 x 32 (store of a full strip)
    CUtensorMap st_tail;  // box 32 x (NY % 32) (store of the partial strip of a downward sweep)
};

// d = |particle - cell corner (i dx, j dx)| - dr  (src/FluidSim2D.cpp:768,785)
__device__ __forceinline__ double corner_dist(double2 p, int i, int j, double dx, double dr) {
    double ax = p.x - i * dx, ay = p.y - j * dx;
    return sqrt(ax * ax + ay * ay) - dr;
}

// Current choice of a cell: particle t (-1 none), its float-pair position,
// FP32 squared distance q and error bound E.
struct CpCur {
    int t;
    float4 p;
    float q, E;
};

__device__ __forceinline__ void cp_q32(float4 p, float2 xc, float2 yc, const CpConst& k, float& q, float& E) {
    const float ax = __fadd_rn(__fsub_rn(p.x, xc.x), __fsub_rn(p.y, xc.y));
    const float ay = __fadd_rn(__fsub_rn(p.z, yc.x), __fsub_rn(p.w, yc.y));
    q = __fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay));
    E = __fadd_rn(__fadd_rn(__fmul_rn(0x1p-20f, q), __fmul_rn(k.A42, __fadd_rn(fabsf(ax), fabsf(ay)))), k.C0);
}

// d(e) < d(c), evaluated as the reference does (c < 0: the cell's HUGE_VAL).
__device__ __noinline__ bool cp_exact_less(const double2* __restrict__ pos, int e, int c, int i, int j, double dx,
                                           double dr) {
    const double dc = c < 0 ? HUGE_VAL : corner_dist(pos[c], i, j, dx, dr);
    return corner_dist(pos[e], i, j, dx, dr) < dc;
}

// Double-float squared distance q = qh + ql (not normalised) and the bound
// of its error against the reference's FP64 value.
__device__ __forceinline__ void cp_qdf(float4 p, float2 xc, float2 yc, const CpConst& k, float& qh, float& ql,
                                       float& E) {
    // ex = (ph - xh) + (pl - xl): two-sum of the high parts, the rest in the low part
    const float sx = __fsub_rn(p.x, xc.x);
    const float bx = __fsub_rn(sx, p.x);
    const float ex_err = __fadd_rn(__fsub_rn(p.x, __fsub_rn(sx, bx)), __fsub_rn(__fsub_rn(0.f, xc.x), bx));
    const float exl = __fadd_rn(ex_err, __fsub_rn(p.y, xc.y));
    const float sy = __fsub_rn(p.z, yc.x);
    const float by = __fsub_rn(sy, p.z);
    const float ey_err = __fadd_rn(__fsub_rn(p.z, __fsub_rn(sy, by)), __fsub_rn(__fsub_rn(0.f, yc.x), by));
    const float eyl = __fadd_rn(ey_err, __fsub_rn(p.w, yc.y));
    // squares: exact product of the high parts (FMA), cross and low terms in FP32
    const float px = __fmul_rn(sx, sx);
    const float pxe = __fmaf_rn(sx, sx, -px);
    const float py = __fmul_rn(sy, sy);
    const float pye = __fmaf_rn(sy, sy, -py);
    const float cx = __fmaf_rn(__fmul_rn(2.f, sx), exl, __fmul_rn(exl, exl));
    const float cy = __fmaf_rn(__fmul_rn(2.f, sy), eyl, __fmul_rn(eyl, eyl));
    // qh + ql = px + py (two-sum) + the low terms
    qh = __fadd_rn(px, py);
    const float bq = __fsub_rn(qh, px);
    const float q_err = __fadd_rn(__fsub_rn(px, __fsub_rn(qh, bq)), __fsub_rn(py, bq));
    ql = __fadd_rn(__fadd_rn(q_err, __fadd_rn(pxe, pye)), __fadd_rn(cx, cy));
    // |q - q_ref| <= 2^-44 q + 2^-42.4 A (|ex| + |ey|) + 2^-89 A^2: E doubles the
    // first two terms
    E = __fadd_rn(__fadd_rn(__fmul_rn(0x1p-42f, qh), __fmul_rn(__fmul_rn(k.A42, 2.f), __fadd_rn(fabsf(sx), fabsf(sy)))),
                  k.C0);
}

// Decision from double-float distances: 1 yes, 0 no, -1 undecided.
__device__ __noinline__ int cp_decide_df(float4 pe, float4 pc, float2 xc, float2 yc, const CpConst& k) {
    float eh, el, Ee, ch, cl, Ec;
    cp_qdf(pe, xc, yc, k, eh, el, Ee);
    cp_qdf(pc, xc, yc, k, ch, cl, Ec);
    // D = q(c) - q(e); the high difference is exact when the two are close
    const float D = __fadd_rn(__fsub_rn(ch, eh), __fsub_rn(cl, el));
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(2.f, __fadd_rn(Ee, Ec)), __fmul_rn(0x1p-40f, ch)),
                              __fmul_rn(0x1p-22f, fabsf(D)));
    if (!(D == D) || !(T <= 3.0e38f)) return -1;
    if (D <= -T) return 0;
    if (D >= __fadd_rn(T, __fmul_rn(0x1p-38f, ch)) && ch > k.tiny_q) return 1;
    return -1;
}

// One candidate of the reference's loop: neighbour particle e (ok: the
// neighbour lies inside the grid) replaces the current choice iff d(e) < d(cur).
__device__ __forceinline__ void cp_offer(int e, float4 pe, bool ok, CpCur& cur, float2 xc, float2 yc,
                                         const CpConst& k, const double2* __restrict__ pos, int i, int j, double dx,
                                         double dr) {
    if (!ok || e < 0 || e == cur.t) return;
    float q, E;
    cp_q32(pe, xc, yc, k, q, E);
    bool win;
    if (!k.fast) {
        win = cp_exact_less(pos, e, cur.t, i, j, dx, dr);
    } else if (cur.t < 0) {
        // a finite q32 means a finite d(e), below the cell's HUGE_VAL
        win = (q <= 3.0e38f) ? true : cp_exact_less(pos, e, cur.t, i, j, dx, dr);
    } else if (__fsub_rn(q, E) >= __fadd_rn(cur.q, cur.E)) {
        win = false;
    } else if (__fadd_rn(q, E) < __fsub_rn(cur.q, cur.E) && cur.q > k.tiny_q) {
        win = true;
    } else {
        const int dd = cp_decide_df(pe, cur.p, xc, yc, k);
        win = dd >= 0 ? dd == 1 : cp_exact_less(pos, e, cur.t, i, j, dx, dr);
    }
    if (win) {
        cur.t = e;
        cur.p = pe;
        cur.q = q;
        cur.E = E;
    }
}

// Branch-free FP32 test of one candidate.  Sets `und` when the bound cannot
// decide (the cell is then redone by cp_cell_slow); the choice it leaves is
// only meaningful while `und` is clear.
__device__ __forceinline__ void cp_offer_fast(int e, float4 pe, bool ok, CpCur& cur, float2 xc, float2 yc,
                                              const CpConst& k, bool& und) {
    float q, E;
    cp_q32(pe, xc, yc, k, q, E);
    const bool cand = ok && e >= 0 && e != cur.t;
    const bool lose = __fsub_rn(q, E) >= __fadd_rn(cur.q, cur.E);
    const bool win = cur.t < 0 ? (q <= 3.0e38f) : (__fadd_rn(q, E) < __fsub_rn(cur.q, cur.E) && cur.q > k.tiny_q);
    und |= cand && (!k.fast || (cur.t >= 0 && !lose && !win) || (cur.t < 0 && !win));
    const bool take = cand && win && (cur.t < 0 || !lose);
    cur.t = take ? e : cur.t;
    cur.p = take ? pe : cur.p;
    cur.q = take ? q : cur.q;
    cur.E = take ? E : cur.E;
}

// The whole candidate sequence of one cell with the tiered decision (rare).
__device__ __noinline__ int cp_cell_slow(int own, float4 own_p, int e0, float4 p0, bool ok0, int e1, float4 p1,
                                         bool ok1, int e2, float4 p2, bool ok2, int e3, float4 p3, bool ok3,
                                         float2 xc, float2 yc, const CpConst& k, const double2* __restrict__ pos,
                                         int i, int j, double dx, double dr, float4* out_p) {
    CpCur cur;
    cur.t = own;
    cur.p = own_p;
    cur.q = cur.E = 0.f;
    if (own >= 0) cp_q32(own_p, xc, yc, k, cur.q, cur.E);
    cp_offer(e0, p0, ok0, cur, xc, yc, k, pos, i, j, dx, dr);
    cp_offer(e1, p1, ok1, cur, xc, yc, k, pos, i, j, dx, dr);
    cp_offer(e2, p2, ok2, cur, xc, yc, k, pos, i, j, dx, dr);
    cp_offer(e3, p3, ok3, cur, xc, yc, k, pos, i, j, dx, dr);
    *out_p = cur.p;
    return cur.t;
}

__device__ __forceinline__ float4 shfl_up_f4(float4 v) {
    v.x = __shfl_up_sync(0xffffffffu, v.x, 1);
    v.y = __shfl_up_sync(0xffffffffu, v.y, 1);
    v.z = __shfl_up_sync(0xffffffffu, v.z, 1);
    v.w = __shfl_up_sync(0xffffffffu, v.w, 1);
    return v;
}

struct CpArgs {
    const float4* pos_df;   // float-pair positions (xh, xl, yh, yl)
    const double2* pos;     // positions (exact decisions)
    const float2* xtab;     // float-pair corner x coordinate of column i, P entries
    const float2* ytab;     // of row j, NY entries
    const CpConst* kc;
    int* hb_t;              // strip hand-off rows: [strip][sweep column]
    float4* hb_p;
    unsigned long long* progress;
    unsigned long long base;
    int* err;
    const int* skip;
    int np, NX, NY, P;
    double dx, dr;
};

// One scene of a launch over several scenes: its tensor maps and arguments
// (progress, base, err and skip come from the launch's WaveWork).
struct CpScene {   // aligned as CUtensorMap
    CpMaps maps;
    CpArgs a;
};

// Sweep direction (SX, SY): columns visited in +x (SX > 0) or -x order, rows
// in +y or -y order.  SEVERAL = false: one scene, CTA b = strip b.
// SEVERAL = true: persistent CTAs over w's work items (see WaveWork).
template <int SX, int SY, bool SEVERAL>
__global__ void __launch_bounds__(64) cp_sweep_kernel(const __grid_constant__ CpMaps maps1, const CpArgs a1,
                                                      const WaveWork w) {
    if (!SEVERAL && a1.skip != nullptr && *a1.skip) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    int* tiles = reinterpret_cast<int*>(smem_raw);
    float4* gring = reinterpret_cast<float4*>(smem_raw + (size_t)kCpSlots * kCpTileBytes);  // [33][kCpR]
    float4* bnd_p = gring + 33 * kCpR;
    int* bnd_t = reinterpret_cast<int*>(bnd_p + kCpBndChunks * kCpCH);
    float4* top_p = reinterpret_cast<float4*>(bnd_t + kCpBndChunks * kCpCH);
    int* top_t = reinterpret_cast<int*>(top_p + kCpTopRing);
    volatile int* ctr = reinterpret_cast<volatile int*>(top_t + kCpTopRing);
    volatile int* bnd_ready = ctr + 0;
    volatile int* bnd_used = ctr + 1;
    volatile int* top_ready = ctr + 2;
    volatile int* top_done = ctr + 3;
    volatile int* quit = ctr + 4;
    volatile int* tiles_done = ctr + 5;
    volatile int* tiles_freed = ctr + 6;
    volatile int* cur_item = ctr + 7;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(const_cast<int*>(ctr) + 16);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;

  // One strip of one scene (the whole grid of a launch per scene, or one
  // work item of a launch over several scenes).
  constexpr int kCpUnroll = cp_unroll<SEVERAL>();
  auto run_strip = [&](const CpMaps& maps, const CpArgs& a, const int strip) {
    const int NX = a.NX, NY = a.NY, P = a.P;
    const int nstrips = (NY + 31) / 32;
    const int nt = P / kCpCols;
    const int nchunks = P / kCpCH;
    const bool has_next = strip + 1 < nstrips;
    // this strip hands its top row to the next one (unless the test hook holds it back)
    const bool publishes = has_next && !wave_held(a.err, kWaveKindCp, strip);
    const long long spin = wave_spin(a.err);
    const bool below_in_grid = strip > 0;
    const int y0 = SY > 0 ? 32 * strip : NY - 33 - 32 * strip;   // memory row of box row 0

    if (threadIdx.x == 0) {
        for (int k = 0; k < kCpSlots; k++) mbar_init(bars + k, 1);
        fence_mbar_init();
        *bnd_ready = below_in_grid ? 0 : nchunks;
        *bnd_used = 0;
        *top_ready = 0;
        *top_done = 0;
        *quit = 0;
        *tiles_done = 0;
        *tiles_freed = 0;
    }
    // the row below starts as "no particle" in every strip: the first strip
    // keeps it (the reference's border), the others overwrite it with the
    // previous strip's row; a strip whose wait gave up reads -1, never a
    // stale shared-memory word, so every index it stores stays a particle
    // index or -1
    for (int k = threadIdx.x; k < kCpBndChunks * kCpCH; k += blockDim.x) {
        bnd_t[k] = -1;
        bnd_p[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();

    if (warp == 1) {
        // ---------------- I/O warp ----------------
        const unsigned long long* gprev = below_in_grid ? a.progress + (strip - 1) : nullptr;
        int hbk = below_in_grid ? 0 : nchunks;
        int tc = 0;
        const int tend = publishes ? P : 0;
        int ts = 0;
        unsigned long long gavail = 0;
        long long idle = 0;
        while (hbk < nchunks || tc < tend || ts < nt) {
            bool moved = false;
            if (ts < nt && *tiles_done > ts) {
                if (lane == 0) {
                    const int* src = tiles + (size_t)(ts % kCpSlots) * kCpTileInts;
                    const int x = SX > 0 ? ts * kCpCols : P - (ts + 1) * kCpCols;
                    if (SY > 0) {
                        tma_store_2d(&maps.st, x, 32 * strip, src);
                    } else if (y0 + 1 >= 0) {
                        tma_store_2d(&maps.st, x, y0 + 1, src + kCpCols);
                    } else {
                        const int tail = NY - 32 * strip;
                        tma_store_2d(&maps.st_tail, x, 0, src + (kCpBoxRows - tail) * kCpCols);
                    }
                    bulk_commit();
                    // no wait for this store's own read: once every store but the
                    // newest has read its tile, tiles < ts are free (the compute
                    // warp reuses a slot kCpSlots tiles later)
                    bulk_wait_read<1>();
                    *tiles_freed = ts;
                }
                __syncwarp();
                ts++;
                moved = true;
            }
            if (hbk < nchunks && hbk < *bnd_used + kCpBndChunks - 1) {
                const unsigned long long need = a.base + (unsigned long long)min((hbk + 1) * kCpCH, P);
                if (gavail < need) {
                    unsigned long long v = 0;
                    if (lane == 0) v = ld_acquire(gprev);
                    gavail = __shfl_sync(0xffffffffu, v, 0);
                }
                if (gavail >= need) {
                    if (lane < kCpCH) {
                        const int c = hbk * kCpCH + lane;
                        const int slot = (hbk % kCpBndChunks) * kCpCH + lane;
                        const size_t g = (size_t)(strip - 1) * P + c;
                        bnd_t[slot] = __ldcg(a.hb_t + g);
                        bnd_p[slot] = __ldcg(a.hb_p + g);
                    }
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
                    __threadfence_block();  // acquire: the columns were written before top_ready
                    for (int c = tc + lane; c < tr; c += 32) {
                        const size_t g = (size_t)strip * P + c;
                        a.hb_t[g] = top_t[c % kCpTopRing];
                        a.hb_p[g] = top_p[c % kCpTopRing];
                    }
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
            } else if (++idle > 16 * spin || *quit || ((idle & 1023) == 0 && wave_failed(a.err))) {
                if (lane == 0) {
                    atomicOr(a.err, kWaitStrip | (kWaveKindCp << 4));
                    *quit = 1;
                }
                break;
            }
        }
        if (lane == 0) bulk_wait_all();
        __syncwarp();
        return;
    }

    // ---------------- compute warp ----------------
    const CpConst kc = *a.kc;
    const bool rowvalid = 32 * strip + lane < NY;
    const int j = SY > 0 ? 32 * strip + lane : NY - 1 - 32 * strip - lane;
    const int brow = SY > 0 ? lane : 32 - lane;          // box row of the lane's row
    const int urow = SY > 0 ? lane + 1 : 31 - lane;      // box row of the next row in sweep order
    const float2 yc = rowvalid ? a.ytab[j] : make_float2(0.f, 0.f);
    auto tile_x = [&](int t) { return SX > 0 ? t * kCpCols : P - (t + 1) * kCpCols; };
    auto tile_base = [&](int t) { return tiles + (size_t)(t % kCpSlots) * kCpTileInts; };
    auto at = [&](int c, int r) -> int& {   // element (sweep column c >= 0, box row r)
        const int bc = SX > 0 ? (c & 31) : 31 - (c & 31);
        return tile_base(c >> 5)[r * kCpCols + bc];
    };
    // Tiles keep being loaded after a failed wait (the loads complete on
    // their own and are all waited for below): every slot then holds indices
    // read from t, so whatever this strip computes stays a particle index or
    // -1, never a stale shared-memory word.
    auto issue = [&](int t) {
        if (lane == 0 && t < nt) {
            unsigned long long* bar = bars + (t % kCpSlots);
            mbar_expect_tx(bar, kCpTileBytes);
            tma_load_2d(tile_base(t), &maps.ld, tile_x(t), y0, bar);
        }
    };
    bool failed = false;
    auto wait_tile = [&](int t) {
        unsigned long long* bar = bars + (t % kCpSlots);
        const unsigned parity = (unsigned)((t / kCpSlots) & 1);
        long long polls = 0;
        while (!mbar_try_wait(bar, parity)) {
            if (++polls > kWaveSpinLimit) {
                failed = true;
                atomicOr(a.err, kWaitTile | (kWaveKindCp << 4));
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
                atomicOr(a.err, kWaitWarp | (kWaveKindCp << 4));
                *quit = 1;
                return;
            }
        }
    };
    // gathers of step s: the particle position of column s - lane + kCpD of
    // the lane's row (lane 31 also of the row above the strip)
    // (every lane copies, zero-filled where its cell has no particle or lies
    // outside the strip, so that no branch surrounds the gather; a ring slot
    // is only read for a cell with a particle)
    auto gather = [&](int s) {
        const int g = s - lane + kCpD;
        const bool in = rowvalid && g >= 0 && g < P;
        const int e = at(in ? g : 0, brow);   // a word of the tile ring either way
        const bool has = in && e >= 0 && e < a.np;
        cp_async16_zfill(gring + lane * kCpR + (g & (kCpR - 1)), a.pos_df + (has ? e : 0), has ? 16u : 0u);
        if (in) {
            if (lane == 31) {
                const int e2 = at(g, urow);
                if (e2 >= 0 && e2 < a.np) cp_async16(gring + 32 * kCpR + (g & (kCpR - 1)), a.pos_df + e2);
            }
        }
        cp_async_commit();
    };

    for (int t = 0; t < kCpAhead; t++) issue(t);
    wait_tile(0);
    __syncwarp();
    for (int v = -kCpD; v < 0; v++) gather(v);

    int o_t = -1;                                  // output of the previous step (the left candidate)
    float4 o_p = make_float4(0.f, 0.f, 0.f, 0.f);

    auto tile_steps = [&](int t, auto check_tag) {
        constexpr bool check = decltype(check_tag)::value;
#pragma unroll kCpUnroll
        for (int u = 0; u < kCpCols; u++) {
            const int s = t * kCpCols + u;
            const int c = s - lane;
            if ((s % kCpCH) == 0 && s < P) {   // lane 0 enters a new chunk of the row below
                const int h = s / kCpCH;
                if (*bnd_ready <= h) spin_ge(bnd_ready, h + 1);
                __threadfence_block();
                if (lane == 0) *bnd_used = h;
                __syncwarp();
            }
            gather(s);
            cp_async_wait<kCpD - 1>();
            __syncwarp();
            int b_t = __shfl_up_sync(0xffffffffu, o_t, 1);
            float4 b_p = shfl_up_f4(o_p);
            if (lane == 0) {
                const int slot = ((s / kCpCH) % kCpBndChunks) * kCpCH + (s % kCpCH);
                b_t = bnd_t[slot];
                b_p = bnd_p[slot];
            }
            const bool cin = !check || (c >= 0 && c < P);
            const int i = SX > 0 ? c : P - 1 - c;
            if (rowvalid && cin && i < NX) {
                const int own = at(c, brow);
                const int r_t = (c + 1 < P) ? at(c + 1, brow) : -1;
                const int u_t = at(c, urow);
                const float4 own_p = gring[lane * kCpR + (c & (kCpR - 1))];
                const float4 r_p = gring[lane * kCpR + ((c + 1) & (kCpR - 1))];
                const float4 u_p = gring[(lane + 1) * kCpR + (c & (kCpR - 1))];
                const float2 xc = __ldg(a.xtab + i);
                CpCur cur;
                cur.t = own;
                cur.p = own_p;
                cur.q = 0.f;
                cur.E = 0.f;
                if (own >= 0) cp_q32(own_p, xc, yc, kc, cur.q, cur.E);
                // the reference's order: (i-1,j), (i+1,j), (i,j-1), (i,j+1)
                const int e0 = SX > 0 ? o_t : r_t, e1 = SX > 0 ? r_t : o_t;
                const float4 p0 = SX > 0 ? o_p : r_p, p1 = SX > 0 ? r_p : o_p;
                const int e2 = SY > 0 ? b_t : u_t, e3 = SY > 0 ? u_t : b_t;
                const float4 p2 = SY > 0 ? b_p : u_p, p3 = SY > 0 ? u_p : b_p;
                const bool ok0 = i - 1 >= 0, ok1 = i + 1 < NX, ok2 = j - 1 >= 0, ok3 = j + 1 < NY;
                bool und = false;
                cp_offer_fast(e0, p0, ok0, cur, xc, yc, kc, und);
                cp_offer_fast(e1, p1, ok1, cur, xc, yc, kc, und);
                cp_offer_fast(e2, p2, ok2, cur, xc, yc, kc, und);
                cp_offer_fast(e3, p3, ok3, cur, xc, yc, kc, und);
                if (und) {
                    float4 sp;
                    cur.t = cp_cell_slow(own, own_p, e0, p0, ok0, e1, p1, ok1, e2, p2, ok2, e3, p3, ok3, xc, yc, kc,
                                         a.pos, i, j, a.dx, a.dr, &sp);
                    cur.p = sp;
                }
                if (cur.t != own) at(c, brow) = cur.t;
                o_t = cur.t;
                o_p = cur.p;
            } else {
                o_t = -1;
            }
            if (publishes && lane == 31 && cin) {
                top_t[c % kCpTopRing] = o_t;
                top_p[c % kCpTopRing] = o_p;
                if (((c + 1) % 8) == 0 || c == P - 1) {
                    __threadfence_block();
                    *top_ready = c + 1;
                }
            }
        }
    };

    const int nsteps = P + 31;
    for (int t = 0; t * kCpCols < nsteps; t++) {
        if (t + 1 < nt) wait_tile(t + 1);
        if (publishes && t * kCpCols - 31 - *top_done > kCpTopRing / 2)
            spin_ge(top_done, t * kCpCols - 31 - kCpTopRing / 2);
        __syncwarp();
        if (t == 0 || t >= nt - 1)
            tile_steps(t, BoolTag<true>{});
        else
            tile_steps(t, BoolTag<false>{});
        // tile t-1 is final: hand it to the I/O warp for its store
        if (t >= 1 && t - 1 < nt) {
            fence_async_smem();
            __syncwarp();
            if (lane == 0) *tiles_done = t;
        }
        const int nx = t + kCpAhead;
        if (nx < nt) {
            if (nx >= kCpSlots && *tiles_freed < nx - kCpSlots + 1) spin_ge(tiles_freed, nx - kCpSlots + 1);
            __syncwarp();
            issue(nx);
        }
    }
    cp_async_wait<0>();
    __syncwarp();
    // every issued tile was waited for in the loop (wait_tile(t + 1) for each
    // t + 1 < nt), so no TMA load is in flight when the CTA exits
    if (lane == 0) *tiles_done = nt;
    (void)failed;
  };

    if (!SEVERAL) {
        run_strip(maps1, a1, blockIdx.x);
        return;
    }
    const CpScene* scenes = static_cast<const CpScene*>(w.scenes);
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
        const CpScene* sc = scenes + item.scene;
        CpArgs a = sc->a;
        a.progress = w.progress + (item.pidx - item.strip);
        a.base = w.base;
        a.err = w.err;
        a.skip = nullptr;
        if (used && threadIdx.x == 0)   // run_strip initialises them again (same thread, in order)
            for (int k = 0; k < kCpSlots; k++) mbar_inval(bars + k);
        used = true;
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
