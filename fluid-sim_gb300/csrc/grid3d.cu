// grid3d.cu — bulk device counterparts of the reference's 3D containers,
// Array3D<double> (include/Array3D.h:15-128) and MACGrid3D
// (include/MACGrid3D.h:12-168), behind the C ABI of include/fs3d.h.
//
// Every method becomes one launch over a whole array, every cell, every face
// of one axis, or a batch of sample points: grid-stride loops over a grid of
// a few CTAs per SM, 16-byte accesses where every operand is 16-byte
// aligned.  The two reductions are fixed trees (per-thread runs, warp
// shuffles, one partial per CTA, one CTA over the partials), so a result
// never depends on timing.  Arithmetic follows the reference's expressions
// in its operation order; the file is compiled without FMA contraction, so
// every result that is not a reduction equals the serial C++ result bit for
// bit.  GB300 issues FP64 at a small fraction of its FP32 rate, and the
// stencils' FP64 additions, not HBM, bound most of these kernels: FP64 work
// that can be done exactly without the FP64 pipe is done without it (the
// exact halving and quartering of scale_down, the norm's integer compares).
//
// Where the reference's code cannot be followed literally (loops that run
// past the array, triCubic's swapped x/z indices) include/fs3d.h states the
// rule used instead.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "fs2d_internal.cuh"
#include "fs3d.h"

namespace fs2d {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocksPerSM = 8;   // 8 x 256 threads fill an SM
constexpr int kFinalThreads = 1024;

int sm_count(int* out) {
    static std::mutex mu;
    static int cached[64] = {};
    int dev = 0;
    FS2D_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64) {
        *out = 152;
        return 0;
    }
    if (!cached[dev]) FS2D_CUDA(cudaDeviceGetAttribute(&cached[dev], cudaDevAttrMultiProcessorCount, dev));
    *out = cached[dev];
    return 0;
}

// Blocks of kThreads for `work` items: at most kBlocksPerSM per SM (the
// kernels loop), at least one.
int grid_for(size_t work, unsigned int* blocks) {
    int sms = 0;
    int rc = sm_count(&sms);
    if (rc) return rc;
    const size_t need = (work + kThreads - 1) / kThreads;
    const size_t cap = (size_t)sms * kBlocksPerSM;
    *blocks = (unsigned int)(need < 1 ? 1 : (need < cap ? need : cap));
    return 0;
}

// CTAs for a row walker over `rows` rows: one per row, at most kBlocksPerSM
// per SM.
int grid_rows(size_t rows, unsigned int* blocks) {
    int sms = 0;
    int rc = sm_count(&sms);
    if (rc) return rc;
    const size_t cap = (size_t)sms * kBlocksPerSM;
    *blocks = (unsigned int)(rows < 1 ? 1 : (rows < cap ? rows : cap));
    return 0;
}

size_t count(const fs3d_array& a) { return (size_t)a.NX * a.NY * a.NZ; }

bool dims_ok(const fs3d_array* a) { return a && a->NX >= 0 && a->NY >= 0 && a->NZ >= 0; }

bool same_dims(const fs3d_array& a, const fs3d_array& b) { return a.NX == b.NX && a.NY == b.NY && a.NZ == b.NZ; }

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// Refuses anything but device (or managed) memory of the current device, so
// that no kernel is ever handed a host address.
int device_ptr(const void* p, const char* fn, const char* what) {
    if (!p) {
        set_error("%s: %s is NULL", fn, what);
        return FS2D_ERR_INVALID;
    }
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: %s: cudaPointerGetAttributes: %s", fn, what, cudaGetErrorString(e));
        return FS2D_ERR_CUDA;
    }
    int dev = 0;
    FS2D_CUDA(cudaGetDevice(&dev));
    if (at.type == cudaMemoryTypeManaged) return 0;
    if (at.type != cudaMemoryTypeDevice || at.device != dev) {
        set_error("%s: %s is not device memory of the current device", fn, what);
        return FS2D_ERR_INVALID;
    }
    return 0;
}

int launched(const char* fn) { return check_cuda(cudaGetLastError(), fn); }

// ---- MAC grid accessors: element (i, j, k) of an NX x NY x NZ array ----
struct A3 {
    const double* d;
    int NX, NY;
    __device__ __forceinline__ double operator()(int i, int j, int k) const {
        return d[((size_t)k * NY + j) * NX + i];
    }
};

struct Mac {
    A3 u, v, w;
    int sx, sy, sz;
};

Mac mac_of(const fs3d_mac& g) {
    return Mac{A3{g.u.data, g.u.NX, g.u.NY}, A3{g.v.data, g.v.NX, g.v.NY}, A3{g.w.data, g.w.NX, g.w.NY},
               g.sizeX, g.sizeY, g.sizeZ};
}

// ---- Array3D::operator+= (include/Array3D.h:39-45) ----
template <bool VEC>
__global__ void k_add(double* a, const double* b, size_t n) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    if (VEC) {
        double2* a2 = reinterpret_cast<double2*>(a);
        const double2* b2 = reinterpret_cast<const double2*>(b);
        for (size_t e = t; e < n / 2; e += stride) {
            double2 x = a2[e];
            const double2 y = b2[e];
            x.x += y.x;
            x.y += y.y;
            a2[e] = x;
        }
        if (t == 0 && (n & 1)) a[n - 1] += b[n - 1];
    } else {
        for (size_t e = t; e < n; e += stride) a[e] += b[e];
    }
}

// ---- Array3D::setMultiplyAdd (include/Array3D.h:48-53): out = a + s*c ----
template <bool VEC>
__global__ void k_smadd(double* out, const double* a, double s, const double* c, size_t n) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    if (VEC) {
        double2* o2 = reinterpret_cast<double2*>(out);
        const double2* a2 = reinterpret_cast<const double2*>(a);
        const double2* c2 = reinterpret_cast<const double2*>(c);
        for (size_t e = t; e < n / 2; e += stride) {
            const double2 x = a2[e], y = c2[e];
            o2[e] = make_double2(x.x + s * y.x, x.y + s * y.y);
        }
        if (t == 0 && (n & 1)) out[n - 1] = a[n - 1] + s * c[n - 1];
    } else {
        for (size_t e = t; e < n; e += stride) out[e] = a[e] + s * c[e];
    }
}

// ---- fixed-order reductions ----
// GB300 issues FP64 at a small fraction of its FP32 rate, so a reduction
// over HBM-resident doubles is bound by its FP64 instructions unless it
// issues at most about one per element: the dot product accumulates with one
// fused multiply-add per element, and the norm compares magnitudes as
// integers (for non-negative doubles the order of the bit patterns is the
// order of the values).
struct SumOp {
    typedef double T;
    __device__ __forceinline__ static double id() { return 0.0; }
    __device__ __forceinline__ static double join(double a, double b) { return a + b; }
};
// infiniteNorm's update `if (abs(x) > result) result = abs(x)`: NaN never wins.
struct MaxOp {
    typedef double T;
    __device__ __forceinline__ static double id() { return 0.0; }
    __device__ __forceinline__ static double join(double a, double b) { return b > a ? b : a; }
};
// The same update on the bit patterns of |x|: a NaN's pattern (above that
// of +inf) never wins.
struct MaxBitsOp {
    typedef unsigned long long T;
    __device__ __forceinline__ static T id() { return 0ull; }
    __device__ __forceinline__ static T join(T a, T b) { return (b > a && b <= 0x7FF0000000000000ull) ? b : a; }
};

__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

template <class Op>
__device__ typename Op::T block_reduce(typename Op::T x, typename Op::T* sh) {
    for (int o = 16; o > 0; o >>= 1) x = Op::join(x, __shfl_down_sync(0xffffffffu, x, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) sh[warp] = x;
    __syncthreads();
    x = Op::id();
    if (warp == 0) {
        x = lane < nw ? sh[lane] : Op::id();
        for (int o = 16; o > 0; o >>= 1) x = Op::join(x, __shfl_down_sync(0xffffffffu, x, o));
    }
    return x;
}

template <bool VEC>
__global__ void k_dot_part(const double* a, const double* b, size_t n, double* part) {
    __shared__ double sh[32];
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    double acc = 0.0;
    if (VEC) {
        const double2* a2 = reinterpret_cast<const double2*>(a);
        const double2* b2 = reinterpret_cast<const double2*>(b);
        for (size_t e = t; e < n / 2; e += stride) {
            const double2 x = a2[e], y = b2[e];
            acc = fma(x.x, y.x, acc);
            acc = fma(x.y, y.y, acc);
        }
        if (t == 0 && (n & 1)) acc = fma(a[n - 1], b[n - 1], acc);
    } else {
        for (size_t e = t; e < n; e += stride) acc = fma(a[e], b[e], acc);
    }
    acc = block_reduce<SumOp>(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

template <bool VEC>
__global__ void k_absmax_part(const double* a, size_t n, double* part) {
    __shared__ unsigned long long sh[32];
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    unsigned long long m = 0ull;
    if (VEC) {
        const double2* a2 = reinterpret_cast<const double2*>(a);
        for (size_t e = t; e < n / 2; e += stride) {
            const double2 x = a2[e];
            m = MaxBitsOp::join(m, abs_bits(x.x));
            m = MaxBitsOp::join(m, abs_bits(x.y));
        }
        if (t == 0 && (n & 1)) m = MaxBitsOp::join(m, abs_bits(a[n - 1]));
    } else {
        for (size_t e = t; e < n; e += stride) m = MaxBitsOp::join(m, abs_bits(a[e]));
    }
    m = block_reduce<MaxBitsOp>(m, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = __longlong_as_double((long long)m);
}

template <class Op>
__global__ void k_final(const double* part, int n, double* out) {
    __shared__ double sh[32];
    double x = Op::id();
    for (int e = threadIdx.x; e < n; e += blockDim.x) x = Op::join(x, part[e]);
    x = block_reduce<Op>(x, sh);
    if (threadIdx.x == 0) *out = x;
}

// x * 2^-S (S = 1: the reference's 0.5 * x, S = 2: its 0.25 * x), rounded
// as the FP64 multiply rounds it, in integer arithmetic: for a normal x whose
// product stays normal the exponent drops by S; where the product is
// subnormal (or x is), the significand shifts right by the remaining amount
// with round-to-nearest-even; infinities and NaN pass through.  No FP64
// instruction, on any path.
template <int S>
__device__ __forceinline__ double scale_down(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int e = (unsigned int)(b >> 52) & 0x7FFu;
    if (e == 0x7FFu) return x;
    if (e > (unsigned int)S) return __longlong_as_double((long long)(b - ((unsigned long long)S << 52)));
    const unsigned long long m = (b & 0x000FFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
    const unsigned int sh = (unsigned int)S + 1u - (e ? e : 1u);   // 1 .. S
    unsigned long long q = m >> sh;
    const unsigned long long rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1u);
    q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
    return __longlong_as_double((long long)((b & 0x8000000000000000ull) | q));
}

// ---- Array3D::triCubic (include/Array3D.h:75-124) at one point ----
// The Catmull-Rom weights keep the reference's CUBE / SQR groupings.
__device__ __forceinline__ void cr_weights(double t, double* c) {
    const double t3 = t * t * t, t2 = t * t;
    c[0] = -0.5 * t3 + t2 - 0.5 * t;
    c[1] = 1.5 * t3 - 2.5 * t2 + 1;
    c[2] = -1.5 * t3 + 2 * t2 + 0.5 * t;
    c[3] = 0.5 * t3 - 0.5 * t2;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// A coordinate whose truncation is no int (NaN, infinities, |p| >= 2^31)
// counts as outside the array.
__device__ __forceinline__ bool int_range(double p) { return p > -2147483649.0 && p < 2147483648.0; }

__device__ double tricubic(const double* __restrict__ a, int NX, int NY, int NZ, double px, double py, double pz) {
    if (!int_range(px) || !int_range(py) || !int_range(pz)) return 0.0;
    const int x = (int)px, y = (int)py, z = (int)pz;
    if (x < 0 || x >= NX || y < 0 || y >= NY || z < 0 || z >= NZ) return 0.0;
    double cu[4], cv[4], cw[4];
    cr_weights(px - (double)x, cu);
    cr_weights(py - (double)y, cv);
    cr_weights(pz - (double)z, cw);
    int xs[4];
#pragma unroll
    for (int i = 0; i < 4; i++) xs[i] = clampi(x + i - 1, 0, NX - 1);
    double vox = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int zp = clampi(z + k - 1, 0, NZ - 1);
        double q = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int yp = clampi(y + j - 1, 0, NY - 1);
            const double* row = a + ((size_t)zp * NY + yp) * NX;
            double r = 0;
#pragma unroll
            for (int i = 0; i < 4; i++) r += cu[i] * __ldg(row + xs[i]);
            q += cv[j] * r;
        }
        vox += cw[k] * q;
    }
    return vox < 0 ? 0.0 : vox;
}

__global__ void k_tricubic(const double* __restrict__ a, int NX, int NY, int NZ, const double* __restrict__ pts,
                           size_t n, double* __restrict__ out) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += stride)
        out[e] = tricubic(a, NX, NY, NZ, pts[3 * e], pts[3 * e + 1], pts[3 * e + 2]);
}

// ---- MACGrid3D::velInterpU/V/W, velInterp (include/MACGrid3D.h:143-163) ----
template <int COMP>
__global__ void k_vel_interp(Mac g, int uNZ, int vNZ, int wNZ, const double* __restrict__ pts, size_t n,
                             double* __restrict__ out) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += stride) {
        const double x = pts[3 * e], y = pts[3 * e + 1], z = pts[3 * e + 2];
        // velInterpU: y, z shifted by half a cell; V: z, x; W: x, y
        if (COMP == FS3D_U || COMP == FS3D_UVW) {
            const double r = tricubic(g.u.d, g.u.NX, g.u.NY, uNZ, x, y - 0.5, z - 0.5);
            if (COMP == FS3D_U) out[e] = r; else out[3 * e] = r;
        }
        if (COMP == FS3D_V || COMP == FS3D_UVW) {
            const double r = tricubic(g.v.d, g.v.NX, g.v.NY, vNZ, x - 0.5, y, z - 0.5);
            if (COMP == FS3D_V) out[e] = r; else out[3 * e + 1] = r;
        }
        if (COMP == FS3D_W || COMP == FS3D_UVW) {
            const double r = tricubic(g.w.d, g.w.NX, g.w.NY, wNZ, x - 0.5, y - 0.5, z);
            if (COMP == FS3D_W) out[e] = r; else out[3 * e + 2] = r;
        }
    }
}

// ---- row walkers over cells and faces ----
// A CTA takes whole rows (j, k) of the output grid in grid-stride order, its
// threads covering i in chunks of kThreads; (j, k) advance incrementally, so
// no thread divides per cell.  vec3 results are staged in shared memory and
// leave as one contiguous run of 3 x kThreads doubles per chunk.  The loop
// trip counts are the same for every thread of a CTA, so the barriers are
// reached by all of them.
struct RowWalk {
    long long r;   // row index j + k * ny
    int j;
    long long k;
    int dj;
    long long dk;
    __device__ RowWalk(int ny) {
        r = blockIdx.x;
        j = (int)(blockIdx.x % (unsigned)ny);
        k = blockIdx.x / (unsigned)ny;
        dj = (int)(gridDim.x % (unsigned)ny);
        dk = gridDim.x / (unsigned)ny;
    }
    __device__ void next(int ny) {
        r += gridDim.x;
        j += dj;
        k += dk;
        if (j >= ny) {
            j -= ny;
            k++;
        }
    }
};

__device__ __forceinline__ void put3(double* st, double* out, size_t first, int i0, int nx, double x, double y,
                                     double z) {
    const int t = threadIdx.x;
    if (i0 + t < nx) {
        st[3 * t] = x;
        st[3 * t + 1] = y;
        st[3 * t + 2] = z;
    }
    __syncthreads();
    const int nv = min(kThreads, nx - i0);
    for (int e = t; e < 3 * nv; e += kThreads) out[3 * (first + i0) + e] = st[e];
    __syncthreads();
}

// ---- MACGrid3D::vel (include/MACGrid3D.h:73-78) and velDiv (:165-167) at every cell ----
template <bool DIV>
__global__ void __launch_bounds__(kThreads) k_cells(Mac g, double* __restrict__ out) {
    __shared__ double st[3 * kThreads];
    const long long rows = (long long)g.sy * g.sz;
    for (RowWalk w(g.sy); w.r < rows; w.next(g.sy)) {
        const int j = w.j, k = (int)w.k;
        const size_t first = (size_t)w.r * g.sx;
        for (int i0 = 0; i0 < g.sx; i0 += kThreads) {
            const int i = i0 + threadIdx.x;
            if (DIV) {
                if (i < g.sx)
                    out[first + i] = g.u(i + 1, j, k) - g.u(i, j, k) + g.v(i, j + 1, k) - g.v(i, j, k) +
                                     g.w(i, j, k + 1) - g.w(i, j, k);
            } else {
                double x = 0, y = 0, z = 0;
                if (i < g.sx) {
                    x = scale_down<1>(g.u(i + 1, j, k) + g.u(i, j, k));
                    y = scale_down<1>(g.v(i, j + 1, k) + g.v(i, j, k));
                    z = scale_down<1>(g.w(i, j, k + 1) + g.w(i, j, k));
                }
                put3(st, out, first, i0, g.sx, x, y, z);
            }
        }
    }
}

// ---- MACGrid3D::velU / velV / velW (include/MACGrid3D.h:80-141) at every face of one axis ----
template <int AXIS>
__device__ __forceinline__ void face_vel(const Mac& g, int i, int j, int k, double& rx, double& ry, double& rz) {
    if (AXIS == FS3D_U) {
        rx = g.u(i, j, k);
        if (i > 0 && i < g.sx) {
            ry = scale_down<2>(g.v(i - 1, j, k) + g.v(i - 1, j + 1, k) + g.v(i, j, k) + g.v(i, j + 1, k));
            rz = scale_down<2>(g.w(i - 1, j, k) + g.w(i - 1, j, k + 1) + g.w(i, j, k) + g.w(i, j, k + 1));
        } else if (i == 0) {
            ry = scale_down<2>(g.v(i, j, k) + g.v(i, j + 1, k));
            rz = scale_down<2>(g.w(i, j, k) + g.w(i, j, k + 1));
        } else {
            ry = scale_down<2>(g.v(i - 1, j, k) + g.v(i - 1, j + 1, k));
            rz = scale_down<2>(g.w(i - 1, j, k) + g.w(i - 1, j, k + 1));
        }
    } else if (AXIS == FS3D_V) {
        ry = g.v(i, j, k);
        if (j > 0 && j < g.sy) {
            rx = scale_down<2>(g.u(i, j - 1, k) + g.u(i, j, k) + g.u(i + 1, j - 1, k) + g.u(i + 1, j, k));
            rz = scale_down<2>(g.w(i, j - 1, k) + g.w(i, j - 1, k + 1) + g.w(i, j, k) + g.w(i, j, k + 1));
        } else if (j == 0) {
            rx = scale_down<2>(g.u(i, j, k) + g.u(i + 1, j, k));
            rz = scale_down<2>(g.w(i, j, k) + g.w(i, j, k + 1));
        } else {
            rx = scale_down<2>(g.u(i, j - 1, k) + g.u(i + 1, j - 1, k));
            rz = scale_down<2>(g.w(i, j - 1, k) + g.w(i, j - 1, k + 1));
        }
    } else {
        rz = g.w(i, j, k);
        if (k > 0 && k < g.sz) {
            rx = scale_down<2>(g.u(i, j, k - 1) + g.u(i + 1, j, k - 1) + g.u(i, j, k) + g.u(i + 1, j, k));
            ry = scale_down<2>(g.v(i, j, k - 1) + g.v(i, j + 1, k - 1) + g.v(i, j, k) + g.v(i, j + 1, k));
        } else if (k == 0) {
            rx = scale_down<2>(g.u(i, j, k) + g.u(i + 1, j, k));
            ry = scale_down<2>(g.v(i, j, k) + g.v(i, j + 1, k));
        } else {
            rx = scale_down<2>(g.u(i, j, k - 1) + g.u(i + 1, j, k - 1));
            ry = scale_down<2>(g.v(i, j, k - 1) + g.v(i, j + 1, k - 1));
        }
    }
}

template <int AXIS>
__global__ void __launch_bounds__(kThreads) k_face_vel(Mac g, double* __restrict__ out) {
    __shared__ double st[3 * kThreads];
    const int fx = g.sx + (AXIS == FS3D_U), fy = g.sy + (AXIS == FS3D_V), fz = g.sz + (AXIS == FS3D_W);
    const long long rows = (long long)fy * fz;
    for (RowWalk w(fy); w.r < rows; w.next(fy)) {
        const int j = w.j, k = (int)w.k;
        const size_t first = (size_t)w.r * fx;
        for (int i0 = 0; i0 < fx; i0 += kThreads) {
            const int i = i0 + threadIdx.x;
            double x = 0, y = 0, z = 0;
            if (i < fx) face_vel<AXIS>(g, i, j, k, x, y, z);
            put3(st, out, first, i0, fx, x, y, z);
        }
    }
}

// ---- argument checks ----
int check_array(const fs3d_array* a, const char* fn, const char* what) {
    if (!dims_ok(a)) {
        set_error("%s: %s: NULL or negative extents", fn, what);
        return FS2D_ERR_INVALID;
    }
    return 0;
}

int check_mac(const fs3d_mac* g, const char* fn) {
    if (!g || g->sizeX < 1 || g->sizeY < 1 || g->sizeZ < 1) {
        set_error("%s: NULL grid or a size below 1", fn);
        return FS2D_ERR_INVALID;
    }
    const int sx = g->sizeX, sy = g->sizeY, sz = g->sizeZ;
    if (g->u.NX != sx + 1 || g->u.NY != sy || g->u.NZ != sz || g->v.NX != sx || g->v.NY != sy + 1 ||
        g->v.NZ != sz || g->w.NX != sx || g->w.NY != sy || g->w.NZ != sz + 1) {
        set_error("%s: face arrays must be (sizeX+1) x sizeY x sizeZ, sizeX x (sizeY+1) x sizeZ and "
                  "sizeX x sizeY x (sizeZ+1)", fn);
        return FS2D_ERR_INVALID;
    }
    return 0;
}

int check_mac_memory(const fs3d_mac* g, const char* fn) {
    int rc;
    if ((rc = device_ptr(g->u.data, fn, "u"))) return rc;
    if ((rc = device_ptr(g->v.data, fn, "v"))) return rc;
    return device_ptr(g->w.data, fn, "w");
}

// Reduction driver: partials in stream-ordered scratch, one CTA over them,
// the scalar copied to the host after the stream drained.
template <class Op, class Launch>
int reduce(size_t n, cudaStream_t st, double* result, const char* fn, Launch launch_part) {
    unsigned int blocks = 0;
    int rc = grid_for((n + 1) / 2, &blocks);
    if (rc) return rc;
    double* part = nullptr;
    if ((rc = check_cuda(cudaMallocAsync((void**)&part, (blocks + 1) * sizeof(double), st), "cudaMallocAsync")))
        return rc;
    launch_part(blocks, part);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_final<Op><<<1, kFinalThreads, 0, st>>>(part, (int)blocks, part + blocks);
        e = cudaGetLastError();
    }
    double h = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, part + blocks, sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaError_t f = cudaFreeAsync(part, st);
    cudaError_t s = cudaStreamSynchronize(st);
    if ((rc = check_cuda(e, fn)) || (rc = check_cuda(f, "cudaFreeAsync")) || (rc = check_cuda(s, fn))) return rc;
    *result = h;
    return 0;
}

}  // namespace
}  // namespace fs2d

using namespace fs2d;

extern "C" int fs3d_add(const fs3d_array* a, const fs3d_array* b, void* stream) {
    const char* fn = "fs3d_add";
    int rc;
    if ((rc = check_array(a, fn, "a")) || (rc = check_array(b, fn, "b"))) return rc;
    if (!same_dims(*a, *b)) {
        set_error("%s: extents differ", fn);
        return FS2D_ERR_INVALID;
    }
    const size_t n = count(*a);
    if (n == 0) return 0;
    if ((rc = device_ptr(a->data, fn, "a")) || (rc = device_ptr(b->data, fn, "b"))) return rc;
    unsigned int blocks = 0;
    const bool vec = aligned16(a->data) && aligned16(b->data);
    if ((rc = grid_for(vec ? (n + 1) / 2 : n, &blocks))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (vec) k_add<true><<<blocks, kThreads, 0, st>>>(a->data, b->data, n);
    else k_add<false><<<blocks, kThreads, 0, st>>>(a->data, b->data, n);
    return launched(fn);
}

extern "C" int fs3d_set_multiply_add(const fs3d_array* out, const fs3d_array* a, double s, const fs3d_array* c,
                                     void* stream) {
    const char* fn = "fs3d_set_multiply_add";
    int rc;
    if ((rc = check_array(out, fn, "out")) || (rc = check_array(a, fn, "a")) || (rc = check_array(c, fn, "c")))
        return rc;
    if (!same_dims(*out, *a) || !same_dims(*out, *c)) {
        set_error("%s: extents differ", fn);
        return FS2D_ERR_INVALID;
    }
    const size_t n = count(*out);
    if (n == 0) return 0;
    if ((rc = device_ptr(out->data, fn, "out")) || (rc = device_ptr(a->data, fn, "a")) ||
        (rc = device_ptr(c->data, fn, "c")))
        return rc;
    unsigned int blocks = 0;
    const bool vec = aligned16(out->data) && aligned16(a->data) && aligned16(c->data);
    if ((rc = grid_for(vec ? (n + 1) / 2 : n, &blocks))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (vec) k_smadd<true><<<blocks, kThreads, 0, st>>>(out->data, a->data, s, c->data, n);
    else k_smadd<false><<<blocks, kThreads, 0, st>>>(out->data, a->data, s, c->data, n);
    return launched(fn);
}

extern "C" int fs3d_inner_product(const fs3d_array* a, const fs3d_array* b, double* result, void* stream) {
    const char* fn = "fs3d_inner_product";
    int rc;
    if ((rc = check_array(a, fn, "a")) || (rc = check_array(b, fn, "b"))) return rc;
    if (!result || !same_dims(*a, *b)) {
        set_error("%s: NULL result or extents differ", fn);
        return FS2D_ERR_INVALID;
    }
    const size_t n = count(*a);
    if (n == 0) {
        *result = 0.0;
        return 0;
    }
    if ((rc = device_ptr(a->data, fn, "a")) || (rc = device_ptr(b->data, fn, "b"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const bool vec = aligned16(a->data) && aligned16(b->data);
    const double *pa = a->data, *pb = b->data;
    return reduce<SumOp>(n, st, result, fn, [&](unsigned int blocks, double* part) {
        if (vec) k_dot_part<true><<<blocks, kThreads, 0, st>>>(pa, pb, n, part);
        else k_dot_part<false><<<blocks, kThreads, 0, st>>>(pa, pb, n, part);
    });
}

extern "C" int fs3d_infinite_norm(const fs3d_array* a, double* result, void* stream) {
    const char* fn = "fs3d_infinite_norm";
    int rc;
    if ((rc = check_array(a, fn, "a"))) return rc;
    if (!result) {
        set_error("%s: NULL result", fn);
        return FS2D_ERR_INVALID;
    }
    const size_t n = count(*a);
    if (n == 0) {
        *result = 0.0;
        return 0;
    }
    if ((rc = device_ptr(a->data, fn, "a"))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const bool vec = aligned16(a->data);
    const double* pa = a->data;
    return reduce<MaxOp>(n, st, result, fn, [&](unsigned int blocks, double* part) {
        if (vec) k_absmax_part<true><<<blocks, kThreads, 0, st>>>(pa, n, part);
        else k_absmax_part<false><<<blocks, kThreads, 0, st>>>(pa, n, part);
    });
}

extern "C" int fs3d_tricubic(const fs3d_array* a, const double* points, size_t n, double* out, void* stream) {
    const char* fn = "fs3d_tricubic";
    int rc;
    if ((rc = check_array(a, fn, "a"))) return rc;
    if (n == 0) return 0;
    if ((rc = device_ptr(points, fn, "points")) || (rc = device_ptr(out, fn, "out"))) return rc;
    if (count(*a) == 0) {
        // every point lies outside an empty array
        return check_cuda(cudaMemsetAsync(out, 0, n * sizeof(double), (cudaStream_t)stream), fn);
    }
    if ((rc = device_ptr(a->data, fn, "a"))) return rc;
    unsigned int blocks = 0;
    if ((rc = grid_for(n, &blocks))) return rc;
    k_tricubic<<<blocks, kThreads, 0, (cudaStream_t)stream>>>(a->data, a->NX, a->NY, a->NZ, points, n, out);
    return launched(fn);
}

extern "C" int fs3d_mac_vel(const fs3d_mac* g, double* out, void* stream) {
    const char* fn = "fs3d_mac_vel";
    int rc;
    if ((rc = check_mac(g, fn))) return rc;
    if ((rc = check_mac_memory(g, fn)) || (rc = device_ptr(out, fn, "out"))) return rc;
    unsigned int blocks = 0;
    if ((rc = grid_rows((size_t)g->sizeY * g->sizeZ, &blocks))) return rc;
    k_cells<false><<<blocks, kThreads, 0, (cudaStream_t)stream>>>(mac_of(*g), out);
    return launched(fn);
}

extern "C" int fs3d_mac_vel_div(const fs3d_mac* g, double* out, void* stream) {
    const char* fn = "fs3d_mac_vel_div";
    int rc;
    if ((rc = check_mac(g, fn))) return rc;
    if ((rc = check_mac_memory(g, fn)) || (rc = device_ptr(out, fn, "out"))) return rc;
    unsigned int blocks = 0;
    if ((rc = grid_rows((size_t)g->sizeY * g->sizeZ, &blocks))) return rc;
    k_cells<true><<<blocks, kThreads, 0, (cudaStream_t)stream>>>(mac_of(*g), out);
    return launched(fn);
}

extern "C" int fs3d_mac_face_vel(const fs3d_mac* g, int axis, double* out, void* stream) {
    const char* fn = "fs3d_mac_face_vel";
    int rc;
    if ((rc = check_mac(g, fn))) return rc;
    if (axis != FS3D_U && axis != FS3D_V && axis != FS3D_W) {
        set_error("%s: axis must be FS3D_U, FS3D_V or FS3D_W", fn);
        return FS2D_ERR_INVALID;
    }
    if ((rc = check_mac_memory(g, fn)) || (rc = device_ptr(out, fn, "out"))) return rc;
    const fs3d_array& f = axis == FS3D_U ? g->u : (axis == FS3D_V ? g->v : g->w);
    unsigned int blocks = 0;
    if ((rc = grid_rows((size_t)f.NY * f.NZ, &blocks))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const Mac m = mac_of(*g);
    if (axis == FS3D_U) k_face_vel<FS3D_U><<<blocks, kThreads, 0, st>>>(m, out);
    else if (axis == FS3D_V) k_face_vel<FS3D_V><<<blocks, kThreads, 0, st>>>(m, out);
    else k_face_vel<FS3D_W><<<blocks, kThreads, 0, st>>>(m, out);
    return launched(fn);
}

extern "C" int fs3d_mac_vel_interp(const fs3d_mac* g, int component, const double* points, size_t n, double* out,
                                   void* stream) {
    const char* fn = "fs3d_mac_vel_interp";
    int rc;
    if ((rc = check_mac(g, fn))) return rc;
    if (component < FS3D_U || component > FS3D_UVW) {
        set_error("%s: component must be FS3D_U, FS3D_V, FS3D_W or FS3D_UVW", fn);
        return FS2D_ERR_INVALID;
    }
    if (n == 0) return 0;
    if ((rc = check_mac_memory(g, fn)) || (rc = device_ptr(points, fn, "points")) ||
        (rc = device_ptr(out, fn, "out")))
        return rc;
    unsigned int blocks = 0;
    if ((rc = grid_for(n, &blocks))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const Mac m = mac_of(*g);
    const int uz = g->u.NZ, vz = g->v.NZ, wz = g->w.NZ;
    switch (component) {
        case FS3D_U: k_vel_interp<FS3D_U><<<blocks, kThreads, 0, st>>>(m, uz, vz, wz, points, n, out); break;
        case FS3D_V: k_vel_interp<FS3D_V><<<blocks, kThreads, 0, st>>>(m, uz, vz, wz, points, n, out); break;
        case FS3D_W: k_vel_interp<FS3D_W><<<blocks, kThreads, 0, st>>>(m, uz, vz, wz, points, n, out); break;
        default: k_vel_interp<FS3D_UVW><<<blocks, kThreads, 0, st>>>(m, uz, vz, wz, points, n, out); break;
    }
    return launched(fn);
}
