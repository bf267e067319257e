// adjoint.cu — reverse-mode derivative of the semi-Lagrangian step on a closed
// box of fluid (labels FLUID inside, SOLID border, no EMPTY cell, so the
// projection is a fixed linear map).
//
// Forward step k (the reference's SL-mode stages without the level set and
// particles): u* = SL(u_k) (applySemiLagrangianAdvection, src/FluidSim2D.cpp:
// 206-235, double-buffered), + dt g (applyGravity), p = A^-1 b(u*)
// (applyProjection :252-467, FP64 PCG or FP32 PCG inside FP64 refinement,
// solved to the handle's tolerance), u_{k+1} = E(W(u*, p)) (updateVelocity :469-550:
// W zeroes the faces next to a solid cell, subtracts dt/(rho dx) grad p on
// fluid-fluid faces and keeps u* on the faces the loop never visits; E is
// Array2D::extrapolate of the faces without a fluid side).
//
// Adjoint step, given lambda_{k+1} = dL/du_{k+1}:
//   E^T     layers from the deepest down: each extrapolated face hands its
//           adjoint in equal parts (1/count) to its lower-layer neighbours
//           and drops it (its own value was overwritten);
//   W^T     u*bar = mu on fluid-fluid and never-visited faces, 0 on faces
//           next to a solid; pbar = -dt/(rho dx) G^T mu on fluid-fluid faces;
//   A^-T    bbar = A^-1 pbar (A is symmetric: a second Poisson solve with the
//           same matrix, preconditioner and precision);
//   B^T     u*bar += the transposed divergence of the right-hand side
//           (faces next to a solid do not enter it);
//   SL^T    per face, the RK3 back-trace in reverse: the sampled value
//           scatters its adjoint with the Catmull-Rom weights at the
//           departure point, and the departure point's adjoint (derivatives
//           of the weights; zero where a position was clamped) flows back
//           through k3, k2, k1, each of which scatters into u and v with the
//           weights at its own point (atomic adds).
//
// The host driver (rollout_forward / rollout_backward) keeps the state before
// every `every`-th step (default ceil(sqrt(T))), and in reverse recomputes
// each segment from its checkpoint before walking it backwards; the forward
// pass already leaves the last segment's states in the segment buffer.
// extrap_adjoint (E^T of one face grid) is shared with the particle-transfer
// transposes in transfer.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <algorithm>
#include <vector>
#include "fs2d_device.cuh"

namespace fs2d {
namespace {

constexpr int kAT = 256;

// Catmull-Rom weights and their derivatives.
__device__ __forceinline__ void cr_weights(double t, double* w, double* dw) {
    w[0] = -0.5 * (t * t * t) + (t * t) - 0.5 * t;
    w[1] = 1.5 * (t * t * t) - 2.5 * (t * t) + 1.0;
    w[2] = -1.5 * (t * t * t) + 2.0 * (t * t) + 0.5 * t;
    w[3] = 0.5 * (t * t * t) - 0.5 * (t * t);
    dw[0] = -1.5 * t * t + 2.0 * t - 0.5;
    dw[1] = 4.5 * t * t - 5.0 * t;
    dw[2] = -4.5 * t * t + 4.0 * t + 0.5;
    dw[3] = 1.5 * t * t - t;
}

// Bicubic sample of data (W x H) at grid coordinates (px, py) with its
// gradient in grid units; optionally scatters `bar` times the weights into
// data_bar.  (px, py) are already clamped into the grid.
__device__ double cr_sample(const double* __restrict__ data, double* data_bar, double bar, int W, int H, double px,
                            double py, double& gx, double& gy) {
    const int x = (int)px, y = (int)py;
    const double fx = px - x, fy = py - y;
    double wx[4], dwx[4], wy[4], dwy[4];
    cr_weights(fx, wx, dwx);
    cr_weights(fy, wy, dwy);
    double val = 0, ddx = 0, ddy = 0;
    for (int j = 0; j < 4; j++) {
        const int yy = iclamp(y + j - 1, 0, H - 1);
        double r = 0, rd = 0;
        for (int i = 0; i < 4; i++) {
            const int xx = iclamp(x + i - 1, 0, W - 1);
            const double d = data[(size_t)yy * W + xx];
            r += wx[i] * d;
            rd += dwx[i] * d;
            if (data_bar && bar != 0.0) atomicAdd(data_bar + (size_t)yy * W + xx, bar * wx[i] * wy[j]);
        }
        val += wy[j] * r;
        ddx += wy[j] * rd;
        ddy += dwy[j] * r;
    }
    gx = ddx;
    gy = ddy;
    return val;
}

// velInterpU / velInterpV (include/MACGrid2D.h:80-94) with the derivative
// with respect to the world position (0 in a clamped direction) and the
// optional scatter of `bar`.
__device__ double interp_u(const double* __restrict__ u, double* u_bar, double bar, int NX, int NY, double dx,
                           double x, double y, double& dxw, double& dyw) {
    double px = x / dx, py = y / dx - 0.5;
    const double lx = 1e-6, hx = (double)(NX - 1) - 1e-6, hy = (double)(NY - 1) - 1e-6;
    const bool mx = px >= lx && px <= hx, my = py >= lx && py <= hy;
    px = dclamp(px, lx, hx);
    py = dclamp(py, lx, hy);
    double gx, gy;
    const double v = cr_sample(u, u_bar, bar, NX + 1, NY, px, py, gx, gy);
    dxw = mx ? gx / dx : 0.0;
    dyw = my ? gy / dx : 0.0;
    return v;
}
__device__ double interp_v(const double* __restrict__ v, double* v_bar, double bar, int NX, int NY, double dx,
                           double x, double y, double& dxw, double& dyw) {
    double px = x / dx - 0.5, py = y / dx;
    const double lx = 1e-6, hx = (double)(NX - 1) - 1e-6, hy = (double)(NY - 1) - 1e-6;
    const bool mx = px >= lx && px <= hx, my = py >= lx && py <= hy;
    px = dclamp(px, lx, hx);
    py = dclamp(py, lx, hy);
    double gx, gy;
    const double r = cr_sample(v, v_bar, bar, NX, NY + 1, px, py, gx, gy);
    dxw = mx ? gx / dx : 0.0;
    dyw = my ? gy / dx : 0.0;
    return r;
}

// Reverse of one face's semi-Lagrangian update.  comp 0: u face (i, j) at
// (i dx, (j + .5) dx) sampling u; comp 1: v face at ((i + .5) dx, j dx).
__global__ void k_sl_adjoint(const double* __restrict__ u, const double* __restrict__ v,
                             const double* __restrict__ ubar_star, const double* __restrict__ vbar_star, double* ubar,
                             double* vbar, int NX, int NY, double dx, double dt) {
    const int comp = blockIdx.z;
    const int W = comp == 0 ? NX + 1 : NX, H = comp == 0 ? NY : NY + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= W || j >= H) return;
    const double abar = comp == 0 ? ubar_star[(size_t)j * W + i] : vbar_star[(size_t)j * W + i];
    if (abar == 0.0) return;
    const double x0 = comp == 0 ? i * dx : (i + 0.5) * dx;
    const double y0 = comp == 0 ? (j + 0.5) * dx : j * dx;
    double d0, d1, d2, d3;
    // forward back-trace (as advect.cu computes it)
    const double k1x = interp_u(u, nullptr, 0, NX, NY, dx, x0, y0, d0, d1);
    const double k1y = interp_v(v, nullptr, 0, NX, NY, dx, x0, y0, d0, d1);
    const double x1 = x0 - 0.5 * dt * k1x, y1 = y0 - 0.5 * dt * k1y;
    double ux1x, ux1y, vx1x, vx1y;
    const double k2x = interp_u(u, nullptr, 0, NX, NY, dx, x1, y1, ux1x, ux1y);
    const double k2y = interp_v(v, nullptr, 0, NX, NY, dx, x1, y1, vx1x, vx1y);
    const double x2 = x0 - 0.75 * dt * k2x, y2 = y0 - 0.75 * dt * k2y;
    double ux2x, ux2y, vx2x, vx2y;
    const double k3x = interp_u(u, nullptr, 0, NX, NY, dx, x2, y2, ux2x, ux2y);
    const double k3y = interp_v(v, nullptr, 0, NX, NY, dx, x2, y2, vx2x, vx2y);
    const double Xr = x0 - ((2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x);
    const double Yr = y0 - ((2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y);
    const double off = 1e-3;
    const double lo = (1.0 + off) * dx, hxw = (NX - 1.0 - off) * dx, hyw = (NY - 1.0 - off) * dx;
    const bool cx = Xr >= lo && Xr <= hxw, cy = Yr >= lo && Yr <= hyw;
    const double X = dclamp(Xr, lo, hxw), Y = dclamp(Yr, lo, hyw);
    // reverse
    double gX, gY;
    if (comp == 0) interp_u(u, ubar, abar, NX, NY, dx, X, Y, gX, gY);
    else interp_v(v, vbar, abar, NX, NY, dx, X, Y, gX, gY);
    const double Xb = cx ? abar * gX : 0.0, Yb = cy ? abar * gY : 0.0;
    double k1bx = -(2. / 9.) * dt * Xb, k1by = -(2. / 9.) * dt * Yb;
    double k2bx = -(3. / 9.) * dt * Xb, k2by = -(3. / 9.) * dt * Yb;
    const double k3bx = -(4. / 9.) * dt * Xb, k3by = -(4. / 9.) * dt * Yb;
    // k3 = V(x2)
    interp_u(u, ubar, k3bx, NX, NY, dx, x2, y2, d0, d1);
    interp_v(v, vbar, k3by, NX, NY, dx, x2, y2, d2, d3);
    const double x2b = k3bx * ux2x + k3by * vx2x, y2b = k3bx * ux2y + k3by * vx2y;
    k2bx += -0.75 * dt * x2b;
    k2by += -0.75 * dt * y2b;
    // k2 = V(x1)
    interp_u(u, ubar, k2bx, NX, NY, dx, x1, y1, d0, d1);
    interp_v(v, vbar, k2by, NX, NY, dx, x1, y1, d2, d3);
    const double x1b = k2bx * ux1x + k2by * vx1x, y1b = k2bx * ux1y + k2by * vx1y;
    k1bx += -0.5 * dt * x1b;
    k1by += -0.5 * dt * y1b;
    // k1 = V(x0)
    interp_u(u, ubar, k1bx, NX, NY, dx, x0, y0, d0, d1);
    interp_v(v, vbar, k1by, NX, NY, dx, x0, y0, d2, d3);
}

// E^T for one layer L of one face grid (layers as Array2D::extrapolate left them).
__global__ void k_extrap_adjoint(double* mu, const uint32_t* __restrict__ layer, int W, int H, uint32_t L) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= W || j >= H) return;
    const size_t c = (size_t)j * W + i;
    if (layer[c] != L) return;
    const size_t nb[4] = {c - 1, c + 1, c - W, c + W};
    const bool in[4] = {i > 0, i < W - 1, j > 0, j < H - 1};
    int count = 0;
    for (int k = 0; k < 4; k++)
        if (in[k] && layer[nb[k]] < L) count++;
    const double m = mu[c];
    mu[c] = 0.0;
    if (count == 0 || m == 0.0) return;
    const double share = m / count;
    for (int k = 0; k < 4; k++)
        if (in[k] && layer[nb[k]] < L) atomicAdd(mu + nb[k], share);
}

// Class of a face in updateVelocity's loop (src/FluidSim2D.cpp:478-541) on a
// grid without EMPTY cells: 0 kept (never visited), 1 fluid-fluid, 2 zeroed
// (next to a solid), 3 no fluid side (extrapolated).
__device__ __forceinline__ int u_face_class(const uint8_t* __restrict__ cell, int NX, int i, int j) {
    if (i == NX) return 0;
    const uint8_t a = i > 0 ? cell[(size_t)j * NX + i - 1] : kSolid, b = cell[(size_t)j * NX + i];
    if (!((i > 0 && a == kFluid) || b == kFluid)) return 3;
    if (i == 0 || a == kSolid || b == kSolid) return 2;
    return 1;
}
__device__ __forceinline__ int v_face_class(const uint8_t* __restrict__ cell, int NX, int NY, int i, int j) {
    if (j == NY) return 0;
    const uint8_t a = j > 0 ? cell[(size_t)(j - 1) * NX + i] : kSolid, b = cell[(size_t)j * NX + i];
    if (!((j > 0 && a == kFluid) || b == kFluid)) return 3;
    if (j == 0 || a == kSolid || b == kSolid) return 2;
    return 1;
}

// W^T on the faces: u*bar from mu (after E^T).  Faces of class 3 that the
// extrapolation did not overwrite (never reached, or deeper than the band
// limit `lim`) keep their value in the forward, so they pass their adjoint
// through.
__global__ void k_update_adjoint(const uint8_t* __restrict__ cell, const double* __restrict__ mu_u,
                                 const double* __restrict__ mu_v, const uint32_t* __restrict__ lay_u,
                                 const uint32_t* __restrict__ lay_v, double* sbar_u, double* sbar_v, int NX, int NY,
                                 uint32_t lim) {
    const int comp = blockIdx.z;
    const int W = comp == 0 ? NX + 1 : NX, H = comp == 0 ? NY : NY + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= W || j >= H) return;
    const size_t c = (size_t)j * W + i;
    const int cls = comp == 0 ? u_face_class(cell, NX, i, j) : v_face_class(cell, NX, NY, i, j);
    const double m = comp == 0 ? mu_u[c] : mu_v[c];
    const uint32_t L = comp == 0 ? lay_u[c] : lay_v[c];
    const double s = (cls == 0 || cls == 1 || (cls == 3 && L > lim)) ? m : 0.0;
    if (comp == 0) sbar_u[c] = s;
    else sbar_v[c] = s;
}

// pbar = -dt/(rho dx) G^T mu over the fluid-fluid faces (per cell).
__global__ void k_pbar(const uint8_t* __restrict__ cell, const double* __restrict__ mu_u,
                       const double* __restrict__ mu_v, double* pbar, int NX, int NY, double scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= NX || j >= NY) return;
    const size_t c = (size_t)j * NX + i;
    double s = 0.0;
    if (cell[c] == kFluid) {
        const int U = NX + 1;
        if (u_face_class(cell, NX, i, j) == 1) s -= mu_u[(size_t)j * U + i];
        if (u_face_class(cell, NX, i + 1, j) == 1) s += mu_u[(size_t)j * U + i + 1];
        if (v_face_class(cell, NX, NY, i, j) == 1) s -= mu_v[(size_t)j * NX + i];
        if (v_face_class(cell, NX, NY, i, j + 1) == 1) s += mu_v[(size_t)(j + 1) * NX + i];
    }
    pbar[c] = scale * s;
}

// u*bar += B^T bbar: rhs(i,j) = -(1/dx) (u(i+1)[i+1 not solid] - u(i)[i-1 not
// solid] + v(j+1)[..] - v(j)[..]) on fluid cells.
__global__ void k_div_adjoint(const uint8_t* __restrict__ cell, const double* __restrict__ bbar, double* sbar_u,
                              double* sbar_v, int NX, int NY, double inv_dx) {
    const int comp = blockIdx.z;
    const int W = comp == 0 ? NX + 1 : NX, H = comp == 0 ? NY : NY + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= W || j >= H) return;
    double s = 0.0;
    if (comp == 0) {
        if (i < NX && cell[(size_t)j * NX + i] == kFluid && i > 0 && cell[(size_t)j * NX + i - 1] != kSolid)
            s += inv_dx * bbar[(size_t)j * NX + i];
        if (i > 0 && cell[(size_t)j * NX + i - 1] == kFluid && i < NX && cell[(size_t)j * NX + i] != kSolid)
            s -= inv_dx * bbar[(size_t)j * NX + i - 1];
        sbar_u[(size_t)j * W + i] += s;
    } else {
        if (j < NY && cell[(size_t)j * NX + i] == kFluid && j > 0 && cell[(size_t)(j - 1) * NX + i] != kSolid)
            s += inv_dx * bbar[(size_t)j * NX + i];
        if (j > 0 && cell[(size_t)(j - 1) * NX + i] == kFluid && j < NY && cell[(size_t)j * NX + i] != kSolid)
            s -= inv_dx * bbar[(size_t)(j - 1) * NX + i];
        sbar_v[(size_t)j * W + i] += s;
    }
}

__global__ void k_max_layer(const uint32_t* __restrict__ lay, size_t n, unsigned int* out) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n && lay[c] != kUnknown) atomicMax(out, lay[c]);
}

// sum of (a - b)^2 over n entries into partial sums, then one block adds them
__global__ void k_sqdiff(const double* __restrict__ a, const double* __restrict__ b, size_t n, double* partial) {
    __shared__ double sh[32];
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double d = c < n ? (a[c] - b[c]) * (a[c] - b[c]) : 0.0;
    d = block_sum(d, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = d;
}
__global__ void k_sum_partials(const double* __restrict__ partial, int n, double* out) {
    __shared__ double sh[32];
    double s = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) s += partial[k];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) *out = s;
}
__global__ void k_loss_grad(const double* __restrict__ a, const double* __restrict__ b, size_t n, double inv_l,
                            double* g) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n) g[c] = (a[c] - b[c]) * inv_l;
}

}  // namespace

// ---- host driver ----

struct Rollout {
    int steps = 0, every = 0, nck = 0;
    size_t NU = 0, NV = 0;
    double* ck = nullptr;     // nck states (u then v), the state before steps 0, every, 2 every, ...
    double* seg = nullptr;    // `every` states of the segment being reversed
    double *lu = nullptr, *lv = nullptr;    // adjoint of the state
    double *sbu = nullptr, *sbv = nullptr;  // adjoint of the advected state u*
    double* pbar = nullptr;                 // adjoint of the pressure (cells)
    double* dscr = nullptr;
    double loss = 0;
    uint32_t umax = 0, vmax = 0, lim = 0;
    int last_seg_stored = 0;  // the forward pass left the last segment's states in `seg`
    bool ready = false;       // a forward pass completed
};

namespace {

int ro_alloc(double** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, (n ? n : 1) * sizeof(double));
    if (e != cudaSuccess) {
        *p = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", n * sizeof(double), cudaGetErrorString(e));
        return FS2D_ERR_ALLOC;
    }
    return 0;
}

// One forward step of the rollout: the semi-Lagrangian frame's velocity
// stages (applySemiLagrangianAdvection, applyGravity, applyProjection with
// the handle's precision, updateVelocity; src/FluidSim2D.cpp:100-113).  The
// labels are fixed, so createWaterLevelSet and applyAdvection (particles)
// do not enter.
int forward_step(Sim* s) {
    int rc = sl_advect(s);
    if (!rc) rc = apply_gravity(s);
    int status = 0;
    if (!rc) rc = s->opt.precision != FS2D_PRECISION_FP64 ? projection_mixed(s, &status) : projection(s, &status);
    if (!rc) rc = update_velocity(s);
    if (!rc && status) {
        set_error("rollout: the pressure solve hit its iteration cap");
        rc = status;
    }
    return rc;
}

int copy_state_out(Sim* s, double* dst) {
    FS2D_CUDA(cudaMemcpyAsync(dst, s->u, s->NU * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(dst + s->NU, s->v, s->NV * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    return 0;
}
int copy_state_in(Sim* s, const double* src) {
    FS2D_CUDA(cudaMemcpyAsync(s->u, src, s->NU * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(s->v, src + s->NU, s->NV * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    return 0;
}

// Deepest extrapolation layer of each face grid (masks of the last updateVelocity).
int deepest_layers(Sim* s, uint32_t* umax, uint32_t* vmax) {
    unsigned int* d = s->max_layer + 8;
    FS2D_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned int), s->stream));
    FS2D_LAUNCH(s, k_max_layer, blocks_for(s->NU, kAT), kAT, 0, s->mask_u, s->NU, d);
    FS2D_LAUNCH(s, k_max_layer, blocks_for(s->NV, kAT), kAT, 0, s->mask_v, s->NV, d + 1);
    unsigned int h[2] = {0, 0};
    FS2D_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    *umax = h[0];
    *vmax = h[1];
    return 0;
}

// One reverse step: on entry ro->lu/lv = dL/du_{k+1}; on exit dL/du_k, with
// `uk` the state u_k (u then v).
int adjoint_step(Sim* s, Rollout* ro, const double* uk) {
    const int NX = s->NX, NY = s->NY;
    double *lu = ro->lu, *lv = ro->lv;
    for (uint32_t L = ro->lim < ro->umax ? ro->lim : ro->umax; L >= 1; L--)
        FS2D_LAUNCH(s, k_extrap_adjoint, dim3(blocks_for(NX + 1, 128), NY), 128, 0, lu, s->mask_u, NX + 1, NY, L);
    for (uint32_t L = ro->lim < ro->vmax ? ro->lim : ro->vmax; L >= 1; L--)
        FS2D_LAUNCH(s, k_extrap_adjoint, dim3(blocks_for(NX, 128), NY + 1), 128, 0, lv, s->mask_v, NX, NY + 1, L);
    const dim3 gf(blocks_for(NX + 1, 128), NY + 1, 2);
    FS2D_LAUNCH(s, k_update_adjoint, gf, 128, 0, s->cell, lu, lv, s->mask_u, s->mask_v, ro->sbu, ro->sbv, NX, NY,
                ro->lim);
    FS2D_LAUNCH(s, k_pbar, dim3(blocks_for(NX, 128), NY), 128, 0, s->cell, lu, lv, ro->pbar, NX, NY,
                s->dt / (s->rho * s->dx));
    int status = 0;
    int rc = projection_solve_custom(s, ro->pbar, &status);
    if (rc) return rc;
    if (status) {
        set_error("rollout: the adjoint pressure solve hit its iteration cap");
        return status;
    }
    FS2D_LAUNCH(s, k_div_adjoint, gf, 128, 0, s->cell, s->p, ro->sbu, ro->sbv, NX, NY, 1.0 / s->dx);
    FS2D_CUDA(cudaMemsetAsync(lu, 0, s->NU * sizeof(double), s->stream));
    FS2D_CUDA(cudaMemsetAsync(lv, 0, s->NV * sizeof(double), s->stream));
    FS2D_LAUNCH(s, k_sl_adjoint, gf, 128, 0, uk, uk + s->NU, ro->sbu, ro->sbv, lu, lv, NX, NY, s->dx, s->dt);
    return 0;
}

int check_scene(Sim* s) {
    if (s->mode != FS2D_SEMILAGRANGIAN) {
        set_error("rollout: the scene must be in semi-Lagrangian mode");
        return FS2D_ERR_INVALID;
    }
    std::vector<uint8_t> cell(s->N);
    FS2D_CUDA(cudaMemcpyAsync(cell.data(), s->cell, s->N, cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    for (size_t c = 0; c < s->N; c++)
        if (cell[c] == kEmpty) {
            set_error("rollout: cell (%zu, %zu) is EMPTY; the differentiable rollout needs a box without air",
                      c % s->NX, c / s->NX);
            return FS2D_ERR_INVALID;
        }
    return 0;
}

}  // namespace

// E^T of one face grid, in place: the layers as the last extrapolation left
// them in `layer`, deepest first, layers above `lim` (a band limit) left out.
int extrap_adjoint(Sim* s, double* mu, const uint32_t* layer, int W, int H, uint32_t lim) {
    const size_t n = (size_t)W * H;
    unsigned int* d = s->max_layer + 10;
    FS2D_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned int), s->stream));
    FS2D_LAUNCH(s, k_max_layer, blocks_for(n, kAT), kAT, 0, layer, n, d);
    unsigned int h = 0;
    FS2D_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    for (uint32_t L = h < lim ? h : lim; L >= 1; L--)
        FS2D_LAUNCH(s, k_extrap_adjoint, dim3(blocks_for(W, 128), H), 128, 0, mu, layer, W, H, L);
    return 0;
}

void rollout_free(Sim* s) {
    Rollout* ro = s->ro;
    if (!ro) return;
    double* ptrs[] = {ro->ck, ro->seg, ro->lu, ro->lv, ro->sbu, ro->sbv, ro->pbar, ro->dscr};
    for (double* p : ptrs)
        if (p) cudaFree(p);
    delete ro;
    s->ro = nullptr;
}

// Runs `steps` forward steps from (u0, v0), keeping the state before every
// `every`-th step, and returns sqrt(sum over faces of (u_T - ut)^2 + (v_T - vt)^2).
// Pointers may be host or device memory.
int rollout_forward(Sim* s, int steps, int every, const double* u0, const double* v0, const double* ut,
                    const double* vt, double* loss) {
    if (steps < 1 || every < 0 || !u0 || !v0 || !ut || !vt) {
        set_error("rollout: steps >= 1, every >= 0 and u0, v0, uTarget, vTarget are required");
        return FS2D_ERR_INVALID;
    }
    if (every == 0) every = (int)ceil(sqrt((double)steps));
    if (every > steps) every = steps;
    int rc = check_scene(s);
    if (rc) return rc;
    const int nck = (steps + every - 1) / every;
    Rollout* ro = s->ro;
    if (!ro || ro->steps != steps || ro->every != every || ro->NU != s->NU || ro->NV != s->NV) {
        rollout_free(s);
        ro = s->ro = new Rollout;
        ro->steps = steps;
        ro->every = every;
        ro->nck = nck;
        ro->NU = s->NU;
        ro->NV = s->NV;
        const size_t F = s->NU + s->NV;
        if ((rc = ro_alloc(&ro->ck, (size_t)nck * F)) || (rc = ro_alloc(&ro->seg, (size_t)every * F)) ||
            (rc = ro_alloc(&ro->lu, s->NU)) || (rc = ro_alloc(&ro->lv, s->NV)) || (rc = ro_alloc(&ro->sbu, s->NU)) ||
            (rc = ro_alloc(&ro->sbv, s->NV)) || (rc = ro_alloc(&ro->pbar, s->N)) || (rc = ro_alloc(&ro->dscr, 1))) {
            rollout_free(s);
            return rc;
        }
    }
    ro->ready = false;
    const size_t F = s->NU + s->NV;
    FS2D_CUDA(cudaMemcpyAsync(s->u, u0, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(s->v, v0, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    // targets go to the gradient buffers, replaced by dL/du_T at the end
    FS2D_CUDA(cudaMemcpyAsync(ro->lu, ut, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(ro->lv, vt, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    const int last_start = (nck - 1) * every;
    for (int k = 0; k < steps; k++) {
        if (k % every == 0 && (rc = copy_state_out(s, ro->ck + (size_t)(k / every) * F))) return rc;
        if (k > last_start && (rc = copy_state_out(s, ro->seg + (size_t)(k - last_start) * F))) return rc;
        if ((rc = forward_step(s))) return rc;
    }
    // loss and its gradient at u_T
    const unsigned bu = blocks_for(s->NU, kAT), bv = blocks_for(s->NV, kAT);
    FS2D_LAUNCH(s, k_sqdiff, bu, kAT, 0, s->u, ro->lu, s->NU, s->partial);
    FS2D_LAUNCH(s, k_sqdiff, bv, kAT, 0, s->v, ro->lv, s->NV, s->partial + bu);
    FS2D_LAUNCH(s, k_sum_partials, 1, 1024, 0, s->partial, (int)(bu + bv), ro->dscr);
    double sq = 0;
    FS2D_CUDA(cudaMemcpyAsync(&sq, ro->dscr, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    ro->loss = sqrt(sq);
    const double inv = ro->loss > 0 ? 1.0 / ro->loss : 0.0;
    FS2D_LAUNCH(s, k_loss_grad, bu, kAT, 0, s->u, ro->lu, s->NU, inv, ro->lu);
    FS2D_LAUNCH(s, k_loss_grad, bv, kAT, 0, s->v, ro->lv, s->NV, inv, ro->lv);
    if ((rc = deepest_layers(s, &ro->umax, &ro->vmax))) return rc;
    ro->lim = s->opt.extrapolate_band > 0 ? (uint32_t)s->opt.extrapolate_band : 0xFFFFFFFEu;
    ro->last_seg_stored = 1;
    ro->ready = true;
    *loss = ro->loss;
    return 0;
}

// dL/du_0 and dL/dv_0 of the last rollout_forward, written to gu, gv (host or
// device).  The segments are recomputed from their checkpoints, newest first.
int rollout_backward(Sim* s, double* gu, double* gv) {
    Rollout* ro = s->ro;
    if (!ro || !ro->ready || !gu || !gv) {
        set_error("rollout: call fs2d_forward first; gradU0 and gradV0 are required");
        return FS2D_ERR_INVALID;
    }
    const size_t F = s->NU + s->NV;
    int rc;
    for (int seg = ro->nck - 1; seg >= 0; seg--) {
        const int start = seg * ro->every;
        const int len = std::min(ro->every, ro->steps - start);
        const double* ck = ro->ck + (size_t)seg * F;
        if (!(seg == ro->nck - 1 && ro->last_seg_stored)) {
            if ((rc = copy_state_in(s, ck))) return rc;
            for (int m = 1; m < len; m++) {
                if ((rc = forward_step(s))) return rc;
                if ((rc = copy_state_out(s, ro->seg + (size_t)m * F))) return rc;
            }
        }
        for (int m = len - 1; m >= 0; m--)
            if ((rc = adjoint_step(s, ro, m == 0 ? ck : ro->seg + (size_t)m * F))) return rc;
    }
    FS2D_CUDA(cudaMemcpyAsync(gu, ro->lu, s->NU * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(gv, ro->lv, s->NV * sizeof(double), cudaMemcpyDefault, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    ro->ready = false;   // the adjoint buffers now hold dL/du_0
    return 0;
}

}  // namespace fs2d
