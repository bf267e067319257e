// advect.cu — advection and body forces (FP64, exact operation order).
//
//   FluidSim2D::applySemiLagrangianAdvection  src/FluidSim2D.cpp:206-235
//   FluidSim2D::applyGravity                  src/FluidSim2D.cpp:237-250
//   FluidSim2D::applyAdvection                src/FluidSim2D.cpp:570-604
// Compiled with --fmad=false.
//
// Semi-Lagrangian advection is double-buffered: every face traces back
// through, and samples, the velocity as it was before the stage.  The
// reference overwrites mac.u while later faces (and all v faces) still read
// it, which makes its result depend on the loop order; a parallel GPU
// cannot reproduce that, and the oracle provides both variants.
#include <cuda_runtime.h>
#include <cstring>
#include "fs2d_device.cuh"

namespace fs2d {
namespace {

// RK3 backtrace with Ralston weights 2/9, 3/9, 4/9 through (u0, v0), then
// clampPos (src/FluidSim2D.cpp:212-217).
__device__ __forceinline__ void backtrace(const double* __restrict__ u0, const double* __restrict__ v0, int NX,
                                          int NY, double dx, double dt, double xpx, double xpy, double& ox,
                                          double& oy) {
    double k1x = vel_interp_u(u0, NX, NY, dx, xpx, xpy), k1y = vel_interp_v(v0, NX, NY, dx, xpx, xpy);
    double ax = xpx - 0.5 * dt * k1x, ay = xpy - 0.5 * dt * k1y;
    double k2x = vel_interp_u(u0, NX, NY, dx, ax, ay), k2y = vel_interp_v(v0, NX, NY, dx, ax, ay);
    double bx = xpx - 0.75 * dt * k2x, by = xpy - 0.75 * dt * k2y;
    double k3x = vel_interp_u(u0, NX, NY, dx, bx, by), k3y = vel_interp_v(v0, NX, NY, dx, bx, by);
    ox = xpx - ((2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x);
    oy = xpy - ((2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y);
    clamp_pos(NX, NY, dx, ox, oy);
}

// One thread per face; blockIdx.z selects the u (0) or v (1) grid.
__global__ void k_sl_advect(const double* __restrict__ u0, const double* __restrict__ v0, double* u, double* v, int NX,
                            int NY, double dx, double dt) {
    int comp = blockIdx.z;
    int W = comp == 0 ? NX + 1 : NX;
    int H = comp == 0 ? NY : NY + 1;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= W || j >= H) return;
    double x, y;
    if (comp == 0) {
        x = (double)i * dx;
        y = ((double)j + 0.5) * dx;
    } else {
        x = ((double)i + 0.5) * dx;
        y = (double)j * dx;
    }
    double nx, ny;
    backtrace(u0, v0, NX, NY, dx, dt, x, y, nx, ny);
    if (comp == 0) u[(size_t)j * W + i] = vel_interp_u(u0, NX, NY, dx, nx, ny);
    else v[(size_t)j * W + i] = vel_interp_v(v0, NX, NY, dx, nx, ny);
}

__global__ void k_gravity(double* u, size_t nu, double du, double* v, size_t nv, double dv) {
    size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k < nu) u[k] += du;
    if (k < nv) v[k] += dv;
}

// Particle RK3 forward through the grid velocity (src/FluidSim2D.cpp:588-603).
// A non-finite result sets bit 1 of *err (the reference exits instead).
__global__ void k_advect_particles(double2* pos, size_t np, const double* __restrict__ u, const double* __restrict__ v,
                                   int NX, int NY, double dx, double dt, int* err) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    double2 p = pos[e];
    double k1x = vel_interp_u(u, NX, NY, dx, p.x, p.y), k1y = vel_interp_v(v, NX, NY, dx, p.x, p.y);
    double ax = p.x + 0.5 * dt * k1x, ay = p.y + 0.5 * dt * k1y;
    double k2x = vel_interp_u(u, NX, NY, dx, ax, ay), k2y = vel_interp_v(v, NX, NY, dx, ax, ay);
    double bx = p.x + 0.75 * dt * k2x, by = p.y + 0.75 * dt * k2y;
    double k3x = vel_interp_u(u, NX, NY, dx, bx, by), k3y = vel_interp_v(v, NX, NY, dx, bx, by);
    double nx = p.x + (2. / 9.) * dt * k1x + (3. / 9.) * dt * k2x + (4. / 9.) * dt * k3x;
    double ny = p.y + (2. / 9.) * dt * k1y + (3. / 9.) * dt * k2y + (4. / 9.) * dt * k3y;
    clamp_pos(NX, NY, dx, nx, ny);
    if (!isfinite(nx) || !isfinite(ny)) atomicOr(err, 2);
    pos[e] = make_double2(nx, ny);
}

}  // namespace

int sl_advect(Sim* s) {
    FS2D_CUDA(cudaMemcpyAsync(s->u0, s->u, s->NU * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    FS2D_CUDA(cudaMemcpyAsync(s->v0, s->v, s->NV * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    dim3 grid(blocks_for(s->NX + 1, 128), s->NY + 1, 2);
    FS2D_LAUNCH(s, k_sl_advect, grid, 128, 0, s->u0, s->v0, s->u, s->v, s->NX, s->NY, s->dx, s->dt);
    return 0;
}

int apply_gravity(Sim* s) {
    size_t n = s->NU > s->NV ? s->NU : s->NV;
    FS2D_LAUNCH(s, k_gravity, blocks_for(n, 256), 256, 0, s->u, s->NU, s->dt * s->gx, s->v, s->NV, s->dt * s->gy);
    return 0;
}

namespace {

// applyAdvection's CFL check (src/FluidSim2D.cpp:571-585): c = (vx + vy) *
// dt / dx.  For c > 0 the order of the bit patterns is the order of the
// values, so an integer maximum finds the largest c and an integer minimum
// the first particle that reaches it, whatever the thread order.
__device__ __forceinline__ double cfl_of(double2 v, double dt, double dx) { return (v.x + v.y) * dt / dx; }

__global__ void k_cfl_max(const double2* __restrict__ vel, size_t np, double dt, double dx,
                          unsigned long long* best) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    const double c = cfl_of(vel[e], dt, dx);
    if (c > 0.0) atomicMax(best, (unsigned long long)__double_as_longlong(c));
}

__global__ void k_cfl_first(const double2* __restrict__ vel, size_t np, double dt, double dx,
                            const unsigned long long* __restrict__ best, unsigned long long* first) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    const double c = cfl_of(vel[e], dt, dx);
    if (c > 0.0 && (unsigned long long)__double_as_longlong(c) == *best) atomicMin(first, (unsigned long long)e);
}

}  // namespace

int cfl_check(Sim* s, double* cfl, long long* particle) {
    // two words of the reduction scratch: the best bit pattern (0: none) and its first particle
    unsigned long long* w = reinterpret_cast<unsigned long long*>(s->partial);
    FS2D_CUDA(cudaMemsetAsync(w, 0, sizeof(unsigned long long), s->stream));
    FS2D_CUDA(cudaMemsetAsync(w + 1, 0xff, sizeof(unsigned long long), s->stream));
    if (s->np) {
        FS2D_LAUNCH(s, k_cfl_max, blocks_for(s->np, 256), 256, 0, s->vel, s->np, s->dt, s->dx, w);
        FS2D_LAUNCH(s, k_cfl_first, blocks_for(s->np, 256), 256, 0, s->vel, s->np, s->dt, s->dx, w, w + 1);
    }
    unsigned long long h[2] = {0, 0};
    FS2D_CUDA(cudaMemcpyAsync(h, w, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    if (h[0] == 0) {
        *cfl = 0.0;
        *particle = -1;
    } else {
        std::memcpy(cfl, &h[0], sizeof(double));
        *particle = (long long)h[1];
    }
    return 0;
}

int advect_particles(Sim* s) {
    if (s->np == 0) return 0;
    FS2D_LAUNCH(s, k_advect_particles, blocks_for(s->np, 128), 128, 0, s->pos, s->np, s->u, s->v, s->NX, s->NY, s->dx,
                s->dt, s->err);
    return 0;
}

}  // namespace fs2d
