// render.cu — headless render-data export: what the reference's renderer
// gathers from the simulation each frame (FluidRenderer2D::updateBuffers,
// demo/FluidRenderer2D.cpp:435-486), computed on the device into
// caller-owned device buffers instead of host vectors uploaded to OpenGL.
//
//   water / solid cells   corner (i dx, j dx) of every FLUID / SOLID cell, in
//                         the row-major order of FluidSim2D::iterate
//                         (include/FluidSim2D.h:152-159), as float pairs;
//   cell velocities       for i < NX-1, j < NY-1: the centre ((i+.5)dx,
//                         (j+.5)dx) and centre + dt * velInterp(centre);
//   pressure cells        corner and sigmoid(0.01 p) of every cell with p != 0;
//   particle lines        each particle and particle + dt * velInterp(particle),
//                         with the renderer's float casts;
//   level set             sigmoid(100 phi) of every cell (100 phi formed in double).
//
// Compaction keeps the reference's order with an exclusive scan of the
// selection flags.  The FP64 interpolation (compiled with --fmad=false) is
// the simulation's own velInterp; results are cast to float as the
// renderer casts them.  sigmoid is 1 / (1 + e^-x) in FP32.
#include <cuda_runtime.h>
#include <math.h>
#include "fs2d_device.cuh"

namespace fs2d {
namespace {

__device__ __forceinline__ float sigmoidf(float x) { return 1.0f / (1.0f + expf(-x)); }

__global__ void k_flag_cells(const uint8_t* __restrict__ cell, uint32_t* flags, size_t n, uint8_t label) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n) flags[c] = cell[c] == label ? 1u : 0u;
}

__global__ void k_flag_pressure(const double* __restrict__ p, uint32_t* flags, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n) flags[c] = p[c] != 0.0 ? 1u : 0u;
}

// After the scan: offs[c] = number of selected cells before c, offs[n] = total.
__global__ void k_scatter_cells(const uint8_t* __restrict__ cell, const uint32_t* __restrict__ offs, float2* out,
                                size_t cap, int NX, size_t n, uint8_t label, double dx) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n || cell[c] != label) return;
    const uint32_t k = offs[c];
    if (k >= cap) return;
    const int i = (int)(c % NX), j = (int)(c / NX);
    out[k] = make_float2((float)(i * dx), (float)(j * dx));
}

__global__ void k_scatter_pressure(const double* __restrict__ p, const uint32_t* __restrict__ offs, float2* loc,
                                   float* val, size_t cap, int NX, size_t n, double dx) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n || p[c] == 0.0) return;
    const uint32_t k = offs[c];
    if (k >= cap) return;
    const int i = (int)(c % NX), j = (int)(c / NX);
    if (loc) loc[k] = make_float2((float)(i * dx), (float)(j * dx));
    if (val) val[k] = sigmoidf(0.01f * (float)p[c]);
}

__global__ void k_cell_vels(const double* __restrict__ u, const double* __restrict__ v, float2* out, int NX, int NY,
                            double dx, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= NX - 1 || j >= NY - 1) return;
    const double x = (i + 0.5) * dx, y = (j + 0.5) * dx;
    const double vx = vel_interp_u(u, NX, NY, dx, x, y);
    const double vy = vel_interp_v(v, NX, NY, dx, x, y);
    const size_t k = 2 * ((size_t)j * (NX - 1) + i);
    out[k] = make_float2((float)x, (float)y);
    out[k + 1] = make_float2((float)(x + vx * dt), (float)(y + vy * dt));
}

__global__ void k_particle_lines(const double2* __restrict__ pos, size_t np, const double* __restrict__ u,
                                 const double* __restrict__ v, float2* out, int NX, int NY, double dx, double dt) {
    size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= np) return;
    const double2 p = pos[e];
    const double vx = vel_interp_u(u, NX, NY, dx, p.x, p.y);
    const double vy = vel_interp_v(v, NX, NY, dx, p.x, p.y);
    out[2 * e] = make_float2((float)p.x, (float)p.y);
    out[2 * e + 1] = make_float2((float)p.x + (float)dt * (float)vx, (float)p.y + (float)dt * (float)vy);
}

__global__ void k_phi_values(const double* __restrict__ phi, float* out, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c < n) out[c] = sigmoidf((float)(100.0 * phi[c]));   // the product is formed in double, as in the renderer
}

}  // namespace

int exclusive_scan_u32(Sim* s, uint32_t* data, size_t n);

int render_export(Sim* s, fs2d_render* r) {
    const int NX = s->NX, NY = s->NY, T = 256;
    const size_t N = s->N;
    uint32_t* flags = s->cnt_u;   // N + 1 entries of scratch (P2G counts are free between frames)
    unsigned int total = 0;
    auto count_of = [&](size_t* out) -> int {
        FS2D_CUDA(cudaMemcpyAsync(&total, flags + N, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->stream));
        FS2D_CUDA(cudaStreamSynchronize(s->stream));
        *out = total;
        return 0;
    };
    int rc;
    if (r->waterCells || r->waterCount) {
        FS2D_LAUNCH(s, k_flag_cells, blocks_for(N, T), T, 0, s->cell, flags, N, kFluid);
        if ((rc = exclusive_scan_u32(s, flags, N))) return rc;
        if (r->waterCells)
            FS2D_LAUNCH(s, k_scatter_cells, blocks_for(N, T), T, 0, s->cell, flags, (float2*)r->waterCells,
                        r->waterCap, NX, N, kFluid, s->dx);
        size_t n = 0;
        if ((rc = count_of(&n))) return rc;
        if (r->waterCount) *r->waterCount = n;
    }
    if (r->solidCells || r->solidCount) {
        FS2D_LAUNCH(s, k_flag_cells, blocks_for(N, T), T, 0, s->cell, flags, N, kSolid);
        if ((rc = exclusive_scan_u32(s, flags, N))) return rc;
        if (r->solidCells)
            FS2D_LAUNCH(s, k_scatter_cells, blocks_for(N, T), T, 0, s->cell, flags, (float2*)r->solidCells,
                        r->solidCap, NX, N, kSolid, s->dx);
        size_t n = 0;
        if ((rc = count_of(&n))) return rc;
        if (r->solidCount) *r->solidCount = n;
    }
    if (r->pressureCells || r->pressureValues || r->pressureCount) {
        FS2D_LAUNCH(s, k_flag_pressure, blocks_for(N, T), T, 0, s->p, flags, N);
        if ((rc = exclusive_scan_u32(s, flags, N))) return rc;
        if (r->pressureCells || r->pressureValues)
            FS2D_LAUNCH(s, k_scatter_pressure, blocks_for(N, T), T, 0, s->p, flags, (float2*)r->pressureCells,
                        r->pressureValues, r->pressureCap, NX, N, s->dx);
        size_t n = 0;
        if ((rc = count_of(&n))) return rc;
        if (r->pressureCount) *r->pressureCount = n;
    }
    if (r->cellVels && NX > 1 && NY > 1) {
        dim3 g(blocks_for(NX - 1, 128), NY - 1);
        FS2D_LAUNCH(s, k_cell_vels, g, 128, 0, s->u, s->v, (float2*)r->cellVels, NX, NY, s->dx, s->dt);
    }
    if (r->particleLines && s->np > 0)
        FS2D_LAUNCH(s, k_particle_lines, blocks_for(s->np, T), T, 0, s->pos, s->np, s->u, s->v,
                    (float2*)r->particleLines, NX, NY, s->dx, s->dt);
    if (r->phiValues) FS2D_LAUNCH(s, k_phi_values, blocks_for(N, T), T, 0, s->phi, r->phiValues, N);
    FS2D_CUDA(cudaStreamSynchronize(s->stream));
    return 0;
}

}  // namespace fs2d
