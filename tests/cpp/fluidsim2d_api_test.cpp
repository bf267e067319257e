// The reference's C++ API (FluidSim2D_gb300.hpp) on the GPU library: a dam
// break advanced with runFrame() and, in a second instance, with the stage
// methods called one by one in runFrame's order (src/FluidSim2D.cpp:94-138),
// must give bit-identical host mirrors; diagnostics and the host-side MAC
// helpers must be usable on the mirrored fields; perfCounter must fill as
// the reference's does and save the same perf.csv as the library.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "FluidSim2D_gb300.hpp"

static std::vector<FluidCellType> dam_break(int nx, int ny) {
    std::vector<FluidCellType> c((size_t)nx * ny, FS_EMPTY);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const double x = (i + 0.5) / nx, y = (j + 0.5) / ny;
            if (i == 0 || j == 0 || i == nx - 1 || j == ny - 1) c[(size_t)j * nx + i] = FS_SOLID;
            else if (x < 0.4 && y < 0.6) c[(size_t)j * nx + i] = FS_FLUID;
        }
    return c;
}

static bool same(const void* a, const void* b, size_t n) { return std::memcmp(a, b, n) == 0; }

int main(int argc, char** argv) {
    const int nx = 64, ny = 48;
    const FluidSimMode mode = (argc > 1 && std::strcmp(argv[1], "pic") == 0) ? FS_PICFLIP : FS_SEMILAGRANGIAN;
    std::vector<FluidCellType> cells = dam_break(nx, ny);
    FluidSim2DConfig cfg{nx, ny, 2, 1.0 / 120, 1.0 / nx, 997.0, 0.0, -9.8, mode, 0.05, cells.data()};
    fs2d_options opt;
    fs2d_default_options(&opt);
    opt.use_seed = 1;
    opt.seed = 7;

    FluidSim2D a = FluidSim2D::create(cfg, &opt);
    FluidSim2D b = FluidSim2D::create(cfg, &opt);
    if (a.particles.size == 0 || a.particles.size != b.particles.size) {
        std::printf("FAIL particle count %zu %zu\n", a.particles.size, b.particles.size);
        return 1;
    }
    for (int f = 0; f < 5; f++) {
        a.runFrame();
        b.createWaterLevelSet();
        if (mode == FS_PICFLIP) b.transferVelocityToGrid();
        else b.applySemiLagrangianAdvection();
        b.applyGravity();
        b.createSolidLevelSet();
        b.applyProjection();
        b.updateVelocity();
        if (mode == FS_PICFLIP) b.updateParticleVelocities();
        b.applyAdvection();
    }
    const size_t nu = (size_t)(nx + 1) * ny, nv = (size_t)nx * (ny + 1), nc = (size_t)nx * ny;
    bool ok = same(a.mac.u.data, b.mac.u.data, nu * 8) && same(a.mac.v.data, b.mac.v.data, nv * 8) &&
              same(a.p.data, b.p.data, nc * 8) && same(a.cell.data, b.cell.data, nc) &&
              same(a.waterLevelSet.phi.data, b.waterLevelSet.phi.data, nc * 8) &&
              same(a.particles.data, b.particles.data, a.particles.size * 16);
    if (!ok) {
        std::printf("FAIL runFrame and the stage sequence differ\n");
        return 1;
    }
    int fluid = 0;
    for (size_t k = 0; k < nc; k++) fluid += a.cell.data[k] == FS_FLUID;
    const double vmax = a.maxVelocity();
    const vec2d c = a.getGridCenter();
    const vec2d w = a.mac.velInterp(c);
    if (fluid == 0 || !(vmax > 0 && std::isfinite(vmax)) || !std::isfinite(w.x) || !std::isfinite(w.y) ||
        a.waterVolumeData.size != 5 || !(a.waterVolume > 0)) {
        std::printf("FAIL fluid %d vmax %g volume %g history %zu\n", fluid, vmax, a.waterVolume, a.waterVolumeData.size);
        return 1;
    }
    // a host edit travels to the device with syncToDevice
    a.sync = FS2D_SYNC_ON_DEMAND;
    for (size_t k = 0; k < nu; k++) a.mac.u.data[k] = 0.0;
    for (size_t k = 0; k < nv; k++) a.mac.v.data[k] = 0.0;
    a.syncToDevice();
    a.syncToHost();
    for (size_t k = 0; k < nu; k++)
        if (a.mac.u.data[k] != 0.0) {
            std::printf("FAIL syncToDevice\n");
            return 1;
        }
    // the Performance panel of the reference's UI (demo/FluidRenderer2D.cpp:421-430)
    // reads perfCounter.sampleFinished, average and avgTimePerFrame
    a.sync = FS2D_SYNC_ON_DEMAND;
    if (a.perfCounter.sampleFinished) {
        std::printf("FAIL perfCounter finished after 5 frames\n");
        return 1;
    }
    for (int f = 5; f < 32; f++) a.runFrame();
    FluidSim2D* sim = &a;
    float sum = 0.0f;
    if (sim->perfCounter.sampleFinished) {
        for (int i = 0; i < (int)sim->perfCounter.average.size; i++) {
            if (!(sim->perfCounter.average[i] >= 0.0f)) {
                std::printf("FAIL stage %d: %f ms\n", i, sim->perfCounter.average[i]);
                return 1;
            }
            sum += sim->perfCounter.average[i];
        }
    }
    if (!sim->perfCounter.sampleFinished || (int)sim->perfCounter.average.size != a.numStages ||
        !(sim->perfCounter.avgTimePerFrame > 0.0f) || sum != sim->perfCounter.avgTimePerFrame) {
        std::printf("FAIL perfCounter finished %d stages %d avg %f\n", (int)sim->perfCounter.sampleFinished,
                    (int)sim->perfCounter.average.size, sim->perfCounter.avgTimePerFrame);
        return 1;
    }
    // the mirror's PerformanceCounter and the library's perf.csv writer agree byte for byte
    if (argc > 2) {
        const std::string dir = argv[2];
        const std::string p1 = dir + "/mirror_perf.csv", p2 = dir + "/lib_perf.csv";
        a.perfCounter.saveToFile(p1.c_str());
        if (fs2d_save_stats(a.device, p2.c_str(), nullptr) != FS2D_OK) {
            std::printf("FAIL fs2d_save_stats\n");
            return 1;
        }
        std::FILE* f1 = std::fopen(p1.c_str(), "rb");
        std::FILE* f2 = std::fopen(p2.c_str(), "rb");
        std::string b1, b2;
        for (int ch; f1 && (ch = std::fgetc(f1)) != EOF;) b1 += (char)ch;
        for (int ch; f2 && (ch = std::fgetc(f2)) != EOF;) b2 += (char)ch;
        if (f1) std::fclose(f1);
        if (f2) std::fclose(f2);
        if (b1.empty() || b1 != b2) {
            std::printf("FAIL perf.csv of the mirror (%zu bytes) and the library (%zu bytes) differ\n", b1.size(),
                        b2.size());
            return 1;
        }
    }
    a.free();
    b.free();
    std::printf("OK %s fluid=%d particles=%zu maxVelocity=%.6g\n", mode == FS_PICFLIP ? "pic" : "sl", fluid,
                (size_t)a.particles.size, vmax);
    return 0;
}
