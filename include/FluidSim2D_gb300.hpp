/*
 * FluidSim2D_gb300.hpp — the reference's C++ API (include/FluidSim2D.h,
 * MACGrid2D.h, Array2D.h) over the GB300 library's C ABI (fs2d.h).
 *
 * A program written against the reference's FluidSim2D includes this header
 * instead of FluidSim2D.h and links libfs2d.so: the types keep their names,
 * public fields and method names (FluidSim2D, FluidSim2DConfig, MACGrid2D,
 * Array2D<T>, LevelSet, FS_* enums, StageType), the simulation runs on the
 * GPU, and the public fields are host mirrors of the device state:
 *
 *   FS2D_SYNC_EVERY_FRAME (default)  runFrame() and every stage method
 *       download the state into the fields when they return, so reading
 *       `mac`, `p`, `cell`, `particles`, `waterLevelSet.phi` works as with
 *       the reference;
 *   FS2D_SYNC_ON_DEMAND  nothing is downloaded until syncToHost().
 *
 * After changing a field on the host (mac.u/v, particles, ...) call
 * syncToDevice() before the next frame.  gravity, picFlipAlpha and dt are
 * pushed to the device at every frame and stage call.
 *
 * Errors follow the reference: a failing create or frame logs the library's
 * message and exits the process (the reference exit()s on its errors); a
 * pressure solve that hits its iteration cap logs and continues, as the
 * reference's does.  lastStatus holds the status of the last call.
 *
 * Define FS2D_GB300_NO_VEC_TYPES when the program already has the
 * reference's vec2d and Vec<T> (altmath / altlib); otherwise this header
 * provides minimal versions with the members the API uses.
 */
#ifndef FLUIDSIM2D_GB300_HPP
#define FLUIDSIM2D_GB300_HPP

#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "fs2d.h"

#ifndef FS2D_GB300_NO_VEC_TYPES
struct vec2d {
    double x, y;
    vec2d operator+(vec2d o) const { return {x + o.x, y + o.y}; }
    vec2d operator-(vec2d o) const { return {x - o.x, y - o.y}; }
    vec2d operator*(double s) const { return {x * s, y * s}; }
    vec2d operator/(double s) const { return {x / s, y / s}; }
    vec2d& operator+=(vec2d o) { x += o.x; y += o.y; return *this; }
    vec2d& operator-=(vec2d o) { x -= o.x; y -= o.y; return *this; }
    vec2d& operator*=(double s) { x *= s; y *= s; return *this; }
    vec2d& operator/=(double s) { x /= s; y /= s; return *this; }
};

// Growable array with the altlib Vec members the API uses (data, size, free).
template <typename T>
struct Vec {
    T* data = nullptr;
    size_t size = 0;
    size_t capacity = 0;

    static Vec create(size_t cap) {
        Vec v;
        v.reserve(cap);
        return v;
    }
    static Vec emptyWithSize(size_t n) {
        Vec v;
        v.resize(n);
        return v;
    }
    void reserve(size_t cap) {
        if (cap <= capacity) return;
        T* p = static_cast<T*>(std::realloc(data, cap * sizeof(T)));
        if (!p) {
            std::fprintf(stderr, "fs2d: out of host memory\n");
            std::exit(EXIT_FAILURE);
        }
        data = p;
        capacity = cap;
    }
    void resize(size_t n) {
        reserve(n);
        if (n > size) std::memset(static_cast<void*>(data + size), 0, (n - size) * sizeof(T));
        size = n;
    }
    void push(const T& x) {
        if (size == capacity) reserve(capacity ? 2 * capacity : 16);
        data[size++] = x;
    }
    T& operator[](size_t i) { return data[i]; }
    const T& operator[](size_t i) const { return data[i]; }
    void free() {
        std::free(data);
        data = nullptr;
        size = capacity = 0;
    }
};
#endif

// Row-major 2D array, element (i, j) at data[j*NX + i] (include/Array2D.h:21-54).
template <typename T>
struct Array2D {
    T* data = nullptr;
    int NX;
    int NY;

    static Array2D create(int nx, int ny) {
        T* p = new (std::nothrow) T[(size_t)nx * ny];
        if (!p) {
            std::fprintf(stderr, "fs2d: out of host memory\n");
            std::exit(EXIT_FAILURE);
        }
        std::memset(static_cast<void*>(p), 0, sizeof(T) * (size_t)nx * ny);
        return {p, nx, ny};
    }
    void free() {
        delete[] data;
        data = nullptr;
    }
    void copyFrom(const Array2D& arr) { std::memcpy(static_cast<void*>(data), arr.data, sizeof(T) * (size_t)NX * NY); }
    T& operator()(int i, int j) {
        assert(i >= 0 && i < NX && j >= 0 && j < NY);
        return data[(size_t)j * NX + i];
    }
    const T& operator()(int i, int j) const {
        assert(i >= 0 && i < NX && j >= 0 && j < NY);
        return data[(size_t)j * NX + i];
    }
    void reset() { std::memset(static_cast<void*>(data), 0, sizeof(T) * (size_t)NX * NY); }

    // Catmull-Rom bicubic sample at grid coordinates (x, y) with clamped
    // neighbour indices, rows accumulated in order (Array2D::triCubic,
    // include/Array2D.h:244-359); 0 outside the grid.
    T triCubic(vec2d pos) const {
        const int x = (int)pos.x, y = (int)pos.y;
        if (x < 0 || x >= NX || y < 0 || y >= NY) return T(0);
        const T fx = (T)pos.x - (T)x, fy = (T)pos.y - (T)y;
        T wx[4], wy[4];
        weights(fx, wx);
        weights(fy, wy);
        T acc = T(0);
        for (int jj = 0; jj < 4; jj++) {
            const int yy = clampi(y + jj - 1, 0, NY - 1);
            T row = T(0);
            for (int ii = 0; ii < 4; ii++) row += wx[ii] * data[(size_t)yy * NX + clampi(x + ii - 1, 0, NX - 1)];
            acc += wy[jj] * row;
        }
        return acc;
    }

  private:
    static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
    static void weights(T t, T* w) {
        w[0] = T(-0.5) * (t * t * t) + (t * t) - T(0.5) * t;
        w[1] = T(1.5) * (t * t * t) - T(2.5) * (t * t) + T(1);
        w[2] = T(-1.5) * (t * t * t) + T(2) * (t * t) + T(0.5) * t;
        w[3] = T(0.5) * (t * t * t) - T(0.5) * (t * t);
    }
};

// Staggered MAC grid: u on (NX+1) x NY faces, v on NX x (NY+1) (include/MACGrid2D.h).
struct MACGrid2D {
    Array2D<double> u;
    Array2D<double> v;
    size_t NX;
    size_t NY;
    double dx = 1;

    static MACGrid2D create(size_t nx, size_t ny, double dx) {
        return {Array2D<double>::create((int)nx + 1, (int)ny), Array2D<double>::create((int)nx, (int)ny + 1), nx, ny, dx};
    }
    void free() {
        u.free();
        v.free();
    }
    void copyFrom(const MACGrid2D& rhs) {
        u.copyFrom(rhs.u);
        v.copyFrom(rhs.v);
    }
    // Velocity at a u face: v averaged over the (up to four) adjacent v faces.
    vec2d velU(size_t i, size_t j) {
        if (i > 0 && i < NX) return {u(i, j), 0.25 * (v(i - 1, j) + v(i - 1, j + 1) + v(i, j) + v(i, j + 1))};
        if (i == 0) return {u(i, j), 0.25 * (v(i, j) + v(i, j + 1))};
        return {u(i, j), 0.25 * (v(i - 1, j) + v(i - 1, j + 1))};
    }
    // Velocity at a v face: u averaged over the adjacent u faces.
    vec2d velV(size_t i, size_t j) {
        if (j > 0 && j < NY) return {0.25 * (u(i, j - 1) + u(i + 1, j - 1) + u(i, j) + u(i + 1, j)), v(i, j)};
        if (j == 0) return {0.25 * (u(i, j) + u(i + 1, j)), v(i, j)};
        return {0.25 * (u(i, j - 1) + u(i + 1, j - 1)), v(i, j)};
    }
    // Cell-centre velocity.
    vec2d vel(size_t i, size_t j) { return {0.5 * (u(i + 1, j) + u(i, j)), 0.5 * (v(i, j + 1) + v(i, j))}; }
    // Bicubic velocity at a world position (positions clamped to
    // [1e-6, N-1-1e-6] in cell units, include/MACGrid2D.h:80-97).
    double velInterpU(vec2d pos) {
        pos /= dx;
        pos.y -= 0.5;
        pos.x = clampd(pos.x, 1e-6, (double)NX - 1 - 1e-6);
        pos.y = clampd(pos.y, 1e-6, (double)NY - 1 - 1e-6);
        return u.triCubic(pos);
    }
    double velInterpV(vec2d pos) {
        pos /= dx;
        pos.x -= 0.5;
        pos.x = clampd(pos.x, 1e-6, (double)NX - 1 - 1e-6);
        pos.y = clampd(pos.y, 1e-6, (double)NY - 1 - 1e-6);
        return v.triCubic(pos);
    }
    vec2d velInterp(vec2d pos) { return {velInterpU(pos), velInterpV(pos)}; }
    double velDiv(size_t i, size_t j) { return (u(i + 1, j) - u(i, j) + v(i, j + 1) - v(i, j)) / dx; }

  private:
    static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }
};

struct LevelSet {
    Array2D<double> phi;   // negative inside the water
    int sizeX;
    int sizeY;
    double dx;

    static LevelSet create(int sizeX, int sizeY, double dx) {
        return {Array2D<double>::create(sizeX, sizeY), sizeX, sizeY, dx};
    }
    void free() { phi.free(); }
};

// PerformanceCounter (include/PerformanceCounter.h:11-35,
// src/PerformanceCounter.cpp:9-74): the reference's per-stage timer ring with
// the same public fields and the same averaging.  FluidSim2D::runFrame feeds
// it each frame's stage times (CUDA events around each stage on the device,
// in ms) where the reference feeds host clock readings: endStage(ms) stores
// one stage's time for the current frame, endFrame() averages the last
// SampleCount frames once that many were sampled (sampleFinished), sums the
// averages into avgTimePerFrame and appends them to averageStore, and
// saveToFile writes perf.csv from averageStore in the reference's format.
struct PerformanceCounter {
    static constexpr int SampleCount = 30;
    int currentStage = 0;
    int currentFrame = 0;
    Vec<float[SampleCount]> samples = {};
    Vec<float> average = {};
    float avgTimePerFrame = 0.0f;
    bool sampleFinished = false;
    Vec<float> averageStore = {};

    static PerformanceCounter create(int numStages) {
        PerformanceCounter counter = {};
        counter.samples.resize(numStages);
        counter.average.resize(numStages);
        return counter;
    }
    void endStage(float ms) {
        samples[currentStage][currentFrame] = ms;
        currentStage++;
    }
    void endFrame() {
        if (sampleFinished) {
            for (size_t i = 0; i < (size_t)samples.size; i++) {
                average[i] = 0.0f;
                for (int k = 0; k < SampleCount; k++) average[i] += samples[i][k];
                average[i] /= SampleCount;
            }
        }
        currentStage = 0;
        if (currentFrame == SampleCount - 1) sampleFinished = true;
        currentFrame = (currentFrame + 1) % SampleCount;
        avgTimePerFrame = 0.0f;
        for (size_t i = 0; i < (size_t)average.size; i++) {
            averageStore.push(average[i]);
            avgTimePerFrame += average[i];
        }
    }
    // perf.csv rows from frame SampleCount on: each stage's average, then ','.
    void saveToFile(const char* filename) {
        std::FILE* fp = std::fopen(filename, "w+");
        if (!fp) {
            std::fprintf(stderr, "fs2d: cannot open %s\n", filename);
            std::exit(EXIT_FAILURE);
        }
        const size_t numStages = (size_t)average.size;
        for (size_t i = SampleCount; numStages && i < (size_t)averageStore.size / numStages; i++) {
            for (size_t j = 0; j < numStages; j++) std::fprintf(fp, "%f,", (double)averageStore[numStages * i + j]);
            std::fputc('\n', fp);
        }
        std::fclose(fp);
    }
    void free() {
        samples.free();
        average.free();
        averageStore.free();
    }
};

enum FluidSimMode { FS_SEMILAGRANGIAN, FS_PICFLIP };
enum FluidCellType : uint8_t { FS_EMPTY, FS_FLUID, FS_SOLID };

// Same fields, order and types as the reference's FluidSim2DConfig, so it
// can be handed to fs2d_create as an fs2d_config.
struct FluidSim2DConfig {
    int sizeX;
    int sizeY;
    int particlesPerCellSqrt;
    double dt;
    double dx;
    double rho;
    double gravityX;
    double gravityY;
    FluidSimMode mode;
    double picFlipAlpha;
    FluidCellType* initialValues;
};

enum FluidSim2DSync { FS2D_SYNC_EVERY_FRAME, FS2D_SYNC_ON_DEMAND };

struct FluidSim2D {
    int sizeX;
    int sizeY;
    int particlesPerCellSqrt;
    int particlesPerCell;

    MACGrid2D mac;
    MACGrid2D newMac;
    Array2D<double> p;
    Array2D<FluidCellType> cell;
    Vec<vec2d> particles = {};
    Vec<vec2d> particleVels = {};

    LevelSet waterLevelSet;
    PerformanceCounter perfCounter;

    vec2d gravity = {0, -9.81};
    vec2d origGravity = {0, -9.81};
    double rho = 997.0;
    double picFlipAlpha;
    bool rendered = false;
    double currentTime = 0.0;
    double dt = 0.0001;
    double dx = 0.001;
    double dr = 0.0009;

    enum class StageType {
        Init, CreateWaterLevelSet, TransferVelocityToGrid,
        ApplySemiLagrangianAdvection, ApplyGravity, CreateSolidLevelSet, ApplyProjection,
        UpdateVelocity, UpdateParticleVelocities, ApplyAdvection
    };
    int numStages;
    StageType stage = StageType::Init;
    FluidSimMode mode;

    double origWaterVolume = 0.0;
    double waterVolume = 0.0;
    Vec<double> waterVolumeData = {};
    double totalEnergy = 0.0;
    Vec<double> totalEnergyData = {};
    double particleTotalEnergy = 0.0;
    Vec<double> particleTotalEnergyData = {};

    // GPU side
    fs2d_sim* device = nullptr;
    FluidSim2DSync sync = FS2D_SYNC_EVERY_FRAME;
    int lastStatus = 0;

    // FluidSim2D::create (src/FluidSim2D.cpp:23-76) on the GPU; `opt` selects
    // precision and solver settings (NULL: the reference's).
    static FluidSim2D create(const FluidSim2DConfig& config, const fs2d_options* opt = nullptr) {
        static_assert(sizeof(FluidSim2DConfig) == sizeof(fs2d_config), "config layout");
        FluidSim2D s;
        s.sizeX = config.sizeX;
        s.sizeY = config.sizeY;
        s.particlesPerCellSqrt = config.particlesPerCellSqrt;
        s.particlesPerCell = config.particlesPerCellSqrt * config.particlesPerCellSqrt;
        s.dt = config.dt;
        s.dx = config.dx;
        s.dr = 0.9 * config.dx;
        s.rho = config.rho;
        s.gravity = {config.gravityX, config.gravityY};
        s.origGravity = s.gravity;
        s.mode = config.mode;
        s.picFlipAlpha = config.picFlipAlpha;
        s.numStages = s.mode == FS_SEMILAGRANGIAN ? 7 : 8;
        s.mac = MACGrid2D::create(s.sizeX, s.sizeY, s.dx);
        s.newMac = MACGrid2D::create(s.sizeX, s.sizeY, s.dx);
        s.p = Array2D<double>::create(s.sizeX, s.sizeY);
        s.cell = Array2D<FluidCellType>::create(s.sizeX, s.sizeY);
        s.waterLevelSet = LevelSet::create(s.sizeX, s.sizeY, s.dx);
        s.perfCounter = PerformanceCounter::create(s.numStages);
        s.check(fs2d_create(reinterpret_cast<const fs2d_config*>(&config), opt, &s.device), "create");
        s.syncToHost();
        return s;
    }

    void free() {
        if (device) fs2d_destroy(device);
        device = nullptr;
        mac.free();
        newMac.free();
        p.free();
        cell.free();
        particles.free();
        particleVels.free();
        waterLevelSet.free();
        perfCounter.free();
        waterVolumeData.free();
        totalEnergyData.free();
        particleTotalEnergyData.free();
    }

    void runFrame() {
        pushParams();
        check(fs2d_run_frame(device), "runFrame");
        float ms[16];
        int n = 0;
        check(fs2d_get_stage_times(device, ms, 16, &n), "get_stage_times");
        for (int k = 0; k < n && k < numStages; k++) perfCounter.endStage(ms[k]);
        perfCounter.endFrame();
        afterDeviceWork();
    }
    void update() { runFrame(); }

    void createWaterLevelSet() { runStage(FS2D_STAGE_CREATE_WATER_LEVEL_SET, StageType::CreateWaterLevelSet); }
    void applySemiLagrangianAdvection() {
        runStage(FS2D_STAGE_APPLY_SEMI_LAGRANGIAN_ADVECTION, StageType::ApplySemiLagrangianAdvection);
    }
    void transferVelocityToGrid() { runStage(FS2D_STAGE_TRANSFER_VELOCITY_TO_GRID, StageType::TransferVelocityToGrid); }
    void applyGravity() { runStage(FS2D_STAGE_APPLY_GRAVITY, StageType::ApplyGravity); }
    void createSolidLevelSet() { runStage(FS2D_STAGE_CREATE_SOLID_LEVEL_SET, StageType::CreateSolidLevelSet); }
    void applyProjection() { runStage(FS2D_STAGE_APPLY_PROJECTION, StageType::ApplyProjection); }
    void updateVelocity() { runStage(FS2D_STAGE_UPDATE_VELOCITY, StageType::UpdateVelocity); }
    void updateParticleVelocities() {
        runStage(FS2D_STAGE_UPDATE_PARTICLE_VELOCITIES, StageType::UpdateParticleVelocities);
    }
    void applyAdvection() { runStage(FS2D_STAGE_APPLY_ADVECTION, StageType::ApplyAdvection); }

    // Diagnostics (src/FluidSim2D.cpp:607-638), reduced on the device.
    double avgPressure() { return diag(fs2d_avg_pressure, "avgPressure"); }
    double avgPressureInFluid() { return diag(fs2d_avg_pressure_in_fluid, "avgPressureInFluid"); }
    double maxVelocity() { return diag(fs2d_max_velocity, "maxVelocity"); }

    vec2d getGridCenter() { return {sizeX * dx / 2, sizeY * dx / 2}; }

    // perf.csv and conservation.csv in the reference's formats (src/FluidSim2D.cpp:738-750).
    void saveStats() { check(fs2d_save_stats(device, "perf.csv", "conservation.csv"), "saveStats"); }

    // Beyond the reference's API (include/fs2d.h): particle reseeding and
    // volume correction (the README's TODOs), the CFL check applyAdvection
    // only logs, and checkpoint / resume of the whole state.  They act on
    // the device state: reseed and loadCheckpoint refresh the mirrors as a
    // frame does under the sync policy.  gravity, picFlipAlpha and dt stay
    // the mirror's, pushed at the next frame as always, also after a load.
    fs2d_reseed_stats reseed(int minPerCell, int maxPerCell, unsigned int seed = 0) {
        fs2d_reseed_stats out{};
        check(fs2d_reseed(device, minPerCell, maxPerCell, seed, &out), "reseed");
        afterDeviceWork();
        return out;
    }
    void setVolumeCorrection(double rate) { check(fs2d_set_volume_correction(device, rate), "setVolumeCorrection"); }
    double cfl(long long* particle = nullptr) {
        double c = 0;
        check(fs2d_cfl(device, &c, particle), "cfl");
        return c;
    }
    void saveCheckpoint(const char* path) { check(fs2d_save_checkpoint(device, path), "saveCheckpoint"); }
    void loadCheckpoint(const char* path) {
        check(fs2d_load_checkpoint(device, path), "loadCheckpoint");
        afterDeviceWork();
    }

    vec2d clampPos(vec2d to) {
        constexpr double offset = 1e-3;
        const double lx = (1.0 + offset) * dx, hx = (sizeX - 1.0 - offset) * dx;
        const double ly = (1.0 + offset) * dx, hy = (sizeY - 1.0 - offset) * dx;
        return {to.x < lx ? lx : (to.x > hx ? hx : to.x), to.y < ly ? ly : (to.y > hy ? hy : to.y)};
    }

    // Device -> host mirrors (all public fields and statistics).
    void syncToHost() {
        size_t n = 0;
        check(fs2d_num_particles(device, &n), "num_particles");
        particles.resize(n);
        particleVels.resize(n);
        fs2d_state st{};
        st.cell = reinterpret_cast<uint8_t*>(cell.data);
        st.phi = waterLevelSet.phi.data;
        st.p = p.data;
        st.u = mac.u.data;
        st.v = mac.v.data;
        st.newU = newMac.u.data;
        st.newV = newMac.v.data;
        st.particles = reinterpret_cast<double*>(particles.data);
        st.particleVels = reinterpret_cast<double*>(particleVels.data);
        st.numParticles = n;
        check(fs2d_download_state(device, &st), "download_state");
        syncStats();
    }
    // Host mirrors -> device (after the caller changed a field).
    void syncToDevice() {
        fs2d_state st{};
        st.cell = reinterpret_cast<uint8_t*>(cell.data);
        st.phi = waterLevelSet.phi.data;
        st.p = p.data;
        st.u = mac.u.data;
        st.v = mac.v.data;
        st.newU = newMac.u.data;
        st.newV = newMac.v.data;
        st.particles = reinterpret_cast<double*>(particles.data);
        st.particleVels = reinterpret_cast<double*>(particleVels.data);
        st.numParticles = particles.size;
        check(fs2d_upload_state(device, &st), "upload_state");
        pushParams();
    }

  private:
    static_assert(sizeof(vec2d) == 2 * sizeof(double), "vec2d is two doubles");

    void check(int rc, const char* what) {
        lastStatus = rc;
        if (rc == FS2D_OK) return;
        if (rc == FS2D_ERR_NOT_CONVERGED) {
            std::fprintf(stderr, "fs2d %s: pressure solve did not converge: %s\n", what, fs2d_last_error());
            return;
        }
        std::fprintf(stderr, "fs2d %s failed (%d): %s\n", what, rc, fs2d_last_error());
        std::exit(EXIT_FAILURE);
    }
    void pushParams() { check(fs2d_set_params(device, gravity.x, gravity.y, picFlipAlpha, dt), "set_params"); }
    void runStage(int id, StageType t) {
        pushParams();
        stage = t;
        check(fs2d_run_stage(device, id), "stage");
        afterDeviceWork();
    }
    void afterDeviceWork() {
        if (sync == FS2D_SYNC_EVERY_FRAME) syncToHost();
        else syncStats();
    }
    void syncStats() {
        fs2d_stats st{};
        check(fs2d_get_stats(device, &st), "get_stats");
        waterVolume = st.waterVolume;
        totalEnergy = st.totalEnergy;
        particleTotalEnergy = st.particleTotalEnergy;
        origWaterVolume = st.origWaterVolume;
        currentTime = st.currentTime;
        size_t n = 0;
        check(fs2d_get_history(device, nullptr, nullptr, nullptr, 0, &n), "get_history");
        waterVolumeData.resize(n);
        totalEnergyData.resize(n);
        particleTotalEnergyData.resize(n);
        check(fs2d_get_history(device, waterVolumeData.data, totalEnergyData.data, particleTotalEnergyData.data, n, &n),
              "get_history");
    }
    double diag(int (*fn)(fs2d_sim*, double*), const char* what) {
        double v = 0;
        check(fn(device, &v), what);
        return v;
    }
};

#endif /* FLUIDSIM2D_GB300_HPP */
