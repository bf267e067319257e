// grid3d_api_test.cpp — the reference's 3D containers through
// include/MACGrid3D_gb300.hpp.
//
//   grid3d_api_test host   runs every host method on exact rational inputs
//                          and prints the results as hex floats, one
//                          "<name> <values...>" line each (tests/
//                          test_cpp_grid3d.py compares them with the oracle);
//   grid3d_api_test gpu    copies the same inputs to the device, runs the
//                          fs3d_device:: versions and checks them against the
//                          host methods: bit for bit, innerProduct within the
//                          bound of any summation order; prints OK.
#include <cstdio>
#include <cstring>
#include <vector>

#include "MACGrid3D_gb300.hpp"

#ifdef GRID3D_TEST_GPU
#include <cuda_runtime.h>
#endif

static const int SX = 9, SY = 7, SZ = 5;
static const int NPTS = 64;

// exact rational test values (multiples of 1/16 and 1/8)
static double value(size_t e, int salt) { return (double)((long)((e * 37 + salt * 11) % 101) - 50) / 16.0; }

static void fill(Array3D<double>& a, int salt) {
    for (size_t e = 0; e < a.count(); e++) a.data[e] = value(e, salt);
}

static std::vector<vec3d> points() {
    std::vector<vec3d> p(NPTS);
    for (int e = 0; e < NPTS; e++)
        p[e] = vec3d{(double)((e * 13) % 97) / 8.0 - 1.0, (double)((e * 29) % 89) / 8.0 - 1.0,
                     (double)((e * 7) % 61) / 8.0 - 1.0};
    return p;
}

static void put(const char* name, const double* v, size_t n) {
    std::printf("%s", name);
    for (size_t e = 0; e < n; e++) std::printf(" %a", v[e]);
    std::printf("\n");
}

struct Case {
    MACGrid3D g;
    Array3D<double> a, b, c;
    std::vector<vec3d> pts;
};

static Case make_case() {
    Case k;
    k.g = MACGrid3D::create(SX, SY, SZ);
    fill(k.g.u, 1);
    fill(k.g.v, 2);
    fill(k.g.w, 3);
    k.a = Array3D<double>::create(SX, SY, SZ);
    k.b = Array3D<double>::create(SX, SY, SZ);
    k.c = Array3D<double>::create(SX, SY, SZ);
    fill(k.a, 4);
    fill(k.b, 5);
    k.pts = points();
    return k;
}

// every host method; results keyed by name
static std::vector<std::pair<const char*, std::vector<double>>> host_results(Case& k) {
    std::vector<std::pair<const char*, std::vector<double>>> out;
    Array3D<double> s = Array3D<double>::create(SX, SY, SZ);
    s.copyFrom(k.a);
    s += k.b;
    out.push_back({"add", std::vector<double>(s.data, s.data + s.count())});
    s.setMultiplyAdd(k.a, 0.375, k.b);
    out.push_back({"sma", std::vector<double>(s.data, s.data + s.count())});
    out.push_back({"dot", {k.a.innerProduct(k.b)}});
    out.push_back({"norm", {k.a.infiniteNorm()}});
    std::vector<double> tc;
    for (const vec3d& p : k.pts) tc.push_back(k.a.triCubic(p));
    out.push_back({"tricubic", tc});
    std::vector<double> vel, div, vu, vv, vw, vi;
    k.g.iterate([&](int i, int j, int kk) {
        const vec3d r = k.g.vel(i, j, kk);
        vel.insert(vel.end(), {r.x, r.y, r.z});
        div.push_back(k.g.velDiv(i, j, kk));
    });
    k.g.iterateU([&](int i, int j, int kk) { const vec3d r = k.g.velU(i, j, kk); vu.insert(vu.end(), {r.x, r.y, r.z}); });
    k.g.iterateV([&](int i, int j, int kk) { const vec3d r = k.g.velV(i, j, kk); vv.insert(vv.end(), {r.x, r.y, r.z}); });
    k.g.iterateW([&](int i, int j, int kk) { const vec3d r = k.g.velW(i, j, kk); vw.insert(vw.end(), {r.x, r.y, r.z}); });
    for (const vec3d& p : k.pts) {
        const vec3d r = k.g.velInterp(p);
        vi.insert(vi.end(), {r.x, r.y, r.z});
    }
    out.push_back({"vel", vel});
    out.push_back({"velu", vu});
    out.push_back({"velv", vv});
    out.push_back({"velw", vw});
    out.push_back({"div", div});
    out.push_back({"interp", vi});
    s.free();
    return out;
}

#ifdef GRID3D_TEST_GPU
static bool check(const char* what, const std::vector<double>& got, const std::vector<double>& want) {
    if (got.size() != want.size() || std::memcmp(got.data(), want.data(), got.size() * sizeof(double)) != 0) {
        std::printf("FAIL %s differs from the host method\n", what);
        return false;
    }
    return true;
}

static double* upload(const double* h, size_t n) {
    double* d = nullptr;
    if (cudaMalloc((void**)&d, (n ? n : 1) * sizeof(double)) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice);
    return d;
}

static std::vector<double> download(const double* d, size_t n) {
    std::vector<double> h(n);
    cudaMemcpy(h.data(), d, n * sizeof(double), cudaMemcpyDeviceToHost);
    return h;
}

static int run_gpu(Case& k) {
    auto want = host_results(k);
    auto get = [&](const char* name) -> const std::vector<double>& {
        for (auto& p : want)
            if (!std::strcmp(p.first, name)) return p.second;
        static std::vector<double> none;
        return none;
    };
    const size_t n = k.a.count();
    MACGrid3D dg = k.g;   // same extents, device data
    dg.u.data = upload(k.g.u.data, k.g.u.count());
    dg.v.data = upload(k.g.v.data, k.g.v.count());
    dg.w.data = upload(k.g.w.data, k.g.w.count());
    Array3D<double> da = k.a, db = k.b, ds = k.a;
    da.data = upload(k.a.data, n);
    db.data = upload(k.b.data, n);
    ds.data = upload(k.a.data, n);
    const size_t nmax = 3 * (size_t)(SX + 1) * (SY + 1) * (SZ + 1);
    double* dout = upload(std::vector<double>(nmax).data(), nmax);
    vec3d* dpts = (vec3d*)upload(reinterpret_cast<const double*>(k.pts.data()), 3 * k.pts.size());
    bool good = true;
    auto ok = [&](int rc, const char* what) {
        if (rc != 0) {
            std::printf("FAIL %s: %s\n", what, fs2d_last_error());
            good = false;
        }
    };
    ok(fs3d_device::add(ds, db), "add");
    good = good && check("add", download(ds.data, n), get("add"));
    ok(fs3d_device::setMultiplyAdd(ds, da, 0.375, db), "setMultiplyAdd");
    good = good && check("setMultiplyAdd", download(ds.data, n), get("sma"));
    double dot = 0, norm = 0;
    ok(fs3d_device::innerProduct(da, db, &dot), "innerProduct");
    ok(fs3d_device::infiniteNorm(da, &norm), "infiniteNorm");
    double mag = 0;
    for (size_t e = 0; e < n; e++) mag += std::fabs(k.a.data[e] * k.b.data[e]);
    if (std::fabs(dot - get("dot")[0]) > 2.0 * n * std::ldexp(1.0, -53) * mag) {
        std::printf("FAIL innerProduct %a vs %a\n", dot, get("dot")[0]);
        good = false;
    }
    good = good && check("infiniteNorm", {norm}, get("norm"));
    ok(fs3d_device::triCubic(da, dpts, k.pts.size(), dout), "triCubic");
    good = good && check("triCubic", download(dout, k.pts.size()), get("tricubic"));
    ok(fs3d_device::vel(dg, (vec3d*)dout), "vel");
    good = good && check("vel", download(dout, 3 * (size_t)SX * SY * SZ), get("vel"));
    ok(fs3d_device::velU(dg, (vec3d*)dout), "velU");
    good = good && check("velU", download(dout, 3 * k.g.u.count()), get("velu"));
    ok(fs3d_device::velV(dg, (vec3d*)dout), "velV");
    good = good && check("velV", download(dout, 3 * k.g.v.count()), get("velv"));
    ok(fs3d_device::velW(dg, (vec3d*)dout), "velW");
    good = good && check("velW", download(dout, 3 * k.g.w.count()), get("velw"));
    ok(fs3d_device::velDiv(dg, dout), "velDiv");
    good = good && check("velDiv", download(dout, (size_t)SX * SY * SZ), get("div"));
    ok(fs3d_device::velInterp(dg, dpts, k.pts.size(), (vec3d*)dout), "velInterp");
    good = good && check("velInterp", download(dout, 3 * k.pts.size()), get("interp"));
    for (void* p : {(void*)dg.u.data, (void*)dg.v.data, (void*)dg.w.data, (void*)da.data, (void*)db.data,
                    (void*)ds.data, (void*)dout, (void*)dpts})
        cudaFree(p);
    if (cudaDeviceSynchronize() != cudaSuccess) good = false;
    std::printf(good ? "OK\n" : "FAIL\n");
    return good ? 0 : 1;
}
#endif

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && !std::strcmp(argv[1], "gpu");
    Case k = make_case();
    int rc = 0;
    if (!gpu) {
        for (auto& r : host_results(k)) put(r.first, r.second.data(), r.second.size());
    } else {
#ifdef GRID3D_TEST_GPU
        rc = run_gpu(k);
#else
        std::printf("FAIL built without GRID3D_TEST_GPU\n");
        rc = 1;
#endif
    }
    k.g.free();
    k.a.free();
    k.b.free();
    k.c.free();
    return rc;
}
