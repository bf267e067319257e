// batch.cu — many independent scenes advanced together (host code only).
//
// No reference counterpart: the reference runs one FluidSim2D per process
// (demo/App.cpp:162-213).  A batch owns one handle per scene, each with its
// own CUDA stream, and a set of host worker threads that drive them: every
// worker issues the frames of its scenes in turn, so the GPU executes the
// kernels of as many scenes at once as there are workers, and the small
// grids of a batch fill the 152 SMs together instead of one after another.
// A frame's few host synchronisations (the pressure solver's convergence
// polls, the extrapolation depth) block only the worker that issued it.
// (Blocking-sync events instead of spinning waits, with up to twice as many
// workers as cores, measured slightly slower on the 256-scene batch.)
//
// Scenes go to workers longest-first onto the least-loaded worker (load =
// cells), which balances uneven grid sizes.  The differentiable rollout
// (fs2d_forward / fs2d_backward) of every scene runs the same way.  With workers = 0 the first
// frames of fs2d_batch_step pick the worker count: candidate counts are
// timed on one frame each and the fastest is kept.  Those frames are real
// frames: a scene's results do not depend on the worker count, as every
// scene runs the same kernels on its own stream.
#include <algorithm>
#include <chrono>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "fs2d_internal.cuh"

struct fs2d_batch {
    std::vector<fs2d_sim*> sims;
    std::vector<long long> cells;
    int workers = 0;          // 0: not tuned yet
    int device = 0;
    std::vector<int> status;  // last frame's status per scene
    std::vector<std::string> status_msg;  // message of a scene's last NOT_CONVERGED frame
    std::vector<double> tuning_ms;
};

namespace fs2d {
namespace {

// Longest-first assignment of scenes to `w` workers.
std::vector<std::vector<int>> assign(const fs2d_batch* b, int w) {
    std::vector<int> order(b->sims.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cells[x] > b->cells[y]; });
    std::vector<std::vector<int>> out(w);
    std::vector<long long> load(w, 0);
    for (int k : order) {
        int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        out[best].push_back(k);
        load[best] += b->cells[k];
    }
    return out;
}

// The error message of a failing call lives in its worker thread
// (fs2d_last_error is per thread): each worker keeps the message of its
// first error, and the calling thread re-raises the first failing worker's
// code and message.
struct WorkerStatus {
    int rc = 0;
    std::string msg;
    void fail(int r) {
        rc = r;
        msg = fs2d_last_error();
    }
};
int first_error(const std::vector<WorkerStatus>& ws) {
    for (const WorkerStatus& w : ws)
        if (w.rc) {
            set_error("%s", w.msg.c_str());
            return w.rc;
        }
    return 0;
}

// Runs `nframes` frames of every scene with `w` workers; returns the first
// hard error (NOT_CONVERGED is recorded per scene, as fs2d_step does).
int run(fs2d_batch* b, int w, int nframes) {
    auto parts = assign(b, w);
    std::vector<WorkerStatus> ws(w);
    auto body = [&](int t) {
        cudaSetDevice(b->device);
        for (int f = 0; f < nframes && ws[t].rc == 0; f++)
            for (int k : parts[t]) {
                int r = fs2d_run_frame(b->sims[k]);
                b->status[k] = r;
                if (r && r != FS2D_ERR_NOT_CONVERGED) {
                    ws[t].fail(r);
                    break;
                }
                if (r) b->status_msg[k] = fs2d_last_error();
            }
    };
    if (w == 1) {
        body(0);
    } else {
        std::vector<std::thread> th;
        th.reserve(w);
        for (int t = 0; t < w; t++) th.emplace_back(body, t);
        for (auto& x : th) x.join();
    }
    return first_error(ws);
}

// Runs fn(k) for every scene with `w` workers (scenes longest-first onto the
// least-loaded worker); returns the first error.
template <typename F>
int run_each(fs2d_batch* b, int w, F fn) {
    auto parts = assign(b, w);
    std::vector<WorkerStatus> ws(w);
    auto body = [&](int t) {
        cudaSetDevice(b->device);
        for (int k : parts[t]) {
            int r = fn(k);
            if (r) {
                ws[t].fail(r);
                return;
            }
        }
    };
    if (w == 1) {
        body(0);
    } else {
        std::vector<std::thread> th;
        th.reserve(w);
        for (int t = 0; t < w; t++) th.emplace_back(body, t);
        for (auto& x : th) x.join();
    }
    return first_error(ws);
}

int workers_for(const fs2d_batch* b) {
    if (b->workers > 0) return b->workers;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return std::max(1, std::min({(int)b->sims.size(), hw, 16}));
}

}  // namespace
}  // namespace fs2d

extern "C" {

int fs2d_batch_forward(fs2d_batch* b, int steps, int checkpointEvery, const double* const* u0, const double* const* v0,
                       const double* const* uTarget, const double* const* vTarget, double* losses) {
    using namespace fs2d;
    if (!b || !u0 || !v0 || !uTarget || !vTarget || !losses) {
        set_error("fs2d_batch_forward: per-scene arrays and losses are required");
        return FS2D_ERR_INVALID;
    }
    return run_each(b, workers_for(b), [&](int k) {
        return fs2d_forward(b->sims[k], steps, checkpointEvery, u0[k], v0[k], uTarget[k], vTarget[k], &losses[k]);
    });
}

int fs2d_batch_backward(fs2d_batch* b, double* const* gradU0, double* const* gradV0) {
    using namespace fs2d;
    if (!b || !gradU0 || !gradV0) {
        set_error("fs2d_batch_backward: per-scene gradient arrays are required");
        return FS2D_ERR_INVALID;
    }
    return run_each(b, workers_for(b), [&](int k) { return fs2d_backward(b->sims[k], gradU0[k], gradV0[k]); });
}


int fs2d_batch_create(const fs2d_config* cfgs, int n, const fs2d_options* opt, int workers, fs2d_batch** out) {
    using namespace fs2d;
    if (!cfgs || n < 1 || !out || workers < 0) {
        set_error("fs2d_batch_create: scenes, n >= 1, workers >= 0 and out are required");
        return FS2D_ERR_INVALID;
    }
    *out = nullptr;
    fs2d_options o;
    if (opt) o = *opt;
    else fs2d_default_options(&o);
    auto* b = new fs2d_batch;
    b->device = o.device;
    for (int k = 0; k < n; k++) {
        fs2d_options ok = o;
        if (o.use_seed) ok.seed = o.seed + (unsigned)k;
        fs2d_sim* s = nullptr;
        int rc = fs2d_create(&cfgs[k], &ok, &s);
        if (rc) {
            fs2d_batch_destroy(b);
            return rc;
        }
        b->sims.push_back(s);
        b->cells.push_back((long long)cfgs[k].sizeX * cfgs[k].sizeY);
    }
    b->status.assign(n, 0);
    b->status_msg.assign(n, std::string());
    b->workers = workers == 0 ? 0 : std::min({workers, n, 64});
    *out = b;
    return FS2D_OK;
}

int fs2d_batch_step(fs2d_batch* b, int nframes) {
    using namespace fs2d;
    if (!b || nframes < 0) return FS2D_ERR_INVALID;
    const int n = (int)b->sims.size();
    if (b->workers == 0 && nframes > 0) {
        // tune on the first frames: one frame per candidate worker count
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        std::vector<int> cand;
        for (int w = 4; w <= std::min({n, hw, 32}); w *= 2) cand.push_back(w);
        if (cand.empty()) cand.push_back(std::max(1, std::min(n, hw)));
        int best = cand[0];
        double best_ms = 1e300;
        for (int w : cand) {
            if (nframes == 0) break;
            auto t0 = std::chrono::steady_clock::now();
            int rc = run(b, w, 1);
            if (rc) return rc;
            double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            b->tuning_ms.push_back(ms);
            nframes--;
            if (ms < best_ms) {
                best_ms = ms;
                best = w;
            }
        }
        b->workers = best;
    }
    if (nframes == 0) return FS2D_OK;
    int rc = run(b, b->workers, nframes);
    if (rc) return rc;
    for (size_t k = 0; k < b->status.size(); k++)
        if (b->status[k]) {
            set_error("scene %zu: %s", k, b->status_msg[k].c_str());
            return b->status[k];
        }
    return FS2D_OK;
}

int fs2d_batch_size(fs2d_batch* b, int* n) {
    if (!b || !n) return FS2D_ERR_INVALID;
    *n = (int)b->sims.size();
    return FS2D_OK;
}

int fs2d_batch_scene(fs2d_batch* b, int k, fs2d_sim** sim) {
    if (!b || !sim || k < 0 || k >= (int)b->sims.size()) {
        fs2d::set_error("fs2d_batch_scene: index %d out of range", k);
        return FS2D_ERR_INVALID;
    }
    *sim = b->sims[k];
    return FS2D_OK;
}

int fs2d_batch_workers(fs2d_batch* b, int* workers) {
    if (!b || !workers) return FS2D_ERR_INVALID;
    *workers = b->workers;
    return FS2D_OK;
}

int fs2d_batch_set_workers(fs2d_batch* b, int workers) {
    if (!b || workers < 0) return FS2D_ERR_INVALID;
    b->workers = workers == 0 ? 0 : std::min({workers, (int)b->sims.size(), 64});
    return FS2D_OK;
}

int fs2d_batch_destroy(fs2d_batch* b) {
    if (!b) return FS2D_OK;
    for (fs2d_sim* s : b->sims) fs2d_destroy(s);
    delete b;
    return FS2D_OK;
}

}  // extern "C"
