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
#include <string.h>
#include <algorithm>
#include <chrono>
#include <numeric>
#include <string>
#include <thread>
#include <array>
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
    // mixed precision: every scene's pressure solve in one pack (one launch
    // per kernel of the inner solve for all scenes) on the batch's stream
    fs2d::Pack* pack = nullptr;
    fs2d_options opt{};
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> ready;       // per scene: its solve's setup is queued
    cudaEvent_t solved = nullptr;
    int* err = nullptr;                   // error word and wait controls of the pack's sweeps
    unsigned long long launches = 0;      // kernels of the pack solves
    double sweep_us = 0;                  // the tuned persistent sweep's time (pack_tune)
    // last fs2d_batch_step: before the solve, the solve, after it (host
    // clock), and the batched level-set sweeps (device time, within the first)
    double phase_ms[4] = {0, 0, 0, 0};
    // createWaterLevelSet's sweeps of every scene, one launch per sweep
    fs2d::LsBatch* ls = nullptr;
    cudaEvent_t swept = nullptr;          // the batched sweeps are done
    cudaEvent_t ls_t0 = nullptr, ls_t1 = nullptr;
    // per scene, the device work of its three phases of a frame (before the
    // batched level-set sweeps, between them and the joint solve, after it)
    // as CUDA graphs, captured on the phase's second run and replayed after
    struct PhaseGraph {
        cudaGraphExec_t exec = nullptr;
        unsigned long long generation = 0;   // the scene's generation when captured
        unsigned long long kernels = 0;      // kernels per replay
        int runs = 0;
        bool direct = false;                 // capture failed: launch directly
    };
    std::vector<std::array<PhaseGraph, 3>> graphs;
    bool use_graphs = true;
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

// Runs fn(k) on the scenes of each worker, `w` workers in parallel; returns
// the first error (with its message on the calling thread).
template <typename F>
int on_workers(const std::vector<std::vector<int>>& parts, int device, F fn) {
    const int w = (int)parts.size();
    std::vector<WorkerStatus> ws(w);
    auto body = [&](int t) {
        cudaSetDevice(device);
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

// One per-scene phase of a batch frame: `body` queues its device work on
// the scene's stream (no host synchronisation inside).  The first run
// launches directly (and fills the caches of kernel attributes), the second
// captures the work into a graph, later runs replay it; a changed scene
// (new buffers or parameters) is captured again, and a phase that cannot be
// captured keeps launching directly.
template <class Body>
int run_phase(fs2d_batch* b, int k, int ph, Body&& body) {
    Sim* s = sim_of(b->sims[k]);
    fs2d_batch::PhaseGraph& g = b->graphs[k][ph];
    if (!b->use_graphs || g.direct || g.runs++ == 0) return body();
    if (g.exec && g.generation == s->generation) {
        s->launches += g.kernels;
        return check_cuda(cudaGraphLaunch(g.exec, s->stream), "cudaGraphLaunch");
    }
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        g.direct = true;
        return body();
    }
    const unsigned long long l0 = s->launches;
    s->capturing = true;
    int rc = body();
    s->capturing = false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
    if (!rc && e == cudaSuccess && graph) e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc || e != cudaSuccess || !g.exec) {
        // nothing of the capture ran: launch the phase directly, now and from
        // now on (a real error of the work shows up again there)
        (void)cudaGetLastError();
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        s->launches = l0;
        g.direct = true;
        return body();
    }
    g.generation = s->generation;
    g.kernels = s->launches - l0;
    return check_cuda(cudaGraphLaunch(g.exec, s->stream), "cudaGraphLaunch");
}

// Frames of a mixed-precision batch: the workers queue every scene's stages
// up to its pressure solve's setup; one pack solve then solves all scenes
// together on the batch's stream (one launch per kernel of the inner solve
// for every scene); the workers queue the remaining stages and finish each
// scene's frame.  A scene computes exactly what it computes alone.
int run_packed(fs2d_batch* b, int w, int nframes) {
    auto parts = assign(b, w);
    const int n = (int)b->sims.size();
    std::vector<int> st(n, 0);
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    for (int f = 0; f < nframes; f++) {
        auto t0 = clk::now();
        // createWaterLevelSet: seeds per scene, every scene's sweeps in one
        // launch per sweep on the batch's stream, the rest per scene
        int rc = on_workers(parts, b->device, [&](int k) {
            st[k] = 0;
            fs2d_sim* p = b->sims[k];
            int r = run_phase(b, k, 0, [&] { return frame_levelset(p, 1); });
            if (!r) r = check_cuda(cudaEventRecord(b->ready[k], sim_of(p)->stream), "cudaEventRecord");
            return r;
        });
        if (rc) return rc;
        for (int k = 0; k < n; k++) FS2D_CUDA(cudaStreamWaitEvent(b->stream, b->ready[k], 0));
        FS2D_CUDA(cudaEventRecord(b->ls_t0, b->stream));
        if ((rc = ls_batch_sweeps(b->ls, b->stream, b->err, &b->launches))) return rc;
        FS2D_CUDA(cudaEventRecord(b->ls_t1, b->stream));
        FS2D_CUDA(cudaEventRecord(b->swept, b->stream));
        rc = on_workers(parts, b->device, [&](int k) {
            fs2d_sim* p = b->sims[k];
            int r = check_cuda(cudaStreamWaitEvent(sim_of(p)->stream, b->swept, 0), "cudaStreamWaitEvent");
            if (!r) r = run_phase(b, k, 1, [&] {
                int q = frame_levelset(p, 2);
                if (!q) q = frame_stages(p, 1, frame_solve_stage(p) + 1, &st[k], 1);
                return q;
            });
            if (!r) frame_mark(p, 1);
            if (!r) r = check_cuda(cudaEventRecord(b->ready[k], sim_of(p)->stream), "cudaEventRecord");
            return r;
        });
        if (rc) return rc;
        for (int k = 0; k < n; k++) FS2D_CUDA(cudaStreamWaitEvent(b->stream, b->ready[k], 0));
        FS2D_CUDA(cudaStreamSynchronize(b->stream));   // the scenes' stages before the solve are done
        b->phase_ms[0] += ms_since(t0);
        float ls_ms = 0;
        if (cudaEventElapsedTime(&ls_ms, b->ls_t0, b->ls_t1) != cudaSuccess) {
            ls_ms = 0;
            (void)cudaGetLastError();
        }
        b->phase_ms[3] += ls_ms;
        t0 = clk::now();
        rc = pack_solve(b->pack, b->opt, b->stream, &b->launches, b->err, b->device, nullptr);
        if (rc) return rc;
        int perr = 0;
        FS2D_CUDA(cudaMemcpyAsync(&perr, b->err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        FS2D_CUDA(cudaStreamSynchronize(b->stream));
        if (perr) {
            FS2D_CUDA(cudaMemset(b->err, 0, sizeof(int)));
            set_error("a wavefront sweep of the batch (level set or pressure solve) timed out");
            return FS2D_ERR_TIMEOUT;
        }
        FS2D_CUDA(cudaEventRecord(b->solved, b->stream));
        b->phase_ms[1] += ms_since(t0);
        t0 = clk::now();
        rc = on_workers(parts, b->device, [&](int k) {
            fs2d_sim* p = b->sims[k];
            int r = check_cuda(cudaStreamWaitEvent(sim_of(p)->stream, b->solved, 0), "cudaStreamWaitEvent");
            if (!r) r = run_phase(b, k, 2, [&] { return frame_stages(p, frame_solve_stage(p), -1, &st[k], 2); });
            if (!r) frame_mark(p, 2);
            r = frame_close(p, r, st[k]);
            b->status[k] = r;
            if (r == FS2D_ERR_NOT_CONVERGED) {
                b->status_msg[k] = fs2d_last_error();
                r = 0;
            }
            return r;
        });
        b->phase_ms[2] += ms_since(t0);
        if (rc) return rc;
    }
    return 0;
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
    b->opt = o;
    if (o.precision != FS2D_PRECISION_FP64) {
        std::vector<Sim*> ss(n);
        for (int k = 0; k < n; k++) ss[k] = sim_of(b->sims[k]);
        int rc = pack_create_batch(ss.data(), n, &b->pack);
        if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        b->ready.assign(n, nullptr);
        for (int k = 0; k < n && !rc; k++)
            rc = check_cuda(cudaEventCreateWithFlags(&b->ready[k], cudaEventDisableTiming), "cudaEventCreate");
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&b->solved, cudaEventDisableTiming), "cudaEventCreate");
        if (!rc) rc = check_cuda(cudaMalloc((void**)&b->err, kErrWords * sizeof(int)), "cudaMalloc");
        if (!rc) {
            int wd[kErrWords] = {0};
            wd[2] = -1;
            const long long polls = kWaveSpinLimit;
            memcpy(&wd[4], &polls, sizeof(polls));
            rc = check_cuda(cudaMemcpy(b->err, wd, sizeof(wd), cudaMemcpyHostToDevice), "cudaMemcpy");
        }
        if (!rc) rc = pack_tune(b->pack, b->stream, b->err, b->device, &b->launches, &b->sweep_us);
        if (!rc) b->ls = ls_batch_create(ss.data(), n, b->device, &rc);
        b->graphs.resize(n);
        if (!rc) rc = check_cuda(cudaEventCreateWithFlags(&b->swept, cudaEventDisableTiming), "cudaEventCreate");
        if (!rc) rc = check_cuda(cudaEventCreate(&b->ls_t0), "cudaEventCreate");
        if (!rc) rc = check_cuda(cudaEventCreate(&b->ls_t1), "cudaEventCreate");
        if (rc) {
            fs2d_batch_destroy(b);
            return rc;
        }
    }
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
            int rc = b->pack ? run_packed(b, w, 1) : run(b, w, 1);
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
    b->phase_ms[0] = b->phase_ms[1] = b->phase_ms[2] = b->phase_ms[3] = 0;
    int rc = b->pack ? run_packed(b, b->workers, nframes) : run(b, b->workers, nframes);
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
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (fs2d_sim* s : b->sims) fs2d_destroy(s);
    fs2d::pack_free(b->pack);
    for (cudaEvent_t e : b->ready)
        if (e) cudaEventDestroy(e);
    if (b->solved) cudaEventDestroy(b->solved);
    fs2d::ls_batch_free(b->ls);
    for (auto& gs : b->graphs)
        for (auto& g : gs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
    for (cudaEvent_t e : {b->swept, b->ls_t0, b->ls_t1})
        if (e) cudaEventDestroy(e);
    if (b->err) cudaFree(b->err);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return FS2D_OK;
}

int fs2d_batch_sweep_schedule(fs2d_batch* b, int* schedule, int* ctas, int* items, double* sweep_us) {
    if (!b) return FS2D_ERR_INVALID;
    fs2d::Pack* pk = b->pack;
    if (schedule) *schedule = pk ? pk->schedule : -1;
    if (ctas) *ctas = pk ? pk->sweep_ctas : 0;
    if (items) *items = pk ? pk->nitems : 0;
    if (sweep_us) *sweep_us = pk ? b->sweep_us : 0.0;
    return FS2D_OK;
}

int fs2d_batch_set_schedule(fs2d_batch* b, int schedule, int ctas) {
    if (!b || !b->pack) {
        fs2d::set_error("fs2d_batch_set_schedule: not a mixed-precision batch");
        return FS2D_ERR_INVALID;
    }
    return fs2d::pack_set_schedule(b->pack, schedule, ctas, b->stream);
}

int fs2d_batch_set_graphs(fs2d_batch* b, int on) {
    if (!b) return FS2D_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (fs2d_sim* p : b->sims) cudaStreamSynchronize(fs2d::sim_of(p)->stream);
    for (auto& gs : b->graphs)
        for (auto& g : gs) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = fs2d_batch::PhaseGraph();
        }
    b->use_graphs = on != 0;
    return FS2D_OK;
}

int fs2d_batch_phase_ms(fs2d_batch* b, double* ms) {
    if (!b || !ms) return FS2D_ERR_INVALID;
    for (int k = 0; k < 4; k++) ms[k] = b->phase_ms[k];
    return FS2D_OK;
}

int fs2d_batch_launch_count(fs2d_batch* b, unsigned long long* out) {
    if (!b || !out) return FS2D_ERR_INVALID;
    unsigned long long n = b->launches;
    for (fs2d_sim* s : b->sims) n += fs2d::sim_of(s)->launches;
    *out = n;
    return FS2D_OK;
}

}  // extern "C"
