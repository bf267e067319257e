#!/usr/bin/env python
"""Benchmark of the GB300 FluidSim2D time step.

Workload: the PIC/FLIP dam break (x < 0.4, y < 0.6) united with a disk of
radius 0.1 at (0.7, 0.7), 1024 x 1024 cells, dx = 1/1024, 4 particles per
fluid cell (~1.1 M particles), FLIP ratio 0.95 (picFlipAlpha = 0.05),
dt = 1/960, pressure solve MIC(0)-PCG to a relative residual of 1e-6
(infinity norm, the reference's convention), at most 200 iterations.
Seeded synthetic input (the reference ships no datasets).

A step is one FluidSim2D::runFrame (all eight stages).  Metric: grid-cell
steps/s = NX * NY * steps / time.  The headline runs the mixed-precision
projection (FP32 MIC(0)-PCG inside FP64 iterative refinement, the same FP64
stopping test); the all-FP64 GPU path is measured beside it ("fp64_path").

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
  python bench.py --impl reference ...   # the reference's CPU path (oracle port)

One JSON line is printed by rank 0.  Multi-GPU runs are independent
replicas (the step does not shard); value = total cell-steps / max time.
Besides the headline keys the line carries:
  roofline        the dominant kernel (and every timed kernel with a known
                  byte count) against the measured HBM copy peak;
  step_roofline   the compulsory bytes of every stage of a step / step time;
  fp64_path       the all-FP64 GPU step on the same workload;
  error_vs_oracle one projection of the workload by the mixed and FP64
                  device paths at the bench tolerance: time, and error of
                  p, u, v against the FP64 oracle solved to 1e-12;
  sl_path         the semi-Lagrangian dam break at the same size;
  pressure_solve  the standalone 2048^2 solve to 1e-10, FP64 vs mixed;
  adjoint         the differentiable 128^2 closed-box rollout (64 steps):
                  forward and backward times in both precisions;
  batch           256 dam breaks of uneven sizes advanced together (split
                  over the ranks when N > 1);
  batch_adjoint   the rollouts of 32 closed boxes of uneven sizes;
  grid3d          the 3D container kernels (include/fs3d.h) on a 512^3 MAC
                  grid against the HBM copy peak;
  e2e             the headline through the C ABI with host buffers;
  cpu_baseline    the CPU oracle port timed on the host's cores.
Each extra line has a flag that switches it off (e.g. --adjoint-size 0).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fluid-sim_gb300"))
# Hardware work queues of this process's CUDA context (read when the context is
# created): a batch drives one stream per scene, and with the default 8 queues
# streams beyond the eighth share queues and wait behind one another.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "grid-cell steps/s at 1024^2 (PIC/FLIP step, MIC(0)-PCG to 1e-6 rel res)"
UNIT = "grid-cell steps/s"
SEED = 12345
FLUSH_BYTES = 256 << 20          # > 129 MB L2
# kernels timed per launch during the timed region, with their algorithmic
# bytes per grid cell and launch:
#   mic32_*: FP32 MIC(0) solve, read the right-hand side and two folded
#            coefficients, write the result: 4 x 4 B
#   wave2_Mic*64: FP64 MIC(0) solve, read r (or q), two coefficients and the
#            preconditioner, write q (or z): 5 x 8 B
#   eik_sweep: read phi (8 B) and the changeability byte, write phi: 17 B
#   cp_sweep: read the closest-particle index (4 B) and its 16-byte
#            position pair, write the index: 24 B
#   k_spmv32: s = z + beta s_old, w = A s, s.w: reads label (1 B), three
#            matrix arrays, z and s_old, writes s and w: 29 B
#   k_axpy32: e += alpha s, r -= alpha w, r pc^2, ||r||inf: reads e, s, r, w,
#            pc, writes e, r, r pc^2: 32 B
#   k_dot32: z.r: 8 B
KERNEL_BYTES_PER_CELL = {"mic32": 16, "mic32_forward": 16, "mic32_backward": 16, "wave2_MicForward64": 40,
                         "wave2_MicBackward64": 40, "eik_sweep": 17, "cp_sweep": 24, "k_spmv32": 29,
                         "k_axpy32": 32, "k_dot32": 8}
DOMINANT = tuple(KERNEL_BYTES_PER_CELL)


def bench_grid3d(n, local, peak, reps=5):
    """The 3D containers of include/fs3d.h (the reference's Array3D and
    MACGrid3D methods) on an n^3 MAC grid and n^3 arrays of N(0,1) doubles:
    each kernel timed with CUDA events on its stream after one untimed
    launch, mean of `reps`; every array is larger than the L2 cache.
    Algorithmic bytes (each array element read or written once): velDiv
    32 B per cell (u, v, w in, div out), vel 48 B per cell (vec3d out),
    velU 48 B per u face, setMultiplyAdd and += 24 B per element,
    innerProduct 16 B, infiniteNorm 8 B; velInterp (all three components)
    at n^3/8 random points is reported in points/s.  GB300's FP64 rate
    bounds several of them, so each entry also gives the FP64 instructions
    per unit (velDiv 5 additions, vel 3, velU 6 in the interior, the halving
    and quartering being exact integer exponent steps; setMultiplyAdd 2, +=
    1, innerProduct 1 fused multiply-add, infiniteNorm 0: integer compares)
    and the FP64 rate they imply."""
    import ctypes as C
    import torch
    import fs2d

    lib = fs2d.load()
    dev = f"cuda:{local}"
    gen = torch.Generator(device=dev).manual_seed(7)
    f64 = dict(dtype=torch.float64, device=dev)
    A = fs2d.Array3D
    u = torch.randn((n, n, n + 1), generator=gen, **f64)
    v = torch.randn((n, n + 1, n), generator=gen, **f64)
    w = torch.randn((n + 1, n, n), generator=gen, **f64)
    mac = fs2d.MACGrid3D(A(u.data_ptr(), n + 1, n, n), A(v.data_ptr(), n, n + 1, n), A(w.data_ptr(), n, n, n + 1),
                         n, n, n)
    cells = n ** 3
    x, y = torch.randn(cells, generator=gen, **f64), torch.randn(cells, generator=gen, **f64)
    out1 = torch.empty(cells, **f64)
    out3 = torch.empty(3 * (n + 1) * n * n, **f64)
    npts = cells // 8
    pts = torch.rand((npts, 3), generator=gen, **f64) * n
    pout = torch.empty(3 * npts, **f64)
    ax, ay, ao = (A(t.data_ptr(), n, n, n) for t in (x, y, out1))
    res = C.c_double()
    stream = torch.cuda.Stream()
    sp = C.c_void_p(stream.cuda_stream)
    faces = (n + 1) * n * n
    # name: (call, algorithmic bytes, FP64 instructions)
    calls = {
        "velDiv": (lambda: lib.fs3d_mac_vel_div(C.byref(mac), C.c_void_p(out1.data_ptr()), sp), 32 * cells,
                   5 * cells),
        "vel": (lambda: lib.fs3d_mac_vel(C.byref(mac), C.c_void_p(out3.data_ptr()), sp), 48 * cells, 3 * cells),
        "velU": (lambda: lib.fs3d_mac_face_vel(C.byref(mac), 0, C.c_void_p(out3.data_ptr()), sp), 48 * faces,
                 6 * faces),
        "setMultiplyAdd": (lambda: lib.fs3d_set_multiply_add(C.byref(ao), C.byref(ax), 0.5, C.byref(ay), sp),
                           24 * cells, 2 * cells),
        "add": (lambda: lib.fs3d_add(C.byref(ao), C.byref(ay), sp), 24 * cells, cells),
        "innerProduct": (lambda: lib.fs3d_inner_product(C.byref(ax), C.byref(ay), C.byref(res), sp), 16 * cells,
                         cells),
        "infiniteNorm": (lambda: lib.fs3d_infinite_norm(C.byref(ax), C.byref(res), sp), 8 * cells, 0),
        "velInterp": (lambda: lib.fs3d_mac_vel_interp(C.byref(mac), 3, C.c_void_p(pts.data_ptr()), npts,
                                                      C.c_void_p(pout.data_ptr()), sp), None, None),
    }
    out = {"grid": [n, n, n], "points": npts, "peak_gbs": peak,
           "timing": "CUDA events on the call's stream, one untimed call first, mean of %d; every array larger than "
                     "the L2 cache; innerProduct and infiniteNorm include the copy of the scalar to the host" % reps}
    torch.cuda.synchronize()
    for name, (fn, nbytes, fp64) in calls.items():
        rc = fn()
        if rc != 0:
            raise RuntimeError(f"fs3d {name}: {lib.fs2d_last_error().decode()}")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            rc = fn()
            if rc != 0:
                raise RuntimeError(f"fs3d {name}: {lib.fs2d_last_error().decode()}")
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        entry = {"ms": round(ms, 4)}
        if nbytes:
            gbs = nbytes / (ms * 1e-3) / 1e9
            entry.update(gbs=round(gbs, 1), frac=round(gbs / peak, 4),
                         fp64_tops=round(fp64 / (ms * 1e-3) / 1e12, 3))
        else:
            entry["points_per_s"] = npts / (ms * 1e-3)
        out[name] = entry
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=8, help="steps of the all-FP64 path measured beside it")
    ap.add_argument("--pressure-size", type=int, default=2048,
                    help="grid of the standalone pressure-solve comparison (0: skip)")
    ap.add_argument("--adjoint-size", type=int, default=128, help="closed-box rollout grid (0: skip)")
    ap.add_argument("--adjoint-steps", type=int, default=64)
    ap.add_argument("--batch-scenes", type=int, default=256, help="batched dam breaks (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--batch-adjoint-scenes", type=int, default=32, help="batched closed-box rollouts (0: skip)")
    ap.add_argument("--sl-steps", type=int, default=10, help="steps of the semi-Lagrangian 1024^2 variant (0: skip)")
    ap.add_argument("--batch-adjoint-steps", type=int, default=16)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--grid3d-size", type=int, default=512, help="3D container kernels on an n^3 MAC grid (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-baseline sampling")
    ap.add_argument("--no-oracle-error", action="store_true",
                    help="skip the accuracy comparison against the FP64 oracle (error_vs_oracle)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(size):
    import scenes
    return scenes.pic_dam_break_disk(size)


def config_dict(args, n_particles):
    """The workload, identical for both arms; how each arm computes it (the
    precision, threads, iteration counts) lives in top-level keys."""
    return {
        "workload": f"PIC/FLIP dam break + disk r=0.1, {args.size}x{args.size}, dt=1/{int(round(960 * args.size / 1024))}, "
                    f"4 ppc, FLIP 0.95, MIC(0)-PCG tol {args.tol:g} rel (inf-norm), <=200 iters",
        "grid": [args.size, args.size],
        "particles": n_particles,
        "l2": "flushed between timed steps (256 MiB write)",
        "parallelism": f"replicas x{args.gpus}",
    }


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU baseline
def cpu_baseline(args, budget_s, max_frames):
    """The oracle port (OpenMP build, all host threads) on the same workload:
    frames after one warm-up frame until `budget_s` seconds or `max_frames`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    sc = workload(args.size)
    sim = oracle_py.OracleSim(sc, seed=SEED, omp=True, sl_inplace=0, pcg_tol=args.tol, pcg_max_iters=200)
    sim.frame()
    frames, t0 = 0, time.perf_counter()
    while frames < max_frames:
        sim.frame()
        frames += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    value = args.size * args.size * frames / dt
    info = sim.solver_info()
    sim.close()

    def variant(omp, tol, iters_cap):
        # one timed frame after one warm-up frame (the reference's own PCG cap of 200 iterations)
        v = oracle_py.OracleSim(sc, seed=SEED, omp=omp, sl_inplace=0, pcg_tol=tol, pcg_max_iters=iters_cap)
        v.frame()
        t = time.perf_counter()
        v.frame()
        d = time.perf_counter() - t
        it = v.solver_info()["iterations"]
        v.close()
        return {"value": args.size * args.size / d, "unit": UNIT,
                "cores": int(os.environ.get("OMP_NUM_THREADS", threads)) if omp else 1,
                "pcg_tol": tol, "pcg_iterations": it, "s_per_frame": d}

    variants = {}
    if budget_s > 0:
        # the serial build (the reference's default configuration, USE_OPENMP off) and the
        # reference's hard-coded tolerance 1e-12 (OpenMP build)
        variants["serial_tol_%g" % args.tol] = variant(False, args.tol, 200)
        variants["openmp_tol_1e-12"] = variant(True, 1e-12, 200)
    out = {"value": value, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", threads)), "kind": "port",
           "sample": f"{frames} frame(s) of the same {args.size}^2 workload after 1 warm-up frame, "
                     f"{dt:.1f} s; oracle restatement (C, -O3 -fopenmp, the reference's race-free "
                     f"OpenMP loops), PCG tol {args.tol:g} (last solve {info['iterations']} iterations)",
           "variants": variants}
    if getattr(args, "grid3d_size", 0) > 0:
        out["grid3d"] = cpu_grid3d(128)
    return out


def cpu_grid3d(n):
    """The 3D containers' methods on the host (the oracle's C restatement of
    include/Array3D.h and include/MACGrid3D.h, serial like the reference's
    headers): per-unit rates on an n^3 MAC grid, beside the device's
    `grid3d` line.  Best of 3 for each."""
    import numpy as np
    import oracle3d
    R = oracle3d.restated
    rng = np.random.default_rng(7)
    size = (n, n, n)
    u, v, w = (rng.standard_normal(k) for k in ((n + 1) * n * n, n * (n + 1) * n, n * n * (n + 1)))
    a, b = rng.standard_normal(n ** 3), rng.standard_normal(n ** 3)
    pts = rng.random((n ** 3 // 8, 3)) * n

    def best(fn):
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            t.append(time.perf_counter() - t0)
        return min(t)

    cells = n ** 3
    res = {"grid": [n, n, n], "kind": "port", "cores": 1,
           "sample": f"oracle restatement (C, -O2, serial) on a {n}^3 MAC grid and {n}^3 arrays of N(0,1) "
                     f"doubles, {len(pts)} random points; best of 3 per method"}
    res["velDiv_cells_per_s"] = cells / best(lambda: R.mac_vel_div(u, v, w, size))
    res["vel_cells_per_s"] = cells / best(lambda: R.mac_vel(u, v, w, size))
    res["velU_faces_per_s"] = (n + 1) * n * n / best(lambda: R.mac_face_vel(u, v, w, size, "u"))
    res["setMultiplyAdd_elements_per_s"] = cells / best(lambda: R.set_multiply_add(a, 0.5, b, size))
    res["innerProduct_elements_per_s"] = cells / best(lambda: R.inner_product(a, b, size))
    res["infiniteNorm_elements_per_s"] = cells / best(lambda: R.infinite_norm(a, size))
    res["velInterp_points_per_s"] = len(pts) / best(lambda: R.mac_vel_interp(u, v, w, size, "uvw", pts))
    return res


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    budget = 150.0
    t_start = time.perf_counter()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    sc = workload(args.size)
    sim = oracle_py.OracleSim(sc, seed=SEED, omp=True, sl_inplace=0, pcg_tol=args.tol, pcg_max_iters=200)
    n_particles = sim.num_particles()
    warm = min(args.warmup, 5)   # about a second per frame on 16 Grace cores
    for _ in range(warm):
        sim.frame()
    frames, t0 = 0, time.perf_counter()
    while frames < args.steps:
        sim.frame()
        frames += 1
        if time.perf_counter() - t_start > budget:
            break
    dt = time.perf_counter() - t0
    value = args.size * args.size * frames / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": frames, "warmup": warm, "ms_per_step": 1000 * dt / frames, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded dam break + disk)",
        "config": config_dict(args, n_particles),
        "precision": "fp64 (reference CPU path)", "cpu_threads": int(os.environ["OMP_NUM_THREADS"]),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                         "sample": f"{frames} of {args.steps} requested frames after {warm} warm-up frame(s), "
                                   f"capped at {budget:.0f} s; oracle restatement of the reference step "
                                   f"(OpenMP on its race-free loops); the reference checkout does not exist "
                                   f"on this machine, so its own build cannot run here"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm
def state_bytes(st):
    return sum(a.nbytes for a in st.values())


def error_vs_oracle(args, sc, st, stream, local):
    """Accuracy of the two device projections on one system of the headline
    workload.  From the state `st` (a frame boundary of the headline run) the
    oracle (the FP64 C restatement, OpenMP build) advances the stages before
    applyProjection, which gives the pre-projection state S; the oracle then
    solves S to a relative residual of 1e-12 (the FP64 oracle run) and
    applies updateVelocity.  The mixed and the all-FP64 device paths solve S
    at the bench's tolerance (CUDA events around the projection stage, after
    one untimed solve of the same state) and apply updateVelocity; the line
    reports their time and the max-norm relative error of p, u and v against
    the oracle's."""
    import numpy as np
    import torch
    import fs2d
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    t0 = time.perf_counter()
    orc = oracle_py.OracleSim(sc, seed=SEED, omp=True, sl_inplace=0, pcg_tol=1e-12, pcg_max_iters=4000)
    orc.set_state(st)
    for stage in ("createWaterLevelSet", "transferVelocityToGrid", "applyGravity", "createSolidLevelSet"):
        orc.stage(stage)
    pre = orc.get_state()
    orc.stage("applyProjection")
    info = orc.solver_info()
    orc.stage("updateVelocity")
    ref = orc.get_state()
    orc.close()
    out = {"state": "frame boundary of the headline run, advanced to applyProjection by the oracle",
           "oracle": {"pcg_tol": 1e-12, "pcg_iterations": info["iterations"], "rel_residual": info["rel_residual"],
                      "wall_s": round(time.perf_counter() - t0, 1)},
           "error": "max |x - x_oracle| / max |x_oracle| for x = p after applyProjection and the face velocities "
                    "newMac.u, newMac.v after updateVelocity"}

    def rel(a, b):
        return float(np.abs(a - b).max() / (np.abs(b).max() + 1e-300))

    for prec in ("mixed", "fp64"):
        g = fs2d.FluidSim2D(sc, seed=SEED, precision=prec, pcg_tol=args.tol, pcg_max_iters=200, device=local)
        g.set_stream(stream.cuda_stream)
        g.set_state(pre)
        g.stage("applyProjection")
        g.set_state(pre)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.stage("applyProjection")
        e1.record(stream)
        torch.cuda.synchronize()
        stt = g.stats()
        g.stage("updateVelocity")
        got = g.get_state(["p", "newU", "newV"])
        out[prec] = {"pcg_tol": args.tol, "ms_to_tol": round(e0.elapsed_time(e1), 3),
                     "pcg_iterations": stt["pcgIterations"], "refinement_sweeps": stt["irOuterIterations"],
                     "rel_residual": stt["pcgRelResidual"], "p_rel_err": rel(got["p"], ref["p"]),
                     "u_rel_err": rel(got["newU"], ref["newU"]), "v_rel_err": rel(got["newV"], ref["newV"])}
        g.close()
    out["fp64_over_mixed_time"] = out["fp64"]["ms_to_tol"] / out["mixed"]["ms_to_tol"]
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    rank, world, local = dist_env()
    import numpy as np
    import torch
    import fs2d

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sc = workload(args.size)
    opts = dict(precision=args.precision, pcg_tol=args.tol, pcg_max_iters=200, device=local)
    sim = fs2d.FluidSim2D(sc, seed=SEED, **opts)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    n_particles = sim.num_particles()
    for _ in range(args.warmup):
        sim.runFrame()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # ---- timed region: device-resident state, per-step CUDA events ----
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    l0 = sim.launch_count()
    iters, outers = [], []
    barrier()
    torch.cuda.synchronize()
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.runFrame()
        e1.record(stream)
        evs.append((e0, e1))
        st_ = sim.stats()
        iters.append(st_["pcgIterations"])
        outers.append(st_["irOuterIterations"])
    torch.cuda.synchronize()
    barrier()
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    launches = sim.launch_count() - l0
    clk = clocks.stop()
    stage_ms = [round(x, 3) for x in sim.stage_times()]

    # ---- per-kernel times (CUDA events on the simulation's stream around
    # each launch) from a few extra steps outside the headline region ----
    kt_steps = 3
    sim.set_kernel_timing(",".join(DOMINANT))
    kt_total = 0.0
    for _ in range(kt_steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.runFrame()
        e1.record(stream)
        torch.cuda.synchronize()
        kt_total += e0.elapsed_time(e1)
    ktimes = sim.kernel_times()
    sim.set_kernel_timing("")
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    cells = args.size * args.size
    value = cells * args.steps * world / (total_ms / 1000.0)

    # ---- roofline of the dominant kernel ----
    # the FP32 MIC(0) forward and backward sweeps are one kernel template with
    # the same bytes per cell: reported together as "mic32"
    if "mic32_forward" in ktimes and "mic32_backward" in ktimes:
        nf, mf = ktimes.pop("mic32_forward")
        nb_, mb = ktimes.pop("mic32_backward")
        ktimes["mic32"] = (nf + nb_, mf + mb)
    dom = max((k for k in ktimes if k in KERNEL_BYTES_PER_CELL), key=lambda k: ktimes[k][1], default=None)
    roofline = None
    if dom is not None:
        n_launch, ms = ktimes[dom]
        alg_bytes = KERNEL_BYTES_PER_CELL[dom] * cells
        achieved = alg_bytes / (ms / n_launch / 1000.0) / 1e9
        peak, peak_src = 6800.0, "fallback"
        try:
            peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
            peak_src = "measured"
        except Exception:
            pass
        traffic = None
        tf = os.path.join(ROOT, "profiles", "traffic.txt")
        if os.path.exists(tf):
            for line in open(tf):
                parts = line.split()
                if len(parts) >= 3 and parts[0] == dom and parts[1] == args.precision:
                    # measured per launch at 1024^2; a launch reads each cell's operands once
                    traffic = float(parts[2]) * cells / (1024 * 1024)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "peak_source": peak_src,
                    "traffic": traffic, "launches": n_launch, "avg_launch_us": round(1000 * ms / n_launch, 2),
                    "algorithmic_bytes_per_launch": alg_bytes,
                    "share_of_step": round(ktimes[dom][1] / kt_total, 3),
                    "kernel_ms_per_step": {k: round(v[1] / kt_steps, 3) for k, v in sorted(ktimes.items())},
                    "kernels": {k: {"launches_per_step": v[0] / kt_steps, "ms_per_step": round(v[1] / kt_steps, 3),
                                    "achieved_gbs": round(KERNEL_BYTES_PER_CELL[k] * cells * v[0] / (v[1] / 1000.0)
                                                          / 1e9, 1),
                                    "frac": round(KERNEL_BYTES_PER_CELL[k] * cells * v[0] / (v[1] / 1000.0) / 1e9
                                                  / peak, 4)}
                                for k, v in sorted(ktimes.items()) if k in KERNEL_BYTES_PER_CELL and v[1] > 0},
                    "timed_over": f"{kt_steps} extra steps with per-launch events"}

    # ---- whole-step roofline: compulsory bytes of every stage per step ----
    # per cell: PCG 24 b per inner iteration (b = 4 for the mixed inner solve,
    # 8 for FP64), 48 B per FP64 refinement residual, matrix + rhs build 73 B,
    # MIC(0) factor 4 b, velocity update 49 B, level set (16 closest-point
    # sweeps x 24 B, 16 Eikonal sweeps x 16 B, seeding 12 B, smoothing 32 B),
    # grid side of P2G / G2P / particle advection (32 + 32 + 16 B); per
    # particle: P2G 28 B, G2P 24 B, advection 16 B, level-set seeding 8 B.
    # Extrapolation faces are not counted (data dependent, a few % of cells).
    b = 4 if args.precision == "mixed" else 8
    it_mean = float(np.mean(iters))
    out_mean = float(np.mean(outers)) if args.precision == "mixed" else 0.0
    per_cell = 24 * b * it_mean + 48 * out_mean + 73 + 4 * b + 49 + (16 * 24 + 16 * 16 + 12 + 32) + (32 + 32 + 16)
    step_bytes = per_cell * cells + (28 + 24 + 16 + 8) * n_particles
    step_achieved = step_bytes / (total_ms / args.steps / 1000.0) / 1e9
    step_roofline = {"bound": "hbm", "algorithmic_bytes_per_step": int(step_bytes),
                     "achieved": round(step_achieved, 1), "peak": roofline["peak"] if roofline else 6800.0,
                     "unit": "GB/s", "frac": round(step_achieved / (roofline["peak"] if roofline else 6800.0), 4),
                     "pcg_iterations_per_step": it_mean, "refinement_sweeps_per_step": out_mean,
                     "formula": "sum of the stages' compulsory bytes per step / measured step time"}

    # ---- e2e: through the C ABI with host buffers (upload + frame + download) ----
    e2e = None
    st = sim.get_state() if args.e2e_steps > 0 else {}
    host_in = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in st.items()}
    host_out = {k: torch.from_numpy(v.copy()).pin_memory().numpy() for k, v in st.items()}
    h2d = state_bytes(host_in)
    d2h = state_bytes(host_out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        sim.set_state(host_in)
        sim.runFrame()
        sim.get_state(out=host_out)
        host_in, host_out = host_out, host_in
    e2e_s = time.perf_counter() - t0
    if args.e2e_steps > 0:
        e2e = {"value": cells * args.e2e_steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
               "path": "fs2d_upload_state + fs2d_run_frame + fs2d_download_state, full state, pinned host buffers"}

    # ---- accuracy of the mixed and FP64 projections against the FP64 oracle ----
    oracle_err = None
    if rank == 0 and not args.no_oracle_error:
        oracle_err = error_vs_oracle(args, sc, sim.get_state(), stream, local)

    # ---- the all-FP64 GPU path on the same workload (fewer steps) ----
    fp64_path = None
    if args.precision == "mixed" and args.fp64_steps > 0:
        sim64 = fs2d.FluidSim2D(sc, seed=SEED, **dict(opts, precision="fp64"))
        sim64.set_stream(stream.cuda_stream)
        for _ in range(min(args.warmup, 3)):
            sim64.runFrame()
        torch.cuda.synchronize()
        ms64 = 0.0
        for _ in range(args.fp64_steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim64.runFrame()
            e1.record(stream)
            torch.cuda.synchronize()
            ms64 += e0.elapsed_time(e1)
        fp64_path = {"value": cells * args.fp64_steps / (ms64 / 1000.0), "unit": UNIT,
                     "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps,
                     "stage_ms_last_step": [round(x, 3) for x in sim64.stage_times()],
                     "pcg_iterations_last_step": sim64.stats()["pcgIterations"]}
        sim64.close()

    # ---- semi-Lagrangian variant of the plain dam break at the same size ----
    sl_path = None
    if args.sl_steps > 0:
        import scenes
        ssc = scenes.sl_dam_break(args.size, dt=(1.0 / 120) * (64.0 / args.size))
        ssim = fs2d.FluidSim2D(ssc, seed=SEED, **opts)
        ssim.set_stream(stream.cuda_stream)
        for _ in range(3):
            ssim.runFrame()
        torch.cuda.synchronize()
        sms = 0.0
        for _ in range(args.sl_steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ssim.runFrame()
            e1.record(stream)
            torch.cuda.synchronize()
            sms += e0.elapsed_time(e1)
        sl_path = {"scene": f"semi-Lagrangian dam break x<0.4, y<0.6, {args.size}^2, dt 1/120 scaled by 64/{args.size}",
                   "value": cells * args.sl_steps / (sms / 1000.0), "unit": UNIT,
                   "ms_per_step": sms / args.sl_steps, "steps": args.sl_steps, "precision": args.precision,
                   "stage_ms_last_step": [round(x, 3) for x in ssim.stage_times()]}
        ssim.close()

    # ---- standalone pressure solve: random disks, N(0,1) velocities, 1e-10 ----
    pressure = None
    if args.pressure_size > 0:
        import scenes
        n = args.pressure_size
        psc, pcell, pphi, pu, pv = scenes.pressure_disks(n, n, seed=n)
        pressure = {"grid": [n, n], "tol": 1e-10, "labels": "fluid with random air (~25%) and solid (~5%) disks",
                    "rhs": "divergence of N(0,1) FP32 face velocities", "timing": "CUDA events around the solve, "
                    "inputs resident on the device, after one untimed solve"}
        sols = {}
        for prec in ("fp64", "mixed"):
            ps = fs2d.FluidSim2D(psc, seed=1, precision=prec, pcg_tol=1e-10, pcg_max_iters=5000, ir_inner_tol=1e-4,
                                 device=local)
            ps.set_stream(stream.cuda_stream)
            ps.set_state({"cell": pcell, "phi": pphi, "u": pu, "v": pv})
            ps.stage("applyProjection")
            ps.set_state({"cell": pcell, "phi": pphi, "u": pu, "v": pv})
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ps.stage("applyProjection")
            e1.record(stream)
            torch.cuda.synchronize()
            st = ps.stats()
            sols[prec] = ps.get_state(["p"])["p"]
            pressure[prec] = {"ms": e0.elapsed_time(e1), "pcg_iterations": st["pcgIterations"],
                              "refinement_sweeps": st["irOuterIterations"], "rel_residual": st["pcgRelResidual"]}
            ps.close()
        pressure["fp64_over_mixed_time"] = pressure["fp64"]["ms"] / pressure["mixed"]["ms"]
        pressure["max_rel_diff_mixed_vs_fp64"] = float(np.abs(sols["mixed"] - sols["fp64"]).max() /
                                                       np.abs(sols["fp64"]).max())

    # ---- differentiable rollout: closed box, forward and hand-written adjoint ----
    adjoint = None
    if args.adjoint_size > 0:
        import scenes
        n, T = args.adjoint_size, args.adjoint_steps
        asc = scenes.closed_box(n)
        au0, av0 = scenes.fourier_faces(n, n, seed=1)
        aut, avt = scenes.fourier_faces(n, n, seed=2)
        dev = [torch.tensor(a, device=f"cuda:{local}") for a in (au0, av0, aut, avt)]
        gdu, gdv = torch.empty_like(dev[0]), torch.empty_like(dev[1])
        ptrs = [t.data_ptr() for t in dev]
        every = int(np.ceil(np.sqrt(T)))
        adjoint = {"grid": [n, n], "steps": T, "checkpoint_every": every, "dt": asc["dt"], "pcg_tol": 1e-12,
                   "initial": "16-mode Fourier field, amplitude 1",
                   "timing": "CUDA events on the handle's stream, inputs resident on the device, after one untimed "
                             "pair, mean of 3; backward includes recomputing the checkpointed segments"}
        grads = {}
        for prec in ("mixed", "fp64"):
            asim = fs2d.FluidSim2D(asc, seed=1, precision=prec, pcg_tol=1e-12, pcg_max_iters=2000, device=local)
            asim.set_stream(stream.cuda_stream)
            asim.forward(T, *ptrs)                      # warm-up pair
            asim.backward(gdu.data_ptr(), gdv.data_ptr())
            fwd_ms, bwd_ms, reps = 0.0, 0.0, 3
            l0 = asim.launch_count()
            for _ in range(reps):
                torch.cuda.synchronize()
                e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
                e0.record(stream)
                loss = asim.forward(T, *ptrs)
                e1.record(stream)
                asim.backward(gdu.data_ptr(), gdv.data_ptr())
                e2.record(stream)
                torch.cuda.synchronize()
                fwd_ms += e0.elapsed_time(e1)
                bwd_ms += e1.elapsed_time(e2)
            grads[prec] = torch.cat([gdu, gdv]).cpu().numpy()
            adjoint[prec] = {"loss": loss, "forward_ms": fwd_ms / reps, "backward_ms": bwd_ms / reps,
                             "backward_over_forward": bwd_ms / fwd_ms,
                             "cell_steps_per_s_forward": n * n * T / (fwd_ms / reps / 1000.0),
                             "gpu_launches_per_pair": (asim.launch_count() - l0) // reps}
            asim.close()
        adjoint["backward_over_forward"] = adjoint["mixed"]["backward_over_forward"]
        adjoint["max_rel_diff_grad_mixed_vs_fp64"] = float(np.abs(grads["mixed"] - grads["fp64"]).max() /
                                                           np.abs(grads["fp64"]).max())

    # ---- batch: independent PIC/FLIP dam breaks of uneven sizes ----
    batch = None
    if args.batch_scenes > 0:
        import scenes
        import shard
        all_b = scenes.batch_dam_breaks(args.batch_scenes, seed=SEED)
        bcells = sum(sc["sizeX"] * sc["sizeY"] for sc in all_b)
        # several GPUs: the scenes are split over the ranks (no exchange during the steps)
        bparts = shard.partition([sc["sizeX"] * sc["sizeY"] for sc in all_b], world)
        bscs = [all_b[k] for k in bparts[rank]]
        bt = fs2d.Batch(bscs, workers=0, seed=SEED, precision="mixed", pcg_tol=args.tol, pcg_max_iters=200,
                        device=local)
        t0 = time.perf_counter()
        bt.step(max(args.warmup, 3))                 # the first frames choose the worker count
        warm_s = time.perf_counter() - t0
        torch.cuda.synchronize()
        l0 = bt.launch_count()
        t0 = time.perf_counter()
        bt.step(args.batch_steps)
        torch.cuda.synchronize()
        conc_s = time.perf_counter() - t0
        phases = bt.phase_ms()
        if world > 1:
            t = torch.tensor([conc_s], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            conc_s = float(t.item())
        l1 = bt.launch_count()
        workers = bt.workers
        bt.workers = 1
        t0 = time.perf_counter()
        bt.step(1)
        torch.cuda.synchronize()
        seq_s = time.perf_counter() - t0
        sides = sorted(sc["sizeX"] for sc in all_b)
        # the persistent sweep of the pack (FP32 MIC(0) forward, every scene's
        # strips as work items) as the autotuner timed it at batch creation
        # (CUDA events, warm), against 16 B per cell (3 operands in, 1 out)
        sched = bt.sweep_schedule()
        my_cells = sum(sc["sizeX"] * sc["sizeY"] for sc in bscs)
        peak = 6800.0
        try:
            peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        except Exception:
            pass
        sweep_gbs = 16.0 * my_cells / (sched["sweep_us"] * 1e-6) / 1e9 if sched["sweep_us"] > 0 else None
        batch_roofline = {"kernel": "mic32 (several scenes, persistent)", "bound": "hbm",
                          "algorithmic_bytes_per_launch": 16 * my_cells, "avg_launch_us": round(sched["sweep_us"], 2),
                          "achieved": round(sweep_gbs, 1) if sweep_gbs else None, "peak": peak, "unit": "GB/s",
                          "frac": round(sweep_gbs / peak, 4) if sweep_gbs else None,
                          "schedule": sched["schedule"], "ctas": sched["ctas"], "work_items": sched["items"],
                          "timing": "CUDA events over 3 forward sweeps of every scene, after a warm-up sweep, "
                                    "by the batch's autotuner at creation"}
        batch = {"scenes": len(all_b), "scenes_per_rank": [len(p) for p in bparts], "cells": bcells, "side_min": sides[0], "side_median": sides[len(sides) // 2],
                 "side_max": sides[-1], "steps": args.batch_steps, "workers": workers,
                 "value": bcells * args.batch_steps / conc_s, "unit": UNIT,
                 "ms_per_batch_step": 1000.0 * conc_s / args.batch_steps,
                 "sequential_value_rank0": sum(sc["sizeX"] * sc["sizeY"] for sc in bscs) / seq_s,
                 "concurrency_speedup_rank0": seq_s / (conc_s / args.batch_steps),
                 "gpu_launches_per_batch_step": (l1 - l0) // max(args.batch_steps, 1),
                 "roofline": batch_roofline,
                 "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                 "phase_ms_per_batch_step": {"stages_before_solve": round(phases[0] / args.batch_steps, 2),
                                             "joint_pressure_solve": round(phases[1] / args.batch_steps, 2),
                                             "stages_after_solve": round(phases[2] / args.batch_steps, 2),
                                             "level_set_sweeps_device": round(phases[3] / args.batch_steps, 2)},
                 "warmup_s": warm_s,
                 "timing": "host wall clock around fs2d_batch_step (each frame returns after its device work), "
                           "max over ranks; sequential = rank 0's scenes with one worker, one step"}
        bt.close()

    # ---- batched rollouts: closed boxes of uneven sizes, forward and adjoint ----
    batch_adjoint = None
    if args.batch_adjoint_scenes > 0:
        import scenes
        T = args.batch_adjoint_steps
        import shard
        all_c = scenes.batch_closed_boxes(args.batch_adjoint_scenes, seed=SEED)
        ccells = sum(sc["sizeX"] * sc["sizeY"] for sc in all_c)
        cparts = shard.partition([sc["sizeX"] * sc["sizeY"] for sc in all_c], world)
        cscs = [all_c[k] for k in cparts[rank]]
        ins = [scenes.fourier_faces(sc["sizeX"], sc["sizeY"], seed=1 + k) for k, sc in zip(cparts[rank], cscs)]
        tgs = [scenes.fourier_faces(sc["sizeX"], sc["sizeY"], seed=1000 + k) for k, sc in zip(cparts[rank], cscs)]
        dins = [[torch.tensor(a, device=f"cuda:{local}") for a in pair] for pair in ins]
        dtgs = [[torch.tensor(a, device=f"cuda:{local}") for a in pair] for pair in tgs]
        grads = [[torch.empty_like(p[0]), torch.empty_like(p[1])] for p in dins]
        ba = fs2d.Batch(cscs, workers=8, seed=SEED, precision="mixed", pcg_tol=1e-12, pcg_max_iters=2000,
                        device=local)
        u0p = [p[0].data_ptr() for p in dins]
        v0p = [p[1].data_ptr() for p in dins]
        utp = [p[0].data_ptr() for p in dtgs]
        vtp = [p[1].data_ptr() for p in dtgs]
        gup = (ctypes.c_void_p * len(cscs))(*[g[0].data_ptr() for g in grads])
        gvp = (ctypes.c_void_p * len(cscs))(*[g[1].data_ptr() for g in grads])

        def bwd():
            fs2d._check(fs2d.load().fs2d_batch_backward(ba.h, ctypes.cast(gup, ctypes.c_void_p),
                                                        ctypes.cast(gvp, ctypes.c_void_p)))

        ba.forward(T, u0p, v0p, utp, vtp)           # warm-up pair
        bwd()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        my_losses = ba.forward(T, u0p, v0p, utp, vtp)
        torch.cuda.synchronize()
        f_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        bwd()
        torch.cuda.synchronize()
        b_s = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([f_s, b_s], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            f_s, b_s = (float(x) for x in t.tolist())
        # host gather of the per-scene losses (the batch's only exchange)
        losses_all = shard.gather(dict(zip(cparts[rank], my_losses.tolist())), cparts, rank, world)
        sides = sorted(sc["sizeX"] for sc in all_c)
        batch_adjoint = {"scenes": len(all_c), "scenes_per_rank": [len(p) for p in cparts], "cells": ccells,
                         "loss_sum": float(sum(losses_all)), "side_min": sides[0], "side_max": sides[-1],
                         "steps": T, "checkpoint_every": int(np.ceil(np.sqrt(T))), "workers": 8, "precision": "mixed",
                         "pcg_tol": 1e-12, "forward_s": f_s, "backward_s": b_s, "backward_over_forward": b_s / f_s,
                         "forward_cell_steps_per_s": ccells * T / f_s,
                         "timing": "host wall clock around fs2d_batch_forward / fs2d_batch_backward (each returns after "
                                   "its device work), max over ranks, inputs resident on the device, after one untimed "
                                   "pair"}
        ba.close()

    # ---- the 3D containers (include/fs3d.h) ----
    grid3d = None
    if args.grid3d_size > 0 and rank == 0:
        try:
            peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        except (OSError, ValueError, KeyError):
            peak = 6800.0
        try:
            grid3d = bench_grid3d(args.grid3d_size, local, peak)
        except RuntimeError as e:   # reported in the line, not a failed headline
            grid3d = {"error": str(e)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded dam break + disk, libc rand() particle jitter)",
        "config": config_dict(args, n_particles),
        "precision": args.precision, "pcg_iterations_per_step": iters,
        "stage_ms_last_step": stage_ms,
        "fp64_path": fp64_path,
        "error_vs_oracle": oracle_err,
        "sl_path": sl_path,
        "pressure_solve": pressure,
        "adjoint": adjoint,
        "batch": batch,
        "batch_adjoint": batch_adjoint,
        "grid3d": grid3d,
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": roofline,
        "step_roofline": step_roofline,
        "e2e": e2e,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, args.cpu_budget, 10)
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
