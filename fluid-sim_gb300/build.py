"""Build recipe of the GB300 FluidSim2D library (libfs2d.so, in-tree).

Compiles every CUDA translation unit in csrc/ for sm_103a only, in parallel,
and links them into fluid-sim_gb300/libfs2d.so exposing the C ABI declared in
include/fs2d.h.  Stage files whose FP64 arithmetic must round like the
reference's serial C++ are compiled with --fmad=false (no fused
multiply-add); the others keep the default contraction.

    python fluid-sim_gb300/build.py [-f]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build", "obj")
LIB = os.path.join(HERE, "libfs2d.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation unit -> extra flags
UNITS = {
    "capi.cu": [],
    "levelset.cu": ["--fmad=false"],
    "transfer.cu": ["--fmad=false"],
    "advect.cu": ["--fmad=false"],
    "projection.cu": ["--fmad=false"],
    "projection_mixed.cu": [],
    "render.cu": ["--fmad=false"],
    "adjoint.cu": ["--fmad=false"],
    "batch.cu": [],
    "grid3d.cu": ["--fmad=false"],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(ROOT, "include", h) for h in ("fs2d.h", "fs3d.h")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-6000:])
    return r.stdout + r.stderr


def build(force=False, verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    base = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
            *extra]
    if verbose:
        base += ["-Xptxas", "-v"]
    jobs, objs = [], []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src, __file__] + headers):
            jobs.append(base + flags + ["-c", src, "-o", obj])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-Xlinker", "--no-undefined", "-o", LIB, *objs])
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(force="-f" in sys.argv, verbose="-v" in sys.argv)
    for l in logs:
        if l.strip():
            print(l)
    print(lib)
