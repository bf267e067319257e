"""Build recipe for the oracle (test infrastructure).

Two kinds of artefacts:

* ``oracle/_build/liboracle.so`` (and ``liboracle_omp.so``): the C
  restatement in ``oracle/restate/``, always buildable (here and on the GPU
  box).  The plain build is serial with ``-ffp-contract=off`` (bit-exact
  parity); the ``_omp`` build adds ``-O3 -fopenmp`` for CPU timing.
* ``oracle/_ref/libfs2d_ref*.so``: the UNMODIFIED reference simulator
  (``src/FluidSim2D.cpp``, ``src/PerformanceCounter.cpp``), compiled in
  place from the reference checkout together with the compatibility shim
  (``oracle/shim``) and a C wrapper (``oracle/ref_capi.cpp``).  Only built
  when the location of a reference checkout is given, as the argument of
  ``build_reference`` or in the environment variable ``FS2D_REFERENCE_DIR``
  (there is no default location).  Variants:
    - ``libfs2d_ref.so``      scalar path (USE_AVX off), serial,
                              ``-O2 -ffp-contract=off`` — the parity build;
    - ``libfs2d_ref_avx.so``  the reference's Release configuration on x86:
                              ``-O3 -mavx -mfma -DUSE_AVX_SIMD`` (timing);
    - ``libfs2d_ref_omp.so``  the same plus ``-fopenmp`` (USE_OPENMP=ON);
    - ``libfs3d_ref.so``      the header-only 3D containers
                              (``include/Array3D.h``, ``include/MACGrid3D.h``)
                              behind ``oracle/ref3d_capi.cpp``, serial,
                              ``-O2 -ffp-contract=off``.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in inputs if os.path.exists(p))


def build_restatement(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "restate", "fs2d_oracle.c"), os.path.join(HERE, "restate", "fs3d_oracle.c")]
    deps = srcs + [os.path.join(HERE, "restate", "fs2d_oracle.h"), os.path.join(HERE, "restate", "fs3d_oracle.h"),
                   os.path.join(HERE, "..", "include", "fs2d.h")]
    jobs = []
    plain = os.path.join(BUILD, "liboracle.so")
    omp = os.path.join(BUILD, "liboracle_omp.so")
    common = ["gcc", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]
    if force or _stale(plain, deps):
        jobs.append(common + ["-O2", *srcs, "-o", plain, "-lm"])
    if force or _stale(omp, deps):
        jobs.append(common + ["-O3", "-DNDEBUG", "-fopenmp", *srcs, "-o", omp, "-lm"])
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return plain


def reference_dir(path=None):
    """The reference checkout: `path`, else $FS2D_REFERENCE_DIR; None when
    neither names a directory holding src/FluidSim2D.cpp."""
    path = path or os.environ.get("FS2D_REFERENCE_DIR")
    if path and os.path.exists(os.path.join(path, "src", "FluidSim2D.cpp")):
        return path
    return None


def reference_available(path=None):
    return reference_dir(path) is not None


def build_reference(force=False, path=None):
    """Compile the reference in place; returns the list of built libraries
    (empty when no reference checkout is given)."""
    ref_dir = reference_dir(path)
    if ref_dir is None:
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    srcs = [os.path.join(ref_dir, "src", "FluidSim2D.cpp"),
            os.path.join(ref_dir, "src", "PerformanceCounter.cpp"),
            os.path.join(HERE, "ref_capi.cpp")]
    shim = os.path.join(HERE, "shim", "altlib")
    noavx = os.path.join(HERE, "shim", "noavx")
    inc = os.path.join(ref_dir, "include")
    deps = srcs + [os.path.join(shim, f) for f in os.listdir(shim)] + \
        [os.path.join(inc, f) for f in os.listdir(inc)]
    base = ["g++", "-std=gnu++14", "-fPIC", "-shared", "-Wno-format", "-I", shim, "-I", inc]
    variants = {
        "libfs2d_ref.so": ["-O2", "-ffp-contract=off", "-I", noavx],
    }
    if platform.machine() in ("x86_64", "AMD64"):
        variants["libfs2d_ref_avx.so"] = ["-O3", "-DNDEBUG", "-mavx", "-mfma", "-DUSE_AVX_SIMD"]
        variants["libfs2d_ref_omp.so"] = ["-O3", "-DNDEBUG", "-mavx", "-mfma", "-DUSE_AVX_SIMD", "-fopenmp"]
    else:
        variants["libfs2d_ref_omp.so"] = ["-O3", "-DNDEBUG", "-fopenmp", "-I", noavx]
    jobs, outs = [], []
    for name, flags in variants.items():
        out = os.path.join(REF_OUT, name)
        outs.append(out)
        if force or _stale(out, deps):
            jobs.append(base + flags + srcs + ["-o", out])
    # the 3D containers are header-only: one wrapper translation unit
    src3 = os.path.join(HERE, "ref3d_capi.cpp")
    out3 = os.path.join(REF_OUT, "libfs3d_ref.so")
    outs.append(out3)
    deps3 = [src3, os.path.join(inc, "Array3D.h"), os.path.join(inc, "MACGrid3D.h")] + \
        [os.path.join(shim, f) for f in os.listdir(shim)]
    if force or _stale(out3, deps3):
        jobs.append(base + ["-O2", "-ffp-contract=off", "-I", noavx, src3, "-o", out3])
    with ThreadPoolExecutor(max_workers=4) as ex:
        list(ex.map(_run, jobs))
    return outs


if __name__ == "__main__":
    # python oracle/build_oracle.py [-f] [REFERENCE_DIR]
    rest = [a for a in sys.argv[1:] if a != "-f"]
    print(build_restatement(force="-f" in sys.argv))
    print(build_reference(force="-f" in sys.argv, path=rest[0] if rest else None))
