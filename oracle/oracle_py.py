"""ctypes bindings for the oracle (test infrastructure only).

Imported by tests/, by ``__graft_entry__.smoke()`` (as the checker) and by
bench.py's CPU-baseline leg.  Nothing in the product imports this module.

Two interchangeable simulators with the same Python surface:

* :class:`OracleSim` — the C restatement (``oracle/restate``), built on
  every machine;
* :class:`RefSim` — the unmodified reference compiled from its sources
  (``oracle/_ref``), only where the reference checkout exists.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

STAGES = {
    "createWaterLevelSet": 1,
    "transferVelocityToGrid": 2,
    "applySemiLagrangianAdvection": 3,
    "applyGravity": 4,
    "createSolidLevelSet": 5,
    "applyProjection": 6,
    "updateVelocity": 7,
    "updateParticleVelocities": 8,
    "applyAdvection": 9,
}


class Config(C.Structure):
    """Mirror of fs2d_config / FluidSim2DConfig (include/FluidSim2D.h:48-63)."""
    _fields_ = [("sizeX", C.c_int), ("sizeY", C.c_int), ("particlesPerCellSqrt", C.c_int),
                ("dt", C.c_double), ("dx", C.c_double), ("rho", C.c_double),
                ("gravityX", C.c_double), ("gravityY", C.c_double),
                ("mode", C.c_int), ("picFlipAlpha", C.c_double),
                ("initialValues", C.POINTER(C.c_uint8))]


class State(C.Structure):
    _fields_ = [("cell", C.POINTER(C.c_uint8)), ("phi", C.POINTER(C.c_double)),
                ("p", C.POINTER(C.c_double)), ("u", C.POINTER(C.c_double)),
                ("v", C.POINTER(C.c_double)), ("newU", C.POINTER(C.c_double)),
                ("newV", C.POINTER(C.c_double)), ("particles", C.POINTER(C.c_double)),
                ("particleVels", C.POINTER(C.c_double)), ("numParticles", C.c_size_t)]


class OrOptions(C.Structure):
    _fields_ = [("mic_tau", C.c_double), ("mic_sigma", C.c_double), ("pcg_tol", C.c_double),
                ("pcg_max_iters", C.c_int), ("sl_inplace", C.c_int), ("extrapolate_band", C.c_int),
                ("volume_rate", C.c_double)]


def make_config(scene):
    """fs2d_config from a scene dict (see fluid-sim_gb300/scenes.py); keeps
    the label array alive on the returned object."""
    cells = np.ascontiguousarray(scene["cells"], dtype=np.uint8)
    cfg = Config(scene["sizeX"], scene["sizeY"], scene["ppcSqrt"], scene["dt"], scene["dx"],
                 scene["rho"], scene["gravityX"], scene["gravityY"], scene["mode"],
                 scene["picFlipAlpha"], cells.ctypes.data_as(C.POINTER(C.c_uint8)))
    cfg._keep = cells
    return cfg


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def state_arrays(nx, ny, n_particles):
    return {
        "cell": np.zeros(nx * ny, np.uint8),
        "phi": np.zeros(nx * ny),
        "p": np.zeros(nx * ny),
        "u": np.zeros((nx + 1) * ny),
        "v": np.zeros(nx * (ny + 1)),
        "newU": np.zeros((nx + 1) * ny),
        "newV": np.zeros(nx * (ny + 1)),
        "particles": np.zeros(2 * n_particles),
        "particleVels": np.zeros(2 * n_particles),
    }


def state_view(arrs):
    st = State()
    for name in ("phi", "p", "u", "v", "newU", "newV", "particles", "particleVels"):
        a = arrs.get(name)
        setattr(st, name, _ptr(a, C.c_double) if a is not None else None)
    st.cell = _ptr(arrs.get("cell"), C.c_uint8) if arrs.get("cell") is not None else None
    parts = arrs.get("particles")
    st.numParticles = 0 if parts is None else len(parts) // 2
    return st


class _SimBase:
    lib = None
    prefix = ""

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def stage(self, name):
        rc = self._f("run_stage")(self.h, STAGES[name] if isinstance(name, str) else name)
        return rc

    def num_particles(self):
        return int(self._f("num_particles")(self.h))

    def get_state(self):
        arrs = state_arrays(self.nx, self.ny, self.num_particles())
        st = state_view(arrs)
        rc = self._f("get_state")(self.h, C.byref(st))
        assert rc == 0
        return arrs

    def set_state(self, arrs):
        arrs = {k: (np.ascontiguousarray(v) if v is not None else None) for k, v in arrs.items()}
        st = state_view(arrs)
        rc = self._f("set_state")(self.h, C.byref(st))
        assert rc == 0

    def stats(self):
        out = (C.c_double * 6)()
        self._f("stats")(self.h, out)
        keys = ("waterVolume", "totalEnergy", "particleTotalEnergy", "avgPressure",
                "avgPressureInFluid", "maxVelocity")
        return dict(zip(keys, list(out)))

    def close(self):
        if getattr(self, "h", None):
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _load(path, prefix):
    lib = C.CDLL(path)
    getattr(lib, prefix + "create").restype = C.c_void_p
    getattr(lib, prefix + "num_particles").restype = C.c_size_t
    getattr(lib, prefix + "num_particles").argtypes = [C.c_void_p]
    getattr(lib, prefix + "run_stage").argtypes = [C.c_void_p, C.c_int]
    getattr(lib, prefix + "run_frame").argtypes = [C.c_void_p]
    getattr(lib, prefix + "destroy").argtypes = [C.c_void_p]
    getattr(lib, prefix + "get_state").argtypes = [C.c_void_p, C.POINTER(State)]
    getattr(lib, prefix + "set_state").argtypes = [C.c_void_p, C.POINTER(State)]
    getattr(lib, prefix + "stats").argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    return lib


_libs = {}


def _oracle_path(omp):
    import importlib.util
    spec = importlib.util.spec_from_file_location("fs2d_build_oracle", os.path.join(HERE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_restatement()
    return os.path.join(HERE, "_build", "liboracle_omp.so" if omp else "liboracle.so")


def get_oracle_lib(omp=False):
    key = "oracle_omp" if omp else "oracle"
    if key not in _libs:
        lib = _load(_oracle_path(omp), "or_")
        lib.or_create.argtypes = [C.POINTER(Config), C.POINTER(OrOptions), C.c_int, C.c_uint]
        lib.or_set_options.argtypes = [C.c_void_p, C.POINTER(OrOptions)]
        lib.or_solver_info.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.or_set_params.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]
        lib.or_tricubic.restype = C.c_double
        lib.or_tricubic.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.c_double, C.c_double]
        lib.or_extrapolate.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_uint32), C.c_int]
        lib.or_reseed.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint, C.POINTER(C.c_size_t)]
        lib.or_reseed_jitter.argtypes = [C.c_uint, C.c_size_t, C.c_uint, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
        _libs[key] = lib
    return _libs[key]


def reference_lib_path(variant=""):
    return os.path.join(HERE, "_ref", f"libfs2d_ref{variant}.so")


def get_reference_lib(variant=""):
    """The compiled reference, or None where it was not built (e.g. on a
    machine without the reference checkout)."""
    key = "ref" + variant
    if key not in _libs:
        path = reference_lib_path(variant)
        if not os.path.exists(path):
            return None
        lib = _load(path, "ref_")
        lib.ref_create.argtypes = [C.POINTER(Config), C.c_int, C.c_uint]
        lib.ref_set_gravity.argtypes = [C.c_void_p, C.c_double, C.c_double]
        lib.ref_save_stats.argtypes = [C.c_void_p]
        lib.ref_num_stages.argtypes = [C.c_void_p]
        lib.ref_feed_stats.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        _libs[key] = lib
    return _libs[key]


def default_or_options(**kw):
    o = OrOptions(0.999, 0.25, 1e-12, 200, 1, 0)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class OracleSim(_SimBase):
    """The C restatement.  Options: mic_tau, mic_sigma, pcg_tol,
    pcg_max_iters, sl_inplace (1 = reference semantics), extrapolate_band,
    volume_rate (0 = reference semantics)."""
    prefix = "or_"

    def __init__(self, scene, seed=None, omp=False, **opts):
        self.lib = get_oracle_lib(omp)
        self.nx, self.ny = scene["sizeX"], scene["sizeY"]
        self.cfg = make_config(scene)
        self.opts = default_or_options(**opts)
        self.h = self.lib.or_create(C.byref(self.cfg), C.byref(self.opts),
                                    0 if seed is None else 1, 0 if seed is None else seed)

    def set_options(self, **opts):
        for k, v in opts.items():
            setattr(self.opts, k, v)
        self.lib.or_set_options(self.h, C.byref(self.opts))

    def frame(self):
        return self.lib.or_run_frame(self.h)

    def solver_info(self):
        out = (C.c_double * 2)()
        self.lib.or_solver_info(self.h, out)
        return {"iterations": int(out[0]), "rel_residual": out[1]}

    def set_params(self, gx, gy, alpha, dt):
        self.lib.or_set_params(self.h, gx, gy, alpha, dt)

    def reseed(self, min_per_cell, max_per_cell, seed):
        """Particle reseeding (an option the reference lacks; see or_reseed)."""
        out = (C.c_size_t * 2)()
        self.lib.or_reseed(self.h, min_per_cell, max_per_cell, seed, out)
        return {"removed": int(out[0]), "added": int(out[1]), "numParticles": self.num_particles()}


class RefSim(_SimBase):
    """The unmodified reference (oracle/_ref)."""
    prefix = "ref_"

    def __init__(self, scene, seed=None, variant=""):
        self.lib = get_reference_lib(variant)
        if self.lib is None:
            raise RuntimeError("reference library not built")
        self.nx, self.ny = scene["sizeX"], scene["sizeY"]
        self.cfg = make_config(scene)
        self.h = self.lib.ref_create(C.byref(self.cfg), 0 if seed is None else 1, 0 if seed is None else seed)

    def frame(self):
        self.lib.ref_run_frame(self.h)
        return 0

    def save_stats_of(self, stage_ms, vol, en, pen, directory):
        """The reference's own saveStats (perf.csv, conservation.csv written
        into `directory`) after feeding it the given series: `stage_ms`
        (frames x stages, float32) through PerformanceCounter::endFrame and
        the three conservation series; returns the two files' bytes."""
        stage_ms = np.ascontiguousarray(stage_ms, dtype=np.float32)
        assert stage_ms.shape[1] == self.lib.ref_num_stages(self.h)
        vol, en, pen = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, en, pen))
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)
        self.lib.ref_feed_stats(self.h, stage_ms.ctypes.data_as(fp), stage_ms.shape[0], vol.ctypes.data_as(dp),
                                en.ctypes.data_as(dp), pen.ctypes.data_as(dp), len(vol))
        cwd = os.getcwd()
        os.chdir(directory)
        try:
            self.lib.ref_save_stats(self.h)   # writes ./perf.csv and ./conservation.csv
        finally:
            os.chdir(cwd)
        return (open(os.path.join(directory, "perf.csv"), "rb").read(),
                open(os.path.join(directory, "conservation.csv"), "rb").read())


def tricubic(data, nx, ny, px, py):
    lib = get_oracle_lib()
    a = np.ascontiguousarray(data, dtype=np.float64)
    return lib.or_tricubic(a.ctypes.data_as(C.POINTER(C.c_double)), nx, ny, px, py)


def extrapolate(data, mask, nx, ny, band=0):
    lib = get_oracle_lib()
    a = np.ascontiguousarray(data, dtype=np.float64).copy()
    m = np.ascontiguousarray(mask, dtype=np.uint32).copy()
    lib.or_extrapolate(a.ctypes.data_as(C.POINTER(C.c_double)), nx, ny,
                       m.ctypes.data_as(C.POINTER(C.c_uint32)), band)
    return a, m
