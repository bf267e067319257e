"""Python binding of the GB300 FluidSim2D library (ctypes over include/fs2d.h).

The class mirrors the reference's C++ API (include/FluidSim2D.h:116-150):
``FluidSim2D.create(config)``, ``runFrame()``, ``update()``, the stage
methods (``createWaterLevelSet()``, ``transferVelocityToGrid()``, ...) and
the diagnostics (``avgPressure()``, ``avgPressureInFluid()``,
``maxVelocity()``, ``saveStats()``).  State fields are read and written
through ``get_state()`` / ``set_state()`` as numpy arrays in the
reference's layouts.

There is no CPU fallback: if libfs2d.so is missing or no CUDA device is
usable, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfs2d.so")

PRECISION = {"fp64": 0, "mixed": 1, "fp32": 2}
P2G = {"ordered": 0, "atomic": 1}
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
ERRORS = {0: "OK", 1: "INVALID", 2: "ALLOC", 3: "CUDA", 4: "NOT_CONVERGED", 5: "NONFINITE", 6: "TIMEOUT"}


class Config(C.Structure):
    _fields_ = [("sizeX", C.c_int), ("sizeY", C.c_int), ("particlesPerCellSqrt", C.c_int),
                ("dt", C.c_double), ("dx", C.c_double), ("rho", C.c_double),
                ("gravityX", C.c_double), ("gravityY", C.c_double),
                ("mode", C.c_int), ("picFlipAlpha", C.c_double),
                ("initialValues", C.POINTER(C.c_uint8))]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("mic_tau", C.c_double), ("mic_sigma", C.c_double),
                ("pcg_tol", C.c_double), ("pcg_max_iters", C.c_int), ("ir_inner_tol", C.c_double),
                ("ir_max_outer", C.c_int), ("p2g_mode", C.c_int), ("extrapolate_band", C.c_int),
                ("use_seed", C.c_int), ("seed", C.c_uint), ("device", C.c_int)]


class State(C.Structure):
    _fields_ = [("cell", C.POINTER(C.c_uint8)), ("phi", C.POINTER(C.c_double)),
                ("p", C.POINTER(C.c_double)), ("u", C.POINTER(C.c_double)),
                ("v", C.POINTER(C.c_double)), ("newU", C.POINTER(C.c_double)),
                ("newV", C.POINTER(C.c_double)), ("particles", C.POINTER(C.c_double)),
                ("particleVels", C.POINTER(C.c_double)), ("numParticles", C.c_size_t)]


class Stats(C.Structure):
    _fields_ = [("waterVolume", C.c_double), ("totalEnergy", C.c_double),
                ("particleTotalEnergy", C.c_double), ("origWaterVolume", C.c_double),
                ("currentTime", C.c_double), ("frames", C.c_longlong), ("pcgIterations", C.c_int),
                ("irOuterIterations", C.c_int), ("pcgRelResidual", C.c_double), ("lastStatus", C.c_int)]


class ReseedStats(C.Structure):
    _fields_ = [("removed", C.c_size_t), ("added", C.c_size_t), ("numParticles", C.c_size_t)]


class Array3D(C.Structure):
    """fs3d_array (include/fs3d.h): the reference's Array3D<double> layout with
    a device data pointer."""
    _fields_ = [("data", C.c_void_p), ("NX", C.c_int), ("NY", C.c_int), ("NZ", C.c_int)]


class MACGrid3D(C.Structure):
    """fs3d_mac (include/fs3d.h): the reference's MACGrid3D layout."""
    _fields_ = [("u", Array3D), ("v", Array3D), ("w", Array3D),
                ("sizeX", C.c_int), ("sizeY", C.c_int), ("sizeZ", C.c_int)]


FS3D_AXES = {"u": 0, "v": 1, "w": 2, "uvw": 3}

# Every entry point declared in include/fs2d.h and include/fs3d.h, with its
# ctypes signature.
SIGNATURES = {
    "fs2d_default_options": (None, [C.POINTER(Options)]),
    "fs2d_create": (C.c_int, [C.POINTER(Config), C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "fs2d_destroy": (C.c_int, [C.c_void_p]),
    "fs2d_run_frame": (C.c_int, [C.c_void_p]),
    "fs2d_step": (C.c_int, [C.c_void_p, C.c_int]),
    "fs2d_run_stage": (C.c_int, [C.c_void_p, C.c_int]),
    "fs2d_upload_state": (C.c_int, [C.c_void_p, C.POINTER(State)]),
    "fs2d_download_state": (C.c_int, [C.c_void_p, C.POINTER(State)]),
    "fs2d_num_particles": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "fs2d_set_params": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]),
    "fs2d_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "fs2d_get_history": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_size_t, C.POINTER(C.c_size_t)]),
    "fs2d_avg_pressure": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fs2d_avg_pressure_in_fluid": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fs2d_max_velocity": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fs2d_solve_pressure": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "fs2d_render_export": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fs2d_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_double)]),
    "fs2d_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fs2d_p2g_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fs2d_g2p_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "fs2d_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "fs2d_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "fs2d_batch_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "fs2d_batch_scene": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]),
    "fs2d_batch_workers": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "fs2d_batch_set_workers": (C.c_int, [C.c_void_p, C.c_int]),
    "fs2d_batch_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "fs2d_batch_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fs2d_batch_destroy": (C.c_int, [C.c_void_p]),
    "fs2d_batch_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong)]),
    "fs2d_batch_phase_ms": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "fs2d_batch_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "fs2d_batch_set_schedule": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "fs2d_batch_sweep_schedule": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]),
    "fs2d_get_stage_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]),
    "fs2d_save_stats": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "fs2d_write_stats": (C.c_int, [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                   C.c_char_p, C.c_char_p]),
    "fs2d_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fs2d_debug_wavefront": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.c_int]),
    "fs2d_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong)]),
    "fs2d_last_error": (C.c_char_p, []),
    "fs2d_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_char_p]),
    "fs2d_extrapolate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "fs2d_extrapolate_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "fs2d_get_kernel_times": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "fs2d_reseed": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_uint, C.POINTER(ReseedStats)]),
    "fs2d_cfl": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "fs2d_save_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p]),
    "fs2d_load_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p]),
    "fs2d_debug_fail_alloc": (C.c_int, [C.c_longlong]),
    "fs2d_set_volume_correction": (C.c_int, [C.c_void_p, C.c_double]),
    "fs3d_add": (C.c_int, [C.POINTER(Array3D), C.POINTER(Array3D), C.c_void_p]),
    "fs3d_set_multiply_add": (C.c_int, [C.POINTER(Array3D), C.POINTER(Array3D), C.c_double, C.POINTER(Array3D),
                                        C.c_void_p]),
    "fs3d_inner_product": (C.c_int, [C.POINTER(Array3D), C.POINTER(Array3D), C.POINTER(C.c_double), C.c_void_p]),
    "fs3d_infinite_norm": (C.c_int, [C.POINTER(Array3D), C.POINTER(C.c_double), C.c_void_p]),
    "fs3d_tricubic": (C.c_int, [C.POINTER(Array3D), C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "fs3d_mac_vel": (C.c_int, [C.POINTER(MACGrid3D), C.c_void_p, C.c_void_p]),
    "fs3d_mac_face_vel": (C.c_int, [C.POINTER(MACGrid3D), C.c_int, C.c_void_p, C.c_void_p]),
    "fs3d_mac_vel_interp": (C.c_int, [C.POINTER(MACGrid3D), C.c_int, C.c_void_p, C.c_size_t, C.c_void_p,
                                      C.c_void_p]),
    "fs3d_mac_vel_div": (C.c_int, [C.POINTER(MACGrid3D), C.c_void_p, C.c_void_p]),
}

_lib = None


class FS2DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fs2d error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Load libfs2d.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library {path} is missing: run fluid-sim_gb300/build.py "
                               "(there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(rc, allow=()):
    if rc != 0 and rc not in allow:
        raise FS2DError(rc, load().fs2d_last_error().decode())
    return rc


def default_options(**kw):
    o = Options()
    load().fs2d_default_options(C.byref(o))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = PRECISION[v]
        if k == "p2g_mode" and isinstance(v, str):
            v = P2G[v]
        setattr(o, k, v)
    return o


def make_config(scene):
    cells = np.ascontiguousarray(scene["cells"], dtype=np.uint8)
    cfg = Config(scene["sizeX"], scene["sizeY"], scene["ppcSqrt"], scene["dt"], scene["dx"], scene["rho"],
                 scene["gravityX"], scene["gravityY"], scene["mode"], scene["picFlipAlpha"],
                 cells.ctypes.data_as(C.POINTER(C.c_uint8)))
    cfg._keep = cells
    return cfg


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def state_view(arrs):
    st = State()
    for name in ("phi", "p", "u", "v", "newU", "newV", "particles", "particleVels"):
        a = arrs.get(name)
        setattr(st, name, _dptr(a))
    c = arrs.get("cell")
    st.cell = c.ctypes.data_as(C.POINTER(C.c_uint8)) if c is not None else None
    parts = arrs.get("particles")
    st.numParticles = 0 if parts is None else len(parts) // 2
    return st


class Render(C.Structure):
    _fields_ = [("waterCells", C.c_void_p), ("waterCap", C.c_size_t), ("waterCount", C.POINTER(C.c_size_t)),
                ("solidCells", C.c_void_p), ("solidCap", C.c_size_t), ("solidCount", C.POINTER(C.c_size_t)),
                ("pressureCells", C.c_void_p), ("pressureValues", C.c_void_p), ("pressureCap", C.c_size_t),
                ("pressureCount", C.POINTER(C.c_size_t)), ("cellVels", C.c_void_p), ("particleLines", C.c_void_p),
                ("phiValues", C.c_void_p)]


class FluidSim2D:
    """One simulation on the GPU.  ``scene`` is a dict as made by scenes.py
    (the fields of FluidSim2DConfig plus the label array)."""

    def __init__(self, scene, seed=None, **options):
        lib = load()
        self.nx, self.ny = scene["sizeX"], scene["sizeY"]
        self.mode = scene["mode"]
        self.cfg = make_config(scene)
        if seed is not None:
            options.setdefault("use_seed", 1)
            options.setdefault("seed", seed)
        self.opt = default_options(**options)
        h = C.c_void_p()
        _check(lib.fs2d_create(C.byref(self.cfg), C.byref(self.opt), C.byref(h)))
        self.h = h

    create = classmethod(lambda cls, scene, **kw: cls(scene, **kw))

    # ---- frame and stages (FluidSim2D::runFrame / update / stage methods) ----
    def runFrame(self):
        return _check(load().fs2d_run_frame(self.h), allow=(4,))

    update = runFrame

    def step(self, n):
        return _check(load().fs2d_step(self.h, n), allow=(4,))

    def stage(self, name):
        return _check(load().fs2d_run_stage(self.h, STAGES[name] if isinstance(name, str) else name), allow=(4,))

    def __getattr__(self, name):
        if name in STAGES:
            return lambda: self.stage(name)
        raise AttributeError(name)

    # ---- state ----
    def num_particles(self):
        n = C.c_size_t()
        _check(load().fs2d_num_particles(self.h, C.byref(n)))
        return n.value

    def get_state(self, fields=None, out=None):
        """Download the state; `out` may supply the destination arrays
        (e.g. pinned host memory), which are filled in place."""
        n = self.num_particles()
        nx, ny = self.nx, self.ny
        shapes = {"cell": (nx * ny, np.uint8), "phi": (nx * ny, np.float64), "p": (nx * ny, np.float64),
                  "u": ((nx + 1) * ny, np.float64), "v": (nx * (ny + 1), np.float64),
                  "newU": ((nx + 1) * ny, np.float64), "newV": (nx * (ny + 1), np.float64),
                  "particles": (2 * n, np.float64), "particleVels": (2 * n, np.float64)}
        names = fields or (list(out) if out is not None else list(shapes))
        arrs = out if out is not None else {k: np.zeros(shapes[k][0], shapes[k][1]) for k in names}
        for k in names:
            if arrs[k].shape != (shapes[k][0],) or arrs[k].dtype != shapes[k][1]:
                raise ValueError(f"get_state: buffer {k} has the wrong shape or dtype")
        st = state_view(arrs)
        st.numParticles = n
        _check(load().fs2d_download_state(self.h, C.byref(st)))
        return arrs

    def set_state(self, arrs):
        arrs = {k: np.ascontiguousarray(v) for k, v in arrs.items() if v is not None}
        st = state_view(arrs)
        _check(load().fs2d_upload_state(self.h, C.byref(st)))

    def solve_pressure(self, cell, phi, u, v):
        """The projection's pressure solve on the given labels, level set and
        face velocities; returns (pressure, stats)."""
        NX, NY = self.nx, self.ny
        cell = np.ascontiguousarray(cell, dtype=np.uint8).reshape(-1)
        phi, u, v = (np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (phi, u, v))
        assert cell.size == NX * NY and phi.size == NX * NY and u.size == (NX + 1) * NY and v.size == NX * (NY + 1)
        out = np.empty(NX * NY)
        st = Stats()
        rc = load().fs2d_solve_pressure(self.h, cell.ctypes.data, phi.ctypes.data, u.ctypes.data, v.ctypes.data,
                                        out.ctypes.data, C.byref(st))
        _check(rc, allow=(4,))
        return out, {k: getattr(st, k) for k, _ in Stats._fields_}

    def forward(self, steps, u0, v0, u_target, v_target, checkpoint_every=0):
        """Differentiable rollout of `steps` semi-Lagrangian velocity steps
        from (u0, v0) on the scene's fixed labels; returns the loss
        ||(u_T, v_T) - (u_target, v_target)||_2.  Arrays are host numpy
        arrays or device addresses (ints)."""
        NX, NY = self.nx, self.ny
        keep = []

        def ptr(a, n):
            if isinstance(a, int):
                return a
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
            assert a.size == n
            keep.append(a)
            return a.ctypes.data

        NU, NV = (NX + 1) * NY, NX * (NY + 1)
        loss = C.c_double(0.0)
        _check(load().fs2d_forward(self.h, int(steps), int(checkpoint_every), ptr(u0, NU), ptr(v0, NV),
                                   ptr(u_target, NU), ptr(v_target, NV), C.byref(loss)))
        return loss.value

    def backward(self, grad_u=None, grad_v=None):
        """dL/du0, dL/dv0 of the last forward(); into the given device
        addresses, else returned as numpy arrays."""
        NX, NY = self.nx, self.ny
        if grad_u is not None:
            _check(load().fs2d_backward(self.h, grad_u, grad_v))
            return None
        gu, gv = np.empty((NX + 1) * NY), np.empty(NX * (NY + 1))
        _check(load().fs2d_backward(self.h, gu.ctypes.data, gv.ctypes.data))
        return gu, gv

    def p2g_adjoint(self, u_bar, v_bar):
        """Transpose of transferVelocityToGrid at the current particle
        positions (after that stage ran): face adjoints -> particle velocity
        adjoints (2 per particle)."""
        NX, NY = self.nx, self.ny
        ub = np.ascontiguousarray(u_bar, dtype=np.float64).reshape(-1)
        vb = np.ascontiguousarray(v_bar, dtype=np.float64).reshape(-1)
        assert ub.size == (NX + 1) * NY and vb.size == NX * (NY + 1)
        out = np.zeros(2 * self.num_particles())
        _check(load().fs2d_p2g_adjoint(self.h, ub.ctypes.data, vb.ctypes.data, out.ctypes.data))
        return out

    def g2p_adjoint(self, vel_bar):
        """Transpose of updateParticleVelocities: adjoint of the new particle
        velocities -> adjoints of (newU, newV, u, v, old velocities)."""
        NX, NY = self.nx, self.ny
        gb = np.ascontiguousarray(vel_bar, dtype=np.float64).reshape(-1)
        assert gb.size == 2 * self.num_particles()
        nub, ub = np.zeros((NX + 1) * NY), np.zeros((NX + 1) * NY)
        nvb, vb = np.zeros(NX * (NY + 1)), np.zeros(NX * (NY + 1))
        ib = np.zeros_like(gb)
        _check(load().fs2d_g2p_adjoint(self.h, gb.ctypes.data, nub.ctypes.data, nvb.ctypes.data, ub.ctypes.data,
                                       vb.ctypes.data, ib.ctypes.data))
        return nub, nvb, ub, vb, ib

    def render_export(self, buffers, caps):
        """fs2d_render_export into device buffers: `buffers` maps field names
        of fs2d_render to device pointers (ints), `caps` the list capacities;
        returns the list counts (water, solid, pressure)."""
        r = Render()
        counts = [C.c_size_t(0) for _ in range(3)]
        for k, v in buffers.items():
            setattr(r, k, v)
        r.waterCap, r.solidCap, r.pressureCap = caps.get("water", 0), caps.get("solid", 0), caps.get("pressure", 0)
        r.waterCount, r.solidCount, r.pressureCount = (C.pointer(c) for c in counts)
        _check(load().fs2d_render_export(self.h, C.byref(r)))
        return tuple(c.value for c in counts)

    def reseed(self, minPerCell, maxPerCell, seed=0):
        """Particle reseeding (fs2d_reseed; the reference lists it as a TODO)."""
        st = ReseedStats()
        _check(load().fs2d_reseed(self.h, minPerCell, maxPerCell, seed, C.byref(st)))
        return {"removed": st.removed, "added": st.added, "numParticles": st.numParticles}

    def cfl(self):
        """applyAdvection's CFL check (fs2d_cfl): (largest c, first particle)."""
        c, e = C.c_double(), C.c_longlong()
        _check(load().fs2d_cfl(self.h, C.byref(c), C.byref(e)))
        return c.value, e.value

    def save_checkpoint(self, path):
        _check(load().fs2d_save_checkpoint(self.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        _check(load().fs2d_load_checkpoint(self.h, os.fsencode(path)))

    def set_volume_correction(self, rate):
        """Volume correction in the projection (fs2d_set_volume_correction)."""
        _check(load().fs2d_set_volume_correction(self.h, rate))

    def set_params(self, gravityX, gravityY, picFlipAlpha, dt):
        _check(load().fs2d_set_params(self.h, gravityX, gravityY, picFlipAlpha, dt))

    # ---- statistics and diagnostics ----
    def stats(self):
        s = Stats()
        _check(load().fs2d_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def history(self):
        n = C.c_size_t()
        _check(load().fs2d_get_history(self.h, None, None, None, 0, C.byref(n)))
        a, b, c = (np.zeros(n.value) for _ in range(3))
        _check(load().fs2d_get_history(self.h, _dptr(a), _dptr(b), _dptr(c), n.value, C.byref(n)))
        return a, b, c

    def _diag(self, fn):
        out = C.c_double()
        _check(fn(self.h, C.byref(out)))
        return out.value

    def avgPressure(self):
        return self._diag(load().fs2d_avg_pressure)

    def avgPressureInFluid(self):
        return self._diag(load().fs2d_avg_pressure_in_fluid)

    def maxVelocity(self):
        return self._diag(load().fs2d_max_velocity)

    def saveStats(self, perf="perf.csv", conservation="conservation.csv"):
        _check(load().fs2d_save_stats(self.h, perf.encode() if perf else None,
                                      conservation.encode() if conservation else None))

    def stage_times(self):
        buf = (C.c_float * 16)()
        n = C.c_int()
        _check(load().fs2d_get_stage_times(self.h, buf, 16, C.byref(n)))
        return list(buf[:n.value])

    def launch_count(self):
        n = C.c_ulonglong()
        _check(load().fs2d_launch_count(self.h, C.byref(n)))
        return n.value

    def set_kernel_timing(self, patterns):
        """Time (CUDA events) every launch whose kernel name contains one of
        the comma-separated patterns; "" turns timing off."""
        _check(load().fs2d_set_kernel_timing(self.h, patterns.encode() if patterns else None))

    def kernel_times(self):
        """{kernel name: (launches, total ms)} since the previous call."""
        buf = C.create_string_buffer(1 << 16)
        _check(load().fs2d_get_kernel_times(self.h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    def set_stream(self, stream_ptr):
        _check(load().fs2d_set_stream(self.h, C.c_void_p(stream_ptr)))

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                load().fs2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @classmethod
    def _view(cls, handle, scene):
        """A non-owning wrapper of a handle that a batch owns."""
        self = cls.__new__(cls)
        self.nx, self.ny, self.mode = scene["sizeX"], scene["sizeY"], scene["mode"]
        self.h = handle
        self._owned = False
        return self


class Batch:
    """fs2d_batch: independent scenes advanced together by `workers` host
    threads (0: chosen on the first frames).  With use_seed, scene k is
    seeded with seed + k."""

    def __init__(self, scenes, workers=0, seed=None, **options):
        lib = load()
        self.scenes = list(scenes)
        n = len(self.scenes)
        self.cfgs = (Config * n)()
        self._keep = []
        for k, sc in enumerate(self.scenes):
            cfg = make_config(sc)
            self._keep.append(cfg._keep)
            self.cfgs[k] = cfg
        if seed is not None:
            options.setdefault("use_seed", 1)
            options.setdefault("seed", seed)
        self.opt = default_options(**options)
        h = C.c_void_p()
        _check(lib.fs2d_batch_create(C.cast(self.cfgs, C.c_void_p), n, C.byref(self.opt), int(workers), C.byref(h)))
        self.h = h

    def step(self, nframes=1):
        return _check(load().fs2d_batch_step(self.h, int(nframes)), allow=(4,))

    def __len__(self):
        n = C.c_int()
        _check(load().fs2d_batch_size(self.h, C.byref(n)))
        return n.value

    def scene(self, k):
        """Scene k as a FluidSim2D view (state, statistics); owned by the batch."""
        h = C.c_void_p()
        _check(load().fs2d_batch_scene(self.h, int(k), C.byref(h)))
        return FluidSim2D._view(h, self.scenes[k])

    def sweep_schedule(self):
        """The tuned persistent sweep of a mixed-precision batch: schedule,
        CTAs, work items and the sweep's time in microseconds."""
        sc, ct, it, us = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _check(load().fs2d_batch_sweep_schedule(self.h, C.byref(sc), C.byref(ct), C.byref(it), C.byref(us)))
        return {"schedule": sc.value, "ctas": ct.value, "items": it.value, "sweep_us": us.value}

    def set_schedule(self, schedule, ctas=0):
        """Override the autotuned sweep schedule (0..4) and CTA count."""
        _check(load().fs2d_batch_set_schedule(self.h, int(schedule), int(ctas)))

    def set_graphs(self, on):
        """Replay each scene's per-frame phases from CUDA graphs (default) or
        launch them directly."""
        _check(load().fs2d_batch_set_graphs(self.h, 1 if on else 0))

    def phase_ms(self):
        """ms of the last step() of a mixed-precision batch: wall clock of the
        scenes' stages before the solve, the joint solve, the stages after it,
        and the device time of the batched level-set sweeps (within the first)."""
        ms = (C.c_double * 4)()
        _check(load().fs2d_batch_phase_ms(self.h, ms))
        return list(ms)

    def launch_count(self):
        """Kernels launched so far by the batch and its scenes."""
        n = C.c_ulonglong()
        _check(load().fs2d_batch_launch_count(self.h, C.byref(n)))
        return n.value

    @property
    def workers(self):
        w = C.c_int()
        _check(load().fs2d_batch_workers(self.h, C.byref(w)))
        return w.value

    @workers.setter
    def workers(self, w):
        _check(load().fs2d_batch_set_workers(self.h, int(w)))

    def _ptrs(self, arrays, sizes, keep):
        out = (C.c_void_p * len(self.scenes))()
        for k, a in enumerate(arrays):
            if isinstance(a, int):
                out[k] = a
            else:
                a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                assert a.size == sizes[k]
                keep.append(a)
                out[k] = a.ctypes.data
        return out

    def forward(self, steps, u0s, v0s, u_targets, v_targets, checkpoint_every=0):
        """fs2d_batch_forward: every scene's rollout; returns the losses."""
        nu = [(sc["sizeX"] + 1) * sc["sizeY"] for sc in self.scenes]
        nv = [sc["sizeX"] * (sc["sizeY"] + 1) for sc in self.scenes]
        keep = []
        args = [self._ptrs(a, n, keep) for a, n in ((u0s, nu), (v0s, nv), (u_targets, nu), (v_targets, nv))]
        losses = np.zeros(len(self.scenes))
        _check(load().fs2d_batch_forward(self.h, int(steps), int(checkpoint_every), *(C.cast(a, C.c_void_p) for a in args),
                                         losses.ctypes.data))
        return losses

    def backward(self):
        """fs2d_batch_backward into host arrays: [(dL/du0, dL/dv0) per scene]."""
        gus = [np.empty((sc["sizeX"] + 1) * sc["sizeY"]) for sc in self.scenes]
        gvs = [np.empty(sc["sizeX"] * (sc["sizeY"] + 1)) for sc in self.scenes]
        pu = (C.c_void_p * len(gus))(*[g.ctypes.data for g in gus])
        pv = (C.c_void_p * len(gvs))(*[g.ctypes.data for g in gvs])
        _check(load().fs2d_batch_backward(self.h, C.cast(pu, C.c_void_p), C.cast(pv, C.c_void_p)))
        return list(zip(gus, gvs))

    def close(self):
        if getattr(self, "h", None):
            load().fs2d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
