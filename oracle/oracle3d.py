"""ctypes bindings of the oracle for the 3D grid containers (test infrastructure only).

Imported by tests/ as the checker of the device kernels behind
include/fs3d.h; nothing in the product imports this module.

Two implementations with the same Python surface, on numpy arrays in the
reference's layout (element (i, j, k) of an (nx, ny, nz) array at
k*ny*nx + j*nx + i; face arrays of an (sx, sy, sz) MAC grid of extents
(sx+1, sy, sz), (sx, sy+1, sz), (sx, sy, sz+1); points and vectors as
(n, 3) rows of (x, y, z)):

* :data:`restated` — the C restatement ``oracle/restate/fs3d_oracle.c``,
  built on every machine;
* :func:`reference` — the reference's own ``include/Array3D.h`` and
  ``include/MACGrid3D.h`` compiled behind ``oracle/ref3d_capi.cpp``
  (``oracle/_ref/libfs3d_ref.so``), only where the reference checkout
  exists.  Its bulk loops touch NX elements past an array and its
  triCubic reads element (z, y, x); the wrappers here pad every buffer with
  zeros so that those reads stay in memory the caller owns, and
  ``tricubic`` / ``mac_vel_interp_cubes`` are only meaningful on cubes.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import oracle_py

HERE = os.path.dirname(os.path.abspath(__file__))
D = C.POINTER(C.c_double)
AXES = {"u": 0, "v": 1, "w": 2, "uvw": 3}


def _d(a):
    return a.ctypes.data_as(D)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64).ravel()


def face_dims(sx, sy, sz):
    return (sx + 1, sy, sz), (sx, sy + 1, sz), (sx, sy, sz + 1)


class _Restated:
    """The C restatement (oracle/restate/fs3d_oracle.c)."""

    def __init__(self):
        self._lib = None

    @property
    def lib(self):
        if self._lib is None:
            lib = oracle_py.get_oracle_lib()
            lib.or3_inner_product.restype = C.c_double
            lib.or3_infinite_norm.restype = C.c_double
            lib.or3_set_multiply_add.argtypes = [D, D, C.c_double, D, C.c_int, C.c_int, C.c_int]
            lib.or3_tricubic.argtypes = [D, C.c_int, C.c_int, C.c_int, D, C.c_size_t, D]
            lib.or3_mac_vel_interp.argtypes = [D, D, D, C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_size_t, D]
            self._lib = lib
        return self._lib

    def add(self, a, b, dims):
        out = _f64(a).copy()
        self.lib.or3_add(_d(out), _d(_f64(b)), *dims)
        return out

    def set_multiply_add(self, a, s, c, dims):
        a, c = _f64(a), _f64(c)
        out = np.empty_like(a)
        self.lib.or3_set_multiply_add(_d(out), _d(a), s, _d(c), *dims)
        return out

    def inner_product(self, a, b, dims):
        return self.lib.or3_inner_product(_d(_f64(a)), _d(_f64(b)), *dims)

    def infinite_norm(self, a, dims):
        return self.lib.or3_infinite_norm(_d(_f64(a)), *dims)

    def tricubic(self, a, dims, pts):
        pts = _f64(pts)
        out = np.empty(pts.size // 3)
        self.lib.or3_tricubic(_d(_f64(a)), *dims, _d(pts), out.size, _d(out))
        return out

    def mac_vel(self, u, v, w, size):
        out = np.empty(3 * size[0] * size[1] * size[2])
        self.lib.or3_mac_vel(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, _d(out))
        return out.reshape(-1, 3)

    def mac_vel_div(self, u, v, w, size):
        out = np.empty(size[0] * size[1] * size[2])
        self.lib.or3_mac_vel_div(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, _d(out))
        return out

    def mac_face_vel(self, u, v, w, size, axis):
        ax = AXES[axis]
        fd = face_dims(*size)[ax]
        out = np.empty(3 * fd[0] * fd[1] * fd[2])
        self.lib.or3_mac_face_vel(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, ax, _d(out))
        return out.reshape(-1, 3)

    def mac_vel_interp(self, u, v, w, size, component, pts):
        comp = AXES[component]
        pts = _f64(pts)
        n = pts.size // 3
        out = np.empty(3 * n if comp == 3 else n)
        self.lib.or3_mac_vel_interp(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, comp, _d(pts), n, _d(out))
        return out.reshape(-1, 3) if comp == 3 else out


restated = _Restated()


class _Reference:
    """The reference's own 3D containers (oracle/_ref/libfs3d_ref.so)."""

    def __init__(self, lib):
        lib.r3_inner_product.restype = C.c_double
        lib.r3_infinite_norm.restype = C.c_double
        lib.r3_set_multiply_add.argtypes = [D, D, C.c_double, D, C.c_int, C.c_int, C.c_int]
        lib.r3_tricubic.argtypes = [D, C.c_int, C.c_int, C.c_int, D, C.c_size_t, D]
        lib.r3_mac_vel_interp_cubes.argtypes = [D, D, D, C.c_int, C.c_int, D, C.c_size_t, D]
        self.lib = lib

    @staticmethod
    def _padded(a, dims):
        """A copy of `a` followed by nx zeros, room for the reference's loops
        that run one row past the array."""
        a = _f64(a)
        out = np.zeros(a.size + max(dims[0], 1))
        out[:a.size] = a
        return out

    def add(self, a, b, dims):
        pa, pb = self._padded(a, dims), self._padded(b, dims)
        self.lib.r3_add(_d(pa), _d(pb), *dims)
        return pa[:_f64(a).size]

    def set_multiply_add(self, a, s, c, dims):
        pa, pc = self._padded(a, dims), self._padded(c, dims)
        out = np.zeros_like(pa)
        self.lib.r3_set_multiply_add(_d(out), _d(pa), s, _d(pc), *dims)
        return out[:_f64(a).size]

    def inner_product(self, a, b, dims):
        return self.lib.r3_inner_product(_d(self._padded(a, dims)), _d(self._padded(b, dims)), *dims)

    def infinite_norm(self, a, dims):
        return self.lib.r3_infinite_norm(_d(self._padded(a, dims)), *dims)

    def tricubic(self, a, dims, pts):
        pts = _f64(pts)
        out = np.empty(pts.size // 3)
        self.lib.r3_tricubic(_d(_f64(a)), *dims, _d(pts), out.size, _d(out))
        return out

    def mac_vel(self, u, v, w, size):
        out = np.empty(3 * size[0] * size[1] * size[2])
        self.lib.r3_mac_vel(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, _d(out))
        return out.reshape(-1, 3)

    def mac_vel_div(self, u, v, w, size):
        out = np.empty(size[0] * size[1] * size[2])
        self.lib.r3_mac_vel_div(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, _d(out))
        return out

    def mac_face_vel(self, u, v, w, size, axis):
        ax = AXES[axis]
        fd = face_dims(*size)[ax]
        out = np.empty(3 * fd[0] * fd[1] * fd[2])
        self.lib.r3_mac_face_vel(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), *size, ax, _d(out))
        return out.reshape(-1, 3)

    def mac_vel_interp_cubes(self, u, v, w, n, component, pts):
        comp = AXES[component]
        pts = _f64(pts)
        npts = pts.size // 3
        out = np.empty(3 * npts if comp == 3 else npts)
        self.lib.r3_mac_vel_interp_cubes(_d(_f64(u)), _d(_f64(v)), _d(_f64(w)), n, comp, _d(pts), npts, _d(out))
        return out.reshape(-1, 3) if comp == 3 else out


_ref = []


def reference():
    """The compiled reference containers, or None where they were not built."""
    if not _ref:
        path = os.path.join(HERE, "_ref", "libfs3d_ref.so")
        _ref.append(_Reference(C.CDLL(path)) if os.path.exists(path) else None)
    return _ref[0]


def swap_xz(a, dims):
    """The array with its x and z axes exchanged: element (i, j, k) of the
    result is element (k, j, i) of `a` (a cube, dims (n, n, n))."""
    nx, ny, nz = dims
    return np.ascontiguousarray(_f64(a).reshape(nz, ny, nx).transpose(2, 1, 0)).ravel()
