"""Seeded inputs of the 3D container tests (include/fs3d.h), shared by the
golden-vector generator (tests/golden/make_golden_grid3d.py), the CPU tests
of the oracle and the GPU tests.

Arrays are flat float64 in the reference's layout (element (i, j, k) at
k*ny*nx + j*nx + i); points are (n, 3) rows of grid coordinates.
"""
from __future__ import annotations

import numpy as np

# (nx, ny, nz) of the Array3D cases: non-cubic, a single element, a cube, a
# long thin one with an odd element count
ARRAY_DIMS = [(5, 4, 3), (1, 1, 1), (7, 7, 7), (16, 9, 5)]
# cubes for triCubic, where the reference's (z, y, x) read stays in bounds
CUBES = [4, 7]
# (sizeX, sizeY, sizeZ) of the MACGrid3D cases
MAC_SIZES = [(4, 3, 2), (1, 1, 1), (6, 5, 7)]
INTERP_CUBE = 6
SCALE = 0.37


def array(dims, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(dims[0] * dims[1] * dims[2])


def zero_aliased_rows(a, dims):
    """`a` with row 0 of every slab k >= 1 set to zero: the reference's loops
    visit those rows twice (as row NY of slab k-1), which then adds zero."""
    nx, ny, nz = dims
    out = a.copy().reshape(nz, ny, nx)
    out[1:, 0, :] = 0.0
    return out.ravel()


def points(n_side, count, seed, lo=-1.5, hi=None):
    """Random points over and around an n_side cube plus fixed special
    points: integer nodes, a negative fraction (truncated to 0 like the
    reference's (int) cast), the upper edge, outside on each side."""
    rng = np.random.default_rng(seed)
    hi = n_side + 0.5 if hi is None else hi
    pts = rng.uniform(lo, hi, size=(count, 3))
    m = float(n_side)
    special = np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 1.0], [-0.5, 0.25, 0.75], [-0.999, -0.5, -0.25],
                        [m - 1e-9, m - 1e-9, m - 1e-9], [m, 0.5, 0.5], [0.5, m, 0.5], [0.5, 0.5, m],
                        [-1.0, 0.5, 0.5], [0.5, -1.0, 0.5], [0.5, 0.5, -1.0], [1e300, 0.5, 0.5],
                        [0.5, -1e300, 0.5], [m / 2 + 0.5, m / 3, m / 4]])
    return np.concatenate([special, pts])


def mac_fields(size, seed):
    sx, sy, sz = size
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((sx + 1) * sy * sz)
    v = rng.standard_normal(sx * (sy + 1) * sz)
    w = rng.standard_normal(sx * sy * (sz + 1))
    return u, v, w


def cube_fields(n, seed):
    rng = np.random.default_rng(seed)
    return tuple(rng.standard_normal(n ** 3) for _ in range(3))
