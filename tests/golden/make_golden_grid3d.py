"""Generate tests/golden/grid3d.npz from the REFERENCE's own 3D containers.

Calls the unmodified include/Array3D.h and include/MACGrid3D.h (compiled by
oracle/build_oracle.py behind oracle/ref3d_capi.cpp into
oracle/_ref/libfs3d_ref.so: serial, -ffp-contract=off) on the seeded inputs
of tests/grid3d_cases.py and stores inputs and outputs:

* ``arr{d}_*``    Array3D cases of extents ARRAY_DIMS[d]: inputs a, b, the
                  b with its aliased rows zeroed (``bz``), and the results
                  of operator+= (``add``, on a and bz), setMultiplyAdd
                  (``sma``, scale SCALE), innerProduct (``dot``, a with bz)
                  and infiniteNorm (``norm``);
* ``cube{n}_*``   triCubic on an n^3 cube: data, points, results;
* ``mac{m}_*``    MACGrid3D cases of sizes MAC_SIZES[m]: u, v, w and the
                  results of vel, velU, velV, velW, velDiv at every cell or
                  face;
* ``interp_*``    velInterpU/V/W and velInterp on a grid of three cubes.

Usage (needs the reference checkout, named by FS2D_REFERENCE_DIR):
    FS2D_REFERENCE_DIR=<checkout> python tests/golden/make_golden_grid3d.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import build_oracle  # noqa: E402
import grid3d_cases as K  # noqa: E402
import oracle3d  # noqa: E402


def main():
    if not build_oracle.build_reference():
        sys.exit("the reference checkout is not available (set FS2D_REFERENCE_DIR)")
    ref = oracle3d.reference()
    out = {}
    for d, dims in enumerate(K.ARRAY_DIMS):
        a, b = K.array(dims, 10 + d), K.array(dims, 20 + d)
        bz = K.zero_aliased_rows(b, dims)
        out[f"arr{d}_a"], out[f"arr{d}_b"], out[f"arr{d}_bz"] = a, b, bz
        out[f"arr{d}_add"] = ref.add(a, bz, dims)
        out[f"arr{d}_sma"] = ref.set_multiply_add(a, K.SCALE, b, dims)
        out[f"arr{d}_dot"] = np.float64(ref.inner_product(a, bz, dims))
        out[f"arr{d}_norm"] = np.float64(ref.infinite_norm(a, dims))
    for n in K.CUBES:
        data = K.array((n, n, n), 30 + n)
        pts = K.points(n, 200, 40 + n)
        out[f"cube{n}_data"], out[f"cube{n}_pts"] = data, pts
        out[f"cube{n}_tricubic"] = ref.tricubic(data, (n, n, n), pts)
    for m, size in enumerate(K.MAC_SIZES):
        u, v, w = K.mac_fields(size, 50 + m)
        out[f"mac{m}_u"], out[f"mac{m}_v"], out[f"mac{m}_w"] = u, v, w
        out[f"mac{m}_vel"] = ref.mac_vel(u, v, w, size)
        for axis in ("u", "v", "w"):
            out[f"mac{m}_vel{axis}"] = ref.mac_face_vel(u, v, w, size, axis)
        out[f"mac{m}_div"] = ref.mac_vel_div(u, v, w, size)
    n = K.INTERP_CUBE
    u, v, w = K.cube_fields(n, 60)
    pts = K.points(n, 200, 61)
    out["interp_u"], out["interp_v"], out["interp_w"], out["interp_pts"] = u, v, w, pts
    for comp in ("u", "v", "w", "uvw"):
        out[f"interp_{comp}_out"] = ref.mac_vel_interp_cubes(u, v, w, n, comp, pts)
    path = os.path.join(HERE, "grid3d.npz")
    np.savez_compressed(path, **out)
    print(path, len(out), "arrays")


if __name__ == "__main__":
    main()
