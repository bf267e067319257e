"""Standalone pressure solve (fs2d_solve_pressure): seeded labels of random
disks over a fluid background (about 70 % fluid, 25 % air, 5 % solid, solid
border) and the divergence of a seeded N(0, 1) velocity field, solved to a
1e-10 relative residual by the FP64 path and by FP32 MIC(0)-PCG inside FP64
iterative refinement (inner tolerance 1e-4).

* small grids: both against the oracle's projection stage, which builds the
  same matrix and right-hand side (the oracle solved to 1e-13 stands in for
  the exact solution);
* 2048 x 2048: the two GPU paths against each other.

Both paths must stop on the reference's FP64 test ||b - A p||inf <= tol ||b||inf.
"""
import numpy as np
import pytest

import oracle_py as O

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

TOL = 1e-10
FP64_VS_ORACLE = 1e-8       # same algorithm, tree-ordered reductions: relative max-norm difference
MIXED_VS_ORACLE = 1e-6      # different Krylov path to the same 1e-10 residual
MIXED_VS_FP64_2048 = 1e-5


def disk_scene(nx, ny, seed):
    return scenes.pressure_disks(nx, ny, seed)


def oracle_pressure(sc, cell, phi, u, v, tol):
    orc = O.OracleSim(sc, seed=7, sl_inplace=0, pcg_tol=tol, pcg_max_iters=5000)
    orc.set_state({"cell": cell, "phi": phi, "u": u, "v": v})
    orc.stage("applyProjection")
    p = orc.get_state()["p"].copy()
    orc.close()
    return p


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("shape", [(96, 80), (130, 64)])
def test_pressure_solve_against_oracle(shape):
    nx, ny = shape
    sc, cell, phi, u, v = disk_scene(nx, ny, seed=nx * 1000 + ny)
    ref_same_tol = oracle_pressure(sc, cell, phi, u, v, TOL)
    ref_exact = oracle_pressure(sc, cell, phi, u, v, 1e-13)
    out = {}
    for prec in ("fp64", "mixed"):
        sim = fs2d.FluidSim2D(sc, seed=1, precision=prec, pcg_tol=TOL, pcg_max_iters=5000, ir_inner_tol=1e-4)
        p, st = sim.solve_pressure(cell, phi, u, v)
        sim.close()
        assert st["lastStatus"] == 0
        assert st["pcgRelResidual"] <= TOL, (prec, st)
        out[prec] = (p, st)
    assert rel(out["fp64"][0], ref_same_tol) <= FP64_VS_ORACLE
    assert rel(out["mixed"][0], ref_exact) <= MIXED_VS_ORACLE
    assert out["mixed"][1]["irOuterIterations"] >= 2


def test_pressure_solve_2048_mixed_vs_fp64():
    sc, cell, phi, u, v = disk_scene(2048, 2048, seed=2048)
    res = {}
    for prec in ("fp64", "mixed"):
        sim = fs2d.FluidSim2D(sc, seed=1, precision=prec, pcg_tol=TOL, pcg_max_iters=5000, ir_inner_tol=1e-4)
        p, st = sim.solve_pressure(cell, phi, u, v)
        sim.close()
        assert st["pcgRelResidual"] <= TOL, (prec, st)
        res[prec] = p
    assert rel(res["mixed"], res["fp64"]) <= MIXED_VS_FP64_2048
