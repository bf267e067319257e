"""Failure paths that the reference only logs, made on the host (no GPU
fault): a pressure solve capped below convergence returns
FS2D_ERR_NOT_CONVERGED while the frame still completes (the reference logs
"PCG did not converge" and continues, src/FluidSim2D.cpp:464-466), the status
is reported by the statistics, and the next frames run normally."""
import numpy as np
import pytest

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

NOT_CONVERGED = 4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_cap_reports_not_converged_and_continues(precision):
    sc = scenes.pic_dam_break_disk(64)
    sim = fs2d.FluidSim2D(sc, seed=2, precision=precision, pcg_tol=1e-12, pcg_max_iters=3, ir_max_outer=2)
    rc = sim.runFrame()
    assert rc == NOT_CONVERGED
    st = sim.stats()
    assert st["lastStatus"] == NOT_CONVERGED and st["frames"] == 1
    assert st["pcgRelResidual"] > 1e-12
    for _ in range(2):
        assert sim.runFrame() == NOT_CONVERGED
    state = sim.get_state(["u", "v", "particles"])
    for k, a in state.items():
        assert np.isfinite(a).all(), k
    sim.close()


def test_standalone_solve_reports_not_converged():
    sc, cell, phi, u, v = scenes.pressure_disks(96, 96, seed=9)
    sim = fs2d.FluidSim2D(sc, seed=1, precision="fp64", pcg_tol=1e-12, pcg_max_iters=2)
    p, st = sim.solve_pressure(cell, phi, u, v)
    assert st["lastStatus"] == NOT_CONVERGED or st["pcgIterations"] == 2
    assert st["pcgRelResidual"] > 1e-12 and np.isfinite(p).all()
    sim.close()
