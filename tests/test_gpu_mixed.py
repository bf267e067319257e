"""Mixed-precision projection (FP32 MIC(0)-PCG inside FP64 iterative
refinement) against the reference.

The stop test is the reference's, ||r||inf <= tol * ||b||inf, evaluated on
the FP64 residual b - A p, so at the reference's tol = 1e-12 the mixed
pressure agrees with the reference's FP64 solve to PRESSURE_RTOL, the same
tolerance the FP64 path is held to."""
import numpy as np
import pytest

import golden_util as G
import oracle_py as O

fs2d = pytest.importorskip("fs2d")
pytestmark = pytest.mark.gpu

PRESSURE_RTOL = 1e-8


@pytest.mark.parametrize("name", G.NAMES)
def test_mixed_projection_matches_reference(name):
    g = G.load(name)
    sc = G.scene(g)
    k = G.stage_order(sc).index("applyProjection")
    sim = fs2d.FluidSim2D(sc, seed=7, precision="mixed")
    sim.set_state(G.pre_stage(g, k))
    sim.stage("applyProjection")
    p = sim.get_state(["p"])["p"]
    ref = g[f"s{k}_post_p"]
    scale = np.abs(ref).max()
    assert np.abs(p - ref).max() <= PRESSURE_RTOL * scale
    st = sim.stats()
    assert st["pcgRelResidual"] <= 1e-12
    assert st["irOuterIterations"] >= 1


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_mixed_meets_tolerance_on_fp64_residual(tol):
    import scenes
    sc = scenes.pic_dam_break_disk(96)
    sim = fs2d.FluidSim2D(sc, seed=3, precision="mixed", pcg_tol=tol)
    ref = fs2d.FluidSim2D(sc, seed=3, precision="fp64", pcg_tol=1e-13, pcg_max_iters=2000)
    for _ in range(3):
        sim.runFrame()
        ref.runFrame()
    st = sim.stats()
    assert st["pcgRelResidual"] <= tol
    # same pre-projection state for both: compare one projection stage
    pre = ref.get_state()
    sim.set_state(pre)
    ref.set_state(pre)
    for s in ("createWaterLevelSet", "transferVelocityToGrid", "applyGravity"):
        sim.stage(s)
        ref.stage(s)
    sim.stage("applyProjection")
    ref.stage("applyProjection")
    p, pr = sim.get_state(["p"])["p"], ref.get_state(["p"])["p"]
    # ||p - p*|| is bounded by cond(A) * tol; check a loose multiple
    assert np.abs(p - pr).max() <= 1e4 * tol * np.abs(pr).max()


@pytest.mark.parametrize("name", ["pic_disk_32", "sl_dam_32"])
def test_mixed_frames_against_oracle(name):
    g = G.load(name)
    sc = G.scene(g)
    sim = fs2d.FluidSim2D(sc, seed=7, precision="mixed")
    orc = O.OracleSim(sc, seed=7, sl_inplace=0)
    for frame in range(10):
        sim.runFrame()
        orc.frame()
        a, b = sim.get_state(), orc.get_state()
        assert np.array_equal(a["cell"], b["cell"]), frame
        for f in ("p", "u", "v", "particles", "particleVels"):
            scale = np.abs(b[f]).max() + 1e-30
            assert np.abs(a[f] - b[f]).max() <= 1e-6 * scale, (frame, f)


def test_graph_replay_matches_direct_launches():
    """The inner PCG loop replayed from a captured CUDA graph gives the same
    bits as the same loop launched kernel by kernel (per-kernel timing turns
    the graph off)."""
    import scenes
    sc = scenes.pic_dam_break_disk(96)
    a = fs2d.FluidSim2D(sc, seed=5, precision="mixed", pcg_tol=1e-6)
    b = fs2d.FluidSim2D(sc, seed=5, precision="mixed", pcg_tol=1e-6)
    b.set_kernel_timing("mic32")
    for _ in range(3):
        a.runFrame()
        b.runFrame()
    sa, sb = a.get_state(), b.get_state()
    for f in ("cell", "p", "u", "v", "particles", "particleVels"):
        assert np.array_equal(sa[f], sb[f]), f
    assert a.stats()["pcgIterations"] == b.stats()["pcgIterations"]
    a.close()
    b.close()


def test_plain_fp32_pcg():
    """Config 1's first GPU form: plain FP32 MIC(0)-PCG (FP32 dot products, one
    solve to the tolerance on the FP32 residual, no FP64 refinement).  Its
    FP64 residual is reported (NOT_CONVERGED when FP32 rounding keeps it above
    the tolerance) and its pressure stays within FP32_RTOL of the FP64
    solution solved to 1e-12, the mixed path within MIXED_RTOL."""
    import scenes
    FP32_RTOL, MIXED_RTOL = 1e-4, 1e-5
    sc, cell, phi, u, v = scenes.pressure_disks(256, 256, seed=9)
    ref = fs2d.FluidSim2D(sc, seed=1, precision="fp64", pcg_tol=1e-12, pcg_max_iters=2000)
    p64, _ = ref.solve_pressure(cell, phi, u, v)
    ref.close()
    for prec, rtol in (("fp32", FP32_RTOL), ("mixed", MIXED_RTOL)):
        sim = fs2d.FluidSim2D(sc, seed=1, precision=prec, pcg_tol=1e-6, pcg_max_iters=400)
        p, st = sim.solve_pressure(cell, phi, u, v)
        sim.close()
        assert np.abs(p - p64).max() <= rtol * np.abs(p64).max(), (prec, st)
        if prec == "fp32":
            assert st["irOuterIterations"] == 1 and st["pcgRelResidual"] < 1e-4
            assert st["lastStatus"] in (0, 4) and (st["lastStatus"] == 4) == (st["pcgRelResidual"] > 1e-6)
        else:
            assert st["lastStatus"] == 0 and st["pcgRelResidual"] <= 1e-6
