"""Parity at the benchmark's own workload: the PIC/FLIP dam break + disk at
1024 x 1024 that bench.py times (dt 1/960, 4 particles per fluid cell,
FLIP 0.95, particles seeded with srand(12345)), against the oracle (the C
restatement, bit-exact to the reference's src/FluidSim2D.cpp:94-138).

The oracle runs two frames (PCG to 1e-6, as the bench); the third frame is
then checked two ways:

* FP64 device path, stage by stage: each stage gets the oracle's pre-stage
  state and its output is compared with the oracle's post-stage state.
  Labels and level set, P2G (ordered), gravity, velocity update with
  extrapolation, G2P and particle advection bit for bit; the pressure within
  PRESSURE_RTOL of max|p| with the reference's solver settings (1e-12,
  200 iterations: at this size both solves stop at the cap).
* one whole frame of each device path from the oracle's state at the
  bench's tolerance 1e-6, against the oracle's frame at the same tolerance:
  labels identical, pressure within FRAME_P_RTOL and face velocities within
  FRAME_U_RTOL of the largest value (two solves stopped at the same relative
  residual differ by about that much).
"""
import numpy as np
import pytest

import oracle_py as O

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

SIZE = 1024
SEED = 12345
PRESSURE_RTOL = 1e-8      # stage test, 200 iterations on both sides
FRAME_P_RTOL = 2e-4       # whole frame at 1e-6, |p - p_oracle|_inf / |p_oracle|_inf
FRAME_U_RTOL = 2e-4       # whole frame at 1e-6, velocities
EXACT = {
    "createWaterLevelSet": ("cell", "phi"),
    "transferVelocityToGrid": ("u", "v"),
    "applyGravity": ("u", "v"),
    "createSolidLevelSet": ("cell", "phi", "u", "v"),
    "updateVelocity": ("newU", "newV", "u", "v"),
    "updateParticleVelocities": ("particleVels", "u", "v"),
    "applyAdvection": ("particles",),
}
ORDER = ["createWaterLevelSet", "transferVelocityToGrid", "applyGravity", "createSolidLevelSet", "applyProjection",
         "updateVelocity", "updateParticleVelocities", "applyAdvection"]


def _same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def _rel(a, b):
    return float(np.abs(a - b).max() / (np.abs(b).max() + 1e-300))


@pytest.fixture(scope="module")
def start_state():
    """The oracle's state after two frames of the bench workload."""
    sc = scenes.pic_dam_break_disk(SIZE)
    orc = O.OracleSim(sc, seed=SEED, sl_inplace=0, pcg_tol=1e-6, pcg_max_iters=200)
    for _ in range(2):
        orc.frame()
    st = orc.get_state()
    orc.close()
    return sc, st


def test_stages_fp64_against_oracle(start_state):
    sc, st = start_state
    orc = O.OracleSim(sc, seed=SEED, sl_inplace=0, pcg_tol=1e-12, pcg_max_iters=200)
    orc.set_state(st)
    sim = fs2d.FluidSim2D(sc, seed=SEED, precision="fp64", pcg_tol=1e-12, pcg_max_iters=200)
    report = {}
    for stage in ORDER:
        pre = orc.get_state()
        orc.stage(stage)
        post = orc.get_state()
        sim.set_state(pre)
        sim.stage(stage)
        got = sim.get_state()
        if stage in EXACT:
            for f in EXACT[stage]:
                assert _same(got[f], post[f]), (stage, f, _rel(got[f], post[f]))
        elif stage == "applyProjection":
            report["p"] = _rel(got["p"], post["p"])
            assert report["p"] <= PRESSURE_RTOL, report
    print("1024^2 FP64 stages: pressure rel. error", report)
    sim.close()
    orc.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_whole_frame_against_oracle(start_state, precision):
    sc, st = start_state
    orc = O.OracleSim(sc, seed=SEED, sl_inplace=0, pcg_tol=1e-6, pcg_max_iters=200)
    orc.set_state(st)
    orc.frame()
    ref = orc.get_state()
    orc.close()
    sim = fs2d.FluidSim2D(sc, seed=SEED, precision=precision, pcg_tol=1e-6, pcg_max_iters=200)
    sim.set_state(st)
    assert sim.runFrame() == 0
    got = sim.get_state()
    assert _same(got["cell"], ref["cell"])
    errs = {f: _rel(got[f], ref[f]) for f in ("p", "u", "v", "particleVels")}
    print(f"1024^2 whole frame, {precision}: rel. errors vs the FP64 oracle", errs, sim.stats()["pcgIterations"])
    assert errs["p"] <= FRAME_P_RTOL, errs
    for f in ("u", "v", "particleVels"):
        assert errs[f] <= FRAME_U_RTOL, errs
    sim.close()
