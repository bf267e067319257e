"""The FP64 CPU adjoint restatement (oracle/rollout_autograd.py) pinned on
the CPU before it checks the GPU adjoint:

* its forward step equals the oracle's stages (applySemiLagrangianAdvection
  double-buffered, applyGravity, applyProjection solved to 1e-12,
  updateVelocity) on a closed box, within 1e-10 of the largest velocity
  (the PCG stopping rule against the dense solve);
* its reverse mode equals central differences of its own forward.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import oracle_py as O
import rollout_autograd as RA
import scenes

STAGES = ("applySemiLagrangianAdvection", "applyGravity", "applyProjection", "updateVelocity")


@pytest.mark.parametrize("nx,ny", [(24, 24), (20, 28)])
def test_forward_matches_oracle_stages(nx, ny):
    sc = scenes.closed_box(nx, ny)
    sc["gravityY"] = -9.8
    u0, v0 = scenes.fourier_faces(nx, ny, seed=nx + ny)
    model = RA.ClosedBoxRollout(sc)
    orc = O.OracleSim(sc, seed=1, sl_inplace=0, pcg_tol=1e-12, pcg_max_iters=2000)
    orc.set_state({"u": u0, "v": v0})
    for _ in range(3):
        for st in STAGES:
            orc.stage(st)
        assert orc.solver_info()["rel_residual"] <= 1e-12
    s = orc.get_state()
    orc.close()
    u, v = model.rollout(u0, v0, 3)
    scale = max(np.abs(u).max(), np.abs(v).max())
    assert np.abs(s["u"] - u).max() <= 1e-10 * scale
    assert np.abs(s["v"] - v).max() <= 1e-10 * scale


def test_reverse_mode_matches_central_differences():
    nx, steps = 20, 4
    sc = scenes.closed_box(nx)
    u0, v0 = scenes.fourier_faces(nx, nx, seed=1)
    ut, vt = scenes.fourier_faces(nx, nx, seed=2)
    model = RA.ClosedBoxRollout(sc)
    L, gu, gv, _, _ = model.loss_and_grad(u0, v0, ut, vt, steps)

    def loss(u, v):
        a, b = model.rollout(u, v, steps)
        return np.sqrt(((a - ut) ** 2).sum() + ((b - vt) ** 2).sum())

    assert abs(loss(u0, v0) - L) <= 1e-14 * L
    rng = np.random.default_rng(0)
    eps = 1e-4
    for _ in range(3):
        du, dv = rng.standard_normal(gu.size), rng.standard_normal(gv.size)
        fd = (loss(u0 + eps * du, v0 + eps * dv) - loss(u0 - eps * du, v0 - eps * dv)) / (2 * eps)
        ad = gu @ du + gv @ dv
        assert abs(fd - ad) <= 1e-6 * abs(ad)
