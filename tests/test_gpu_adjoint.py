"""Differentiable rollout (fs2d_forward / fs2d_backward) on a closed box of
fluid: semi-Lagrangian advection, projection and the velocity update, FP64.

* small box, through the C ABI: the loss against the FP64 CPU restatement
  (dense pressure solve) and the gradient against that restatement's
  reverse mode (torch.autograd on the CPU, oracle/rollout_autograd.py);
* 128 x 128, 64 steps, dt 1/60, 16-mode Fourier initial field of amplitude
  1, checkpoints every sqrt(T) = 8 steps: the hand-written adjoint against
  FP64 central differences of the GPU forward along 8 seeded random
  directions (eps = 1e-4 per face), within 1e-4 relative;
* both with the FP64 projection and with the mixed one (FP32 MIC(0)-PCG in
  FP64 refinement), each solved to 1e-12;
* the gradient does not depend on the checkpoint spacing, and device
  pointers work like host ones;
* scenes the rollout does not cover are refused.
"""
import numpy as np
import pytest

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

FD_REL = 1e-4          # central differences vs adjoint, per direction
CPU_GRAD_REL = 1e-7    # GPU adjoint vs CPU reverse mode, max-norm relative
CPU_LOSS_REL = 1e-10   # GPU forward (PCG to 1e-12) vs dense solve
CKPT_REL = 1e-12       # gradients with different checkpoint spacings


def make(nx, **kw):
    sc = scenes.closed_box(nx)
    opts = dict(pcg_tol=1e-12, pcg_max_iters=2000)
    opts.update(kw)
    return sc, fs2d.FluidSim2D(sc, seed=1, **opts)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_matches_cpu_reverse_mode(precision):
    torch = pytest.importorskip("torch")
    RA = pytest.importorskip("rollout_autograd")
    nx, steps = 32, 8
    sc, sim = make(nx, precision=precision)
    u0, v0 = scenes.fourier_faces(nx, nx, seed=11)
    ut, vt = scenes.fourier_faces(nx, nx, seed=12)
    loss = sim.forward(steps, u0, v0, ut, vt, checkpoint_every=3)
    gu, gv = sim.backward()
    sim.close()
    ref = RA.ClosedBoxRollout(sc)
    L, ru, rv, _, _ = ref.loss_and_grad(u0, v0, ut, vt, steps)
    assert abs(loss - L) <= CPU_LOSS_REL * L
    g, r = np.concatenate([gu, gv]), np.concatenate([ru, rv])
    assert np.abs(g - r).max() <= CPU_GRAD_REL * np.abs(r).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_finite_differences_128(precision):
    nx, steps = 128, 64
    sc, sim = make(nx, precision=precision)
    u0, v0 = scenes.fourier_faces(nx, nx, seed=1)
    ut, vt = scenes.fourier_faces(nx, nx, seed=2)
    sim.forward(steps, u0, v0, ut, vt)
    gu, gv = sim.backward()
    rng = np.random.default_rng(3)
    eps = 1e-4
    worst = 0.0
    for _ in range(8):
        du, dv = rng.standard_normal(gu.size), rng.standard_normal(gv.size)
        lp = sim.forward(steps, u0 + eps * du, v0 + eps * dv, ut, vt)
        lm = sim.forward(steps, u0 - eps * du, v0 - eps * dv, ut, vt)
        fd = (lp - lm) / (2 * eps)
        ad = gu @ du + gv @ dv
        worst = max(worst, abs(fd - ad) / abs(ad))
    sim.close()
    assert worst <= FD_REL, worst


def test_checkpoint_spacing_and_device_pointers():
    torch = pytest.importorskip("torch")
    nx, steps = 64, 12
    _, sim = make(nx)
    u0, v0 = scenes.fourier_faces(nx, nx, seed=5)
    ut, vt = scenes.fourier_faces(nx, nx, seed=6)
    grads, losses = [], []
    for every in (1, 0, 5, 12):
        losses.append(sim.forward(steps, u0, v0, ut, vt, checkpoint_every=every))
        grads.append(np.concatenate(sim.backward()))
    dev = [torch.tensor(a, device="cuda") for a in (u0, v0, ut, vt)]
    losses.append(sim.forward(steps, *(t.data_ptr() for t in dev), checkpoint_every=4))
    gdu = torch.empty(u0.size, dtype=torch.float64, device="cuda")
    gdv = torch.empty(v0.size, dtype=torch.float64, device="cuda")
    sim.backward(gdu.data_ptr(), gdv.data_ptr())
    grads.append(np.concatenate([gdu.cpu().numpy(), gdv.cpu().numpy()]))
    sim.close()
    scale = np.abs(grads[0]).max()
    for L, g in zip(losses[1:], grads[1:]):
        assert L == losses[0]
        assert np.abs(g - grads[0]).max() <= CKPT_REL * scale


def test_rollout_refuses_other_scenes():
    nx = 32
    u0, v0 = scenes.fourier_faces(nx, nx, seed=5)
    sim = fs2d.FluidSim2D(scenes.sl_dam_break(nx), seed=1)   # has EMPTY cells
    with pytest.raises(fs2d.FS2DError) as e:
        sim.forward(4, u0, v0, u0, v0)
    assert e.value.code == 1
    with pytest.raises(fs2d.FS2DError) as e:
        sim.backward()
    assert e.value.code == 1
    sim.close()
    sc = scenes.closed_box(nx)
    sc["mode"] = scenes.PICFLIP
    sim = fs2d.FluidSim2D(sc, seed=1)
    with pytest.raises(fs2d.FS2DError) as e:
        sim.forward(4, u0, v0, u0, v0)
    assert e.value.code == 1
    sim.close()
