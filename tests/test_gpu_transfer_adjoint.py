"""Transposes of the particle transfers (fs2d_p2g_adjoint, fs2d_g2p_adjoint)
at fixed particle positions, checked by the dot-product identity
<A x, y> = <x, A^T y> against the forward stages run by the library itself
(transferVelocityToGrid and updateParticleVelocities, which are bit-exact to
the reference), with seeded random vectors:

* P2G: x = particle velocities, A x = the face velocities after the splat,
  the division by the summed weights and the extrapolation of unknown faces;
* G2P: x = (newMac, mac, particle velocities), A x = the new particle
  velocities (PIC/FLIP blend).

Tolerance DOT_RTOL relative to sum |terms| (rounding of FP64 sums in
different orders, and the weight sums accumulated atomically in the
transpose)."""
import numpy as np
import pytest

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

DOT_RTOL = 1e-12


def setup(nx, seed):
    sc = scenes.pic_dam_break_disk(nx)
    sim = fs2d.FluidSim2D(sc, seed=seed)
    for _ in range(2):   # particles away from their seeding lattice
        sim.runFrame()
    return sc, sim


@pytest.mark.parametrize("nx,band", [(48, 0), (64, 0), (64, 3)])
def test_p2g_adjoint_dot_product(nx, band):
    sc = scenes.pic_dam_break_disk(nx)
    sim = fs2d.FluidSim2D(sc, seed=2, extrapolate_band=band)
    for _ in range(2):
        sim.runFrame()
    rng = np.random.default_rng(nx + band)
    n = sim.num_particles()
    vel = rng.standard_normal(2 * n)
    pos = sim.get_state(["particles"])["particles"]
    sim.set_state({"particles": pos, "particleVels": vel})
    sim.stage("transferVelocityToGrid")
    st = sim.get_state(["u", "v"])
    ub = rng.standard_normal(st["u"].size)
    vb = rng.standard_normal(st["v"].size)
    gb = sim.p2g_adjoint(ub, vb)
    lhs = st["u"] @ ub + st["v"] @ vb
    rhs = vel @ gb
    scale = np.abs(st["u"] * ub).sum() + np.abs(st["v"] * vb).sum()
    assert abs(lhs - rhs) <= DOT_RTOL * scale, (lhs, rhs, scale)
    sim.close()


@pytest.mark.parametrize("nx", [48, 64])
def test_g2p_adjoint_dot_product(nx):
    sc, sim = setup(nx, 4)
    rng = np.random.default_rng(nx)
    n = sim.num_particles()
    NU, NV = (nx + 1) * nx, nx * (nx + 1)
    x = {"newU": rng.standard_normal(NU), "newV": rng.standard_normal(NV), "u": rng.standard_normal(NU),
         "v": rng.standard_normal(NV), "particleVels": rng.standard_normal(2 * n)}
    sim.set_state(dict(x, particles=sim.get_state(["particles"])["particles"]))
    sim.stage("updateParticleVelocities")
    out = sim.get_state(["particleVels"])["particleVels"]
    y = rng.standard_normal(2 * n)
    nub, nvb, ubar, vbar, ib = sim.g2p_adjoint(y)
    lhs = out @ y
    rhs = x["newU"] @ nub + x["newV"] @ nvb + x["u"] @ ubar + x["v"] @ vbar + x["particleVels"] @ ib
    scale = np.abs(out * y).sum()
    assert abs(lhs - rhs) <= DOT_RTOL * scale * 10, (lhs, rhs, scale)
    sim.close()
