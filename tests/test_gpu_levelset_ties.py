"""GPU parity of createWaterLevelSet on particle sets built to defeat
approximate distance comparisons.

The closest-point sweeps decide "d(e) < phi" from FP32 squared distances
with an error bound, then from double-float distances, and only then in
FP64 (cp_sweep.cuh).  These sets put many decisions inside or near the
bounds: exact ties from mirror-symmetric lattices, duplicate particles,
particles on cell corners, pairs whose distances to a corner differ by a
relative 1e-6 ... 1e-16, and far-field cells that are nearly equidistant
from many particles.  phi and the labels must be bit-identical to the
oracle, which is bit-exact to the reference.
"""
import numpy as np
import pytest

import oracle_py as O

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

NX, NY = 48, 40


def lattice(dx, rng):
    # 2x2 particles per cell without jitter, in a block: mirror-symmetric ties
    pts = []
    for j in range(4, 16):
        for i in range(5, 21):
            for a in range(2):
                for b in range(2):
                    pts.append(((i + 0.25 + 0.5 * a) * dx, (j + 0.25 + 0.5 * b) * dx))
    return np.array(pts)


def duplicates(dx, rng):
    base = rng.uniform([3 * dx, 3 * dx], [(NX - 3) * dx, (NY - 3) * dx], size=(150, 2))
    return np.concatenate([base, base, base[::-1]])


def on_corners(dx, rng):
    ij = rng.integers([2, 2], [NX - 2, NY - 2], size=(200, 2))
    p = ij * dx
    jitter = rng.uniform(-0.5 * dx, 0.5 * dx, size=(200, 2))
    return np.concatenate([p, p[:50] + jitter[:50]])


def near_ties(dx, rng):
    # particle pairs around corners at distances r and r (1 + eps)
    pts = []
    for k, eps in enumerate([0.0, 1e-16, 1e-15, 1e-13, 1e-12, 1e-10, 1e-9, 1e-7, 1e-6, 1e-5, 3e-5]):
        for m in range(6):
            ci = 4 + 3 * ((k * 6 + m) % 13)
            cj = 4 + 3 * ((k * 6 + m) // 13)
            r = (0.3 + 0.1 * m) * dx
            ang = rng.uniform(0, 2 * np.pi)
            pts.append((ci * dx + r * np.cos(ang), cj * dx + r * np.sin(ang)))
            ang2 = ang + rng.uniform(0.5, 2.5)
            r2 = r * (1 + eps)
            pts.append((ci * dx + r2 * np.cos(ang2), cj * dx + r2 * np.sin(ang2)))
    return np.array(pts)


def far_field(dx, rng):
    # a small cluster in one corner: the rest of the grid is far and sees
    # nearly equidistant particles
    c = rng.uniform([2 * dx, 2 * dx], [5 * dx, 5 * dx], size=(40, 2))
    line = np.stack([np.linspace(3 * dx, 30 * dx, 28), np.full(28, 3.5 * dx)], axis=1)
    return np.concatenate([c, line])


def random_blob(dx, rng):
    return rng.uniform([6 * dx, 4 * dx], [30 * dx, 25 * dx], size=(1500, 2))


SETS = {"lattice": lattice, "duplicates": duplicates, "on_corners": on_corners, "near_ties": near_ties,
        "far_field": far_field, "random": random_blob}


@pytest.mark.parametrize("name", sorted(SETS))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_levelset_exact_on_adversarial_particles(name, precision):
    sc = scenes.dam_break(NX, NY, mode=scenes.PICFLIP, extent=(0.3, 0.5))
    rng = np.random.default_rng(11)
    sim = fs2d.FluidSim2D(sc, seed=7, precision=precision)
    orc = O.OracleSim(sc, seed=7, sl_inplace=0)
    dx = sc["dx"]
    pts = SETS[name](dx, rng)
    lo, hi = 1.0001 * dx, np.array([NX - 1.0001, NY - 1.0001]) * dx
    pts = np.clip(pts, lo, hi)
    parts = np.ascontiguousarray(pts.reshape(-1))
    vels = np.zeros_like(parts)
    for s in (sim, orc):
        s.set_state({"particles": parts, "particleVels": vels})
        s.stage("createWaterLevelSet")
    a, b = sim.get_state(), orc.get_state()
    for f in ("phi", "cell"):
        x, y = np.ascontiguousarray(a[f]), np.ascontiguousarray(b[f])
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), (name, f, np.nonzero(x != y)[0][:5])
