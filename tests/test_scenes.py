"""Seeded scene generators of the workloads (host logic, no GPU)."""
import numpy as np

import scenes


def test_batch_dam_breaks_seeded_and_in_range():
    a = scenes.batch_dam_breaks(64, seed=5)
    b = scenes.batch_dam_breaks(64, seed=5)
    assert [s["sizeX"] for s in a] == [s["sizeX"] for s in b]
    for s in a:
        n = s["sizeX"]
        assert 64 <= n <= 512 and s["sizeY"] == n
        cells = s["cells"].reshape(n, n)
        assert (cells[0] == scenes.SOLID).all() and (cells[:, -1] == scenes.SOLID).all()
        assert (cells == scenes.FLUID).any() and s["mode"] == scenes.PICFLIP
        assert abs(s["dt"] - (1.0 / 240) * 256.0 / n) < 1e-15
    sides = np.array([s["sizeX"] for s in scenes.batch_dam_breaks(2000, seed=1)])
    # log-uniform: the median side is near sqrt(64 * 512)
    assert abs(np.median(sides) - np.sqrt(64 * 512)) < 20


def test_closed_box_has_no_air():
    sc = scenes.closed_box(20, 24)
    c = sc["cells"].reshape(24, 20)
    assert not (c == scenes.EMPTY).any()
    assert (c[1:-1, 1:-1] == scenes.FLUID).all()
    assert sc["mode"] == scenes.SEMILAGRANGIAN and sc["gravityY"] == 0.0


def test_fourier_faces_amplitude_and_determinism():
    u, v = scenes.fourier_faces(32, 40, seed=3)
    u2, v2 = scenes.fourier_faces(32, 40, seed=3)
    assert u.shape == (33 * 40,) and v.shape == (32 * 41,)
    assert np.array_equal(u, u2) and np.array_equal(v, v2)
    assert abs(max(np.abs(u).max(), np.abs(v).max()) - 1.0) < 1e-12


def test_pressure_disks_fractions():
    sc, cell, phi, u, v = scenes.pressure_disks(256, 256, seed=256)
    frac = lambda lab: float((cell == lab).mean())
    assert 0.2 <= frac(scenes.EMPTY) <= 0.3
    assert 0.04 <= frac(scenes.SOLID) <= 0.1
    assert np.all((phi < 0) == (cell == scenes.FLUID))
