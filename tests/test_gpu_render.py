"""Headless render-data export (fs2d_render_export) against the same
quantities computed on the host from the downloaded state, following
FluidRenderer2D::updateBuffers (demo/FluidRenderer2D.cpp:435-486):
compacted FLUID / SOLID / nonzero-pressure cell lists in row-major order,
cell and particle velocity segments from velInterp (the oracle's triCubic,
bit-exact after the renderer's float casts), sigmoid values within 2 ulp
(FP32 exponential)."""
import numpy as np
import pytest

import oracle_py as O

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def vel_interp(u, v, nx, ny, dx, x, y):
    def clamp(a, lo, hi):
        return min(max(a, lo), hi)
    px, py = clamp(x / dx, 1e-6, nx - 1 - 1e-6), clamp(y / dx - 0.5, 1e-6, ny - 1 - 1e-6)
    vx = O.tricubic(u, nx + 1, ny, px, py)
    px, py = clamp(x / dx - 0.5, 1e-6, nx - 1 - 1e-6), clamp(y / dx, 1e-6, ny - 1 - 1e-6)
    vy = O.tricubic(v, nx, ny + 1, px, py)
    return vx, vy


def sigmoid32(x):
    x = np.asarray(x, np.float32)
    return (np.float32(1) / (np.float32(1) + np.exp(-x))).astype(np.float32)


def ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b).max() if a.size else 0


def test_render_export_matches_host():
    nx, ny = 48, 40
    sc = scenes.dam_break(nx, ny, mode=scenes.PICFLIP, dt=1.0 / 240, extent=(0.4, 0.6), disk=(0.7, 0.7, 0.1))
    sim = fs2d.FluidSim2D(sc, seed=3)
    for _ in range(3):
        sim.runFrame()
    st = sim.get_state()
    dx, dt = sc["dx"], sc["dt"]
    N = nx * ny
    np_ = sim.num_particles()
    dev = lambda n: torch.zeros(n, dtype=torch.float32, device="cuda")
    bufs = {"waterCells": dev(2 * N), "solidCells": dev(2 * N), "pressureCells": dev(2 * N),
            "pressureValues": dev(N), "cellVels": dev(4 * (nx - 1) * (ny - 1)), "particleLines": dev(4 * np_),
            "phiValues": dev(N)}
    torch.cuda.synchronize()
    counts = sim.render_export({k: t.data_ptr() for k, t in bufs.items()}, {"water": N, "solid": N, "pressure": N})
    out = {k: t.cpu().numpy() for k, t in bufs.items()}

    cell = st["cell"].reshape(ny, nx)
    jj, ii = np.mgrid[0:ny, 0:nx]
    corners = np.stack([(ii * dx).astype(np.float32), (jj * dx).astype(np.float32)], axis=-1)
    for name, label, cnt in (("waterCells", scenes.FLUID, counts[0]), ("solidCells", scenes.SOLID, counts[1])):
        want = corners[cell == label].reshape(-1)
        assert cnt == (cell == label).sum()
        assert np.array_equal(out[name][:2 * cnt], want), name
    p = st["p"].reshape(ny, nx)
    sel = p != 0
    assert counts[2] == sel.sum() and counts[2] > 0
    assert np.array_equal(out["pressureCells"][:2 * counts[2]], corners[sel].reshape(-1))
    assert ulps(out["pressureValues"][:counts[2]], sigmoid32(np.float32(0.01) * p[sel].astype(np.float32))) <= 2
    assert ulps(out["phiValues"], sigmoid32((100.0 * st["phi"]).astype(np.float32))) <= 2

    u, v = st["u"], st["v"]
    cv = []
    for j in range(ny - 1):
        for i in range(nx - 1):
            x, y = (i + 0.5) * dx, (j + 0.5) * dx
            vx, vy = vel_interp(u, v, nx, ny, dx, x, y)
            cv += [x, y, x + vx * dt, y + vy * dt]
    assert np.array_equal(out["cellVels"], np.asarray(cv).astype(np.float32))
    pl = []
    pos = st["particles"].reshape(-1, 2)
    f32 = np.float32
    for x, y in pos:
        vx, vy = vel_interp(u, v, nx, ny, dx, x, y)
        pl += [f32(x), f32(y), f32(x) + f32(dt) * f32(vx), f32(y) + f32(dt) * f32(vy)]
    assert np.array_equal(out["particleLines"], np.asarray(pl, np.float32))
