"""Checkpoint and resume (fs2d_save_checkpoint / fs2d_load_checkpoint), the
injected allocation failure (fs2d_debug_fail_alloc) and applyAdvection's CFL
check (fs2d_cfl) on the GPU.

* A handle resumed from a checkpoint runs the frames the saved handle runs,
  bit for bit (FP64 path, ordered P2G; PIC/FLIP and semi-Lagrangian, with
  and without volume correction); files for another grid, with a wrong magic
  or truncated are refused and the handle stays usable.
* A create whose device allocations fail part-way returns FS2D_ERR_ALLOC,
  frees what it had allocated, and the next create works.
* fs2d_cfl returns the largest (vx + vy) dt / dx above 0 and the first
  particle reaching it, as the reference's loop does
  (src/FluidSim2D.cpp:571-585), restated here in numpy.
"""
import numpy as np
import pytest

import scenes

fs2d = pytest.importorskip("fs2d")
pytestmark = pytest.mark.gpu

FIELDS = ("cell", "phi", "p", "u", "v", "newU", "newV", "particles", "particleVels")


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("kind,rate", [("pic", 0.0), ("sl", 0.0), ("pic", 0.1)])
def test_resume_reproduces_the_frames(tmp_path, kind, rate):
    sc = scenes.pic_dam_break_disk(48) if kind == "pic" else scenes.sl_dam_break(48)
    path = str(tmp_path / "state.fs2d")
    a = fs2d.FluidSim2D(sc, seed=3)
    if rate:
        a.set_volume_correction(rate)
    for _ in range(3):
        a.runFrame()
    a.save_checkpoint(path)
    for _ in range(3):
        a.runFrame()
    b = fs2d.FluidSim2D(sc, seed=99)   # other particles until the checkpoint replaces them
    b.load_checkpoint(path)
    for _ in range(3):
        b.runFrame()
    sa, sb = a.get_state(), b.get_state()
    for f in FIELDS:
        assert same(sa[f], sb[f]), f
    ta, tb = a.stats(), b.stats()
    assert ta["currentTime"] == tb["currentTime"] and ta["frames"] == tb["frames"] == 6
    assert ta["waterVolume"] == tb["waterVolume"] and ta["origWaterVolume"] == tb["origWaterVolume"]
    a.close()
    b.close()


def test_bad_checkpoints_are_refused(tmp_path):
    sc = scenes.pic_dam_break_disk(48)
    a = fs2d.FluidSim2D(sc, seed=3)
    a.runFrame()
    good = tmp_path / "good.fs2d"
    a.save_checkpoint(str(good))
    data = good.read_bytes()
    other = fs2d.FluidSim2D(scenes.pic_dam_break_disk(32), seed=3)
    with pytest.raises(fs2d.FS2DError) as e:
        other.load_checkpoint(str(good))
    assert e.value.code == 1 and "grid" in str(e.value)
    bad_magic = tmp_path / "magic.fs2d"
    bad_magic.write_bytes(b"XXXXXXXX" + data[8:])
    truncated = tmp_path / "short.fs2d"
    truncated.write_bytes(data[:-8])
    longer = tmp_path / "long.fs2d"
    longer.write_bytes(data + b"\0")
    for path in (bad_magic, truncated, longer, tmp_path / "missing.fs2d"):
        with pytest.raises(fs2d.FS2DError) as e:
            a.load_checkpoint(str(path))
        assert e.value.code == 1, path
    assert a.runFrame() == 0   # still usable
    a.load_checkpoint(str(good))
    assert a.runFrame() == 0
    a.close()
    other.close()


def test_injected_allocation_failure_frees_and_recovers():
    torch = pytest.importorskip("torch")
    sc = scenes.pic_dam_break_disk(64)
    lib = fs2d.load()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failed = 0
    try:
        for after in (0, 1, 2, 5, 10, 20, 40):
            lib.fs2d_debug_fail_alloc(after)
            try:
                sim = fs2d.FluidSim2D(sc, seed=1, precision="mixed")
            except fs2d.FS2DError as e:
                assert e.code == 2 and "injected" in str(e), e
                failed += 1
            else:
                sim.close()
    finally:
        lib.fs2d_debug_fail_alloc(-1)
    assert failed >= 4
    torch.cuda.synchronize()
    assert free0 - torch.cuda.mem_get_info()[0] < 64 << 20   # nothing of the failed creates is left
    sim = fs2d.FluidSim2D(sc, seed=1, precision="mixed")
    assert sim.runFrame() == 0
    sim.close()


def cfl_reference(vel, dt, dx):
    """applyAdvection's loop (src/FluidSim2D.cpp:572-580): strict > from 0."""
    cmax, emax = 0.0, -1
    c = (vel[:, 0] + vel[:, 1]) * dt / dx
    for e in np.flatnonzero(c > 0.0):
        if c[e] > cmax:
            cmax, emax = float(c[e]), int(e)
    return cmax, emax


def test_cfl_matches_the_reference_loop():
    sc = scenes.pic_dam_break_disk(48)
    sim = fs2d.FluidSim2D(sc, seed=3)
    assert sim.cfl() == (0.0, -1)   # particles at rest
    for _ in range(5):
        sim.runFrame()
    st = sim.get_state()
    vel = st["particleVels"].reshape(-1, 2)
    got = sim.cfl()
    want = cfl_reference(vel, sc["dt"], sc["dx"])
    assert want[1] >= 0 and got[1] == want[1] and same(np.float64(got[0]), np.float64(want[0]))
    # ties go to the first particle, NaN never counts, nothing above 0 gives (0, -1)
    v = vel.copy()
    v[7] = v[want[1]]
    v[3] = (np.nan, 1.0)
    sim.set_state({"particles": st["particles"], "particleVels": v.ravel()})
    assert sim.cfl()[1] == min(7, want[1])
    sim.set_state({"particles": st["particles"], "particleVels": -np.abs(v.ravel())})
    assert sim.cfl() == (0.0, -1)
    sim.close()
