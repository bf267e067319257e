"""Batches of independent scenes (fs2d_batch_*): PIC/FLIP dam breaks of
uneven sizes.  Host worker threads queue each scene's stages on its own
stream; with mixed precision every scene's pressure solve runs in one pack
(one launch per kernel of the inner solve for all scenes, the sweeps as
persistent work items).  Every scene's state after the batch's frames must
equal, bit for bit, the state of the same scene run alone through
fs2d_run_frame (same seed), whatever the worker count, including the count
the batch chooses itself on its first frames, and a scene of a batch must
still run alone on its region of the batch's arrays."""
import numpy as np
import pytest

fs2d = pytest.importorskip("fs2d")
scenes = pytest.importorskip("scenes")
pytestmark = pytest.mark.gpu

FIELDS = ("cell", "phi", "p", "u", "v", "particles", "particleVels")
OPTS = dict(precision="mixed", pcg_tol=1e-6)


def alone(sc, seed, frames):
    sim = fs2d.FluidSim2D(sc, seed=seed, **OPTS)
    sim.step(frames)
    st = sim.get_state(FIELDS)
    sim.close()
    return st


def assert_same(a, b):
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("workers", [1, 3])
def test_batch_matches_scenes_run_alone(workers):
    scs = scenes.batch_dam_breaks(5, seed=7, lo=40, hi=100)
    b = fs2d.Batch(scs, workers=workers, seed=100, **OPTS)
    assert len(b) == 5 and b.workers == workers
    b.step(3)
    for k, sc in enumerate(scs):
        assert_same(b.scene(k).get_state(FIELDS), alone(sc, 100 + k, 3))
        assert b.scene(k).stats()["frames"] == 3
    b.close()


@pytest.mark.parametrize("schedule,ctas", [(None, 0), (0, 0), (1, 3), (2, 0), (3, 2), (4, 5)])
def test_batch_of_wide_scenes_matches_scenes_run_alone(schedule, ctas):
    """Scenes of one to three strips of the FP32 sweeps (strips of 128
    columns): the persistent sweep's work items hand columns over between
    the strips of each scene only, whatever the schedule of the work list
    (the autotuner's choice, or each schedule forced, with few CTAs)."""
    scs = scenes.batch_dam_breaks(6, seed=11, lo=100, hi=300)
    b = fs2d.Batch(scs, workers=2, seed=30, **OPTS)
    sch = b.sweep_schedule()
    assert 0 <= sch["schedule"] <= 4 and sch["items"] >= 6 and sch["sweep_us"] > 0
    if schedule is not None:
        b.set_schedule(schedule, ctas)
        assert b.sweep_schedule()["schedule"] == schedule
    b.step(2)
    for k, sc in enumerate(scs):
        assert_same(b.scene(k).get_state(FIELDS), alone(sc, 30 + k, 2))
    assert b.launch_count() > 0
    assert all(ms > 0 for ms in b.phase_ms())
    if schedule is not None:
        b.close()
        return
    # a scene of the batch run alone, on its region of the batch's arrays
    v = b.scene(4)
    assert v.runFrame() in (0, 4)
    assert_same(v.get_state(FIELDS), alone(scs[4], 34, 3))
    b.close()


def test_graph_replay_matches_direct_launches():
    """Each scene's per-frame phases replayed from CUDA graphs (captured on
    the second frame) give the bits of direct launches, also after a scene's
    state is replaced between steps (its phases are captured again)."""
    scs = scenes.batch_dam_breaks(4, seed=5, lo=40, hi=90)
    g = fs2d.Batch(scs, workers=2, seed=50, **OPTS)
    d = fs2d.Batch(scs, workers=2, seed=50, **OPTS)
    d.set_graphs(False)
    g.step(4)
    d.step(4)
    for k in range(len(scs)):
        assert_same(g.scene(k).get_state(FIELDS), d.scene(k).get_state(FIELDS))
    st = g.scene(1).get_state(["particles", "particleVels"])
    st["particleVels"] = st["particleVels"] * 0.5
    g.scene(1).set_state(st)
    d.scene(1).set_state(st)
    g.step(3)
    d.step(3)
    for k in range(len(scs)):
        assert_same(g.scene(k).get_state(FIELDS), d.scene(k).get_state(FIELDS))
        assert g.scene(k).stats()["frames"] == 7
    assert g.launch_count() > 0
    g.close()
    d.close()


def test_batch_chooses_its_worker_count():
    scs = scenes.batch_dam_breaks(12, seed=8, lo=32, hi=72)
    b = fs2d.Batch(scs, workers=0, seed=5, **OPTS)
    assert b.workers == 0
    b.step(4)
    assert b.workers in (4, 8, 16, 32) or 1 <= b.workers <= 12
    for k in (0, 5, 11):
        assert_same(b.scene(k).get_state(FIELDS), alone(scs[k], 5 + k, 4))
    b.close()


def test_batch_rejects_bad_arguments():
    scs = scenes.batch_dam_breaks(2, seed=1, lo=32, hi=40)
    with pytest.raises(fs2d.FS2DError):
        fs2d.Batch([], workers=1)
    with pytest.raises(fs2d.FS2DError):
        fs2d.Batch(scs, workers=-1)
    b = fs2d.Batch(scs, workers=2, seed=1)
    with pytest.raises(fs2d.FS2DError):
        b.scene(2)
    b.close()


def test_batch_rollout_matches_scenes_alone():
    scs = scenes.batch_closed_boxes(4, seed=3, lo=24, hi=48)
    fields = [scenes.fourier_faces(sc["sizeX"], sc["sizeY"], seed=10 + k) for k, sc in enumerate(scs)]
    targets = [scenes.fourier_faces(sc["sizeX"], sc["sizeY"], seed=20 + k) for k, sc in enumerate(scs)]
    opts = dict(precision="mixed", pcg_tol=1e-12, pcg_max_iters=2000)
    b = fs2d.Batch(scs, workers=3, seed=1, **opts)
    losses = b.forward(6, [f[0] for f in fields], [f[1] for f in fields], [t[0] for t in targets],
                       [t[1] for t in targets], checkpoint_every=2)
    grads = b.backward()
    b.close()
    for k, sc in enumerate(scs):
        sim = fs2d.FluidSim2D(sc, seed=1 + k, **opts)
        L = sim.forward(6, fields[k][0], fields[k][1], targets[k][0], targets[k][1], checkpoint_every=2)
        gu, gv = sim.backward()
        sim.close()
        assert L == losses[k]
        g, r = np.concatenate(grads[k]), np.concatenate([gu, gv])
        assert np.abs(g - r).max() <= 1e-12 * np.abs(r).max()
