"""The C restatement (oracle/restate) reproduces the reference's golden
vectors bit for bit: creation (libc rand() jitter), every stage of the first
frame from the reference's own pre-stage state, and whole frames."""
import numpy as np
import pytest

import golden_util as G
import oracle_py as O


def _same(a, b):
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint8),
                                                  np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("name", G.NAMES)
def test_create_matches(name):
    g = G.load(name)
    sim = O.OracleSim(G.scene(g), seed=7)
    st = sim.get_state()
    for f in G.FIELDS:
        assert _same(st[f], g["init_" + f]), f


@pytest.mark.parametrize("name", G.NAMES)
def test_each_stage_bit_exact(name):
    g = G.load(name)
    sc = G.scene(g)
    sim = O.OracleSim(sc, seed=7)
    for k, stage in enumerate(G.stage_order(sc)):
        sim.set_state(G.pre_stage(g, k))
        sim.stage(stage)
        st = sim.get_state()
        for f in G.FIELDS:
            assert _same(st[f], g[f"s{k}_post_{f}"]), (stage, f)


@pytest.mark.parametrize("name", G.NAMES)
def test_frames_bit_exact(name):
    g = G.load(name)
    sim = O.OracleSim(G.scene(g), seed=7)
    for frame in range(1, 11):
        sim.frame()
        if f"f{frame}_p" in g:
            st = sim.get_state()
            for f in G.FIELDS:
                assert _same(st[f], g[f"f{frame}_{f}"]), (frame, f)
            np.testing.assert_array_equal(np.array(list(sim.stats().values())), g[f"stats_f{frame}"])
