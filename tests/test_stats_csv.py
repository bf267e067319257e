"""The statistics files of FluidSim2D::saveStats (src/FluidSim2D.cpp:738-750)
and PerformanceCounter::saveToFile (src/PerformanceCounter.cpp:58-74),
byte for byte.

fs2d_write_stats is the library's writer behind fs2d_save_stats, callable on
the host alone.  Fed the same series as the reference, it must write the
same bytes as the reference's own code:

* against tests/golden/stats_csv.npz, made by the compiled reference
  (tests/golden/make_golden.py), on every machine;
* against the compiled reference live (oracle/_ref), with other seeds, where
  that build exists.
"""
import ctypes as C
import os

import numpy as np
import pytest

import golden_util as G
import oracle_py as O
import scenes

fs2d = pytest.importorskip("fs2d")


def write_stats(tmp_path, ms, vol, en, pen, tag="x"):
    lib = fs2d.load()
    ms = np.ascontiguousarray(ms, dtype=np.float32)
    vol, en, pen = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, en, pen))
    perf, cons = str(tmp_path / f"{tag}_perf.csv"), str(tmp_path / f"{tag}_cons.csv")
    rc = lib.fs2d_write_stats(ms.ctypes.data, ms.shape[1], ms.shape[0], vol.ctypes.data, en.ctypes.data,
                              pen.ctypes.data, len(vol), perf.encode(), cons.encode())
    assert rc == 0, lib.fs2d_last_error()
    return open(perf, "rb").read(), open(cons, "rb").read()


@pytest.mark.parametrize("tag", ["sl", "pic"])
def test_write_stats_matches_reference_golden(tmp_path, tag):
    z = np.load(os.path.join(G.GOLDEN, "stats_csv.npz"))
    perf, cons = write_stats(tmp_path, z[f"{tag}_stage_ms"], z[f"{tag}_vol"], z[f"{tag}_en"], z[f"{tag}_pen"], tag)
    assert perf == z[f"{tag}_perf"].tobytes()
    assert cons == z[f"{tag}_cons"].tobytes()
    # 45 frames: the reference writes the rows of frames 30..44
    assert perf.count(b"\n") == len(z[f"{tag}_vol"]) - 30


def test_write_stats_short_runs_and_no_paths(tmp_path):
    """Fewer than 31 frames: an empty perf file, as the reference writes;
    NULL paths skip a file."""
    ms, vol, en, pen = G.stats_series(3, 12, 8)
    perf, cons = write_stats(tmp_path, ms, vol, en, pen)
    assert perf == b""
    assert cons.startswith(b"Total Volume, Total Energy, Total Energy (Particle) \n")
    assert cons.count(b"\n") == 13
    lib = fs2d.load()
    assert lib.fs2d_write_stats(None, 8, 0, None, None, None, 0, None, None) == 0


@pytest.mark.skipif(O.get_reference_lib() is None, reason="reference library not built here")
@pytest.mark.parametrize("mode,frames,seed", [("sl", 61, 11), ("pic", 31, 12), ("pic", 90, 13)])
def test_write_stats_matches_live_reference(tmp_path, mode, frames, seed):
    scene = scenes.sl_dam_break(16) if mode == "sl" else scenes.pic_dam_break_disk(16)
    stages = 7 if mode == "sl" else 8
    ms, vol, en, pen = G.stats_series(seed, frames, stages)
    ref = O.RefSim(scene, seed=1)
    d = tmp_path / "ref"
    d.mkdir()
    rperf, rcons = ref.save_stats_of(ms, vol, en, pen, str(d))
    ref.close()
    perf, cons = write_stats(tmp_path, ms, vol, en, pen)
    assert perf == rperf
    assert cons == rcons
