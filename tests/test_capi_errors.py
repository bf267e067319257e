"""Argument checking of the C ABI, which happens before any device work (runs
without a GPU): invalid configurations and options are refused with
FS2D_ERR_INVALID and a message; null handles are refused; and on a machine
without a CUDA device a valid configuration fails with FS2D_ERR_CUDA (there is
no CPU fallback)."""
import ctypes as C

import numpy as np
import pytest

import fs2d
import scenes

INVALID, CUDA = 1, 3


def create(sc, **opts):
    lib = fs2d.load()
    cfg = fs2d.make_config(sc)
    o = fs2d.default_options(**opts)
    h = C.c_void_p()
    rc = lib.fs2d_create(C.byref(cfg), C.byref(o), C.byref(h))
    return rc, lib.fs2d_last_error().decode(), h


def test_invalid_configurations_are_refused():
    sc = scenes.sl_dam_break(16)
    bad = dict(sc, sizeX=2, sizeY=2, cells=np.full(4, scenes.SOLID, np.uint8))
    assert create(bad)[0] == INVALID
    border = dict(sc, cells=sc["cells"].copy())
    border["cells"][0] = scenes.FLUID
    rc, msg, _ = create(border)
    assert rc == INVALID and "border" in msg
    label = dict(sc, cells=sc["cells"].copy())
    label["cells"][5 * 16 + 5] = 7
    assert create(label)[0] == INVALID
    assert create(dict(sc, ppcSqrt=0))[0] == INVALID
    assert create(dict(sc, dx=0.0))[0] == INVALID
    assert create(dict(sc, mode=5))[0] == INVALID
    # the size limit is checked before the labels are read
    huge = dict(sc, sizeX=20000, sizeY=20000)
    rc, msg, _ = create(huge)
    assert rc == INVALID and "too large" in msg


def test_invalid_options_are_refused():
    sc = scenes.sl_dam_break(16)
    assert create(sc, precision=7)[0] == INVALID
    assert create(sc, pcg_tol=-1.0)[0] == INVALID
    assert create(sc, pcg_max_iters=-1)[0] == INVALID
    assert create(sc, ir_inner_tol=0.0)[0] == INVALID
    assert create(sc, ir_max_outer=0)[0] == INVALID


def test_null_handles_are_refused():
    lib = fs2d.load()
    assert lib.fs2d_run_frame(None) == INVALID
    assert lib.fs2d_run_stage(None, 1) == INVALID
    assert lib.fs2d_step(None, 1) == INVALID
    assert lib.fs2d_forward(None, 4, 0, None, None, None, None, None) == INVALID
    assert lib.fs2d_backward(None, None, None) == INVALID
    assert lib.fs2d_p2g_adjoint(None, None, None, None) == INVALID
    assert lib.fs2d_g2p_adjoint(None, None, None, None, None, None, None) == INVALID
    assert lib.fs2d_batch_create(None, 0, None, 0, None) == INVALID
    assert lib.fs2d_batch_step(None, 1) == INVALID
    assert lib.fs2d_render_export(None, None) == INVALID
    assert lib.fs2d_destroy(None) == 0
    assert lib.fs2d_batch_destroy(None) == 0


def test_no_cpu_fallback_without_a_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    rc, msg, h = create(scenes.sl_dam_break(16))
    assert rc == CUDA and "device" in msg
    assert not h.value
