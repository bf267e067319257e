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
    assert lib.fs2d_reseed(None, 4, 8, 0, None) == INVALID
    assert lib.fs2d_set_volume_correction(None, 0.1) == INVALID
    assert lib.fs2d_cfl(None, None, None) == INVALID
    assert lib.fs2d_save_checkpoint(None, b"x") == INVALID
    assert lib.fs2d_load_checkpoint(None, b"x") == INVALID
    assert lib.fs2d_destroy(None) == 0
    assert lib.fs2d_batch_destroy(None) == 0


def test_no_cpu_fallback_without_a_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    rc, msg, h = create(scenes.sl_dam_break(16))
    assert rc == CUDA and "device" in msg
    assert not h.value


def arr3(data, nx, ny, nz):
    return fs2d.Array3D(data, nx, ny, nz)


def mac3(sx, sy, sz, ptr=None):
    return fs2d.MACGrid3D(arr3(ptr, sx + 1, sy, sz), arr3(ptr, sx, sy + 1, sz), arr3(ptr, sx, sy, sz + 1), sx, sy, sz)


def test_grid3d_arguments_are_checked_before_device_work():
    """include/fs3d.h: NULL structs, negative or mismatched extents, a bad
    axis or component are refused with FS2D_ERR_INVALID before any CUDA
    call; empty arrays are a no-op (0 for the reductions), also without a
    device."""
    lib = fs2d.load()
    res = C.c_double(7.0)
    a = arr3(None, 2, 3, 4)
    assert lib.fs3d_add(None, C.byref(a), None) == INVALID
    assert lib.fs3d_add(C.byref(arr3(None, -1, 3, 4)), C.byref(a), None) == INVALID
    assert lib.fs3d_add(C.byref(arr3(None, 2, 3, 5)), C.byref(a), None) == INVALID
    assert lib.fs3d_set_multiply_add(C.byref(a), C.byref(a), 2.0, C.byref(arr3(None, 3, 3, 4)), None) == INVALID
    assert lib.fs3d_inner_product(C.byref(a), C.byref(a), None, None) == INVALID
    assert lib.fs3d_inner_product(C.byref(a), C.byref(arr3(None, 2, 4, 3)), C.byref(res), None) == INVALID
    assert lib.fs3d_infinite_norm(C.byref(a), None, None) == INVALID
    assert lib.fs3d_tricubic(None, None, 4, None, None) == INVALID
    g = mac3(3, 2, 2)
    assert lib.fs3d_mac_vel(None, None, None) == INVALID
    assert lib.fs3d_mac_vel(C.byref(mac3(0, 2, 2)), None, None) == INVALID
    bad = mac3(3, 2, 2)
    bad.v = arr3(None, 3, 2, 2)   # v must have sizeY + 1 rows
    assert lib.fs3d_mac_vel_div(C.byref(bad), None, None) == INVALID
    assert "sizeY+1" in lib.fs2d_last_error().decode()
    assert lib.fs3d_mac_face_vel(C.byref(g), 3, None, None) == INVALID
    assert lib.fs3d_mac_vel_interp(C.byref(g), 4, None, 1, None, None) == INVALID
    # empty arrays and empty point sets need no device
    e = arr3(None, 0, 3, 4)
    assert lib.fs3d_add(C.byref(e), C.byref(e), None) == 0
    assert lib.fs3d_inner_product(C.byref(e), C.byref(e), C.byref(res), None) == 0 and res.value == 0.0
    res.value = 7.0
    assert lib.fs3d_infinite_norm(C.byref(e), C.byref(res), None) == 0 and res.value == 0.0
    assert lib.fs3d_tricubic(C.byref(a), None, 0, None, None) == 0
    assert lib.fs3d_mac_vel_interp(C.byref(g), 3, None, 0, None, None) == 0


def test_grid3d_without_a_device_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    lib = fs2d.load()
    host = np.zeros(24)
    a = arr3(host.ctypes.data, 2, 3, 4)
    assert lib.fs3d_add(C.byref(a), C.byref(a), None) == CUDA
    g = mac3(1, 1, 1, host.ctypes.data)
    assert lib.fs3d_mac_vel_div(C.byref(g), host.ctypes.data, None) == CUDA
