"""fs2d_extrapolate (Array2D::extrapolate on device buffers) against the
oracle's breadth-first restatement: values and layers bit-exact, on random
and structured masks, including the edge cases the reference's BFS has
(no known face, every face known, a single known face, banded mode)."""
import ctypes as C

import numpy as np
import pytest

import oracle_py as O

fs2d = pytest.importorskip("fs2d")
torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

UNKNOWN = 0xFFFFFFFF


def make_case(kind, w, h, seed):
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal(w * h)
    if kind == "random":
        mask = np.where(rng.random(w * h) < 0.15, 0, UNKNOWN)
    elif kind == "blob":
        x, y = np.meshgrid(np.arange(w), np.arange(h))
        mask = np.where(((x - w * 0.3) ** 2 + (y - h * 0.4) ** 2 < (0.2 * min(w, h)) ** 2).ravel(), 0, UNKNOWN)
    elif kind == "none":
        mask = np.full(w * h, UNKNOWN)
    elif kind == "all":
        mask = np.zeros(w * h)
    elif kind == "single":
        mask = np.full(w * h, UNKNOWN)
        mask[(h // 2) * w + w // 3] = 0
    return vals, mask.astype(np.uint32)


def run_gpu(vals, mask, w, h, band=0, fn="fs2d_extrapolate"):
    dv = torch.from_numpy(vals.copy()).cuda()
    dm = torch.from_numpy(mask.astype(np.int64)).to(torch.int32).cuda()
    lib = fs2d.load()
    rc = getattr(lib, fn)(C.c_void_p(dv.data_ptr()), C.c_void_p(dm.data_ptr()), w, h, band, None)
    assert rc == 0, lib.fs2d_last_error()
    torch.cuda.synchronize()
    return dv.cpu().numpy(), dm.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("kind,w,h,seed", [("random", 67, 45, 1), ("blob", 130, 97, 2), ("none", 40, 33, 3),
                                           ("all", 31, 29, 4), ("single", 200, 150, 5), ("blob", 1025, 64, 6)])
def test_extrapolate_matches_oracle(kind, w, h, seed):
    vals, mask = make_case(kind, w, h, seed)
    ov, om = O.extrapolate(vals, mask, w, h)
    gv, gm = run_gpu(vals, mask, w, h)
    assert np.array_equal(gm, om)
    assert np.array_equal(gv.view(np.uint64), ov.view(np.uint64))


def test_extrapolate_banded_matches_oracle():
    vals, mask = make_case("blob", 150, 120, 7)
    ov, om = O.extrapolate(vals, mask, 150, 120, band=5)
    gv, _ = run_gpu(vals, mask, 150, 120, band=5)
    assert np.array_equal(gv.view(np.uint64), ov.view(np.uint64))
