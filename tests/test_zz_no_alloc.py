"""fs2d_extrapolate_noalloc — the extrapolation for callers that cannot
allocate device memory (its scratch is a static device array) — gives the
same results as fs2d_extrapolate.

Called through the C ABI on device buffers the test owns, twice in a row
with different inputs (the shared scratch keeps the previous call's
contents, which must not leak into the next result), at the size limits,
banded, with a small grid right after the largest, and with grids beyond
the static capacity (by face count and by side), which must be refused.  Extrapolation is exact
arithmetic on both paths, so the comparison is bit for bit.  This file is
collected last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

fs2d = pytest.importorskip("fs2d")
torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

UNKNOWN = 0xFFFFFFFF


def case(w, h, seed, frac):
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal(w * h)
    x, y = np.meshgrid(np.arange(w), np.arange(h))
    blob = ((x - w * 0.35) ** 2 + (y - h * 0.45) ** 2 < (0.25 * min(w, h)) ** 2).ravel()
    mask = np.where(blob | (rng.random(w * h) < frac), 0, UNKNOWN).astype(np.uint32)
    return vals, mask


def call(fn, vals, mask, w, h, band=0):
    lib = fs2d.load()
    dv = torch.from_numpy(vals.copy()).cuda()
    dm = torch.from_numpy(mask.view(np.int32).copy()).cuda()
    torch.cuda.synchronize()
    rc = getattr(lib, fn)(C.c_void_p(dv.data_ptr()), C.c_void_p(dm.data_ptr()), w, h, band, None)
    torch.cuda.synchronize()
    return rc, dv.cpu().numpy(), dm.cpu().numpy().view(np.uint32)


def check_pair(w, h, seed, frac, band):
    vals, mask = case(w, h, seed, frac)
    rc_a, va, ma = call("fs2d_extrapolate", vals, mask, w, h, band)
    rc_b, vb, mb = call("fs2d_extrapolate_noalloc", vals, mask, w, h, band)
    assert rc_a == 0 and rc_b == 0, fs2d.load().fs2d_last_error()
    assert np.array_equal(ma, mb), (w, h, band)
    assert np.array_equal(va.view(np.uint64), vb.view(np.uint64)), (w, h, band)


def test_noalloc_matches_allocating_entry_point_twice():
    for (w, h, seed, frac, band) in [(333, 211, 11, 0.01, 0), (1025, 1024, 12, 0.002, 0)]:
        check_pair(w, h, seed, frac, band)


def test_noalloc_at_its_limits_and_after_a_larger_call():
    """Grids of exactly FS2D_NOALLOC_MAX_FACES faces with one side at
    FS2D_NOALLOC_MAX_SIDE, both orientations; a banded call; then a small
    grid right after the largest one, so that scratch left by a larger call
    is present and must not leak into the smaller result."""
    cases = [(8192, 256, 21, 0.001, 0), (256, 8192, 22, 0.001, 0), (8192, 256, 23, 0.001, 5),
             (97, 61, 24, 0.02, 0), (97, 61, 25, 0.02, 3)]
    for (w, h, seed, frac, band) in cases:
        check_pair(w, h, seed, frac, band)


def test_noalloc_rejects_oversized_grid():
    lib = fs2d.load()
    dv = torch.zeros(8, dtype=torch.float64, device="cuda")
    dm = torch.zeros(8, dtype=torch.int32, device="cuda")
    # by face count (4096 x 1024 = 2^22 faces) and by side (8193 x 1)
    for (w, h) in [(4096, 1024), (8193, 1), (1, 8193)]:
        rc = lib.fs2d_extrapolate_noalloc(C.c_void_p(dv.data_ptr()), C.c_void_p(dm.data_ptr()), w, h, 0, None)
        assert rc == 1, (w, h)
        assert b"static scratch" in lib.fs2d_last_error()
