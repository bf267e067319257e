"""The device kernels behind include/fs3d.h (the reference's Array3D and
MACGrid3D methods, include/Array3D.h and include/MACGrid3D.h) against the
oracle, through the C ABI:

* bit for bit against the C restatement (oracle/restate/fs3d_oracle.c) for
  operator+=, setMultiplyAdd, infiniteNorm, triCubic, vel, velU/V/W,
  velInterp and velDiv, at the golden sizes and at sizes where every thread
  of the grid-stride loops takes several elements, with 16-byte aligned
  (vector path) and 8-byte aligned (scalar path) operands;
* bit for bit against the reference's own outputs (tests/golden/grid3d.npz)
  where those are defined (triCubic and velInterp on x/z-exchanged cubes,
  the MAC stencils, the array operations with the aliased rows zeroed);
* innerProduct within the bound of any summation order,
  2 n 2^-53 sum |a b|, exactly on integer data, and the same bits on every
  call;
* edge cases: NaN, infinite and far-away sample points, NaN and signed-zero
  elements in the norm, empty arrays, host pointers refused.
"""
import ctypes as C
import os

import numpy as np
import pytest

import grid3d_cases as K
import oracle3d

fs2d = pytest.importorskip("fs2d")
torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

R = oracle3d.restated
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grid3d.npz")
U53 = 2.0 ** -53


def lib():
    return fs2d.load()


def ok(rc):
    assert rc == 0, lib().fs2d_last_error().decode()


def dev(a, pad_front=0):
    """Device copy of a flat float64 array; with pad_front=1 the data starts
    8 bytes into the allocation (not 16-byte aligned)."""
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    t = torch.zeros(a.size + pad_front + 1, dtype=torch.float64, device="cuda")
    t[pad_front:pad_front + a.size] = torch.from_numpy(a).cuda()
    return t, t.data_ptr() + 8 * pad_front


def host(t, ptr, n):
    torch.cuda.synchronize()
    off = (ptr - t.data_ptr()) // 8
    return t[off:off + n].cpu().numpy().copy()


def arr(ptr, dims):
    return fs2d.Array3D(ptr, *dims)


def same(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


# ---- Array3D: +=, setMultiplyAdd, innerProduct, infiniteNorm ----

def gpu_array_ops(a, b, dims, s, pad):
    n = a.size
    ta, pa = dev(a, pad)
    tb, pb = dev(b, pad)
    ok(lib().fs3d_add(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), None))
    added = host(ta, pa, n)
    to, po = dev(np.zeros(n), pad)
    ta, pa = dev(a, pad)
    ok(lib().fs3d_set_multiply_add(C.byref(arr(po, dims)), C.byref(arr(pa, dims)), s, C.byref(arr(pb, dims)), None))
    sma = host(to, po, n)
    dot, dot2, norm = C.c_double(), C.c_double(), C.c_double()
    ok(lib().fs3d_inner_product(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), C.byref(dot), None))
    ok(lib().fs3d_inner_product(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), C.byref(dot2), None))
    ok(lib().fs3d_infinite_norm(C.byref(arr(pa, dims)), C.byref(norm), None))
    return added, sma, dot.value, dot2.value, norm.value


@pytest.mark.parametrize("dims", K.ARRAY_DIMS + [(100, 80, 61), (257, 129, 65)])
@pytest.mark.parametrize("pad", [0, 1])
def test_array_ops_match_oracle(dims, pad):
    a, b = K.array(dims, 71), K.array(dims, 72)
    added, sma, dot, dot2, norm = gpu_array_ops(a, b, dims, -0.6180339887, pad)
    assert same(added, R.add(a, b, dims))
    assert same(sma, R.set_multiply_add(a, -0.6180339887, b, dims))
    assert same(norm, R.infinite_norm(a, dims))
    n = a.size
    assert abs(dot - R.inner_product(a, b, dims)) <= 2.0 * n * U53 * np.abs(a * b).sum()
    assert same(dot, dot2)


@pytest.mark.parametrize("d", range(len(K.ARRAY_DIMS)))
def test_array_ops_match_reference_golden(golden, d):
    dims = K.ARRAY_DIMS[d]
    a, b, bz = golden[f"arr{d}_a"], golden[f"arr{d}_b"], golden[f"arr{d}_bz"]
    added, _, dot, _, norm = gpu_array_ops(a, bz, dims, K.SCALE, 0)
    _, sma, _, _, _ = gpu_array_ops(a, b, dims, K.SCALE, 0)
    assert same(added, golden[f"arr{d}_add"])
    assert same(sma, golden[f"arr{d}_sma"])
    assert same(norm, golden[f"arr{d}_norm"])
    ref_dot = float(golden[f"arr{d}_dot"])
    assert abs(dot - ref_dot) <= 2.0 * a.size * U53 * np.abs(a * bz).sum()


def test_set_multiply_add_in_place():
    dims = (31, 17, 9)
    a, c = K.array(dims, 81), K.array(dims, 82)
    ta, pa = dev(a)
    tc, pc = dev(c)
    ok(lib().fs3d_set_multiply_add(C.byref(arr(pa, dims)), C.byref(arr(pa, dims)), 2.5, C.byref(arr(pc, dims)), None))
    assert same(host(ta, pa, a.size), R.set_multiply_add(a, 2.5, c, dims))
    ok(lib().fs3d_set_multiply_add(C.byref(arr(pc, dims)), C.byref(arr(pa, dims)), -1.0, C.byref(arr(pc, dims)), None))
    assert same(host(tc, pc, c.size), R.set_multiply_add(R.set_multiply_add(a, 2.5, c, dims), -1.0, c, dims))


def test_reductions_exact_on_integer_data():
    """Small integers: every product and partial sum is exact, so any order
    gives the exact value; checked at 4.2 M elements (several per thread)."""
    dims = (256, 256, 64)
    rng = np.random.default_rng(5)
    a = rng.integers(-8, 9, size=dims[0] * dims[1] * dims[2]).astype(np.float64)
    b = rng.integers(-8, 9, size=a.size).astype(np.float64)
    for pad in (0, 1):
        ta, pa = dev(a, pad)
        tb, pb = dev(b, pad)
        dot, norm = C.c_double(), C.c_double()
        ok(lib().fs3d_inner_product(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), C.byref(dot), None))
        ok(lib().fs3d_infinite_norm(C.byref(arr(pb, dims)), C.byref(norm), None))
        assert dot.value == float(np.dot(a.astype(np.int64), b.astype(np.int64)))
        assert norm.value == 8.0


def test_infinite_norm_passes_over_nan_and_signed_zero():
    dims = (9, 5, 3)
    a = np.zeros(dims[0] * dims[1] * dims[2])
    a[::7] = np.nan
    a[3] = -0.0
    a[10] = -2.5
    a[-1] = 2.25
    ta, pa = dev(a)
    norm = C.c_double()
    ok(lib().fs3d_infinite_norm(C.byref(arr(pa, dims)), C.byref(norm), None))
    assert norm.value == 2.5 == R.infinite_norm(a, dims)
    t2, p2 = dev(np.full(a.size, np.nan))
    ok(lib().fs3d_infinite_norm(C.byref(arr(p2, dims)), C.byref(norm), None))
    assert same(norm.value, 0.0)
    t3, p3 = dev(np.full(a.size, -0.0))
    ok(lib().fs3d_infinite_norm(C.byref(arr(p3, dims)), C.byref(norm), None))
    assert same(norm.value, 0.0)


# ---- triCubic ----

def gpu_tricubic(data, dims, pts, pad=0):
    td, pd = dev(data)
    tp, pp = dev(np.asarray(pts, dtype=np.float64).ravel(), pad)
    n = np.asarray(pts).reshape(-1, 3).shape[0]
    to, po = dev(np.full(n, -1.0))
    ok(lib().fs3d_tricubic(C.byref(arr(pd, dims)), C.c_void_p(pp), n, C.c_void_p(po), None))
    return host(to, po, n)


@pytest.mark.parametrize("n", K.CUBES)
def test_tricubic_matches_reference_golden_on_swapped_cube(golden, n):
    data, pts = golden[f"cube{n}_data"], golden[f"cube{n}_pts"]
    got = gpu_tricubic(oracle3d.swap_xz(data, (n, n, n)), (n, n, n), pts)
    assert same(got, golden[f"cube{n}_tricubic"])


@pytest.mark.parametrize("dims", [(5, 4, 3), (1, 1, 1), (2, 9, 4), (64, 48, 40)])
@pytest.mark.parametrize("pad", [0, 1])
def test_tricubic_matches_oracle(dims, pad):
    data = K.array(dims, 91)
    pts = K.points(max(dims), 5000, 92)
    pts = np.concatenate([pts, [[np.nan, 0.5, 0.5], [0.5, np.inf, 0.5], [0.5, 0.5, -np.inf],
                                [2.5e9, 0.5, 0.5], [-2.5e9, 0.5, 0.5]]])
    got = gpu_tricubic(data, dims, pts, pad)
    assert same(got, R.tricubic(data, dims, pts))
    assert np.all(got[-5:] == 0.0)


def test_tricubic_on_an_empty_array_writes_zeros():
    pts = K.points(3, 10, 93)
    got = gpu_tricubic(np.zeros(1), (0, 3, 3), pts)
    assert np.all(got == 0.0)


# ---- MACGrid3D: vel, velU/V/W, velDiv, velInterp ----

def gpu_mac(u, v, w, size):
    tu, pu = dev(u)
    tv, pv = dev(v)
    tw, pw = dev(w)
    du, dv, dw = oracle3d.face_dims(*size)
    g = fs2d.MACGrid3D(arr(pu, du), arr(pv, dv), arr(pw, dw), *size)
    return g, (tu, tv, tw)


def gpu_stencils(u, v, w, size):
    g, keep = gpu_mac(u, v, w, size)
    ncell = size[0] * size[1] * size[2]
    out = {}
    to, po = dev(np.zeros(3 * ncell))
    ok(lib().fs3d_mac_vel(C.byref(g), C.c_void_p(po), None))
    out["vel"] = host(to, po, 3 * ncell).reshape(-1, 3)
    for axis, fd in zip(("u", "v", "w"), oracle3d.face_dims(*size)):
        nf = fd[0] * fd[1] * fd[2]
        to, po = dev(np.zeros(3 * nf))
        ok(lib().fs3d_mac_face_vel(C.byref(g), fs2d.FS3D_AXES[axis], C.c_void_p(po), None))
        out["vel" + axis] = host(to, po, 3 * nf).reshape(-1, 3)
    to, po = dev(np.zeros(ncell))
    ok(lib().fs3d_mac_vel_div(C.byref(g), C.c_void_p(po), None))
    out["div"] = host(to, po, ncell)
    return out


@pytest.mark.parametrize("m", range(len(K.MAC_SIZES)))
def test_mac_stencils_match_reference_golden(golden, m):
    size = K.MAC_SIZES[m]
    out = gpu_stencils(golden[f"mac{m}_u"], golden[f"mac{m}_v"], golden[f"mac{m}_w"], size)
    for key in ("vel", "velu", "velv", "velw", "div"):
        assert same(out[key], golden[f"mac{m}_{key}"]), key


@pytest.mark.parametrize("size", [(37, 29, 23), (128, 96, 80), (1, 7, 2)])
def test_mac_stencils_match_oracle(size):
    u, v, w = K.mac_fields(size, 101)
    out = gpu_stencils(u, v, w, size)
    assert same(out["vel"], R.mac_vel(u, v, w, size))
    for axis in ("u", "v", "w"):
        assert same(out["vel" + axis], R.mac_face_vel(u, v, w, size, axis)), axis
    assert same(out["div"], R.mac_vel_div(u, v, w, size))


def special_fields(size, seed):
    """N(0,1) faces with about one in ten replaced by a value whose half or
    quarter the kernels must take from the FP64 multiply rather than from
    an exponent decrement: zeros of both signs, subnormals, the smallest
    normals (whose half or quarter is subnormal) and values near the largest
    double (sums of two overflow to +inf; no sum can form a NaN)."""
    u, v, w = K.mac_fields(size, seed)
    rng = np.random.default_rng(seed + 1)
    specials = np.array([0.0, -0.0, 1e-310, -3e-310, 2.2250738585072014e-308, -4.4e-308, 1.7e308])
    for f in (u, v, w):
        m = rng.random(f.size) < 0.1
        f[m] = rng.choice(specials, size=int(m.sum()))
    return u, v, w


@pytest.mark.parametrize("size", [(37, 29, 23), (2, 3, 4)])
def test_mac_stencils_special_values_match_oracle(size):
    u, v, w = special_fields(size, 131)
    out = gpu_stencils(u, v, w, size)
    assert same(out["vel"], R.mac_vel(u, v, w, size))
    for axis in ("u", "v", "w"):
        assert same(out["vel" + axis], R.mac_face_vel(u, v, w, size, axis)), axis
    assert same(out["div"], R.mac_vel_div(u, v, w, size))
    if size[0] > 2:   # the large case reaches every branch of the scaling
        assert np.isinf(out["vel"]).any() and (out["vel"] == 0).any()
        assert (np.abs(out["velu"]) < 2.3e-308).any()


def test_infinite_norm_with_infinity():
    dims = (17, 3, 2)
    a = K.array(dims, 141)
    a[20] = -np.inf
    ta, pa = dev(a)
    norm = C.c_double()
    ok(lib().fs3d_infinite_norm(C.byref(arr(pa, dims)), C.byref(norm), None))
    assert norm.value == np.inf == R.infinite_norm(a, dims)


def gpu_interp(g, comp, pts):
    n = np.asarray(pts).reshape(-1, 3).shape[0]
    tp, pp = dev(pts)
    width = 3 if comp == "uvw" else 1
    to, po = dev(np.full(width * n, -1.0))
    ok(lib().fs3d_mac_vel_interp(C.byref(g), fs2d.FS3D_AXES[comp], C.c_void_p(pp), n, C.c_void_p(po), None))
    out = host(to, po, width * n)
    return out.reshape(-1, 3) if width == 3 else out


@pytest.mark.parametrize("size", [(5, 4, 3), (40, 33, 27)])
@pytest.mark.parametrize("comp", ["u", "v", "w", "uvw"])
def test_mac_vel_interp_matches_oracle(size, comp):
    u, v, w = K.mac_fields(size, 111)
    pts = K.points(max(size), 4000, 112)
    g, keep = gpu_mac(u, v, w, size)
    assert same(gpu_interp(g, comp, pts), R.mac_vel_interp(u, v, w, size, comp, pts))


@pytest.mark.parametrize("comp", ["u", "v", "w"])
def test_vel_interp_shifts_match_reference_golden(golden, comp):
    """velInterp's half-cell shifts against the reference's own velInterp on
    a grid of three cubes: the device triCubic of the x/z-exchanged cube at
    the shifted points."""
    n = K.INTERP_CUBE
    pts = np.array(golden["interp_pts"], dtype=np.float64).reshape(-1, 3).copy()
    shift = {"u": (1, 2), "v": (2, 0), "w": (0, 1)}[comp]
    for ax in shift:
        pts[:, ax] -= 0.5
    got = gpu_tricubic(oracle3d.swap_xz(golden[f"interp_{comp}"], (n, n, n)), (n, n, n), pts)
    assert same(got, golden[f"interp_{comp}_out"])
    assert same(golden["interp_uvw_out"][:, "uvw".index(comp)], golden[f"interp_{comp}_out"])


# ---- streams and refusals ----

def test_work_runs_on_the_given_stream():
    dims = (64, 32, 16)
    a, b = K.array(dims, 121), K.array(dims, 122)
    ta, pa = dev(a)
    tb, pb = dev(b)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    ok(lib().fs3d_add(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), C.c_void_p(s.cuda_stream)))
    dot = C.c_double()
    ok(lib().fs3d_inner_product(C.byref(arr(pa, dims)), C.byref(arr(pb, dims)), C.byref(dot),
                                C.c_void_p(s.cuda_stream)))
    s.synchronize()
    summed = R.add(a, b, dims)
    assert same(host(ta, pa, a.size), summed)
    assert abs(dot.value - R.inner_product(summed, b, dims)) <= 2.0 * a.size * U53 * np.abs(summed * b).sum()


def test_host_pointers_are_refused():
    dims = (4, 4, 4)
    h = np.zeros(64)
    td, pd = dev(h)
    INVALID = 1
    assert lib().fs3d_add(C.byref(arr(h.ctypes.data, dims)), C.byref(arr(pd, dims)), None) == INVALID
    assert "not device memory" in lib().fs2d_last_error().decode()
    pts = np.zeros(3)
    out = np.zeros(1)
    assert lib().fs3d_tricubic(C.byref(arr(pd, dims)), C.c_void_p(pts.ctypes.data), 1, C.c_void_p(out.ctypes.data),
                               None) == INVALID
    # the device is still usable after the refusals
    ok(lib().fs3d_add(C.byref(arr(pd, dims)), C.byref(arr(pd, dims)), None))
    torch.cuda.synchronize()
