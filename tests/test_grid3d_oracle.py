"""The restatement of the reference's 3D containers (oracle/restate/
fs3d_oracle.c) against the reference's own include/Array3D.h and
include/MACGrid3D.h: live against the compiled headers where the reference
checkout exists (oracle/_ref/libfs3d_ref.so), and always against the golden
vectors that build made (tests/golden/grid3d.npz).  Bit for bit, on inputs
where the reference's literal code stays inside its arrays:

* operator+= and innerProduct with row 0 of every slab k >= 1 of the second
  operand zero (the reference visits those rows twice), setMultiplyAdd and
  infiniteNorm on any input (a second visit changes nothing);
* triCubic and velInterp on cubes, the restatement on the array with x and z
  exchanged (the reference reads element (z, y, x));
* vel, velU, velV, velW and velDiv on MAC grids of any size.

Two further tests record how the literal code differs where it is not
followed: the double visit of the aliased rows, and triCubic's swapped axes.
"""
import os

import numpy as np
import pytest

import grid3d_cases as K
import oracle3d

R = oracle3d.restated
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grid3d.npz")


def same(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def ref():
    r = oracle3d.reference()
    if r is None:
        pytest.skip("reference 3D containers not built here")
    return r


# ---- against the golden vectors (every machine) ----

@pytest.mark.parametrize("d", range(len(K.ARRAY_DIMS)))
def test_array_ops_match_golden(golden, d):
    dims = K.ARRAY_DIMS[d]
    a, b, bz = golden[f"arr{d}_a"], golden[f"arr{d}_b"], golden[f"arr{d}_bz"]
    assert same(R.add(a, bz, dims), golden[f"arr{d}_add"])
    assert same(R.set_multiply_add(a, K.SCALE, b, dims), golden[f"arr{d}_sma"])
    assert same(R.inner_product(a, bz, dims), golden[f"arr{d}_dot"])
    assert same(R.infinite_norm(a, dims), golden[f"arr{d}_norm"])


@pytest.mark.parametrize("n", K.CUBES)
def test_tricubic_matches_golden_on_swapped_cube(golden, n):
    data, pts = golden[f"cube{n}_data"], golden[f"cube{n}_pts"]
    got = R.tricubic(oracle3d.swap_xz(data, (n, n, n)), (n, n, n), pts)
    assert same(got, golden[f"cube{n}_tricubic"])
    # the clamp to zero and the outside rule are exercised
    assert (got == 0).sum() > 10 and (got > 0).sum() > 10


@pytest.mark.parametrize("m", range(len(K.MAC_SIZES)))
def test_mac_stencils_match_golden(golden, m):
    size = K.MAC_SIZES[m]
    u, v, w = golden[f"mac{m}_u"], golden[f"mac{m}_v"], golden[f"mac{m}_w"]
    assert same(R.mac_vel(u, v, w, size), golden[f"mac{m}_vel"])
    for axis in ("u", "v", "w"):
        assert same(R.mac_face_vel(u, v, w, size, axis), golden[f"mac{m}_vel{axis}"]), axis
    assert same(R.mac_vel_div(u, v, w, size), golden[f"mac{m}_div"])


def shifted(pts, comp):
    """velInterpU/V/W's half-cell shifts (include/MACGrid3D.h:143-159)."""
    p = np.array(pts, dtype=np.float64).reshape(-1, 3).copy()
    if comp == "u":
        p[:, 1] -= 0.5
        p[:, 2] -= 0.5
    elif comp == "v":
        p[:, 2] -= 0.5
        p[:, 0] -= 0.5
    else:
        p[:, 0] -= 0.5
        p[:, 1] -= 0.5
    return p


def interp_cubes_restated(u, v, w, n, comp, pts):
    dims = (n, n, n)
    f = {"u": u, "v": v, "w": w}
    if comp != "uvw":
        return R.tricubic(oracle3d.swap_xz(f[comp], dims), dims, shifted(pts, comp))
    return np.stack([interp_cubes_restated(u, v, w, n, c, pts) for c in ("u", "v", "w")], axis=1)


@pytest.mark.parametrize("comp", ["u", "v", "w", "uvw"])
def test_vel_interp_shifts_match_golden(golden, comp):
    n = K.INTERP_CUBE
    u, v, w, pts = golden["interp_u"], golden["interp_v"], golden["interp_w"], golden["interp_pts"]
    assert same(interp_cubes_restated(u, v, w, n, comp, pts), golden[f"interp_{comp}_out"])


def test_mac_vel_interp_is_tricubic_of_shifted_points():
    """The restatement's velInterp on a MAC grid samples each face array at
    the shifted point (its own layout, no cube needed)."""
    size = (5, 4, 3)
    u, v, w = K.mac_fields(size, 7)
    pts = K.points(5, 100, 8)
    du, dv, dw = oracle3d.face_dims(*size)
    got = R.mac_vel_interp(u, v, w, size, "uvw", pts)
    assert same(got[:, 0], R.tricubic(u, du, shifted(pts, "u")))
    assert same(got[:, 1], R.tricubic(v, dv, shifted(pts, "v")))
    assert same(got[:, 2], R.tricubic(w, dw, shifted(pts, "w")))
    for c, col in (("u", 0), ("v", 1), ("w", 2)):
        assert same(R.mac_vel_interp(u, v, w, size, c, pts), got[:, col])


# ---- live against the compiled reference headers ----

@pytest.mark.parametrize("dims", K.ARRAY_DIMS + [(3, 8, 2), (9, 2, 4)])
def test_array_ops_match_reference(ref, dims):
    a, b = K.array(dims, 1), K.array(dims, 2)
    bz = K.zero_aliased_rows(b, dims)
    assert same(R.add(a, bz, dims), ref.add(a, bz, dims))
    assert same(R.set_multiply_add(a, -1.75, b, dims), ref.set_multiply_add(a, -1.75, b, dims))
    assert same(R.inner_product(a, bz, dims), ref.inner_product(a, bz, dims))
    assert same(R.infinite_norm(a, dims), ref.infinite_norm(a, dims))


def test_infinite_norm_takes_the_double_absolute_value(ref):
    """The reference's `abs` resolves to the double overload: fractions are
    not truncated, negative values count by magnitude."""
    a = np.array([0.25, -0.75, 0.5, -0.125])
    assert ref.infinite_norm(a, (4, 1, 1)) == 0.75 == R.infinite_norm(a, (4, 1, 1))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8])
def test_tricubic_matches_reference_on_swapped_cube(ref, n):
    data = K.array((n, n, n), 100 + n)
    pts = K.points(n, 300, 200 + n)
    assert same(R.tricubic(oracle3d.swap_xz(data, (n, n, n)), (n, n, n), pts), ref.tricubic(data, (n, n, n), pts))


@pytest.mark.parametrize("size", K.MAC_SIZES + [(2, 7, 3), (8, 1, 5)])
def test_mac_stencils_match_reference(ref, size):
    u, v, w = K.mac_fields(size, 300)
    assert same(R.mac_vel(u, v, w, size), ref.mac_vel(u, v, w, size))
    for axis in ("u", "v", "w"):
        assert same(R.mac_face_vel(u, v, w, size, axis), ref.mac_face_vel(u, v, w, size, axis)), axis
    assert same(R.mac_vel_div(u, v, w, size), ref.mac_vel_div(u, v, w, size))


@pytest.mark.parametrize("comp", ["u", "v", "w", "uvw"])
def test_vel_interp_matches_reference_on_cubes(ref, comp):
    n = 5
    u, v, w = K.cube_fields(n, 400)
    pts = K.points(n, 300, 401)
    assert same(interp_cubes_restated(u, v, w, n, comp, pts), ref.mac_vel_interp_cubes(u, v, w, n, comp, pts))


def test_literal_loops_visit_aliased_rows_twice(ref):
    """Where the second operand's aliased rows are not zero, the reference
    adds them twice (as row NY of slab k-1 and as row 0 of slab k); the
    restatement adds every element once.  Everything else agrees."""
    dims = (4, 3, 3)
    a, b = K.array(dims, 5), K.array(dims, 6)
    lit, once = ref.add(a, b, dims).reshape(3, 3, 4), R.add(a, b, dims).reshape(3, 3, 4)
    b3 = b.reshape(3, 3, 4)
    assert same(lit[1:, 0, :], (a.reshape(3, 3, 4)[1:, 0, :] + b3[1:, 0, :]) + b3[1:, 0, :])
    assert same(lit[:, 1:, :], once[:, 1:, :]) and same(lit[0], once[0])


def test_literal_tricubic_swaps_x_and_z(ref):
    """On a cube that is not symmetric in x and z the reference's read of
    (z, y, x) gives another value than the restatement on the same array."""
    n = 4
    data = K.array((n, n, n), 9)
    pts = np.array([[1.3, 1.7, 2.2], [2.6, 0.4, 1.1]])
    lit = ref.tricubic(data, (n, n, n), pts)
    assert not same(lit, R.tricubic(data, (n, n, n), pts))
    assert same(lit, R.tricubic(oracle3d.swap_xz(data, (n, n, n)), (n, n, n), pts))
