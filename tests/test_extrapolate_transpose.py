"""The transposed extrapolation used by the adjoint kernels (k_extrap_adjoint,
E^T applied layer by layer, deepest first: each face of layer L hands its
adjoint in equal parts to its neighbours of lower layer and drops its own),
restated in numpy and checked on the CPU against the oracle's
Array2D::extrapolate (include/Array2D.h:552-591) by the dot-product identity
<E x, y> = <x, E^T y>, for random masks, with and without a band limit."""
import numpy as np
import pytest

import oracle_py as O


def extrap_transpose(y, layers, W, H, band=0):
    mu = y.astype(np.float64).copy().reshape(H, W)
    lay = layers.reshape(H, W).astype(np.int64)
    unknown = np.uint32(0xFFFFFFFF)
    finite = layers != unknown
    maxL = int(layers[finite].max()) if finite.any() else 0
    if band > 0:
        maxL = min(maxL, band)
    for L in range(maxL, 0, -1):
        js, is_ = np.nonzero(lay == L)
        for j, i in zip(js, is_):
            nb = [(i - 1, j), (i + 1, j), (i, j - 1), (i, j + 1)]
            low = [(a, b) for a, b in nb if 0 <= a < W and 0 <= b < H and lay[b, a] < L]
            m = mu[j, i]
            mu[j, i] = 0.0
            for a, b in low:
                mu[b, a] += m / len(low)
    return mu.reshape(-1)


@pytest.mark.parametrize("W,H,frac,band,seed", [(17, 13, 0.3, 0, 1), (24, 24, 0.05, 0, 2), (30, 11, 0.5, 0, 3),
                                                 (20, 20, 0.08, 3, 4), (16, 16, 0.0, 0, 5)])
def test_extrapolation_transpose_dot_product(W, H, frac, band, seed):
    rng = np.random.default_rng(seed)
    known = rng.random(W * H) < frac
    if frac > 0 and not known.any():
        known[0] = True
    mask = np.where(known, 0, 0xFFFFFFFF).astype(np.uint32)
    x = rng.standard_normal(W * H)
    Ex, layers = O.extrapolate(x, mask, W, H, band)
    y = rng.standard_normal(W * H)
    # E is linear in the values; known faces, unreached faces (no known face)
    # and faces beyond the band keep their value, and E^T passes their
    # adjoint through
    Ety = extrap_transpose(y, layers, W, H, band)
    lhs = Ex @ y
    rhs = x @ Ety
    assert abs(lhs - rhs) <= 1e-12 * (np.abs(Ex * y).sum() + 1.0), (lhs, rhs)
