"""Scar maps on the CPU: the oracle (oracle/fk_scars.py) pinned to fixtures made by the
reference's own deepx/utils_scars.py (tests/golden/make_scar_golden.py), and the package's host
geometry (outlines, blur width, Gaussian weights) against the oracle, bit for bit."""
import numpy as np
import pytest

import fk_scars as S
from cardiax_gb300 import scars as P


def _cases(golden):
    g = golden("scars.npz")
    for k in range(int(g["n_cases"])):
        p = f"c{k}_"
        shape = tuple(int(x) for x in g[p + "shape"])
        d = S.Draws(g[p + "centroid_normals"], int(g[p + "n_blobs"]), int(g[p + "first"]),
                    g[p + "blob_normals"], g[p + "ux"][()], g[p + "uy"][()],
                    g[p + "sigma_normal"][()])
        mask = np.unpackbits(g[p + "mask"])[:shape[0] * shape[1]].reshape(shape)
        yield shape, d, mask, g[p + "field"], int(g[p + "ksize"]), g[p + "sigma"]


def test_oracle_matches_the_reference_code(golden):
    n = 0
    for shape, d, mask, field, K, sigma in _cases(golden):
        assert np.array_equal(S.composite_mask(d, shape), mask.astype(np.float32)), shape
        k2, s2 = S.blur_params(d, shape)
        assert k2 == K and np.float32(s2) == sigma[0]
        assert np.array_equal(S.diffusivity_scar(d, shape), field), shape
        n += 1
    assert n == 7


def test_narrow_blur_case_zeroes_far_weights(golden):
    kinds = [(S.gauss2d(K, sigma[0]) == 0).sum() for _, _, _, _, K, sigma in _cases(golden)]
    assert kinds[-1] > 0 and all(k == 0 for k in kinds[:-1])


def test_host_geometry_matches_oracle(golden):
    for shape, d, _, _, _, _ in _cases(golden):
        pd = P.ScarDraws(*d)
        rows, cols = P.outlines(pd, shape)
        orows, ocols = S.blob_polygons(d, shape)
        assert len(rows) == d.n_blobs
        for a, b in zip(rows + cols, orows + ocols):
            assert a.dtype == np.float32 and np.array_equal(a, b)
        K, sigma = P.blur_width(pd, shape)
        assert (K, sigma) == S.blur_params(d, shape)
        assert np.array_equal(P.gaussian_weights(K, sigma), S.gauss2d(K, sigma))


def test_draws_follow_the_reference_order():
    a = P.draw(np.random.default_rng(5))
    b = S.draws_from(np.random.default_rng(5))
    assert a.n_blobs == b.n_blobs and a.first == b.first
    for x, y in zip(a, b):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    assert 3 <= a.n_blobs < 7 and 0 <= a.first < 12
    assert a.blob_normals.shape == (a.n_blobs, 11)
    assert all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(P.draw(7), P.draw(7)))


@pytest.mark.parametrize("shape", [(200, 200), (300, 240)])
def test_polygon_fill_is_pnpoly(shape):
    """The oracle's vectorised fill against a direct per-cell PNPOLY on random polygons."""
    rng = np.random.default_rng(sum(shape))
    for _ in range(3):
        n = int(rng.integers(3, 40))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(10, 60, n)
        r = (shape[0] / 2 + rad * np.sin(ang)).astype(np.float32)
        c = (shape[1] / 2 + rad * np.cos(ang)).astype(np.float32)
        got = S.polygon_fill(r, c, shape)
        want = np.zeros(shape, bool)
        yp, xp = r.astype(np.float64), c.astype(np.float64)
        for y in range(int(yp.min()) - 1, int(np.ceil(yp.max())) + 2):
            for x in range(int(xp.min()) - 1, int(np.ceil(xp.max())) + 2):
                inside, j = False, n - 1
                for i in range(n):
                    if ((yp[i] <= y < yp[j]) or (yp[j] <= y < yp[i])) and \
                            x < (xp[j] - xp[i]) * (y - yp[i]) / (yp[j] - yp[i]) + xp[i]:
                        inside = not inside
                    j = i
                if 0 <= y < shape[0] and 0 <= x < shape[1]:
                    want[y, x] = inside
        assert np.array_equal(got, want)
