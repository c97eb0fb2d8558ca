"""GPU: scar maps (deepx/utils_scars.py:409-426) -- the polygon fill bit for bit against the
reference's own mask (tests/golden/scars.npz) and the oracle, the blur against SciPy.

Tolerance of the blur: the kernel accumulates the K*K products in float32, one rounding of at
most 2^-24 * |partial sum| each, against a float64 sum rounded once, so
|gpu - reference| <= (K*K + 2) * 2^-24 * sum|k| * max|a|."""
import numpy as np
import pytest
import torch
from scipy.signal import convolve2d

import fk_scars as S

pytestmark = pytest.mark.gpu


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _tol(K, k, a):
    return (K * K + 2) * 2.0 ** -24 * float(np.abs(k).sum()) * float(np.abs(a).max())


def _cases(golden):
    from cardiax_gb300 import scars as P
    g = golden("scars.npz")
    for k in range(int(g["n_cases"])):
        p = f"c{k}_"
        shape = tuple(int(x) for x in g[p + "shape"])
        d = P.ScarDraws(g[p + "centroid_normals"], int(g[p + "n_blobs"]), int(g[p + "first"]),
                        g[p + "blob_normals"], g[p + "ux"][()], g[p + "uy"][()],
                        g[p + "sigma_normal"][()])
        mask = np.unpackbits(g[p + "mask"])[:shape[0] * shape[1]].reshape(shape)
        yield shape, d, mask, g[p + "field"]


def test_raster_matches_reference_mask(golden):
    _gpu()
    from cardiax_gb300 import scars as P
    for shape, d, mask, _ in _cases(golden):
        rows, cols = P.outlines(d, shape)
        got, count = P.rasterize(rows, cols, shape)
        assert np.array_equal(got.cpu().numpy(), mask.astype(np.float32)), shape
        assert count == int(mask.sum())


def test_scar_field_matches_reference(golden):
    _gpu()
    from cardiax_gb300 import scars as P
    for shape, d, _, field in _cases(golden):
        got = P.random_diffusivity_scar(d, shape).cpu().numpy()
        K, sigma = P.blur_width(d, shape)
        w = P.gaussian_weights(K, sigma)
        assert got.shape == shape and got.dtype == np.float32
        assert np.abs(got - field).max() <= _tol(K, w, np.ones(1)), shape


@pytest.mark.parametrize("H,W,K", [(H, W, K) for H, W in [(17, 23), (64, 64), (40, 100), (3, 5),
                                                          (130, 70)]
                                   for K in [1, 2, 5, 8, 25, 41]]
                         + [(20, 30, 520), (70, 66, 512)])
def test_conv2d_same_matches_scipy(H, W, K):
    """The tiled kernel (K <= 512) and the per-output fallback (K > 512)."""
    _gpu()
    from cardiax_gb300 import scars as P
    rng = np.random.default_rng(H * 1000 + W * 10 + K)
    a = rng.standard_normal((H, W)).astype(np.float32)
    k = rng.random((K, K)).astype(np.float32)
    ref = convolve2d(a.astype(np.float64), k.astype(np.float64), "same")
    got = P.blur_same(torch.as_tensor(a).cuda(), k).cpu().numpy()
    assert np.abs(got - ref).max() <= _tol(K, k, a)
    got1 = P.blur_same(torch.as_tensor(a).cuda(), k, one_minus=True).cpu().numpy()
    assert np.abs(got1 - (1.0 - ref)).max() <= _tol(K, k, a) + 2.0 ** -23 * (1 + np.abs(ref).max())


def test_large_scar_at_the_reference_default_size():
    """1200 x 1200 (utils_scars.py:49 RequiredImageSize): the fill bit for bit against the
    oracle, the blur (K = 120) on sampled cells against float64 sums."""
    _gpu()
    from cardiax_gb300 import scars as P
    shape = (1200, 1200)
    d = P.draw(np.random.default_rng(11))
    rows, cols = P.outlines(d, shape)
    mask, count = P.rasterize(rows, cols, shape)
    want = S.composite_mask(S.Draws(*d), shape)
    m = mask.cpu().numpy()
    assert np.array_equal(m, want) and count == int(want.sum())
    K, sigma = P.blur_width(d, shape)
    w = P.gaussian_weights(K, sigma).astype(np.float64)
    field = P.random_diffusivity_scar(d, shape).cpu().numpy()
    rng = np.random.default_rng(3)
    s = (K - 1) // 2
    pad = np.pad(want.astype(np.float64), K)
    edge = np.argwhere((want > 0) & (np.roll(want, 1, 0) == 0))
    picks = np.concatenate([rng.integers(0, 1200, (48, 2)), edge[rng.integers(0, len(edge), 16)]])
    for i, j in picks:
        win = pad[i + s - (K - 1) + K:i + s + 1 + K, j + s - (K - 1) + K:j + s + 1 + K]
        ref = 1.0 - float((win[::-1, ::-1] * w).sum())
        assert abs(field[i, j] - ref) <= _tol(K, w, np.ones(1)) + 2.0 ** -23, (i, j)


def test_degenerate_union_gives_the_centre_cell(monkeypatch):
    _gpu()
    from cardiax_gb300 import scars as P
    d = P.draw(np.random.default_rng(2))
    empty = np.zeros(5, np.float32)
    monkeypatch.setattr(P, "outlines", lambda d, shape: ([empty], [empty]))
    shape = (64, 48)
    got = P.random_diffusivity_scar(d, shape).cpu().numpy()
    K, sigma = P.blur_width(d, shape)
    delta = np.zeros(shape)
    delta[32, 24] = 1.0
    ref = 1.0 - convolve2d(delta, P.gaussian_weights(K, sigma).astype(np.float64), "same")
    assert np.abs(got - ref).max() <= 1e-6


def test_random_diffusivity_spans_the_domain():
    _gpu()
    from cardiax_gb300 import generate
    D = generate.random_diffusivity(4, (256, 256), domain=(0.0001, 0.001)).cpu().numpy()
    assert D.shape == (256, 256)
    assert abs(D.min() - 0.0001) <= 1e-9 and abs(D.max() - 0.001) <= 1e-8


def test_argument_errors():
    _gpu()
    from cardiax_gb300 import _native as N
    from cardiax_gb300 import scars as P
    with pytest.raises(ValueError):
        P.random_diffusivity_scar(1, (9, 64))
    tri = [np.array([1, 5, 1], np.float32)] * 17
    with pytest.raises(N.FkError):
        P.rasterize(tri, tri, (16, 16))
    with pytest.raises(N.FkError):
        P.rasterize([np.array([1, 5], np.float32)], [np.array([1, 5], np.float32)], (16, 16))
    x = torch.zeros((8, 8), device="cuda")
    k = torch.ones((3, 3), device="cuda")
    with pytest.raises(N.FkError):
        N.call("fk_conv2d_same", x.data_ptr(), 8, 8, 8, k.data_ptr(), 3, x.data_ptr(), 8, 0,
               None)
