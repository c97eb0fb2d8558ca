"""CPU oracle for the scar-map generator -- TEST INFRASTRUCTURE ONLY.

A NumPy/SciPy restatement of ``deepx/utils_scars.py:64-426`` (``random_diffusivity_scar`` and
the functions it calls), used by the tests as the checker of ``cardiax_gb300.scars``.  Nothing
on the product path imports it.

The reference draws its random numbers from JAX's PRNG; here the draws are an explicit
:class:`Draws` record consumed in the reference's order (centroid-polygon normals, the number
of blobs, the first centroid index, one normal vector per blob, the two uniforms of the global
centroid, the blur normal).  Everything downstream follows the reference operation by
operation with JAX's single-precision typing (x64 off):

* ``makePolyAndSplineCurve`` (utils_scars.py:100-125) -> :func:`poly_and_spline`: float32
  polygon, SciPy ``splprep(s=0)`` / ``splev`` at float32 parameters (the reference calls SciPy
  itself, so this part is the reference's own library);
* ``CreateSplineCentroids`` (:224-243) -> :func:`spline_centroids`;
* ``MakeAndSumCompositeBlob`` (:246-395, ``ADD_GAP`` off as in ``def_params``) ->
  :func:`composite_mask`: blob outlines in float64, shifted and scaled by float32 factors,
  clipped to the canvas in float32 (``jnp.clip`` of a float64 NumPy array yields float32), filled
  with skimage.draw.polygon's crossing test and summed/clipped at 1;
* ``makegauss2D`` (:64-76) -> :func:`gauss2d`: float32 weights, entries below eps * max zeroed;
* ``blur_scar`` (:402-406) -> :func:`blur_same`: ``convolve2d(..., "same")`` in float64,
  rounded to float32;
* ``random_diffusivity_scar`` (:409-426) -> :func:`diffusivity_scar`.

skimage.draw.polygon (skimage is not installed here) is restated by :func:`polygon_fill`: the
bounding box of the vertices, each cell tested with W. R. Franklin's PNPOLY crossing rule in
float64.  Pinned against the reference's own ``utils_scars.py`` run under a NumPy stand-in for
JAX (``tests/golden/make_scar_golden.py``); the stand-in uses the same PNPOLY restatement for
skimage and SciPy's convolution for JAX's, so those two third-party pieces are restatements
whose parity with skimage/JAX themselves is unpinned.
"""
from __future__ import annotations

from typing import NamedTuple, Sequence, Tuple

import numpy as np
from scipy import interpolate
from scipy.signal import convolve2d

F32 = np.float32

# deepx/utils_scars.py:45-55 def_params (the values random_diffusivity_scar uses)
R0_CENTROID, PROTRUDE_CENTROID = 1.5, 0.2
R0_BLOB, PROTRUDE_BLOB = 1, 0.2
SCAR_SCALE = 0.4


class Draws(NamedTuple):
    centroid_normals: np.ndarray  # (12,) float32
    n_blobs: int                  # in [3, 7)
    first: int                    # in [0, 12)
    blob_normals: np.ndarray      # (n_blobs, 11) float32
    ux: float                     # float32 in [0, 1)
    uy: float
    sigma_normal: float           # float32


def draws_from(rng: np.random.Generator) -> Draws:
    c = rng.standard_normal(12).astype(F32)
    n = int(rng.integers(3, 7))
    first = int(rng.integers(0, 12))
    blobs = rng.standard_normal((n, 11)).astype(F32)
    ux, uy = F32(rng.random()), F32(rng.random())
    return Draws(c, n, first, blobs, ux, uy, F32(rng.standard_normal()))


def poly_and_spline(normals, r0, protrude, ngon=11, nspline=100):
    """utils_scars.py:100-125: ((Px, Py) float32, [sx, sy] float64 spline samples)."""
    max_perturb = protrude * r0
    step = 1 / (ngon - 1)
    t = np.arange(0, 1 + step, step, dtype=F32)
    rpert = (np.asarray(normals, F32) + F32(0.5)) * (F32(0.6) * F32(0.6))
    rdash = (F32(max_perturb) * rpert + F32(r0)).astype(F32)
    ang = F32(2 * np.pi) * t
    Px = (rdash * np.sin(ang)).astype(F32)
    Py = (rdash * np.cos(ang)).astype(F32)
    Px[-1], Py[-1] = Px[0], Py[0]
    tck, _ = interpolate.splprep([Px, Py], s=0)
    du = 1 / nspline
    unew = np.arange(0, 1 + du, du, dtype=F32)
    sx, sy = interpolate.splev(unew, tck)
    return (Px, Py), [np.asarray(sx, np.float64), np.asarray(sy, np.float64)]


def spline_centroids(d: Draws):
    """utils_scars.py:224-243: the blob centres, float32."""
    (Px, Py), _ = poly_and_spline(d.centroid_normals, R0_CENTROID, PROTRUDE_CENTROID, ngon=12)
    m = len(Px)
    sel = np.arange(d.first, d.first + d.n_blobs) % m
    return Px[sel], Py[sel]


def polygon_fill(r, c, shape):
    """skimage.draw.polygon(r, c) restated, then the cells inside ``shape`` kept (JAX drops
    out-of-range scatter indices): a boolean (shape) mask."""
    r = np.asarray(r, np.float64)
    c = np.asarray(c, np.float64)
    H, W = shape
    out = np.zeros(shape, bool)
    if len(r) == 0:
        return out
    r0, r1 = int(max(0.0, r.min())), int(np.ceil(r.max()))
    c0, c1 = int(max(0.0, c.min())), int(np.ceil(c.max()))
    r1, c1 = min(r1, H - 1), min(c1, W - 1)
    if r1 < r0 or c1 < c0:
        return out
    yi, yj = r, np.roll(r, 1)  # edge (i, j = i - 1 cyclically)
    xi, xj = c, np.roll(c, 1)
    for y in range(r0, r1 + 1):
        fy = float(y)
        hit = ((yi <= fy) & (fy < yj)) | ((yj <= fy) & (fy < yi))
        if not hit.any():
            continue
        with np.errstate(divide="ignore", invalid="ignore"):
            xc = (xj[hit] - xi[hit]) * (fy - yi[hit]) / (yj[hit] - yi[hit]) + xi[hit]
        xs = np.arange(c0, c1 + 1, dtype=np.float64)
        odd = ((xs[:, None] < xc[None, :]).sum(axis=1) & 1).astype(bool)
        out[y, c0:c1 + 1] = odd
    return out


def blob_polygons(d: Draws, shape) -> Tuple[list, list]:
    """utils_scars.py:282-356: per blob the (rows, cols) vertices handed to the fill, as the
    float32 values ``jnp.clip`` produces (utils_scars.py:87-94)."""
    cx, cy = spline_centroids(d)
    n = d.n_blobs
    max_ext = R0_CENTROID + PROTRUDE_CENTROID + PROTRUDE_BLOB + R0_BLOB
    double_ext = max_ext * 2
    pts = []
    for i in range(n):
        _, sp = poly_and_spline(d.blob_normals[i], R0_BLOB, PROTRUDE_BLOB)
        sp[0] = sp[0] + np.float64(cx[i])
        sp[1] = sp[1] + np.float64(cy[i])
        pts.append(sp)
    max_field = F32(np.ceil(F32(max_ext / SCAR_SCALE)))
    ratio = shape[0] / shape[1]
    if ratio == 1:
        fx, fy = max_field, max_field
    elif ratio > 1:
        fx, fy = F32(np.ceil(F32(ratio))) * max_field, max_field
    else:
        fx, fy = max_field, F32(np.ceil(F32(ratio))) * max_field
    gc = ((fx - F32(double_ext)) * F32(d.ux) + F32(max_ext),
          (fy - F32(double_ext)) * F32(d.uy) + F32(max_ext))
    fr = (F32(fx / F32(shape[0])), F32(fy / F32(shape[1])))
    rows, cols = [], []
    for sp in pts:
        for j in range(2):
            sp[j] = sp[j] + np.float64(gc[j])
            sp[j] = sp[j] / np.float64(fr[j])
            sp[j] = sp[j] * (sp[j] > 0)
        R = np.clip((shape[1] - sp[1]).astype(F32), 0, shape[1]).astype(F32)
        C = np.clip(sp[0].astype(F32), 0, shape[0]).astype(F32)
        rows.append(R)
        cols.append(C)
    return rows, cols


def composite_mask(d: Draws, shape) -> np.ndarray:
    """The float32 union mask of utils_scars.py:356-380 (binary; the min-max normalisation is
    then the identity)."""
    rows, cols = blob_polygons(d, shape)
    scar = np.zeros(shape, F32)
    for R, C in zip(rows, cols):
        scar += polygon_fill(R, C, shape).astype(F32)
    scar = np.minimum(scar, F32(1.0))
    if not scar.max() > scar.min():
        raise ValueError("degenerate scar (the reference fails here)")
    return scar


def gauss2d(n: int, sigma) -> np.ndarray:
    """utils_scars.py:64-76 in float32."""
    m = (n - 1.0) / 2.0
    a = np.arange(-m, m + 1, dtype=F32)
    y, x = np.meshgrid(a, a)
    s = F32(sigma)
    h = np.exp(-(x * x + y * y) / (F32(2.0) * s * s)).astype(F32)
    h[h < np.finfo(F32).eps * h.max()] = 0
    total = h.sum(dtype=F32)
    if total != 0:
        h = (h / total).astype(F32)
    return h


def blur_same(a, k) -> np.ndarray:
    return convolve2d(np.asarray(a, np.float64), np.asarray(k, np.float64), "same").astype(F32)


def blur_params(d: Draws, shape) -> Tuple[int, np.float32]:
    """utils_scars.py:420-424: kernel size int(0.1 * H) and sigma = normal * H / 10."""
    return int(shape[0] * 0.1), F32(F32(d.sigma_normal) * F32(shape[0])) / F32(10)


def diffusivity_scar(d: Draws, shape: Sequence[int]) -> np.ndarray:
    """utils_scars.py:409-426: 1 - blur(union mask), float32."""
    shape = tuple(int(s) for s in shape)
    K, sigma = blur_params(d, shape)
    return (F32(1) - blur_same(composite_mask(d, shape), gauss2d(K, sigma))).astype(F32)
