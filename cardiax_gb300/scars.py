"""Scar maps for the diffusivity field: ``random_diffusivity_scar`` of
deepx/utils_scars.py:409-426, with the field-sized work on the GPU.

The reference builds a scar as the union of 3-6 filled blobs -- closed cubic splines through
randomly perturbed polygons, placed along a section of a larger perturbed spline -- then tapers
its edge with a Gaussian blur and returns ``1 - blurred``.  Here the blob outlines (a few hundred
points: SciPy's ``splprep``/``splev``, the library the reference calls) are computed on the
host in the reference's arithmetic; the fill (``fk_scar_raster``: PNPOLY's crossing test per
cell, as skimage.draw.polygon does) and the blur (``fk_conv2d_same``: SciPy's "same"
convolution, fused with ``1 - x``) run as CUDA kernels.

Random draws: the reference uses JAX's PRNG, which is not available to this package.  The draws
are a :class:`ScarDraws` record -- given explicitly, or taken from a NumPy ``Generator`` (or an
integer seed) in the reference's order: 12 normals for the centroid polygon, the blob count in
[3, 7), the first centroid index in [0, 12), 11 normals per blob, two uniforms for the global
centroid, one normal for the blur width.

When the union is empty or covers the whole grid the reference's normalisation writes one
cell of an immutable JAX array and fails; here that case yields the evident intent, a single
set cell at the centre.
"""
from __future__ import annotations

from typing import List, NamedTuple, Sequence, Tuple, Union

import numpy as np
import torch

from . import _native as N
from .tissue import _device, stream_handle

_F32 = np.float32

# deepx/utils_scars.py:45-55 (the defaults random_diffusivity_scar runs with)
R0_CENTROID = 1.5
PROTRUDE_CENTROID = 0.2
R0_BLOB = 1
PROTRUDE_BLOB = 0.2
SCAR_SCALE = 0.4
NGON_CENTROID, NGON_BLOB, SPLINE_POINTS = 12, 11, 100


class ScarDraws(NamedTuple):
    centroid_normals: np.ndarray  # (12,) standard normals
    n_blobs: int                  # 3..6
    first: int                    # 0..11, the first centroid index
    blob_normals: np.ndarray      # (n_blobs, 11) standard normals
    ux: float                     # uniforms in [0, 1) placing the scar
    uy: float
    sigma_normal: float           # standard normal scaling the blur width


def draw(rng: Union[int, np.random.Generator]) -> ScarDraws:
    """The random draws of one scar, in the reference's order (utils_scars.py:224-243,
    246-352, 420-424)."""
    g = np.random.default_rng(rng) if not isinstance(rng, np.random.Generator) else rng
    centroid = g.standard_normal(NGON_CENTROID).astype(_F32)
    n = int(g.integers(3, 7))
    first = int(g.integers(0, NGON_CENTROID))
    blobs = g.standard_normal((n, NGON_BLOB)).astype(_F32)
    ux, uy = _F32(g.random()), _F32(g.random())
    return ScarDraws(centroid, n, first, blobs, ux, uy, _F32(g.standard_normal()))


def _closed_spline(normals, r0: float, protrude: float, ngon: int):
    """makePolyAndSplineCurve (utils_scars.py:100-125): the float32 polygon with radii
    r0 + protrude * r0 * 0.36 * (normal + 0.5) and the float64 samples of the interpolating
    cubic spline through it at 101 float32 parameters."""
    from scipy import interpolate

    step = 1 / (ngon - 1)
    t = np.arange(0, 1 + step, step, dtype=_F32)
    radius = _F32(r0) + _F32(protrude * r0) * ((np.asarray(normals, _F32) + _F32(0.5))
                                               * (_F32(0.6) * _F32(0.6)))
    angle = _F32(2 * np.pi) * t
    px, py = radius * np.sin(angle), radius * np.cos(angle)
    px[-1], py[-1] = px[0], py[0]
    tck, _ = interpolate.splprep([px, py], s=0)
    u = np.arange(0, 1 + 1 / SPLINE_POINTS, 1 / SPLINE_POINTS, dtype=_F32)
    sx, sy = interpolate.splev(u, tck)
    return (px, py), np.stack([np.asarray(sx, np.float64), np.asarray(sy, np.float64)])


def outlines(d: ScarDraws, shape: Sequence[int]) -> Tuple[List[np.ndarray], List[np.ndarray]]:
    """Per blob the (rows, columns) vertices of its filled outline on the H x W canvas
    (utils_scars.py:224-356 and 79-94): float32 values, as the reference's ``jnp.clip`` leaves
    them."""
    H, W = int(shape[0]), int(shape[1])
    (cx, cy), _ = _closed_spline(d.centroid_normals, R0_CENTROID, PROTRUDE_CENTROID,
                                 NGON_CENTROID)
    pick = np.arange(d.first, d.first + d.n_blobs) % len(cx)
    centres = np.stack([cx[pick], cy[pick]]).astype(np.float64)  # (2, n)
    reach = R0_CENTROID + PROTRUDE_CENTROID + PROTRUDE_BLOB + R0_BLOB
    field = _F32(np.ceil(_F32(reach / SCAR_SCALE)))
    ratio = H / W
    widen = _F32(np.ceil(_F32(ratio)))
    fx = widen * field if ratio > 1 else field
    fy = widen * field if ratio < 1 else field
    origin = np.array([(fx - _F32(2 * reach)) * _F32(d.ux) + _F32(reach),
                       (fy - _F32(2 * reach)) * _F32(d.uy) + _F32(reach)], np.float64)
    scale = np.array([fx / _F32(H), fy / _F32(W)], np.float64)
    rows, cols = [], []
    for b in range(d.n_blobs):
        _, pts = _closed_spline(d.blob_normals[b], R0_BLOB, PROTRUDE_BLOB, NGON_BLOB)
        pts = pts + centres[:, b:b + 1]
        pts = (pts + origin[:, None]) / scale[:, None]
        pts = pts * (pts > 0)
        rows.append(np.clip((W - pts[1]).astype(_F32), 0, W))
        cols.append(np.clip(pts[0].astype(_F32), 0, H))
    return rows, cols


def blur_width(d: ScarDraws, shape: Sequence[int]) -> Tuple[int, np.float32]:
    """Kernel size int(0.1 * H) and width sigma = normal * H / 10 (utils_scars.py:420-424)."""
    H = int(shape[0])
    return int(H * 0.1), (_F32(d.sigma_normal) * _F32(H)) / _F32(10)


def gaussian_weights(size: int, sigma) -> np.ndarray:
    """makegauss2D (utils_scars.py:64-76): exp(-(x^2 + y^2) / (2 sigma^2)) on a size x size
    grid centred on 0, entries below eps * max set to 0, normalised to sum 1; float32."""
    half = (size - 1.0) / 2.0
    axis = np.arange(-half, half + 1, dtype=_F32)
    gy, gx = np.meshgrid(axis, axis)
    s = _F32(sigma)
    w = np.exp(-(gx * gx + gy * gy) / (_F32(2.0) * s * s)).astype(_F32)
    w[w < np.finfo(_F32).eps * w.max()] = 0
    total = w.sum(dtype=_F32)
    return (w / total).astype(_F32) if total != 0 else w


def rasterize(rows: Sequence[np.ndarray], cols: Sequence[np.ndarray], shape: Sequence[int],
              device=None) -> Tuple[torch.Tensor, int]:
    """The union of the filled polygons as an (H, W) float32 0/1 device plane, and the number
    of set cells (``fk_scar_raster``)."""
    dev = _device(device)
    H, W = int(shape[0]), int(shape[1])
    offsets = np.zeros(len(rows) + 1, np.int32)
    offsets[1:] = np.cumsum([len(r) for r in rows])
    ys = torch.as_tensor(np.concatenate(rows).astype(np.float64) if rows else np.zeros(1),
                         device=dev)
    xs = torch.as_tensor(np.concatenate(cols).astype(np.float64) if cols else np.zeros(1),
                         device=dev)
    out = torch.empty((H, W), dtype=torch.float32, device=dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    N.call("fk_scar_raster", xs.data_ptr(), ys.data_ptr(), offsets.ctypes.data, len(rows), H, W,
           out.data_ptr(), W, count.data_ptr(), stream_handle())
    return out, int(count.item())


def blur_same(plane: torch.Tensor, weights: np.ndarray, one_minus: bool = False) -> torch.Tensor:
    """scipy.signal.convolve2d(plane, weights, "same") in float32 (``fk_conv2d_same``), or
    1 minus it."""
    H, W = int(plane.shape[0]), int(plane.shape[1])
    K = int(weights.shape[0])
    if weights.shape != (K, K):
        raise ValueError("the weights must be square")
    src = plane.to(torch.float32).contiguous()
    k = torch.as_tensor(np.ascontiguousarray(weights, _F32), device=src.device)
    out = torch.empty((H, W), dtype=torch.float32, device=src.device)
    N.call("fk_conv2d_same", src.data_ptr(), H, W, W, k.data_ptr(), K, out.data_ptr(), W,
           int(bool(one_minus)), stream_handle())
    return out


def random_diffusivity_scar(rng, shape: Sequence[int], device=None) -> torch.Tensor:
    """``1 - blur(scar)`` on an H x W grid (deepx/utils_scars.py:409-426): 1 in healthy tissue,
    tapering to 0 inside the scar; an (H, W) float32 device tensor.  ``rng``: a
    :class:`ScarDraws`, a NumPy ``Generator`` or an integer seed."""
    H, W = int(shape[0]), int(shape[1])
    K = int(H * 0.1)
    if K < 1 or W < 1:
        raise ValueError("the blur needs H >= 10 (its kernel has int(0.1 * H) taps)")
    d = rng if isinstance(rng, ScarDraws) else draw(rng)
    K, sigma = blur_width(d, (H, W))
    if sigma == 0:
        raise ValueError("a blur of width 0")
    rows, cols = outlines(d, (H, W))
    mask, count = rasterize(rows, cols, (H, W), device)
    if count == 0 or count == H * W:
        mask.zero_()
        mask[H // 2, W // 2] = 1.0
    return blur_same(mask, gaussian_weights(K, sigma), one_minus=True)
