"""Checkpoint emission: ``imresize`` of cardiax/io.py:118-124 as a CUDA op, and the data-set
layout that cardiax/io.py:13-78 writes.

``imresize(a, size)`` resizes the last two axes of a device array with the bilinear resampling of
``jax.image.resize`` (what the reference calls), through ``fk_resize_bilinear``.

The reference stores generated sequences in HDF5 (h5py).  h5py is not available to this
package, so :func:`save` writes the same datasets -- ``states`` (t, 3, H, W), ``field``,
``start``, ``duration``, ``period``, ``diffusivity`` and ``params/<name>`` (including
``params/D``, ``params/dt``, ``params/dx``) -- under the same names into a NumPy ``.npz``
archive, and :func:`load` reads them back.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import _native as N
from .tissue import _device, as_cuda_f32, stream_handle


def resize_planes(src: torch.Tensor, H: int, W: int, out: torch.Tensor, antialias: bool = True):
    """Resizes the planes of ``src`` ((P, H, pitch) float32, CUDA, only the first W columns are
    read) into ``out`` ((P, OH, out_pitch) float32, CUDA)."""
    P = int(src.shape[0])
    if out.shape[0] != P:
        raise ValueError("plane counts differ")
    if src.stride(-1) != 1 or out.stride(-1) != 1 or src.stride(0) != src.shape[1] * src.stride(1) \
            or out.stride(0) != out.shape[1] * out.stride(1):
        raise ValueError("planes must be row-major with a uniform pitch")
    N.call("fk_resize_bilinear", src.data_ptr(), P, int(H), int(W), int(src.stride(1)),
           out.data_ptr(), int(out.shape[1]), int(out.shape[2]), int(out.stride(1)),
           int(bool(antialias)), stream_handle())
    return out


def imresize(a, size: Sequence[int], method: str = "bilinear", antialias: bool = True,
             device=None) -> torch.Tensor:
    """``a`` (..., H, W) resized to (..., size[0], size[1]) (cardiax/io.py:118-124)."""
    if method not in ("bilinear", "linear"):
        raise NotImplementedError("only bilinear resizing is implemented")
    dev = a.device if isinstance(a, torch.Tensor) and a.is_cuda else _device(device)
    x = as_cuda_f32(a, dev)
    if x.dim() < 2:
        raise ValueError("imresize needs at least two axes")
    lead = tuple(x.shape[:-2])
    H, W = int(x.shape[-2]), int(x.shape[-1])
    OH, OW = int(size[0]), int(size[1])
    src = x.reshape((-1, H, W)).contiguous()
    out = torch.empty((src.shape[0], OH, OW), dtype=torch.float32, device=dev)
    if src.shape[0]:
        resize_planes(src, H, W, out, antialias)
    return out.reshape(lead + (OH, OW))


def _np(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def save(path: str, states, params, diffusivity, stimuli, dt: float, dx: float,
         shape: Sequence[int] = None) -> str:
    """Writes a generated sequence with the datasets of cardiax/io.py:13-78 (``shape``: the
    stored resolution; fields are resized to it as the reference's ``add_*`` do)."""
    from .params import Params

    d = as_cuda_f32(diffusivity, _device(None))
    fields = [as_cuda_f32(s[1], d.device) for s in stimuli]
    if shape is not None:
        d = imresize(d, shape)
        fields = [imresize(f, shape) for f in fields]
    data = {"states": _np(states), "diffusivity": _np(d),
            "field": np.stack([_np(f) for f in fields]) if fields else np.zeros((0,)),
            "start": np.array([float(s[0][0]) for s in stimuli]),
            "duration": np.array([float(s[0][1]) for s in stimuli]),
            "period": np.array([float(s[0][2]) for s in stimuli]),
            "params/D": _np(d), "params/dt": np.float64(dt), "params/dx": np.float64(dx)}
    for name, value in zip(Params._fields, params):
        data["params/" + name] = np.float64(float(value))
    np.savez(path, **data)
    return path if path.endswith(".npz") else path + ".npz"


def load(path: str) -> dict:
    """The datasets written by :func:`save`, by name."""
    with np.load(path) as f:
        return {k: f[k] for k in f.files}
