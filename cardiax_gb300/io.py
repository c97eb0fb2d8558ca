"""Checkpoint storage and emission: the HDF5 data set of cardiax/io.py:13-115 and ``imresize``
of cardiax/io.py:118-124 as a CUDA op.

``init`` / ``add_params`` / ``add_diffusivity`` / ``add_stimuli`` / ``add_state`` /
``add_states`` / ``load`` / ``load_state`` / ``load_stimuli`` / ``load_params`` /
``load_diffusivity`` keep the reference's names, arguments and dataset layout: ``states``
(t, 3, H, W) and ``stimuli`` (n, H, W) float32 created by ``init``; ``params/D``,
``params/dt``, ``params/dx`` and ``params/<field>`` (float64 scalars, as h5py stores Python
floats); ``diffusivity``; ``field`` (n, H, W), ``start``, ``duration``, ``period``.  Files are
written and read by :mod:`cardiax_gb300.h5` (no h5py needed).

``imresize(a, size)`` resizes the last two axes of a device array with the bilinear resampling
of ``jax.image.resize`` (what the reference calls), through ``fk_resize_bilinear``.
"""
from __future__ import annotations

import os
from typing import List, Sequence

import numpy as np
import torch

from . import _native as N
from . import h5
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


def _resized(x, shape):
    """``x`` as a host array, resized on the device to ``shape`` (last two axes) when given."""
    if shape is None:
        return _np(x)
    return _np(imresize(x, tuple(shape)[-2:]))


def init(path: str, shape: Sequence[int], n_iter: int, n_stimuli: int,
         n_variables: int = 3) -> h5.File:
    """A new data set at ``path`` with ``states`` (n_iter, n_variables, *shape) and ``stimuli``
    (n_stimuli, *shape), float32 (cardiax/io.py:13-23).  The containing folder is created
    when the path has one."""
    folder = os.path.dirname(path)
    if folder:
        os.makedirs(folder, exist_ok=True)
    f = h5.File(path, "w")
    shape = tuple(int(s) for s in shape)
    f.create_dataset("states", shape=(int(n_iter), int(n_variables)) + shape, dtype="float32")
    f.create_dataset("stimuli", shape=(int(n_stimuli),) + shape, dtype="float32")
    return f


def add_params(hdf5: h5.Group, params, diffusivity, dt, dx, shape=None) -> bool:
    """``params/D`` (resized to ``shape`` when given), ``params/dt``, ``params/dx`` and one
    scalar per parameter field (cardiax/io.py:26-36)."""
    hdf5.create_dataset("params/D", data=_resized(diffusivity, shape))
    hdf5.create_dataset("params/dt", data=_scalar(dt))
    hdf5.create_dataset("params/dx", data=_scalar(dx))
    from .params import Params

    names = getattr(type(params), "_fields", Params._fields)  # a plain tuple in Params order
    for name, value in zip(names, params):
        hdf5.create_dataset("params/" + name, data=_scalar(value))
    return True


def add_diffusivity(hdf5: h5.Group, diffusivity, shape=None) -> bool:
    """``diffusivity`` (resized to ``shape`` when given; cardiax/io.py:39-44)."""
    hdf5.create_dataset("diffusivity", data=_resized(diffusivity, shape))
    return True


def add_stimuli(hdf5: h5.Group, stimuli, shape=None) -> bool:
    """``field`` (n, H, W) and the protocols as ``start``, ``duration``, ``period``
    (cardiax/io.py:47-64)."""
    fields = [_resized(s.field, shape) for s in stimuli]
    hdf5.create_dataset("field", data=np.stack(fields) if fields else np.asarray([]))
    for key in ("start", "duration", "period"):
        hdf5.create_dataset(key, data=np.asarray([_scalar(getattr(s.protocol, key))
                                                  for s in stimuli]))
    return True


def add_state(dset: h5.Dataset, state, t: int, shape=None) -> bool:
    """Row ``t`` of ``states``; with ``shape`` the state is resized on the device first
    (cardiax/io.py:67-72; ``shape`` may be (H, W) or (n_variables, H, W))."""
    if isinstance(state, torch.Tensor) and state.dim() == 3:
        array = state
    elif isinstance(state, (tuple, list)) and all(isinstance(x, torch.Tensor) for x in state):
        array = torch.stack([x.to(torch.float32) for x in state])
    else:
        array = np.asarray([_np(x) for x in state], dtype=np.float32)
    dset[int(t)] = _resized(array, shape)
    return True


def add_states(dset: h5.Dataset, states, start: int, end: int) -> bool:
    """Rows ``start:end`` of ``states`` (cardiax/io.py:75-78)."""
    if isinstance(states, (list, tuple)):
        states = np.stack([_np(x) for x in states]) if states else np.zeros((0,) + dset.shape[1:])
    dset[start:end] = _np(states)
    return True


def load(path: str, start=None, end=None, step=None) -> List[np.ndarray]:
    """``file[name][start:end:step]`` for every member of the root group, in name order
    (cardiax/io.py:81-83).  A group among them cannot be sliced and raises ``TypeError``, as
    it does with h5py."""
    with h5.File(path, "r") as f:
        out = []
        for name in f:
            obj = f[name]
            if isinstance(obj, h5.Group):
                raise TypeError(f"Accessing a group is done with bytes or str, not {slice}")
            out.append(obj[start:end:step])
        return out


def load_state(dset: h5.Dataset, start, end, step) -> np.ndarray:
    """``dset[start:end:step]`` (cardiax/io.py:86-87)."""
    return dset[start:end:step]


def load_stimuli(file: h5.Group) -> list:
    """The stimuli stored by :func:`add_stimuli` (cardiax/io.py:90-96)."""
    from .stimulus import Protocol, Stimulus

    out = []
    for i in range(len(file["field"])):
        protocol = Protocol(file["start"][i], file["duration"][i], file["period"][i])
        out.append(Stimulus(protocol, file["field"][i]))
    return out


def load_params(filepath: str):
    """(Params, D) from ``params/`` (cardiax/io.py:99-110).  Fields are matched by name: the
    reference passes every stored value, ``dt`` and ``dx`` included, positionally in name
    order, which does not build a valid ``Params``."""
    from .params import Params

    with h5.File(filepath, "r") as f:
        g = f["params"]
        D = g["D"][...] if "D" in g else None
        values = {k: g[k][()] for k in g if k != "D"}
    missing = [n for n in Params._fields if n not in values]
    if missing:
        raise KeyError(f"parameters missing from {filepath}: {missing}")
    return Params(*(float(values[n]) for n in Params._fields)), D


def load_diffusivity(filepath: str) -> np.ndarray:
    """``diffusivity`` (cardiax/io.py:113-115)."""
    with h5.File(filepath, "r") as f:
        return f["diffusivity"][:]


def _scalar(x):
    """Python numbers as h5py stores them (float64, int64); array scalars keep their type."""
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    if isinstance(x, np.ndarray) and x.ndim == 0:
        return x[()]
    return x
