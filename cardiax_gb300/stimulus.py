"""Stimulus protocols and field generators (cardiax/stimulus.py:13-140).

``Protocol`` values are in simulation steps.  ``Stimulus.field`` is a dense float32 field of the
grid's shape, as in the reference; the stepper turns constant-valued rectangular fields into
rectangle descriptors so they cost no memory traffic.  Fields are torch tensors (created on
``device``, by default the current CUDA device when one is present).
"""
from __future__ import annotations

from enum import IntEnum
from typing import Any, NamedTuple, Tuple

import numpy as np
import torch

Shape = Tuple[int, ...]
Point2D = Tuple[int, int]


class Protocol(NamedTuple):
    start: float
    duration: float
    period: float


class Stimulus(NamedTuple):
    protocol: Protocol
    field: Any


class Direction(IntEnum):
    NORTH = 0
    EAST = 1
    SOUTH = 2
    WEST = 3


def _device(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def rectangular(shape: Shape, centre: Point2D, size: Point2D, modulus: float,
                protocol: Protocol, device=None) -> Stimulus:
    """Rectangle ``[int(c0 - s0/2):int(c0 + s0/2), int(c1 - s1/2):int(c1 + s1/2)]`` set to
    ``modulus`` (cardiax/stimulus.py:31-60)."""
    field = torch.zeros(tuple(shape), dtype=torch.float32, device=_device(device))
    x1, x2 = int(centre[0] - size[0] / 2), int(centre[0] + size[0] / 2)
    y1, y2 = int(centre[1] - size[1] / 2), int(centre[1] + size[1] / 2)
    field[x1:x2, y1:y2] = modulus
    return Stimulus(protocol, field)


def linear(shape: Shape, direction: Direction, coverage: float, modulus: float,
           protocol: Protocol, device=None) -> Stimulus:
    """A stripe of width ``int(shape[0] * coverage)`` along one edge (cardiax/stimulus.py:63-106;
    the width uses ``shape[0]`` for every direction, as the reference does)."""
    n = int(shape[0] * coverage)
    field = torch.zeros(tuple(shape), dtype=torch.float32, device=_device(device))
    if direction == Direction.WEST:
        field[:, :n] = modulus
    elif direction == Direction.EAST:
        field[:, -n:] = modulus  # n == 0 selects every column, as the reference's -0: does
    elif direction == Direction.NORTH:
        field[:n, :] = modulus
    elif direction == Direction.SOUTH:
        field[-n:, :] = modulus
    else:
        raise ValueError(
            "direction mus be either 'left', 'right', 'up', or 'down' not %s" % direction)
    return Stimulus(protocol, field)


def triangular(shape: Shape, direction: Direction, angle: float, coverage: float,
               modulus: float, protocol: Protocol, device=None) -> Stimulus:
    """``linear`` rotated by ``angle`` degrees about the centre (cardiax/stimulus.py:109-140):
    the reference's scipy.ndimage.rotate(mode="nearest", prefilter=False, reshape=False), as a
    CUDA kernel (``fk_rotate_field``)."""
    from . import _native as N
    from .tissue import stream_handle

    dev = _device(device)
    if dev.type != "cuda":
        raise RuntimeError("triangular fields are built on a CUDA device (there is no CPU path)")
    stim = linear(shape, direction, coverage, modulus, protocol, device=dev)
    src = stim.field.to(device=dev, dtype=torch.float32).contiguous()
    H, W = int(src.shape[0]), int(src.shape[1])
    out = torch.empty_like(src)
    N.call("fk_rotate_field", src.data_ptr(), H, W, W, out.data_ptr(), W, float(angle),
           stream_handle())
    return Stimulus(protocol, out)