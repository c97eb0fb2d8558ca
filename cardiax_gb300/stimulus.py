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
    """``linear`` rotated by ``angle`` degrees with nearest-edge filling and no prefilter
    (cardiax/stimulus.py:109-140).  Host-side set-up through SciPy."""
    from scipy.ndimage import rotate

    stim = linear(shape, direction, coverage, modulus, protocol, device="cpu")
    field = rotate(stim.field.numpy(), angle=angle, mode="nearest", prefilter=False,
                   reshape=False)
    return Stimulus(protocol, torch.as_tensor(np.ascontiguousarray(field, dtype=np.float32),
                                              device=_device(device)))
