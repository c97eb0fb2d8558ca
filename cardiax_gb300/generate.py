"""The data-generation caller of the stepper: ``sequence`` of deepx/generate.py:135-210.

Advances a tissue from rest through ``checkpoints = range(start, stop, step)`` with the stepper
(``_forward_euler`` per interval, cardiax/solve.py:92-100) and emits the state after every
interval resized to ``reshape`` (``io.imresize``, cardiax/io.py:118-124).  The emission is a
resize kernel that reads the stepper's state buffer and writes straight into the output slot on
the GPU, so nothing leaves the device until the caller reads the result.

Like the reference's ``states`` dataset, the result has ``len(checkpoints)`` rows of which the
first ``len(checkpoints) - 1`` are written (row i: the state at ``checkpoints[i + 1]``) and the
last stays zero.  With ``filename`` the data set is also written (``io.save``: the reference's
HDF5 dataset names in a ``.npz`` archive).  Plotting and progress printing are not part of this
package.
"""
from __future__ import annotations

from typing import Sequence

import torch

from . import io
from .tissue import Tissue


def sequence(start: int, stop: int, step: int, dt: float, dx: float, params, diffusivity,
             stimuli: Sequence, filename: str = None, reshape: Sequence[int] = None,
             use_memory: bool = True, plot_while: bool = False, antialias: bool = True,
             device=None) -> torch.Tensor:
    """(len(checkpoints), 3, *out_shape) float32 device tensor of the emitted states
    (deepx/generate.py:135-210; ``start``/``stop``/``step`` in steps)."""
    if plot_while:
        raise NotImplementedError("plotting is not part of cardiax_gb300")
    D = diffusivity
    shape = tuple(int(x) for x in (D.shape if hasattr(D, "shape") else torch.as_tensor(D).shape))
    out_shape = tuple(int(x) for x in reshape) if reshape is not None else shape
    checkpoints = list(range(int(start), int(stop), int(step)))
    tis = Tissue(shape, params, diffusivity, stimuli, dt=dt, dx=dx, device=device)
    n = len(checkpoints)
    states = torch.zeros((n, 3) + out_shape, dtype=torch.float32, device=tis.device)
    for i in range(n - 1):
        tis.advance(checkpoints[i], checkpoints[i + 1])
        io.resize_planes(tis.state, tis.H, tis.W, states[i], antialias)
    if filename is not None:
        io.save(filename, states, params, diffusivity, stimuli, dt, dx,
                shape=out_shape if reshape is not None else None)
    return states
