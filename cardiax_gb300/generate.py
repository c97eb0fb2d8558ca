"""The data-generation caller of the stepper: ``sequence`` of deepx/generate.py:135-210.

Advances a tissue from rest through ``checkpoints = range(start, stop, step)`` with the stepper
(``_forward_euler`` per interval, cardiax/solve.py:92-100) and emits the state after every
interval resized to ``reshape`` (``io.imresize``, cardiax/io.py:118-124).  The emission is a
resize kernel that reads the stepper's state buffer and writes straight into the output slot on
the GPU, so nothing leaves the device until the caller reads the result.

Like the reference's ``states`` dataset, the result has ``len(checkpoints)`` rows of which the
first ``len(checkpoints) - 1`` are written (row i: the state at ``checkpoints[i + 1]``) and the
last stays zero.  With ``filename`` the data set is also written as the reference writes it
(``io.init``, ``add_params``, ``add_stimuli``, ``add_diffusivity`` at the output shape, then
the states: row by row as they are computed, or all at the end with ``use_memory``).
Plotting and progress printing are not part of this package.
"""
from __future__ import annotations

from typing import Sequence

import torch

from . import convert, io, scars
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
    hdf5 = None
    if filename is not None:
        hdf5 = io.init(filename, out_shape, n_iter=n, n_stimuli=len(stimuli))
        io.add_params(hdf5, params, diffusivity, dt, dx, shape=out_shape)
        io.add_stimuli(hdf5, stimuli, shape=out_shape)
        io.add_diffusivity(hdf5, diffusivity, shape=out_shape)
    try:
        for i in range(n - 1):
            tis.advance(checkpoints[i], checkpoints[i + 1])
            io.resize_planes(tis.state, tis.H, tis.W, states[i], antialias)
            if hdf5 is not None and not use_memory:
                io.add_state(hdf5["states"], states[i], i)
        if hdf5 is not None and use_memory and n > 1:
            io.add_states(hdf5["states"], states[:n - 1], 0, n - 1)
    finally:
        if hdf5 is not None:
            hdf5.close()
    return states


def random_diffusivity(rng, shape: Sequence[int], domain: Sequence[float] = (0.0001, 0.001),
                       device=None) -> torch.Tensor:
    """A scar map (``scars.random_diffusivity_scar``) rescaled onto ``domain``
    (deepx/generate.py:79-83): an (H, W) float32 device tensor."""
    c = scars.random_diffusivity_scar(rng, shape, device)
    return convert.diffusivity_rescale(c, domain)
