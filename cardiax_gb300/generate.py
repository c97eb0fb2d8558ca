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

import numpy as np

from . import convert, io, scars
from . import stimulus as S
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


# ---- randomised experiments (deepx/generate.py:16-133) ---------------------------------------
# The reference draws from JAX's PRNG; here every function takes a NumPy Generator (or a seed)
# and draws the same distributions in the reference's order.

def _rng(rng) -> np.random.Generator:
    return rng if isinstance(rng, np.random.Generator) else np.random.default_rng(rng)


def random_protocol(rng, min_start: int = 0, max_start: int = 1000, min_period: int = 400,
                    max_period: int = int(1e9)) -> S.Protocol:
    """Start in [min_start, max_start), duration 2 (instantaneous), period in
    [min_period, max_period) (deepx/generate.py:16-27)."""
    g = _rng(rng)
    start = int(g.integers(int(min_start), int(max_start)))
    period = int(g.integers(int(min_period), int(max_period)))
    return S.Protocol(start, 2, period)


def random_rectangular_stimulus(rng, shape, protocol: S.Protocol, modulus: float = 0.6,
                                device=None) -> S.Stimulus:
    """A rectangle of size in [max(H // 100, 10), H // 3) per side, centred in
    [min(size), H) (deepx/generate.py:30-36)."""
    g = _rng(rng)
    size = g.integers(max(shape[0] // 100, 10), shape[0] // 3, size=2)
    centre = g.integers(int(size.min()), shape[0], size=2)
    return S.rectangular(shape, (int(centre[0]), int(centre[1])), (int(size[0]), int(size[1])),
                         modulus, protocol, device=device)


def random_linear_stimulus(rng, shape, protocol: S.Protocol, modulus: float = 0.6,
                           device=None) -> S.Stimulus:
    """A stripe of coverage 0.2 |N(0, 1)| along the north, east or south edge (the reference
    draws the direction from [0, 3), so never west; deepx/generate.py:39-45)."""
    g = _rng(rng)
    coverage = abs(float(g.standard_normal()))
    direction = S.Direction(int(g.integers(0, 3)))
    return S.linear(shape, direction, coverage * 0.2, modulus, protocol, device=device)


def random_triangular_stimulus(rng, shape, protocol: S.Protocol, modulus: float = 0.6,
                               device=None) -> S.Stimulus:
    """A stripe of coverage 0.2 |N(0, 1)| rotated by 45 |N(0, 1)| degrees
    (deepx/generate.py:48-56)."""
    g = _rng(rng)
    angle, coverage = np.abs(g.standard_normal(2))
    direction = S.Direction(int(g.integers(0, 3)))
    return S.triangular(shape, direction, float(angle) * 45, float(coverage) * 0.2, modulus,
                        protocol, device=device)


def random_stimulus(rng, shape, min_start: int = 0, max_start: int = 0,
                    device=None) -> S.Stimulus:
    """A rectangular, triangular or linear stimulus of amplitude 20 with a random protocol
    (deepx/generate.py:59-76; the reference's default max_start = 0 is an empty range, so callers
    pass one)."""
    g = _rng(rng)
    protocol = random_protocol(g, min_start=min_start, max_start=max_start)
    fns = (random_rectangular_stimulus, random_triangular_stimulus, random_linear_stimulus)
    fn = fns[int(g.integers(0, len(fns)))]
    return fn(g, shape, protocol=protocol, modulus=20.0, device=device)


def random_sequence(rng, params, filepath: str = None, shape: Sequence[int] = (1200, 1200),
                    n_stimuli: int = 2, start: float = 0, stop: float = 1000, step: float = 1,
                    dt: float = 0.01, dx: float = 0.01, reshape: Sequence[int] = None,
                    use_memory: bool = False, plot_while: bool = False, device=None):
    """A random experiment (deepx/generate.py:86-133): ``n_stimuli`` stimuli whose starts are
    spaced by ``tau_d`` seconds, a scar diffusivity map, and the sequence of states from
    ``start`` to ``stop`` ms every ``step`` ms (:func:`sequence`).  Times in ms."""
    g = _rng(rng)
    shape = tuple(int(x) for x in shape)
    starts = np.arange(1, convert.ms_to_units(stop, dt),
                       convert.ms_to_units(params.tau_d * 1000, dt))
    if len(starts) < n_stimuli:
        raise ValueError("too few stimulus start slots before `stop`")
    stimuli = [random_stimulus(g, shape, min_start=int(starts[i]), max_start=int(starts[i]) + 1,
                               device=device) for i in range(n_stimuli)]
    diffusivity = random_diffusivity(g, shape, device=device)
    return sequence(start=convert.ms_to_units(start, dt), stop=convert.ms_to_units(stop, dt),
                    step=convert.ms_to_units(step, dt), dt=dt, dx=dx, params=params,
                    diffusivity=diffusivity, stimuli=stimuli, filename=filepath,
                    reshape=reshape, use_memory=use_memory, plot_while=plot_while,
                    device=device)
