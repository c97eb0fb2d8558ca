"""Drop-in replacement for the reference's stepper API (cardiax/solve.py).

Same names, argument order and meaning as the reference:

=======================  =======================================  ==========================
function                 reference                                 C ABI
=======================  =======================================  ==========================
``State``                cardiax/solve.py:12-15 (v, w, u)          state = 3 planes v, w, u
``init``                 cardiax/solve.py:18-23                    ``fk_init``
``step``                 cardiax/solve.py:26-65                    ``fk_step``
``step_euler``           cardiax/solve.py:68-70                    ``fk_euler_step``
``_forward_euler``       cardiax/solve.py:92-100                   ``fk_forward_euler``
``forward``              cardiax/solve.py:168-222                  ``fk_forward``
``forward_dimensional``  cardiax/solve.py:133-165                  ``fk_forward``
``step_heun``            cardiax/solve.py:73-85                    ``fk_heun_step``
``_forward_heun``        cardiax/solve.py:103-111                  ``fk_forward_heun``
=======================  =======================================  ==========================

Arrays may be NumPy arrays or torch tensors; results are float32 torch tensors on the current
CUDA device (views of pitched device buffers).  Like the reference these functions are pure:
inputs are never modified.  The Euler and Heun integrators are implemented; Dormand-Prince and
plotting are not part of this package.
"""
from __future__ import annotations

from enum import Enum
from typing import List, NamedTuple

import torch

from . import convert
from .tissue import Tissue, _scalar


class State(NamedTuple):
    v: torch.Tensor
    w: torch.Tensor
    u: torch.Tensor


class TimeIntegrator(Enum):
    EULER = "euler"
    HEUN = "heun"
    DORMANDPRINCE = "dormandprince"


def _shape_of(state) -> tuple:
    u = state[2]
    return tuple(int(s) for s in (u.shape if hasattr(u, "shape") else torch.as_tensor(u).shape))


def _tissue(state, params, diffusivity, stimuli, dt, dx) -> Tissue:
    tis = Tissue(_shape_of(state), params, diffusivity, stimuli, dt=dt, dx=dx)
    tis.set_state(state)
    return tis


def _states(tis: Tissue, buf: torch.Tensor) -> List[State]:
    v, w, u = tis.view(buf)
    return [State(v[i], w[i], u[i]) for i in range(buf.shape[0])]


def init(shape, device=None) -> State:
    """v = w = 1, u = 0 on a grid of ``shape`` (cardiax/solve.py:18-23)."""
    from .params import PARAMSET_3

    H, W = int(shape[0]), int(shape[1])
    tis = Tissue((H, W), PARAMSET_3, torch.zeros((H, W)), (), device=device)
    return State(*tis.view())


def step(state, t, params, diffusivity, stimuli, dx) -> State:
    """Time derivative (dv, dw, du) of ``state`` at step ``t`` (cardiax/solve.py:26-65)."""
    tis = _tissue(state, params, diffusivity, stimuli, 0.0, dx)
    return State(*tis.view(tis.derivative(int(_scalar(t)))))


def step_euler(state, t, params, diffusivity, stimuli, dt, dx) -> State:
    """One explicit Euler step (cardiax/solve.py:68-70)."""
    tis = _tissue(state, params, diffusivity, stimuli, dt, dx)
    return State(*tis.view(tis.euler_step(int(_scalar(t)))))


def _forward_euler(state, t, t_end, params, diffusivity, stimuli, dt, dx) -> State:
    """The state after steps t .. t_end-1 (cardiax/solve.py:92-100)."""
    tis = _tissue(state, params, diffusivity, stimuli, dt, dx)
    out = tis.forward([int(_scalar(t)), int(_scalar(t_end))])
    return _states(tis, out)[0]


def step_heun(state, t, params, diffusivity, stimuli, dt, dx) -> State:
    """One Heun step, both stages at step t (cardiax/solve.py:73-85)."""
    tis = _tissue(state, params, diffusivity, stimuli, dt, dx)
    tis.advance_heun(int(_scalar(t)), int(_scalar(t)) + 1)
    return State(*tis.view())


def _forward_heun(state, t, t_end, params, diffusivity, stimuli, dt, dx) -> State:
    """The state after Heun steps t .. t_end-1 (cardiax/solve.py:103-111)."""
    tis = _tissue(state, params, diffusivity, stimuli, dt, dx)
    tis.advance_heun(int(_scalar(t)), int(_scalar(t_end)))
    return State(*tis.view())


def forward(state, checkpoints, params, diffusivity, stimuli, dt, dx,
            integrator=TimeIntegrator.EULER, plot_while=False) -> List[State]:
    """States at ``checkpoints[1:]`` (the initial state is not included), advancing with the
    absolute step index driving the stimuli (cardiax/solve.py:168-222).  Euler and Heun
    integrators; Dormand-Prince is not implemented."""
    if plot_while:
        raise NotImplementedError("plotting is not part of cardiax_gb300")
    tis = _tissue(state, params, diffusivity, stimuli, dt, dx)
    if integrator in (TimeIntegrator.EULER, "euler"):
        return _states(tis, tis.forward(list(checkpoints)))
    if integrator in (TimeIntegrator.HEUN, "heun"):
        ck = [int(_scalar(c)) for c in checkpoints]
        out = []
        for a, b in zip(ck[:-1], ck[1:]):
            tis.advance_heun(a, b)
            out.append(State(*(x.clone() for x in tis.view())))
        return out
    raise NotImplementedError("only the Euler and Heun integrators are implemented")


def forward_dimensional(tissue_size, final_time, ms_step, params, diffusivity, stimuli, dt, dx,
                        integrator=TimeIntegrator.EULER, plot_while=False) -> List[State]:
    """``forward`` from physical sizes and times (cardiax/solve.py:133-165): checkpoints are
    ``range(0, int(final_time/dt), int(ms_step/dt))``."""
    shape = convert.realsize_to_shape(tissue_size, dx)
    stop = convert.ms_to_units(final_time, dt)
    stride = convert.ms_to_units(ms_step, dt)
    assert shape == tuple(diffusivity.shape)
    assert all(tuple(s.field.shape) == shape for s in stimuli)
    state = init(shape)
    checkpoints = list(range(0, stop, stride))
    return forward(state, checkpoints, params, diffusivity, stimuli, dt, dx, integrator,
                   plot_while)
