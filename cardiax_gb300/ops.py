"""The C ABI as PyTorch operators: ``torch.ops.cardiax_gb300.*`` (``torch.library.custom_op``).

Each operator is a thin functional wrapper over the same C entry points that
:mod:`cardiax_gb300.solve` calls, so results are bit-identical to the ctypes path.  Every
operator has a fake (meta) kernel, so it is opaque to ``torch.compile`` / ``torch.export`` and
traces with shapes only; ``forward_euler`` also has an autograd formula (the hand-written adjoint
kernel with sqrt(T) checkpoint-recompute), so gradients flow through the dispatcher.

Conventions shared by the operators (the reference's, cardiax/solve.py:12-15,26-100):

* ``state``: a (3, H, W) float32 CUDA tensor holding v, w, u (the reference's State order);
  results are fresh (3, H, W) tensors, inputs are never modified;
* ``D``: the (H, W) diffusivity map;
* ``params``: a 14-element tensor in cardiax ``Params`` field order (any device);
* stimuli: ``stim_protocols`` a flat list [start, duration, period] * n (in steps) and
  ``stim_fields`` the n (H, W) fields (cardiax/stimulus.py:13-21);
* step indices are integers; ``dt``, ``dx`` floats.

=================================  ===========================================  ====================
operator                           reference                                     C ABI
=================================  ===========================================  ====================
``step``                           cardiax/solve.py:26-65 (derivative)           ``fk_step``
``euler_step``                     cardiax/solve.py:68-70                        ``fk_euler_step``
``forward_euler``                  cardiax/solve.py:92-100                       ``fk_forward_euler``
``forward``                        cardiax/solve.py:168-222 (Euler)              ``fk_forward``
``batch_forward_euler``            (none: many tissues per launch)               ``fk_batch_*``
``adjoint_step``                   (none: reverse of step_euler)                 ``fk_adjoint_step``
=================================  ===========================================  ====================
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import torch
from torch import Tensor

from .stimulus import Protocol, Stimulus
from .tissue import Tissue

NS = "cardiax_gb300"


def _stimuli(protocols: Sequence[float], fields: Sequence[Tensor]):
    if len(protocols) != 3 * len(fields):
        raise ValueError("stim_protocols must hold (start, duration, period) per stimulus field")
    return [Stimulus(Protocol(protocols[3 * k], protocols[3 * k + 1], protocols[3 * k + 2]), f)
            for k, f in enumerate(fields)]


def _params(params: Tensor) -> List[float]:
    vals = [float(x) for x in params.detach().reshape(-1).cpu().tolist()]
    if len(vals) != 14:
        raise ValueError("params must hold the 14 fields of cardiax Params")
    return vals


def _check_state(state: Tensor):
    if state.dim() != 3 or state.shape[0] != 3:
        raise ValueError(f"state must be (3, H, W), got {tuple(state.shape)}")
    if not state.is_cuda:
        raise ValueError("cardiax_gb300 operators run on CUDA tensors only")


def _tissue(state, D, params, protocols, fields, dt, dx) -> Tissue:
    _check_state(state)
    H, W = int(state.shape[1]), int(state.shape[2])
    tis = Tissue((H, W), _params(params), D.detach(), _stimuli(protocols, fields), dt=dt, dx=dx,
                 device=state.device)
    tis.set_state(state.detach())
    return tis


def _unpitched(buf: Tensor, W: int) -> Tensor:
    return buf[..., :W].contiguous()


# ---- step / euler_step ----------------------------------------------------------------------
@torch.library.custom_op(f"{NS}::step", mutates_args=())
def step(state: Tensor, D: Tensor, params: Tensor, stim_protocols: Sequence[float],
         stim_fields: Sequence[Tensor], t: int, dx: float) -> Tensor:
    """(dv, dw, du) of ``state`` at step ``t`` (cardiax/solve.py:26-65)."""
    tis = _tissue(state, D, params, stim_protocols, stim_fields, 0.0, dx)
    return _unpitched(tis.derivative(int(t)), tis.W)


@step.register_fake
def _(state, D, params, stim_protocols, stim_fields, t, dx):
    return torch.empty_like(state, memory_format=torch.contiguous_format)


@torch.library.custom_op(f"{NS}::euler_step", mutates_args=())
def euler_step(state: Tensor, D: Tensor, params: Tensor, stim_protocols: Sequence[float],
               stim_fields: Sequence[Tensor], t: int, dt: float, dx: float) -> Tensor:
    """One explicit Euler step from step ``t`` (cardiax/solve.py:68-70)."""
    tis = _tissue(state, D, params, stim_protocols, stim_fields, dt, dx)
    return _unpitched(tis.euler_step(int(t)), tis.W)


@euler_step.register_fake
def _(state, D, params, stim_protocols, stim_fields, t, dt, dx):
    return torch.empty_like(state, memory_format=torch.contiguous_format)


# ---- forward_euler (differentiable) ---------------------------------------------------------
@torch.library.custom_op(f"{NS}::forward_euler", mutates_args=())
def forward_euler(state: Tensor, D: Tensor, params: Tensor, stim_protocols: Sequence[float],
                  stim_fields: Sequence[Tensor], t0: int, t1: int, dt: float,
                  dx: float) -> Tensor:
    """The state after steps t0 .. t1-1 (cardiax/solve.py:92-100)."""
    tis = _tissue(state, D, params, stim_protocols, stim_fields, dt, dx)
    tis.advance(int(t0), int(t1))
    return _unpitched(tis.state, tis.W)


@forward_euler.register_fake
def _(state, D, params, stim_protocols, stim_fields, t0, t1, dt, dx):
    return torch.empty_like(state, memory_format=torch.contiguous_format)


def _forward_euler_setup(ctx, inputs, output):
    state, D, params, protos, fields, t0, t1, dt, dx = inputs
    ctx.save_for_backward(state, D, params)
    ctx.rest = (list(protos), list(fields), int(t0), int(t1), float(dt), float(dx))


def _forward_euler_backward(ctx, grad):
    from .adjoint import Adjoint
    state, D, params = ctx.saved_tensors
    protos, fields, t0, t1, dt, dx = ctx.rest
    tis = _tissue(state, D, params, protos, fields, dt, dx)
    W = tis.W
    g = torch.zeros((1,) + tuple(tis.state.shape), dtype=torch.float32, device=tis.device)
    g[0, ..., :W] = grad.to(torch.float32)
    adj = Adjoint(tis)
    lam0 = adj.rollout_gradient(tis.state.clone(), t0, t1, [t1], g)
    g_params = torch.zeros(14, dtype=params.dtype, device=params.device)
    g_params[:13] = adj.grad_theta().to(device=params.device, dtype=params.dtype)
    # one entry per input, the stimulus-field list answered with a list
    return (lam0[..., :W].contiguous(), adj.grad_D().clone().to(D.dtype), g_params, None,
            [None] * len(fields), None, None, None, None)


torch.library.register_autograd(f"{NS}::forward_euler", _forward_euler_backward,
                                setup_context=_forward_euler_setup)


# ---- forward (checkpoints) ------------------------------------------------------------------
@torch.library.custom_op(f"{NS}::forward", mutates_args=())
def forward(state: Tensor, checkpoints: Sequence[int], D: Tensor, params: Tensor,
            stim_protocols: Sequence[float], stim_fields: Sequence[Tensor], dt: float,
            dx: float) -> Tensor:
    """States at ``checkpoints[1:]`` as a (len - 1, 3, H, W) tensor (cardiax/solve.py:168-222,
    Euler integrator; the initial state is not included)."""
    tis = _tissue(state, D, params, stim_protocols, stim_fields, dt, dx)
    return _unpitched(tis.forward([int(c) for c in checkpoints]), tis.W)


@forward.register_fake
def _(state, checkpoints, D, params, stim_protocols, stim_fields, dt, dx):
    n = max(0, len(checkpoints) - 1)
    return state.new_empty((n,) + tuple(state.shape))


# ---- batched tissues ------------------------------------------------------------------------
@torch.library.custom_op(f"{NS}::batch_forward_euler", mutates_args=())
def batch_forward_euler(states: Sequence[Tensor], Ds: Sequence[Tensor], params: Tensor,
                        stim_counts: Sequence[int], stim_protocols: Sequence[float],
                        stim_fields: Sequence[Tensor], t0: int, t1: int, dt: float, dx: float,
                        graph_steps: int = 64) -> List[Tensor]:
    """Steps t0 .. t1-1 of many tissues (any shapes; ``params`` is (n, 14)) in one persistent
    launch per step; tissue k owns ``stim_counts[k]`` consecutive entries of the stimulus
    lists.  Per tissue the result equals ``forward_euler`` bit for bit."""
    from .batch import TissueBatch
    n = len(states)
    if len(Ds) != n or len(stim_counts) != n or tuple(params.shape) != (n, 14):
        raise ValueError("one D map, one parameter row and one stimulus count per tissue")
    if sum(stim_counts) != len(stim_fields):
        raise ValueError("stim_counts must add up to the number of stimulus fields")
    tissues, k = [], 0
    for i in range(n):
        c = int(stim_counts[i])
        tissues.append(_tissue(states[i], Ds[i], params[i], stim_protocols[3 * k:3 * (k + c)],
                               stim_fields[k:k + c], dt, dx))
        k += c
    batch = TissueBatch(tissues, graph_steps=graph_steps)
    try:
        batch.advance(int(t0), int(t1))
    finally:
        batch.close()
    return [_unpitched(t.state, t.W) for t in tissues]


@batch_forward_euler.register_fake
def _(states, Ds, params, stim_counts, stim_protocols, stim_fields, t0, t1, dt, dx,
      graph_steps=64):
    return [torch.empty_like(s, memory_format=torch.contiguous_format) for s in states]


# ---- reverse mode ---------------------------------------------------------------------------
@torch.library.custom_op(f"{NS}::adjoint_step", mutates_args=())
def adjoint_step(state: Tensor, D: Tensor, params: Tensor, stim_protocols: Sequence[float],
                 stim_fields: Sequence[Tensor], t: int, dt: float, dx: float,
                 lam_next: Tensor) -> Tuple[Tensor, Tensor, Tensor]:
    """Reverse of one Euler step at ``state`` = x_t: given the cotangent ``lam_next`` of x_{t+1}
    ((3, H, W)), returns (cotangent of x_t, dL/dD of this step (H, W), dL/dtheta of this step
    (13, cardiax Params order without Cm)) -- Heaviside gates and the stimulus replacement
    with zero derivative, as jax.grad of the reference's step_euler defines."""
    from .adjoint import Adjoint
    tis = _tissue(state, D, params, stim_protocols, stim_fields, dt, dx)
    W = tis.W
    ln = torch.zeros_like(tis.state)
    ln[..., :W] = lam_next.to(torch.float32)
    lam = torch.empty_like(tis.state)
    adj = Adjoint(tis)
    adj.step(tis.state, int(t), ln, lam)
    return (_unpitched(lam, W), adj.grad_D().clone(), adj.grad_theta().to(torch.float32))


@adjoint_step.register_fake
def _(state, D, params, stim_protocols, stim_fields, t, dt, dx, lam_next):
    H, W = state.shape[1], state.shape[2]
    return (torch.empty_like(state, memory_format=torch.contiguous_format),
            state.new_empty((H, W)), state.new_empty((13,)))
