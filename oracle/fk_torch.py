"""Autodiff oracle for the Fenton-Karma stepper -- TEST INFRASTRUCTURE ONLY.

A PyTorch (CPU, float64 by default) restatement of cardiax/solve.py:26-70,225-271 with the same
formulas as ``fk_oracle.py``.  Differentiating it with ``torch.autograd`` stands in for
``jax.grad`` of the reference (JAX is not installable here).  As in JAX, the Heaviside gates
(comparisons) and ``where``-based stimulus replacement have zero derivative with respect to u.

The 13 differentiable parameters are the first 13 fields of cardiax Params
(cardiax/params.py:4-17); Cm is held fixed.
"""
from __future__ import annotations

import torch

PARAM_FIELDS = ("tau_v_plus", "tau_v1_minus", "tau_v2_minus", "tau_w_plus", "tau_w_minus",
                "tau_d", "tau_0", "tau_r", "tau_si", "k", "V_csi", "V_c", "V_v", "Cm")


def gradient(a: torch.Tensor, axis: int) -> torch.Tensor:
    """cardiax/solve.py:225-254 (un-scaled)."""
    n = a.shape[axis]

    def s(lo, hi):
        return a.narrow(axis, lo, hi - lo)

    head = (-11 / 6) * s(0, 2) + 3 * s(1, 3) - (3 / 2) * s(2, 4) + (1 / 3) * s(3, 5)
    body = (1 / 12) * s(0, n - 4) - (2 / 3) * s(1, n - 3) + (2 / 3) * s(3, n - 1) \
        - (1 / 12) * s(4, n)
    tail = (-1 / 3) * s(n - 5, n - 3) + (3 / 2) * s(n - 4, n - 2) - 3 * s(n - 3, n - 1) \
        + (11 / 6) * s(n - 2, n)
    return torch.cat((head, body, tail), axis)


def _pad(x):
    return torch.nn.functional.pad(x[None, None], (1, 1, 1, 1), mode="replicate")[0, 0]


def active(t, start, duration, period) -> bool:
    """Protocol test of cardiax/solve.py:262-267 (float64 here; integer steps)."""
    if not (t >= start):
        return False
    m = (start - t + 1) % period  # Python's % is a floor modulo, like jnp.mod
    return m < duration


def euler_step(state, t, theta, Cm, D, stimuli, dt, dx):
    """One Euler step; ``state`` = (v, w, u) tensors, ``theta`` a 13-vector (requires_grad ok),
    ``stimuli`` = [(start, duration, period, field)]."""
    v, w, u = state
    (tvp, tv1m, tv2m, twp, twm, td, t0, tr, tsi, k, vcsi, vc, vv) = (theta[i] for i in range(13))
    vp, wp, up, Dp = _pad(v), _pad(w), _pad(u), _pad(D)
    p = (up >= vc).to(up.dtype).detach()
    q = (up >= vv).to(up.dtype).detach()
    tvm = (1 - q) * tv1m + q * tv2m
    j_fi = -vp * p * (up - vc) * (1 - up) / td
    j_so = (up * (1 - p) / t0) + (p / tr)
    j_si = -(wp * (1 + torch.tanh(k * (up - vcsi)))) / (2 * tsi)
    j_ion = -(j_fi + j_so + j_si) / Cm
    acc = torch.zeros_like(j_ion)
    for (st, du_, per, f) in stimuli:
        if active(t, st, du_, per):
            fp = _pad(f)
            acc = torch.where(fp != 0, fp, acc)
    j_ion = torch.where(acc != 0, acc, j_ion)
    u_x = gradient(up, 0) / dx
    u_y = gradient(up, 1) / dx
    u_xx = gradient(u_x, 0) / dx
    u_yy = gradient(u_y, 1) / dx
    D_x = gradient(Dp, 0) / dx
    D_y = gradient(Dp, 1) / dx
    del_u = Dp * (u_xx + u_yy) + (D_x * u_x) + (D_y * u_y)
    d_v = ((1 - p) * (1 - vp) / tvm) - ((p * vp) / tvp)
    d_w = ((1 - p) * (1 - wp) / twm) - ((p * wp) / twp)
    d_u = del_u + j_ion
    c = (slice(1, -1), slice(1, -1))
    return (v + d_v[c] * dt, w + d_w[c] * dt, u + d_u[c] * dt)


def forward(state, t0, t1, theta, Cm, D, stimuli, dt, dx, keep_every: int = 0):
    """Steps t0 .. t1-1; returns the final state (and, with keep_every > 0, the list of states
    at t0 + keep_every, t0 + 2 keep_every, ...)."""
    kept = []
    for t in range(int(t0), int(t1)):
        state = euler_step(state, t, theta, Cm, D, stimuli, dt, dx)
        if keep_every and (t + 1 - t0) % keep_every == 0:
            kept.append(state)
    return (state, kept) if keep_every else state
