"""CPU oracle for the Fenton-Karma Euler stepper -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference's forward path (epignatelli/cardiax), used by the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline as the checker.  It is never the
thing measured as the product and nothing on the product path imports it.

It follows, operation for operation and in the same evaluation order (so that float32 results
round the same way):

* ``cardiax/solve.py:26-65``   ``step``       -> :func:`derivative`
* ``cardiax/solve.py:68-70``   ``step_euler`` -> :func:`euler_step`
* ``cardiax/solve.py:92-100``  ``_forward_euler`` -> :func:`forward_euler`
* ``cardiax/solve.py:73-85,103-111`` ``step_heun``/``_forward_heun`` -> :func:`heun_step`,
  :func:`forward_heun`
* ``cardiax/solve.py:168-222`` ``forward``    -> :func:`forward`
* ``cardiax/solve.py:225-254`` ``gradient``   -> :func:`gradient`
* ``cardiax/solve.py:257-271`` ``stimulate``  -> :func:`stimulate`
* ``cardiax/stimulus.py:63-106,31-60`` ``linear``/``rectangular`` -> :func:`linear_field`,
  :func:`rectangular_field`
* ``cardiax/stimulus.py:109-140`` ``triangular`` -> :func:`rotate_field` (the reference's
  ``scipy.ndimage.rotate(mode="nearest", prefilter=False, reshape=False)`` restated; pinned to
  SciPy itself in ``tests/test_oracle.py``)
* ``cardiax/io.py:118-124`` ``imresize`` -> :func:`imresize_bilinear` (the reference calls
  ``jax.image.resize(a, shape, "bilinear")``; JAX, pinned through jaxlib 0.1.64 in
  ``install_jax.sh``, is not vendored and cannot be installed here, so this is a restatement of
  its published resampling algorithm -- parity unpinned, checked on known answers of the
  triangle kernel in ``tests/test_oracle.py``)

Pinning: the float32 path is checked bit for bit against golden vectors produced by running
the reference's own ``solve.py`` (under a NumPy stand-in for JAX, see
``tests/golden/make_golden.py``) and against the stimulus schedule that the reference's
``tests/macro/stimulate_test.py:16-18`` lists.  ``dtype=np.float64`` gives the FP64 oracle
(the reference with x64 enabled).
"""
from __future__ import annotations

from typing import NamedTuple, Sequence

import numpy as np

# Field order of cardiax/params.py:4-18.
PARAM_FIELDS = ("tau_v_plus", "tau_v1_minus", "tau_v2_minus", "tau_w_plus", "tau_w_minus",
                "tau_d", "tau_0", "tau_r", "tau_si", "k", "V_csi", "V_c", "V_v", "Cm")


class OState(NamedTuple):
    """(v, w, u), the field order of cardiax/solve.py:12-15."""
    v: np.ndarray
    w: np.ndarray
    u: np.ndarray


class OStim(NamedTuple):
    """One stimulus: protocol in steps (cardiax/stimulus.py:13-21) and a dense field."""
    start: float
    duration: float
    period: float
    field: np.ndarray


# --- derivative along one axis (cardiax/solve.py:225-254) --------------------------------------
def gradient(a: np.ndarray, axis: int) -> np.ndarray:
    """Un-scaled 1-D derivative of an (already padded) array along ``axis``.

    Two 3rd-order one-sided rows at each end, the 4th-order central stencil inside; the
    coefficient products are rounded to the array's dtype and summed left to right.
    """
    f = a.dtype.type
    n = a.shape[axis]

    def s(lo, hi):
        idx = [slice(None)] * a.ndim
        idx[axis] = slice(lo, hi)
        return a[tuple(idx)]

    head = f(-11 / 6) * s(0, 2) + f(3) * s(1, 3) - f(3 / 2) * s(2, 4) + f(1 / 3) * s(3, 5)
    body = f(1 / 12) * s(0, n - 4) - f(2 / 3) * s(1, n - 3) + f(2 / 3) * s(3, n - 1) \
        - f(1 / 12) * s(4, n)
    tail = f(-1 / 3) * s(n - 5, n - 3) + f(3 / 2) * s(n - 4, n - 2) - f(3) * s(n - 3, n - 1) \
        + f(11 / 6) * s(n - 2, n)
    return np.concatenate((head, body, tail), axis)


# --- stimulus (cardiax/solve.py:257-271) --------------------------------------------------------
def stimulus_active(t, start, duration, period, dtype=np.float32) -> bool:
    """Whether a protocol is on at step ``t``: ``t >= start`` and
    ``floor_mod(start - t + 1, period) < duration`` (cardiax/solve.py:262-267).

    The loop index of ``forward`` is a float (``float(checkpoints[i])``), so the modulo is
    evaluated in the working float type.
    """
    f = np.dtype(dtype).type
    if not (f(t) >= f(start)):
        return False
    return bool(np.mod(f(start) - f(t) + f(1), f(period)) < f(duration))


def stimulate(t, j_ion: np.ndarray, stimuli: Sequence[OStim]) -> np.ndarray:
    """Replace the ionic current by the field of every active stimulus, later ones winning
    where fields overlap; zero field values leave the current unchanged."""
    acc = np.zeros_like(j_ion)
    for s in stimuli:
        if stimulus_active(t, s.start, s.duration, s.period, j_ion.dtype):
            acc = np.where(s.field != 0, s.field, acc)
    return np.where(acc != 0, acc, j_ion)


# --- d/dt of the state (cardiax/solve.py:26-65) -------------------------------------------------
def derivative(state: OState, t, params: Sequence[float], diffusivity: np.ndarray,
               stimuli: Sequence[OStim], dx: float) -> OState:
    """Time derivative (dv, dw, du) of the Fenton-Karma model on the interior of an edge-padded
    grid (zero-flux boundary)."""
    f = state.u.dtype.type
    P = dict(zip(PARAM_FIELDS, (f(x) for x in params)))
    one = f(1)
    v = np.pad(state.v, 1, mode="edge")
    w = np.pad(state.w, 1, mode="edge")
    u = np.pad(state.u, 1, mode="edge")
    d = np.pad(diffusivity.astype(state.u.dtype, copy=False), 1, mode="edge")

    p = (u >= P["V_c"]).astype(u.dtype)          # gate for the fast inward current
    q = (u >= P["V_v"]).astype(u.dtype)          # selects tau_v1_minus / tau_v2_minus
    tau_vm = (one - q) * P["tau_v1_minus"] + q * P["tau_v2_minus"]

    j_fi = -v * p * (u - P["V_c"]) * (one - u) / P["tau_d"]
    j_so = (u * (one - p) / P["tau_0"]) + (p / P["tau_r"])
    j_si = -(w * (one + np.tanh(P["k"] * (u - P["V_csi"])))) / (f(2) * P["tau_si"])
    j_ion = -(j_fi + j_so + j_si) / P["Cm"]

    padded = [s._replace(field=np.pad(s.field.astype(u.dtype, copy=False), 1, mode="edge"))
              for s in stimuli]
    j_ion = stimulate(t, j_ion, padded)

    h = f(dx)
    u_x = gradient(u, 0) / h
    u_y = gradient(u, 1) / h
    u_xx = gradient(u_x, 0) / h
    u_yy = gradient(u_y, 1) / h
    d_x = gradient(d, 0) / h
    d_y = gradient(d, 1) / h
    del_u = d * (u_xx + u_yy) + (d_x * u_x) + (d_y * u_y)

    dv = ((one - p) * (one - v) / tau_vm) - ((p * v) / P["tau_v_plus"])
    dw = ((one - p) * (one - w) / P["tau_w_minus"]) - ((p * w) / P["tau_w_plus"])
    du = del_u + j_ion
    crop = (slice(1, -1), slice(1, -1))
    return OState(dv[crop], dw[crop], du[crop])


def euler_step(state: OState, t, params, diffusivity, stimuli, dt, dx) -> OState:
    """x <- x + dx/dt * dt for v, w and u (cardiax/solve.py:68-70)."""
    g = derivative(state, t, params, diffusivity, stimuli, dx)
    h = state.u.dtype.type(dt)
    return OState(*(x + dxdt * h for x, dxdt in zip(state, g)))


def heun_step(state: OState, t, params, diffusivity, stimuli, dt, dx) -> OState:
    """Heun's method with both stages at step index t (cardiax/solve.py:73-85):
    x1 = x + dt f(x, t);  x' = x + (f(x, t) + f(x1, t)) (dt / 2)."""
    f = state.u.dtype.type
    d1 = derivative(state, t, params, diffusivity, stimuli, dx)
    x1 = OState(*(x + d * f(dt) for x, d in zip(state, d1)))
    d2 = derivative(x1, t, params, diffusivity, stimuli, dx)
    h = f(dt) * f(0.5)
    return OState(*(x + (a + b) * h for x, a, b in zip(state, d1, d2)))


def forward_heun(state: OState, t0, t1, params, diffusivity, stimuli, dt, dx) -> OState:
    """Heun steps t0 .. t1-1 (cardiax/solve.py:103-111)."""
    f = state.u.dtype.type
    for i in range(int(t0), int(t1)):
        state = heun_step(state, f(i), params, diffusivity, stimuli, dt, dx)
    return state


def forward_euler(state: OState, t0, t1, params, diffusivity, stimuli, dt, dx) -> OState:
    """Steps t0, t0+1, ..., t1-1 with the absolute step index driving the stimuli
    (cardiax/solve.py:92-100)."""
    f = state.u.dtype.type
    for i in range(int(t0), int(t1)):
        state = euler_step(state, f(i), params, diffusivity, stimuli, dt, dx)
    return state


def forward(state: OState, checkpoints, params, diffusivity, stimuli, dt, dx):
    """The states at checkpoints[1:], the initial state excluded (cardiax/solve.py:197-222)."""
    out = []
    for a, b in zip(checkpoints[:-1], checkpoints[1:]):
        state = forward_euler(state, a, b, params, diffusivity, stimuli, dt, dx)
        out.append(state)
    return out


def init(shape, dtype=np.float32) -> OState:
    """v = w = 1, u = 0 (cardiax/solve.py:18-23)."""
    return OState(np.ones(shape, dtype), np.ones(shape, dtype), np.zeros(shape, dtype))


# --- dense stimulus fields (cardiax/stimulus.py:31-106) -----------------------------------------
def linear_field(shape, direction: int, coverage: float, modulus: float, dtype=np.float32):
    """Stripe of width ``int(shape[0] * coverage)`` (N=0, E=1, S=2, W=3)."""
    a = np.zeros(shape, dtype)
    n = int(shape[0] * coverage)
    if direction == 3:
        a[:, :n] = modulus
    elif direction == 1:
        a[:, -n:] = modulus
    elif direction == 0:
        a[:n, :] = modulus
    elif direction == 2:
        a[-n:, :] = modulus
    else:
        raise ValueError(direction)
    return a


def rectangular_field(shape, centre, size, modulus: float, dtype=np.float32):
    """Rectangle ``[int(c0 - s0/2):int(c0 + s0/2), int(c1 - s1/2):int(c1 + s1/2)]``."""
    a = np.zeros(shape, dtype)
    x1, x2 = int(centre[0] - size[0] / 2), int(centre[0] + size[0] / 2)
    y1, y2 = int(centre[1] - size[1] / 2), int(centre[1] + size[1] / 2)
    a[x1:x2, y1:y2] = modulus
    return a


# --- bilinear resize (cardiax/io.py:118-124 -> jax.image.resize "bilinear") -------------------
def resize_weights(n_in: int, n_out: int, antialias: bool = True, dtype=np.float32) -> np.ndarray:
    """(n_in, n_out) float32 weights of one resized axis: the triangle kernel max(0, 1 - |x|)
    at half-pixel centres, output p sampling s = (p + 0.5) / scale - 0.5 (scale = n_out /
    n_in), widened by 1 / scale when downsampling with ``antialias``, normalised per output.
    ``dtype=np.float64`` evaluates the same formulas in double (for comparisons with other
    implementations of the algorithm)."""
    f = dtype
    inv = f(1.0 / (n_out / n_in))
    ks = max(inv, f(1)) if antialias else f(1)
    s = (np.arange(n_out, dtype=f) + f(0.5)) * inv - f(0.5)
    x = np.abs(s[None, :] - np.arange(n_in, dtype=f)[:, None]) / ks
    w = np.maximum(f(0), f(1) - x)
    tot = w.sum(0, keepdims=True, dtype=f)
    w = np.where(np.abs(tot) > f(1000) * np.finfo(f).eps, w / np.where(tot != 0, tot, f(1)), f(0))
    valid = (s >= f(-0.5)) & (s <= f(n_in) - f(0.5))
    return np.where(valid[None, :], w, f(0)).astype(f)


def imresize_bilinear(a: np.ndarray, size, antialias: bool = True, dtype=np.float32) -> np.ndarray:
    """The last two axes of ``a`` resized to ``size``; an axis whose size does not change is
    left as it is.  Float32 like JAX (``dtype=np.float64``: the same in double)."""
    out = np.asarray(a, dtype=dtype)
    H, W = out.shape[-2:]
    if int(size[0]) != H:
        out = np.einsum("...hw,ho->...ow", out, resize_weights(H, int(size[0]), antialias, dtype))
    if int(size[1]) != W:
        out = np.einsum("...hw,wo->...ho", out, resize_weights(W, int(size[1]), antialias, dtype))
    return out.astype(dtype)


# --- rotated fields (cardiax/stimulus.py:109-140 -> scipy.ndimage.rotate) ----------------------
def _bspline3(t):
    t = np.abs(t)
    return np.where(t < 1, 2.0 / 3.0 - t * t + 0.5 * t ** 3, np.where(t < 2, (2 - t) ** 3 / 6, 0.0))


def rotate_field(a: np.ndarray, angle: float) -> np.ndarray:
    """``a`` rotated by ``angle`` degrees about its centre: output (i, j) samples (x, y) =
    R (i, j) + o, R = [[c, s], [-s, c]], o = (n-1)/2 - R (n-1)/2, with the order-3 B-spline
    of the samples (no prefilter) and edge-replicated indices; float64 inside, float32 out."""
    a = np.asarray(a, dtype=np.float32)
    H, W = a.shape
    r = float(angle) % 360.0
    exact = {0.0: (1.0, 0.0), 90.0: (0.0, 1.0), 180.0: (-1.0, 0.0), 270.0: (0.0, -1.0)}
    c, s = exact.get(r, (np.cos(np.deg2rad(angle)), np.sin(np.deg2rad(angle))))
    ch, cw = (H - 1) / 2.0, (W - 1) / 2.0
    o0, o1 = ch - (c * ch + s * cw), cw - (-s * ch + c * cw)
    i, j = np.meshgrid(np.arange(H, dtype=np.float64), np.arange(W, dtype=np.float64),
                       indexing="ij")
    x, y = c * i + s * j + o0, -s * i + c * j + o1
    i0, j0 = np.floor(x).astype(np.int64) - 1, np.floor(y).astype(np.int64) - 1
    acc = np.zeros((H, W))
    for p in range(4):
        wx = _bspline3(x - (i0 + p))
        ii = np.clip(i0 + p, 0, H - 1)
        for q in range(4):
            jj = np.clip(j0 + q, 0, W - 1)
            acc += wx * _bspline3(y - (j0 + q)) * a[ii, jj]
    return acc.astype(np.float32)
