"""Load the reference's own ``deepx/utils_scars.py`` with NumPy stand-ins for JAX and skimage.

``utils_scars.py`` imports JAX (PRNG, ``jax.numpy``, ``jax.scipy.signal.convolve2d``), SciPy
(``interpolate.splprep``/``splev``, used as is) and ``skimage.draw.polygon``; neither JAX nor
skimage is installed here.  The stand-ins:

* ``jax.random``: keys are placeholders and every ``normal`` / ``uniform`` / ``randint`` call
  takes the next value from a scripted tape (:class:`Tape`), checking the kind and the shape, so
  the reference's code runs with chosen draws in its own call order;
* ``jax.numpy``: NumPy with JAX's x64-off typing (float64 inputs become float32, Python scalars
  are weakly typed) and an ``.at[...].set`` that, like XLA's scatter, drops out-of-range indices;
* ``jax.scipy.signal.convolve2d``: SciPy's, evaluated in float64 and rounded to float32;
* ``skimage.draw.polygon``: the cells of the vertices' bounding box whose centre passes
  PNPOLY's crossing test (W. R. Franklin), one cell at a time in float64.

Test infrastructure for ``make_scar_golden.py`` only; nothing on the product path imports it.
"""
from __future__ import annotations

import importlib.util
import math
import os
import sys
import types

import numpy as np
from scipy.signal import convolve2d as _sp_convolve2d

# the reference checkout: set CARDIAX_REFERENCE (there is no default location)
REFERENCE_ROOT = os.environ.get("CARDIAX_REFERENCE")


class Tape:
    """Scripted draws: a list of (kind, shape, values) consumed in order."""

    def __init__(self, items):
        self.items = list(items)
        self.pos = 0

    def take(self, kind, shape):
        if self.pos >= len(self.items):
            raise RuntimeError(f"tape exhausted at a {kind}{shape} draw")
        k, s, v = self.items[self.pos]
        if k != kind or tuple(s) != tuple(shape):
            raise RuntimeError(f"draw {self.pos}: tape has {k}{s}, code asks {kind}{shape}")
        self.pos += 1
        return v


class JArr(np.ndarray):
    """An ndarray with JAX's functional ``.at[idx].set(v)``."""

    @property
    def at(self):
        arr = self

        class _At:
            def __getitem__(self, idx):
                class _Set:
                    def set(self, value):
                        out = np.array(arr, copy=True).view(JArr)
                        ix = idx
                        if isinstance(ix, tuple) and all(
                                isinstance(i, np.ndarray) and i.dtype.kind in "iu" for i in ix):
                            keep = np.ones(ix[0].shape, bool)
                            for ax, i in enumerate(ix):
                                keep &= (i >= 0) & (i < out.shape[ax])
                            ix = tuple(i[keep] for i in ix)
                        out[ix] = value
                        return out
                return _Set()
        return _At()


def _j(x, dtype=None):
    a = np.asarray(x, dtype=dtype)
    if a.dtype == np.float64:
        a = a.astype(np.float32)
    elif a.dtype == np.int64:
        a = a.astype(np.int32)
    return a.view(JArr)


def _scalar(v):
    a = np.asarray(v)
    return a.reshape(()).item() if a.size == 1 else v


def _make_jnp():
    jnp = types.ModuleType("jax.numpy")
    jnp.pi = np.pi
    jnp.finfo = np.finfo
    jnp.ndarray = np.ndarray

    def arange(start, stop=None, step=None, dtype=None):
        start = _scalar(start)
        stop = None if stop is None else _scalar(stop)
        step = None if step is None else _scalar(step)
        args = [x for x in (start, stop, step) if x is not None]
        if dtype is None:
            dtype = np.float32 if any(isinstance(x, float) for x in args) else np.int32
        if stop is None:
            return np.arange(start, dtype=dtype).view(JArr)
        return np.arange(start, stop, step, dtype=dtype).view(JArr)

    def zeros(shape, dtype=None):
        if dtype in (None, float):
            dtype = np.float32
        return np.zeros(shape, dtype).view(JArr)

    def meshgrid(*xs, **k):
        return [m.view(JArr) for m in np.meshgrid(*[np.asarray(x) for x in xs], **k)]

    def power(a, b):
        a = _j(a)
        if isinstance(b, int):  # lax.integer_pow: repeated multiplication
            out = np.ones_like(a)
            for _ in range(b):
                out = (out * a).astype(a.dtype)
            return out.view(JArr)
        return np.power(a, b).view(JArr)

    def clip(a, a_min=None, a_max=None):
        return np.clip(_j(a), a_min, a_max).view(JArr)

    jnp.arange, jnp.zeros, jnp.meshgrid, jnp.power, jnp.clip = arange, zeros, meshgrid, power, clip
    jnp.array = lambda x, dtype=None: _j(x, dtype)
    jnp.asarray = jnp.array
    for name in ("exp", "sin", "cos", "abs", "ceil"):
        f = getattr(np, name)
        setattr(jnp, name, (lambda f: lambda x: f(_j(x)).view(JArr))(f))
    jnp.mean = lambda x: np.mean(_j(x))
    jnp.argmin = lambda x: int(np.argmin(np.asarray(x)))
    jnp.where = lambda *a: np.where(*a)
    return jnp


def _make_random(tape: Tape):
    rnd = types.ModuleType("jax.random")

    def split(key, num=2):
        return tuple(("key", key, i) for i in range(num))

    def normal(key, shape=()):
        return _j(np.asarray(tape.take("normal", shape), np.float32).reshape(shape))

    def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
        return _j(np.asarray(tape.take("uniform", shape), np.float32).reshape(shape))

    def randint(key, shape, minval, maxval):
        v = np.asarray(tape.take("randint", shape), np.int32).reshape(shape)
        assert np.all((v >= minval) & (v < maxval))
        return v.view(JArr)

    rnd.split, rnd.normal, rnd.uniform, rnd.randint = split, normal, uniform, randint
    rnd.PRNGKey = lambda seed: ("key", seed)
    return rnd


def _polygon(r, c, shape=None):
    """skimage.draw.polygon: bounding box, PNPOLY per cell centre, float64."""
    r = np.asarray(r, np.float64)
    c = np.asarray(c, np.float64)
    minr, maxr = int(max(0, r.min())), int(math.ceil(r.max()))
    minc, maxc = int(max(0, c.min())), int(math.ceil(c.max()))
    if shape is not None:
        maxr, maxc = min(shape[0] - 1, maxr), min(shape[1] - 1, maxc)
    xp, yp = c.tolist(), r.tolist()
    n = len(xp)
    rr, cc = [], []
    for ri in range(minr, maxr + 1):
        y = float(ri)
        crossings = []
        j = n - 1
        for i in range(n):
            if (yp[i] <= y < yp[j]) or (yp[j] <= y < yp[i]):
                crossings.append((xp[j] - xp[i]) * (y - yp[i]) / (yp[j] - yp[i]) + xp[i])
            j = i
        for ci in range(minc, maxc + 1):
            x = float(ci)
            inside = False
            for xc in crossings:
                if x < xc:
                    inside = not inside
            if inside:
                rr.append(ri)
                cc.append(ci)
    return np.array(rr, dtype=np.intp), np.array(cc, dtype=np.intp)


def load_utils_scars(tape: Tape, root: str = REFERENCE_ROOT):
    """The reference's ``deepx/utils_scars.py`` module, bound to the scripted ``tape``."""
    if not root:
        raise FileNotFoundError("no reference checkout: set CARDIAX_REFERENCE or pass root")
    path = os.path.join(root, "deepx", "utils_scars.py")
    if not os.path.isfile(path):
        raise FileNotFoundError(f"reference checkout not found under {root}")
    jax = types.ModuleType("jax")
    jax.__path__ = []
    jax.numpy = _make_jnp()
    jax.random = _make_random(tape)
    jsp = types.ModuleType("jax.scipy")
    jsp.__path__ = []
    sig = types.ModuleType("jax.scipy.signal")
    sig.convolve2d = lambda a, b, mode="full": _j(_sp_convolve2d(
        np.asarray(a, np.float64), np.asarray(b, np.float64), mode)).astype(np.float32)
    jsp.signal = sig
    jax.scipy = jsp
    sk = types.ModuleType("skimage")
    sk.__path__ = []
    draw = types.ModuleType("skimage.draw")
    draw.polygon = _polygon
    sk.draw = draw
    mods = {"jax": jax, "jax.numpy": jax.numpy, "jax.random": jax.random, "jax.scipy": jsp,
            "jax.scipy.signal": sig, "skimage": sk, "skimage.draw": draw}
    saved = {k: sys.modules.get(k) for k in mods}
    sys.modules.update(mods)
    try:
        spec = importlib.util.spec_from_file_location("_ref_utils_scars", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod
