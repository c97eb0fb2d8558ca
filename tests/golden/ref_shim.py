"""Load the reference's own ``cardiax`` package with a NumPy stand-in for JAX.

The reference (epignatelli/cardiax) computes its Fenton-Karma stepper with JAX, which is not
installed here.  Its hot-path modules (``cardiax/solve.py``, ``cardiax/stimulus.py``,
``cardiax/convert.py``, ``cardiax/params.py``) only use a small slice of the JAX API, so this
module provides that slice on top of NumPy, with JAX's single-precision typing rules
(x64 disabled: ``jnp.ones`` is float32, Python scalars are weakly typed, boolean masks turn
into 0/1 in arithmetic) and then imports the reference's UNMODIFIED source files from the
reference checkout.  The reference's own expression trees therefore run operation for
operation, in float32 (or float64 with ``x64=True``, the equivalent of
``jax.config.update("jax_enable_x64", True)``).

This is test infrastructure: it is used only by ``make_golden.py`` (fixture generation) and by
an optional CPU test that runs when the reference checkout is present.  Nothing on the
product path imports it.

JAX API covered (everything that the four modules above touch on the forward path):
``jax.jit`` (identity), ``jax.tree_multimap``, ``jax.lax.slice_in_dim``,
``jax.lax.fori_loop``, ``jax.ops.index``/``index_update``, ``jax.numpy.{ones, zeros,
zeros_like, pad, greater_equal, tanh, concatenate, where, mod, add, arange}``.
"""
from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np

# the reference checkout: set CARDIAX_REFERENCE (there is no default location)
REFERENCE_ROOT = os.environ.get("CARDIAX_REFERENCE")


def _jbool_class(float_t):
    """A boolean mask class that behaves like JAX's bool arrays in arithmetic.

    JAX promotes ``bool`` with a weakly typed Python scalar or a float32 array to float32
    (x64 off).  NumPy would promote ``1 - mask`` to int64 and then to float64, so arithmetic
    on this subclass converts the mask to ``float_t`` 0/1 first.  Logical operators keep bool.
    """

    class _JBool(_JBoolBase):
        def _f(self):
            return np.asarray(self, dtype=float_t)

    return _JBool


class _JBoolBase(np.ndarray):
    def _f(self):
        raise NotImplementedError

    def __mul__(self, o):
        return self._f() * o

    def __rmul__(self, o):
        return o * self._f()

    def __sub__(self, o):
        return self._f() - o

    def __rsub__(self, o):
        return o - self._f()

    def __add__(self, o):
        return self._f() + o

    def __radd__(self, o):
        return o + self._f()

    def __truediv__(self, o):
        return self._f() / o

    def __rtruediv__(self, o):
        return o / self._f()


def _make_jnp(float_t, int_t):
    jbool = _jbool_class(float_t)
    jnp = types.ModuleType("jax.numpy")
    jnp.ndarray = np.ndarray

    def ones(shape, dtype=None):
        return np.ones(shape, dtype=dtype or float_t)

    def zeros(shape, dtype=None):
        return np.zeros(shape, dtype=dtype or float_t)

    def zeros_like(x, dtype=None):
        return np.zeros_like(x, dtype=dtype)

    def pad(x, width, mode="constant"):
        return np.pad(x, width, mode=mode)

    def greater_equal(a, b):
        r = np.greater_equal(a, b)
        if isinstance(r, np.ndarray) and r.ndim > 0:
            return r.view(jbool)
        return np.bool_(r)

    def tanh(x):
        return np.tanh(x)

    def concatenate(xs, axis=0):
        return np.concatenate([np.asarray(x) for x in xs], axis)

    def where(c, a, b):
        return np.where(np.asarray(c, dtype=bool) if np.asarray(c).dtype == bool
                        else np.asarray(c) != 0, a, b)

    def mod(a, b):
        # JAX evaluates Python scalars as weakly typed float32 (x64 off) when the
        # divisor is a float; integers stay integers.
        if isinstance(a, (float, np.floating)) or isinstance(b, (float, np.floating)):
            return np.mod(float_t(a), float_t(b))
        return np.mod(a, b)

    def add(a, b):
        return np.add(a, b)

    def arange(*a, **k):
        r = np.arange(*a, **k)
        if r.dtype.kind == "i":
            return r.astype(int_t)
        return r.astype(float_t)

    def array(x, dtype=None):
        return np.array(x, dtype=dtype)

    jnp.ones, jnp.zeros, jnp.zeros_like, jnp.pad = ones, zeros, zeros_like, pad
    jnp.greater_equal, jnp.tanh, jnp.concatenate = greater_equal, tanh, concatenate
    jnp.where, jnp.mod, jnp.add, jnp.arange, jnp.array = where, mod, add, arange, array
    jnp.float32 = np.float32
    return jnp


def _make_jax(float_t, int_t):
    jax = types.ModuleType("jax")
    jax.__path__ = []  # a package, so that "jax.numpy" / "jax.experimental" import

    def jit(fun=None, static_argnums=None, **_):
        if fun is None:
            return lambda f: f
        return fun

    def tree_multimap(f, tree, *rest):
        return type(tree)(*[f(*xs) for xs in zip(tree, *rest)])

    lax = types.ModuleType("jax.lax")

    def slice_in_dim(a, start_index, limit_index, stride=1, axis=0):
        idx = [slice(None)] * a.ndim
        idx[axis] = slice(start_index, limit_index, stride)
        return a[tuple(idx)]

    def fori_loop(lower, upper, body, init_val):
        # With float bounds (``forward`` passes ``float(checkpoints[i])``) JAX's loop index
        # is a float32; with integer bounds it is an int32.
        is_float = isinstance(lower, (float, np.floating))
        val = init_val
        for i in range(int(lower), int(upper)):
            val = body(float_t(i) if is_float else int_t(i), val)
        return val

    lax.slice_in_dim, lax.fori_loop = slice_in_dim, fori_loop

    ops = types.ModuleType("jax.ops")

    class _Index:
        def __getitem__(self, idx):
            return idx

    def index_update(x, idx, y):
        x = np.array(x, copy=True)
        x[idx] = y
        return x

    ops.index, ops.index_update = _Index(), index_update

    experimental = types.ModuleType("jax.experimental")
    experimental.__path__ = []
    ode = types.ModuleType("jax.experimental.ode")

    def odeint(*_a, **_k):  # not on the Euler path
        raise NotImplementedError("odeint is not part of the NumPy stand-in")

    ode.odeint = odeint
    experimental.ode = ode

    jax.jit, jax.tree_multimap, jax.lax, jax.ops = jit, tree_multimap, lax, ops
    jax.experimental = experimental
    jax.numpy = _make_jnp(float_t, int_t)
    return jax, {"jax": jax, "jax.numpy": jax.numpy, "jax.lax": lax, "jax.ops": ops,
                 "jax.experimental": experimental, "jax.experimental.ode": ode}


def load_reference(x64: bool = False, root: str = REFERENCE_ROOT):
    """Import the reference's ``cardiax`` hot-path modules under the NumPy stand-in.

    Returns a namespace with ``solve``, ``params``, ``stimulus`` and ``convert``.
    ``x64=True`` runs the same code in float64 (the reference with x64 enabled).
    """
    if not root:
        raise FileNotFoundError("no reference checkout: set CARDIAX_REFERENCE or pass root")
    if not os.path.isdir(os.path.join(root, "cardiax")):
        raise FileNotFoundError(f"reference checkout not found under {root}")
    float_t, int_t = (np.float64, np.int64) if x64 else (np.float32, np.int32)
    saved = {k: sys.modules.get(k) for k in list(sys.modules)
             if k == "cardiax" or k.startswith("cardiax.") or k == "jax" or k.startswith("jax.")
             or k.startswith("matplotlib")}
    for k in saved:
        sys.modules.pop(k, None)
    _, mods = _make_jax(float_t, int_t)
    sys.modules.update(mods)
    mpl = types.ModuleType("matplotlib")
    mpl.__path__ = []
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"], sys.modules["matplotlib.pyplot"] = mpl, plt
    pkg = types.ModuleType("cardiax")
    pkg.__path__ = [os.path.join(root, "cardiax")]
    sys.modules["cardiax"] = pkg
    # plotting and HDF5 I/O are off the stepper path; stand-ins keep solve.py importable
    for name in ("plot", "io"):
        m = types.ModuleType("cardiax." + name)
        sys.modules["cardiax." + name] = m
        setattr(pkg, name, m)
    ns = types.SimpleNamespace()
    try:
        for name in ("params", "convert", "stimulus", "solve"):
            setattr(ns, name, importlib.import_module("cardiax." + name))
    finally:
        for k in [k for k in sys.modules if k == "cardiax" or k.startswith("cardiax.")
                  or k == "jax" or k.startswith("jax.") or k.startswith("matplotlib")]:
            sys.modules.pop(k, None)
        for k, v in saved.items():
            if v is not None:
                sys.modules[k] = v
    return ns
