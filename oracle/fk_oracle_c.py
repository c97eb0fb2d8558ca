"""ctypes binding of the C oracle (``oracle/fk_oracle.c``) -- TEST INFRASTRUCTURE ONLY.

Used by the tests (large-grid checks) and by ``bench.py``'s CPU-baseline leg.  The C code
restates cardiax/solve.py:26-100,225-271 in the reference's evaluation order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "libfk_oracle.so")
_lib = None


class _Stim(ctypes.Structure):
    _fields_ = [("start", ctypes.c_double), ("duration", ctypes.c_double),
                ("period", ctypes.c_double), ("field", ctypes.c_void_p)]


def build(force: bool = False) -> str:
    """Compile the C oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(_LIB) or \
            os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "fk_oracle.c")):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", _HERE, "libfk_oracle.so"],
                       check=True)
    return _LIB


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB)
        for name, T in (("fko_forward_euler_f32", ctypes.c_float),
                        ("fko_forward_euler_f64", ctypes.c_double)):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_long, ctypes.c_long,
                                                   ctypes.POINTER(ctypes.c_double),
                                                   ctypes.POINTER(_Stim), ctypes.c_int,
                                                   ctypes.c_long, ctypes.c_long,
                                                   ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                   ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_double]
        lib.fko_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def max_threads() -> int:
    return int(_load().fko_max_threads())


def forward_euler(state, t0, t1, params, diffusivity, stimuli, dt, dx, threads: int = 1,
                  activation=None):
    """Advance ``state`` = (v, w, u) from step t0 to t1; returns new arrays (v, w, u).

    ``stimuli``: sequence of (start, duration, period, field) in steps.  The working type is the
    dtype of ``state`` (float32 or float64).  ``activation``: optional (first, last, count,
    threshold) with int32 (H, W) arrays updated in place -- an upstroke of u through the threshold
    during step s -> s+1 records time s+1.
    """
    lib = _load()
    dtype = np.dtype(state[0].dtype)
    fn = lib.fko_forward_euler_f32 if dtype == np.float32 else lib.fko_forward_euler_f64
    v, w, u = (np.ascontiguousarray(x, dtype=dtype).copy() for x in state)
    D = np.ascontiguousarray(diffusivity, dtype=dtype)
    H, W = u.shape
    prm = (ctypes.c_double * 14)(*[float(x) for x in params])
    fields = [np.ascontiguousarray(s[3], dtype=dtype) for s in stimuli]
    arr = (_Stim * max(1, len(stimuli)))()
    for i, s in enumerate(stimuli):
        arr[i] = _Stim(float(s[0]), float(s[1]), float(s[2]), fields[i].ctypes.data)
    if activation is not None:
        first, last, count, thr = activation
        for a in (first, last, count):
            assert a.dtype == np.int32 and a.flags.c_contiguous and a.shape == (H, W)
        act = (first.ctypes.data, last.ctypes.data, count.ctypes.data, float(thr))
    else:
        act = (None, None, None, 0.0)
    rc = fn(v.ctypes.data, w.ctypes.data, u.ctypes.data, D.ctypes.data, H, W, prm, arr,
            len(stimuli), int(t0), int(t1), float(dt), float(dx), int(threads), *act)
    if rc != 0:
        raise RuntimeError(f"C oracle failed with status {rc}")
    return v, w, u
