"""ctypes binding of ``libcardiax_gb300.so`` (the C ABI of ``include/cardiax_gb300.h``).

There is no CPU implementation behind these calls: if the library is missing or no CUDA device
is present, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

# include/cardiax_gb300.h: stimuli per call, and stimuli active at once within one launch
FK_MAX_STIMULI = 64
FK_MAX_ACTIVE_STIMULI = 8


class FkError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib().fk_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (status {status})")


class Grid(ctypes.Structure):
    _fields_ = [("H", ctypes.c_int64), ("W", ctypes.c_int64), ("pitch", ctypes.c_int64)]


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in (
        "tau_v_plus", "tau_v1_minus", "tau_v2_minus", "tau_w_plus", "tau_w_minus", "tau_d",
        "tau_0", "tau_r", "tau_si", "k", "V_csi", "V_c", "V_v", "Cm")]


class Stimulus(ctypes.Structure):
    _fields_ = [("start", ctypes.c_double), ("duration", ctypes.c_double),
                ("period", ctypes.c_double), ("field", ctypes.c_void_p),
                ("r0", ctypes.c_int32), ("r1", ctypes.c_int32), ("c0", ctypes.c_int32),
                ("c1", ctypes.c_int32), ("amplitude", ctypes.c_float)]


class Activation(ctypes.Structure):
    _fields_ = [("first", ctypes.c_void_p), ("last", ctypes.c_void_p), ("count", ctypes.c_void_p),
                ("threshold", ctypes.c_float)]


class TissueDesc(ctypes.Structure):
    _fields_ = [("g", Grid), ("state", ctypes.c_void_p), ("scratch", ctypes.c_void_p),
                ("D", ctypes.c_void_p), ("params", Params),
                ("stimuli", ctypes.POINTER(Stimulus)), ("n_stimuli", ctypes.c_int),
                ("dt", ctypes.c_double), ("dx", ctypes.c_double), ("act", Activation)]


_lib = None
_lock = threading.Lock()
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int

# name -> argtypes (all return int status)
_SIGNATURES = {
    "fk_device_status": [_INT, ctypes.POINTER(_INT)],
    "fk_select_step_kernel": [_INT],
    "fk_selftest_wait_timeout": [_I64, _P],
    "fk_init": [Grid, _P, _P],
    "fk_step": [Grid, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT, _I64, _D,
                _P, _P],
    "fk_euler_step": [Grid, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT, _I64,
                      _D, _D, _P, _P],
    "fk_forward_euler": [Grid, _P, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT,
                         _I64, _I64, _D, _D, _P],
    "fk_forward": [Grid, _P, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT,
                   ctypes.POINTER(_I64), _INT, _D, _D, _P, _P],
    "fk_forward_euler_tracked": [Grid, _P, _P, _P, ctypes.POINTER(Params),
                                 ctypes.POINTER(Stimulus), _INT, _I64, _I64, _D, _D,
                                 ctypes.POINTER(Activation), _P],
    "fk_forward_euler_flow": [Grid, _P, _P, _P, _P, ctypes.POINTER(Params),
                              ctypes.POINTER(Stimulus), _INT, _I64, _I64, _D, _D,
                              ctypes.POINTER(Activation), _P, _I64, _P],
    "fk_forward_euler_tb": [Grid, _P, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus),
                            _INT, _I64, _I64, _D, _D, _INT, _P],
    "fk_forward_flow": [Grid, _P, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT,
                        ctypes.POINTER(_I64), _INT, _D, _D, _P, _P, _I64, _P],
    "fk_heun_step": [Grid, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT, _I64,
                     _D, _D, _P, _P, _P],
    "fk_forward_heun": [Grid, _P, _P, _P, ctypes.POINTER(Params), ctypes.POINTER(Stimulus), _INT,
                        _I64, _I64, _D, _D, _P],
    "fk_resize_bilinear": [_P, _I64, _I64, _I64, _I64, _P, _I64, _I64, _I64, _INT, _P],
    "fk_rotate_field": [_P, _I64, _I64, _I64, _P, _I64, _D, _P],
    "fk_scar_raster": [_P, _P, _P, _I64, _I64, _I64, _P, _I64, _P, _P],
    "fk_conv2d_same": [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _INT, _P],
    "fk_batch_create": [ctypes.POINTER(TissueDesc), _INT, _P, ctypes.c_size_t, _P,
                        ctypes.POINTER(_P)],
    "fk_batch_forward_euler": [_P, _I64, _I64, _INT, _P],
    "fk_batch_set_grid": [_P, _INT],
    "fk_batch_set_tile_rows": [_P, _INT],
    "fk_batch_set_options": [_P, _INT, _INT],
    "fk_batch_set_depth": [_P, _INT],
    "fk_batch_destroy": [_P],
}


def lib_path() -> str:
    return _build.LIB


def lib(build: bool = True):
    """The loaded library (built first when it is missing or older than its sources)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build() if build else _build.LIB
            if not os.path.exists(path):
                raise RuntimeError(f"CUDA library not built: {path}")
            L = ctypes.CDLL(path)
            L.fk_status_string.restype = ctypes.c_char_p
            L.fk_status_string.argtypes = [_INT]
            for name, args in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = _INT
                fn.argtypes = args
            L.fk_batch_workspace_bytes.restype = ctypes.c_size_t
            L.fk_batch_workspace_bytes.argtypes = [ctypes.POINTER(TissueDesc), _INT]
            L.fk_flow_flag_words.restype = _I64
            L.fk_flow_flag_words.argtypes = [Grid]
            _lib = L
    return _lib


def call(name: str, *args) -> None:
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        raise FkError(rc, name)


def exported_symbols():
    return (["fk_status_string", "fk_batch_workspace_bytes", "fk_flow_flag_words"]
            + list(_SIGNATURES))
