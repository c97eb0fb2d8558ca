"""cardiax_gb300: a GB300-native Fenton-Karma reaction-diffusion stepper.

A drop-in for the forward path of epignatelli/cardiax (``cardiax.solve``): hand-written sm_103a
CUDA kernels behind a C ABI (``include/cardiax_gb300.h``), driven from Python through ctypes on
torch CUDA tensors and streams, and registered as PyTorch operators
(``torch.ops.cardiax_gb300.*``, :mod:`cardiax_gb300.ops`).
"""
from . import convert, params, stimulus  # noqa: F401
from . import generate, io, ops, scars, solve  # noqa: F401
from .tissue import Tissue  # noqa: F401

__all__ = ["convert", "generate", "io", "ops", "params", "scars", "stimulus", "solve", "Tissue"]
