"""Device-resident tissue: the prepared inputs of the stepper and its state buffers.

A :class:`Tissue` holds, in the layout the kernels read (float32 planes with a row pitch that is
a multiple of 4 floats):

* ``state``   -- (3, H, pitch): v, w, u (the reference's State order, cardiax/solve.py:12-15)
* ``scratch`` -- a second state buffer for the ping-pong between steps
* ``D``       -- (H, pitch) diffusivity
* the stimulus table: constant rectangles as descriptors, other fields as pitched planes

and advances it through the C ABI on the current torch CUDA stream.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _native as N


def pitch_of(W: int) -> int:
    return (int(W) + 3) // 4 * 4


def _device(device=None) -> torch.device:
    if device is not None:
        d = torch.device(device)
        if d.type != "cuda":
            raise ValueError("cardiax_gb300 runs on CUDA devices only")
        return d
    if not torch.cuda.is_available():
        raise RuntimeError("cardiax_gb300 needs a CUDA device (there is no CPU path)")
    return torch.device("cuda", torch.cuda.current_device())


def as_cuda_f32(x, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float32)
    return torch.as_tensor(np.asarray(x, dtype=np.float32), device=device)


def to_pitched(plane, H: int, W: int, pitch: int, device) -> torch.Tensor:
    """An (H, pitch) float32 copy of an (H, W) array (zero in the padding columns), or the
    tensor itself when it already has that layout."""
    t = as_cuda_f32(plane, device)
    if tuple(t.shape) != (H, W):
        raise ValueError(f"expected shape {(H, W)}, got {tuple(t.shape)}")
    if pitch == W and t.is_contiguous() and t.data_ptr() % 16 == 0:
        return t
    out = torch.zeros((H, pitch), dtype=torch.float32, device=device)
    out[:, :W] = t
    return out


def _scalar(x) -> float:
    return float(np.asarray(x if not isinstance(x, torch.Tensor) else x.detach().cpu(),
                            dtype=np.float64).reshape(-1)[0])


def params_struct(params) -> N.Params:
    vals = [float(_scalar(v)) for v in params]
    if len(vals) != 14:
        raise ValueError("params must have the 14 fields of cardiax Params")
    return N.Params(*vals)


def analyse_field(field: torch.Tensor):
    """Classifies a stimulus field: ``("empty",)`` (all zero), ``("rect", r0, r1, c0, c1, a)``
    (a constant ``a`` on a rectangle, zero elsewhere) or ``("dense",)``.  Runs a few reductions
    on the device and one synchronisation (set-up cost, once per tissue)."""
    nz = field != 0
    rows = torch.nonzero(nz.any(1)).flatten()
    if rows.numel() == 0:
        return ("empty",)
    cols = torch.nonzero(nz.any(0)).flatten()
    r0, r1 = int(rows[0]), int(rows[-1]) + 1
    c0, c1 = int(cols[0]), int(cols[-1]) + 1
    box = field[r0:r1, c0:c1]
    a = box[0, 0]
    if bool((box == a).all()):
        return ("rect", r0, r1, c0, c1, float(a))
    return ("dense",)


def stimulus_table(stimuli: Sequence, H: int, W: int, pitch: int, device):
    """The C stimulus table for ``stimuli`` (sequence of cardiax-style Stimulus), plus the
    device buffers it points to (kept alive by the caller)."""
    entries, keep = [], []
    for s in stimuli:
        proto, field = s[0], s[1]
        start, duration, period = (_scalar(proto[0]), _scalar(proto[1]), _scalar(proto[2]))
        f = as_cuda_f32(field, device)
        if tuple(f.shape) != (H, W):
            raise ValueError(f"stimulus field shape {tuple(f.shape)} != grid {(H, W)}")
        kind = analyse_field(f)
        if kind[0] == "empty":
            continue  # a zero field never replaces the current
        if kind[0] == "rect":
            _, r0, r1, c0, c1, a = kind
            entries.append(N.Stimulus(start, duration, period, None, r0, r1, c0, c1, a))
        else:
            p = to_pitched(f, H, W, pitch, device)
            keep.append(p)
            entries.append(N.Stimulus(start, duration, period, p.data_ptr(), 0, 0, 0, 0, 0.0))
    if len(entries) > N.FK_MAX_STIMULI:
        raise ValueError(f"at most {N.FK_MAX_STIMULI} non-zero stimuli are supported per tissue "
                         f"(of which at most {N.FK_MAX_ACTIVE_STIMULI} active at one step)")
    arr = (N.Stimulus * max(1, len(entries)))(*entries)
    return arr, len(entries), keep


def stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


class Tissue:
    """A tissue prepared for stepping on one CUDA device."""

    def __init__(self, shape, params, diffusivity, stimuli=(), dt: float = 0.01,
                 dx: float = 0.01, device=None):
        self.device = _device(device)
        H, W = int(shape[0]), int(shape[1])
        if H < 3 or W < 3:
            raise ValueError("the stencil needs at least 3 cells along each axis")
        self.H, self.W, self.pitch = H, W, pitch_of(W)
        self.grid = N.Grid(H, W, self.pitch)
        self.params = params_struct(params)
        self.dt, self.dx = float(dt), float(dx)
        with torch.cuda.device(self.device):
            self.D = to_pitched(diffusivity, H, W, self.pitch, self.device)
            self.stim, self.n_stim, self._keep = stimulus_table(stimuli, H, W, self.pitch,
                                                                self.device)
            self.state = torch.empty((3, H, self.pitch), dtype=torch.float32, device=self.device)
            self.scratch = torch.empty_like(self.state)
        self.activation = None
        self._batches = {}  # one-tissue batch plans by tile rows (schedule="batch")
        self.init()

    # -- state ----------------------------------------------------------------------------
    def init(self):
        """v = w = 1, u = 0 (cardiax/solve.py:18-23)."""
        N.call("fk_init", self.grid, self.state.data_ptr(), stream_handle())
        return self

    def set_state(self, state) -> "Tissue":
        """Copies a (v, w, u) triple of (H, W) arrays into the device state."""
        for k in range(3):
            self.state[k, :, :self.W] = as_cuda_f32(state[k], self.device)
        return self

    def view(self, buf: torch.Tensor = None):
        """(v, w, u) views of a (…, 3, H, pitch) buffer without the padding columns."""
        buf = self.state if buf is None else buf
        return buf[..., 0, :, :self.W], buf[..., 1, :, :self.W], buf[..., 2, :, :self.W]

    def track_activation(self, threshold: float = 0.5) -> "Tissue":
        """Records activation times during ``advance``: an upstroke of u through ``threshold``
        during step t -> t+1 is recorded as t+1 in ``act_first`` (first one), ``act_last`` (most
        recent) and counted in ``act_count`` (int32 (H, pitch) planes; -1 / 0 when none)."""
        kw = dict(dtype=torch.int32, device=self.device)
        self.act_first = torch.full((self.H, self.pitch), -1, **kw)
        self.act_last = torch.full((self.H, self.pitch), -1, **kw)
        self.act_count = torch.zeros((self.H, self.pitch), **kw)
        self.activation = N.Activation(self.act_first.data_ptr(), self.act_last.data_ptr(),
                                       self.act_count.data_ptr(), float(threshold))
        self._drop_batches()  # their plans were built without tracking
        return self

    def _drop_batches(self):
        for b in self._batches.values():
            b.close()
        self._batches = {}

    def activation_maps(self):
        """(first, last, count) activation maps without the padding columns."""
        W = self.W
        return self.act_first[:, :W], self.act_last[:, :W], self.act_count[:, :W]

    # -- stepping -------------------------------------------------------------------------
    def _flow_flags(self) -> torch.Tensor:
        """Tile-progress words of the dataflow kernel (owned by this tissue; its calls are
        ordered on one stream)."""
        if getattr(self, "_flags", None) is None:
            n = int(N.lib().fk_flow_flag_words(self.grid))
            self._flags = torch.zeros(n, dtype=torch.int32, device=self.device)
        return self._flags

    def _one_batch(self, tile_rows: int):
        """A batch plan holding this tissue alone, with ``tile_rows`` x 64 work items (kept
        until activation tracking changes)."""
        from .batch import TissueBatch
        b = self._batches.get(tile_rows)
        if b is None:
            b = TissueBatch([self], tile_rows=tile_rows)
            self._batches[tile_rows] = b
        return b

    def advance(self, t0: int, t1: int, schedule: str = "step", depth: int = 1,
                tile_rows: int = 16) -> "Tissue":
        """Steps t0 .. t1-1 in place (cardiax/solve.py:92-100).  ``schedule="step"``: one launch
        per step (chained with programmatic dependent launch), or with ``depth`` 2, 4 or 8 that
        many steps per launch (temporal blocking); ``"flow"``: one cooperative dataflow launch
        for the whole range; ``"batch"``: the batched kernel on this tissue alone, with
        ``tile_rows`` x 64 work items (16-row items put twice the CTAs on a small grid and
        shorten each step's critical path) and CUDA-graph replay; ``"auto"``: whichever of these
        (and of the tiled and strip step kernels) ``autotune.tune_tissue`` measured fastest on
        this grid.  All give identical results.  With more stimuli than one launch holds
        (``FK_MAX_ACTIVE_STIMULI``) each launch takes the stimuli that can be active during its
        steps, so ``"flow"``, ``"batch"`` and ``"auto"`` step one launch per step instead."""
        if self.n_stim > N.FK_MAX_ACTIVE_STIMULI and schedule in ("flow", "batch", "auto"):
            schedule, depth = "step", 1
        if schedule == "batch":
            self._one_batch(int(tile_rows)).advance(t0, t1)
            return self
        if schedule == "auto":
            from . import autotune
            autotune._run(self, t0, t1, autotune.tune_tissue(self)["choice"])
            return self
        act = ctypes.byref(self.activation) if self.activation is not None else None
        if schedule == "step" and depth != 1:
            if act is not None:
                raise ValueError("activation tracking runs one step per launch (depth=1)")
            N.call("fk_forward_euler_tb", self.grid, self.state.data_ptr(),
                   self.scratch.data_ptr(), self.D.data_ptr(), ctypes.byref(self.params),
                   self.stim, self.n_stim, int(t0), int(t1), self.dt, self.dx, int(depth),
                   stream_handle())
            return self
        if schedule == "step":
            N.call("fk_forward_euler_tracked", self.grid, self.state.data_ptr(),
                   self.scratch.data_ptr(), self.D.data_ptr(), ctypes.byref(self.params),
                   self.stim, self.n_stim, int(t0), int(t1), self.dt, self.dx, act,
                   stream_handle())
            return self
        if schedule != "flow":
            raise ValueError(f"unknown schedule {schedule!r}")
        flags = self._flow_flags()
        N.call("fk_forward_euler_flow", self.grid, self.state.data_ptr(), self.state.data_ptr(),
               self.scratch.data_ptr(), self.D.data_ptr(), ctypes.byref(self.params), self.stim,
               self.n_stim, int(t0), int(t1), self.dt, self.dx, act, flags.data_ptr(),
               flags.numel(), stream_handle())
        return self

    def advance_heun(self, t0: int, t1: int) -> "Tissue":
        """Heun steps t0 .. t1-1 in place (cardiax/solve.py:103-111)."""
        if getattr(self, "_heun_work", None) is None:
            self._heun_work = torch.empty((4,) + tuple(self.state.shape), dtype=torch.float32,
                                          device=self.device)
        N.call("fk_forward_heun", self.grid, self.state.data_ptr(), self._heun_work.data_ptr(),
               self.D.data_ptr(), ctypes.byref(self.params), self.stim, self.n_stim, int(t0),
               int(t1), self.dt, self.dx, stream_handle())
        return self

    def forward(self, checkpoints, out: torch.Tensor = None,
                schedule: str = "step") -> torch.Tensor:
        """States at checkpoints[1:] starting from the current state, as a
        (len-1, 3, H, pitch) tensor (cardiax/solve.py:168-222).  The current state is not
        modified.  ``schedule`` as in :meth:`advance`."""
        ck = [int(_scalar(c)) for c in checkpoints]
        n = max(0, len(ck) - 1)
        if out is None:
            out = torch.empty((n, 3, self.H, self.pitch), dtype=torch.float32,
                              device=self.device)
        if n == 0:
            return out
        arr = (ctypes.c_int64 * len(ck))(*ck)
        if schedule == "step" or self.n_stim > N.FK_MAX_ACTIVE_STIMULI:
            N.call("fk_forward", self.grid, self.state.data_ptr(), self.scratch.data_ptr(),
                   self.D.data_ptr(), ctypes.byref(self.params), self.stim, self.n_stim, arr,
                   len(ck), self.dt, self.dx, out.data_ptr(), stream_handle())
            return out
        if schedule != "flow":
            raise ValueError(f"unknown schedule {schedule!r}")
        flags = self._flow_flags()
        N.call("fk_forward_flow", self.grid, self.state.data_ptr(), self.scratch.data_ptr(),
               self.D.data_ptr(), ctypes.byref(self.params), self.stim, self.n_stim, arr,
               len(ck), self.dt, self.dx, out.data_ptr(), flags.data_ptr(), flags.numel(),
               stream_handle())
        return out

    def derivative(self, t: int, out: torch.Tensor = None) -> torch.Tensor:
        """d/dt of the current state at step t (cardiax/solve.py:26-65)."""
        out = torch.empty_like(self.state) if out is None else out
        N.call("fk_step", self.grid, self.state.data_ptr(), self.D.data_ptr(),
               ctypes.byref(self.params), self.stim, self.n_stim, int(t), self.dx,
               out.data_ptr(), stream_handle())
        return out

    def euler_step(self, t: int, out: torch.Tensor = None) -> torch.Tensor:
        """One Euler step of the current state at step t into ``out`` (cardiax/solve.py:68-70)."""
        out = torch.empty_like(self.state) if out is None else out
        N.call("fk_euler_step", self.grid, self.state.data_ptr(), self.D.data_ptr(),
               ctypes.byref(self.params), self.stim, self.n_stim, int(t), self.dt, self.dx,
               out.data_ptr(), stream_handle())
        return out
