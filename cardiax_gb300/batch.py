"""Many tissues advanced together: one persistent kernel per step over the tiles of all tissues,
runs of steps replayed from a captured CUDA graph (``fk_batch_*`` in the C ABI).

The reference has no counterpart (its data generation steps one tissue per call and loops in
Python, deepx/generate.py:135-210).  Per tissue the result is bit-identical to
:meth:`cardiax_gb300.Tissue.advance`.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _native as N
from .tissue import Tissue, stream_handle


class TissueBatch:
    """A batch of :class:`Tissue` objects on one device (shapes, parameters, D maps, stimuli and
    dt/dx may all differ).  ``advance(t0, t1)`` steps every tissue in place."""

    def __init__(self, tissues: Sequence[Tissue], graph_steps: int = 64, ctas: int = None,
                 tile_rows: int = 32):
        if not tissues:
            raise ValueError("empty batch")
        dev = tissues[0].device
        if any(t.device != dev for t in tissues):
            raise ValueError("all tissues of a batch must live on one device")
        tracked = [t.activation is not None for t in tissues]
        if any(tracked) and not all(tracked):
            raise ValueError("activation tracking must be on for all tissues of a batch or none")
        self.tissues = list(tissues)
        self.device = dev
        self.graph_steps = int(graph_steps)
        descs = (N.TissueDesc * len(tissues))()
        for k, t in enumerate(tissues):
            act = t.activation if t.activation is not None else N.Activation(None, None, None, 0.0)
            descs[k] = N.TissueDesc(t.grid, t.state.data_ptr(), t.scratch.data_ptr(),
                                    t.D.data_ptr(), t.params, t.stim, t.n_stim, t.dt, t.dx, act)
        self._descs = descs
        L = N.lib()
        nbytes = L.fk_batch_workspace_bytes(descs, len(tissues))
        with torch.cuda.device(dev):
            self.workspace = torch.empty(nbytes + 128, dtype=torch.uint8, device=dev)
        base = (self.workspace.data_ptr() + 127) // 128 * 128
        plan = ctypes.c_void_p()
        N.call("fk_batch_create", descs, len(tissues), base, nbytes, stream_handle(),
               ctypes.byref(plan))
        self._plan = plan
        self.tile_rows = 32
        self.interleave, self.packed = 1, False
        self.depth = 1
        if ctas is not None:
            self.set_ctas(ctas)
        if tile_rows != 32:
            self.set_tile_rows(tile_rows)

    def set_ctas(self, ctas: int) -> "TissueBatch":
        N.call("fk_batch_set_grid", self._plan, int(ctas))
        return self

    def set_options(self, interleave=True, packed: bool = False) -> "TissueBatch":
        """Work order and arithmetic of the batched kernel; same results.  ``interleave``:
        True or 1 -- CTAs take every G-th item of the work list; 2, 4 or 8 -- every G-th chunk
        of that many neighbouring items; False or 0 -- contiguous runs of the list.  ``packed``:
        packed two-cell or scalar FP32 arithmetic."""
        il = int(interleave) if not isinstance(interleave, bool) else int(interleave)
        N.call("fk_batch_set_options", self._plan, il, int(bool(packed)))
        self.interleave, self.packed = il, bool(packed)
        return self

    def set_depth(self, depth: int) -> "TissueBatch":
        """Euler steps per launch: 1, or 2 (the temporally blocked kernel: each 32 x 64 tile
        advanced two steps between one load and one store).  Depth 2 needs every tissue's last
        tile row and column to hold more than one cell and no activation tracking (raises
        FkError otherwise); the results do not change."""
        N.call("fk_batch_set_depth", self._plan, int(depth))
        self.depth = int(depth)
        return self

    def can_block(self) -> bool:
        """Whether depth 2 is available for this batch."""
        return (all(t.activation is None for t in self.tissues) and
                all(t.H % 32 != 1 and t.W % 64 != 1 for t in self.tissues))

    def set_tile_rows(self, rows: int) -> "TissueBatch":
        """Work items of ``rows`` x 64 cells (32 or 16); the results do not change."""
        N.call("fk_batch_set_tile_rows", self._plan, int(rows))
        self.tile_rows = int(rows)
        return self

    @property
    def cells(self) -> int:
        return sum(t.H * t.W for t in self.tissues)

    def advance(self, t0: int, t1: int, graph_steps: int = None) -> "TissueBatch":
        g = self.graph_steps if graph_steps is None else int(graph_steps)
        N.call("fk_batch_forward_euler", self._plan, int(t0), int(t1), g, stream_handle())
        return self

    def close(self):
        if getattr(self, "_plan", None):
            N.lib().fk_batch_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
