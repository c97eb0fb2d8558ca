"""Autotuners of the stepping configuration.

``tune_batch``: for a batch, times on the batch's own tissues every combination of the
temporal-block depth (one Euler step per launch, or two: the blocked kernel), and at depth 1
the batched kernel's tile geometry (work items of 32 x 64 or 16 x 64 cells), work order (the
CTAs deal the work list round-robin, or each takes a contiguous run of it) and arithmetic
(scalar or packed two-cell FP32), each with every ``graph_steps`` (how many steps one captured
CUDA graph replays), over a short run with CUDA events, and keeps the fastest.  Every
combination gives the same bits.

``tune_tissue``: for one tissue, times every way of taking its Euler steps -- the tiled step
kernel (32 x 64-cell tiles), the strip kernel (128-column strips walked row by row), the
temporally blocked kernel at depth k in {2, 4, 8} (k steps per launch), and the dataflow
schedule -- on the tissue's own grid, and keeps the fastest.  All of them produce the same bits,
so the choice changes only the speed (``Tissue.advance(..., schedule="auto")``).

Both restore the timed state afterwards and cache their choice per (device name, shapes) for the
process.
"""
from __future__ import annotations

import torch

from . import _native as N
from .batch import TissueBatch

_CACHE: dict = {}
_TISSUE_CACHE: dict = {}

# (schedule, depth, step kernel) candidates of tune_tissue; step kernel 0 = tiled, 1 = strip
# (schedule, depth, third): the step kernel (0 tiled, 1 strip) for "step" and "flow", the work
# item rows for "batch" (the batched kernel on the one tissue)
TISSUE_CANDIDATES = (("step", 1, 0), ("step", 1, 1), ("step", 2, 0), ("step", 4, 0),
                     ("step", 8, 0), ("flow", 1, 0), ("batch", 1, 16), ("batch", 1, 32))

GRAPH_CANDIDATES = (0, 64)
TILE_ROW_CANDIDATES = (32, 16)
# (work order, packed) of the batched kernel: round-robin single items (1) or chunks of 2 or 4
# neighbouring items, or contiguous runs (0); scalar or packed arithmetic
OPTION_CANDIDATES = ((1, False), (2, False), (4, False), (0, False), (1, True), (0, True))


def _signature(batch: TissueBatch):
    shapes = tuple(sorted((t.H, t.W) for t in batch.tissues))
    return (torch.cuda.get_device_name(batch.device), shapes)


DEPTH_CANDIDATES = (1, 2)


def _set_batch(batch: TissueBatch, cfg) -> None:
    depth, rows, (interleave, packed), g = cfg
    batch.set_depth(depth)
    batch.set_tile_rows(rows)
    batch.set_options(interleave, packed)
    batch.graph_steps = g


def tune_batch(batch: TissueBatch, trial_steps: int = 256, candidates=GRAPH_CANDIDATES,
               tile_rows=TILE_ROW_CANDIDATES, options=OPTION_CANDIDATES,
               depths=DEPTH_CANDIDATES, verbose: bool = False) -> dict:
    """Picks the depth, tile geometry, work order, arithmetic and ``graph_steps`` for ``batch``
    (set on it) and returns ``{"depth", "tile_rows", "interleave", "packed", "graph_steps",
    "ms_per_step": {(depth, rows, (interleave, packed), graph_steps): ms}}``; the tissues'
    states are restored.  Depth 2 is tried only when the batch can be blocked; its tiles are
    32 x 64 and it takes no work-order or arithmetic options."""
    depths = tuple(d for d in depths if d == 1 or batch.can_block())
    key = (_signature(batch), trial_steps, tuple(candidates), tuple(tile_rows), tuple(options),
           depths)
    if key in _CACHE:
        res = _CACHE[key]
        _set_batch(batch, res["choice"])
        return res
    saved = [(t.state.clone(), None if t.activation is None else
              (t.act_first.clone(), t.act_last.clone(), t.act_count.clone()))
             for t in batch.tissues]
    timings = {}
    configs = [(1, rows, tuple(opt), g) for rows in tile_rows for opt in options
               for g in candidates]
    configs += [(d, 32, (1, False), g) for d in depths if d != 1 for g in candidates]
    for cfg in configs:
        depth, rows, opt, g = cfg
        _set_batch(batch, cfg)
        batch.advance(0, 2, graph_steps=0)  # warm-up
        if g:
            batch.advance(0, g, graph_steps=g)  # captures the graph outside the timing
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        batch.advance(0, trial_steps, graph_steps=g)
        e1.record()
        torch.cuda.synchronize()
        timings[cfg] = e0.elapsed_time(e1) / trial_steps
        if verbose:
            print(f"autotune depth={depth} tile_rows={rows} interleave={opt[0]} "
                  f"packed={opt[1]} graph_steps={g}: {timings[cfg] * 1e3:.1f} us/step")
    for t, (st, act) in zip(batch.tissues, saved):
        t.state.copy_(st)
        if act is not None:
            t.act_first.copy_(act[0])
            t.act_last.copy_(act[1])
            t.act_count.copy_(act[2])
    best = min(timings, key=timings.get)
    _set_batch(batch, best)
    res = {"choice": best, "depth": best[0], "tile_rows": best[1], "interleave": best[2][0],
           "packed": best[2][1], "graph_steps": best[3], "ms_per_step": timings}
    _CACHE[key] = res
    return res


def _run(tis, t0: int, t1: int, choice) -> None:
    schedule, depth, kernel = choice
    if schedule == "batch":
        tis.advance(t0, t1, schedule="batch", tile_rows=kernel)
        return
    if kernel:
        N.call("fk_select_step_kernel", int(kernel))
    try:
        if schedule == "flow":
            tis.advance(t0, t1, schedule="flow")
        else:
            tis.advance(t0, t1, schedule="step", depth=depth)
    finally:
        if kernel:
            N.call("fk_select_step_kernel", 0)


def tune_tissue(tis, trial_steps: int = 64, candidates=TISSUE_CANDIDATES,
                verbose: bool = False) -> dict:
    """The fastest way to step ``tis`` (a :class:`~cardiax_gb300.tissue.Tissue`): returns
    ``{"choice": (schedule, depth, step_kernel or tile rows), "us_per_step": {choice: us}}``
    (candidates: ``TISSUE_CANDIDATES``); the tissue's
    state is restored.  With activation tracking on, only one-step-per-launch candidates
    qualify (temporal blocking does not track activations)."""
    tracking = tis.activation is not None
    cands = tuple(c for c in candidates if not (tracking and c[1] != 1))
    key = (torch.cuda.get_device_name(tis.device), tis.H, tis.W, tracking, trial_steps, cands)
    if key in _TISSUE_CACHE:
        return _TISSUE_CACHE[key]
    saved = tis.state.clone()
    saved_act = None if not tracking else (tis.act_first.clone(), tis.act_last.clone(),
                                           tis.act_count.clone())
    timings = {}
    try:
        for c in cands:
            try:
                _run(tis, 0, 8, c)  # warm-up: kernel attributes, descriptors
            except N.FkError:
                continue  # a schedule that does not take this grid
            best = None
            for rep in range(2):  # the better of two runs
                t0 = 8 + rep * trial_steps
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                _run(tis, t0, t0 + trial_steps, c)
                e1.record()
                torch.cuda.synchronize()
                us = e0.elapsed_time(e1) * 1e3 / trial_steps
                best = us if best is None else min(best, us)
            timings[c] = best
            if verbose:
                print(f"autotune {c}: {timings[c]:.2f} us/step")
    finally:
        tis.state.copy_(saved)
        if saved_act is not None:
            tis.act_first.copy_(saved_act[0])
            tis.act_last.copy_(saved_act[1])
            tis.act_count.copy_(saved_act[2])
    best = min(timings, key=timings.get)
    res = {"choice": best, "us_per_step": timings}
    _TISSUE_CACHE[key] = res
    return res
