"""Autotuner of the stepping configuration.

For a batch it times, on the batch's own tissues, every candidate of
(graph_steps ∈ {0, 16, 64, 256}) × (persistent CTAs per SM ∈ {1}) over a short run of steps with
CUDA events and keeps the fastest; the tissues are restored to their initial state afterwards.
Choices are cached per (device name, batch signature) for the process.
"""
from __future__ import annotations

import torch

from .batch import TissueBatch

_CACHE: dict = {}

GRAPH_CANDIDATES = (0, 16, 64, 256)


def _signature(batch: TissueBatch):
    shapes = tuple(sorted((t.H, t.W) for t in batch.tissues))
    return (torch.cuda.get_device_name(batch.device), shapes)


def tune_batch(batch: TissueBatch, trial_steps: int = 256, candidates=GRAPH_CANDIDATES,
               verbose: bool = False) -> dict:
    """Picks ``graph_steps`` for ``batch`` (stored on it) and returns the timings."""
    key = (_signature(batch), trial_steps, tuple(candidates))
    if key in _CACHE:
        batch.graph_steps = _CACHE[key]["graph_steps"]
        return _CACHE[key]
    saved = [(t.state.clone(), None if t.activation is None else
              (t.act_first.clone(), t.act_last.clone(), t.act_count.clone()))
             for t in batch.tissues]
    timings = {}
    for g in candidates:
        batch.advance(0, 2, graph_steps=0)  # warm-up
        if g:
            batch.advance(0, g, graph_steps=g)  # captures the graph outside the timed run
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        batch.advance(0, trial_steps, graph_steps=g)
        e1.record()
        torch.cuda.synchronize()
        timings[g] = e0.elapsed_time(e1) / trial_steps
        if verbose:
            print(f"autotune graph_steps={g}: {timings[g] * 1e3:.1f} us/step")
    for t, (st, act) in zip(batch.tissues, saved):
        t.state.copy_(st)
        if act is not None:
            t.act_first.copy_(act[0])
            t.act_last.copy_(act[1])
            t.act_count.copy_(act[2])
    best = min(timings, key=timings.get)
    batch.graph_steps = best
    res = {"graph_steps": best, "ms_per_step": timings}
    _CACHE[key] = res
    return res
