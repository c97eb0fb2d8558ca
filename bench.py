"""Benchmark of the Fenton-Karma stepper on the 2048x2048 roofline workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one bench "step"): a 2048x2048 float32 tissue with parameter set 3, diffusivity
D = 0.001 (1 + 0.05 n) clipped at 0, n seeded unit Gaussian noise smoothed over 2 cells (per-cell
white noise makes the reference's own scheme diverge), a periodic left-edge stimulus (5 columns,
amplitude 20, Protocol(start=0, duration=200, period=20000) in steps), advanced from rest through
10 000 Euler steps (dt = dx = 0.01).  Inputs are synthetic and seeded.

* ``value``        GCUPS (1e9 cell-updates/s) with the tissue resident in HBM, timed with CUDA
                   events on the launching stream; L2 is flushed (256 MB write) between steps.
* ``e2e``          the same metric through the public API (``solve.forward``) from pinned host
                   arrays, host<->device copies of inputs and the returned state included.
* ``roofline``     the step kernel against the measured HBM copy bandwidth: 28 algorithmic bytes
                   per cell-update (read u, v, w, D; write u, v, w).
* ``cpu_baseline`` the C restatement of the reference's stepper (the oracle port) on the host's
                   cores, on a bounded sample of the same workload.
* ``headline``     the figures below in one short block: plain stepper at 2048^2 and 4096^2,
                   batched, adjoint and inverse problem.
* ``parity``       max|du| of the GPU against the reference's own float32 run (every
                   checkpoint) and its x64 run (1000 steps) on the 128^2 configuration, and
                   against the float32 and float64 oracle on the CPU-baseline sample of the
                   2048^2 workload, with the float32-vs-float64 gap beside each.
* ``roofline_4096`` the same workload at 4096^2 (DRAM-bound: nothing stays in L2).
* ``batched``      256 mixed tissues in one launch per step vs a loop of per-tissue calls,
                   10^4 steps each.
* ``adjoint``      gradient throughput of the 16-experiment inverse problem (dL/dD, dL/dtheta)
                   against 116 algorithmic bytes per experiment cell and gradient step, and
                   ``inverse``: 200 Adam iterations on D with the loss curve.
* ``schedules``    the roofline workload at 256^2, 512^2, 1024^2 and 2048^2 (a few hundred
                   steps each) under every schedule: one launch per step (k = 1), temporal
                   blocking with k = 2, 4, 8 steps per launch, the dataflow launch, and "auto"
                   (the tissue autotuner's choice); all give identical bits.
* ``next_rows``    Heun, the data-generation caller, the HDF5 write, the scar generator.

``--impl reference`` times that CPU implementation alone on the same workload (the reference's
own JAX CPU path cannot be installed here; the port is its restatement).  Multi-GPU runs are
replicas (one tissue per rank, no data exchange): ``value`` sums all ranks' cell-updates over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_UPDATE = 28  # read u, v, w, D + write u, v, w (float32)
# one gradient step of one experiment cell (float32): the forward step (28), its recomputation
# (28) and the store of the recomputed state into the segment buffer (12), and the adjoint step
# (read x_t 12, D 4, lambda_{t+1} 12; write lambda_t 12; read and write dL/dD 8 = 48)
ADJ_BYTES_PER_GRAD_STEP = 28 + 28 + 12 + 48
L2_FLUSH_BYTES = 256 << 20


def noisy_diffusivity(H: int, W: int, seed: int, sigma_cells: float = 2.0):
    """D = 0.001 (1 + 0.05 n), clipped at 0, with n seeded Gaussian noise of unit standard
    deviation smoothed over ``sigma_cells`` cells.  (Uncorrelated per-cell noise makes the
    reference's own discretisation diverge at the grid corners within a few hundred steps.)"""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    n = gaussian_filter(rng.standard_normal((H, W)), sigma_cells, mode="reflect")
    n /= n.std()
    return np.clip(0.001 * (1.0 + 0.05 * n), 0.0, None).astype(np.float32)


def scar_diffusivity(rng, H: int, W: int, blur: float = 2.0):
    """D = 0.001 with 1-4 elliptical scars (semi-axes 20-80 cells, random orientation) scaled by
    a factor in [0, 0.1], floored at 1e-4 (the reference's own D domain, deepx/generate.py:80;
    below it the reference's scheme is unstable inside scars) and blurred over ``blur`` cells."""
    from scipy.ndimage import gaussian_filter

    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    D = np.full((H, W), 1e-3)
    for _ in range(int(rng.integers(1, 5))):
        a, b = rng.uniform(20, 80, 2)
        th = rng.uniform(0, np.pi)
        ci, cj = rng.uniform(0, H), rng.uniform(0, W)
        x = (i - ci) * np.cos(th) + (j - cj) * np.sin(th)
        y = -(i - ci) * np.sin(th) + (j - cj) * np.cos(th)
        D[(x / a) ** 2 + (y / b) ** 2 <= 1] *= rng.uniform(0.0, 0.1)
    D = np.maximum(D, 1e-4)
    return gaussian_filter(D, blur, mode="reflect").astype(np.float32)


BATCH_SHAPES = ((64, 64), (128, 128), (256, 256), (512, 512), (256, 1024))


def batched_workload(n: int = 256, seed: int = 99):
    """The mixed batch: sizes from BATCH_SHAPES, parameter sets {1A, 3, 4A, 5}, scar D maps, a
    planar (left 5 columns) or 10x10 point stimulus of amplitude 20 at a random site, start in
    [0, 5000] steps, period in [15000, 40000] steps, duration 200 steps."""
    from cardiax_gb300 import params as Pm

    sets = (Pm.PARAMSET_1A, Pm.PARAMSET_3, Pm.PARAMSET_4A, Pm.PARAMSET_5)
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        H, W = BATCH_SHAPES[int(rng.integers(0, len(BATCH_SHAPES)))]
        P = sets[int(rng.integers(0, 4))]
        D = scar_diffusivity(rng, H, W)
        f = np.zeros((H, W), np.float32)
        if rng.uniform() < 0.5:
            f[:, :5] = 20.0
        else:
            r, c = int(rng.integers(0, H - 10)), int(rng.integers(0, W - 10))
            f[r:r + 10, c:c + 10] = 20.0
        proto = (int(rng.integers(0, 5001)), 200, int(rng.integers(15000, 40001)))
        out.append(((H, W), P, D, f, proto))
    return out


def run_batched(steps: int, reps: int, dev):
    """GCUPS of the batched path (autotuned graph replay) and of a loop of single-tissue calls
    over the same tissues, on the same GPU."""
    import torch
    from cardiax_gb300.autotune import tune_batch
    from cardiax_gb300.batch import TissueBatch
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue

    spec = batched_workload()
    tissues = [Tissue(shape, P, D, [Stimulus(Protocol(*proto), f)], device=dev)
               for shape, P, D, f, proto in spec]
    cells = sum(t.H * t.W for t in tissues)
    batch = TissueBatch(tissues)
    tune = tune_batch(batch, trial_steps=128)

    def timed(fn):
        for t in tissues:
            t.init()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    warm = max(2 * tune["graph_steps"], 64)
    timed(lambda: batch.advance(0, warm))  # warm-up (graph capture)
    tb = min(timed(lambda: batch.advance(0, steps)) for _ in range(reps))

    def loop(n):
        for t in tissues:
            t.advance(0, n)

    timed(lambda: loop(64))  # warm-up
    tl = timed(lambda: loop(steps))  # one run: 256 x 1e4 launches
    batch.close()
    peak, _ = peaks()
    gcups = cells * steps / tb / 1e9
    return {"tissues": len(tissues), "cells": cells, "euler_steps": steps,
            "gcups": gcups, "plain_loop_gcups": cells * steps / tl / 1e9,
            "speedup_vs_plain_loop": tl / tb, "frac": gcups * BYTES_PER_UPDATE / peak,
            "depth": tune["depth"], "tile_rows": tune["tile_rows"],
            "interleave": tune["interleave"], "packed": tune["packed"],
            "graph_steps": tune["graph_steps"],
            "autotune_ms_per_step": {
                f"d{k[0]}_rows{k[1]}_{('rr' + ('' if k[2][0] == 1 else f'x{k[2][0]}')) if k[2][0] else 'runs'}"
                f"_{'pk' if k[2][1] else 'sc'}"
                f"_g{k[3]}": v for k, v in tune["ms_per_step"].items()},
            "workload": "256 tissues, sizes {64^2,128^2,256^2,512^2,256x1024}, sets "
                        "{1A,3,4A,5}, scar D (factor U[0,0.1], floor 1e-4, blur 2), plane or "
                        "10x10 point stimulus, start U[0,5000], period U[15000,40000] steps"}


def run_adjoint(dev, n_tissues: int = 16, steps: int = 5000, n_obs: int = 20, size: int = 256,
                seg: int = None):
    """Gradient throughput of the inverse problem (``inverse_problem``: 16 experiments on one
    256x256 scar-D tissue, u observed at 20 checkpoints over 5000 steps): MSE loss against the
    observations made with the true D, gradient w.r.t. D (65,536 values, shared by the batch)
    and the 13 parameters through the adjoint kernel with sqrt(T) checkpointing (forward,
    segment recomputation and adjoint each one launch per step for all 16 experiments).
    ``grad_steps_per_s`` = experiments x steps / seconds of forward + backward."""
    import torch
    from cardiax_gb300.adjoint import rollout_batch

    s0, D_true, theta0, stims, obs_t, obs = inverse_problem(dev, n_tissues, steps, n_obs, size)
    H = W = size
    theta = theta0.clone().requires_grad_(True)
    D = torch.full((H, W), 1e-3, device=dev, requires_grad=True)
    times = []
    for _ in range(2):
        D.grad = None
        theta.grad = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = rollout_batch(s0, D, theta, stims, 0, steps, obs_t, seg=seg)
        loss = ((out[:, :, 2] - obs) ** 2).mean()
        loss.backward()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t_best = min(times)
    peak, _ = peaks()
    gbs = n_tissues * steps * H * W * ADJ_BYTES_PER_GRAD_STEP / t_best / 1e9
    return {"experiments": n_tissues, "size": f"{H}x{W}", "euler_steps": steps,
            "observations": n_obs, "seconds_per_gradient": t_best,
            "grad_steps_per_s": n_tissues * steps / t_best,
            "algorithmic_bytes_per_grad_cell_step": ADJ_BYTES_PER_GRAD_STEP,
            "achieved_gbs": gbs, "frac": gbs / peak,
            "gradient": "dL/dD (per cell, shared D) and dL/dtheta (13 parameters), MSE on u at "
                        "the observations, hand-written adjoint with sqrt(T) checkpoint-recompute",
            "checked": "relative error <= 1e-3 vs float64 autodiff of the oracle and central "
                       "finite differences (tests/test_gpu_adjoint.py)"}


def inverse_problem(dev, n_tissues: int = 16, steps: int = 5000, n_obs: int = 20,
                    size: int = 256, seed: int = 4):
    """The inverse problem's data: 16 experiments on one 256x256 scar-D tissue (parameter set
    3), each with its own 10x10 point stimulus (amplitude 20, start in [0, 500) steps); u
    observed at 20 evenly spaced checkpoints over 5000 steps with the true D.  Returns
    (states0, D_true, theta, stimuli, obs_times, observations)."""
    import torch
    from cardiax_gb300 import params as Pm
    from cardiax_gb300.adjoint import rollout_batch
    from cardiax_gb300.stimulus import Protocol, Stimulus

    rng = np.random.default_rng(seed)
    H = W = size
    obs_t = [steps * (k + 1) // n_obs for k in range(n_obs)]
    theta = torch.tensor(Pm.PARAMSET_3[:13], dtype=torch.float32, device=dev)
    stims = []
    for _ in range(n_tissues):
        f = np.zeros((H, W), np.float32)
        r, c = int(rng.integers(0, H - 10)), int(rng.integers(0, W - 10))
        f[r:r + 10, c:c + 10] = 20.0
        stims.append([Stimulus(Protocol(int(rng.integers(0, 500)), 200, 20000), f)])
    s0 = torch.zeros((n_tissues, 3, H, W), device=dev)
    s0[:, :2] = 1.0
    D_true = torch.as_tensor(scar_diffusivity(rng, H, W), device=dev)
    with torch.no_grad():
        obs = rollout_batch(s0, D_true, theta, stims, 0, steps, obs_t)[:, :, 2]
    return s0, D_true, theta, stims, obs_t, obs


def run_inverse(dev, iterations: int = 200, lr: float = 2e-5):
    """The inverse problem end to end: Adam on D (65,536 values) from a uniform D = 0.001,
    ``iterations`` gradient evaluations of the 16 x 5000-step rollout (adjoint.fit_diffusivity:
    D the 2-cell Gaussian blur of the map Adam updates, clipped to [1e-4, 2e-3])."""
    import torch
    from cardiax_gb300.adjoint import fit_diffusivity

    s0, D_true, theta, stims, obs_t, obs = inverse_problem(dev)
    D0 = torch.full_like(D_true, 1e-3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    D, losses = fit_diffusivity(s0, D0, theta, stims, 0, obs_t[-1], obs_t, obs,
                                iterations=iterations, lr=lr)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    rel = lambda X: float((X - D_true).norm() / D_true.norm())  # noqa: E731
    drops = sum(1 for a, b in zip(losses, losses[1:]) if b < a)
    return {"iterations": iterations, "optimizer": f"Adam(lr={lr:g}) on D = blur_2cells(phi), phi clipped to [1e-4, 2e-3]",
            "seconds_per_iteration": dt / max(1, iterations),
            "loss_first": losses[0] if losses else None,
            "loss_last": losses[-1] if losses else None,
            "loss_min": min(losses) if losses else None,
            "loss_decreasing_steps": f"{drops}/{max(0, len(losses) - 1)}",
            "loss_every_20": losses[::20],
            "D_rel_error_first": rel(D0), "D_rel_error_last": rel(D)}


def run_roofline_sample(dev, size: int = 4096, steps: int = 300):
    """The roofline workload at ``size`` (4096^2: the state, D and the new state do not fit in
    L2, so the step is DRAM-bound): best of 2 runs of ``steps`` steps, L2 flushed before each."""
    import torch
    from cardiax_gb300 import params
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue

    D, field, proto = workload(size, size)
    tis = Tissue((size, size), params.PARAMSET_3, D, [Stimulus(Protocol(*proto), field)],
                 device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    tis.advance(0, 8)
    best = None
    for rep in range(2):
        tis.init()
        flush.fill_(float(rep))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        tis.advance(0, steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del flush
    us = best * 1e3 / steps
    peak, _ = peaks()
    gbs = BYTES_PER_UPDATE * size * size / (us * 1e-6) / 1e9
    return {"size": f"{size}x{size}", "steps": steps, "us_per_step": us,
            "gcups": size * size / (us * 1e-6) / 1e9, "achieved_gbs": gbs, "frac": gbs / peak,
            "traffic": profiled_traffic(f"fk_step_kernel_{size}.md"),
            "traffic_source": f"profiles/fk_step_kernel_{size}.md (ncu, one launch)"}


def run_parity_config1(dev):
    """The 128x128 configuration, 1000 steps, checkpoints every 100 (plain: amplitude 1 for the
    2 active steps, no wave; excite: amplitude 20, a travelling wave) against the reference's
    own float32 run at every checkpoint and its x64 run at 1000 steps (tests/golden fixtures
    made by running the reference's solve.py)."""
    from cardiax_gb300 import params, solve
    from cardiax_gb300.stimulus import Protocol, Stimulus

    gdir = os.path.join(ROOT, "tests", "golden")
    g32 = np.load(os.path.join(gdir, "config0.npz"))
    g64 = np.load(os.path.join(gdir, "config0_x64.npz"))
    out = {}
    for tag, proto in (("plain", (0, 200, 1e9)), ("excite", (0, 2, 1e9))):
        D = np.full((128, 128), 0.001, np.float32)
        states = solve.forward(solve.init((128, 128), device=dev), list(range(0, 1001, 100)),
                               params.PARAMSET_3, D,
                               [Stimulus(Protocol(*proto), g32[f"{tag}_field"])], 0.01, 0.01)
        e32 = max(float(np.abs(s.u.cpu().numpy() - g32[f"{tag}_u_{(i + 1) * 100}"]).max())
                  for i, s in enumerate(states))
        u = states[-1].u.cpu().numpy().astype(np.float64)
        out[tag] = {"max_du_vs_ref_f32": e32,
                    "du_vs_ref_x64_1000": float(np.abs(u - g64[f"{tag}_u_1000"]).max()),
                    "ref_f32_vs_x64_1000": float(np.abs(g32[f"{tag}_u_1000"] -
                                                        g64[f"{tag}_u_1000"]).max())}
    return out


def cpu_baseline_leg(tis, H, W, D, field, proto, seconds: float, threads: int):
    """The CPU baseline: the C oracle (float32, ``threads`` host threads) timed on a bounded
    sample of the workload (the first n steps from rest, n chosen for about ``seconds``); then,
    as the checker, the same sample in float64, and the GPU's state after the same n steps
    compared with both."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fk_oracle as O
    import fk_oracle_c as C
    C.build()
    from cardiax_gb300 import params
    P3 = params.PARAMSET_3
    stims = [(proto[0], proto[1], proto[2], field)]
    st = O.init((H, W))
    t0 = time.perf_counter()
    C.forward_euler(st, 0, 2, P3, D, stims, 0.01, 0.01, threads=threads)
    per = max((time.perf_counter() - t0) / 2, 1e-4)
    n = int(max(2, min(2000, seconds / per)))
    t0 = time.perf_counter()
    v, w, u = C.forward_euler(st, 0, n, P3, D, stims, 0.01, 0.01, threads=threads)
    dt = time.perf_counter() - t0
    rate = H * W * n / dt / 1e9
    cpu = {"value": rate, "unit": "GCUPS", "cores": threads, "kind": "port",
           "sample": f"{H}x{W}, the first {n} Euler steps from rest ({dt:.1f} s), C "
                     f"restatement of cardiax/solve.py with OpenMP over rows"}
    st64 = O.init((H, W), np.float64)
    stims64 = [(proto[0], proto[1], proto[2], field.astype(np.float64))]
    _, _, u64 = C.forward_euler(st64, 0, n, P3, D.astype(np.float64), stims64, 0.01, 0.01,
                                threads=threads)
    tis.init()
    tis.advance(0, n)
    ug = tis.view()[2].cpu().numpy()
    parity = {"size": f"{H}x{W}", "steps": n,
              "max_du_vs_oracle_f32": float(np.abs(ug - u).max()),
              "max_du_vs_oracle_f64": float(np.abs(ug.astype(np.float64) - u64).max()),
              "oracle_f32_vs_f64": float(np.abs(u.astype(np.float64) - u64).max())}
    return cpu, parity


def workload(H: int, W: int, seed: int = 1234):
    D = noisy_diffusivity(H, W, seed)
    field = np.zeros((H, W), np.float32)
    field[:, :5] = 20.0
    proto = (0, 200, 20000)
    return D, field, proto


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name: str):
    """dram bytes per launch from a committed ncu summary (``dram_bytes_per_launch: N``)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.path = index, None, None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[4:8]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, device) -> float:
    """The largest ``x`` over the ranks of the default process group (``x`` itself without
    one): each replica's time, so that the whole-job figure is set by the slowest replica."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gcups(updates_per_rank: float, seconds: float, world: int) -> float:
    """Whole-job GCUPS of ``world`` independent replicas that each made ``updates_per_rank``
    cell updates in at most ``seconds`` (the max over ranks)."""
    return world * updates_per_rank / seconds / 1e9


def cpu_port_rate(H, W, D, field, proto, seconds: float, threads: int):
    """GCUPS of the C oracle on a bounded sample (steps chosen to take about ``seconds``)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fk_oracle as O
    import fk_oracle_c as C
    C.build()
    P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
    st = O.init((H, W))
    stims = [(proto[0], proto[1], proto[2], field)]
    t0 = time.perf_counter()
    C.forward_euler(st, 0, 2, P3, D, stims, 0.01, 0.01, threads=threads)
    per = max((time.perf_counter() - t0) / 2, 1e-4)
    n = int(max(2, min(2000, seconds / per)))
    t0 = time.perf_counter()
    C.forward_euler(st, 0, n, P3, D, stims, 0.01, 0.01, threads=threads)
    dt = time.perf_counter() - t0
    return H * W * n / dt / 1e9, n, dt


def run_reference(args):
    """The CPU implementation (oracle port of cardiax/solve.py) on the same workload."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    H = W = args.size
    D, field, proto = workload(H, W)
    threads = os.cpu_count() or 1
    rates, samples = [], []
    for k in range(args.warmup + args.steps):
        r, n, dt = cpu_port_rate(H, W, D, field, proto, args.cpu_seconds, threads)
        if k >= args.warmup:
            rates.append(r)
            samples.append((n, dt))
    total_updates = sum(H * W * n for n, _ in samples)
    total_time = sum(dt for _, dt in samples)
    value = total_updates / total_time / 1e9
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GCUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total_time / len(samples), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": config(args),
        "cpu_baseline": {"value": value, "unit": "GCUPS", "cores": threads, "kind": "port",
                         "sample": f"{H}x{W}, {samples[0][0]} Euler steps per sample, "
                                   f"C restatement of cardiax/solve.py with OpenMP over rows"},
        "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


METRIC = "GCUPS (1e9 Fenton-Karma cell-updates/s), fused FP32 Euler stepper; roofline.frac = % of HBM roofline"


def run_next_rows(dev, reps: int = 2):
    """The callers either side of the stepper, each timed on the device (best of ``reps``):

    * ``heun``: the Heun integrator (cardiax/solve.py:73-85,103-111) on the 2048^2 roofline
      workload, 2000 steps, GCUPS;
    * ``sequence``: deepx/generate.py:135-210 as the reference's data generation runs it --
      a 1200^2 tissue from rest, two triangular stimuli (modulus 20, 2 steps), 10 000 Euler
      steps, the state emitted every 100 steps resized to 256^2 on the device -- GCUPS of the
      stepping with the emission included, and emitted states per second;
    * ``hdf5``: those 101 emitted states written as the reference's HDF5 data set
      (cardiax/io.py:13-78; ``io.init`` + ``io.add_states``) from host memory, MB/s;
    * ``scar``: deepx/utils_scars.py:409-426 at its default 1200^2 -- ms per scar map end to end
      (host outlines, fill and blur kernels), and the blur kernel alone (K = 120 taps per axis)
      in TFLOP/s."""
    import torch
    from cardiax_gb300 import generate, params as Pm
    from cardiax_gb300.stimulus import Direction, Protocol, Stimulus, triangular
    from cardiax_gb300.tissue import Tissue

    def best(fn):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    H = W = 2048
    D = noisy_diffusivity(H, W, seed=1)
    f = np.zeros((H, W), np.float32)
    f[:, :5] = 20.0
    tis = Tissue((H, W), Pm.PARAMSET_3, D, [Stimulus(Protocol(0, 200, 20000), f)], device=dev)
    n_heun = 2000

    def heun():
        tis.init()
        tis.advance_heun(0, n_heun)
    t_h = best(heun)
    heun_r = {"size": f"{H}x{W}", "steps": n_heun, "gcups": H * W * n_heun / t_h / 1e9,
              "us_per_step": t_h / n_heun * 1e6}

    S, n_steps, every, out = 1200, 10000, 100, (256, 256)
    Ds = np.full((S, S), 1e-3, np.float32)
    stims = [triangular((S, S), Direction.WEST, 30.0, 0.2, 20.0, Protocol(0, 2, 1e9), device=dev),
             triangular((S, S), Direction.SOUTH, -45.0, 0.2, 20.0, Protocol(3000, 2, 1e9),
                        device=dev)]

    emitted = {}

    def seq():
        emitted["states"] = generate.sequence(0, n_steps + every, every, 0.01, 0.01,
                                              Pm.PARAMSET_3, Ds, stims, reshape=out, device=dev)
    t_s = best(seq)
    seq_r = {"grid": f"{S}x{S}", "euler_steps": n_steps, "emit_every": every,
             "reshape": f"{out[0]}x{out[1]}", "gcups": S * S * n_steps / t_s / 1e9,
             "states_per_s": (n_steps // every) / t_s}

    from cardiax_gb300 import io, scars
    host = emitted["states"].cpu().numpy()
    with tempfile.TemporaryDirectory() as tdir:
        path = os.path.join(tdir, "sequence.hdf5")

        def write():
            f = io.init(path, out, n_iter=host.shape[0], n_stimuli=0)
            io.add_states(f["states"], host, 0, host.shape[0])
            f.close()
        t_w = best(write)
        file_bytes = os.path.getsize(path)
    h5_r = {"states": int(host.shape[0]), "bytes": int(host.nbytes), "file_bytes": file_bytes,
            "mb_per_s": host.nbytes / t_w / 1e6}

    Hs = 1200
    d = scars.draw(np.random.default_rng(7))
    t_sc = best(lambda: scars.random_diffusivity_scar(d, (Hs, Hs), device=dev))
    rows, cols = scars.outlines(d, (Hs, Hs))
    K, sigma = scars.blur_width(d, (Hs, Hs))
    wts = scars.gaussian_weights(K, sigma)
    mask, _ = scars.rasterize(rows, cols, (Hs, Hs), dev)
    scars.blur_same(mask, wts, one_minus=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        scars.blur_same(mask, wts, one_minus=True)
    e1.record()
    torch.cuda.synchronize()
    t_blur = e0.elapsed_time(e1) / 5 / 1e3
    scar_r = {"size": f"{Hs}x{Hs}", "blobs": d.n_blobs, "taps": K,
              "ms_per_map": t_sc * 1e3, "blur_ms": t_blur * 1e3,
              "blur_tflops": 2.0 * K * K * Hs * Hs / t_blur / 1e12}
    return {"heun": heun_r, "sequence": seq_r, "hdf5": h5_r, "scar": scar_r}


def run_schedules(dev, sizes=(256, 512, 1024, 2048), steps: int = 400):
    """GCUPS of each stepping schedule on the roofline workload (best of 2 runs of ``steps``
    steps, L2 flushed before each run), and of ``schedule="auto"`` with the choice the tissue
    autotuner made."""
    import torch
    from cardiax_gb300 import params
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    from cardiax_gb300 import autotune
    modes = {"k1": {}, "k2": {"depth": 2}, "k4": {"depth": 4}, "k8": {"depth": 8},
             "flow": {"schedule": "flow"}, "batch16": {"schedule": "batch", "tile_rows": 16},
             "auto": {"schedule": "auto"}}
    out = {}
    for size in sizes:
        D, field, proto = workload(size, size)
        tis = Tissue((size, size), params.PARAMSET_3, D, [Stimulus(Protocol(*proto), field)],
                     device=dev)
        row = {}
        for name, kw in modes.items():
            tis.init()
            tis.advance(0, 16, **kw)  # warm-up (kernel attributes, maps)
            best = None
            for rep in range(2):
                flush.fill_(float(rep))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                tis.advance(16 + rep * steps, 16 + (rep + 1) * steps, **kw)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            row[name] = {"gcups": size * size * steps / (best / 1e3) / 1e9,
                         "us_per_step": best * 1e3 / steps}
            if name == "auto":
                sched, depth, kernel = autotune.tune_tissue(tis)["choice"]
                row[name]["choice"] = {"schedule": sched, "depth": depth,
                                       "kernel": (f"batched, {kernel}-row items"
                                                  if sched == "batch" else
                                                  "strip" if kernel else "tiled")}
        out[f"{size}x{size}"] = row
    return out


def config(args):
    return {"workload": f"roofline_{args.size}: {args.size}x{args.size} FP32, PARAMSET_3, "
                        f"D=0.001(1+0.05n) clipped>=0, n=N(0,1) smoothed over 2 cells, "
                        f"periodic left-edge stimulus "
                        f"(5 columns, amplitude 20, Protocol(0,200,20000)), "
                        f"{args.euler_steps} Euler steps from rest per bench step, dt=dx=0.01",
            "H": args.size, "W": args.size, "euler_steps_per_step": args.euler_steps,
            "l2": "flushed between timed steps (256 MB write)",
            "kernel": "fk_step_kernel (one launch per Euler step)"}


def run_ours(args):
    import torch
    import torch.distributed as dist

    world, rank, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    from cardiax_gb300 import params, solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue

    H = W = args.size
    S = args.euler_steps
    D, field, proto = workload(H, W, seed=1234 + rank)
    P = params.PARAMSET_3
    tis = Tissue((H, W), P, D, [Stimulus(Protocol(*proto), field)], dt=0.01, dx=0.01, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def one_step():
        tis.init()
        tis.advance(0, S)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(torch.cuda.current_device()).start()
    t_wall = time.perf_counter()
    evs = []
    for k in range(args.steps):
        flush.fill_(float(k))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        one_step()
        e1.record()
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), dev)
    value = replica_gcups(args.steps * H * W * S, ms / 1e3, world)

    # end to end through the public API from pinned host memory
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.as_tensor(a).pin_memory()  # noqa: E731
        st0 = solve.State(pin(np.ones((H, W), np.float32)), pin(np.ones((H, W), np.float32)),
                          pin(np.zeros((H, W), np.float32)))
        Dp, fp = pin(D), pin(field)
        h2d = 4 * H * W * 5  # v, w, u, D, stimulus field
        d2h = 4 * H * W * 3  # returned v, w, u
        times = []
        for k in range(max(1, args.e2e_steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            states = solve.forward(st0, [0, S], P, Dp, [Stimulus(Protocol(*proto), fp)], 0.01,
                                   0.01)
            host = [x.cpu() for x in states[-1]]
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            del states, host
        e2e_s = max_over_ranks(sum(times), dev)
        e2e = {"value": replica_gcups(len(times) * H * W * S, e2e_s, world), "unit": "GCUPS",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    peak, peak_kind = peaks()
    launch_ms = ms / (args.steps * S)
    achieved = BYTES_PER_UPDATE * H * W / (launch_ms / 1e3) / 1e9
    traffic = profiled_traffic(f"fk_step_kernel_{args.size}.md")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": BYTES_PER_UPDATE * H * W,
                "avg_launch_us": launch_ms * 1e3}

    # sub-benchmarks (rank 0 of a replica run only: they are per-GPU figures)
    solo = rank == 0
    sample = run_roofline_sample(dev) if solo and not args.no_4096 else None
    parity = None
    if solo and not args.no_parity:
        parity = {"config1_128x128_1000_steps": run_parity_config1(dev)}
    cpu = None
    if solo and world == 1 and not args.no_cpu:
        cpu, parity_2048 = cpu_baseline_leg(tis, H, W, D, field, proto, args.cpu_seconds,
                                            os.cpu_count() or 1)
        if parity is not None:
            parity[f"roofline_{H}_sample"] = parity_2048
    batched = run_batched(args.batched_steps, 2, dev) if solo and not args.no_batched else None
    adjoint = None
    if solo and not args.no_adjoint:
        adjoint = run_adjoint(dev)
        if args.inverse_iterations > 0:
            adjoint["inverse"] = run_inverse(dev, iterations=args.inverse_iterations)
    schedules = run_schedules(dev) if solo and not args.no_schedules else None
    next_rows = run_next_rows(dev) if solo and not args.no_next else None

    if rank == 0:
        def pick(d, *keys):
            return None if d is None else {k: d.get(k) for k in keys}
        headline = {
            f"plain_{H}": {"gcups": value / world, "frac": roofline["frac"]},
            "plain_4096": pick(sample, "gcups", "frac", "us_per_step"),
            "batched": pick(batched, "gcups", "frac", "plain_loop_gcups",
                            "speedup_vs_plain_loop", "euler_steps"),
            "adjoint": pick(adjoint, "grad_steps_per_s", "seconds_per_gradient", "frac"),
            "inverse": pick((adjoint or {}).get("inverse"), "iterations",
                            "seconds_per_iteration", "loss_first", "loss_last",
                            "D_rel_error_first", "D_rel_error_last"),
        }
        out = {"metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
               "config": config(args), "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu,
               "gpu_launches": args.steps * (S + 1), "clocks": clk,
               "headline": headline, "parity": parity, "roofline_4096": sample,
               "batched": batched, "adjoint": adjoint, "wall_s_timed_region": t_wall,
               "schedules": schedules, "next_rows": next_rows}
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--euler-steps", type=int, default=10000)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-schedules", action="store_true")
    ap.add_argument("--no-next", action="store_true", help="skip the Heun and sequence timings")
    ap.add_argument("--batched-steps", type=int, default=10000)
    ap.add_argument("--inverse-iterations", type=int, default=200,
                    help="Adam iterations of the inverse problem (0: skip)")
    ap.add_argument("--no-4096", action="store_true", help="skip the 4096^2 roofline sample")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity figures")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
