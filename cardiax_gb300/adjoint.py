"""Reverse mode through the stepper: adjoint Euler steps with sqrt(T) checkpoint-and-recompute,
exposed as a ``torch.autograd.Function``.

The reference never differentiates its stepper; this provides the derivative that ``jax.grad``
of a scan over ``cardiax.solve.step_euler`` (cardiax/solve.py:68-70) defines, with the Heaviside
gates and the stimulus replacement contributing zero derivative.  Gradients are taken with
respect to the initial state, the per-cell diffusivity D and the first 13 fields of ``Params``
(``Cm`` is held fixed).

Memory: a rollout of T steps keeps ceil(T / K) checkpoints plus one segment of K recomputed
states, K = ceil(sqrt(T)) by default (e.g. 1e4 steps at 512^2: 200 states of 3 MiB).
"""
from __future__ import annotations

import ctypes
import math
import os
from concurrent.futures import ThreadPoolExecutor
from typing import Sequence

import torch

from . import _native as N
from .tissue import Tissue, as_cuda_f32, stream_handle

N_THETA = 13


def _lib():
    L = N.lib()
    if not getattr(L, "_adjoint_bound", False):
        L.fk_adjoint_slots.restype = ctypes.c_int64
        L.fk_adjoint_slots.argtypes = [N.Grid]
        L.fk_adjoint_step.restype = ctypes.c_int
        L.fk_adjoint_step.argtypes = [N.Grid, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.POINTER(N.Params), ctypes.POINTER(N.Stimulus),
                                      ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.fk_recompute.restype = ctypes.c_int
        L.fk_recompute.argtypes = [N.Grid, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                   ctypes.c_void_p, ctypes.POINTER(N.Params),
                                   ctypes.POINTER(N.Stimulus), ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.fk_adjoint_range.restype = ctypes.c_int
        L.fk_adjoint_range.argtypes = [N.Grid, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_void_p, ctypes.POINTER(N.Params),
                                       ctypes.POINTER(N.Stimulus), ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L._adjoint_bound = True
    return L


class Adjoint:
    """Reverse-mode helper bound to one :class:`Tissue` (its D, parameters and stimuli)."""

    def __init__(self, tissue: Tissue):
        self.t = tissue
        L = _lib()
        self.slots = int(L.fk_adjoint_slots(tissue.grid))
        dev = tissue.device
        self.gD = torch.zeros((tissue.H, tissue.pitch), dtype=torch.float32, device=dev)
        self.gtheta = torch.zeros((self.slots, 16), dtype=torch.float64, device=dev)

    def zero_grad(self):
        self.gD.zero_()
        self.gtheta.zero_()

    def step(self, state: torch.Tensor, t: int, lam_next: torch.Tensor, lam: torch.Tensor):
        """lam <- cotangent of x_t given the cotangent lam_next of x_{t+1}; accumulates dL/dD
        and dL/dtheta."""
        T = self.t
        rc = _lib().fk_adjoint_step(T.grid, state.data_ptr(), T.D.data_ptr(),
                                    ctypes.byref(T.params), T.stim, T.n_stim, int(t), T.dt, T.dx,
                                    lam_next.data_ptr(), lam.data_ptr(), self.gD.data_ptr(),
                                    self.gtheta.data_ptr(), stream_handle())
        if rc:
            raise N.FkError(rc, "fk_adjoint_step")

    def grad_theta(self) -> torch.Tensor:
        """dL/dtheta (13 values, cardiax Params order), summed over the slots in index order."""
        return self.gtheta[:, :N_THETA].sum(0)

    def grad_D(self) -> torch.Tensor:
        return self.gD[:, :self.t.W]

    # -- rollouts -----------------------------------------------------------------------------
    def rollout_gradient(self, state0: torch.Tensor, t0: int, t1: int, obs_times: Sequence[int],
                         obs_grads: torch.Tensor, seg: int = None, ckpts=None) -> torch.Tensor:
        """Backward pass of a rollout from ``state0`` ((3, H, pitch)) over steps t0 .. t1-1,
        where the loss depends on the states at ``obs_times`` (each in [t0, t1]) with
        dL/dx_{obs_times[k]} = obs_grads[k] ((n_obs, 3, H, pitch)).  Returns dL/dx_{t0};
        dL/dD and dL/dtheta accumulate in this object.  Uses checkpoints every ``seg`` steps
        (default ceil(sqrt(T))) and recomputes one segment at a time; ``ckpts`` = the
        [(step, state)] checkpoints at t0, t0+seg, ... when the caller kept them."""
        T = self.t
        n = t1 - t0
        seg = seg or default_segment(n)
        obs_index = {}
        for k, tt in enumerate(obs_times):
            obs_index.setdefault(int(tt), []).append(k)
        if ckpts is None:  # forward: checkpoints at t0, t0+seg, ...
            ckpts = forward_checkpoints(T, state0, t0, t1, seg)
        L = _lib()
        lam = torch.zeros_like(state0)
        lam_tmp = torch.empty_like(state0)
        if t1 in obs_index:
            for k in obs_index[t1]:
                lam += obs_grads[k]
        buf = torch.empty((seg,) + tuple(state0.shape), dtype=state0.dtype, device=state0.device)
        for s, st in reversed(ckpts):
            e = min(s + seg, t1)
            rc = L.fk_recompute(T.grid, st.data_ptr(), s, e - s, T.D.data_ptr(),
                                ctypes.byref(T.params), T.stim, T.n_stim, T.dt, T.dx,
                                buf.data_ptr(), stream_handle())
            if rc:
                raise N.FkError(rc, "fk_recompute")
            inj = [(tt, k) for tt in range(s, e) for k in obs_index.get(tt, [])]
            steps = (ctypes.c_int64 * max(1, len(inj)))(*[tt for tt, _ in inj])
            grads = (ctypes.c_void_p * max(1, len(inj)))(*[obs_grads[k].data_ptr() for _, k in inj])
            rc = L.fk_adjoint_range(T.grid, buf.data_ptr(), s, e - s, T.D.data_ptr(),
                                    ctypes.byref(T.params), T.stim, T.n_stim, T.dt, T.dx,
                                    lam.data_ptr(), lam_tmp.data_ptr(), steps, grads, len(inj),
                                    self.gD.data_ptr(), self.gtheta.data_ptr(), stream_handle())
            if rc:
                raise N.FkError(rc, "fk_adjoint_range")
        return lam


def default_segment(n_steps: int) -> int:
    return max(1, math.ceil(math.sqrt(max(n_steps, 1))))


def forward_checkpoints(T: Tissue, state0: torch.Tensor, t0: int, t1: int, seg: int,
                        stops: Sequence[int] = ()):
    """Advances ``T`` from ``state0`` over t0 .. t1-1 keeping the states at t0, t0+seg, ...;
    also returns clones of the (v, w, u) planes at each step in ``stops``."""
    ckpts, snaps = [], {}
    T.state.copy_(state0)
    marks = sorted(set(range(t0, t1, seg)) | {int(x) for x in stops if t0 <= int(x) <= t1})
    cur = t0
    for m in marks:
        if m > cur:
            T.advance(cur, m)
            cur = m
        if (m - t0) % seg == 0 and m < t1:
            ckpts.append((m, T.state.clone()))
        if m in stops:
            snaps[m] = T.state[:, :, :T.W].clone()
    if t1 > cur:
        T.advance(cur, t1)
        if t1 in stops:
            snaps[t1] = T.state[:, :, :T.W].clone()
    return (ckpts, snaps) if stops else ckpts


class _Rollout(torch.autograd.Function):
    """States at ``obs_times`` of a rollout, differentiable w.r.t. (v0, w0, u0, D, theta)."""

    @staticmethod
    def forward(ctx, v0, w0, u0, D, theta, Cm, stimuli, t0, t1, obs_times, dt, dx, seg):
        params = [float(x) for x in theta.detach().cpu().tolist()] + [float(Cm)]
        H, W = u0.shape
        tis = Tissue((H, W), params, D.detach(), stimuli, dt=dt, dx=dx, device=u0.device)
        tis.set_state((v0.detach(), w0.detach(), u0.detach()))
        state0 = tis.state.clone()
        t_end = max([t0] + [int(t) for t in obs_times])
        seg = seg or default_segment(t_end - t0)
        ckpts, snaps = forward_checkpoints(tis, state0, t0, t_end, seg, stops=list(obs_times))
        out = torch.empty((len(obs_times), 3, H, W), dtype=torch.float32, device=u0.device)
        for k, t in enumerate(obs_times):
            out[k] = snaps[int(t)]
        ctx.save_for_backward(state0)
        ctx.tis, ctx.t0, ctx.t1, ctx.obs_times, ctx.seg, ctx.W = tis, t0, t_end, list(obs_times), seg, W
        ctx.ckpts = ckpts
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (state0,) = ctx.saved_tensors
        tis, W = ctx.tis, ctx.W
        adj = Adjoint(tis)
        g = torch.zeros((len(ctx.obs_times),) + tuple(state0.shape), dtype=torch.float32,
                        device=state0.device)
        g[..., :W] = grad_out.to(torch.float32)
        lam0 = adj.rollout_gradient(state0, ctx.t0, ctx.t1, ctx.obs_times, g, seg=ctx.seg,
                                    ckpts=ctx.ckpts)
        ctx.ckpts = None
        gth = adj.grad_theta().to(torch.float32)
        return (lam0[0, :, :W], lam0[1, :, :W], lam0[2, :, :W], adj.grad_D().clone(), gth,
                None, None, None, None, None, None, None, None)


def rollout(v0, w0, u0, D, theta, stimuli, t0: int, t1: int, obs_times: Sequence[int],
            dt: float = 0.01, dx: float = 0.01, Cm: float = 1.0, seg: int = None):
    """Differentiable rollout: the states (n_obs, 3, H, W) at ``obs_times`` (steps in
    [t0, t1]) starting from (v0, w0, u0) at step t0.  Gradients flow to v0, w0, u0, D and
    ``theta`` (the 13 first Params fields) through the hand-written adjoint kernel with
    sqrt(T) checkpointing."""
    dev = u0.device if isinstance(u0, torch.Tensor) and u0.is_cuda else torch.device("cuda")
    to = lambda x: x if isinstance(x, torch.Tensor) and x.is_cuda else as_cuda_f32(x, dev)  # noqa: E731
    return _Rollout.apply(to(v0), to(w0), to(u0), to(D), to(theta), Cm, list(stimuli), int(t0),
                          int(t1), list(obs_times), float(dt), float(dx), seg)


def _per_experiment(fn, n: int):
    """Runs fn(b) for b in 0..n-1 from a pool of host threads.  Each experiment's steps are
    C loops that release the GIL, so the experiments' launches are issued in parallel (one
    thread issuing thousands of small launches is what bounds a batch of small tissues)."""
    workers = max(1, min(n, os.cpu_count() or 1))
    if workers == 1:
        return [fn(b) for b in range(n)]
    with ThreadPoolExecutor(workers) as ex:
        return list(ex.map(fn, range(n)))


class _RolloutBatch(torch.autograd.Function):
    """States at ``obs_times`` of B tissues sharing D and theta (one stimulus list per tissue);
    each tissue's forward and backward run on its own CUDA stream, issued from its own host
    thread, so the GPU overlaps them."""

    @staticmethod
    def forward(ctx, states0, D, theta, Cm, stimuli, t0, t1, obs_times, dt, dx, seg):
        params = [float(x) for x in theta.detach().cpu().tolist()] + [float(Cm)]
        B, _, H, W = states0.shape
        dev = states0.device
        t_end = max([t0] + [int(t) for t in obs_times])
        seg = seg or default_segment(t_end - t0)
        out = torch.empty((B, len(obs_times), 3, H, W), dtype=torch.float32, device=dev)
        main = torch.cuda.current_stream(dev)
        streams = [torch.cuda.Stream(dev) for _ in range(B)]
        Dd = D.detach()

        def one(b):
            streams[b].wait_stream(main)
            with torch.cuda.device(dev), torch.cuda.stream(streams[b]):
                tis = Tissue((H, W), params, Dd, stimuli[b], dt=dt, dx=dx, device=dev)
                tis.set_state(states0[b].detach())
                s0 = tis.state.clone()
                ck, snaps = forward_checkpoints(tis, s0, t0, t_end, seg, stops=list(obs_times))
                for k, t in enumerate(obs_times):
                    out[b, k] = snaps[int(t)]
            return tis, ck, s0

        res = _per_experiment(one, B)
        for s in streams:
            main.wait_stream(s)
        ctx.tissues = [r[0] for r in res]
        ctx.ckpts = [r[1] for r in res]
        ctx.state0s = [r[2] for r in res]
        ctx.streams = streams
        ctx.t0, ctx.t1, ctx.obs_times, ctx.seg, ctx.W = t0, t_end, list(obs_times), seg, W
        return out

    @staticmethod
    def backward(ctx, grad_out):
        W = ctx.W
        main = torch.cuda.current_stream()
        B = len(ctx.tissues)
        grad_out = grad_out.contiguous()

        def one(b):
            s = ctx.streams[b]
            s.wait_stream(main)
            tis = ctx.tissues[b]
            with torch.cuda.device(tis.device), torch.cuda.stream(s):
                adj = Adjoint(tis)
                g = torch.zeros((len(ctx.obs_times),) + tuple(ctx.state0s[b].shape),
                                dtype=torch.float32, device=tis.device)
                g[..., :W] = grad_out[b].to(torch.float32)
                lam0 = adj.rollout_gradient(ctx.state0s[b], ctx.t0, ctx.t1, ctx.obs_times, g,
                                            seg=ctx.seg, ckpts=ctx.ckpts[b])
            return lam0[:, :, :W], adj

        res = _per_experiment(one, B)
        for s in ctx.streams:
            main.wait_stream(s)
        ctx.ckpts = None
        g0 = [r[0] for r in res]
        adjs = [r[1] for r in res]
        gD = adjs[0].grad_D().clone()
        gth = adjs[0].grad_theta()
        for a in adjs[1:]:  # fixed order: deterministic sums
            gD += a.grad_D()
            gth = gth + a.grad_theta()
        return (torch.stack(g0), gD, gth.to(torch.float32), None, None, None, None, None, None,
                None, None)


def rollout_batch(states0, D, theta, stimuli_per_tissue, t0: int, t1: int,
                  obs_times: Sequence[int], dt: float = 0.01, dx: float = 0.01, Cm: float = 1.0,
                  seg: int = None):
    """Differentiable rollouts of B tissues that share D and theta: ``states0`` is
    (B, 3, H, W) (v, w, u), ``stimuli_per_tissue`` a list of B stimulus lists.  Returns
    (B, n_obs, 3, H, W); gradients flow to states0, D (summed over tissues) and theta."""
    return _RolloutBatch.apply(states0, D, theta, Cm, [list(s) for s in stimuli_per_tissue],
                               int(t0), int(t1), list(obs_times), float(dt), float(dx), seg)
