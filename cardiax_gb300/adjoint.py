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
from typing import Sequence

import torch

from . import _native as N
from .tissue import (Tissue, as_cuda_f32, params_struct, pitch_of, stimulus_table, stream_handle,
                     to_pitched)

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
        L.fk_adjoint_batch_workspace_bytes.restype = ctypes.c_size_t
        L.fk_adjoint_batch_workspace_bytes.argtypes = [ctypes.c_int]
        L.fk_batch_recompute.restype = ctypes.c_int
        L.fk_batch_recompute.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.fk_adjoint_batch_range.restype = ctypes.c_int
        L.fk_adjoint_batch_range.argtypes = [
            ctypes.c_int, N.Grid, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
            ctypes.c_void_p, ctypes.POINTER(N.Params),
            ctypes.POINTER(ctypes.POINTER(N.Stimulus)), ctypes.POINTER(ctypes.c_int),
            ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
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


class _BatchPlan:
    """B experiments on one grid sharing D and the parameters, as one fk_batch plan (their
    forward steps and recomputed segments are one launch per step for all of them)."""

    def __init__(self, states0, Dp, params, stimuli, dt, dx):
        B, _, H, W = states0.shape
        dev = states0.device
        self.B, self.H, self.W, self.pitch = B, H, W, pitch_of(W)
        self.grid = N.Grid(H, W, self.pitch)
        self.params = params_struct(params)
        self.dt, self.dx = float(dt), float(dx)
        self.D = Dp
        self.S = torch.zeros((B, 3, H, self.pitch), dtype=torch.float32, device=dev)
        self.S[..., :W] = states0
        self.scratch = torch.empty_like(self.S)
        self.stims, self.keep = [], []
        descs = (N.TissueDesc * B)()
        none = N.Activation(None, None, None, 0.0)
        for b in range(B):
            arr, n, keep = stimulus_table(stimuli[b], H, W, self.pitch, dev)
            self.stims.append((arr, n))
            self.keep.append(keep)
            descs[b] = N.TissueDesc(self.grid, self.S[b].data_ptr(), self.scratch[b].data_ptr(),
                                    Dp.data_ptr(), self.params, arr, n, self.dt, self.dx, none)
        self._descs = descs
        L = N.lib()
        nbytes = L.fk_batch_workspace_bytes(descs, B)
        self.workspace = torch.empty(nbytes + 128, dtype=torch.uint8, device=dev)
        base = (self.workspace.data_ptr() + 127) // 128 * 128
        plan = ctypes.c_void_p()
        N.call("fk_batch_create", descs, B, base, nbytes, stream_handle(), ctypes.byref(plan))
        self.plan = plan

    def advance(self, t0: int, t1: int):
        N.call("fk_batch_forward_euler", self.plan, int(t0), int(t1), 0, stream_handle())

    def close(self):
        if getattr(self, "plan", None):
            N.lib().fk_batch_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _RolloutBatch(torch.autograd.Function):
    """States at ``obs_times`` of B tissues sharing D and theta (one stimulus list per tissue).
    Forward, segment recomputation and the adjoint are each one launch per step for all B
    tissues (fk_batch_forward_euler, fk_batch_recompute, fk_adjoint_batch_range), with
    checkpoints every ``seg`` steps as in :func:`rollout`."""

    @staticmethod
    def forward(ctx, states0, D, theta, Cm, stimuli, t0, t1, obs_times, dt, dx, seg):
        params = [float(x) for x in theta.detach().cpu().tolist()] + [float(Cm)]
        B, _, H, W = states0.shape
        dev = states0.device
        t_end = max([t0] + [int(t) for t in obs_times])
        seg = seg or default_segment(t_end - t0)
        Dp = to_pitched(D.detach(), H, W, pitch_of(W), dev)
        bp = _BatchPlan(states0.detach(), Dp, params, stimuli, dt, dx)
        out = torch.empty((B, len(obs_times), 3, H, W), dtype=torch.float32, device=dev)
        obs_at = {}
        for k, t in enumerate(obs_times):
            obs_at.setdefault(int(t), []).append(k)
        marks = sorted(set(range(t0, t_end, seg)) | set(obs_at))
        ckpts, cur = [], t0
        for m in marks:
            if m > cur:
                bp.advance(cur, m)
                cur = m
            if (m - t0) % seg == 0 and m < t_end:
                ckpts.append((m, bp.S.clone()))
            for k in obs_at.get(m, []):
                out[:, k] = bp.S[..., :W]
        if t_end > cur:
            bp.advance(cur, t_end)
            for k in obs_at.get(t_end, []):
                out[:, k] = bp.S[..., :W]
        ctx.bp, ctx.ckpts = bp, ckpts
        ctx.t0, ctx.t1, ctx.obs_times, ctx.seg = t0, t_end, list(obs_times), seg
        return out

    @staticmethod
    def backward(ctx, grad_out):
        bp = ctx.bp
        B, H, W, pitch = bp.B, bp.H, bp.W, bp.pitch
        dev = bp.S.device
        L = _lib()
        seg, t1 = ctx.seg, ctx.t1
        n_obs = len(ctx.obs_times)
        g = torch.zeros((n_obs, B, 3, H, pitch), dtype=torch.float32, device=dev)
        g[..., :W] = grad_out.to(torch.float32).transpose(0, 1)
        obs_index = {}
        for k, tt in enumerate(ctx.obs_times):
            obs_index.setdefault(int(tt), []).append(k)
        lam = torch.zeros((B, 3, H, pitch), dtype=torch.float32, device=dev)
        lam_tmp = torch.empty_like(lam)
        for k in obs_index.get(t1, []):
            lam += g[k]
        ns = 3 * H * pitch
        buf = torch.empty((B, seg, 3, H, pitch), dtype=torch.float32, device=dev)
        slots = int(L.fk_adjoint_slots(bp.grid))
        gD = torch.zeros((B, H, pitch), dtype=torch.float32, device=dev)
        gth = torch.zeros((B, slots, 16), dtype=torch.float64, device=dev)
        wsb = int(L.fk_adjoint_batch_workspace_bytes(B))
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        stim_ptrs = (ctypes.POINTER(N.Stimulus) * B)(
            *[ctypes.cast(a, ctypes.POINTER(N.Stimulus)) for a, _ in bp.stims])
        n_stims = (ctypes.c_int * B)(*[n for _, n in bp.stims])
        for s, st in reversed(ctx.ckpts):
            e = min(s + seg, t1)
            bp.S.copy_(st)
            rc = L.fk_batch_recompute(bp.plan, s, e - s, buf.data_ptr(), seg * ns,
                                      stream_handle())
            if rc:
                raise N.FkError(rc, "fk_batch_recompute")
            inj = [(tt, k) for tt in range(s, e) for k in obs_index.get(tt, [])]
            steps = (ctypes.c_int64 * max(1, len(inj)))(*[tt for tt, _ in inj])
            grads = (ctypes.c_void_p * max(1, len(inj)))(*[g[k].data_ptr() for _, k in inj])
            rc = L.fk_adjoint_batch_range(B, bp.grid, buf.data_ptr(), seg * ns, s, e - s,
                                          bp.D.data_ptr(), ctypes.byref(bp.params), stim_ptrs,
                                          n_stims, bp.dt, bp.dx, lam.data_ptr(),
                                          lam_tmp.data_ptr(), steps, grads, len(inj),
                                          gD.data_ptr(), gth.data_ptr(), ws.data_ptr(), wsb,
                                          stream_handle())
            if rc:
                raise N.FkError(rc, "fk_adjoint_batch_range")
        ctx.ckpts = None
        gD_sum = gD[0, :, :W].clone()
        gth_sum = gth[0, :, :N_THETA].sum(0)
        for b in range(1, B):  # fixed order: deterministic sums
            gD_sum += gD[b, :, :W]
            gth_sum = gth_sum + gth[b, :, :N_THETA].sum(0)
        ctx.bp = None
        bp.close()
        return (lam[..., :W], gD_sum, gth_sum.to(torch.float32), None, None, None, None, None,
                None, None, None)


def rollout_batch(states0, D, theta, stimuli_per_tissue, t0: int, t1: int,
                  obs_times: Sequence[int], dt: float = 0.01, dx: float = 0.01, Cm: float = 1.0,
                  seg: int = None):
    """Differentiable rollouts of B tissues that share D and theta: ``states0`` is
    (B, 3, H, W) (v, w, u), ``stimuli_per_tissue`` a list of B stimulus lists.  Returns
    (B, n_obs, 3, H, W); gradients flow to states0, D (summed over tissues) and theta."""
    return _RolloutBatch.apply(states0, D, theta, Cm, [list(s) for s in stimuli_per_tissue],
                               int(t0), int(t1), list(obs_times), float(dt), float(dx), seg)


def gaussian_blur(x: torch.Tensor, sigma_cells: float) -> torch.Tensor:
    """A separable Gaussian blur of an (H, W) map (radius ceil(3 sigma), mirrored edges),
    differentiable through torch (a constant map stays constant)."""
    r = int(math.ceil(3.0 * sigma_cells))
    if r < 1:
        return x
    k = torch.arange(-r, r + 1, dtype=torch.float32, device=x.device)
    k = torch.exp(-k * k / (2.0 * sigma_cells * sigma_cells))
    k = k / k.sum()
    F = torch.nn.functional
    y = F.conv2d(F.pad(x[None, None], (r, r, 0, 0), mode="reflect"), k.view(1, 1, 1, -1))
    return F.conv2d(F.pad(y, (0, 0, r, r), mode="reflect"), k.view(1, 1, -1, 1))[0, 0]


def fit_diffusivity(states0, D_init, theta, stimuli_per_tissue, t0: int, t1: int,
                    obs_times: Sequence[int], observations, iterations: int = 200,
                    lr: float = 2e-5, bounds=(1e-4, 2e-3), smooth_cells: float = 2.0,
                    dt: float = 0.01, dx: float = 0.01, Cm: float = 1.0, seg: int = None,
                    callback=None):
    """The inverse problem: fits the per-cell diffusivity map to recordings of u.

    ``observations`` is (B, n_obs, H, W): u of B experiments (sharing D and the parameters
    ``theta``, each with its own initial state in ``states0`` (B, 3, H, W) and stimulus list)
    at ``obs_times``.  Each iteration runs :func:`rollout_batch` (forward, then the adjoint
    with sqrt(T) checkpoint-recompute), takes the mean squared error of u against the
    observations, and makes one Adam step (learning rate ``lr``, in the units of D).

    D is the Gaussian blur (``smooth_cells`` cells; 0: none) of a free map that Adam updates
    and that is clipped to ``bounds`` after each step: independent per-cell steps make D rough,
    and on a rough D the explicit scheme -- its D_x u_x term and one-sided edge rows -- diverges
    within a few hundred steps (as it does for per-cell noise in D), while the blurred map stays
    smooth and inside the bounds (a blur of a clipped map is a convex combination).
    ``callback(it, loss, D)`` is called after every step.  Returns the fitted D and the list of
    losses (the loss of each iteration's D, before its step)."""
    phi = D_init.detach().clone().to(torch.float32).requires_grad_(True)
    theta = theta.detach()
    opt = torch.optim.Adam([phi], lr=lr)
    to_D = (lambda f: gaussian_blur(f, smooth_cells)) if smooth_cells > 0 else (lambda f: f)
    losses = []
    for it in range(int(iterations)):
        opt.zero_grad(set_to_none=True)
        D = to_D(phi)
        out = rollout_batch(states0, D, theta, stimuli_per_tissue, t0, t1, obs_times, dt, dx,
                            Cm, seg)
        loss = ((out[:, :, 2] - observations) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            phi.clamp_(float(bounds[0]), float(bounds[1]))
        losses.append(float(loss.detach()))
        if callback is not None:
            callback(it, losses[-1], D.detach())
    with torch.no_grad():
        return to_D(phi).detach(), losses
