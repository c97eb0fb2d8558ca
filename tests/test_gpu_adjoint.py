"""The hand-written adjoint (through torch.autograd) against float64 autodiff of the oracle
(the stand-in for jax.grad of the reference) and central finite differences.

Regime: smooth sub-threshold states (no gate flips between float32 and float64 trajectories),
a sub-threshold stimulus so that the stimulated-cell masking is exercised.  Bar: relative error
(norm-wise per gradient) <= 1e-3.
"""
import numpy as np
import pytest
import torch

import fk_torch as FT

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
TOL = 1e-3


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _smooth(rng, shape, lo, hi):
    H, W = shape
    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    f = np.zeros(shape)
    for _ in range(3):
        ci, cj, s = rng.uniform(0, H), rng.uniform(0, W), rng.uniform(0.2, 0.5) * max(H, W)
        f += rng.uniform(-1, 1) * np.exp(-((i - ci) ** 2 + (j - cj) ** 2) / (2 * s * s))
    f = (f - f.min()) / (f.max() - f.min() + 1e-12)
    return lo + (hi - lo) * f


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    H, W = shape
    v0 = _smooth(rng, shape, 0.8, 1.0)
    w0 = _smooth(rng, shape, 0.8, 1.0)
    u0 = _smooth(rng, shape, 0.0, 0.09)
    D = _smooth(rng, shape, 3e-4, 1e-3)
    f = np.zeros(shape)
    f[H // 3: H // 3 + 4, 2:7] = 0.5
    stim = (3, 2, 1e9, f)
    obs = [10, 30]
    R = rng.standard_normal((len(obs), 3, H, W)) * np.array([0.1, 0.1, 1.0])[None, :, None, None]
    return v0, w0, u0, D, stim, obs, R


def _oracle_grads(v0, w0, u0, D, stim, obs, R):
    t = lambda x: torch.tensor(x, dtype=torch.float64, requires_grad=True)  # noqa: E731
    V, Wt, U, Dt = t(v0), t(w0), t(u0), t(D)
    th = torch.tensor(P3[:13], dtype=torch.float64, requires_grad=True)
    st = [(stim[0], stim[1], stim[2], torch.tensor(stim[3], dtype=torch.float64))]
    state = (V, Wt, U)
    L = 0
    tcur = 0
    for k, to in enumerate(obs):
        state = FT.forward(state, tcur, to, th, 1.0, Dt, st, 0.01, 0.01)
        tcur = to
        L = L + sum((state[c] * torch.tensor(R[k, c])).sum() for c in range(3))
    L.backward()
    return V.grad.numpy(), Wt.grad.numpy(), U.grad.numpy(), Dt.grad.numpy(), th.grad.numpy()


def _gpu_grads(v0, w0, u0, D, stim, obs, R, seg=None):
    from cardiax_gb300.adjoint import rollout
    from cardiax_gb300.stimulus import Protocol, Stimulus
    dev = torch.device("cuda", 0)
    g = lambda x: torch.tensor(x, dtype=torch.float32, device=dev, requires_grad=True)  # noqa: E731
    V, Wt, U, Dt = g(v0), g(w0), g(u0), g(D)
    th = torch.tensor(P3[:13], dtype=torch.float32, device=dev, requires_grad=True)
    out = rollout(V, Wt, U, Dt, th, [Stimulus(Protocol(*stim[:3]), stim[3].astype(np.float32))],
                  0, max(obs), obs, seg=seg)
    L = (out * torch.tensor(R, dtype=torch.float32, device=dev)).sum()
    L.backward()
    return tuple(x.grad.detach().cpu().numpy() for x in (V, Wt, U, Dt, th))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("shape,seg", [((20, 24), None), ((48, 40), 7), ((13, 70), 30),
                                       ((64, 72), 16)])
def test_adjoint_matches_fp64_autodiff(shape, seg):
    _gpu()
    case = _case(shape, sum(shape))
    ref = _oracle_grads(*case)
    got = _gpu_grads(*case, seg=seg)
    names = ("v0", "w0", "u0", "D", "theta")
    for n, a, b in zip(names, got, ref):
        e = _rel(a, b)
        print(f"{shape} grad {n}: relative error {e:.2e}")
        assert e <= TOL, (n, e)
    # V_v enters only through a Heaviside gate
    assert got[4][12] == 0.0


def test_adjoint_matches_finite_differences_on_D():
    """Central differences (eps = 1e-3 relative) of the float64 oracle on 8 seeded D entries."""
    _gpu()
    shape = (24, 28)
    v0, w0, u0, D, stim, obs, R = _case(shape, 5)
    got = _gpu_grads(v0, w0, u0, D, stim, obs, R)[3]
    rng = np.random.default_rng(0)
    st = [(stim[0], stim[1], stim[2], torch.tensor(stim[3], dtype=torch.float64))]
    th = torch.tensor(P3[:13], dtype=torch.float64)

    def loss(Dm):
        state = tuple(torch.tensor(x, dtype=torch.float64) for x in (v0, w0, u0))
        L, tcur = 0.0, 0
        for k, to in enumerate(obs):
            state = FT.forward(state, tcur, to, th, 1.0, torch.tensor(Dm), st, 0.01, 0.01)
            tcur = to
            L += float(sum((state[c] * torch.tensor(R[k, c])).sum() for c in range(3)))
        return L

    for _ in range(8):
        i, j = int(rng.integers(0, shape[0])), int(rng.integers(0, shape[1]))
        eps = 1e-3 * D[i, j]
        Dp, Dm = D.copy(), D.copy()
        Dp[i, j] += eps
        Dm[i, j] -= eps
        fd = (loss(Dp) - loss(Dm)) / (2 * eps)
        assert abs(got[i, j] - fd) <= 1e-3 * max(abs(fd), 1e-3 * np.abs(got).max()), (i, j, got[i, j], fd)


def test_batched_rollout_equals_single_rollouts():
    """rollout_batch (one stream per experiment, shared D and theta) gives the sums of the
    single-experiment gradients."""
    _gpu()
    from cardiax_gb300.adjoint import rollout, rollout_batch
    from cardiax_gb300.stimulus import Protocol, Stimulus
    dev = torch.device("cuda", 0)
    shape = (40, 52)
    cases = [_case(shape, s) for s in (21, 22, 23)]
    D = torch.tensor(cases[0][3], dtype=torch.float32, device=dev, requires_grad=True)
    th = torch.tensor(P3[:13], dtype=torch.float32, device=dev, requires_grad=True)
    s0 = torch.tensor(np.stack([np.stack(c[:3]) for c in cases]), dtype=torch.float32, device=dev)
    stims = [[Stimulus(Protocol(*c[4][:3]), c[4][3].astype(np.float32))] for c in cases]
    obs = cases[0][5]
    R = torch.tensor(np.stack([c[6] for c in cases]), dtype=torch.float32, device=dev)
    out = rollout_batch(s0, D, th, stims, 0, max(obs), obs)
    (out * R).sum().backward()
    gD_b, gth_b = D.grad.clone(), th.grad.clone()
    D.grad = None
    th.grad = None
    total = 0
    for b in range(3):
        o = rollout(s0[b, 0], s0[b, 1], s0[b, 2], D, th, stims[b], 0, max(obs), obs)
        total = total + (o * R[b]).sum()
    total.backward()
    # the per-experiment gradients are summed in a different order (float32): compare relative
    # to the largest entry, as cancellation leaves a few entries near zero
    torch.testing.assert_close(gD_b, D.grad, rtol=1e-5, atol=1e-5 * D.grad.abs().max().item())
    torch.testing.assert_close(gth_b, th.grad, rtol=1e-5, atol=1e-5 * th.grad.abs().max().item())


@pytest.mark.parametrize("shape,seg,obs", [((40, 52), 7, [0, 10, 30]), ((33, 130), 5, [12, 23])])
def test_batched_reverse_pass_equals_per_experiment_bit_for_bit(shape, seg, obs):
    """rollout_batch runs the forward, the segment recomputation and the adjoint as one launch
    per step for all experiments; per experiment that is the same arithmetic as the experiment's
    own reverse pass (Adjoint.rollout_gradient on its Tissue), so the cotangent of the initial
    state matches bit for bit, and dL/dD, dL/dtheta are the experiment-order sums of the
    per-experiment values.  Several segments (seg 5, 7), observations on a segment boundary and at
    the first step."""
    _gpu()
    from cardiax_gb300.adjoint import Adjoint, rollout_batch
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    dev = torch.device("cuda", 0)
    H, W = shape
    cases = [_case(shape, s) for s in (31, 32, 33)]
    Dn = cases[0][3].astype(np.float32)
    D = torch.tensor(Dn, device=dev, requires_grad=True)
    th = torch.tensor(P3[:13], dtype=torch.float32, device=dev, requires_grad=True)
    s0 = torch.tensor(np.stack([np.stack(c[:3]) for c in cases]), dtype=torch.float32, device=dev,
                      requires_grad=True)
    stims = [[Stimulus(Protocol(*c[4][:3]), c[4][3].astype(np.float32))] for c in cases]
    rng = np.random.default_rng(5)
    R = torch.tensor(rng.standard_normal((3, len(obs), 3, H, W)), dtype=torch.float32, device=dev)
    out = rollout_batch(s0, D, th, stims, 0, max(obs), obs, seg=seg)
    (out * R).sum().backward()

    gD_sum, gth_sum = None, None
    for b in range(3):
        tis = Tissue(shape, list(P3), Dn, stims[b], device=dev)
        tis.set_state(s0[b].detach())
        state0 = tis.state.clone()
        adj = Adjoint(tis)
        g = torch.zeros((len(obs),) + tuple(state0.shape), dtype=torch.float32, device=dev)
        g[..., :W] = R[b]
        lam0 = adj.rollout_gradient(state0, 0, max(obs), obs, g, seg=seg)
        torch.cuda.synchronize()
        assert torch.equal(lam0[..., :W], s0.grad[b]), b
        gD_sum = adj.grad_D().clone() if gD_sum is None else gD_sum + adj.grad_D()
        gth_sum = adj.grad_theta() if gth_sum is None else gth_sum + adj.grad_theta()
    assert torch.equal(gD_sum, D.grad)
    assert torch.equal(gth_sum.to(torch.float32), th.grad)
