"""torch.ops.cardiax_gb300.* against the ctypes path (the same C entry points): bit for bit,
plus the operators' autograd formula against the adjoint rollout, their traceability by
torch.compile (fake kernels, fullgraph) and torch.library.opcheck's schema / fake checks."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)


def _same(a, b):
    torch.testing.assert_close(a, b, rtol=0, atol=0, equal_nan=True)


def _case(H=70, W=90, seed=5):
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(seed)
    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    D = (1e-3 * (1 - 0.6 * np.exp(-((i - H * rng.uniform()) ** 2 + (j - W * rng.uniform()) ** 2)
                                  / (0.05 * H * W)))).astype(np.float32)
    f1 = np.zeros((H, W), np.float32)
    f1[:, :8] = 20.0
    f2 = np.zeros((H, W), np.float32)
    f2[H // 2:H // 2 + 7, W // 2:W // 2 + 7] = 20.0
    protos = [0.0, 2.0, 1e9, 150.0, 2.0, 1e9]
    fields = [torch.as_tensor(f1, device=dev), torch.as_tensor(f2, device=dev)]
    state = torch.stack([torch.ones((H, W)), torch.ones((H, W)), torch.zeros((H, W))]).to(dev)
    return state, torch.as_tensor(D, device=dev), torch.tensor(P3), protos, fields


def _stims(protos, fields):
    from cardiax_gb300.stimulus import Protocol, Stimulus
    return [Stimulus(Protocol(*protos[3 * k:3 * k + 3]), f) for k, f in enumerate(fields)]


def test_ops_equal_the_ctypes_path_bitwise():
    _gpu()
    from cardiax_gb300 import solve
    ops = torch.ops.cardiax_gb300
    state, D, p, protos, fields = _case()
    st = solve.State(*state)
    stims = _stims(protos, fields)
    # advance to a state with a wave in it first
    x = solve._forward_euler(st, 0, 300, P3, D, stims, 0.01, 0.01)
    xs = torch.stack(list(x))
    _same(ops.step(xs, D, p, protos, fields, 300, 0.01),
          torch.stack(list(solve.step(x, 300, P3, D, stims, 0.01))))
    _same(ops.euler_step(xs, D, p, protos, fields, 300, 0.01, 0.01),
          torch.stack(list(solve.step_euler(x, 300, P3, D, stims, 0.01, 0.01))))
    _same(ops.forward_euler(state, D, p, protos, fields, 0, 300, 0.01, 0.01), xs)
    ck = [0, 100, 250, 400]
    want = solve.forward(st, ck, P3, D, stims, 0.01, 0.01)
    got = ops.forward(state, ck, D, p, protos, fields, 0.01, 0.01)
    assert got.shape == (3, 3) + tuple(state.shape[1:])
    for k in range(3):
        _same(got[k], torch.stack(list(want[k])))
    assert float(xs[2].max()) > 0.8  # the wave is there


def test_batch_op_equals_single_tissue_ops():
    _gpu()
    from cardiax_gb300 import params as Pm
    ops = torch.ops.cardiax_gb300
    cases = [_case(70, 90, 1), _case(33, 130, 2), _case(128, 64, 3)]
    sets = [Pm.PARAMSET_3, Pm.PARAMSET_1A, Pm.PARAMSET_4A]
    params = torch.tensor([list(s) for s in sets])
    outs = ops.batch_forward_euler([c[0] for c in cases], [c[1] for c in cases], params,
                                   [2, 2, 2], sum((c[3] for c in cases), []),
                                   sum((c[4] for c in cases), []), 0, 257, 0.01, 0.01)
    for c, prm, o in zip(cases, params, outs):
        _same(o, ops.forward_euler(c[0], c[1], prm, c[3], c[4], 0, 257, 0.01, 0.01))


def test_adjoint_step_op_equals_adjoint_helper():
    _gpu()
    from cardiax_gb300.adjoint import Adjoint
    from cardiax_gb300.tissue import Tissue
    ops = torch.ops.cardiax_gb300
    state, D, p, protos, fields = _case()
    x = ops.forward_euler(state, D, p, protos, fields, 0, 200, 0.01, 0.01)
    lam_next = torch.randn_like(x)
    lam, gD, gth = ops.adjoint_step(x, D, p, protos, fields, 200, 0.01, 0.01, lam_next)
    tis = Tissue(tuple(x.shape[1:]), P3, D, _stims(protos, fields))
    tis.set_state(x)
    W = tis.W
    ln = torch.zeros_like(tis.state)
    ln[..., :W] = lam_next
    out = torch.empty_like(tis.state)
    adj = Adjoint(tis)
    adj.step(tis.state, 200, ln, out)
    _same(lam, out[..., :W])
    _same(gD, adj.grad_D())
    _same(gth, adj.grad_theta().to(torch.float32))


def test_forward_euler_op_gradient_equals_rollout():
    """d/d(state, D, params) of a loss on forward_euler's output, through the dispatcher's
    autograd (the adjoint kernel), equals the gradient of adjoint.rollout bit for bit."""
    _gpu()
    from cardiax_gb300.adjoint import rollout
    ops = torch.ops.cardiax_gb300
    state, D, p, protos, fields = _case(48, 60)
    target = torch.rand_like(state)
    s1, D1, p1 = (x.clone().requires_grad_(True) for x in (state, D, p.cuda()))
    out = ops.forward_euler(s1, D1, p1, protos, fields, 0, 120, 0.01, 0.01)
    ((out - target) ** 2).sum().backward()
    s2, D2, th2 = (x.clone().requires_grad_(True) for x in (state, D, p[:13].cuda()))
    out2 = rollout(s2[0], s2[1], s2[2], D2, th2, _stims(protos, fields), 0, 120, [120])
    ((out2[0] - target) ** 2).sum().backward()
    _same(out.detach(), out2[0].detach())
    _same(s1.grad, s2.grad)
    _same(D1.grad, D2.grad)
    _same(p1.grad[:13], th2.grad)
    assert float(p1.grad[13]) == 0.0  # Cm is held fixed


def test_ops_trace_under_torch_compile():
    _gpu()
    ops = torch.ops.cardiax_gb300
    state, D, p, protos, fields = _case()

    def fn(s, d):
        y = ops.forward_euler(s, d, p, protos, fields, 0, 50, 0.01, 0.01)
        return ops.euler_step(y * 1.0, d, p, protos, fields, 50, 0.01, 0.01)

    compiled = torch.compile(fn, backend="aot_eager", fullgraph=True)
    _same(compiled(state, D), fn(state, D))


def test_opcheck_schema_and_fake_kernels():
    _gpu()
    state, D, p, protos, fields = _case(20, 24)
    tests = ("test_schema", "test_faketensor")
    torch.library.opcheck(torch.ops.cardiax_gb300.forward_euler.default,
                          (state, D, p, protos, fields, 0, 10, 0.01, 0.01), test_utils=tests)
    torch.library.opcheck(torch.ops.cardiax_gb300.step.default,
                          (state, D, p, protos, fields, 0, 0.01), test_utils=tests)
    torch.library.opcheck(torch.ops.cardiax_gb300.forward.default,
                          (state, [0, 3, 7], D, p, protos, fields, 0.01, 0.01), test_utils=tests)
