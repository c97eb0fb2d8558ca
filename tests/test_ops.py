"""The PyTorch operator registrations (torch.ops.cardiax_gb300.*): present, with schemas and
fake kernels that give the output shapes without a GPU (what torch.compile / torch.export
trace through).  The GPU tests check their values against the ctypes path."""
import pytest
import torch

import cardiax_gb300  # noqa: F401  (registers the operators)

OPS = ("step", "euler_step", "forward_euler", "forward", "batch_forward_euler", "adjoint_step")


def test_every_operator_is_registered():
    for name in OPS:
        op = getattr(torch.ops.cardiax_gb300, name)
        assert op.default._schema.name == f"cardiax_gb300::{name}"


def _meta(*shape):
    return torch.empty(shape, device="meta")


@pytest.mark.parametrize("H,W", [(3, 3), (17, 30)])
def test_fake_kernels_give_the_output_shapes(H, W):
    ops = torch.ops.cardiax_gb300
    s, D, p, f = _meta(3, H, W), _meta(H, W), torch.empty(14), _meta(H, W)
    assert ops.step(s, D, p, [0.0, 2.0, 1e9], [f], 0, 0.01).shape == (3, H, W)
    assert ops.euler_step(s, D, p, [], [], 0, 0.01, 0.01).shape == (3, H, W)
    assert ops.forward_euler(s, D, p, [0.0, 2.0, 1e9], [f], 0, 9, 0.01, 0.01).shape == (3, H, W)
    assert ops.forward(s, [0, 10, 20, 30], D, p, [], [], 0.01, 0.01).shape == (3, 3, H, W)
    lam, gD, gth = ops.adjoint_step(s, D, p, [], [], 5, 0.01, 0.01, s)
    assert lam.shape == (3, H, W) and gD.shape == (H, W) and gth.shape == (13,)
    outs = ops.batch_forward_euler([s, _meta(3, 5, 7)], [D, _meta(5, 7)], torch.empty(2, 14),
                                   [1, 0], [0.0, 2.0, 1e9], [f], 0, 4, 0.01, 0.01)
    assert [tuple(o.shape) for o in outs] == [(3, H, W), (3, 5, 7)]


def test_forward_euler_has_an_autograd_formula():
    from torch._C import _dispatch_has_kernel_for_dispatch_key as has
    assert has("cardiax_gb300::forward_euler", "Autograd")
