"""GPU: the strip kernel (packed FP32 pairs, 128-column strips, register windows) against the
tiled step kernel.  Both evaluate every cell with the same operations in the same order, so the
states must agree bit for bit after any number of steps.

Shapes cover interior-only tiles, every combination of edge rows and edge columns, widths not
divisible by 4 (a last quad with 1, 2 or 3 grid columns, where the one-sided column is the
quad's first, second, third or fourth cell), the smallest grids, tile rows with a single grid
row (H = 1 mod 32), last strips of 2 .. 5 columns, and a width of 1 mod 128, which the strip
kernel leaves to the tiled kernel (the default; fk_select_step_kernel(1) opts into the strip
kernel).  Stimuli: a dense edge field, a rectangle switching on
mid-run and a sparse dense field; activation tracking on.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _select(which):
    from cardiax_gb300 import _native as N
    N.call("fk_select_step_kernel", which)


def _tissue(shape, seed=0):
    import bench
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    H, W = shape
    D = bench.noisy_diffusivity(H, W, seed=seed)
    f1 = np.zeros(shape, np.float32)
    f1[:, : max(1, W // 10)] = 20.0
    f2 = np.zeros(shape, np.float32)
    f2[H // 3: H // 3 + max(1, H // 8), W // 2: W // 2 + max(1, W // 8)] = 15.0
    f3 = np.random.default_rng(seed).uniform(0, 1, shape).astype(np.float32)
    f3[f3 < 0.97] = 0
    stims = [Stimulus(Protocol(0, 2, 1e9), f1), Stimulus(Protocol(5, 3, 1e9), f2),
             Stimulus(Protocol(9, 2, 1e9), 10 * f3)]
    t = Tissue(shape, P3, D, stims)
    # a random non-resting start so that every cell's arithmetic is exercised from step 0
    g = torch.Generator().manual_seed(seed)
    st = torch.rand((3, H, W), generator=g)
    st[2] *= 1.2
    t.set_state(st)
    return t


def _check_status():
    from cardiax_gb300 import _native as N
    v = ctypes.c_int(0)
    N.call("fk_device_status", 1, ctypes.byref(v))
    assert v.value == 0, f"device error word {v.value}"


TILED, STRIP = 0, 1


def _run(shape, steps, which, track=False):
    _select(which)
    try:
        t = _tissue(shape)
        if track:
            t.track_activation(0.5)
        t.advance(0, steps)
        torch.cuda.synchronize()
        out = t.state[:, :, : t.W].clone()
        acts = t.activation_maps() if track else None
    finally:
        _select(0)
    return out, acts


SHAPES = [(3, 3), (3, 7), (4, 5), (5, 9), (7, 130), (9, 4), (17, 33), (20, 30), (33, 70),
          (31, 127), (32, 128), (33, 131), (40, 133), (64, 256), (65, 250), (96, 200),
          (100, 130), (129, 258), (257, 190), (300, 260), (200, 387), (1024, 1024),
          (70, 129), (512, 517)]


@pytest.mark.parametrize("shape", SHAPES)
def test_strip_equals_tiled(shape):
    _gpu()
    steps = 13
    a, _ = _run(shape, steps, TILED)
    b, _ = _run(shape, steps, STRIP)
    _check_status()
    assert torch.isfinite(a).all()
    diff = (a - b).abs()
    assert torch.equal(a, b), (shape, diff.max().item(), torch.nonzero(diff)[:8].tolist())


@pytest.mark.parametrize("shape", [(64, 96), (130, 259), (255, 384)])
def test_strip_activation_maps_equal_tiled(shape):
    _gpu()
    a, ma = _run(shape, 60, TILED, track=True)
    b, mb = _run(shape, 60, STRIP, track=True)
    _check_status()
    assert torch.equal(a, b)
    for x, y in zip(ma, mb):
        assert torch.equal(x, y)


def test_select_rejects_unknown_kernel():
    from cardiax_gb300 import _native as N
    with pytest.raises(N.FkError):
        N.call("fk_select_step_kernel", 7)
