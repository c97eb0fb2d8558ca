"""GPU: the temporally blocked stepper (depth 2, 4, 8 steps per launch) against one step per
launch.  Same per-cell arithmetic, so the results must agree bit for bit; a wrong halo, a missed
edge re-padding between blocked steps or a stale region shows up as a mismatch.

Shapes: interior-only work (large grid), tiles whose blocked halo crosses one or two edges,
tiny grids where every tile is an edge tile, partial last tiles, and one-cell last tile rows /
columns (which fall back to one step per launch); step counts that are not multiples of the
depth (the remainder runs one step per launch); stimuli switching on inside a block.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


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
    f3[f3 < 0.97] = 0  # a sparse dense field (not a rectangle)
    stims = [Stimulus(Protocol(0, 2, 1e9), f1), Stimulus(Protocol(5, 3, 1e9), f2),
             Stimulus(Protocol(9, 2, 1e9), 10 * f3)]
    return Tissue(shape, P3, D, stims)


def _state(t):
    torch.cuda.synchronize()
    return t.state[:, :, : t.W].clone()


def _check_status():
    import ctypes
    from cardiax_gb300 import _native as N
    v = ctypes.c_int(0)
    N.call("fk_device_status", 1, ctypes.byref(v))
    assert v.value == 0, f"device error word {v.value}"


@pytest.mark.parametrize("depth", [2, 4, 8])
@pytest.mark.parametrize("shape,steps", [
    ((3, 3), 9), ((5, 9), 8), ((20, 30), 17), ((64, 128), 24), ((100, 130), 40),
    ((96, 200), 16), ((257, 190), 10), ((33, 70), 8), ((300, 260), 33), ((1024, 1024), 24)])
def test_blocked_equals_per_step(depth, shape, steps):
    _gpu()
    a, b = _tissue(shape), _tissue(shape)
    a.advance(0, steps)
    b.advance(0, steps, depth=depth)
    sa, sb = _state(a), _state(b)
    _check_status()
    assert torch.isfinite(sa).all()
    assert torch.equal(sa, sb), (depth, shape, steps, (sa - sb).abs().max().item())


def test_blocked_continues_across_calls():
    _gpu()
    shape = (200, 330)
    a, b = _tissue(shape, 4), _tissue(shape, 4)
    a.advance(0, 70)
    for t0, t1, k in ((0, 3, 2), (3, 3, 4), (3, 20, 4), (20, 45, 8), (45, 70, 2)):
        b.advance(t0, t1, depth=k)
    _check_status()
    assert torch.equal(_state(a), _state(b))


def test_blocked_rejects_bad_depth():
    _gpu()
    import ctypes
    from cardiax_gb300 import _native as N
    from cardiax_gb300.tissue import stream_handle
    t = _tissue((64, 64))
    rc = N.lib().fk_forward_euler_tb(t.grid, t.state.data_ptr(), t.scratch.data_ptr(),
                                     t.D.data_ptr(), ctypes.byref(t.params), t.stim, t.n_stim,
                                     0, 4, t.dt, t.dx, 3, stream_handle())
    assert rc == 5
