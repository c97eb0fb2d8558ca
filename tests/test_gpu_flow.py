"""GPU: the dataflow kernel (many steps per cooperative launch, tiles ordered by per-tile flags)
against the per-step launches.  Both run the same tile code, so the results must agree bit for
bit -- any ordering bug (a tile reading a neighbour's halo before it was written, or writing a
buffer a neighbour still reads) shows up as a mismatch, usually in the first few steps.

Sizes cover one tile, fewer tiles than resident CTAs, many tiles per CTA, sliver edge tiles (a
last tile row or column of one cell), odd and even step counts, stimuli switching on inside the
launch, activation tracking, and the checkpointed forward.
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
    stims = [Stimulus(Protocol(0, 2, 1e9), f1), Stimulus(Protocol(37, 3, 1e9), f2)]
    return Tissue(shape, P3, D, stims)


def _state(t):
    torch.cuda.synchronize()
    return t.state[:, :, : t.W].clone()


def _check_status():
    from cardiax_gb300 import _native as N
    import ctypes
    v = ctypes.c_int(0)
    N.call("fk_device_status", 1, ctypes.byref(v))
    assert v.value == 0, f"device error word {v.value}"


@pytest.mark.parametrize("shape,steps", [
    ((24, 40), 7), ((32, 64), 50), ((33, 65), 51), ((100, 129), 64), ((257, 190), 41),
    ((1024, 1024), 30), ((2048, 2048), 12), ((4099, 515), 9), ((65, 4097), 10)])
def test_flow_equals_per_step(shape, steps):
    _gpu()
    a = _tissue(shape)
    b = _tissue(shape)
    a.advance(0, steps)
    b.advance(0, steps, schedule="flow")
    sa, sb = _state(a), _state(b)
    _check_status()
    assert torch.isfinite(sa).all()
    assert torch.equal(sa, sb), (shape, steps, (sa - sb).abs().max().item())


def test_flow_continues_across_calls():
    """Intervals of different parity chained in place, and a zero-step call."""
    _gpu()
    shape = (300, 260)
    a, b = _tissue(shape, 3), _tissue(shape, 3)
    a.advance(0, 120)
    for t0, t1 in ((0, 1), (1, 1), (1, 40), (40, 73), (73, 120)):
        b.advance(t0, t1, schedule="flow")
    _check_status()
    assert torch.equal(_state(a), _state(b))


def test_flow_activation_maps():
    _gpu()
    shape = (260, 300)
    a, b = _tissue(shape, 5), _tissue(shape, 5)
    a.track_activation(0.5)
    b.track_activation(0.5)
    a.advance(0, 400)
    b.advance(0, 400, schedule="flow")
    _check_status()
    assert torch.equal(_state(a), _state(b))
    for x, y in zip(a.activation_maps(), b.activation_maps()):
        assert torch.equal(x, y)
    assert (b.activation_maps()[2] > 0).any()


def test_forward_flow_equals_forward():
    """Checkpointed forward: fk_forward_flow (Tissue.forward) vs fk_forward; the initial state
    is left unchanged."""
    _gpu()
    import ctypes
    from cardiax_gb300 import _native as N
    from cardiax_gb300.tissue import stream_handle
    shape = (200, 330)
    t = _tissue(shape, 7)
    t.advance(0, 5)
    before = _state(t)
    ck = [5, 6, 6, 30, 61, 100]
    out_flow = t.forward(ck, schedule="flow")
    out_step = torch.empty_like(out_flow)
    arr = (ctypes.c_int64 * len(ck))(*ck)
    N.call("fk_forward", t.grid, t.state.data_ptr(), t.scratch.data_ptr(), t.D.data_ptr(),
           ctypes.byref(t.params), t.stim, t.n_stim, arr, len(ck), t.dt, t.dx,
           out_step.data_ptr(), stream_handle())
    torch.cuda.synchronize()
    _check_status()
    assert torch.equal(before, _state(t))
    W = t.W
    assert torch.equal(out_flow[..., :W], out_step[..., :W])


def test_flow_rejects_bad_arguments():
    _gpu()
    from cardiax_gb300 import _native as N
    from cardiax_gb300.tissue import stream_handle
    import ctypes
    t = _tissue((64, 64))
    flags = t._flow_flags()
    args = lambda src, dst, scr, nflags: (
        t.grid, src, dst, scr, t.D.data_ptr(), ctypes.byref(t.params), t.stim, t.n_stim, 0, 3,
        t.dt, t.dx, None, flags.data_ptr(), nflags, stream_handle())
    L = N.lib()
    s, x = t.state.data_ptr(), t.scratch.data_ptr()
    assert L.fk_forward_euler_flow(*args(s, s, s, flags.numel())) == 5        # scratch == src
    assert L.fk_forward_euler_flow(*args(s, s, x, flags.numel() - 1)) == 5    # too few flags
    assert L.fk_forward_euler_flow(*args(s, s, x, flags.numel())) == 0
