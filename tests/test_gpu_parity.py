"""GPU parity: the CUDA stepper (through the C ABI) against the reference's golden vectors and
the CPU oracle.

Tolerances (float32, stated per test): the kernels multiply by float32 reciprocals and use
fused multiply-adds where the reference divides and rounds each product, so single-step
derivatives differ from the reference in the last bits; over 1000 steps of a travelling wave
these differences grow to ~1e-5 (the oracle's own float32-vs-float64 gap is the same size), and
the bar is max|du| <= 1e-4.
"""
import numpy as np
import pytest
import torch

import fk_oracle as O

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
TOL_U_1000 = 1e-4   # pointwise max|du| after 1000 steps (the stated parity bar)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _np(t):
    return t.detach().cpu().numpy()


def test_step_derivative_golden(golden):
    """fk_step vs the reference's step on small grids with two stimuli."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    s = golden("step.npz")
    for k in range(4):
        st = solve.State(*(torch.as_tensor(s[f"{n}_{k}"]) for n in "vwu"))
        stims = [Stimulus(Protocol(0, 2, 1e9), s[f"f1_{k}"]), Stimulus(Protocol(1, 3, 7), s[f"f2_{k}"])]
        for t in (0, 1, 5):
            d = solve.step(st, t, P3, s[f"D_{k}"], stims, 0.01)
            for name, arr in zip(("dv", "dw", "du"), d):
                ref = s[f"{name}_{k}_{t}"]
                err = np.abs(_np(arr) - ref).max() / max(1.0, np.abs(ref).max())
                assert err <= (1e-4 if name == "du" else 1e-6), (name, k, t, err)


@pytest.mark.parametrize("tag,dtype", [("f32", np.float32)])
def test_forward_small_golden(golden, tag, dtype):
    """200 steps on 32x40 with a smooth D and two stimuli vs the reference (f32) and the
    reference with x64 (reported)."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    g = golden("forward_small.npz")
    shp = g["D"].shape
    stims = [Stimulus(Protocol(0, 2, 1e9), g["f1"]), Stimulus(Protocol(60, 3, 1e9), g["f2"])]
    res = solve._forward_euler(solve.init(shp), 0, 200, P3, g["D"], stims, 0.01, 0.01)
    for name, arr in zip("vwu", res):
        e32 = np.abs(_np(arr) - g[f"{name}_f32"]).max()
        e64 = np.abs(_np(arr) - g[f"{name}_f64"]).max()
        print(f"forward_small {name}: |gpu-ref32| {e32:.3g}  |gpu-ref64| {e64:.3g}")
        assert e32 <= TOL_U_1000


@pytest.mark.parametrize("tag", ["plain", "excite"])
def test_config0_1000_steps_golden(golden, tag):
    """The 128x128 configuration, 1000 steps, checkpoints every 100: max|du| <= 1e-4 at every
    checkpoint vs the reference."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    g = golden("config0.npz")
    proto = Protocol(0, 200, 1e9) if tag == "plain" else Protocol(0, 2, 1e9)
    D = np.full((128, 128), 0.001, np.float32)
    states = solve.forward(solve.init((128, 128)), list(range(0, 1001, 100)), P3, D,
                           [Stimulus(proto, g[f"{tag}_field"])], 0.01, 0.01)
    assert len(states) == 10
    worst = 0.0
    for i, s in enumerate(states):
        e = np.abs(_np(s.u) - g[f"{tag}_u_{(i + 1) * 100}"]).max()
        worst = max(worst, e)
        assert e <= TOL_U_1000, (tag, (i + 1) * 100, e)
    assert np.abs(_np(states[-1].v) - g[f"{tag}_v_final"]).max() <= TOL_U_1000
    assert np.abs(_np(states[-1].w) - g[f"{tag}_w_final"]).max() <= TOL_U_1000
    print(f"config0 {tag}: max|du| over checkpoints {worst:.3g}")
    if tag == "excite":
        assert float(states[-1].u.max()) > 0.9  # the wave did propagate


def _smooth(rng, shape, lo, hi):
    H, W = shape
    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    f = np.zeros(shape)
    for _ in range(3):
        ci, cj, s = rng.uniform(0, H), rng.uniform(0, W), rng.uniform(0.2, 0.5) * max(H, W)
        f += rng.uniform(-1, 1) * np.exp(-((i - ci) ** 2 + (j - cj) ** 2) / (2 * s * s))
    f = (f - f.min()) / (f.max() - f.min() + 1e-12)
    return (lo + (hi - lo) * f).astype(np.float32)


@pytest.mark.parametrize("shape", [(3, 3), (3, 5), (5, 3), (4, 7), (9, 13), (33, 37), (7, 130),
                                   (130, 7), (64, 64), (100, 260)])
def test_edge_shapes_vs_oracle(shape):
    """Grids that exercise every boundary formula, widths that are not multiples of 4 and tiles
    that are partly outside the grid: derivative and 60 Euler steps vs the oracle."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    rng = np.random.default_rng(sum(shape))
    st = tuple(_smooth(rng, shape, 0.0, 1.0) for _ in range(3))
    D = _smooth(rng, shape, 3e-4, 1e-3)
    f = np.zeros(shape, np.float32)
    f[:, : max(1, shape[1] // 4)] = 15.0
    stims_o = [O.OStim(0, 2, 1e9, f)]
    stims_g = [Stimulus(Protocol(0, 2, 1e9), f)]
    d_ref = O.derivative(O.OState(*st), np.float32(0), P3, D, stims_o, 0.01)
    d_gpu = solve.step(solve.State(*map(torch.as_tensor, st)), 0, P3, D, stims_g, 0.01)
    for a, b in zip(d_gpu, d_ref):
        assert np.abs(_np(a) - b).max() / max(1.0, np.abs(b).max()) <= 1e-4
    ref = O.forward_euler(O.OState(*st), 0, 60, P3, D, stims_o, 0.01, 0.01)
    got = solve._forward_euler(solve.State(*map(torch.as_tensor, st)), 0, 60, P3, D, stims_g,
                               0.01, 0.01)
    for a, b in zip(got, ref):
        assert np.all(np.isfinite(_np(a)))
        assert np.abs(_np(a) - b).max() <= 1e-4, shape


def test_rect_and_dense_stimuli_agree_bitwise():
    """A constant rectangle runs as a descriptor, a field with two values as a dense plane;
    equal fields must give identical bits, and overlapping stimuli follow list order."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    shp = (48, 72)
    r1 = np.zeros(shp, np.float32)
    r1[10:20, 30:50] = 8.0
    r2 = np.zeros(shp, np.float32)
    r2[30:40, 5:9] = 8.0
    dense = r1 + r2  # not a single rectangle -> dense plane
    D = np.full(shp, 8e-4, np.float32)
    a = solve._forward_euler(solve.init(shp), 0, 30, P3, D,
                             [Stimulus(Protocol(0, 5, 10), r1), Stimulus(Protocol(0, 5, 10), r2)],
                             0.01, 0.01)
    b = solve._forward_euler(solve.init(shp), 0, 30, P3, D, [Stimulus(Protocol(0, 5, 10), dense)],
                             0.01, 0.01)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    from cardiax_gb300.tissue import analyse_field
    assert analyse_field(torch.as_tensor(dense).cuda())[0] == "dense"
    assert analyse_field(torch.as_tensor(r1).cuda())[0] == "rect"
    # overlap: later stimulus wins where both are non-zero
    s1 = np.zeros(shp, np.float32); s1[:, :10] = 5.0
    s2 = np.zeros(shp, np.float32); s2[:, 5:15] = 9.0
    stims = [Stimulus(Protocol(0, 2, 1e9), s1), Stimulus(Protocol(0, 2, 1e9), s2)]
    d = solve.step(solve.init(shp), 0, P3, D, stims, 0.01)
    ref = O.derivative(O.init(shp), np.float32(0), P3, D, [O.OStim(0, 2, 1e9, s1), O.OStim(0, 2, 1e9, s2)], 0.01)
    assert np.abs(_np(d.u) - ref.u).max() <= 1e-4


def test_forward_is_deterministic_and_matches_stepwise():
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus, linear, Direction
    shp = (96, 160)
    D = np.full(shp, 1e-3, np.float32)
    stims = [linear(shp, Direction.WEST, 0.05, 20.0, Protocol(0, 2, 1e9))]
    a = solve.forward(solve.init(shp), [0, 7, 20, 20, 45], P3, D, stims, 0.01, 0.01)
    b = solve.forward(solve.init(shp), [0, 7, 20, 20, 45], P3, D, stims, 0.01, 0.01)
    assert len(a) == 4
    for x, y in zip(a, b):
        for p, q in zip(x, y):
            assert torch.equal(p, q)
    assert torch.equal(a[1].u, a[2].u)  # repeated checkpoint
    s = solve.init(shp)
    for t in range(45):
        s = solve.step_euler(s, t, P3, D, stims, 0.01, 0.01)
    for p, q in zip(a[-1], s):
        assert torch.equal(p, q)


def _staggered_stimuli(shp, n, seed):
    """n stimuli (rectangles and dense fields) whose protocols overlap in time a few at once."""
    from cardiax_gb300.stimulus import Protocol, Stimulus
    rng = np.random.default_rng(seed)
    H, W = shp
    out_g, out_o = [], []
    for k in range(n):
        f = np.zeros(shp, np.float32)
        r, c = int(rng.integers(0, H - 6)), int(rng.integers(0, W - 6))
        if k % 3 == 2:  # a field with two values: a dense plane
            f[r:r + 6, c:c + 3] = 6.0 + k
            f[r:r + 6, c + 3:c + 6] = 2.0
        else:
            f[r:r + 6, c:c + 6] = 4.0 + k
        start, dur, period = 7 * k, 3, 40 + 5 * (k % 4)
        out_g.append(Stimulus(Protocol(start, dur, period), f))
        out_o.append(O.OStim(start, dur, period, f))
    return out_g, out_o


def test_more_stimuli_than_a_launch_holds_vs_oracle():
    """20 stimuli, a few active at any step: each launch takes the ones active at its step (in
    list order, overlaps included); 300 Euler and 60 Heun steps against the oracle, and every
    schedule gives the per-step bits."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.tissue import Tissue
    shp = (48, 72)
    rng = np.random.default_rng(5)
    D = _smooth(rng, shp, 4e-4, 1e-3)
    stims_g, stims_o = _staggered_stimuli(shp, 20, 3)
    got = solve._forward_euler(solve.init(shp), 0, 300, P3, D, stims_g, 0.01, 0.01)
    ref = O.forward_euler(O.init(shp), 0, 300, P3, D, stims_o, 0.01, 0.01)
    worst = max(float(np.abs(_np(a) - b).max()) for a, b in zip(got, ref))
    assert worst <= 1e-4, worst
    assert float(got.u.max()) > 0.5  # the stimuli excited the tissue
    d = solve.step(solve.init(shp), 21, P3, D, stims_g, 0.01)
    d_ref = O.derivative(O.init(shp), np.float32(21), P3, D, stims_o, 0.01)
    assert np.abs(_np(d.u) - d_ref.u).max() <= 1e-4
    h = solve._forward_heun(solve.init(shp), 0, 60, P3, D, stims_g, 0.01, 0.01)
    h_ref = O.forward_heun(O.init(shp), 0, 60, P3, D, stims_o, 0.01, 0.01)
    assert max(float(np.abs(_np(a) - b).max()) for a, b in zip(h, h_ref)) <= 1e-4
    ck = [0, 50, 120, 300]
    fw = solve.forward(solve.init(shp), ck, P3, D, stims_g, 0.01, 0.01)
    for p, q in zip(fw[-1], got):
        assert torch.equal(p, q)
    for kw in ({"schedule": "flow"}, {"depth": 2}, {"schedule": "auto"}):
        t = Tissue(shp, P3, D, stims_g)
        t.advance(0, 300, **kw)
        for p, q in zip(t.view(), got):
            assert torch.equal(p, q), kw
    print(f"20 stimuli, 300 steps: max|d| vs oracle {worst:.3g}")


def test_too_many_stimuli_rejected():
    """Nine stimuli active at the same step exceed a launch's slots (FkError from the library);
    more than FK_MAX_STIMULI non-zero stimuli are refused before any launch (ValueError)."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300._native import FK_MAX_STIMULI, FkError
    from cardiax_gb300.stimulus import Protocol, Stimulus
    shp = (16, 16)
    D = np.full(shp, 1e-3, np.float32)
    stims = []
    for k in range(9):
        f = np.zeros(shp, np.float32)
        f[k, :] = 1.0
        stims.append(Stimulus(Protocol(0, 2, 5), f))
    with pytest.raises(FkError):
        solve._forward_euler(solve.init(shp), 0, 3, P3, D, stims, 0.01, 0.01)
    many = []
    for k in range(FK_MAX_STIMULI + 1):
        f = np.zeros(shp, np.float32)
        f[k % 16, k // 16] = 1.0
        many.append(Stimulus(Protocol(1000 * k, 2, 1e9), f))
    with pytest.raises(ValueError):
        solve._forward_euler(solve.init(shp), 0, 3, P3, D, many, 0.01, 0.01)


def _c_oracle():
    import fk_oracle_c as C
    C.build()
    return C


def _roofline_D(H, W, seed):
    import bench
    return bench.noisy_diffusivity(H, W, seed)


def test_full_size_2048_subthreshold_arithmetic():
    """2048x2048 with the roofline D map (5% noise) and a smooth sub-threshold state (u < V_v
    everywhere, so no gate can flip): 100 steps vs the C oracle.  This isolates the stencil and
    diffusion arithmetic at full size; the bound reflects last-bit differences."""
    _gpu()
    C = _c_oracle()
    from cardiax_gb300 import solve
    H = W = 2048
    rng = np.random.default_rng(3)
    D = _roofline_D(H, W, 3)
    st0 = O.init((H, W))
    st0.u[:, :] = _smooth(rng, (H, W), 0.0, 0.03)
    ref = C.forward_euler(st0, 0, 100, P3, D, [], 0.01, 0.01, threads=C.max_threads())
    got = solve._forward_euler(solve.State(*map(torch.as_tensor, st0)), 0, 100, P3, D, [],
                               0.01, 0.01)
    for a, b in zip(got, ref):
        assert np.abs(_np(a) - b).max() <= 1e-6


def test_full_size_2048_planar_wave():
    """2048x2048, noisy D, the periodic left-edge stimulus of the roofline configuration
    (amplitude 20, Protocol(0, 200, 20000)), 400 steps from rest vs the C oracle.  A cell whose u
    lands within one ulp of V_c flips the Heaviside gate a step early or late (then v, w jump by
    ~1e-3 and u by ~2e-4 there); with a 2048-row wave front such near-ties do happen, so at full
    size all but 1e-5 of the cells must agree to 1e-4 and none by more than 1e-2."""
    _gpu()
    C = _c_oracle()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    H = W = 2048
    D = _roofline_D(H, W, 5)
    f = np.zeros((H, W), np.float32)
    f[:, :5] = 20.0
    ref = C.forward_euler(O.init((H, W)), 0, 400, P3, D, [(0, 200, 20000, f)], 0.01, 0.01,
                          threads=C.max_threads())
    got = solve._forward_euler(solve.init((H, W)), 0, 400, P3, D,
                               [Stimulus(Protocol(0, 200, 20000), f)], 0.01, 0.01)
    gu = _np(got.u)
    assert float(gu[:, 12].min()) > 0.5  # the wave has travelled past column 12
    for a, b in zip(got, ref):
        d = np.abs(_np(a) - b)
        assert (d > 1e-4).mean() <= 1e-5 and d.max() <= 1e-2


def test_activation_times_within_one_step():
    """Activation-time maps (upstrokes through u = 0.5) of a planar wave plus a later point
    stimulus on 256x256 with a smooth D (down to 1e-4, where conduction is slow), 6000 steps:
    GPU vs the float32 C oracle.  Where the front crawls through low-D tissue, last-bit
    differences shift activation times: the oracle's own float32 run differs from its float64
    run by up to several steps here.  The bar: at least 99% of the cells within one step, and
    no cell further off than the oracle's float32-vs-float64 spread (and never more than 4)."""
    _gpu()
    C = _c_oracle()
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    H = W = 256
    rng = np.random.default_rng(11)
    D = _smooth(rng, (H, W), 1e-4, 1e-3)
    f1 = np.zeros((H, W), np.float32); f1[:, :5] = 20.0
    f2 = np.zeros((H, W), np.float32); f2[200:210, 100:110] = 20.0
    stims = [(0, 2, 1e9, f1), (1500, 2, 1e9, f2)]
    maps = {}
    for dt_ in (np.float32, np.float64):
        first = np.full((H, W), -1, np.int32); last = first.copy()
        count = np.zeros((H, W), np.int32)
        C.forward_euler(O.init((H, W), dt_), 0, 6000, P3, D.astype(dt_),
                        [s[:3] + (s[3].astype(dt_),) for s in stims], 0.01, 0.01,
                        threads=C.max_threads(), activation=(first, last, count, 0.5))
        maps[dt_] = (first, last, count)
    first, last, count = maps[np.float32]
    tis = Tissue((H, W), P3, D, [Stimulus(Protocol(*s[:3]), s[3]) for s in stims])
    tis.track_activation(0.5).advance(0, 6000)
    gf, gl, gc = (_np(x) for x in tis.activation_maps())
    assert (first >= 0).mean() > 0.8  # the wave reached most of the tissue
    # a cell reached by the front in the last steps may be one step early or late in either run
    settled = ((first < 0) | (first < 5996)) & ((gf < 0) | (gf < 5996))
    assert np.array_equal((gf >= 0)[settled], (first >= 0)[settled])
    both = (gf >= 0) & (first >= 0)
    f64 = maps[np.float64][0]
    both64 = both & (f64 >= 0)
    spread = int(np.abs(first - f64)[both64].max())
    d = np.abs(gf - first)[both]
    print(f"activation: gpu-vs-f32 max {d.max()} (within 1 step: {(d <= 1).mean():.5f}); "
          f"f32-vs-f64 max {spread}")
    assert (d <= 1).mean() >= 0.99
    assert d.max() <= min(max(1, spread), 4)
    dl = np.abs(gl - last)[both]
    assert (dl <= 1).mean() >= 0.99 and dl.max() <= 4


def test_forward_dimensional_vs_oracle():
    """forward_dimensional (cardiax/solve.py:133-165): the grid from the tissue size, the
    checkpoints arange(0, int(final_time/dt), int(ms_step/dt)) -- the stop excluded, the
    initial state not returned -- against the oracle's forward on those checkpoints."""
    _gpu()
    from cardiax_gb300 import convert, solve
    from cardiax_gb300.stimulus import Direction, Protocol, linear
    size, final_time, ms_step, dt, dx = (0.64, 0.8), 5.0, 1.0, 0.01, 0.01
    shape = convert.realsize_to_shape(size, dx)
    assert shape == (64, 80)
    rng = np.random.default_rng(11)
    D = _smooth(rng, shape, 4e-4, 1e-3)
    stim = linear(shape, Direction.WEST, 0.15, 20.0, Protocol(0, 2, 1e9))
    states = solve.forward_dimensional(size, final_time, ms_step, P3, D, [stim], dt, dx)
    ck = list(range(0, int(final_time / dt), int(ms_step / dt)))
    assert ck == [0, 100, 200, 300, 400] and len(states) == len(ck) - 1
    ref = O.forward(O.init(shape), ck, P3, D, [O.OStim(0, 2, 1e9, _np(stim.field))], dt, dx)
    for s, r in zip(states, ref):
        for var in "vwu":
            e = float(np.abs(_np(getattr(s, var)) - getattr(r, var)).max())
            assert e <= TOL_U_1000, (var, e)
    assert float(states[-1].u.max()) > 0.8


def test_stimulus_schedule_on_the_device():
    """The kernels' protocol test step by step against the reference's schedules (its own
    stimulate_test.py cases and the floor-mod quirks, tests/golden/stimulus_schedule.json) and
    negative or fractional periods: the derivative of a resting cell under a one-cell stimulus
    of 5 is 5 exactly when the protocol is on."""
    _gpu()
    import json
    import os
    from conftest import GOLDEN
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    shp = (8, 8)
    D = np.full(shp, 1e-3, np.float32)
    f = np.zeros(shp, np.float32)
    f[4, 4] = 5.0
    sched = json.load(open(os.path.join(GOLDEN, "stimulus_schedule.json")))
    protos = [tuple(rec["protocol"]) for rec in sched.values()]
    protos += [(10, 3, -20), (7, 4, -13), (5, 2, 12.5), (0, 1.5, 7)]
    s0 = solve.init(shp)
    for proto in protos:
        stims = [Stimulus(Protocol(*proto), f)]
        got = [t for t in range(300)
               if abs(float(solve.step(s0, t, P3, D, stims, 0.01).u[4, 4]) - 5.0) < 1e-6]
        want = [t for t in range(300) if O.stimulus_active(t, *proto)]
        assert got == want, proto
