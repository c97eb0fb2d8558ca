"""Heun integrator (cardiax/solve.py:73-85,103-111) on the GPU vs the reference's golden run
and the oracle.  Tolerance: the 1e-4 bar on u (same arithmetic differences as Euler)."""
import numpy as np
import pytest
import torch

import fk_oracle as O

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_heun_small_golden(golden):
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    g = golden("forward_small.npz")
    h = golden("heun_small.npz")
    stims = [Stimulus(Protocol(0, 2, 1e9), g["f1"]), Stimulus(Protocol(60, 3, 1e9), g["f2"])]
    res = solve._forward_heun(solve.init(g["D"].shape), 0, 200, P3, g["D"], stims, 0.01, 0.01)
    for name, arr in zip("vwu", res):
        a = arr.cpu().numpy()
        e32, e64 = np.abs(a - h[f"{name}_f32"]).max(), np.abs(a - h[f"{name}_f64"]).max()
        print(f"heun {name}: |gpu-ref32| {e32:.3g} |gpu-ref64| {e64:.3g}")
        assert e32 <= 1e-4


def test_heun_forward_matches_oracle_and_step():
    """128x128 excitable configuration, 300 Heun steps through forward(integrator=HEUN) vs
    the oracle; step_heun repeated gives the same bits as _forward_heun."""
    _gpu()
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Direction, Protocol, linear
    shp = (128, 128)
    D = np.full(shp, 1e-3, np.float32)
    stim = linear(shp, Direction.WEST, 5 / 128, 20.0, Protocol(0, 2, 1e9))
    states = solve.forward(solve.init(shp), [0, 100, 300], P3, D, [stim], 0.01, 0.01,
                           integrator=solve.TimeIntegrator.HEUN)
    ref = O.forward_heun(O.init(shp), 0, 300, P3, D, [O.OStim(0, 2, 1e9, stim.field.cpu().numpy())],
                         0.01, 0.01)
    assert np.abs(states[-1].u.cpu().numpy() - ref.u).max() <= 1e-4
    s = solve.init(shp)
    for t in range(20):
        s = solve.step_heun(s, t, P3, D, [stim], 0.01, 0.01)
    f = solve._forward_heun(solve.init(shp), 0, 20, P3, D, [stim], 0.01, 0.01)
    for a, b in zip(s, f):
        assert torch.equal(a, b)
