"""GPU: a sweep of small grid shapes against the C oracle.

Every H x W with H, W drawn from the sizes around the tile edges (3..9, 12, 31..33, 36, 63..65,
67, 68, 127..130; 441 shapes): grids smaller than one tile, one tile plus one row or column (the
sliver path), widths not divisible by 4 (pitch padding), and multiples of the 32 x 64 tile.  Each
runs 4 Euler steps from a random sub-threshold state with a stimulated corner (so the reaction's
upper branch is exercised) and per-cell random D.  Bound: 2e-6 on every plane (the kernels'
reciprocal multiplies and hardware exp/reciprocal against the oracle's libm, over 4 steps;
measured worst 2.4e-7)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
SIZES = [3, 4, 5, 6, 7, 8, 9, 12, 31, 32, 33, 36, 63, 64, 65, 67, 68, 127, 128, 129, 130]


def test_shape_sweep_against_the_oracle():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fk_oracle_c as C
    from cardiax_gb300 import solve
    from cardiax_gb300.stimulus import Protocol, Stimulus
    C.build()
    rng = np.random.default_rng(441)
    worst = 0.0
    for H in SIZES:
        for W in SIZES:
            st = (rng.uniform(0.8, 1.0, (H, W)).astype(np.float32),
                  rng.uniform(0.8, 1.0, (H, W)).astype(np.float32),
                  rng.uniform(0.0, 0.05, (H, W)).astype(np.float32))
            D = rng.uniform(5e-4, 1e-3, (H, W)).astype(np.float32)
            f = np.zeros((H, W), np.float32)
            f[:max(1, H // 3), :max(1, W // 3)] = 20.0
            ref = C.forward_euler(st, 0, 4, P3, D, [(0, 2, 1e9, f)], 0.01, 0.01)
            got = solve._forward_euler(solve.State(*map(torch.as_tensor, st)), 0, 4, P3, D,
                                       [Stimulus(Protocol(0, 2, 1e9), f)], 0.01, 0.01)
            for a, b in zip(got, ref):
                d = float(np.abs(a.cpu().numpy() - b).max())
                worst = max(worst, d)
                assert d <= 2e-6, (H, W, d)
    print(f"shape sweep: worst |gpu - oracle| = {worst:.3g}")
