"""GPU: a grid whose state buffer holds more than 2^31 floats.

27000 x 27000 cells: each plane is 729 M cells, the (v, w, u) state 2.19 G floats, so the last
rows of u sit beyond 2^31 elements from the state's base.  Partial tiles on the right (27000 =
421 x 64 + 56) and bottom (27000 = 843 x 32 + 24) edges.  Three Euler steps from a smooth
sub-threshold u with a stimulated left stripe; three row bands (the top edge, the middle, the
bottom edge) are checked against the C oracle run on the same bands.  Rows within 12 of a band's
cut are excluded (each step reaches 4 rows), so the comparison covers the true edges and
interior rows at the largest offsets.  Bound: 1e-6 on the sub-threshold cells and 1e-4 in the
stimulated stripe (the reaction's tanh differs in the last bits between the GPU and libm)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
H = W = 27000
STEPS = 3
BAND = 48
CUT = 4 * STEPS


def test_state_larger_than_2_31_floats():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    free, _ = torch.cuda.mem_get_info()
    if free < 48 * 2**30:
        pytest.skip("needs about 40 GB of free device memory")
    import fk_oracle_c as C
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    C.build()
    dev = torch.device("cuda", 0)
    ii = torch.arange(H, device=dev, dtype=torch.float32)[:, None]
    jj = torch.arange(W, device=dev, dtype=torch.float32)[None, :]
    D = (1.0 + 0.05 * torch.sin(0.37 * ii) * torch.cos(0.23 * jj)) * 1e-3
    field = torch.zeros((H, W), device=dev)
    field[:, :5] = 20.0
    tis = Tissue((H, W), P3, D, [Stimulus(Protocol(0, 2, 1e9), field)], dt=0.01, dx=0.01,
                 device=dev)
    del field
    assert 3 * tis.H * tis.pitch > 2**31
    tis.state[2, :, :W] = 0.02 * (1.0 + torch.sin(0.011 * ii + 0.017 * jj))
    bands = [(0, BAND), (H // 2 - BAND // 2, H // 2 + BAND // 2), (H - BAND, H)]
    before = [(tis.state[:, r0:r1, :W].cpu().numpy(), D[r0:r1].cpu().numpy()) for r0, r1 in bands]
    tis.advance(0, STEPS)
    torch.cuda.synchronize()
    after = [tis.state[:, r0:r1, :W].cpu().numpy() for r0, r1 in bands]
    del tis, D
    torch.cuda.empty_cache()
    for (r0, r1), (st, Db), got in zip(bands, before, after):
        f = np.zeros((r1 - r0, W), np.float32)
        f[:, :5] = 20.0
        ref = C.forward_euler(tuple(st), 0, STEPS, P3, Db, [(0, 2, 1e9, f)], 0.01, 0.01,
                              threads=C.max_threads())
        lo = 0 if r0 == 0 else CUT
        hi = (r1 - r0) if r1 == H else (r1 - r0) - CUT
        for a, b in zip(got, ref):
            d = np.abs(a[lo:hi] - b[lo:hi])
            assert d[:, 16:].max() <= 1e-6, (r0, float(d[:, 16:].max()))
            assert d.max() <= 1e-4, (r0, float(d.max()))
