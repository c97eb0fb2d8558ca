"""GPU: the tissue autotuner (autotune.tune_tissue, Tissue.advance(schedule="auto")) picks one
of its candidates, leaves the tissue's state as it found it, and -- since every candidate
produces the same bits -- steps exactly as the default schedule does."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _tissue(H, W, seed):
    """D with 5 % noise smoothed over 2 cells (per-cell noise makes the explicit scheme
    diverge), and a 10-column strip at 50 for the two steps the protocol is active: u crosses
    0.5 at the first step and a wave starts."""
    import bench
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    f = np.zeros((H, W), np.float32)
    f[:, :10] = 50.0
    return Tissue((H, W), P3, bench.noisy_diffusivity(H, W, seed),
                  [Stimulus(Protocol(0, 2, 1e9), f)])


@pytest.mark.parametrize("H,W", [(96, 130), (256, 256), (37, 300)])
def test_auto_schedule_is_bit_identical(H, W):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cardiax_gb300 import autotune
    a, b = _tissue(H, W, H + W), _tissue(H, W, H + W)
    before = a.state.clone()
    res = autotune.tune_tissue(a, trial_steps=16)
    assert torch.equal(a.state, before)  # restored
    assert res["choice"] in autotune.TISSUE_CANDIDATES
    assert res["choice"] in res["us_per_step"]
    a.advance(0, 120, schedule="auto")
    b.advance(0, 120)
    torch.cuda.synchronize()
    assert torch.equal(a.state[:, :, :W], b.state[:, :, :W])


def test_tracking_restricts_the_candidates():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cardiax_gb300 import autotune
    t = _tissue(64, 64, 3).track_activation(0.5)
    res = autotune.tune_tissue(t, trial_steps=8)
    assert all(c[1] == 1 for c in res["us_per_step"])
    t.advance(0, 50, schedule="auto")
    torch.cuda.synchronize()
    assert int((t.act_first[:, :64] >= 0).sum()) > 0


@pytest.mark.parametrize("H,W", [(37, 90), (128, 128), (200, 64)])
def test_one_tissue_batch_schedule_is_bit_identical(H, W):
    """schedule="batch" (the batched kernel on the one tissue, 16- or 32-row items, graph
    replay plus a remainder) steps exactly as the default, activation maps included."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    a, b = _tissue(H, W, 1), _tissue(H, W, 1)
    for rows in (16, 32):
        a.init()
        b.init()
        a.advance(0, 77, schedule="batch", tile_rows=rows).advance(77, 150, schedule="batch",
                                                                    tile_rows=rows)
        b.advance(0, 150)
        torch.cuda.synchronize()
        assert torch.equal(a.state[:, :, :W], b.state[:, :, :W]), rows
    c, d = _tissue(H, W, 2).track_activation(0.5), _tissue(H, W, 2).track_activation(0.5)
    c.advance(0, 150, schedule="batch")
    d.advance(0, 150)
    torch.cuda.synchronize()
    assert torch.equal(c.state[:, :, :W], d.state[:, :, :W])
    for x, y in zip(c.activation_maps(), d.activation_maps()):
        assert torch.equal(x, y)
    assert int((c.act_first[:, :W] >= 0).sum()) > 0
