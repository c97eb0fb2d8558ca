"""The batched path (one persistent kernel per step over all tissues, CUDA-graph replay) against
the single-tissue path: every tissue must come out bit-identical."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _same(p, q):
    """Bitwise equality, NaN equal to NaN (tiny grids such as 3x5 can blow up, identically)."""
    torch.testing.assert_close(p, q, rtol=0, atol=0, equal_nan=True)


def _mixed_tissues(rng, track=False):
    """Seven tissues of different shapes (3 x 5 .. 256 x 130), parameter sets, D maps,
    stimuli, time steps and cell sizes."""
    from cardiax_gb300 import params as Pm
    from cardiax_gb300.stimulus import Protocol, Stimulus
    from cardiax_gb300.tissue import Tissue
    shapes = [(64, 64), (128, 128), (37, 90), (256, 130), (3, 5), (200, 64), (96, 257)]
    sets = [Pm.PARAMSET_1A, Pm.PARAMSET_3, Pm.PARAMSET_4A, Pm.PARAMSET_5]
    out = []
    for k, (H, W) in enumerate(shapes):
        i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
        D = (1e-3 * (1 - 0.7 * np.exp(-((i - H * rng.uniform()) ** 2 + (j - W * rng.uniform()) ** 2)
                                      / (0.05 * H * W + 1)))).astype(np.float32)
        f = np.zeros((H, W), np.float32)
        if k % 2:
            f[:, : max(1, W // 10)] = 20.0
        else:
            r, c = rng.integers(0, max(1, H - 10)), rng.integers(0, max(1, W - 10))
            f[r:r + 10, c:c + 10] = 20.0
        proto = Protocol(int(rng.integers(0, 20)), 2, int(rng.integers(150, 400)))
        # per-tissue time and space steps (the batch holds each tissue's own dt and 1/dx)
        dt, dx = (0.01, 0.005, 0.02)[k % 3], (0.01, 0.0125)[k % 2]
        t = Tissue((H, W), sets[k % 4], D, [Stimulus(proto, f)], dt=dt, dx=dx)
        if track:
            t.track_activation(0.5)
        out.append(t)
    return out


@pytest.mark.parametrize("graph_steps,n_steps,rows,interleave,packed", [
    (0, 37, 32, True, False), (16, 101, 32, True, False), (64, 64, 32, True, False),
    (0, 37, 16, True, False), (16, 101, 16, True, False), (0, 37, 32, False, False),
    (16, 101, 32, False, True), (0, 37, 16, False, True), (16, 64, 16, True, True),
    (0, 37, 32, 2, False), (16, 101, 16, 4, False), (0, 37, 32, 4, True)])
def test_batch_matches_single_tissue_bitwise(graph_steps, n_steps, rows, interleave, packed):
    """Every tile geometry (32 x 64, 16 x 64 work items), work order and arithmetic of the
    batched kernel."""
    _gpu()
    from cardiax_gb300.batch import TissueBatch
    a = _mixed_tissues(np.random.default_rng(1))
    b = _mixed_tissues(np.random.default_rng(1))
    for t in a:
        t.advance(0, n_steps)
    batch = TissueBatch(b, graph_steps=graph_steps, tile_rows=rows)
    batch.set_options(interleave, packed)
    batch.advance(0, n_steps)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for p, q in zip(x.view(), y.view()):
            _same(p, q)
    batch.close()


def test_batch_continues_across_calls_and_tracks_activation():
    _gpu()
    from cardiax_gb300.batch import TissueBatch
    a = _mixed_tissues(np.random.default_rng(2), track=True)
    b = _mixed_tissues(np.random.default_rng(2), track=True)
    for t in a:
        t.advance(0, 500)
    batch = TissueBatch(b, graph_steps=32)
    batch.advance(0, 123).advance(123, 500)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for p, q in zip(x.view(), y.view()):
            _same(p, q)
        for p, q in zip(x.activation_maps(), y.activation_maps()):
            assert torch.equal(p, q)
    assert any(int((t.activation_maps()[0] >= 0).sum()) > 0 for t in b)


def test_autotuner_restores_state_and_picks_a_candidate():
    _gpu()
    from cardiax_gb300.autotune import tune_batch
    from cardiax_gb300.batch import TissueBatch
    b = _mixed_tissues(np.random.default_rng(3))
    before = [t.state.clone() for t in b]
    batch = TissueBatch(b)
    res = tune_batch(batch, trial_steps=32, candidates=(0, 16))
    assert res["graph_steps"] in (0, 16) and res["tile_rows"] in (32, 16)
    # one tissue (96 x 257) cannot be blocked: depth 1 only
    assert not batch.can_block() and res["depth"] == 1
    assert len(res["ms_per_step"]) == 24 and batch.tile_rows == res["tile_rows"]
    assert (batch.interleave, batch.packed) == (res["interleave"], res["packed"])
    for t, s in zip(b, before):
        assert torch.equal(t.state, s)


def test_tile_geometry_switches_mid_run_and_ctas_change():
    """Changing the tile geometry and the CTA count between calls keeps the results bitwise."""
    _gpu()
    from cardiax_gb300.batch import TissueBatch
    a = _mixed_tissues(np.random.default_rng(4))
    b = _mixed_tissues(np.random.default_rng(4))
    for t in a:
        t.advance(0, 90)
    batch = TissueBatch(b, graph_steps=16)
    batch.advance(0, 33)
    batch.set_tile_rows(16).set_options(2, False).advance(33, 45)
    batch.set_ctas(151).advance(45, 50)  # a chunked order is rebuilt for the new CTA count
    batch.set_options(False, True).advance(50, 61)
    batch.set_ctas(97).set_tile_rows(32).set_options(True, True).advance(61, 90)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for p, q in zip(x.view(), y.view()):
            _same(p, q)
    batch.close()


def _blockable_tissues(rng):
    """Mixed shapes, sets and stimuli whose last tile rows and columns hold more than one cell
    (H % 32 != 1, W % 64 != 1): tiles on every edge, partial tiles, a 3 x 5 grid."""
    ts = _mixed_tissues(rng)
    return [t for t in ts if t.H % 32 != 1 and t.W % 64 != 1]


@pytest.mark.parametrize("graph_steps,n_steps", [(0, 37), (0, 64), (16, 101), (64, 64)])
def test_batch_depth_two_matches_single_tissue_bitwise(graph_steps, n_steps):
    """Two Euler steps per launch (the blocked kernel over the batch's work items; an odd last
    step alone; graph replays of a multiple of 4 steps) give every tissue the bits of one step
    per launch."""
    _gpu()
    from cardiax_gb300.batch import TissueBatch
    a = _blockable_tissues(np.random.default_rng(5))
    b = _blockable_tissues(np.random.default_rng(5))
    assert len(b) >= 5
    for t in a:
        t.advance(0, n_steps)
    batch = TissueBatch(b, graph_steps=graph_steps)
    assert batch.can_block()
    batch.set_depth(2).advance(0, n_steps)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for p, q in zip(x.view(), y.view()):
            _same(p, q)
    batch.close()


def test_batch_depth_two_continues_and_autotunes():
    """Calls that alternate depth 1 and 2 and odd step counts, then the autotuner over both
    depths (the state restored)."""
    _gpu()
    from cardiax_gb300 import _native as N
    from cardiax_gb300.autotune import tune_batch
    from cardiax_gb300.batch import TissueBatch
    a = _blockable_tissues(np.random.default_rng(6))
    b = _blockable_tissues(np.random.default_rng(6))
    for t in a:
        t.advance(0, 99)
    batch = TissueBatch(b, graph_steps=8)
    batch.set_depth(2).advance(0, 13).set_depth(1).advance(13, 40).set_depth(2).advance(40, 99)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        for p, q in zip(x.view(), y.view()):
            _same(p, q)
    before = [t.state.clone() for t in b]
    res = tune_batch(batch, trial_steps=16, candidates=(0, 8), tile_rows=(32,),
                     options=((True, False),))
    assert res["depth"] in (1, 2) and len(res["ms_per_step"]) == 4
    for t, s in zip(b, before):
        assert torch.equal(t.state, s)
    # a batch with a tissue that cannot be blocked refuses depth 2
    c = TissueBatch(_mixed_tissues(np.random.default_rng(7)))
    with pytest.raises(N.FkError):
        c.set_depth(2)
    batch.close()
    c.close()
