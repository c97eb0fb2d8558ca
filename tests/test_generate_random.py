"""Randomised experiments of deepx/generate.py:16-133 (host side, CPU): the distributions the
reference draws from, with a NumPy Generator in place of JAX's PRNG."""
import numpy as np
import pytest

from cardiax_gb300 import generate as G
from cardiax_gb300.stimulus import Direction, Protocol


def test_protocol_ranges():
    g = np.random.default_rng(0)
    for _ in range(200):
        p = G.random_protocol(g, min_start=5, max_start=9, min_period=400, max_period=1000)
        assert 5 <= p.start < 9 and p.duration == 2 and 400 <= p.period < 1000
    assert G.random_protocol(1) == G.random_protocol(1)


def test_rectangular_ranges():
    g = np.random.default_rng(1)
    H = 300
    for _ in range(20):
        s = G.random_rectangular_stimulus(g, (H, H), Protocol(0, 2, 1e9), device="cpu")
        f = s.field.numpy()
        assert set(np.unique(f)) <= {0.0, np.float32(0.6)}
        rows, cols = np.nonzero(f)
        if len(rows):  # a rectangle of side < H // 3 (clipped at the far edges)
            assert rows.max() - rows.min() + 1 < H // 3 + 1
            assert cols.max() - cols.min() + 1 < H // 3 + 1


def test_linear_never_west_and_covers_a_stripe():
    g = np.random.default_rng(2)
    H = W = 200
    seen = set()
    for _ in range(60):
        s = G.random_linear_stimulus(g, (H, W), Protocol(0, 2, 1e9), device="cpu")
        f = s.field.numpy() != 0
        if f.all() or not f.any():
            continue
        if f[0].all():
            seen.add(Direction.NORTH)
        elif f[:, -1].all():
            seen.add(Direction.EAST)
        elif f[-1].all():
            seen.add(Direction.SOUTH)
        else:
            seen.add(Direction.WEST)
    assert Direction.WEST not in seen and seen


def test_random_stimulus_amplitude_and_protocol():
    g = np.random.default_rng(3)
    kinds = 0
    for _ in range(10):
        try:
            s = G.random_stimulus(g, (64, 64), min_start=7, max_start=8, device="cpu")
        except RuntimeError:  # the triangular kind needs a CUDA device
            kinds += 1
            continue
        assert s.protocol.start == 7 and s.protocol.duration == 2
        assert float(s.field.max()) in (0.0, 20.0)
    assert kinds < 10


def test_random_sequence_needs_start_slots():
    from cardiax_gb300 import params
    with pytest.raises(ValueError):
        G.random_sequence(0, params.PARAMSET_3, shape=(32, 32), n_stimuli=3, stop=2)
