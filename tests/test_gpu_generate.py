"""GPU: checkpoint emission -- the bilinear resize kernel (io.imresize, cardiax/io.py:118-124)
against the oracle's restatement of jax.image.resize, and generate.sequence
(deepx/generate.py:135-210) against the oracle stepper followed by the oracle resize.

Tolerances: the resize is a float32 weighted sum of at most a few hundred terms, summed in a
different order than the oracle's einsum: |gpu - oracle| <= 2e-6 * max|a|.  The sequence
inherits the stepper's 1e-4 bound on u (the resize is a convex combination)."""
import numpy as np
import pytest
import torch

import fk_oracle as O

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("shape,size,aa", [
    ((3, 64, 96), (32, 48), True), ((3, 64, 96), (128, 200), True), ((3, 100, 70), (33, 41), True),
    ((2, 100, 70), (33, 41), False), ((1, 256, 256), (64, 64), True), ((3, 17, 23), (17, 23), True),
    ((3, 40, 40), (40, 13), True), ((4, 5, 3), (9, 2), True)])
def test_resize_matches_oracle(shape, size, aa):
    _gpu()
    from cardiax_gb300 import io
    rng = np.random.default_rng(sum(shape) + sum(size))
    a = rng.standard_normal(shape).astype(np.float32)
    got = io.imresize(torch.as_tensor(a).cuda(), size, antialias=aa).cpu().numpy()
    ref = O.imresize_bilinear(a, size, antialias=aa)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(a).max(), np.abs(got - ref).max()
    if tuple(size) == tuple(shape[-2:]):
        assert np.array_equal(got, a)


def test_resize_of_pitched_state_buffer():
    """The emission path reads the stepper's pitched state (row pitch > W) directly."""
    _gpu()
    from cardiax_gb300 import io
    from cardiax_gb300.tissue import Tissue
    H, W = 50, 37
    rng = np.random.default_rng(2)
    t = Tissue((H, W), P3, np.full((H, W), 1e-3, np.float32))
    planes = rng.standard_normal((3, H, W)).astype(np.float32)
    t.set_state(tuple(torch.as_tensor(x) for x in planes))
    assert t.pitch > W
    out = torch.empty((3, 20, 15), device=t.device)
    io.resize_planes(t.state, H, W, out)
    ref = O.imresize_bilinear(planes, (20, 15))
    assert np.abs(out.cpu().numpy() - ref).max() <= 2e-6 * np.abs(planes).max()


def test_sequence_matches_oracle(tmp_path):
    _gpu()
    from cardiax_gb300 import generate, io
    from cardiax_gb300.stimulus import Protocol, Stimulus
    H = W = 64
    D = np.full((H, W), 1e-3, np.float32)
    f = np.zeros((H, W), np.float32)
    f[:, :4] = 20.0
    stims = [Stimulus(Protocol(0, 2, 1e9), f)]
    states = generate.sequence(0, 301, 100, 0.01, 0.01, P3, D, stims,
                               filename=str(tmp_path / "seq"), reshape=(32, 40))
    assert tuple(states.shape) == (4, 3, 32, 40)
    st = O.init((H, W))
    ostim = [O.OStim(0, 2, 1e9, f)]
    for i, (a, b) in enumerate(((0, 100), (100, 200), (200, 300))):
        st = O.forward_euler(st, a, b, P3, D, ostim, 0.01, 0.01)
        ref = O.imresize_bilinear(np.stack(st), (32, 40))
        assert np.abs(states[i].cpu().numpy() - ref).max() <= 1e-4
    assert float(states[3].abs().max()) == 0.0  # the last row is never written
    from cardiax_gb300 import h5
    with h5.File(str(tmp_path / "seq")) as data:
        assert np.array_equal(data["states"][:], states.cpu().numpy())
        assert data["diffusivity"].shape == (32, 40) and data["field"].shape == (1, 32, 40)
        assert data["stimuli"].shape == (1, 32, 40)
        assert np.array_equal(data["params/D"][:], data["diffusivity"][:])
        ref_field = O.imresize_bilinear(f[None], (32, 40))[0]
        assert np.abs(data["field"][0] - ref_field).max() <= 2e-6 * 20.0
        assert float(data["params/tau_d"][()]) == 0.25 and float(data["params/dt"][()]) == 0.01
        assert list(data["period"][:]) == [1e9]
    params, D2 = io.load_params(str(tmp_path / "seq"))
    assert tuple(params) == P3 and D2.shape == (32, 40)


def test_sequence_streams_rows_to_the_file(tmp_path):
    """use_memory=False: each state is written as it is computed (deepx/generate.py:199-200)."""
    _gpu()
    from cardiax_gb300 import generate, h5
    from cardiax_gb300.stimulus import Protocol, Stimulus
    H, W = 48, 40
    D = np.full((H, W), 1e-3, np.float32)
    f = np.zeros((H, W), np.float32)
    f[:4, :] = 20.0
    stims = [Stimulus(Protocol(0, 2, 1e9), f)]
    path = str(tmp_path / "out" / "rows.hdf5")
    states = generate.sequence(0, 250, 50, 0.01, 0.01, P3, D, stims, filename=path,
                               use_memory=False)
    with h5.File(path) as data:
        assert np.array_equal(data["states"][:], states.cpu().numpy())
        assert np.array_equal(data["diffusivity"][:], D)


@pytest.mark.parametrize("shape,angle", [((64, 80), 30.0), ((50, 33), -47.5), ((128, 128), 90.0),
                                         ((37, 41), 12.25)])
def test_triangular_stimulus_matches_scipy(shape, angle):
    """stimulus.triangular on the device vs the reference's own SciPy rotation of the stripe."""
    _gpu()
    from scipy.ndimage import rotate
    from cardiax_gb300.stimulus import Direction, Protocol, linear, triangular
    for d in (Direction.WEST, Direction.NORTH):
        got = triangular(shape, d, angle, 0.2, 20.0, Protocol(0, 2, 1e9)).field.cpu().numpy()
        stripe = linear(shape, d, 0.2, 20.0, Protocol(0, 2, 1e9), device="cpu").field.numpy()
        ref = rotate(stripe, angle=angle, mode="nearest", prefilter=False, reshape=False)
        assert np.abs(got - ref).max() <= 1e-5, np.abs(got - ref).max()


def test_random_sequence_end_to_end(tmp_path):
    """deepx/generate.py:86-133 with NumPy draws: random stimuli (any of the three kinds), a scar
    diffusivity map and the emitted sequence, written to the HDF5 data set."""
    _gpu()
    from cardiax_gb300 import generate, h5, params
    path = str(tmp_path / "rand.hdf5")
    states = generate.random_sequence(5, params.PARAMSET_3, path, shape=(64, 64), n_stimuli=1,
                                      start=0, stop=2, step=0.5, reshape=(32, 32))
    assert tuple(states.shape) == (4, 3, 32, 32)
    assert torch.isfinite(states).all()
    with h5.File(path) as f:
        assert np.array_equal(f["states"][:], states.cpu().numpy())
        D = f["diffusivity"][:]
        assert D.shape == (32, 32) and 0.0001 - 1e-6 <= D.min() and D.max() <= 0.001 + 1e-6
        assert f["start"][0] == 1 and f["duration"][0] == 2
    for seed in range(3):
        s = generate.random_triangular_stimulus(seed, (80, 80), generate.random_protocol(seed))
        assert s.field.is_cuda and float(s.field.max()) <= 0.6 + 1e-6
