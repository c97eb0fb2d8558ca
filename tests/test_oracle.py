"""The CPU oracle against the reference's golden vectors (no GPU).

The fixtures were produced by running the reference's own solve.py (tests/golden/make_golden.py);
the oracle must reproduce them bit for bit in float32 (same evaluation order) and in float64.
"""
import json
import os

import numpy as np
import pytest

import fk_oracle as O
from conftest import GOLDEN

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)


def test_stimulus_schedule_known_answer():
    # tests/macro/stimulate_test.py:16-18 of the reference
    A = {0, 1, 50, 51, 100, 101, 150, 151, 200, 201, 250, 251}
    B = {10, 11, 60, 61, 110, 111, 160, 161, 210, 211, 260, 261}
    C = {30, 31}
    for proto, want in (((0, 2, 50), A), ((10, 2, 50), B), ((30, 2, 1000000), C)):
        got = {t for t in range(300) if O.stimulus_active(t, *proto)}
        assert got == want


def test_stimulus_schedule_golden():
    sched = json.load(open(os.path.join(GOLDEN, "stimulus_schedule.json")))
    for name, rec in sched.items():
        got = [t for t in range(300) if O.stimulus_active(t, *rec["protocol"])]
        assert got == rec["active"], name


def test_gradient_golden(golden):
    g = golden("gradient.npz")
    for k in range(4):
        a = g[f"in{k}"]
        np.testing.assert_array_equal(O.gradient(a, 0), g[f"ax0_{k}"])
        np.testing.assert_array_equal(O.gradient(a, 1), g[f"ax1_{k}"])


def test_step_golden(golden):
    s = golden("step.npz")
    for k in range(4):
        st = O.OState(s[f"v_{k}"], s[f"w_{k}"], s[f"u_{k}"])
        stims = [O.OStim(0, 2, 1e9, s[f"f1_{k}"]), O.OStim(1, 3, 7, s[f"f2_{k}"])]
        for t in (0, 1, 5):
            d = O.derivative(st, np.float32(t), P3, s[f"D_{k}"], stims, 0.01)
            for name, arr in zip(("dv", "dw", "du"), d):
                np.testing.assert_array_equal(arr, s[f"{name}_{k}_{t}"], err_msg=f"{name} {k} {t}")


@pytest.mark.parametrize("tag,dtype", [("f32", np.float32), ("f64", np.float64)])
def test_forward_small_golden(golden, tag, dtype):
    g = golden("forward_small.npz")
    shp = g["D"].shape
    stims = [O.OStim(0, 2, 1e9, g["f1"].astype(dtype)), O.OStim(60, 3, 1e9, g["f2"].astype(dtype))]
    res = O.forward_euler(O.init(shp, dtype), 0, 200, P3, g["D"].astype(dtype), stims, 0.01, 0.01)
    for name, arr in zip("vwu", res):
        np.testing.assert_array_equal(arr, g[f"{name}_{tag}"])


def test_config0_golden(golden):
    g = golden("config0.npz")
    for tag in ("plain", "excite"):
        field = g[f"{tag}_field"]
        proto = (0, 200, 1e9) if tag == "plain" else (0, 2, 1e9)
        np.testing.assert_array_equal(field, O.linear_field((128, 128), 3, 5 / 128,
                                                            1.0 if tag == "plain" else 20.0))
        st = O.init((128, 128))
        D = np.full((128, 128), 0.001, np.float32)
        states = O.forward(st, list(range(0, 1001, 100))[:4], P3, D, [O.OStim(*proto, field)],
                           0.01, 0.01)
        for i, s in enumerate(states):
            np.testing.assert_array_equal(s.u, g[f"{tag}_u_{(i + 1) * 100}"])


def test_c_oracle_matches_numpy_oracle():
    """The C restatement agrees with the NumPy one up to libm-vs-NumPy tanh rounding."""
    import fk_oracle_c as C
    C.build()
    g = np.load(os.path.join(GOLDEN, "forward_small.npz"))
    shp = g["D"].shape
    for dtype, tol in ((np.float32, 5e-5), (np.float64, 1e-12)):
        stims = [(0, 2, 1e9, g["f1"].astype(dtype)), (60, 3, 1e9, g["f2"].astype(dtype))]
        v, w, u = C.forward_euler(O.init(shp, dtype), 0, 200, P3, g["D"].astype(dtype), stims,
                                  0.01, 0.01, threads=2)
        ref = "f32" if dtype == np.float32 else "f64"
        assert np.abs(u - g[f"u_{ref}"]).max() <= tol
        assert np.abs(v - g[f"v_{ref}"]).max() <= tol
        assert np.abs(w - g[f"w_{ref}"]).max() <= tol


def test_params_golden():
    from cardiax_gb300 import params as Pm
    rec = json.load(open(os.path.join(GOLDEN, "params.json")))
    assert list(Pm.Params._fields) == rec["fields"]
    for name, vals in rec["sets"].items():
        assert [float(x) for x in getattr(Pm, name)] == vals, name


@pytest.mark.parametrize("tag,dtype", [("f32", np.float32), ("f64", np.float64)])
def test_heun_golden(golden, tag, dtype):
    """The oracle's Heun integrator against the reference's own _forward_heun."""
    g = golden("forward_small.npz")
    h = golden("heun_small.npz")
    stims = [O.OStim(0, 2, 1e9, g["f1"].astype(dtype)), O.OStim(60, 3, 1e9, g["f2"].astype(dtype))]
    res = O.forward_heun(O.init(g["D"].shape, dtype), 0, 200, P3, g["D"].astype(dtype), stims,
                         0.01, 0.01)
    for name, arr in zip("vwu", res):
        np.testing.assert_array_equal(arr, h[f"{name}_{tag}"])


# --- bilinear resize (restatement of jax.image.resize "bilinear"; known answers) --------------
def test_resize_identity_and_constant():
    rng = np.random.default_rng(3)
    a = rng.standard_normal((3, 17, 23)).astype(np.float32)
    assert np.array_equal(O.imresize_bilinear(a, (17, 23)), a)
    c = np.full((2, 40, 30), 0.7, np.float32)
    for size in ((20, 15), (13, 7), (80, 61), (40, 11)):
        np.testing.assert_allclose(O.imresize_bilinear(c, size), 0.7, rtol=1e-6)


def test_resize_triangle_kernel_known_weights():
    # 2x downsampling with antialiasing: the kernel widens to radius 2, interior weights
    # (1, 3, 3, 1) / 8 on inputs 2p-1 .. 2p+2; the first output renormalises (3, 3, 1) / 7
    w = O.resize_weights(16, 8, antialias=True)
    np.testing.assert_allclose(w[3:7, 2], np.array([1, 3, 3, 1]) / 8, rtol=1e-6)
    np.testing.assert_allclose(w[0:3, 0], np.array([3, 3, 1]) / 7, rtol=1e-6)
    # without antialiasing 2x downsampling averages the two nearest inputs
    w = O.resize_weights(16, 8, antialias=False)
    np.testing.assert_allclose(w[4:6, 2], [0.5, 0.5], rtol=1e-6)
    # 2x upsampling: output p samples p/2 - 1/4 -> (3/4, 1/4) blends, first output = input 0
    w = O.resize_weights(8, 16)
    np.testing.assert_allclose(w[0:2, 1], [0.75, 0.25], rtol=1e-6)
    np.testing.assert_allclose(w[:, 0], np.eye(8)[0], rtol=1e-6)


@pytest.mark.parametrize("src,dst", [((64, 64), (32, 32)), ((1200, 1200), (256, 256)),
                                     ((100, 70), (37, 91)), ((17, 23), (40, 11)),
                                     ((50, 50), (200, 200)), ((3, 5), (11, 2))])
def test_resize_matches_an_independent_implementation(src, dst):
    """jax.image.resize "bilinear" (cardiax/io.py:118-124) is the published triangle-kernel
    algorithm: half-pixel centres, the kernel widened by 1/scale when downsampling, weights
    normalised per output.  PyTorch's bilinear interpolation with antialias=True implements the
    same algorithm independently: the restatement, evaluated in float64, equals it to rounding;
    in float32 (as JAX computes the sample positions) it differs only by the float32 positions,
    within 2e-5 of unit-scale data."""
    import torch
    rng = np.random.default_rng(sum(src) + sum(dst))
    a = rng.standard_normal((2,) + src)
    ref = torch.nn.functional.interpolate(torch.from_numpy(a)[None], size=dst, mode="bilinear",
                                          antialias=True, align_corners=False)[0].numpy()
    assert np.abs(O.imresize_bilinear(a, dst, dtype=np.float64) - ref).max() <= 1e-12
    assert np.abs(O.imresize_bilinear(a.astype(np.float32), dst) - ref).max() <= 2e-5


def test_resize_linear_ramp_upsampling_is_exact_inside():
    a = np.tile(np.arange(10, dtype=np.float32), (4, 1))
    b = O.imresize_bilinear(a, (4, 20))
    p = np.arange(1, 19)
    np.testing.assert_allclose(b[0, p], p / 2 - 0.25, atol=1e-6)


@pytest.mark.parametrize("shape,angle", [((20, 24), 30.0), ((17, 13), 47.5), ((16, 16), 90.0),
                                         ((21, 30), -12.3), ((40, 40), 180.0), ((33, 64), 721.0)])
def test_rotate_field_matches_scipy(shape, angle):
    """The restatement of stimulus.triangular's rotation against SciPy itself."""
    from scipy.ndimage import rotate
    rng = np.random.default_rng(sum(shape) + abs(int(angle)))
    stripe = np.zeros(shape, np.float32)
    stripe[:, : max(1, shape[1] // 5)] = 20.0
    for a in (stripe, rng.uniform(0, 1, shape).astype(np.float32)):
        ref = rotate(a, angle=angle, mode="nearest", prefilter=False, reshape=False)
        np.testing.assert_allclose(O.rotate_field(a, angle), ref, rtol=1e-6, atol=1e-6)


PARAMSET_CASES = ("1A", "4A", "5", "2")


@pytest.mark.parametrize("name", PARAMSET_CASES)
@pytest.mark.parametrize("tag,dtype", [("f32", np.float32), ("f64", np.float64)])
def test_paramsets_golden(golden, name, tag, dtype):
    """The oracle under parameter sets 1A, 4A, 5 and 2 (MAXFLOAT entries) against the
    reference's own forward (tests/golden/make_golden.py), bit for bit."""
    from cardiax_gb300 import params as Pm
    g = golden("paramsets.npz")
    P = getattr(Pm, f"PARAMSET_{name}")
    ck = [int(c) for c in g["checkpoints"]]
    stims = [O.OStim(0, 2, 1e9, g["f1"].astype(dtype)), O.OStim(300, 2, 1e9, g["f2"].astype(dtype))]
    states = O.forward(O.init(g["D"].shape, dtype), ck, P, g["D"].astype(dtype), stims, 0.01,
                       0.01)
    for c, s in zip(ck[1:], states):
        if f"{name}_{tag}_u_{c}" in g:
            np.testing.assert_array_equal(s.u, g[f"{name}_{tag}_u_{c}"], err_msg=f"u at {c}")
    np.testing.assert_array_equal(states[-1].v, g[f"{name}_{tag}_v_{ck[-1]}"])
    np.testing.assert_array_equal(states[-1].w, g[f"{name}_{tag}_w_{ck[-1]}"])


def test_autodiff_oracle_forward_equals_reference_x64(golden):
    """The float64 torch restatement that stands in for jax.grad of the reference runs the
    reference's own x64 forward (forward_small.npz, 200 steps on 32x40) to within 1e-12."""
    import torch
    import fk_torch as T
    g = golden("forward_small.npz")
    shp = g["D"].shape
    f64 = lambda a: torch.as_tensor(np.asarray(a, np.float64))  # noqa: E731
    st = (torch.ones(shp, dtype=torch.float64), torch.ones(shp, dtype=torch.float64),
          torch.zeros(shp, dtype=torch.float64))
    theta = f64(P3[:13])
    stims = [(0, 2, 1e9, f64(g["f1"])), (60, 3, 1e9, f64(g["f2"]))]
    with torch.no_grad():
        v, w, u = T.forward(st, 0, 200, theta, P3[13], f64(g["D"]), stims, 0.01, 0.01)
    for name, arr in zip("vwu", (v, w, u)):
        err = float(np.abs(arr.numpy() - g[f"{name}_f64"]).max())
        assert err <= 1e-12, f"{name}: {err}"


def test_config0_x64_golden(golden):
    """The configuration-0 runs in float64 (the reference with x64) at 1000 steps, bit for bit."""
    g = golden("config0_x64.npz")
    for tag, amp, proto in (("plain", 1.0, (0, 200, 1e9)), ("excite", 20.0, (0, 2, 1e9))):
        field = O.linear_field((128, 128), 3, 5 / 128, amp, dtype=np.float64)
        D = np.full((128, 128), 0.001, np.float64)
        s = O.forward_euler(O.init((128, 128), np.float64), 0, 1000, P3, D,
                            [O.OStim(*proto, field)], 0.01, 0.01)
        np.testing.assert_array_equal(s.u, g[f"{tag}_u_1000"], err_msg=tag)
