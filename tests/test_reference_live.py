"""Oracle vs the reference's own code on fresh random cases, when the reference checkout is
present (it runs under the NumPy stand-in for JAX; no GPU)."""
import os

import numpy as np
import pytest

import fk_oracle as O

# the reference checkout, from CARDIAX_REFERENCE; the tests skip when it is unset or absent
REF = os.environ.get("CARDIAX_REFERENCE")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "cardiax")),
                                reason="reference checkout not given (CARDIAX_REFERENCE)")


@pytest.mark.parametrize("x64", [False, True])
def test_oracle_equals_reference_step(x64):
    from ref_shim import load_reference
    R = load_reference(x64=x64, root=REF)
    dt_ = np.float64 if x64 else np.float32
    rng = np.random.default_rng(7)
    for shape in [(3, 4), (6, 11), (25, 19)]:
        st = tuple(rng.uniform(0, 1, shape).astype(dt_) for _ in range(3))
        D = rng.uniform(1e-4, 1e-3, shape).astype(dt_)
        f = np.zeros(shape, dt_)
        f[1:, :2] = 3.0
        for P in (R.params.PARAMSET_3, R.params.PARAMSET_1A, R.params.PARAMSET_4A):
            for t in (0, 1, 4):
                a = R.solve.step(R.solve.State(*st), dt_(t), P, D,
                                 [R.stimulus.Stimulus(R.stimulus.Protocol(0, 3, 4), f)], 0.01)
                b = O.derivative(O.OState(*st), dt_(t), P, D, [O.OStim(0, 3, 4, f)], 0.01)
                for x, y in zip(a, b):
                    np.testing.assert_array_equal(x, y)


def test_oracle_stimulus_generators_equal_reference():
    from ref_shim import load_reference
    R = load_reference(root=REF)
    for d in range(4):
        for shape in [(20, 30), (17, 17)]:
            ref = R.stimulus.linear(shape, R.stimulus.Direction(d), 0.2, 3.0,
                                    R.stimulus.Protocol(0, 2, 5)).field
            np.testing.assert_array_equal(O.linear_field(shape, d, 0.2, 3.0), ref)
    ref = R.stimulus.rectangular((30, 40), (12, 20), (5, 8), 2.5, R.stimulus.Protocol(0, 2, 5)).field
    np.testing.assert_array_equal(O.rectangular_field((30, 40), (12, 20), (5, 8), 2.5), ref)


def test_convert_equals_reference():
    """cardiax_gb300.convert against the reference's own cardiax/convert.py (pure host
    arithmetic) on a sweep of values."""
    from ref_shim import load_reference
    from cardiax_gb300 import convert as G
    R = load_reference(root=REF).convert
    for dt in (0.01, 0.02, 0.005):
        for ms in (0.0, 1.0, 12.5, 400.0, 1e4, 0.03):
            assert G.ms_to_units(ms, dt) == R.ms_to_units(ms, dt)
            assert G.units_to_ms(G.ms_to_units(ms, dt), dt) == R.units_to_ms(R.ms_to_units(ms, dt), dt)
    for dx in (0.01, 0.015, 0.025):
        for cm in (0.0, 1.0, 6.0, 12.0, 0.33):
            assert G.cm_to_units(cm, dx) == R.cm_to_units(cm, dx)
            assert G.units_to_cm(cm, dx) == R.units_to_cm(cm, dx)
        assert G.realsize_to_shape((12, 7.5), dx) == R.realsize_to_shape((12, 7.5), dx)
        assert G.shape_to_realsize((1200, 800), dx) == R.shape_to_realsize((1200, 800), dx)
    for V in (-85.0, -40.0, 0.0, 15.0):
        assert G.V_to_u(V) == R.V_to_u(V)
        assert G.u_to_V(G.V_to_u(V)) == R.u_to_V(R.V_to_u(V))
    c = np.linspace(0.2, 0.9, 17)
    np.testing.assert_array_equal(G.diffusivity_rescale(c, (1e-4, 1e-3)),
                                  R.diffusivity_rescale(c, (1e-4, 1e-3)))
    p = dict(zip(("tau_v_plus", "tau_v1_minus", "tau_v2_minus", "tau_w_plus", "tau_w_minus",
                  "tau_d", "tau_0", "tau_r", "tau_si", "k", "V_csi", "V_c", "V_v", "Cm"),
                 (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1.0)))
    assert G.params_to_units(p, 0.01, 0.02) == R.params_to_units(dict(p), 0.01, 0.02)
    st = [{"start": 10.0, "duration": 2.0, "period": 400.0}]
    assert G.stimuli_to_units([dict(s) for s in st], 0.01, 0.02) == \
        R.stimuli_to_units([dict(s) for s in st], 0.01, 0.02)
