"""Oracle vs the reference's own code on fresh random cases, when the reference checkout is
present (it runs under the NumPy stand-in for JAX; no GPU)."""
import os

import numpy as np
import pytest

import fk_oracle as O

REF = os.environ.get("CARDIAX_REFERENCE", "/root/reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "cardiax")),
                                reason="reference checkout not present")


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
