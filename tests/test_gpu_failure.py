"""GPU: the failure path of the bounded barrier waits.  A wait on a barrier that nothing
completes runs out after its limit, the kernel sets the device error word and returns, and the
context stays usable (no fault, trap or hang is involved)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _status(reset=1):
    from cardiax_gb300 import _native as N
    v = ctypes.c_int(-1)
    N.call("fk_device_status", reset, ctypes.byref(v))
    return v.value


def test_wait_that_runs_out_sets_the_status_and_the_context_survives():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cardiax_gb300 import _native as N
    from cardiax_gb300 import params, solve
    from cardiax_gb300.tissue import stream_handle
    torch.cuda.set_device(0)
    _status()  # clear
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    N.call("fk_selftest_wait_timeout", 20_000_000, stream_handle())
    e1.record()
    torch.cuda.synchronize()
    assert e0.elapsed_time(e1) >= 19.0  # the wait ran to its 20 ms limit
    assert _status() == 1               # timeout reported
    assert _status() == 0               # and cleared
    # the context is still usable: a forward run works and reports no timeout
    shape = (48, 40)
    D = np.full(shape, 1e-3, np.float32)
    out = solve.forward(solve.init(shape), [0, 50], params.PARAMSET_3, D, [], 0.01, 0.01)
    torch.cuda.synchronize()
    assert np.isfinite(out[-1].u.cpu().numpy()).all()
    assert _status() == 0
