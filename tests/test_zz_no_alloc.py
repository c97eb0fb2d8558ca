"""fk_forward_euler_noalloc, the entry point for callers that cannot allocate device memory.

Some callers of this library cannot call cudaMalloc while they step a tissue -- an XLA custom
call, for example, gets every buffer from XLA's allocator and must not allocate inside the call.
fk_forward_euler_noalloc takes no scratch argument: its ping-pong state lives in a fixed-size
device array of the library.  Its results must match fk_forward_euler (which takes the scratch
from the caller) on consecutive calls, and grids beyond the array's capacity must be refused.

This file is collected last so that a failure here never hides the other tests; it also passes
when run on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

P3 = (3.33, 19.6, 1250, 870, 41, 0.25, 12.5, 33.33, 29, 10, 0.85, 0.13, 0.04, 1)
FK_ERR_CAPACITY = 9
MAX_CELLS = 512 * 512


def _lib():
    from cardiax_gb300 import _native as N
    L = N.lib()
    fn = L.fk_forward_euler_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [N.Grid, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(N.Params),
                   ctypes.POINTER(N.Stimulus), ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                   ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    return N, L


def _setup(H, W):
    N, L = _lib()
    pitch = (W + 3) // 4 * 4
    dev = torch.device("cuda", 0)
    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    D = np.zeros((H, pitch), np.float32)
    D[:, :W] = 1e-3 * (1 - 0.5 * np.exp(-((i - H / 2) ** 2 + (j - W / 3) ** 2) / (0.1 * H * W)))
    state = torch.zeros((3, H, pitch), dtype=torch.float32, device=dev)
    state[0] = 1.0
    state[1] = 1.0
    stims = (N.Stimulus * 2)(N.Stimulus(0, 2, 1e9, None, 0, H, 0, 6, 20.0),
                             N.Stimulus(30, 2, 1e9, None, H // 2, H // 2 + 10, W // 2,
                                        W // 2 + 10, 20.0))
    return N, L, N.Grid(H, W, pitch), state, torch.as_tensor(D, device=dev), stims


def test_noalloc_matches_forward_euler_on_consecutive_calls():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    N, L, g, s0, D, stims = _setup(256, 250)
    params = N.Params(*P3)
    a, b = s0.clone(), s0.clone()
    scratch = torch.empty_like(s0)
    stream = torch.cuda.current_stream().cuda_stream
    for t0, t1 in ((0, 37), (37, 80)):  # odd step counts: the result ends in the scratch first
        rc = L.fk_forward_euler(g, a.data_ptr(), scratch.data_ptr(), D.data_ptr(),
                                ctypes.byref(params), stims, 2, t0, t1, 0.01, 0.01, stream)
        assert rc == 0, L.fk_status_string(rc)
        rc = L.fk_forward_euler_noalloc(g, b.data_ptr(), D.data_ptr(), ctypes.byref(params),
                                        stims, 2, t0, t1, 0.01, 0.01, stream)
        assert rc == 0, L.fk_status_string(rc)
        torch.cuda.synchronize()
        W = g.W
        for p in range(3):
            torch.testing.assert_close(b[p, :, :W], a[p, :, :W], rtol=0, atol=0, equal_nan=True)
    assert float(b[2, :, :W].max()) > 0.5  # the wave is travelling


@pytest.mark.parametrize("H,W", [(512, 512), (1024, 256)])
def test_noalloc_accepts_a_grid_exactly_at_its_capacity(H, W):
    """H * pitch == 512 * 512: the largest grid the array holds, an odd step count (the result
    is copied back from the array), bit for bit against fk_forward_euler."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    N, L, g, s0, D, stims = _setup(H, W)
    assert g.H * g.pitch == MAX_CELLS
    params = N.Params(*P3)
    a, b = s0.clone(), s0.clone()
    scratch = torch.empty_like(s0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.fk_forward_euler(g, a.data_ptr(), scratch.data_ptr(), D.data_ptr(),
                            ctypes.byref(params), stims, 2, 0, 41, 0.01, 0.01, stream)
    assert rc == 0, L.fk_status_string(rc)
    rc = L.fk_forward_euler_noalloc(g, b.data_ptr(), D.data_ptr(), ctypes.byref(params), stims,
                                    2, 0, 41, 0.01, 0.01, stream)
    assert rc == 0, L.fk_status_string(rc)
    torch.cuda.synchronize()
    torch.testing.assert_close(b[:, :, :W], a[:, :, :W], rtol=0, atol=0, equal_nan=True)


def test_noalloc_leaves_the_row_padding_of_the_state_unchanged():
    """After a call on another grid shape has filled the array, an odd step count (whose result
    comes back from the array) returns the caller's padding columns as they were."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    N, L, g1, s1, D1, st1 = _setup(300, 301)  # pitch 304: fills the array's padding with data
    params = N.Params(*P3)
    rc = L.fk_forward_euler_noalloc(g1, s1.data_ptr(), D1.data_ptr(), ctypes.byref(params), st1,
                                    2, 0, 31, 0.01, 0.01, stream)
    assert rc == 0, L.fk_status_string(rc)
    N, L, g, s0, D, stims = _setup(200, 250)  # pitch 252: two padding columns per row
    s0[:, :, 250:] = -7.25  # a marker the kernels never write
    a, b = s0.clone(), s0.clone()
    scratch = torch.empty_like(s0)
    rc = L.fk_forward_euler(g, a.data_ptr(), scratch.data_ptr(), D.data_ptr(),
                            ctypes.byref(params), stims, 2, 0, 33, 0.01, 0.01, stream)
    assert rc == 0, L.fk_status_string(rc)
    rc = L.fk_forward_euler_noalloc(g, b.data_ptr(), D.data_ptr(), ctypes.byref(params), stims,
                                    2, 0, 33, 0.01, 0.01, stream)
    assert rc == 0, L.fk_status_string(rc)
    torch.cuda.synchronize()
    torch.testing.assert_close(b[:, :, :250], a[:, :, :250], rtol=0, atol=0, equal_nan=True)
    assert bool((b[:, :, 250:] == -7.25).all())


def test_noalloc_refuses_grids_beyond_its_capacity():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    N, L = _lib()
    params = N.Params(*P3)
    stims = (N.Stimulus * 1)()
    g = N.Grid(513, 512, 512)  # H * pitch = 513 * 512 > 512 * 512
    assert g.H * g.pitch > MAX_CELLS
    rc = L.fk_forward_euler_noalloc(g, 256, 256, ctypes.byref(params), stims, 0, 0, 1, 0.01,
                                    0.01, None)
    assert rc == FK_ERR_CAPACITY
    assert b"512 * 512" in L.fk_status_string(rc)
