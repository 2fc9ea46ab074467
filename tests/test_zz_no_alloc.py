"""The allocation-free forward transform, through the C ABI.

`pqg_rfft2_noalloc` exists for callers that cannot call cudaMalloc: code
whose device memory belongs to another allocator (a framework's caching
allocator, a fixed arena reserved at start-up) and code that must not stall
the device, as cudaMalloc / cudaFree can.  It keeps its scratch in static
device arrays of the library instead.  This test checks, on consecutive
calls, that it returns what the plan-based `pqg_rfft2` returns, and that an
oversized request is refused with a message.  It runs last so that a
failure here leaves the rest of the suite's results intact.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-14   # the transform tolerance of the other GPU tests


def _plan_rfft2(L, x, nz, ny, nx, stream):
    import torch
    from pyqg_gb300 import _lib
    plan = ctypes.c_void_p()
    _lib.check(L.pqg_plan_create(ctypes.byref(plan), nz, ny, nx))
    try:
        out = torch.empty((x.shape[0], ny, nx // 2 + 1), dtype=torch.complex128, device=x.device)
        _lib.check(L.pqg_rfft2(plan, x.data_ptr(), out.data_ptr(), x.shape[0], stream))
        torch.cuda.synchronize()
    finally:
        L.pqg_plan_destroy(plan)
    return out


def _noalloc_rfft2(L, x, ny, nx, stream):
    import torch
    from pyqg_gb300 import _lib
    out = torch.empty((x.shape[0], ny, nx // 2 + 1), dtype=torch.complex128, device=x.device)
    _lib.check(L.pqg_rfft2_noalloc(x.data_ptr(), out.data_ptr(), x.shape[0], ny, nx, stream))
    torch.cuda.synchronize()
    return out


def test_noalloc_rfft2_matches_plan_rfft2_on_consecutive_calls():
    import torch
    from pyqg_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rng = np.random.default_rng(11)
    # two calls in a row at one size, then a call at another size (tables
    # reloaded) and one back at the first size
    for (nz, n) in [(2, 256), (2, 256), (3, 96), (2, 256)]:
        x = torch.from_numpy(rng.standard_normal((nz, n, n))).to(dev)
        want = _plan_rfft2(L, x, nz, n, n, stream)
        got = _noalloc_rfft2(L, x, n, n, stream)
        assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) < TOL
        assert rel_l2(got.cpu().numpy(), np.fft.rfftn(x.cpu().numpy(), axes=(-2, -1))) < TOL


def test_noalloc_rfft2_rectangular_and_largest_grids():
    """nx != ny (the x and y twiddle tables are sized and reloaded apart),
    and the largest transform lengths: nx/2 = 2048 fills the x table and
    ny = 2048 the y table, each with the scratch close to full."""
    import torch
    from pyqg_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rng = np.random.default_rng(12)
    for (nz, ny, nx) in [(1, 64, 128), (2, 128, 64), (1, 250, 4096), (1, 2048, 480), (1, 64, 128)]:
        assert nz * ny * (nx // 2 + 1) <= _lib.PQG_NOALLOC_MAX_COMPLEX
        x = torch.from_numpy(rng.standard_normal((nz, ny, nx))).to(dev)
        got = _noalloc_rfft2(L, x, ny, nx, stream)
        want = _plan_rfft2(L, x, nz, ny, nx, stream)
        assert rel_l2(got.cpu().numpy(), want.cpu().numpy()) < TOL
        assert rel_l2(got.cpu().numpy(), np.fft.rfftn(x.cpu().numpy(), axes=(-2, -1))) < TOL


def test_noalloc_rfft2_refuses_oversized_request():
    import torch
    from pyqg_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = 1024
    nplanes = 2   # 2 * 1024 * 513 complex values > the static scratch
    x = torch.zeros((nplanes, n, n), dtype=torch.float64, device=dev)
    out = torch.empty((nplanes, n, n // 2 + 1), dtype=torch.complex128, device=dev)
    rc = L.pqg_rfft2_noalloc(x.data_ptr(), out.data_ptr(), nplanes, n, n, None)
    assert rc == _lib.PQG_ERR_UNSUPPORTED
    assert b"exceeds the static scratch" in L.pqg_last_error()
    # the largest lengths together: 2048 * 2049 complex values, refused
    x = torch.zeros((1, 2048, 4096), dtype=torch.float64, device=dev)
    out = torch.empty((1, 2048, 2049), dtype=torch.complex128, device=dev)
    rc = L.pqg_rfft2_noalloc(x.data_ptr(), out.data_ptr(), 1, 2048, 4096, None)
    assert rc == _lib.PQG_ERR_UNSUPPORTED
    assert b"exceeds the static scratch" in L.pqg_last_error()
