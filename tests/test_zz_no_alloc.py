"""The allocation-free Poisson entry point (gpl_poisson_solve_noalloc).

It exists for callers that must not allocate device memory during the call:
a placement server that admits jobs against a fixed HBM budget, a host
framework whose caching allocator owns the device memory, or a loop that
cannot absorb the synchronisation cudaMalloc/cudaFree may cause.  Its scratch
is a fixed static device array shared by all calls.  This file is collected
last so that a failure here cannot hide the result of any other test.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5     # the Poisson tolerance of tests/test_gpu_eval.py


def _solve(lib, fn, rho, nx, ny, bsx, bsy):
    import torch
    d = torch.from_numpy(rho).cuda()
    phi = torch.zeros_like(d); fx = torch.zeros_like(d); fy = torch.zeros_like(d)
    s = torch.cuda.current_stream().cuda_stream
    rc = fn(nx, ny, bsx, bsy, C.c_void_p(d.data_ptr()), C.c_void_p(phi.data_ptr()),
            C.c_void_p(fx.data_ptr()), C.c_void_p(fy.data_ptr()), C.c_void_p(s))
    torch.cuda.synchronize()
    return rc, phi.cpu().numpy(), fx.cpu().numpy(), fy.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import replace_gb300
    lib = replace_gb300.load()
    for name in ("gpl_poisson_solve", "gpl_poisson_solve_noalloc"):
        getattr(lib, name).restype = C.c_int
        getattr(lib, name).argtypes = [C.c_int32] * 4 + [C.c_void_p] * 5
    # two calls in a row (different grids, so the second call overwrites the
    # first one's scratch contents), each against the allocating entry point
    for (nx, ny, bsx, bsy, seed) in ((256, 512, 3901, 3877, 1), (512, 512, 4252, 4200, 2)):
        rho = (np.random.default_rng(seed).random((ny, nx)) * 1.4).astype(np.float32)
        rc0, p0, x0, y0 = _solve(lib, lib.gpl_poisson_solve, rho, nx, ny, bsx, bsy)
        rc1, p1, x1, y1 = _solve(lib, lib.gpl_poisson_solve_noalloc, rho, nx, ny, bsx, bsy)
        assert rc0 == 0 and rc1 == 0, lib.gpl_last_error()
        assert rel_l2(p1, p0) < TOL and rel_l2(x1, x0) < TOL and rel_l2(y1, y0) < TOL


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import replace_gb300
    lib = replace_gb300.load()
    lib.gpl_poisson_solve_noalloc.restype = C.c_int
    lib.gpl_poisson_solve_noalloc.argtypes = [C.c_int32] * 4 + [C.c_void_p] * 5
    rc = lib.gpl_poisson_solve_noalloc(1024, 512, 10, 10, C.c_void_p(8), None, C.c_void_p(8),
                                       C.c_void_p(8), None)
    assert rc == 16
    assert b"exceeds the fixed scratch limit" in lib.gpl_last_error()
