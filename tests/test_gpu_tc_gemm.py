"""The tensor-core GEMM (tcgen05 + TMA) against a float reference of the same
bf16 products."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, m, n, k, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, generator=g).to(torch.bfloat16)
    ad, bd = a.cuda(), b.cuda()
    d = torch.zeros(m, n, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib.gpl_tc_gemm_bf16.restype = C.c_int
    rc = lib.gpl_tc_gemm_bf16(C.c_void_p(ad.data_ptr()), C.c_void_p(bd.data_ptr()), C.c_void_p(d.data_ptr()),
                              m, n, k, C.c_void_p(err.data_ptr()), None)
    assert rc == 0, lib.gpl_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = a.float() @ b.float().T
    return d.cpu(), ref


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (128, 256, 256), (256, 384, 1024), (1024, 1024, 3072)])
def test_tc_gemm_matches_float_products(gpu_lib, m, n, k):
    d, ref = _run(gpu_lib, m, n, k, seed=m + n + k)
    # bf16 inputs are exact in fp32; only the fp32 accumulation order differs
    scale = ref.abs().max().item()
    assert (d - ref).abs().max().item() <= 1e-5 * scale * np.sqrt(k / 64)


def test_tc_gemm_rejects_bad_shapes(gpu_lib):
    import torch
    x = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    d = torch.zeros(128, 128, dtype=torch.float32, device="cuda")
    gpu_lib.gpl_tc_gemm_bf16.restype = C.c_int
    rc = gpu_lib.gpl_tc_gemm_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(d.data_ptr()),
                                  100, 128, 64, None, None)
    assert rc == 16
