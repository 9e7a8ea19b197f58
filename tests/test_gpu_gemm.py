"""The tcgen05 BF16 GEMM of the surrogate network against torch (FP32 accumulation of the same
bf16 inputs).  Tolerance: 2e-3 relative to the output scale (FP32 accumulation order differs)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k,split", [(128, 128, 64, 1), (256, 192, 128, 1), (384, 128, 192, 1),
                                         (128, 128, 4096, 1), (128, 192, 8192, 4), (128, 128, 16384, 8)])
def test_gemm_matches_torch(fwn_lib, m, n, k, split):
    import torch

    import meshlib_gb300 as M
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device="cuda", generator=g).to(torch.bfloat16)
    d = torch.zeros(m, n, device="cuda")
    st = M.lib().gbfwn_debug_gemm_bf16(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                       ctypes.c_void_p(d.data_ptr()), m, n, k, split, None)
    assert st == 0
    torch.cuda.synchronize()
    ref = a.float() @ b.float().T
    err = (d - ref).abs().max().item()
    assert err <= 2e-3 * ref.abs().max().item(), err


def test_wait_timeout_path_keeps_the_device_usable(fwn_lib):
    """A bounded mbarrier wait that nothing completes gives up, reports GBFWN_TIMEOUT, frees its TMEM;
    tensor-core GEMMs still run correctly afterwards on the same context."""
    import torch

    import meshlib_gb300 as M
    for _ in range(2):
        assert M.lib().gbfwn_debug_wait_timeout(1 << 10, None) == M.TIMEOUT
    assert b"gave up" in M.lib().gbfwn_last_error()
    a = torch.randn(128, 64, device="cuda").to(torch.bfloat16)
    b = torch.randn(128, 64, device="cuda").to(torch.bfloat16)
    d = torch.zeros(128, 128, device="cuda")
    assert M.lib().gbfwn_debug_gemm_bf16(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                         ctypes.c_void_p(d.data_ptr()), 128, 128, 64, 1, None) == 0
    torch.cuda.synchronize()
    ref = a.float() @ b.float().T
    assert (d - ref).abs().max().item() <= 2e-3 * ref.abs().max().item()
