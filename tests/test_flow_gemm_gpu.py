"""The tcgen05 BF16 GEMM (ntp_gemm_bf16) against a plain PyTorch FP32 product
of the same BF16 inputs.  Tolerance: the FP32 accumulation order differs, so
|C - C_ref| <= 1e-3 * max|C_ref| + 1e-5; BF16 outputs compare after rounding."""
import pytest

from neutrinotelescopes_gb300 import _abi

pytestmark = pytest.mark.gpu


def run(M, N, K, relu=0, bias=False, out_kind=0, splits=1, seed=0):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = (torch.randn(M, K, device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    B = (torch.randn(N, K, device="cuda", generator=g) * 0.5).to(torch.bfloat16)
    b = torch.randn(N, device="cuda", generator=g) if bias else None
    ref = A.float() @ B.float().T
    if bias:
        ref = ref + b
    if relu:
        ref = torch.relu(ref)
    dtype = torch.bfloat16 if out_kind == 1 else torch.float32
    C = torch.zeros(M, N, device="cuda", dtype=dtype)
    lib = _abi.load_library()
    st = lib.ntp_gemm_bf16(A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N, M, N, K,
                           b.data_ptr() if bias else None, relu, out_kind, splits, None)
    torch.cuda.synchronize()
    assert st == _abi.NTP_OK, st
    tol = 1e-3 * ref.abs().max().item() + 1e-5
    if out_kind == 1:
        tol += 8e-3 * ref.abs().max().item()
    err = (C.float() - ref).abs().max().item()
    assert err <= tol, (err, tol)


def test_gemm_single_tile():
    run(128, 64, 64)


@pytest.mark.parametrize("M,N,K", [(128, 256, 128), (300, 192, 256), (1000, 100, 320), (8192, 256, 256)])
def test_gemm_shapes(M, N, K):
    run(M, N, K)


def test_gemm_bias_relu_bf16_out():
    run(512, 256, 256, relu=1, bias=True, out_kind=1)


def test_gemm_split_k_atomic():
    run(256, 256, 8192, out_kind=2, splits=32)


def test_gemm_rejects_bad_shapes():
    import torch
    A = torch.zeros(128, 60, device="cuda", dtype=torch.bfloat16)
    C = torch.zeros(128, 128, device="cuda")
    lib = _abi.load_library()
    assert lib.ntp_gemm_bf16(A.data_ptr(), 60, A.data_ptr(), 60, C.data_ptr(), 128, 128, 128, 60, None, 0, 0, 1,
                             None) == _abi.NTP_ERR_INVALID


def test_gemm_wait_runs_out_and_the_context_stays_usable():
    """The failure-detection path: with the first pipeline stage's copies
    withheld, the first mbarrier wait has nothing to complete; it gives up
    after the 1 ms limit and the call returns NTP_ERR_TIMEOUT.  The next GEMM
    on the same context, with the default limit, is correct."""
    import time

    import torch
    lib = _abi.load_library()
    M, N, K = 128, 64, 256
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    C = torch.zeros(M, N, device="cuda")
    assert lib.ntp_gemm_set_wait_limit(1_000_000, 1) == _abi.NTP_OK
    try:
        t0 = time.perf_counter()
        st = lib.ntp_gemm_bf16(A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N, M, N, K, None, 0, 0, 1, None)
        elapsed = time.perf_counter() - t0
    finally:
        assert lib.ntp_gemm_set_wait_limit(0, 0) == _abi.NTP_OK
    assert st == _abi.NTP_ERR_TIMEOUT, st
    assert elapsed < 1.0
    torch.cuda.synchronize()
    run(M, N, K)
    run(512, 256, 256, relu=1, bias=True, out_kind=1)
