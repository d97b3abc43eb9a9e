"""The tcgen05 BF16 GEMM and the MLP's elementwise kernels against plain PyTorch FP32 references.

GEMM tolerance: the BF16 products are exact in FP32; only the FP32 summation order differs from torch's, so the
result must agree to 1e-5 of the row-vector norms (|C - C_ref| <= 1e-5 |A_row| |B_row|). BF16 outputs agree to one
BF16 rounding (rtol 1/128)."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def env():
    import torch

    from sosfuse2_gb300 import _abi

    lib = _abi.library()
    return torch, lib


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def check(lib, torch):
    rc = lib.sosb_tc_check(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.sosb_tc_last_error()


@pytest.mark.parametrize('M,N,K', [(128, 128, 64), (256, 384, 512), (512, 512, 1024)])
@pytest.mark.parametrize('epilogue', [0, 1, 2])
def test_gemm_matches_torch(env, M, N, K, epilogue):
    torch, lib = env
    g = torch.Generator(device='cuda').manual_seed(M + N + K + epilogue)
    A = torch.randn(M, K, device='cuda', generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device='cuda', generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device='cuda', generator=g)
    C = torch.full((M, N), float('nan'), device='cuda')
    H = torch.zeros((M, N), device='cuda', dtype=torch.bfloat16)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.sosb_gemm_bf16(ptr(A), ptr(B), M, N, K, ptr(bias), epilogue, ptr(C), ptr(H), stream)
    assert rc == 0, lib.sosb_tc_last_error()
    check(lib, torch)
    ref = A.float() @ B.float().T
    if epilogue:
        ref = ref + bias
    scale = torch.outer(A.float().norm(dim=1), B.float().norm(dim=1))
    assert torch.all((C - ref).abs() <= 1e-5 * scale + 1e-6), float(((C - ref).abs() / scale).max())
    if epilogue == 1:
        act = torch.nn.functional.gelu(ref)
        assert torch.allclose(H.float(), act, rtol=1.0 / 128, atol=1e-2)


def test_rejects_bad_shapes(env):
    torch, lib = env
    A = torch.zeros(100, 64, device='cuda', dtype=torch.bfloat16)
    C = torch.zeros(100, 128, device='cuda')
    rc = lib.sosb_gemm_bf16(ptr(A), ptr(A), 100, 128, 64, None, 0, ptr(C), None, None)
    assert rc != 0 and b'E_SHAPE' in lib.sosb_tc_last_error()


def test_elementwise_kernels(env):
    torch, lib = env
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator(device='cuda').manual_seed(3)
    z = torch.randn(300, 257, device='cuda', generator=g)
    dh = torch.randn(300, 257, device='cuda', generator=g)
    dzb = torch.empty(300, 257, device='cuda', dtype=torch.bfloat16)
    dzf = torch.empty(300, 257, device='cuda')
    assert lib.sosb_mlp_gelu_backward(ptr(dh), ptr(z), z.numel(), ptr(dzb), ptr(dzf), stream) == 0
    zz = z.clone().requires_grad_(True)
    torch.nn.functional.gelu(zz).backward(dh)
    assert torch.allclose(dzf, zz.grad, rtol=1e-5, atol=1e-6)
    tb = torch.empty(257, 300, device='cuda', dtype=torch.bfloat16)
    assert lib.sosb_mlp_transpose(ptr(z), 1, 300, 257, ptr(tb), stream) == 0
    assert torch.equal(tb, z.T.contiguous().to(torch.bfloat16))
    cs = torch.empty(257, device='cuda')
    assert lib.sosb_mlp_column_sum(ptr(z), 300, 257, ptr(cs), stream) == 0
    assert torch.allclose(cs, z.sum(0), rtol=1e-5, atol=1e-5)
    w = torch.randn(1000, device='cuda', generator=g)
    gr = torch.randn(1000, device='cuda', generator=g)
    m = torch.zeros(1000, device='cuda')
    v = torch.zeros(1000, device='cuda')
    wb = torch.empty(1000, device='cuda', dtype=torch.bfloat16)
    w_ref = w.clone()
    assert lib.sosb_mlp_adam(ptr(w), ptr(gr), ptr(m), ptr(v), 1000, 1e-3, 0.9, 0.999, 1e-8, 1, 0.0, ptr(wb),
                             stream) == 0
    mh = 0.1 * gr / 0.1
    vh = 0.001 * gr * gr / 0.001
    assert torch.allclose(w, w_ref - 1e-3 * mh / (vh.sqrt() + 1e-8), rtol=1e-5, atol=1e-6)
    assert torch.equal(wb, w.to(torch.bfloat16))
    check(lib, torch)
