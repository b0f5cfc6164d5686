"""tcgen05 tensor-core GEMM (zml_gpu_gemm_lowp) against a torch fp32 reference.

C (fp32, column-major) <- alpha A B^T + beta C with 16-bit A (M x K) and
B (N x K) stored K-major.  The reference is the same product of the same
16-bit values in fp32 (torch); the tolerance covers fp32 accumulation order:
|C - C_ref| <= 1e-5 * (|alpha| * |A||B|^T + |beta C|).
"""
import numpy as np
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu


def run(M, N, K, prec, alpha=1.0, beta=0.0, seed=0, pad=0):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    dt = torch.bfloat16 if prec == 1 else torch.float16
    ld = ((K + 7) // 8) * 8 + pad
    A = torch.randn(M, ld, device="cuda", generator=g).to(dt)
    B = torch.randn(N, ld, device="cuda", generator=g).to(dt)
    C0 = torch.randn(N, M, device="cuda", generator=g)  # column-major M x N == row-major N x M
    C = C0.clone()
    r = zg.lib().zml_gpu_gemm_lowp(prec, M, N, K, alpha, A.data_ptr(), ld, B.data_ptr(), ld, beta,
                                   C.data_ptr(), M, None)
    assert r == 0, zg.last_error()
    Af, Bf = A[:, :K].float(), B[:, :K].float()
    ref = alpha * (Af @ Bf.T) + beta * C0.T
    bound = 1e-5 * (abs(alpha) * (Af.abs() @ Bf.abs().T) + abs(beta) * C0.T.abs()) + 1e-30
    err = ((C.T - ref).abs() / bound).max().item()
    return err


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 128), (1024, 512, 320),
                                   (200, 72, 100), (129, 130, 17), (1, 1, 1), (4096, 4096, 256)])
@pytest.mark.parametrize("prec", [1, 0])
def test_gemm_lowp_vs_torch(M, N, K, prec):
    assert run(M, N, K, prec) <= 1.0


def test_gemm_lowp_alpha_beta_update():
    # the LU trailing-update form C <- C - L U
    assert run(777, 515, 128, 1, alpha=-1.0, beta=1.0, seed=3, pad=8) <= 1.0


def test_gemm_lowp_k_zero_scales_c():
    import torch
    C = torch.ones(64, 64, device="cuda")
    A = torch.zeros(64, 8, device="cuda", dtype=torch.bfloat16)
    assert zg.lib().zml_gpu_gemm_lowp(1, 64, 64, 0, 1.0, A.data_ptr(), 8, A.data_ptr(), 8, 0.5,
                                      C.data_ptr(), 64, None) == 0
    assert torch.all(C == 0.5)
