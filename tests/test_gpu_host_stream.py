"""zml_dgesv_mpir with A in page-locked host memory (BF16x3 updates, n >= 4096):
A's copy to the device runs in column chunks beside the factorization, each
chunk receiving the updates of the blocks factored before it joined.  The
per-element arithmetic is the device-resident path's, so the solution, the
iteration count and the backward error are bit for bit those of the same
solve from device pointers and from pageable host memory (which is staged
whole before the factorization)."""
import ctypes as C

import numpy as np
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu

BF16X3, GMRES = 3, 1


def _solve(L, n, lda, a_ptr, b_ptr, x_ptr, tol=64 * 2.0 ** -53):
    res = zg.MpirResult()
    rc = L.zml_dgesv_mpir(102, n, 1, a_ptr, lda, b_ptr, n, x_ptr, n, BF16X3, GMRES, tol, 30,
                          C.byref(res))
    assert rc == 0, zg.last_error()
    return res


@pytest.mark.parametrize("n,pad", [(4096, 0), (5000, 0), (8192, 3)])
def test_streamed_host_solve_equals_device_solve(n, pad):
    import torch
    L = zg.lib()
    lda = n + pad
    g = torch.Generator().manual_seed(n)
    A = torch.randn(n, lda, dtype=torch.float64, generator=g)  # row j of storage = column j
    b = torch.rand(n, 1, dtype=torch.float64, generator=g) * 2 - 1

    # device pointers: the whole A resident before the factorization
    Ad, bd = A.cuda(), b.cuda()
    xd = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rd = _solve(L, n, lda, Ad.data_ptr(), bd.data_ptr(), xd.data_ptr())
    assert rd.info == 0 and rd.converged == 1 and rd.fp64_fallback == 0

    # page-locked host A: copied in chunks beside the factorization
    Ah, bh = A.pin_memory(), b.pin_memory()
    xh = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
    rh = _solve(L, n, lda, Ah.data_ptr(), bh.data_ptr(), xh.data_ptr())
    assert rh.info == 0 and rh.converged == 1 and rh.fp64_fallback == 0
    assert rh.iters == rd.iters
    assert rh.berr == rd.berr
    assert torch.equal(xh, xd.cpu())

    # pageable host A: staged whole, then the device-resident path
    An = np.ascontiguousarray(A.numpy())
    bn = b.numpy().copy()
    xn = np.zeros((n, 1))
    rn = _solve(L, n, lda, An.ctypes.data, bn.ctypes.data, xn.ctypes.data)
    assert rn.iters == rd.iters and rn.berr == rd.berr
    assert np.array_equal(xn, xd.cpu().numpy())


def test_streamed_host_solve_repeats_and_interleaves():
    """Back-to-back streamed calls reuse the staged A, the FP32 copy and the
    saved operands; a device-pointer solve of another matrix in between must
    not disturb them (every internal stream starts after the caller's earlier
    work)."""
    import torch
    L = zg.lib()
    n = 4608
    g = torch.Generator().manual_seed(11)
    A1 = torch.randn(n, n, dtype=torch.float64, generator=g).pin_memory()
    A2 = torch.randn(n, n, dtype=torch.float64, generator=g)
    b = (torch.rand(n, 1, dtype=torch.float64, generator=g) * 2 - 1).pin_memory()
    x1 = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
    x2 = torch.zeros_like(x1).pin_memory()
    r1 = _solve(L, n, n, A1.data_ptr(), b.data_ptr(), x1.data_ptr())
    A2d, bd = A2.cuda(), b.cuda()
    xd = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _solve(L, n, n, A2d.data_ptr(), bd.data_ptr(), xd.data_ptr())
    r2 = _solve(L, n, n, A1.data_ptr(), b.data_ptr(), x2.data_ptr())
    assert r1.converged == 1 and r2.converged == 1
    assert r1.iters == r2.iters and r1.berr == r2.berr
    assert torch.equal(x1, x2)
    # and x solves A1 x = b (A1's storage is A1^T in column-major terms)
    assert r2.berr <= 64 * 2.0 ** -53
    A1d = A1.cuda().t()
    r = b.cuda() - A1d @ x2.cuda()
    scale = A1d.abs().sum(1).max() * x2.cuda().abs().max() + b.cuda().abs().max()
    assert float(r.abs().max() / scale) <= 1e-13


def test_streamed_host_solve_repeats_bitwise_at_n32768():
    """The streamed path at n = 32768 keeps about nine streams busy beside the
    factorization, so the thread-block-cluster panel's CTAs share SMs with
    other kernels and drift apart in time.  Repeated solves must stay bit for
    bit those of the device-pointer solve: this caught a missing cluster
    barrier in the panel (a late CTA read rows of A12 that CTA 0 had already
    replaced by U12), which changed pivots in about four solves of ten."""
    import torch
    L = zg.lib()
    n = 32768
    g = torch.Generator(device="cuda").manual_seed(1)
    Ad = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    bd = torch.rand(n, 1, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    Ah = torch.empty(n, n, dtype=torch.float64).pin_memory()
    Ah.copy_(Ad)
    bh = bd.cpu().pin_memory()
    xd = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rd = _solve(L, n, n, Ad.data_ptr(), bd.data_ptr(), xd.data_ptr())
    assert rd.converged == 1 and rd.fp64_fallback == 0
    x_ref = xd.cpu()
    xh = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
    for _ in range(6):
        rh = _solve(L, n, n, Ah.data_ptr(), bh.data_ptr(), xh.data_ptr())
        assert rh.fp64_fallback == 0 and rh.iters == rd.iters
        assert torch.equal(xh, x_ref)


@pytest.mark.parametrize("n,prec", [(1000, BF16X3), (4096, 2)])
def test_pinned_host_below_streaming_scope_equals_device(n, prec):
    """Page-locked A outside the streamed path's scope (n < 4096, or factors
    other than BF16x3) is staged whole first and gives the device solve."""
    import torch
    L = zg.lib()
    g = torch.Generator().manual_seed(n + prec)
    A = torch.randn(n, n, dtype=torch.float64, generator=g)
    b = torch.rand(n, 1, dtype=torch.float64, generator=g) * 2 - 1

    def solve(a, bb, xx):
        res = zg.MpirResult()
        rc = L.zml_dgesv_mpir(102, n, 1, a, n, bb, n, xx, n, prec, GMRES, 64 * 2.0 ** -53, 30,
                              C.byref(res))
        assert rc == 0, zg.last_error()
        return res

    Ad, bd = A.cuda(), b.cuda()
    xd = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rd = solve(Ad.data_ptr(), bd.data_ptr(), xd.data_ptr())
    Ah, bh = A.pin_memory(), b.pin_memory()
    xh = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
    rh = solve(Ah.data_ptr(), bh.data_ptr(), xh.data_ptr())
    assert rd.converged == 1 and rh.iters == rd.iters and rh.berr == rd.berr
    assert torch.equal(xh, xd.cpu())


def test_streamed_host_solve_singular_matches_device():
    """A zero column in page-locked A: the streamed factorization records the
    zero pivot like the device path, refinement is skipped, the FP64 fallback
    finds the matrix singular too, and both calls report the same."""
    import torch
    L = zg.lib()
    n = 4096
    g = torch.Generator().manual_seed(7)
    A = torch.randn(n, n, dtype=torch.float64, generator=g)
    A[1000, :] = 0.0  # storage row 1000 = column 1000 of the column-major matrix
    b = torch.rand(n, 1, dtype=torch.float64, generator=g) * 2 - 1

    def solve(a, bb, xx):
        res = zg.MpirResult()
        rc = L.zml_dgesv_mpir(102, n, 1, a, n, bb, n, xx, n, BF16X3, GMRES, 64 * 2.0 ** -53, 30,
                              C.byref(res))
        return rc, res

    Ad, bd = A.cuda(), b.cuda()
    xd = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rcd, rd = solve(Ad.data_ptr(), bd.data_ptr(), xd.data_ptr())
    Ah, bh = A.pin_memory(), b.pin_memory()
    xh = torch.zeros(n, 1, dtype=torch.float64).pin_memory()
    rch, rh = solve(Ah.data_ptr(), bh.data_ptr(), xh.data_ptr())
    assert rch == rcd
    assert rh.info == rd.info and rh.info > 0
    assert rh.fp64_fallback == rd.fp64_fallback
    assert rh.converged == rd.converged == 0
