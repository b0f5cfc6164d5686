"""GPU parity for geqrf (LAPACKE_dgeqrf / zml_gpu_dgeqrf) against the oracle.

The oracle restates zml's geqrf (nb 32, nx 128, recursive larft, larfb).
Householder QR with larfg's sign convention is unique, so R, tau and the
reflectors below the diagonal must agree to rounding:
    |R - R_ref| <= 1e-11 max|R_ref|,  |tau - tau_ref| <= 1e-11,
and the backward error ||A - Q R|| / (||A|| m u) (Q formed by scipy from
our reflectors) stays below 8.  At sizes the oracle cannot reach in seconds,
the size-independent property ||A(:, j)|| = ||R(0:j, j)|| is checked.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lap

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P, gaussian

pytestmark = pytest.mark.gpu
EPS = 2.0 ** -53


def gpu_geqrf(a, layout=102):
    m, n = a.shape
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    tau = np.zeros(min(m, n))
    ld = m if layout == 102 else n
    assert zg.lib().LAPACKE_dgeqrf(layout, m, n, P(buf), ld, P(tau)) == 0, zg.last_error()
    return np.asfortranarray(buf), tau


@pytest.mark.parametrize("m,n", [(10, 10), (40, 33), (200, 150), (150, 200), (513, 260),
                                 (1000, 64), (2048, 512)])
def test_dgeqrf_vs_oracle(m, n):
    a = gaussian(m, n, seed=m + 3 * n)
    qr, tau = gpu_geqrf(a)
    qr_ref, tau_ref = ol.geqrf(a)
    k = min(m, n)
    scale = np.abs(qr_ref).max()
    np.testing.assert_allclose(np.triu(qr), np.triu(qr_ref), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(np.tril(qr, -1), np.tril(qr_ref, -1), rtol=0, atol=1e-10)
    np.testing.assert_allclose(tau, tau_ref[:k], rtol=0, atol=1e-11)
    q = lap.dorgqr(qr[:, :k].copy(order="F"), tau)[0]
    err = np.linalg.norm(q @ np.triu(qr[:k]) - a) / (np.linalg.norm(a) * m * EPS)
    assert err < 8


def test_dgeqrf_row_major_and_zero_column():
    a = gaussian(300, 100, seed=5)
    a[:, 40] = 0.0
    qr_c, tau_c = gpu_geqrf(a)
    qr_r, tau_r = gpu_geqrf(a, layout=101)
    np.testing.assert_allclose(qr_r, qr_c, rtol=0, atol=1e-13 * np.abs(qr_c).max())
    qr_ref, tau_ref = ol.geqrf(a)
    np.testing.assert_allclose(tau_c, tau_ref[:100], rtol=0, atol=1e-11)


def test_dgeqrf_large_column_norms():
    """8192 x 2048 on device memory: column norms of A equal those of R."""
    import torch
    m, n = 8192, 2048
    g = torch.Generator(device="cuda").manual_seed(9)
    a = torch.randn(n, m, device="cuda", dtype=torch.float64, generator=g)  # col-major m x n
    a0 = a.clone()
    tau = torch.zeros(n, device="cuda", dtype=torch.float64)
    assert zg.lib().zml_gpu_dgeqrf(m, n, a.data_ptr(), m, tau.data_ptr(), None) == 0
    A = a0.t()
    R = torch.triu(a.t()[:n])
    ratio = (A.norm(dim=0) / R.norm(dim=0) - 1).abs().max().item()
    assert ratio < 1e-12
    assert torch.all((tau >= 1) & (tau <= 2) | (tau == 0))


def gpu_orgqr(qr, tau, ncols, layout=102):
    m = qr.shape[0]
    k = len(tau)
    src = np.zeros((m, ncols))
    src[:, :min(ncols, qr.shape[1])] = qr[:, :min(ncols, qr.shape[1])]
    buf = np.array(src, order="F" if layout == 102 else "C", copy=True)
    ld = m if layout == 102 else ncols
    t = np.ascontiguousarray(tau, dtype=np.float64)
    assert zg.lib().LAPACKE_dorgqr(layout, m, ncols, k, P(buf), ld, P(t)) == 0, zg.last_error()
    return np.asfortranarray(buf)


@pytest.mark.parametrize("m,n,full", [(10, 10, False), (200, 150, False), (200, 150, True),
                                      (513, 260, False), (1000, 64, True), (2048, 512, False)])
def test_dorgqr_vs_oracle(m, n, full):
    """Q of the oracle's reflectors: equal to the oracle's orgqr to rounding,
    orthonormal, and Q R = A."""
    a = gaussian(m, n, seed=m + n)
    qr, tau = ol.geqrf(a)
    k = min(m, n)
    ncols = m if full else k
    q = gpu_orgqr(qr, tau[:k], ncols)
    q_ref = ol.orgqr(qr, tau[:k], ncols)
    np.testing.assert_allclose(q, q_ref, rtol=0, atol=1e-12)
    assert np.linalg.norm(q.T @ q - np.eye(ncols)) < 20 * m * EPS
    err = np.linalg.norm(q[:, :k] @ np.triu(qr[:k]) - a) / (np.linalg.norm(a) * m * EPS)
    assert err < 8


def test_dorgqr_row_major_partial_k_and_args():
    a = gaussian(300, 120, seed=9)
    qr, tau = ol.geqrf(a)
    # k < n: columns k.. of Q start as identity columns
    q_c = gpu_orgqr(qr, tau[:50], 120)
    q_r = gpu_orgqr(qr, tau[:50], 120, layout=101)
    np.testing.assert_allclose(q_r, q_c, rtol=0, atol=1e-14)
    np.testing.assert_allclose(q_c, ol.orgqr(qr[:, :50].copy(order="F"), tau[:50], 120),
                               rtol=0, atol=1e-12)
    L = zg.lib()
    buf = np.zeros(16)
    assert L.LAPACKE_dorgqr(102, 4, 5, 2, P(buf), 4, P(buf)) == -3   # n > m
    assert L.LAPACKE_dorgqr(102, 4, 3, 4, P(buf), 4, P(buf)) == -4   # k > n
    assert L.LAPACKE_dorgqr(102, 4, 3, 2, P(buf), 3, P(buf)) == -6   # lda < m
    # k = 0: the identity's first n columns
    e = gpu_orgqr(np.zeros((6, 4)), np.zeros(0), 4)
    np.testing.assert_array_equal(e, np.eye(6, 4))


def test_dorgqr_large_orthonormal():
    """4096 x 1024 on device memory through zml_gpu_dorgqr: orthonormal Q and
    Q R = A (size-independent properties)."""
    import torch
    m, n = 4096, 1024
    g = torch.Generator(device="cuda").manual_seed(3)
    a = torch.randn(n, m, dtype=torch.float64, device="cuda", generator=g)  # column-major A
    qr = a.clone()
    tau = torch.zeros(n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    L = zg.lib()
    assert L.zml_gpu_dgeqrf(m, n, qr.data_ptr(), m, tau.data_ptr(), s) == 0
    q = qr.clone()
    assert L.zml_gpu_dorgqr(m, n, n, q.data_ptr(), m, tau.data_ptr(), s) == 0
    Q = q.T  # logical m x n
    R = torch.triu(qr.T[:n])
    orth = torch.linalg.norm(Q.T @ Q - torch.eye(n, dtype=torch.float64, device="cuda")).item()
    back = (torch.linalg.norm(Q @ R - a.T) / torch.linalg.norm(a)).item()
    assert orth < 20 * m * EPS and back < 8 * m * EPS
