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
