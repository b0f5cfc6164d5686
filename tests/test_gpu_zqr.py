"""GPU complex Householder QR (LAPACKE_zgeqrf / cgeqrf) against the complex
oracle (zml's geqrf over cfloat restated) and scipy's LAPACK zgeqrf.

Householder QR with larfg's convention (beta real, -sign(re alpha) |(alpha, x)|)
is unique, so R, tau and the reflectors below the diagonal must agree to
rounding with both: |R - R_ref| <= 1e-11 max|R_ref|, |tau - tau_ref| <= 1e-11,
|V - V_ref| <= 1e-10 (binary64; 2e-4 relative for binary32), and the
backward error ||A - Q R|| / (||A|| m u) with Q formed by scipy's zungqr from
our reflectors stays below 8.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lap

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P

pytestmark = pytest.mark.gpu


def cmat(m, n, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    return np.asfortranarray((rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))).astype(dtype))


def gpu_zgeqrf(a, layout=102):
    m, n = a.shape
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    tau = np.zeros(min(m, n), dtype=a.dtype)
    f = zg.lib().LAPACKE_zgeqrf if a.dtype == np.complex128 else zg.lib().LAPACKE_cgeqrf
    rc = f(layout, m, n, P(buf), m if layout == 102 else n, P(tau))
    assert rc == 0, (rc, zg.last_error())
    return np.asfortranarray(buf), tau


@pytest.mark.parametrize("m,n", [(1, 1), (10, 10), (40, 33), (200, 150), (150, 200), (513, 260),
                                 (1000, 64), (2048, 300)])
def test_zgeqrf_vs_oracle_and_scipy(m, n):
    a = cmat(m, n, seed=m + 7 * n)
    qr, tau = gpu_zgeqrf(a)
    k = min(m, n)
    qr_ref, tau_ref = ol.geqrf(a)
    scale = np.abs(qr_ref).max()
    np.testing.assert_allclose(np.triu(qr), np.triu(qr_ref), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(np.tril(qr, -1), np.tril(qr_ref, -1), rtol=0, atol=1e-10)
    np.testing.assert_allclose(tau, tau_ref[:k], rtol=0, atol=1e-11)
    qr_s, tau_s, _, info = lap.zgeqrf(a)
    assert info == 0
    np.testing.assert_allclose(np.triu(qr), np.triu(qr_s), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(tau, tau_s, rtol=0, atol=1e-11)
    q = lap.zungqr(qr[:, :k].copy(order="F"), tau)[0]
    err = np.linalg.norm(q @ np.triu(qr[:k]) - a) / (np.linalg.norm(a) * m * 2.0 ** -53)
    assert err < 8


def test_cgeqrf_single():
    a = cmat(700, 300, seed=3, dtype=np.complex64)
    qr, tau = gpu_zgeqrf(a)
    qr_ref, tau_ref = ol.geqrf(a)
    scale = np.abs(qr_ref).max()
    assert np.abs(np.triu(qr) - np.triu(qr_ref)).max() <= 2e-4 * scale
    assert np.abs(tau - tau_ref[:300]).max() <= 2e-4


def test_zgeqrf_row_major_zero_column_and_real_column():
    a = cmat(300, 120, seed=5)
    a[:, 40] = 0.0          # x = 0 and alpha real: H = I, tau = 0
    a[:, 41] = a[:, 41].real  # a real column: tau real only if the rest is
    qr_c, tau_c = gpu_zgeqrf(a)
    qr_r, tau_r = gpu_zgeqrf(a, layout=101)
    np.testing.assert_allclose(qr_r, qr_c, rtol=0, atol=1e-13 * np.abs(qr_c).max())
    np.testing.assert_allclose(tau_r, tau_c, rtol=0, atol=1e-13)
    qr_ref, tau_ref = ol.geqrf(a)
    np.testing.assert_allclose(tau_c, tau_ref[:120], rtol=0, atol=1e-11)
    assert np.all(np.isreal(np.diag(qr_c)))  # beta is real


def test_zgeqrf_large_column_norms():
    """16384 x 1024 on device memory: column norms of A equal those of R."""
    import torch
    m, n = 16384, 1024
    g = torch.Generator(device="cuda").manual_seed(11)
    a = torch.randn(n, m, 2, device="cuda", dtype=torch.float64, generator=g)  # col-major m x n
    a0 = torch.view_as_complex(a.clone()).t()
    tau = torch.zeros(n, 2, device="cuda", dtype=torch.float64)
    assert zg.lib().zml_gpu_zgeqrf(m, n, a.data_ptr(), m, tau.data_ptr(), None) == 0
    R = torch.triu(torch.view_as_complex(a).t()[:n])
    ratio = (a0.abs().pow(2).sum(0).sqrt() / R.abs().pow(2).sum(0).sqrt() - 1).abs().max().item()
    assert ratio < 1e-12
