"""LAPACK-level checks of the complex oracle (CPU only).

zml has no complex LAPACK tests, so zgetrf / zgetrs / zpotrf / zpotrs are
pinned like their real counterparts: normwise backward error bounds and a
cross-check against scipy's bundled LAPACK (izamax picks the first maximum
of |re| + |im|, as zml's iamax does, so pivots agree on inputs without
near-ties).  The complex BLAS below them is pinned by zml's own known-answer
tests (test_oracle_golden.py).

The division of a real by a complex number is pinned by zml's own cfloat
test (test/cfloat/div.zig:42-44); the code as written (cfloat.zig:489-492)
returns the reciprocal quotient, and getrf2 reaches it (getrf2.zig:66-75).
"""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.linalg.lapack as lap

import oracle_lib as ol

EPS = 2.0 ** -53


def cgaussian(n, m=None, seed=0, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    shape = (n, m or n)
    return np.asfortranarray((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype))


def hpd(n, seed=0):
    g = cgaussian(n, seed=seed)
    return np.asfortranarray(g @ g.conj().T / n + np.eye(n))


def perm_matrix(ipiv, m):
    P = np.eye(m)
    for i, p in enumerate(ipiv):
        P[[i, p - 1]] = P[[p - 1, i]]
    return P


@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 65, 130])
def test_zgetrf_backward_error_and_scipy_pivots(n):
    a = cgaussian(n, seed=n)
    lu, ipiv, info = ol.getrf(a)
    assert info == 0
    L, U = np.tril(lu, -1) + np.eye(n), np.triu(lu)
    err = np.linalg.norm(perm_matrix(ipiv, n) @ a - L @ U) / (np.linalg.norm(a) * n * EPS)
    assert err < 10
    lu2, piv2, info2 = lap.zgetrf(a)
    np.testing.assert_array_equal(ipiv, piv2 + 1)
    np.testing.assert_allclose(lu, lu2, rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("m,n", [(90, 40), (40, 90), (1, 7), (7, 1)])
def test_zgetrf_rectangular(m, n):
    a = cgaussian(m, n, seed=m * n)
    lu, ipiv, info = ol.getrf(a)
    k = min(m, n)
    L = np.tril(lu[:, :k], -1) + np.eye(m, k)
    U = np.triu(lu[:k, :])
    np.testing.assert_allclose(perm_matrix(ipiv, m) @ a, L @ U, atol=1e-12 * np.abs(a).max() * n)


def test_cgetrf_single_precision():
    a = cgaussian(70, seed=3, dtype=np.complex64)
    lu, ipiv, info = ol.getrf(a)
    L, U = np.tril(lu, -1) + np.eye(70), np.triu(lu)
    err = np.abs(perm_matrix(ipiv, 70) @ a - L @ U).max() / np.abs(a).max()
    assert info == 0 and err < 70 * 2.0 ** -24 * 10


def test_zgetrf_singular_info():
    a = cgaussian(40, seed=4)
    a[:, 13] = 0
    _, _, info = ol.getrf(a)
    assert info == 14


@pytest.mark.parametrize("trans", [111, 112, 113])
def test_zgetrs(trans):
    n = 120
    a = cgaussian(n, seed=9)
    x = cgaussian(n, 3, seed=10)
    op = {111: a, 112: a.T, 113: a.conj().T}[trans]
    lu, ipiv, _ = ol.getrf(a)
    got = ol.getrs(lu, ipiv, op @ x, trans)
    np.testing.assert_allclose(got, x, atol=1e-11)


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n", [1, 5, 64, 65, 150])
def test_zpotrf_potrs(n, uplo):
    a = hpd(n, seed=n)
    f, info = ol.potrf(a, uplo)
    assert info == 0
    ref = sla.cholesky(a, lower=uplo == 122)
    tri = np.tril if uplo == 122 else np.triu
    np.testing.assert_allclose(tri(f), ref, atol=1e-12)
    # the imaginary parts of the diagonal are zero, the other triangle untouched
    assert not np.diag(f).imag.any()
    other = np.triu(a, 1) if uplo == 122 else np.tril(a, -1)
    np.testing.assert_array_equal(np.triu(f, 1) if uplo == 122 else np.tril(f, -1), other)
    x = cgaussian(n, 2, seed=n + 1)
    np.testing.assert_allclose(ol.potrs(f, a @ x, uplo), x, atol=1e-10)


def test_zpotrf_not_positive_definite_info():
    a = hpd(50, seed=2)
    a[30, 30] = -4.0
    _, info = ol.potrf(a, 122)
    assert info == 31


def test_real_by_complex_division_and_as_written_mode():
    """div(7, 1 + 2i) = 1.4 - 2.8i (zml's cfloat test).  getrf2 scales a
    column by div(1, pivot): as written (the pivot itself) the complex LU's
    multipliers grow without bound; with the tested quotient it is LAPACK's."""
    lib = ol.load()
    a = np.asfortranarray(np.array([[1 + 2j], [7 + 0j]]))  # pivot 7: the column scales by 1/7
    lu, ipiv, _ = ol.getrf(a)
    assert ipiv[0] == 2 and lu[1, 0] == pytest.approx((1 + 2j) / 7, rel=1e-15)
    b = np.asfortranarray(np.array([[1 + 0j], [3 + 4j]]))  # pivot 3 + 4i (|re| + |im| = 7)
    lu, ipiv, _ = ol.getrf(b)
    assert ipiv[0] == 2 and lu[1, 0] == pytest.approx(0.12 - 0.16j, rel=1e-15)  # 1 / (3 + 4i)
    lib.zo_set_cdiv_as_written(1)
    try:
        lu_w, _, _ = ol.getrf(b)
        assert lu_w[1, 0] == 3 + 4j  # scaled by the pivot itself
        big = cgaussian(150, seed=1)
        lu_w, _, _ = ol.getrf(big)
        assert not np.isfinite(lu_w).all() or np.abs(np.tril(lu_w, -1)).max() > 1e10
    finally:
        lib.zo_set_cdiv_as_written(0)


def test_zgesv_row_major_and_zposv():
    n = 60
    a = cgaussian(n, seed=21)
    x = cgaussian(n, 2, seed=22)
    ar, br = np.ascontiguousarray(a), np.ascontiguousarray(a @ x)
    ipiv = np.zeros(n, dtype=np.int32)
    assert ol.fn("gesv", np.complex128)(101, n, 2, ol.ptr(ar), n, ol.ptr(ipiv), ol.ptr(br), 2) == 0
    np.testing.assert_allclose(br, x, atol=1e-11)
    h = hpd(n, seed=23)
    hf, bf = np.asfortranarray(h), np.asfortranarray(h @ x)
    assert ol.fn("posv", np.complex128)(102, 122, n, 2, ol.ptr(hf), n, ol.ptr(bf), n) == 0
    np.testing.assert_allclose(bf, x, atol=1e-11)


def test_zpotrs_row_major_ldb_check_as_written():
    """potrs.zig:30 requires ldb >= n whatever the layout, so a row-major
    right-hand side with nrhs < n is rejected (posv.zig:52-62 then reaches
    `catch unreachable`); the oracle returns the same InvalidArgument."""
    n = 8
    h = np.ascontiguousarray(hpd(n, seed=5))
    f = ol.fn("potrf", np.complex128)
    assert f(101, 122, n, ol.ptr(h), n) == 0
    b = np.ascontiguousarray(cgaussian(n, 2, seed=6))
    assert ol.fn("potrs", np.complex128)(101, 122, n, 2, ol.ptr(h), n, ol.ptr(b), 2) == -1


@pytest.mark.parametrize("m,n", [(1, 1), (5, 3), (3, 5), (64, 40), (200, 150), (300, 260)])
def test_zgeqrf_equals_lapack(m, n):
    """zgeqrf (blocked above nx = 128 columns) against scipy's: R, the
    reflectors and tau to rounding; Q formed by LAPACK's zungqr from the
    oracle's output is unitary and Q R = A."""
    a = cgaussian(m, n, seed=m + n)
    qr, tau = ol.geqrf(a)
    qr2, tau2, _, info = lap.zgeqrf(a)
    k = min(m, n)
    scale = np.abs(qr2).max()
    assert np.abs(np.triu(qr) - np.triu(qr2)).max() <= 1e-12 * scale
    assert np.abs(np.tril(qr, -1) - np.tril(qr2, -1)).max() <= 1e-12 * max(1.0, scale)
    np.testing.assert_allclose(tau[:k], tau2[:k], rtol=0, atol=1e-12)
    q, _, _ = lap.zungqr(qr[:, :k], tau[:k], lwork=max(1, 64 * m))
    assert np.abs(q.conj().T @ q - np.eye(k)).max() < 1e-13
    assert np.abs(q @ np.triu(qr[:k, :]) - a).max() < 1e-13 * np.abs(a).max() * m


def test_cgeqrf_single_precision():
    a = cgaussian(90, 60, seed=4, dtype=np.complex64)
    qr, tau = ol.geqrf(a)
    q, _, _ = lap.cungqr(qr[:, :60], tau[:60], lwork=64 * 90)
    assert np.abs(q.conj().T @ q - np.eye(60)).max() < 1e-5


def test_zlarfg_as_written_breaks_householder():
    """larfg scales x by div(1, alpha - beta) (larfg.zig:130-137): with the
    tested quotient H is unitary; as written (the reciprocal of the intended
    value) the reflectors no longer are."""
    lib = ol.load()
    a = cgaussian(40, 30, seed=7)
    qr, tau = ol.geqrf(a)
    q, _, _ = lap.zungqr(qr[:, :30], tau, lwork=64 * 40)
    assert np.abs(q.conj().T @ q - np.eye(30)).max() < 1e-13
    lib.zo_set_cdiv_as_written(1)
    try:
        qw, tw = ol.geqrf(a)
    finally:
        lib.zo_set_cdiv_as_written(0)
    with np.errstate(all="ignore"):
        q2, _, _ = lap.zungqr(qw[:, :30], tw, lwork=64 * 40)
        err = np.abs(q2 @ np.triu(qw[:30, :]) - a).max()
    assert not err <= 1e-3 * np.abs(a).max()  # far off, or not finite at all
