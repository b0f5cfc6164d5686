"""LAPACK-level checks of the oracle (CPU only).

zml ships no tests for getrf/getrs/potrf/potrs/geqrf, so these routines are
pinned by (a) normwise backward error bounds and (b) an independent
cross-check against scipy's bundled LAPACK (same algorithm family, partial
pivoting with the first-maximum rule, so pivots agree on inputs without
near-ties).
"""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.linalg.lapack as lap

import oracle_lib as ol

EPS = 2.0 ** -53


def gaussian(n, m=None, seed=0):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((n, m or n)))


@pytest.mark.parametrize("n", [1, 2, 3, 17, 63, 64, 65, 130, 200])
def test_getrf_backward_error_and_scipy_pivots(n):
    a = gaussian(n, seed=n)
    lu, ipiv, info = ol.getrf(a)
    assert info == 0
    L = np.tril(lu, -1) + np.eye(n)
    U = np.triu(lu)
    P = np.eye(n)
    for i, p in enumerate(ipiv):
        P[[i, p - 1]] = P[[p - 1, i]]
    err = np.linalg.norm(P @ a - L @ U) / (np.linalg.norm(a) * n * EPS)
    assert err < 10
    lu2, piv2, info2 = lap.dgetrf(a)
    np.testing.assert_array_equal(ipiv, piv2 + 1)
    np.testing.assert_allclose(lu, lu2, rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("m,n", [(50, 30), (30, 50), (129, 70), (70, 129)])
def test_getrf_rectangular(m, n):
    a = gaussian(m, n, seed=m + n)
    lu, ipiv, info = ol.getrf(a)
    lu2, piv2, _ = lap.dgetrf(a)
    np.testing.assert_array_equal(ipiv, piv2 + 1)
    np.testing.assert_allclose(lu, lu2, rtol=1e-9, atol=1e-11)


def test_getrf_row_major_equals_col_major_of_same_matrix():
    a = gaussian(100, seed=3)
    lu_c, ip_c, _ = ol.getrf(a, order=102)
    lu_r, ip_r, _ = ol.getrf(np.ascontiguousarray(a), order=101)
    np.testing.assert_array_equal(ip_c, ip_r)
    np.testing.assert_array_equal(lu_c, lu_r)  # same operations, same order


def test_getrf_singular_info():
    a = gaussian(70, seed=5)
    a[:, 10] = 0.0
    _, _, info = ol.getrf(a)
    assert info == 11
    z = np.zeros((5, 5), order="F")
    _, ipiv, info = ol.getrf(z)
    assert info == 1 and list(ipiv) == [1, 2, 3, 4, 5]


@pytest.mark.parametrize("trans", [111, 112])
def test_getrs(trans):
    n, nrhs = 150, 4
    a = gaussian(n, seed=7)
    x = np.random.default_rng(8).uniform(-1, 1, (n, nrhs))
    b = (a if trans == 111 else a.T) @ x
    lu, ipiv, _ = ol.getrf(a)
    got = ol.getrs(lu, ipiv, b, trans)
    np.testing.assert_allclose(got, x, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("n", [1, 5, 64, 65, 150])
@pytest.mark.parametrize("uplo", [121, 122])
def test_potrf_potrs(n, uplo):
    g = gaussian(n, seed=n)
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    f, info = ol.potrf(a, uplo)
    assert info == 0
    ref = sla.cholesky(a, lower=(uplo == 122))
    tri = np.tril(f) if uplo == 122 else np.triu(f)
    np.testing.assert_allclose(tri, ref, rtol=1e-10, atol=1e-12)
    x = np.random.default_rng(1).uniform(-1, 1, (n, 3))
    got = ol.potrs(f, a @ x, uplo)
    np.testing.assert_allclose(got, x, rtol=1e-8, atol=1e-9)


def test_potrf_not_positive_definite_info():
    n = 100
    g = gaussian(n, seed=2)
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    a[70, 70] = -1.0
    _, info = ol.potrf(a)
    assert 0 < info <= 71


@pytest.mark.parametrize("m,n", [(10, 10), (200, 150), (300, 200), (150, 200), (513, 260)])
def test_geqrf_against_scipy(m, n):
    a = gaussian(m, n, seed=m)
    qr, tau = ol.geqrf(a)
    qr2, tau2, _, _ = lap.dgeqrf(a)
    np.testing.assert_allclose(np.triu(qr), np.triu(qr2), rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(tau[: min(m, n)], tau2, rtol=1e-8, atol=1e-10)
    # backward error of A = Q R with Q formed by scipy from our reflectors
    q = lap.dorgqr(qr[:, : min(m, n)].copy(order="F"), tau[: min(m, n)])[0]
    err = np.linalg.norm(q @ np.triu(qr[: min(m, n)]) - a) / (np.linalg.norm(a) * m * EPS)
    assert err < 10


@pytest.mark.parametrize("m,n,full", [(10, 10, False), (300, 200, False), (300, 200, True),
                                      (513, 260, False), (160, 160, False), (200, 64, True)])
def test_orgqr_against_scipy(m, n, full):
    """orgqr.zig/org2r.zig restatement: the explicit Q of geqrf's reflectors
    equals LAPACK's dorgqr and Q R reproduces A."""
    a = gaussian(m, n, seed=m + n)
    qr, tau = ol.geqrf(a)
    k = min(m, n)
    ncols = m if full else k
    q = ol.orgqr(qr, tau[:k], ncols)
    src = np.zeros((m, ncols), order="F")
    src[:, :k] = qr[:, :k]
    q2 = lap.dorgqr(src, tau[:k], lwork=max(1, ncols) * 64)[0]
    np.testing.assert_allclose(q, q2, rtol=1e-9, atol=1e-12)
    assert np.linalg.norm(q.T @ q - np.eye(ncols)) < 50 * m * EPS
    err = np.linalg.norm(q[:, :k] @ np.triu(qr[:k]) - a) / (np.linalg.norm(a) * m * EPS)
    assert err < 10


def test_ilaenv_orgqr_block_sizes():
    lib = ol.load()
    assert lib.zo_ilaenv(1, b"DORGQR", 100, 100, 100, -1) == 32
    assert lib.zo_ilaenv(2, b"DORGQR", 100, 100, 100, -1) == 2
    assert lib.zo_ilaenv(3, b"DORGQR", 100, 100, 100, -1) == 128


# ---- the threaded drivers used by the parity tests at the workload's sizes ----

@pytest.mark.parametrize("m,n,threads", [(700, 700, 4), (513, 300, 3), (200, 450, 7),
                                         (64, 64, 2), (65, 65, 5)])
def test_getrf_mt_equals_serial(m, n, threads):
    a = gaussian(m, n, seed=m + n)
    a[:, 37 % n] = 0.0  # a zero column: info and the skipped scaling
    lu, ipiv, info = ol.getrf(a)
    lu2, ipiv2, info2, gap = ol.getrf_mt(a, threads=threads, margins=True)
    assert info2 == info
    np.testing.assert_array_equal(ipiv2, ipiv)
    np.testing.assert_array_equal(lu2, lu)
    # one candidate left (the last row): no tie possible, the gap stays inf
    assert gap.shape == (min(m, n),) and np.all(gap >= 0)
    assert np.all((gap <= 1) | np.isinf(gap))


def test_getrf_mt_margins_match_numpy_replay():
    import gpu_util
    a = gaussian(150, seed=9)
    _, _, _, gap = ol.getrf_mt(a, threads=3, margins=True)
    ref = gpu_util.pivot_margins(a)
    np.testing.assert_allclose(gap[:-1], ref[:-1], rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n,threads", [(700, 4), (65, 3), (129, 16)])
def test_potrf_mt_equals_serial(uplo, n, threads):
    g = gaussian(n, seed=n)
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    f, info = ol.potrf(a, uplo)
    f2, info2 = ol.potrf_mt(a, uplo, threads=threads)
    assert info2 == info == 0
    np.testing.assert_array_equal(f2, f)
    a[90 % n, 90 % n] = -1.0  # a non-positive minor: same info
    assert ol.potrf_mt(a, uplo, threads=threads)[1] == ol.potrf(a, uplo)[1]
