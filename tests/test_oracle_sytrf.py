"""Bunch-Kaufman (sytrf / lasyf / sytf2) of the oracle (CPU only).

zml has no sytrf tests and its routines restate LAPACK's dsytrf / dlasyf /
dsytf2 (lapack/sytrf.zig, lasyf.zig, sytf2.zig), so the oracle is pinned
against scipy's bundled LAPACK running the same algorithm: identical ipiv
(the 1x1 / 2x2 pivot blocks and interchanges) and factors to rounding, below
(unblocked) and above (blocked, nb = 64) the block size, both triangles; and
the factors solve A x = b through LAPACK's own dsytrs.  The Hermitian form is
pinned the same way against zhetrf: hetf2 alone (which zhetrf runs itself up
to nb = 64 columns, and which solves through zhetrs beyond), and the blocked
hetrf over lahef at every size.  Complex symmetric matrices (no conjugation)
go through the same sytrf over cfloat and are pinned against zsytrf / csytrf.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lap

import oracle_lib as ol


def sym(n, seed, dtype=np.float64):
    g = np.random.default_rng(seed).standard_normal((n, n))
    return np.asfortranarray(((g + g.T) / 2).astype(dtype))


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n", [1, 2, 5, 33, 64, 65, 150])
def test_dsytrf_equals_lapack(n, uplo):
    a = sym(n, seed=n + uplo)
    f, ipiv, info = ol.sytrf(a, uplo)
    ldu, ipiv2, info2 = lap.dsytrf(a, lower=int(uplo == 122))
    assert info == info2 == 0
    np.testing.assert_array_equal(ipiv, ipiv2)
    tri = np.triu if uplo == 121 else np.tril
    assert np.abs(tri(f) - tri(ldu)).max() <= 1e-10 * max(1.0, np.abs(ldu).max())
    # the factorization solves A x = b with LAPACK's own dsytrs
    x = np.random.default_rng(n).standard_normal((n, 2))
    sol, inf = lap.dsytrs(f, ipiv, a @ x, lower=int(uplo == 122))
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-8, atol=1e-8)


def test_ssytrf_equals_lapack():
    a = sym(100, seed=3, dtype=np.float32)
    f, ipiv, info = ol.sytrf(a, 122)
    ldu, ipiv2, _ = lap.ssytrf(a, lower=1)
    np.testing.assert_array_equal(ipiv, ipiv2)
    assert np.abs(np.tril(f) - np.tril(ldu)).max() <= 1e-3 * np.abs(ldu).max()


def test_dsytrf_row_major_same_pivots():
    a = sym(90, seed=11)
    fc, pc, _ = ol.sytrf(a, 121)
    fr, pr, _ = ol.sytrf(a, 121, order=101)
    np.testing.assert_array_equal(pc, pr)
    np.testing.assert_allclose(np.triu(fr), np.triu(fc), rtol=0, atol=1e-11 * np.abs(fc).max())


def test_dsytrf_zero_column_info():
    a = sym(40, seed=5)
    a[17, :] = 0
    a[:, 17] = 0
    _, _, info = ol.sytrf(a, 122)
    _, _, info2 = lap.dsytrf(a, lower=1)
    assert info == info2 > 0


def test_ilaenv_sytrf():
    lib = ol.load()
    assert lib.zo_ilaenv(1, b"DSYTRF", 500, -1, -1, -1) == 64
    assert lib.zo_ilaenv(2, b"DSYTRF", 500, -1, -1, -1) == 8


def herm(n, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return np.asfortranarray((g + g.conj().T) / 2)


def zhetf2(a, uplo):
    f = a.copy(order="F")
    ipiv = np.zeros(a.shape[0], dtype=np.int32)
    info = ol.fn("hetf2", np.complex128)(102, uplo, a.shape[0], ol.ptr(f), max(1, a.shape[0]),
                                         ol.ptr(ipiv))
    return f, ipiv, info


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n", [1, 2, 5, 20, 64])
def test_zhetf2_equals_lapack_zhetrf(n, uplo):
    a = herm(n, seed=n + uplo)
    f, ipiv, info = zhetf2(a, uplo)
    ldu, ipiv2, info2 = lap.zhetrf(a, lower=int(uplo == 122))
    assert info == info2 == 0
    np.testing.assert_array_equal(ipiv, ipiv2)
    tri = np.triu if uplo == 121 else np.tril
    assert np.abs(tri(f) - tri(ldu)).max() <= 1e-11 * max(1.0, np.abs(ldu).max())
    assert not np.diag(f).imag.any()


@pytest.mark.parametrize("uplo", [121, 122])
def test_zhetf2_solves_through_zhetrs(uplo):
    n = 150
    a = herm(n, seed=uplo)
    f, ipiv, info = zhetf2(a, uplo)
    assert info == 0
    x = np.random.default_rng(2).standard_normal((n, 2)) + 0j
    sol, inf = lap.zhetrs(f, ipiv, a @ x, lower=int(uplo == 122))
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-9, atol=1e-9)


def zhetrf(a, uplo, order=102):
    n = a.shape[0]
    f = a.copy(order="F") if order == 102 else a.copy(order="C")
    ipiv = np.zeros(n, dtype=np.int32)
    lw = max(1, n * 64)
    work = np.zeros(lw, dtype=np.complex128)
    info = ol.fn("hetrf", np.complex128)(order, uplo, n, ol.ptr(f), max(1, n), ol.ptr(ipiv),
                                         ol.ptr(work), lw)
    return f, ipiv, info


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n", [1, 20, 64, 65, 150, 200])
def test_zhetrf_blocked_equals_lapack(n, uplo):
    """hetrf over lahef (nb = 64 columns a block) against LAPACK's zhetrf,
    which runs zlahef the same way: identical pivots, factors to rounding."""
    a = herm(n, seed=7 * n + uplo)
    f, ipiv, info = zhetrf(a, uplo)
    ldu, ipiv2, info2 = lap.zhetrf(a, lower=int(uplo == 122))
    assert info == info2 == 0
    np.testing.assert_array_equal(ipiv, ipiv2)
    tri = np.triu if uplo == 121 else np.tril
    assert np.abs(tri(f) - tri(ldu)).max() <= 1e-10 * max(1.0, np.abs(ldu).max())
    x = np.random.default_rng(n).standard_normal((n, 2)) + 0j
    sol, inf = lap.zhetrs(f, ipiv, a @ x, lower=int(uplo == 122))
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-8, atol=1e-8)


def test_zhetrf_row_major_same_pivots():
    a = herm(130, seed=4)
    fc, pc, _ = zhetrf(a, 122)
    fr, pr, _ = zhetrf(a, 122, order=101)
    np.testing.assert_array_equal(pc, pr)
    np.testing.assert_allclose(np.tril(fr), np.tril(fc), rtol=0, atol=1e-11 * np.abs(fc).max())


def test_zhetrf_zero_column_info():
    a = herm(100, seed=9)
    a[70, :] = 0
    a[:, 70] = 0
    _, _, info = zhetrf(a, 121)
    _, _, info2 = lap.zhetrf(a, lower=0)
    assert info == info2 > 0


def test_ilaenv_hetrf():
    assert ol.load().zo_ilaenv(1, b"CHETRF", 500, -1, -1, -1) == 64


def test_zhetrf_as_written_quotient_breaks_the_factor():
    """lahef's 2x2 step computes d21 = t / d21, a real by complex quotient;
    zml's cfloat returns y / x for it, and with that the blocked factor of a
    150 x 150 Hermitian matrix no longer solves (a zero pivot appears)."""
    a = herm(150, seed=1)
    lib = ol.load()
    lib.zo_set_cdiv_as_written(1)
    try:
        f, ipiv, info = zhetrf(a, 122)
    finally:
        lib.zo_set_cdiv_as_written(0)
    x = np.ones((150, 1)) + 0j
    sol, _ = lap.zhetrs(f, ipiv, a @ x, lower=1)
    assert info > 0 or not np.allclose(sol, x)


def csym(n, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return np.asfortranarray(((g + g.T) / 2).astype(dtype))


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("n", [1, 2, 5, 64, 65, 150])
def test_zsytrf_equals_lapack(n, uplo):
    """Complex symmetric (not Hermitian) Bunch-Kaufman: the same sytrf /
    lasyf / sytf2 over cfloat, against LAPACK's zsytrf."""
    a = csym(n, seed=3 * n + uplo)
    f, ipiv, info = ol.sytrf(a, uplo)
    ldu, ipiv2, info2 = lap.zsytrf(a, lower=int(uplo == 122))
    assert info == info2 == 0
    np.testing.assert_array_equal(ipiv, ipiv2)
    tri = np.triu if uplo == 121 else np.tril
    assert np.abs(tri(f) - tri(ldu)).max() <= 1e-10 * max(1.0, np.abs(ldu).max())
    x = np.random.default_rng(n).standard_normal((n, 2)) + 0j
    sol, inf = lap.zsytrs(f, ipiv, a @ x, lower=int(uplo == 122))
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-8, atol=1e-8)


def test_csytrf_equals_lapack():
    a = csym(100, seed=8, dtype=np.complex64)
    f, ipiv, _ = ol.sytrf(a, 121)
    ldu, ipiv2, _ = lap.csytrf(a, lower=0)
    np.testing.assert_array_equal(ipiv, ipiv2)
    assert np.abs(np.triu(f) - np.triu(ldu)).max() <= 1e-3 * np.abs(ldu).max()


def test_zsytrf_row_major_same_pivots():
    a = csym(90, seed=12)
    fc, pc, _ = ol.sytrf(a, 121)
    fr, pr, _ = ol.sytrf(a, 121, order=101)
    np.testing.assert_array_equal(pc, pr)
    np.testing.assert_allclose(np.triu(fr), np.triu(fc), rtol=0, atol=1e-11 * np.abs(fc).max())


def test_zsytrf_as_written_quotient_breaks_the_factor():
    """The 1x1 step scales by div(1, a(k,k)) and the 2x2 step forms
    t = div(1, d11 d22 - 1), both real by complex; with zml's cfloat
    quotient as written (y / x) the factor no longer solves."""
    a = csym(80, seed=2)
    lib = ol.load()
    lib.zo_set_cdiv_as_written(1)
    try:
        f, ipiv, info = ol.sytrf(a, 122)
    finally:
        lib.zo_set_cdiv_as_written(0)
    x = np.ones((80, 1)) + 0j
    sol, _ = lap.zsytrs(f, ipiv, a @ x, lower=1)
    assert info > 0 or not np.allclose(sol, x)


@pytest.mark.parametrize("uplo", [121, 122])
def test_zsytrf_zero_column_info(uplo):
    a = csym(100, seed=21)
    a[30, :] = 0
    a[:, 30] = 0
    _, _, info = ol.sytrf(a, uplo)
    _, _, info2 = lap.zsytrf(a, lower=int(uplo == 122))
    assert info == info2 > 0


@pytest.mark.parametrize("name", ["sytrf", "hetrf"])
def test_complex_bunch_kaufman_workspace_query_and_empty(name):
    f = ol.fn(name, np.complex128)
    q = np.zeros(1, dtype=np.complex128)
    ipiv = np.zeros(1, dtype=np.int32)
    a = np.zeros((1, 1), dtype=np.complex128)
    assert f(102, 122, 300, ol.ptr(a), 300, ol.ptr(ipiv), ol.ptr(q), -1) == 0
    assert q[0] == 300 * 64
    assert f(102, 122, 0, ol.ptr(a), 1, ol.ptr(ipiv), ol.ptr(q), 1) == 0
    assert f(102, 122, 5, ol.ptr(a), 4, ol.ptr(ipiv), ol.ptr(q), 1) < 0  # lda < n
