"""Bunch-Kaufman (sytrf / lasyf / sytf2) of the oracle (CPU only).

zml has no sytrf tests and its routines restate LAPACK's dsytrf / dlasyf /
dsytf2 (lapack/sytrf.zig, lasyf.zig, sytf2.zig), so the oracle is pinned
against scipy's bundled LAPACK running the same algorithm: identical ipiv
(the 1x1 / 2x2 pivot blocks and interchanges) and factors to rounding, below
(unblocked) and above (blocked, nb = 64) the block size, both triangles; and
the factors solve A x = b through LAPACK's own dsytrs.
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
