"""GPU parity for getrf/getrs/gesv and potrf/potrs/posv through the C ABI.

Against the oracle (the restated zml Zig code) on the same seeded inputs:
  * pivots identical up to the first near-tie column (relative pivot gap
    below 1e-10, where a different summation order may legitimately flip
    the choice; seeded Gaussian inputs have none at these sizes);
  * factors within  |LU_gpu - LU_ref| <= 1e-9 * max|LU_ref|;
  * normwise backward error ||PA-LU||/(||A|| n u) below 8, and never more
    than 4x the oracle's own.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import (P, chol_backward_error, gaussian, lu_backward_error, pivot_margins, spd)

pytestmark = pytest.mark.gpu

FACTOR_RTOL = 1e-9


def gpu_getrf(a, layout=102, lda=None):
    a = np.array(a, dtype=np.float64, order="F" if layout == 102 else "C", copy=True)
    m, n = a.shape
    ld = lda or (m if layout == 102 else n)
    if lda:
        pad = np.zeros((ld, n) if layout == 102 else (m, ld))
        pad[:m, :n] = a
        buf = np.asarray(pad, order="F" if layout == 102 else "C")
    else:
        buf = a
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    info = zg.lib().LAPACKE_dgetrf(layout, m, n, P(buf), ld, P(ipiv))
    return np.array(buf[:m, :n], order="F"), ipiv, info


def check_lu(a, lu, ipiv, info):
    lu_ref, ipiv_ref, info_ref = ol.getrf(a)
    assert info == info_ref
    gaps = pivot_margins(a)
    first_tie = int(np.argmax(gaps < 1e-10)) if (gaps < 1e-10).any() else len(gaps)
    np.testing.assert_array_equal(ipiv[:first_tie], ipiv_ref[:first_tie])
    if first_tie == len(gaps):
        scale = np.abs(lu_ref).max()
        assert np.abs(lu - lu_ref).max() <= FACTOR_RTOL * scale
    be, be_ref = lu_backward_error(a, lu, ipiv), lu_backward_error(a, lu_ref, ipiv_ref)
    assert be < 8 and be <= 4 * be_ref + 1


@pytest.mark.parametrize("n", [1, 2, 3, 17, 63, 64, 65, 128, 200, 513])
def test_dgetrf_square(n):
    a = gaussian(n, seed=100 + n)
    lu, ipiv, info = gpu_getrf(a)
    check_lu(a, lu, ipiv, info)


@pytest.mark.parametrize("m,n", [(300, 200), (200, 300), (1, 50), (50, 1), (129, 64)])
def test_dgetrf_rectangular(m, n):
    a = gaussian(m, n, seed=m * n)
    lu, ipiv, info = gpu_getrf(a)
    check_lu(a, lu, ipiv, info)


@pytest.mark.parametrize("m,n", [(2600, 2100), (2100, 2600)])
def test_dgetrf_rectangular_slice_path(m, n):
    """Rectangular, with a ragged last block, at sizes where the trailing
    updates run as exact slices on the tensor cores (min(m, n) >= 2048) and
    the lookahead splits each update into the next block's columns and the
    rest on two streams."""
    a = gaussian(m, n, seed=m + n)
    lu, ipiv, info = gpu_getrf(a)
    check_lu(a, lu, ipiv, info)


def test_dgetrf_padded_lda_and_row_major():
    a = gaussian(150, seed=9)
    lu, ipiv, info = gpu_getrf(a, lda=173)
    check_lu(a, lu, ipiv, info)
    lu_r, ipiv_r, info_r = gpu_getrf(a, layout=101)
    np.testing.assert_array_equal(ipiv_r, ipiv)
    np.testing.assert_allclose(lu_r, lu, rtol=0, atol=1e-12 * np.abs(lu).max())


def test_dgetrf_singular_and_nan_info():
    a = gaussian(100, seed=11)
    a[:, 37] = 0.0
    lu, ipiv, info = gpu_getrf(a)
    _, _, info_ref = ol.getrf(a)
    assert info == info_ref == 38
    z = np.zeros((70, 70), order="F")
    lu, ipiv, info = gpu_getrf(z)
    assert info == 1 and list(ipiv) == list(range(1, 71))
    b = gaussian(80, seed=12)
    b[5, 5] = np.nan
    lu, ipiv, info = gpu_getrf(b)
    lu_ref, ipiv_ref, _ = ol.getrf(b)
    np.testing.assert_array_equal(ipiv[:5], ipiv_ref[:5])


def test_dgetrf_ties_pick_lowest_row():
    """iamax semantics: equal magnitudes -> the first (lowest) row wins."""
    n = 96
    a = np.asfortranarray(np.ones((n, n)) + np.diag(np.arange(n) * 0.0))
    a[:, 0] = 1.0
    a[50, 0] = -1.0
    lu, ipiv, info = gpu_getrf(a)
    _, ipiv_ref, info_ref = ol.getrf(a)
    assert ipiv[0] == ipiv_ref[0] == 1
    assert info == info_ref


@pytest.mark.parametrize("trans", [b"N", b"T"])
@pytest.mark.parametrize("nrhs", [1, 4, 64])
def test_dgetrs_vs_oracle(trans, nrhs):
    n = 300
    a = gaussian(n, seed=21)
    x = np.random.default_rng(22).uniform(-1, 1, (n, nrhs))
    b = np.asfortranarray((a if trans == b"N" else a.T) @ x)
    lu, ipiv, info = gpu_getrf(a)
    bg = b.copy(order="F")
    assert zg.lib().LAPACKE_dgetrs(102, trans, n, nrhs, P(lu), n, P(ipiv), P(bg), n) == 0
    lu_ref, ipiv_ref, _ = ol.getrf(a)
    br = ol.getrs(lu_ref, ipiv_ref, b, 111 if trans == b"N" else 112)
    np.testing.assert_allclose(bg, br, rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(bg, x, rtol=1e-8, atol=1e-9)


@pytest.mark.parametrize("trans", [b"N", b"T"])
@pytest.mark.parametrize("n,nrhs", [(512, 1), (641, 3), (1300, 1), (2100, 4)])
def test_dgetrs_one_launch_solves_vs_oracle(n, nrhs, trans):
    """Up to four right-hand sides with n >= 512 take the one-launch triangular
    solves (blocks of 128 rows; n = 641, 1300 and 2100 end on a ragged block);
    leading dimensions larger than n on the device."""
    import torch
    a = gaussian(n, seed=n)
    x = np.random.default_rng(n + 1).uniform(-1, 1, (n, nrhs))
    b = (a if trans == b"N" else a.T) @ x
    lda, ldb = n + 3, n + 5
    da = torch.zeros((n, lda), dtype=torch.float64)
    da[:, :n] = torch.from_numpy(a.T.copy())
    da = da.cuda()
    db = torch.zeros((nrhs, ldb), dtype=torch.float64)
    db[:, :n] = torch.from_numpy(b.T.copy())
    db = db.cuda()
    dp = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = np.zeros(1, dtype=np.int32)
    L = zg.lib()
    assert L.zml_gpu_dgetrf(n, n, da.data_ptr(), lda, dp.data_ptr(), P(info), None) == 0
    assert info[0] == 0
    assert L.zml_gpu_dgetrs(trans, n, nrhs, da.data_ptr(), lda, dp.data_ptr(), db.data_ptr(), ldb,
                            None) == 0
    lu = np.asfortranarray(da.cpu().numpy()[:, :n].T)
    ipiv = dp.cpu().numpy()
    br = ol.getrs(lu, ipiv, np.asfortranarray(b), 111 if trans == b"N" else 112)
    xg = db.cpu().numpy()[:, :n].T
    np.testing.assert_allclose(xg, br, rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(xg, x, rtol=1e-7, atol=1e-8)
    # the padding between columns is untouched
    assert not db.cpu().numpy()[:, n:].any()


def test_dgesv_row_major():
    n, nrhs = 200, 3
    a = gaussian(n, seed=31)
    x = np.random.default_rng(32).uniform(-1, 1, (n, nrhs))
    b = a @ x
    ar = np.ascontiguousarray(a)
    br = np.ascontiguousarray(b)
    ipiv = np.zeros(n, dtype=np.int32)
    assert zg.lib().LAPACKE_dgesv(101, n, nrhs, P(ar), n, P(ipiv), P(br), nrhs) == 0
    np.testing.assert_allclose(br, x, rtol=1e-8, atol=1e-9)


def test_dgetrf_2048_vs_oracle():
    a = gaussian(2048, seed=2048)
    lu, ipiv, info = gpu_getrf(a)
    check_lu(a, lu, ipiv, info)


@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("n", [1, 7, 64, 65, 200, 700, 2600])  # 2600: slice updates, ragged
def test_dpotrf_vs_oracle(uplo, n):
    a = spd(n, seed=n)
    f = a.copy(order="F")
    info = zg.lib().LAPACKE_dpotrf(102, uplo, n, P(f), n)
    ul = 122 if uplo == b"L" else 121
    fr, info_ref = ol.potrf(a, ul)
    assert info == info_ref == 0
    tri = np.tril if uplo == b"L" else np.triu
    np.testing.assert_allclose(tri(f), tri(fr), rtol=0, atol=1e-12 * np.abs(fr).max())
    # the other triangle is untouched
    other = np.triu(a, 1) if uplo == b"L" else np.tril(a, -1)
    np.testing.assert_array_equal((np.triu(f, 1) if uplo == b"L" else np.tril(f, -1)), other)
    assert chol_backward_error(a, f, uplo == b"L") < 8


def test_dpotrf_not_spd_info():
    n = 300
    a = spd(n, seed=5)
    a[200, 200] = -5.0
    f = a.copy(order="F")
    info = zg.lib().LAPACKE_dpotrf(102, b"L", n, P(f), n)
    _, info_ref = ol.potrf(a, 122)
    assert info == info_ref == 201


@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("nrhs", [1, 4, 64])
def test_dposv_and_potrs(uplo, nrhs):
    n = 257
    a = spd(n, seed=77)
    x = np.random.default_rng(78).uniform(-1, 1, (n, nrhs))
    b = np.asfortranarray(a @ x)
    f, bg = a.copy(order="F"), b.copy(order="F")
    assert zg.lib().LAPACKE_dposv(102, uplo, n, nrhs, P(f), n, P(bg), n) == 0
    ul = 122 if uplo == b"L" else 121
    fr, _ = ol.potrf(a, ul)
    br = ol.potrs(fr, b, ul)
    np.testing.assert_allclose(bg, br, rtol=1e-10, atol=1e-11)
    b2 = b.copy(order="F")
    assert zg.lib().LAPACKE_dpotrs(102, uplo, n, nrhs, P(f), n, P(b2), n) == 0
    np.testing.assert_allclose(b2, bg, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("n,nrhs", [(512, 2), (1300, 1), (2100, 4)])
def test_dpotrs_one_launch_solves_vs_oracle(uplo, n, nrhs):
    """potrs with up to four right-hand sides and n >= 512 (the one-launch
    solves: L then L^T, or U^T then U, the transposed triangle walked along
    A's columns), leading dimension larger than n; the other triangle holds
    NaNs that must not be read."""
    a = spd(n, seed=n + 5)
    x = np.random.default_rng(n + 6).uniform(-1, 1, (n, nrhs))
    b = a @ x
    lda = n + 3
    f = np.zeros((lda, n), order="F")
    f[:n, :] = a
    assert zg.lib().LAPACKE_dpotrf(102, uplo, n, P(f), lda) == 0
    ul = 122 if uplo == b"L" else 121
    fr, _ = ol.potrf(a, ul)
    other = np.triu_indices(n, 1) if uplo == b"L" else np.tril_indices(n, -1)
    fn = f.copy(order="F")
    fn[other] = np.nan
    bg = np.asfortranarray(b.copy())
    assert zg.lib().LAPACKE_dpotrs(102, uplo, n, nrhs, P(fn), lda, P(bg), n) == 0
    br = ol.potrs(fr, b, ul)
    np.testing.assert_allclose(bg, br, rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(bg, x, rtol=1e-7, atol=1e-8)


def test_device_pointer_getrf_getrs():
    import torch
    n, nrhs = 1000, 2
    a = gaussian(n, seed=41)
    x = np.random.default_rng(42).uniform(-1, 1, (n, nrhs))
    b = a @ x
    da = torch.from_numpy(a.T.copy()).cuda()  # column-major a
    db = torch.from_numpy(np.asfortranarray(b).T.copy()).cuda()
    dp = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = np.zeros(1, dtype=np.int32)
    L = zg.lib()
    assert L.zml_gpu_dgetrf(n, n, da.data_ptr(), n, dp.data_ptr(), P(info), None) == 0
    assert info[0] == 0
    assert L.zml_gpu_dgetrs(b"N", n, nrhs, da.data_ptr(), n, dp.data_ptr(), db.data_ptr(), n, None) == 0
    np.testing.assert_allclose(db.cpu().numpy().T, x, rtol=1e-8, atol=1e-9)


@pytest.mark.parametrize("k1,k2,incx", [(1, 64, 1), (1, 64, -1), (5, 300, 1), (3, 700, -1)])
def test_dlaswp_vs_oracle(k1, k2, incx):
    """Random pivots with repeated targets, forward and backward order, and
    ranges longer than one composed chunk."""
    m, n = 800, 77
    rng = np.random.default_rng(k2)
    a = np.asfortranarray(rng.standard_normal((m, n)))
    ipiv = rng.integers(1, m + 1, size=m).astype(np.int32)
    ipiv[10:20] = 400  # the same target row, many times
    ref, got = a.copy(order="F"), a.copy(order="F")
    assert ol.fn("laswp")(102, n, P(ref), m, k1, k2, P(ipiv), incx) == 0
    assert zg.lib().LAPACKE_dlaswp(102, n, P(got), m, k1, k2, P(ipiv), incx) == 0
    np.testing.assert_array_equal(got, ref)
