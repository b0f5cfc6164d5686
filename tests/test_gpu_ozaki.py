"""FP64 updates on the tensor cores by exact slices (zml_gpu_dgemm_slices) and
the FP64 LU built on them.

C -= A B is computed from eight 7-bit integer slices of every row of A and
column of B, multiplied in BF16 with FP32 accumulation that is exact where it
matters.  Bar, against numpy's FP64 product: |C - C_ref| <= 32 u (|A| |B| +
|C|) elementwise -- the slices' own error (about 6 u on N(0,1) data) plus
numpy's rounding (a few u), at the worst of up to 17 million entries; an FP64
GEMM's error bound is k u |A| |B| = 256 u.  NaN in a row
of A reaches that row of C; rows and columns of very different scales keep
their relative accuracy; the lower form touches only C's lower triangle.
The LU with these updates (LAPACKE_dgetrf from n = 2048 up) is compared with
the same LU on the FP64 pipe: identical pivots, factors within 1e-9 max|LU| --
the bar of every LU parity test here: rounding differences grow through the
elimination towards U's last rows.  The Cholesky, whose factor does not
amplify them, within 1e-12.
"""
import numpy as np
import pytest

import zml_gb300 as zg
from gpu_util import P, gaussian

pytestmark = pytest.mark.gpu
U = 2.0 ** -53


def dev(a):
    import torch
    return torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()


def host(t):
    return t.cpu().numpy().T


def slices_sub(a, b, c, lower=False):
    m, k = a.shape
    n = c.shape[1]
    da, dc = dev(a), dev(c)
    db = dev(b) if b is not None else None
    rc = zg.lib().zml_gpu_dgemm_slices(m, n, k, da.data_ptr(), m,
                                       db.data_ptr() if db is not None else None, max(1, k),
                                       dc.data_ptr(), m, int(lower), None)
    assert rc == 0, (rc, zg.last_error())
    return host(dc)


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (300, 200, 256), (1000, 777, 100), (4096, 4100, 256),
                                   (129, 4500, 64), (33, 2, 255)])
def test_slices_match_fp64(m, n, k):
    rng = np.random.default_rng(m + n + k)
    a, b, c = rng.standard_normal((m, k)), rng.standard_normal((k, n)), rng.standard_normal((m, n))
    out = slices_sub(a, b, c)
    ref = c - a @ b
    bound = 32 * U * (np.abs(a) @ np.abs(b) + np.abs(c))
    assert np.all(np.abs(out - ref) <= bound), np.max(np.abs(out - ref) / bound)


def test_slices_scaled_rows_and_columns():
    rng = np.random.default_rng(5)
    m, n, k = 200, 150, 256
    ra = 10.0 ** rng.uniform(-150, 150, m)
    cb = 10.0 ** rng.uniform(-150, 150, n)
    a = rng.standard_normal((m, k)) * ra[:, None]
    b = rng.standard_normal((k, n)) * cb[None, :]
    c = np.zeros((m, n))
    out = slices_sub(a, b, c)
    ref = -(a @ b)
    bound = 32 * U * (np.abs(a) @ np.abs(b))
    assert np.all(np.abs(out - ref) <= bound)


def test_slices_nan_and_zero_rows():
    rng = np.random.default_rng(6)
    a, b, c = rng.standard_normal((64, 32)), rng.standard_normal((32, 48)), np.ones((64, 48))
    a[7, 3] = np.nan
    a[9, :] = 0.0
    out = slices_sub(a, b, c)
    assert np.all(np.isnan(out[7]))
    np.testing.assert_array_equal(out[9], c[9])
    ok = np.ones(64, bool)
    ok[7] = False
    assert np.all(np.isfinite(out[ok]))


def test_slices_lower_form():
    rng = np.random.default_rng(7)
    n, k = 4200, 256
    a, c = rng.standard_normal((n, k)), rng.standard_normal((n, n))
    out = slices_sub(a, None, c, lower=True)
    ref = c - a @ a.T
    low = np.tril(np.ones((n, n), bool))
    bound = 32 * U * (np.abs(a) @ np.abs(a).T + np.abs(c))
    assert np.all(np.abs(out - ref)[low] <= bound[low])
    np.testing.assert_array_equal(out[~low], c[~low])


@pytest.mark.parametrize("n", [2048, 3000])
def test_lu_with_slice_updates_matches_fp64_pipe(n):
    a = gaussian(n, seed=n + 1)
    L = zg.lib()
    res = {}
    for mode in (1, 0):
        prev = L.zml_gpu_fp64_updates(mode)
        try:
            lu = a.copy(order="F")
            ipiv = np.zeros(n, dtype=np.int32)
            assert L.LAPACKE_dgetrf(102, n, n, P(lu), n, P(ipiv)) == 0
        finally:
            L.zml_gpu_fp64_updates(prev)
        res[mode] = (lu, ipiv)
    np.testing.assert_array_equal(res[1][1], res[0][1])
    assert np.abs(res[1][0] - res[0][0]).max() <= 1e-9 * np.abs(res[0][0]).max()


@pytest.mark.parametrize("n", [2048, 2600])
def test_cholesky_with_slice_updates_matches_fp64_pipe(n):
    g = gaussian(n, seed=n + 2)
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    L = zg.lib()
    res = {}
    for mode in (1, 0):
        prev = L.zml_gpu_fp64_updates(mode)
        try:
            f = a.copy(order="F")
            assert L.LAPACKE_dpotrf(102, b"L", n, P(f), n) == 0
        finally:
            L.zml_gpu_fp64_updates(prev)
        res[mode] = f
    low = np.tril(np.ones((n, n), bool))
    assert np.abs(res[1] - res[0])[low].max() <= 1e-12 * np.abs(res[0]).max()
    np.testing.assert_array_equal(res[1][~low], a[~low])  # the upper triangle untouched


def test_cholesky_with_slice_updates_reports_non_spd():
    n = 2304
    g = gaussian(n, seed=9)
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    a[2000, 2000] = -50.0
    f = a.copy(order="F")
    assert zg.lib().LAPACKE_dpotrf(102, b"L", n, P(f), n) == 2001
