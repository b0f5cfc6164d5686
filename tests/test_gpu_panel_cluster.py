"""FP32 LU panels factored by one thread-block cluster, through LAPACKE_sgetrf.

An m x n FP32 matrix with n <= 128 is one panel; wider matrices run it once
per 128-column block.  Against the oracle's sgetrf on the same inputs:
  * pivots identical up to the first near-tie column (relative gap between
    the two largest candidates below 1e-4, where FP32 summation order may
    flip the choice);
  * factors within 5e-4 * max|LU_ref| while no tie came first;
  * normwise backward error ||PA-LU||/(||A|| max(m,n) u32) below 8 and never
    above 4x the oracle's own;
  * info (first zero pivot) identical, ties resolved to the lowest row.
Panel heights cover one CTA, a partly filled last CTA, thread counts that are
not multiples of 64, 16 CTAs of 2 rows a thread and the 4-rows-a-thread
layout (m > 16384); widths cover 32-column
sub-panels and ragged last sub-panels.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P, perm_from_ipiv, pivot_margins

pytestmark = pytest.mark.gpu

EPS32 = 2.0 ** -24
TIE = 1e-4
FACTOR_RTOL = 5e-4


def gpu_sgetrf(a):
    buf = np.array(a, dtype=np.float32, order="F", copy=True)
    m, n = buf.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    info = zg.lib().LAPACKE_sgetrf(102, m, n, P(buf), m, P(ipiv))
    return buf, ipiv, info


def backward_error(a, lu, ipiv):
    a = a.astype(np.float64)
    lu = lu.astype(np.float64)
    m, n = a.shape
    k = min(m, n)
    L = np.tril(lu[:, :k], -1) + np.eye(m, k)
    U = np.triu(lu[:k, :])
    pa = a[perm_from_ipiv(ipiv, m)]
    return np.linalg.norm(pa - L @ U) / (np.linalg.norm(a) * max(m, n) * EPS32)


def check(a):
    lu, ipiv, info = gpu_sgetrf(a)
    lu_ref, ipiv_ref, info_ref = ol.getrf(np.asfortranarray(a.astype(np.float32)))
    assert info == info_ref
    gaps = pivot_margins(a.astype(np.float64))
    tied = gaps < TIE
    first_tie = int(np.argmax(tied)) if tied.any() else len(gaps)
    np.testing.assert_array_equal(ipiv[:first_tie], ipiv_ref[:first_tie])
    if first_tie == len(gaps) and np.isfinite(lu_ref).all():
        scale = np.abs(lu_ref).max()
        assert np.abs(lu.astype(np.float64) - lu_ref).max() <= FACTOR_RTOL * scale
    if np.isfinite(a).all() and info == 0:
        be, be_ref = backward_error(a, lu, ipiv), backward_error(a, lu_ref, ipiv_ref)
        assert be < 8 and be <= 4 * be_ref + 1, (be, be_ref)
    return lu, ipiv, info


def gauss32(m, n, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32))


@pytest.mark.parametrize("m,n", [(128, 128), (700, 128), (1024, 128), (1025, 128), (2500, 128), (2600, 96),
                                 (5000, 128), (16384, 128), (20000, 128), (32768, 128),
                                 (3000, 100), (3000, 77), (2048, 1), (4096, 33)])
def test_panel_vs_oracle(m, n):
    check(gauss32(m, n, seed=m + n))


@pytest.mark.parametrize("n", [300, 1000, 2048])
def test_square_sgetrf_vs_oracle(n):
    check(gauss32(n, n, seed=7 * n))


def test_zero_column_sets_info_and_keeps_going():
    a = gauss32(3000, 128, seed=5)
    a[:, 40] = 0.0
    a[:, 90] = 0.0
    lu, ipiv, info = check(a)
    assert info == 41


def test_ties_pick_lowest_row():
    a = gauss32(5000, 64, seed=9)
    a[:, 0] = 1.0          # every row ties in column 0
    a[4000, 1] = 1e6       # a decisive pivot for column 1, far down (CTA 3)
    lu, ipiv, info = check(a)
    assert ipiv[0] == 1
    assert ipiv[1] == 4001


def test_pivot_row_in_every_cta():
    """Column k's largest entry planted in a different 1024-row block each time."""
    m, n = 16384, 64
    a = gauss32(m, n, seed=11)
    for k in range(n):
        a[(k % 16) * 1024 + 37 + k, k] = 1e4 * (1 + k)
    check(a)


def test_nan_below_diagonal_is_never_the_pivot():
    a = gauss32(2000, 32, seed=13)
    a[1500, 0] = np.nan
    lu, ipiv, info = gpu_sgetrf(a)
    _, ipiv_ref, info_ref = ol.getrf(a)
    assert ipiv[0] == ipiv_ref[0] != 1501
    assert info == info_ref
