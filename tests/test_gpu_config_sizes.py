"""Parity with the oracle at the workload's own sizes, through the C ABI.

The small-size tests (test_gpu_lapack.py, test_gpu_qr.py) compare every
routine with the oracle; these repeat the comparison on the shapes the
workload names:
  * the CPU case exactly: n = 512, A iid N(0,1) from seed 0, one right-hand
    side b = A x_true, x_true iid U(-1,1); and the SPD case G G^T / 512 + I;
  * the FP64 GPU case at n = 8192: dgetrf on iid N(0,1) and dpotrf on
    G G^T / n + I (the oracle's factors formed by its threaded driver, which
    is bit-identical to the serial restatement);
  * dgeqrf on a 4096 x 512 iid N(0,1) matrix, the 32768 x 4096 shape scaled
    down by 8 in each dimension.
Bars: pivots identical up to the first column whose pivot gap is below 1e-10
(a near-tie that a different summation order may flip), LU factors within
1e-9 max|LU_ref| after it, Cholesky factors within 1e-10 max|L_ref| (the GPU
factors right-looking, zml left-looking: different rounding), QR as
test_gpu_qr.py, and the backward error of each factorization below 8 n u.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lap

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P, chol_backward_error, lu_backward_error

pytestmark = pytest.mark.gpu
EPS = 2.0 ** -53
TIE = 1e-10


def gpu_getrf(a):
    lu = np.array(a, order="F", copy=True)
    n = a.shape[0]
    ipiv = np.zeros(n, dtype=np.int32)
    info = zg.lib().LAPACKE_dgetrf(102, n, n, P(lu), n, P(ipiv))
    return lu, ipiv, info


def compare_lu(a, lu, ipiv, info, threads=None):
    lu_ref, ipiv_ref, info_ref, gap = ol.getrf_mt(a, threads=threads, margins=True)
    assert info == info_ref == 0
    ties = np.flatnonzero(gap < TIE)
    first_tie = int(ties[0]) if ties.size else len(gap)
    np.testing.assert_array_equal(ipiv[:first_tie], ipiv_ref[:first_tie])
    if first_tie == len(gap):
        assert np.abs(lu - lu_ref).max() <= 1e-9 * np.abs(lu_ref).max()
    return lu_ref, ipiv_ref


def test_cpu_case_exact_lu_and_solve():
    n = 512
    rng = np.random.default_rng(0)
    a = np.asfortranarray(rng.standard_normal((n, n)))
    xt = rng.uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    lu, ipiv, info = gpu_getrf(a)
    lu_ref, ipiv_ref = compare_lu(a, lu, ipiv, info)
    x = b.copy(order="F")
    assert zg.lib().LAPACKE_dgetrs(102, b"N", n, 1, P(lu), n, P(ipiv), P(x), n) == 0
    x_ref = ol.getrs(lu_ref, ipiv_ref, b)
    assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max()
    assert lu_backward_error(a, lu, ipiv) < 8


def test_cpu_case_exact_cholesky():
    n = 512
    g = np.random.default_rng(0).standard_normal((n, n))
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    f = a.copy(order="F")
    assert zg.lib().LAPACKE_dpotrf(102, b"L", n, P(f), n) == 0
    fr, info = ol.potrf(a, 122)
    assert info == 0
    np.testing.assert_allclose(np.tril(f), np.tril(fr), rtol=0, atol=1e-12 * np.abs(fr).max())
    assert chol_backward_error(a, f, True) < 8


def test_dgetrf_8192_vs_oracle():
    n = 8192
    a = np.asfortranarray(np.random.default_rng(8192).standard_normal((n, n)))
    lu, ipiv, info = gpu_getrf(a)
    compare_lu(a, lu, ipiv, info)


def test_dpotrf_8192_vs_oracle():
    n = 8192
    g = np.random.default_rng(8193).standard_normal((n, n))
    a = np.asfortranarray(g @ g.T / n + np.eye(n))
    del g
    f = a.copy(order="F")
    assert zg.lib().LAPACKE_dpotrf(102, b"L", n, P(f), n) == 0
    fr, info = ol.potrf_mt(a, 122)
    assert info == 0
    assert np.abs(np.tril(f) - np.tril(fr)).max() <= 1e-10 * np.abs(fr).max()


def test_dgeqrf_4096x512_vs_oracle():
    m, n = 4096, 512
    a = np.asfortranarray(np.random.default_rng(4096).standard_normal((m, n)))
    qr = a.copy(order="F")
    tau = np.zeros(n)
    assert zg.lib().LAPACKE_dgeqrf(102, m, n, P(qr), m, P(tau)) == 0, zg.last_error()
    qr_ref, tau_ref = ol.geqrf(a)
    scale = np.abs(qr_ref).max()
    np.testing.assert_allclose(np.triu(qr), np.triu(qr_ref), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(np.tril(qr, -1), np.tril(qr_ref, -1), rtol=0, atol=1e-10)
    np.testing.assert_allclose(tau, tau_ref[:n], rtol=0, atol=1e-11)
    q = lap.dorgqr(qr.copy(order="F"), tau)[0]
    assert np.linalg.norm(q @ np.triu(qr[:n]) - a) / (np.linalg.norm(a) * m * EPS) < 8
