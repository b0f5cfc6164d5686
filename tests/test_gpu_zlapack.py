"""GPU parity for the complex triangular solve, LU and Cholesky through the
C ABI (cblas_ztrsm, LAPACKE_z{getrf,getrs,gesv,potrf,potrs,posv} and the
single-precision c forms) against the complex oracle.

The GPU keeps the reference's structure (blocked getrf over recursive getrf2
panels, left-looking potrf over recursive potrf2), so on inputs without
near-ties the pivots are the oracle's; factors agree to 1e-9 of their scale
(the level-3 products sum in another order), solutions to the conditioning.
zml's cf64 trsm chain (tests/golden/blas_ztrsm.json) is replayed through
cblas_ztrsm within its own 1e-7 bounds.  Where zml expects an exact 0 from
a cancellation its loop order makes exact, the blocked GPU solve (substitution
on diagonal blocks, GEMM updates) may leave an ulp-level residue (one of the
2,560 expectations: -5.6e-17); those zeros are met within 1e-13 of the
array's largest entry.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from golden_replay import load_fixture, replay
from gpu_util import P

pytestmark = pytest.mark.gpu


def cmat(shape, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    return np.asfortranarray((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype))


def hpd(n, seed, dtype=np.complex128):
    g = cmat((n, n), seed)
    return np.asfortranarray((g @ g.conj().T / n + np.eye(n)).astype(dtype))


def scal(x, dtype=np.complex128):
    return np.array([x.real, x.imag], dtype=np.float64 if dtype == np.complex128 else np.float32)


def test_reference_ztrsm_fixture_through_cblas():
    def call(name, args):
        keep, conv = [], []
        for a in args:
            if isinstance(a, np.ndarray):
                conv.append(P(a))
            elif isinstance(a, complex):
                v = scal(a)
                keep.append(v)
                conv.append(P(v))
            else:
                conv.append(a)
        zg.lib().cblas_ztrsm(*conv)
    fx = load_fixture("ztrsm")
    for st in fx["steps"]:  # alpha by pointer
        if st["op"] == "call" and not isinstance(st["args"][7], dict):
            st["args"][7] = {"c": [float(st["args"][7]), 0.0]}
    checked, failures = replay(fx, call, zero_rtol=1e-13)
    assert checked > 0
    assert not failures, failures[:5]


@pytest.mark.parametrize("side", [141, 142])
@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("ta", [111, 112, 113, 114])
@pytest.mark.parametrize("diag", [131, 132])
def test_ztrsm_vs_oracle(side, uplo, ta, diag):
    m, n = 150, 37
    na = m if side == 141 else n
    a = np.asfortranarray(cmat((na, na), seed=side + uplo + ta + diag) + 4 * np.eye(na))
    b = cmat((m, n), seed=ta * diag)
    alpha = 0.5 - 1j
    br, bg = b.copy(order="F"), b.copy(order="F")
    assert ol.fn("trsm", np.complex128)(102, side, uplo, ta, diag, m, n, ol.cs(alpha), ol.ptr(a),
                                        na, ol.ptr(br), m) == 0
    zg.lib().cblas_ztrsm(102, side, uplo, ta, diag, m, n, P(scal(alpha)), P(a), na, P(bg), m)
    assert np.abs(bg - br).max() <= 1e-11 * np.abs(br).max()


def test_ztrsm_row_major_matches_column_major():
    m, n = 70, 20
    a = np.asfortranarray(cmat((m, m), seed=3) + 4 * np.eye(m))
    b = cmat((m, n), seed=4)
    bc = b.copy(order="F")
    zg.lib().cblas_ztrsm(102, 141, 122, 113, 131, m, n, P(scal(1 + 0j)), P(a), m, P(bc), m)
    ar, br = np.ascontiguousarray(a), np.ascontiguousarray(b)
    zg.lib().cblas_ztrsm(101, 141, 122, 113, 131, m, n, P(scal(1 + 0j)), P(ar), m, P(br), n)
    np.testing.assert_allclose(br, bc, rtol=1e-12, atol=1e-12)


def zgetrf_gpu(a, dtype=np.complex128, layout=102):
    m, n = a.shape
    buf = np.array(a, dtype=dtype, order="F" if layout == 102 else "C", copy=True)
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    f = zg.lib().LAPACKE_zgetrf if dtype == np.complex128 else zg.lib().LAPACKE_cgetrf
    info = f(layout, m, n, P(buf), m if layout == 102 else n, P(ipiv))
    return buf, ipiv, info


@pytest.mark.parametrize("m,n", [(1, 1), (1, 7), (7, 1), (65, 65), (200, 200), (300, 180),
                                 (130, 260)])
def test_zgetrf_vs_oracle(m, n):
    a = cmat((m, n), seed=m * 3 + n)
    lu, ipiv, info = zgetrf_gpu(a)
    lur, ipr, infr = ol.getrf(a)
    assert info == infr == 0
    np.testing.assert_array_equal(ipiv, ipr)
    assert np.abs(lu - lur).max() <= 1e-9 * max(1.0, np.abs(lur).max())


def test_zgetrf_row_major_and_singular_info():
    a = cmat((90, 90), seed=8)
    lc, pc, _ = zgetrf_gpu(a)
    lr, pr, _ = zgetrf_gpu(a, layout=101)
    np.testing.assert_array_equal(pc, pr)
    np.testing.assert_allclose(lr, lc, rtol=0, atol=1e-12 * np.abs(lc).max())
    s = a.copy(order="F")
    s[:, 41] = 0
    _, _, info = zgetrf_gpu(s)
    assert info == ol.getrf(s)[2] == 42


@pytest.mark.parametrize("trans", [b"N", b"T", b"C"])
def test_zgetrs_vs_oracle(trans):
    n, nrhs = 180, 3
    a = cmat((n, n), seed=21)
    x = cmat((n, nrhs), seed=22)
    op = {b"N": a, b"T": a.T, b"C": a.conj().T}[trans]
    b = np.asfortranarray(op @ x)
    lu, ipiv, _ = zgetrf_gpu(a)
    bg = b.copy(order="F")
    assert zg.lib().LAPACKE_zgetrs(102, trans, n, nrhs, P(lu), n, P(ipiv), P(bg), n) == 0
    lur, ipr, _ = ol.getrf(a)
    br = ol.getrs(lur, ipr, b, {b"N": 111, b"T": 112, b"C": 113}[trans])
    np.testing.assert_allclose(bg, br, rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(bg, x, rtol=1e-8, atol=1e-9)


def test_zgesv_row_major_and_cgesv():
    n, nrhs = 120, 2
    a = cmat((n, n), seed=31)
    x = cmat((n, nrhs), seed=32)
    ar, br = np.ascontiguousarray(a), np.ascontiguousarray(a @ x)
    ipiv = np.zeros(n, dtype=np.int32)
    assert zg.lib().LAPACKE_zgesv(101, n, nrhs, P(ar), n, P(ipiv), P(br), nrhs) == 0
    np.testing.assert_allclose(br, x, rtol=1e-9, atol=1e-10)
    a32 = a.astype(np.complex64)
    b32 = np.asfortranarray((a @ x).astype(np.complex64))
    assert zg.lib().LAPACKE_cgesv(102, n, nrhs, P(a32), n, P(ipiv), P(b32), n) == 0
    assert np.abs(b32 - x).max() <= 1e-3 * np.abs(x).max()


@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("n", [1, 5, 64, 65, 200])
def test_zpotrf_vs_oracle(uplo, n):
    a = hpd(n, seed=n)
    f = a.copy(order="F")
    info = zg.lib().LAPACKE_zpotrf(102, uplo, n, P(f), n)
    ul = 122 if uplo == b"L" else 121
    fr, infr = ol.potrf(a, ul)
    assert info == infr == 0
    tri = np.tril if uplo == b"L" else np.triu
    assert np.abs(tri(f) - tri(fr)).max() <= 1e-12 * np.abs(fr).max()
    assert not np.diag(f).imag.any()
    np.testing.assert_array_equal(f - tri(f), a - tri(a))  # the other triangle untouched


def test_zpotrf_not_positive_definite_info():
    a = hpd(100, seed=2)
    a[70, 70] = -4.0
    f = a.copy(order="F")
    assert zg.lib().LAPACKE_zpotrf(102, b"L", 100, P(f), 100) == ol.potrf(a, 122)[1] == 71


@pytest.mark.parametrize("uplo", [b"L", b"U"])
def test_zpotrs_zposv(uplo):
    n, nrhs = 150, 3
    a = hpd(n, seed=77)
    x = cmat((n, nrhs), seed=78)
    b = np.asfortranarray(a @ x)
    f, bg = a.copy(order="F"), b.copy(order="F")
    assert zg.lib().LAPACKE_zposv(102, uplo, n, nrhs, P(f), n, P(bg), n) == 0
    ul = 122 if uplo == b"L" else 121
    fr, _ = ol.potrf(a, ul)
    br = ol.potrs(fr, b, ul)
    np.testing.assert_allclose(bg, br, rtol=1e-10, atol=1e-11)
    b2 = b.copy(order="F")
    assert zg.lib().LAPACKE_zpotrs(102, uplo, n, nrhs, P(f), n, P(b2), n) == 0
    np.testing.assert_allclose(b2, bg, rtol=1e-12, atol=1e-12)


def test_cpotrf_single_precision():
    n = 90
    a = hpd(n, seed=9).astype(np.complex64)
    f = a.copy(order="F")
    assert zg.lib().LAPACKE_cpotrf(102, b"L", n, P(f), n) == 0
    L = np.tril(f).astype(np.complex128)
    assert np.abs(L @ L.conj().T - a).max() <= 1e-4 * np.abs(a).max()
