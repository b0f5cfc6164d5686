"""GPU tests of the decomposition API (include/zml_linalg.h): plu, llt /
utu / cholesky and qr objects against the oracle and their defining
identities (P L U = A, L L^T = A, U^T U = A, Q R = A with Q orthonormal)."""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import gaussian, spd

pytestmark = pytest.mark.gpu
EPS = 2.0 ** -53


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _layout_buf(a, layout):
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    ld = a.shape[0] if layout == 102 else a.shape[1]
    return buf, ld


@pytest.mark.parametrize("m,n", [(200, 150), (150, 200), (300, 300)])
@pytest.mark.parametrize("layout", [101, 102])
def test_plu(m, n, layout):
    L = zg.lib()
    a = gaussian(m, n, seed=m * 7 + n)
    buf, ld = _layout_buf(a, layout)
    h = C.c_void_p()
    assert L.zml_plu(layout, m, n, _ptr(buf), ld, C.byref(h)) == 0, zg.last_error()
    try:
        lo = L.zml_plu_l(h).to_numpy()
        up = L.zml_plu_u(h).to_numpy()
        k = min(m, n)
        assert lo.shape == (m, k) and up.shape == (k, n)
        l_ = np.tril(lo, -1) + np.eye(m, k)
        u_ = np.triu(up)
        perm = np.zeros(m, dtype=np.uint32)
        assert L.zml_plu_p(h, _ptr(perm)) == 0
        lu = l_ @ u_
        # A = P L U: row i of A is row perm[i] of L U
        err = np.linalg.norm(a - lu[perm.astype(int)]) / (np.linalg.norm(a) * max(m, n) * EPS)
        assert err < 20
        # same pivots as the oracle (row-major: the same logical matrix)
        _, ipiv_ref, _ = ol.getrf(a)
        ipiv = np.ctypeslib.as_array(L.zml_plu_ipiv(h), shape=(k,))
        assert np.array_equal(ipiv, ipiv_ref[:k])
        # the input is untouched
        assert np.array_equal(buf, np.array(a, order="F" if layout == 102 else "C"))
    finally:
        L.zml_plu_deinit(h)


def test_plu_singular_is_an_error():
    L = zg.lib()
    a = gaussian(50, seed=1)
    a[:, 7] = 0.0
    buf = np.asfortranarray(a)
    h = C.c_void_p(1)
    assert L.zml_plu(102, 50, 50, _ptr(buf), 50, C.byref(h)) == zg.ERR_SINGULAR_MATRIX
    assert not h.value


@pytest.mark.parametrize("fn,uplo,layout", [("zml_llt", b"L", 102), ("zml_llt", b"U", 101),
                                            ("zml_utu", b"U", 102), ("zml_utu", b"L", 101),
                                            ("zml_cholesky", b"L", 101),
                                            ("zml_cholesky", b"U", 102)])
def test_cholesky_objects(fn, uplo, layout):
    L = zg.lib()
    n = 257
    a = spd(n, seed=3)
    stored = np.tril(a) if uplo == b"L" else np.triu(a)
    stored = stored + (np.triu(np.full((n, n), 7.0), 1) if uplo == b"L" else
                       np.tril(np.full((n, n), 7.0), -1))   # garbage in the unread triangle
    buf, ld = _layout_buf(stored, layout)
    h = C.c_void_p()
    assert getattr(L, fn)(layout, uplo, n, _ptr(buf), ld, C.byref(h)) == 0, zg.last_error()
    try:
        f = L.zml_chol_factor(h)
        lower = fn == "zml_llt" or (fn == "zml_cholesky" and uplo == b"L")
        assert f.uplo == (122 if lower else 121) and f.diag == 131
        t = f.to_numpy()
        t = np.tril(t) if lower else np.triu(t)
        rec = t @ t.T if lower else t.T @ t
        assert np.linalg.norm(rec - a) / (np.linalg.norm(a) * n * EPS) < 10
        ref, _ = ol.potrf(a, 122 if lower else 121)
        ref = np.tril(ref) if lower else np.triu(ref)
        np.testing.assert_allclose(t, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    finally:
        L.zml_chol_deinit(h)


def test_cholesky_not_spd_is_an_error():
    L = zg.lib()
    a = spd(40, seed=2)
    a[10, 10] = -5.0
    buf = np.asfortranarray(a)
    h = C.c_void_p()
    assert L.zml_llt(102, b"L", 40, _ptr(buf), 40, C.byref(h)) == zg.ERR_SINGULAR_MATRIX
    assert not h.value


@pytest.mark.parametrize("m,n", [(300, 200), (200, 300), (256, 256)])
@pytest.mark.parametrize("layout", [101, 102])
def test_qr_objects(m, n, layout):
    L = zg.lib()
    a = gaussian(m, n, seed=m + n)
    buf, ld = _layout_buf(a, layout)
    h = C.c_void_p()
    assert L.zml_qr(layout, m, n, _ptr(buf), ld, C.byref(h)) == 0, zg.last_error()
    try:
        k = min(m, n)
        qr_ref, tau_ref = ol.geqrf(a)
        tau = np.ctypeslib.as_array(L.zml_qr_tau(h), shape=(k,))
        np.testing.assert_allclose(tau, tau_ref[:k], rtol=0, atol=1e-11)
        for mode, qcols, rrows in ((zg.QR_FULL, m, m), (zg.QR_ECONOMICAL, k, k)):
            q = zg.DMatrix()
            assert L.zml_qr_q(h, mode, C.byref(q)) == 0, zg.last_error()
            Q = q.to_numpy()
            L.zml_dmatrix_deinit(C.byref(q))
            r = L.zml_qr_r(h, mode)
            assert (r.rows, r.cols, r.uplo) == (rrows, n, 121)
            R = np.triu(r.to_numpy())
            assert Q.shape == (m, qcols)
            assert np.linalg.norm(Q.T @ Q - np.eye(qcols)) < 20 * m * EPS
            assert np.linalg.norm(Q @ R[:qcols] - a) / (np.linalg.norm(a) * m * EPS) < 10
            np.testing.assert_allclose(R[:k], np.triu(qr_ref[:k]), rtol=0,
                                       atol=1e-11 * np.abs(qr_ref).max())
    finally:
        L.zml_qr_deinit(h)


def _view(a, layout, uplo=0, diag=0):
    buf, ld = _layout_buf(a, layout)
    v = zg.DMatrix()
    v.data = buf.ctypes.data_as(C.POINTER(C.c_double))
    v.rows, v.cols = a.shape
    v.ld = max(1, ld)
    v.layout, v.uplo, v.diag, v.owns_data = layout, uplo, diag, 0
    return v, buf


def _dense(a, uplo, diag):
    if uplo == 0:
        return a
    t = np.triu(a) if uplo == 121 else np.tril(a)
    if diag == 132:
        np.fill_diagonal(t, 1.0)
    return t


@pytest.mark.parametrize("la,lb", [(102, 102), (101, 101), (102, 101), (101, 102)])
@pytest.mark.parametrize("m,k,n", [(150, 90, 70), (64, 257, 33)])
def test_matmul_facade_general(la, lb, m, k, n):
    """c = a b (matmul/dgedge.zig): result in a's layout, any layout of b."""
    L = zg.lib()
    a, b = gaussian(m, k, seed=1), gaussian(k, n, seed=2)
    va, ka = _view(a, la)
    vb, kb = _view(b, lb)
    c = zg.DMatrix()
    assert L.zml_dmatmul(C.byref(va), C.byref(vb), C.byref(c)) == 0
    assert (c.rows, c.cols, c.layout, c.owns_data) == (m, n, la, 1)
    ref = a @ b
    np.testing.assert_allclose(c.to_numpy(), ref, rtol=0, atol=8 * k * EPS * np.abs(a).max() * np.abs(b).max())
    L.zml_dmatrix_deinit(C.byref(c))


@pytest.mark.parametrize("uplo,diag", [(121, 131), (122, 132)])
def test_matmul_facade_triangular_views(uplo, diag):
    """Triangular views multiply as the dense matrices they stand for."""
    L = zg.lib()
    n = 96
    a, b = gaussian(n, seed=3), gaussian(n, 40, seed=4)
    va, ka = _view(a, 101, uplo, diag)
    vb, kb = _view(b, 102)
    c = zg.DMatrix()
    assert L.zml_dmatmul(C.byref(va), C.byref(vb), C.byref(c)) == 0
    np.testing.assert_allclose(c.to_numpy(), _dense(a, uplo, diag) @ b, rtol=0, atol=1e-12)
    L.zml_dmatrix_deinit(C.byref(c))
    # and on the right
    vt, kt = _view(a, 102, uplo, diag)
    vg, kg = _view(gaussian(30, n, seed=5), 101)
    assert L.zml_dmatmul(C.byref(vg), C.byref(vt), C.byref(c)) == 0
    np.testing.assert_allclose(c.to_numpy(), gaussian(30, n, seed=5) @ _dense(a, uplo, diag),
                               rtol=0, atol=1e-12)
    L.zml_dmatrix_deinit(C.byref(c))


@pytest.mark.parametrize("layout", [101, 102])
def test_matvec_and_vecmat_facade(layout):
    """y = a x (dgedv.zig) and y = x^T a (dvdge.zig), with strides."""
    L = zg.lib()
    m, n = 120, 77
    a = gaussian(m, n, seed=6)
    va, ka = _view(a, layout)
    x = np.random.default_rng(7).standard_normal(2 * n)
    y = np.zeros(3 * m)
    assert L.zml_dmatvec(C.byref(va), _ptr(x), 2, _ptr(y), 3) == 0
    np.testing.assert_allclose(y[::3], a @ x[::2], rtol=0, atol=1e-12)
    xv = np.random.default_rng(8).standard_normal(m)
    yv = np.zeros(n)
    assert L.zml_dvecmat(_ptr(xv), -1, C.byref(va), _ptr(yv), 1) == 0
    np.testing.assert_allclose(yv, xv[::-1] @ a, rtol=0, atol=1e-12)
