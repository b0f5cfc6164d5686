"""Host-side checks of the decomposition API (include/zml_linalg.h), no GPU:
argument errors and empty matrices never reach the device."""
import ctypes as C

import numpy as np
import pytest

import zml_gb300 as zg


def test_invalid_arguments():
    L = zg.lib()
    a = np.zeros(16)
    ap = a.ctypes.data_as(C.c_void_p)
    h = C.c_void_p(123)
    E = zg.ERR_INVALID_ARGUMENT
    assert L.zml_plu(103, 4, 4, ap, 4, C.byref(h)) == E and h.value is None
    assert L.zml_plu(102, -1, 4, ap, 4, C.byref(h)) == E
    assert L.zml_plu(102, 4, 4, ap, 3, C.byref(h)) == E
    assert L.zml_plu(101, 4, 5, ap, 4, C.byref(h)) == E
    assert L.zml_plu(102, 4, 4, ap, 4, None) == E
    assert L.zml_llt(102, b"X", 4, ap, 4, C.byref(h)) == E
    assert L.zml_utu(102, b"U", 4, ap, 3, C.byref(h)) == E
    assert L.zml_cholesky(102, b"L", -2, ap, 4, C.byref(h)) == E
    assert L.zml_qr(102, 4, 4, ap, 2, C.byref(h)) == E
    assert L.zml_qr_q(None, 0, None) == E


def test_empty_matrices_make_empty_factors():
    L = zg.lib()
    h = C.c_void_p()
    assert L.zml_plu(102, 0, 3, None, 1, C.byref(h)) == 0 and h.value
    u = L.zml_plu_u(h)
    assert (u.rows, u.cols) == (0, 3)
    assert L.zml_plu_p(h, None) == 0
    L.zml_plu_deinit(h)
    assert L.zml_llt(101, b"L", 0, None, 1, C.byref(h)) == 0
    f = L.zml_chol_factor(h)
    assert (f.rows, f.uplo, f.diag) == (0, 122, 131)
    L.zml_chol_deinit(h)
    assert L.zml_qr(102, 3, 0, None, 3, C.byref(h)) == 0
    q = zg.DMatrix()
    assert L.zml_qr_q(h, zg.QR_FULL, C.byref(q)) == 0
    assert (q.rows, q.cols, q.owns_data) == (3, 3, 1)
    np.testing.assert_array_equal(q.to_numpy(), np.eye(3))  # no reflectors: the identity
    L.zml_dmatrix_deinit(C.byref(q))
    assert q.data is None or not q.data
    L.zml_qr_deinit(h)


def _dm(a, layout=102, uplo=0, diag=0):
    """A zml_dmatrix view of the numpy array a (kept alive by the caller)."""
    m, n = a.shape
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    v = zg.DMatrix()
    v.data = buf.ctypes.data_as(C.POINTER(C.c_double))
    v.rows, v.cols = m, n
    v.ld = max(1, m if layout == 102 else n)
    v.layout, v.uplo, v.diag, v.owns_data = layout, uplo, diag, 0
    return v, buf


def test_matmul_facade_arguments_and_empty_products():
    """The matmul facade's errors (matmul.zig: DimensionMismatch) and products
    with an empty inner dimension, which never reach the GEMM."""
    L = zg.lib()
    a, ka = _dm(np.ones((3, 4)))
    b, kb = _dm(np.ones((5, 2)))
    c = zg.DMatrix()
    assert L.zml_dmatmul(C.byref(a), C.byref(b), C.byref(c)) == zg.ERR_DIMENSION_MISMATCH
    bad, kbad = _dm(np.ones((4, 2)), layout=103)
    assert L.zml_dmatmul(C.byref(a), C.byref(bad), C.byref(c)) == zg.ERR_INVALID_ARGUMENT
    tri, kt = _dm(np.ones((4, 4)), uplo=121, diag=7)
    assert L.zml_dmatmul(C.byref(tri), C.byref(tri), C.byref(c)) == zg.ERR_INVALID_ARGUMENT
    assert L.zml_dmatmul(C.byref(a), C.byref(b), None) == zg.ERR_INVALID_ARGUMENT
    # k = 0: a 3 x 2 zero matrix in a's layout, owned
    e1, k1 = _dm(np.zeros((3, 0)), layout=101)
    e2, k2 = _dm(np.zeros((0, 2)))
    assert L.zml_dmatmul(C.byref(e1), C.byref(e2), C.byref(c)) == 0
    assert (c.rows, c.cols, c.layout, c.owns_data) == (3, 2, 101, 1)
    assert np.array_equal(c.to_numpy(), np.zeros((3, 2)))
    L.zml_dmatrix_deinit(C.byref(c))
    x = np.ones(4)
    y = np.full(3, 7.0)
    assert L.zml_dmatvec(C.byref(a), x.ctypes.data_as(C.c_void_p), 0,
                         y.ctypes.data_as(C.c_void_p), 1) == zg.ERR_INVALID_ARGUMENT
    assert L.zml_dmatvec(C.byref(e1), None, 1, y.ctypes.data_as(C.c_void_p), 1) == 0
    assert np.array_equal(y, np.zeros(3))


def _bk_unpack(L, h, upper, n):
    """(perm, T, D) from a Bunch-Kaufman object through its accessors."""
    pre = "zml_udut_" if upper else "zml_ldlt_"
    perm = np.zeros(n, dtype=np.uint32)
    assert getattr(L, pre + "p")(h, perm.ctypes.data_as(C.c_void_p)) == 0
    m = getattr(L, pre + ("u" if upper else "l"))(h)
    t = m.to_numpy()
    assert m.uplo == (121 if upper else 122) and m.diag == 132 and m.owns_data == 1
    L.zml_dmatrix_deinit(C.byref(m))
    sub, dia, sup = np.zeros(max(1, n - 1)), np.zeros(n), np.zeros(max(1, n - 1))
    assert getattr(L, pre + "d")(h, *(x.ctypes.data_as(C.c_void_p) for x in (sub, dia, sup))) == 0
    D = np.diag(dia) + np.diag(sub[:n - 1], -1) + np.diag(sup[:n - 1], 1)
    return perm, t, D


@pytest.mark.parametrize("layout", [102, 101])
@pytest.mark.parametrize("upper", [False, True])
@pytest.mark.parametrize("n", [1, 2, 7, 40, 150])
def test_bunch_kaufman_accessors_reconstruct(n, upper, layout):
    """LDLT.p / l / d and UDUT.p / u / d (lpermute / lconvert, upermute /
    uconvert) over a dsytrf factor: A(perm, perm) = T D T^T, T unit
    triangular, D block diagonal with the 2x2 blocks ipiv marks."""
    import oracle_lib as ol
    L = zg.lib()
    g = np.random.default_rng(n + 3 * upper).standard_normal((n, n))
    a = (g + g.T) / 2
    f, ipiv, info = ol.sytrf(a, 121 if upper else 122, order=layout)
    assert info == 0
    fc = np.ascontiguousarray(f) if layout == 101 else np.asfortranarray(f)
    h = C.c_void_p()
    init = L.zml_udut_init if upper else L.zml_ldlt_init
    assert init(layout, n, fc.ctypes.data_as(C.c_void_p), n, ipiv.ctypes.data_as(C.c_void_p),
                C.byref(h)) == 0
    perm, t, D = _bk_unpack(L, h, upper, n)
    got = np.ctypeslib.as_array((L.zml_udut_ipiv if upper else L.zml_ldlt_ipiv)(h), shape=(n,))
    np.testing.assert_array_equal(got, ipiv)
    (L.zml_udut_deinit if upper else L.zml_ldlt_deinit)(h)
    assert sorted(perm.tolist()) == list(range(n))
    np.testing.assert_array_equal(np.diag(t), np.ones(n))
    assert not (np.tril(t, -1) if upper else np.triu(t, 1)).any()
    # 2x2 blocks exactly where ipiv is negative
    assert np.count_nonzero(np.diag(D, -1)) == (ipiv < 0).sum() // 2
    err = np.abs(a[np.ix_(perm, perm)] - t @ D @ t.T).max()
    assert err <= 1e-12 * max(1.0, np.abs(a).max()) * n


def test_bunch_kaufman_facade_arguments():
    L = zg.lib()
    a = np.eye(4)
    ap = a.ctypes.data_as(C.c_void_p)
    h, h2 = C.c_void_p(5), C.c_void_p(6)
    E = zg.ERR_INVALID_ARGUMENT
    assert L.zml_ldlt(102, b"X", 4, ap, 4, C.byref(h)) == E and h.value is None
    assert L.zml_udut(102, b"U", 4, ap, 3, C.byref(h)) == E
    assert L.zml_bunchkaufman(102, b"Q", 4, ap, 4, C.byref(h), C.byref(h2)) == E
    assert L.zml_bunchkaufman(102, b"L", 4, ap, 4, None, C.byref(h2)) == E
    bad = np.array([1, 5, 3, 4], dtype=np.int32)  # row 5 of a 4 x 4 matrix
    assert L.zml_ldlt_init(102, 4, ap, 4, bad.ctypes.data_as(C.c_void_p), C.byref(h)) == E
    last2 = np.array([1, 2, 3, -4], dtype=np.int32)  # a 2x2 block past the last column
    assert L.zml_ldlt_init(102, 4, ap, 4, last2.ctypes.data_as(C.c_void_p), C.byref(h)) == E
    ok = np.arange(1, 5, dtype=np.int32)
    assert L.zml_udut_init(102, 4, ap, 4, ok.ctypes.data_as(C.c_void_p), C.byref(h)) == 0
    # an upper object is not an LDLT
    assert L.zml_ldlt_p(h, np.zeros(4, np.uint32).ctypes.data_as(C.c_void_p)) == E
    assert L.zml_ldlt_l(h).data is None or not bool(L.zml_ldlt_l(h).data)
    L.zml_udut_deinit(h)
    # n = 0: an empty factor, no device work
    assert L.zml_ldlt(102, b"L", 0, None, 1, C.byref(h)) == 0 and h.value
    L.zml_ldlt_deinit(h)
