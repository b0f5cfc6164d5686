"""Host-side checks of the decomposition API (include/zml_linalg.h), no GPU:
argument errors and empty matrices never reach the device."""
import ctypes as C

import numpy as np

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
