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
