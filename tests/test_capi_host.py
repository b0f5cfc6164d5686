"""Host-side checks of the C ABI (no GPU needed).

The library must load, export every symbol include/*.h declares, and apply
LAPACKE's argument checks (return -index) before touching the device.
"""
import ctypes as C

import numpy as np
import pytest

import zml_gb300 as zg


def test_library_exports_every_declared_symbol():
    L = zg.lib()
    names = zg.declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.zml_gpu_version() >= 1


@pytest.mark.parametrize("call,expect", [
    (lambda L, a, p: L.LAPACKE_dgetrf(103, 4, 4, a, 4, p), -1),
    (lambda L, a, p: L.LAPACKE_dgetrf(102, -1, 4, a, 4, p), -2),
    (lambda L, a, p: L.LAPACKE_dgetrf(102, 4, -1, a, 4, p), -3),
    (lambda L, a, p: L.LAPACKE_dgetrf(102, 4, 4, a, 3, p), -5),
    (lambda L, a, p: L.LAPACKE_dgetrf(101, 4, 5, a, 4, p), -5),
    (lambda L, a, p: L.LAPACKE_dgetrs(102, b"X", 4, 1, a, 4, p, a, 4), -2),
    (lambda L, a, p: L.LAPACKE_dgetrs(102, b"N", 4, 1, a, 3, p, a, 4), -6),
    (lambda L, a, p: L.LAPACKE_dgetrs(101, b"N", 4, 2, a, 4, p, a, 1), -9),
    (lambda L, a, p: L.LAPACKE_dpotrf(102, b"Q", 4, a, 4), -2),
    (lambda L, a, p: L.LAPACKE_dpotrf(102, b"L", -2, a, 4), -3),
    (lambda L, a, p: L.LAPACKE_dposv(102, b"L", 4, 1, a, 4, a, 2), -8),
    (lambda L, a, p: L.LAPACKE_dgesv(102, 4, -1, a, 4, p, a, 4), -3),
    (lambda L, a, p: L.zml_gpu_dgetrf(4, 4, a, 2, p, None, None), -4),
])
def test_lapacke_argument_checks(call, expect):
    L = zg.lib()
    a = np.zeros(64)
    p = np.zeros(8, dtype=np.int32)
    assert call(L, a.ctypes.data_as(C.c_void_p), p.ctypes.data_as(C.c_void_p)) == expect


def test_quick_returns_touch_nothing():
    L = zg.lib()
    a = np.arange(4.0)
    p = np.zeros(2, dtype=np.int32)
    ap, pp = a.ctypes.data_as(C.c_void_p), p.ctypes.data_as(C.c_void_p)
    assert L.LAPACKE_dgetrf(102, 0, 5, ap, 1, pp) == 0
    assert L.LAPACKE_dpotrf(102, b"U", 0, ap, 1) == 0
    assert L.LAPACKE_dgesv(102, 4, 0, ap, 4, pp, ap, 4) == 0
    # cblas: invalid arguments return silently (zml swallows the error)
    L.cblas_dgemm(102, 111, 111, -1, 2, 2, 1.0, ap, 1, ap, 1, 0.0, ap, 1)
    L.cblas_dtrsm(102, 999, 121, 111, 131, 2, 2, 1.0, ap, 2, ap, 2)
    L.cblas_dsyrk(102, 121, 113, 2, 2, 1.0, ap, 2, 0.0, ap, 2)  # conj_trans rejected
    assert list(a) == [0.0, 1.0, 2.0, 3.0]
