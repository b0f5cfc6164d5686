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


def test_every_declared_function_has_a_ctypes_signature():
    """Without argtypes ctypes passes a Python int as a 32-bit C int, so a
    device pointer given as tensor.data_ptr() would reach the library cut to
    its low 32 bits."""
    missing = [n for n in zg.declared_symbols() if n not in zg._SIGS]
    assert not missing, missing
    L = zg.lib()
    for n in zg.declared_symbols():
        assert getattr(L, n).argtypes is not None, n


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


@pytest.mark.parametrize("call,expect", [
    (lambda L, a, p: L.LAPACKE_zgetrf(103, 4, 4, a, 4, p), -1),
    (lambda L, a, p: L.LAPACKE_zgetrf(102, -1, 4, a, 4, p), -2),
    (lambda L, a, p: L.LAPACKE_zgetrf(102, 4, 4, a, 3, p), -5),
    (lambda L, a, p: L.LAPACKE_cgetrf(101, 4, 5, a, 4, p), -5),
    (lambda L, a, p: L.LAPACKE_zgetrs(102, b"X", 4, 1, a, 4, p, a, 4), -2),
    (lambda L, a, p: L.LAPACKE_zgetrs(102, b"C", 4, 1, a, 3, p, a, 4), -6),
    (lambda L, a, p: L.LAPACKE_zgetrs(101, b"N", 4, 2, a, 4, p, a, 1), -9),
    (lambda L, a, p: L.LAPACKE_zgesv(102, 4, -1, a, 4, p, a, 4), -3),
    (lambda L, a, p: L.LAPACKE_zpotrf(102, b"Q", 4, a, 4), -2),
    (lambda L, a, p: L.LAPACKE_cpotrf(102, b"L", -2, a, 4), -3),
    (lambda L, a, p: L.LAPACKE_zpotrs(102, b"L", 4, -1, a, 4, a, 4), -4),
    (lambda L, a, p: L.LAPACKE_zposv(102, b"L", 4, 1, a, 4, a, 2), -8),
    (lambda L, a, p: L.LAPACKE_dsytrf(103, b"L", 4, a, 4, p), -1),
    (lambda L, a, p: L.LAPACKE_dsytrf(102, b"X", 4, a, 4, p), -2),
    (lambda L, a, p: L.LAPACKE_dsytrf(102, b"U", -1, a, 4, p), -3),
    (lambda L, a, p: L.LAPACKE_ssytrf(102, b"U", 4, a, 3, p), -5),
])
def test_complex_and_sytrf_argument_checks(call, expect):
    """The complex LAPACKE entries and sytrf check their arguments as the real
    ones do, before any device work."""
    L = zg.lib()
    a = np.zeros(128)
    p = np.zeros(8, dtype=np.int32)
    assert call(L, a.ctypes.data_as(C.c_void_p), p.ctypes.data_as(C.c_void_p)) == expect


def test_complex_blas_invalid_arguments_and_quick_returns_touch_nothing():
    """cblas_z* return silently on invalid arguments (zml swallows the error)
    and do nothing for empty products or alpha = 0, beta = 1."""
    L = zg.lib()
    c = np.arange(8.0)  # four complex numbers
    cp = c.ctypes.data_as(C.c_void_p)
    one = np.array([1.0, 0.0]).ctypes.data_as(C.c_void_p)
    zero = np.array([0.0, 0.0]).ctypes.data_as(C.c_void_p)
    L.cblas_zgemm(102, 111, 111, -1, 2, 2, one, cp, 1, cp, 1, zero, cp, 1)   # m < 0
    L.cblas_zgemm(102, 999, 111, 2, 2, 2, one, cp, 2, cp, 2, zero, cp, 2)    # bad transpose
    L.cblas_zgemm(102, 111, 111, 2, 2, 2, zero, cp, 2, cp, 2, one, cp, 2)    # alpha 0, beta 1
    L.cblas_zgemm(102, 111, 111, 0, 2, 2, one, cp, 1, cp, 2, zero, cp, 1)    # m = 0
    L.cblas_zherk(102, 121, 112, 2, 2, 1.0, cp, 2, 0.0, cp, 2)               # trans rejected
    L.cblas_zsyrk(102, 121, 113, 2, 2, one, cp, 2, zero, cp, 2)              # conj_trans rejected
    L.cblas_ztrsm(102, 141, 999, 111, 131, 2, 2, one, cp, 2, cp, 2)          # bad uplo
    L.cblas_zgemm(102, 111, 111, 2, 2, 2, one, cp, 2, cp, 2, None, cp, 2)    # no beta
    assert list(c) == [float(i) for i in range(8)]
