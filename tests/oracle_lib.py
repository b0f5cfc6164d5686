"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: the oracle restates zml's Zig loop nests in C and is the
parity reference for every GPU routine.  Only tests, smoke() and bench.py's
CPU-baseline leg load it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

_lib = None

i32, f64, f32, vp = C.c_int, C.c_double, C.c_float, C.c_void_p


class CF64(C.Structure):
    """zo_cf64: a complex128 scalar passed by value."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class CF32(C.Structure):
    """zo_cf32: a complex64 scalar passed by value."""
    _fields_ = [("re", C.c_float), ("im", C.c_float)]


def cs(x, dtype=np.complex128):
    """A Python / numpy number as the complex scalar struct of `dtype`."""
    x = complex(x)
    return (CF64 if np.dtype(dtype) == np.complex128 else CF32)(x.real, x.imag)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        _lib = C.CDLL(LIB_PATH)
        for pfx, T in (("zo_d_", f64), ("zo_s_", f32)):
            sig = {
                "gemm": (i32, [i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32, T, vp, i32]),
                "trsm": (i32, [i32, i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32]),
                "trmm": (i32, [i32, i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32]),
                "syrk": (i32, [i32, i32, i32, i32, i32, T, vp, i32, T, vp, i32]),
                "gemv": (i32, [i32, i32, i32, i32, T, vp, i32, vp, i32, T, vp, i32]),
                "ger": (i32, [i32, i32, i32, T, vp, i32, vp, i32, vp, i32]),
                "iamax": (i32, [i32, vp, i32]),
                "scal": (i32, [i32, T, vp, i32]),
                "nrm2": (T, [i32, vp, i32]),
                "lamch": (T, [C.c_char]),
                "laswp": (i32, [i32, i32, vp, i32, i32, i32, vp, i32]),
                "getrf2": (i32, [i32, i32, i32, vp, i32, vp]),
                "getrf": (i32, [i32, i32, i32, vp, i32, vp]),
                "getrs": (i32, [i32, i32, i32, i32, vp, i32, vp, vp, i32]),
                "gesv": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
                "potrf2": (i32, [i32, i32, i32, vp, i32]),
                "potrf": (i32, [i32, i32, i32, vp, i32]),
                "potrs": (i32, [i32, i32, i32, i32, vp, i32, vp, i32]),
                "posv": (i32, [i32, i32, i32, i32, vp, i32, vp, i32]),
                "geqr2": (i32, [i32, i32, i32, vp, i32, vp, vp]),
                "geqrf": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
                "orgqr": (i32, [i32, i32, i32, i32, vp, i32, vp, vp, i32]),
                "org2r": (i32, [i32, i32, i32, i32, vp, i32, vp, vp]),
                "larft": (i32, [i32, i32, i32, i32, i32, vp, i32, vp, vp, i32]),
                "larfg": (i32, [i32, vp, vp, i32, vp]),
                "syr": (i32, [i32, i32, i32, T, vp, i32, vp, i32]),
                "gemmtr": (i32, [i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32, T, vp, i32]),
                "sytf2": (i32, [i32, i32, i32, vp, i32, vp]),
                "lasyf": (i32, [i32, i32, i32, i32, vp, vp, i32, vp, vp, i32]),
                "sytrf": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(_lib, pfx + name)
                fn.restype, fn.argtypes = res, args
        for pfx, Z, R in (("zo_z_", CF64, f64), ("zo_c_", CF32, f32)):
            sig = {
                "gemm": (i32, [i32, i32, i32, i32, i32, i32, Z, vp, i32, vp, i32, Z, vp, i32]),
                "trsm": (i32, [i32, i32, i32, i32, i32, i32, i32, Z, vp, i32, vp, i32]),
                "trmm": (i32, [i32, i32, i32, i32, i32, i32, i32, Z, vp, i32, vp, i32]),
                "syrk": (i32, [i32, i32, i32, i32, i32, Z, vp, i32, Z, vp, i32]),
                "herk": (i32, [i32, i32, i32, i32, i32, R, vp, i32, R, vp, i32]),
                "gemv": (i32, [i32, i32, i32, i32, Z, vp, i32, vp, i32, Z, vp, i32]),
                "geru": (i32, [i32, i32, i32, Z, vp, i32, vp, i32, vp, i32]),
                "gerc": (i32, [i32, i32, i32, Z, vp, i32, vp, i32, vp, i32]),
                "iamax": (i32, [i32, vp, i32]),
                "scal": (i32, [i32, Z, vp, i32]),
                "laswp": (i32, [i32, i32, vp, i32, i32, i32, vp, i32]),
                "getrf2": (i32, [i32, i32, i32, vp, i32, vp]),
                "getrf": (i32, [i32, i32, i32, vp, i32, vp]),
                "getrs": (i32, [i32, i32, i32, i32, vp, i32, vp, vp, i32]),
                "gesv": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
                "potrf2": (i32, [i32, i32, i32, vp, i32]),
                "potrf": (i32, [i32, i32, i32, vp, i32]),
                "potrs": (i32, [i32, i32, i32, i32, vp, i32, vp, i32]),
                "posv": (i32, [i32, i32, i32, i32, vp, i32, vp, i32]),
                "nrm2": (R, [i32, vp, i32]),
                "larfg": (i32, [i32, vp, vp, i32, vp]),
                "geqr2": (i32, [i32, i32, i32, vp, i32, vp, vp]),
                "geqrf": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
                "her": (i32, [i32, i32, i32, R, vp, i32, vp, i32]),
                "hetf2": (i32, [i32, i32, i32, vp, i32, vp]),
                "hetrf": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
                "sytf2": (i32, [i32, i32, i32, vp, i32, vp]),
                "sytrf": (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
            }
            for name, (res, args) in sig.items():
                f = getattr(_lib, pfx + name)
                f.restype, f.argtypes = res, args
        _lib.zo_set_cdiv_as_written.argtypes = [i32]
        _lib.zo_set_trsm_as_written.argtypes = [i32]
        _lib.zo_ilaenv.argtypes = [i32, C.c_char_p, i32, i32, i32, i32]
        _lib.zo_ilaenv.restype = i32
    return _lib


def ptr(a):
    return a.ctypes.data_as(vp) if a is not None else None


PREFIX = {np.dtype(np.float64): "zo_d_", np.dtype(np.float32): "zo_s_",
          np.dtype(np.complex128): "zo_z_", np.dtype(np.complex64): "zo_c_"}


def fn(name, dtype=np.float64):
    return getattr(load(), PREFIX[np.dtype(dtype)] + name)


# ---- numpy-level conveniences (column-major, Fortran-ordered arrays) --------

def getrf(a, order=102):
    """LU of a copy of `a` (F-ordered for col-major); returns (lu, ipiv, info)."""
    a = np.array(a, dtype=a.dtype, order="F" if order == 102 else "C", copy=True)
    m, n = a.shape
    lda = m if order == 102 else n
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    info = fn("getrf", a.dtype)(order, m, n, ptr(a), max(1, lda), ptr(ipiv))
    return a, ipiv, info


def getrf_mt(a, threads=None, margins=False):
    """The oracle's getrf of a copy of `a` (binary64, column-major) on host
    threads, bit-identical to getrf(); with margins=True also each column's
    pivot gap (top1 - top2) / top1."""
    f = load().zo_d_getrf_mt
    f.restype, f.argtypes = i32, [i32, i32, vp, i32, vp, vp, i32]
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    m, n = a.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    gap = np.full(min(m, n), np.inf) if margins else None
    info = f(m, n, ptr(a), max(1, m), ptr(ipiv), ptr(gap), threads or os.cpu_count() or 1)
    return (a, ipiv, info, gap) if margins else (a, ipiv, info)


def potrf_mt(a, uplo=122, threads=None):
    """The oracle's potrf (binary64, column-major) on host threads,
    bit-identical to potrf()."""
    f = load().zo_d_potrf_mt
    f.restype, f.argtypes = i32, [i32, i32, vp, i32, i32]
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    n = a.shape[0]
    info = f(uplo, n, ptr(a), max(1, n), threads or os.cpu_count() or 1)
    return a, info


def getrs(lu, ipiv, b, trans=111):
    b = np.array(b, dtype=lu.dtype, order="F", copy=True)
    if b.ndim == 1:
        b = b.reshape(-1, 1, order="F")
    n, nrhs = b.shape
    r = fn("getrs", lu.dtype)(102, trans, n, nrhs, ptr(lu), max(1, n), ptr(ipiv), ptr(b), max(1, n))
    assert r == 0
    return b


def potrf(a, uplo=122):
    a = np.array(a, dtype=a.dtype, order="F", copy=True)
    n = a.shape[0]
    info = fn("potrf", a.dtype)(102, uplo, n, ptr(a), max(1, n))
    return a, info


def potrs(l, b, uplo=122):
    b = np.array(b, dtype=l.dtype, order="F", copy=True)
    if b.ndim == 1:
        b = b.reshape(-1, 1, order="F")
    n, nrhs = b.shape
    r = fn("potrs", l.dtype)(102, uplo, n, nrhs, ptr(l), max(1, n), ptr(b), max(1, n))
    assert r == 0
    return b


def sytrf(a, uplo=122, order=102):
    """Bunch-Kaufman factorization of a copy of symmetric `a` (its `uplo`
    triangle, real or complex, no conjugation); returns (factor, ipiv, info)
    in LAPACK's dsytrf / zsytrf conventions."""
    a = np.array(a, dtype=a.dtype, order="F" if order == 102 else "C", copy=True)
    n = a.shape[0]
    ipiv = np.zeros(n, dtype=np.int32)
    f = fn("sytrf", a.dtype)
    q = np.zeros(1, dtype=a.dtype)
    assert f(order, uplo, n, ptr(a), max(1, n), ptr(ipiv), ptr(q), -1) == 0
    work = np.zeros(max(1, int(np.real(q[0]))), dtype=a.dtype)
    info = f(order, uplo, n, ptr(a), max(1, n), ptr(ipiv), ptr(work), work.size)
    return a, ipiv, info


def geqrf(a):
    a = np.array(a, dtype=a.dtype, order="F", copy=True)
    m, n = a.shape
    tau = np.zeros(max(1, min(m, n)), dtype=a.dtype)
    q = np.zeros(1, dtype=a.dtype)
    f = fn("geqrf", a.dtype)
    assert f(102, m, n, ptr(a), max(1, m), ptr(tau), ptr(q), -1) == 0
    lwork = max(1, int(np.real(q[0])))
    work = np.zeros(lwork, dtype=a.dtype)
    r = f(102, m, n, ptr(a), max(1, m), ptr(tau), ptr(work), lwork)
    assert r == 0
    return a, tau


def orgqr(qr, tau, ncols=None):
    """The first ncols columns of Q from geqrf's output (qr, tau)."""
    m, n = qr.shape
    k = min(m, n)
    ncols = k if ncols is None else ncols
    q = np.zeros((m, ncols), dtype=qr.dtype, order="F")
    q[:, :min(n, ncols)] = qr[:, :min(n, ncols)]
    f = fn("orgqr", qr.dtype)
    w = np.zeros(1, dtype=qr.dtype)
    assert f(102, m, ncols, k, ptr(q), max(1, m), ptr(tau), ptr(w), -1) == 0
    lwork = max(1, int(np.real(w[0])))
    work = np.zeros(lwork, dtype=qr.dtype)
    assert f(102, m, ncols, k, ptr(q), max(1, m), ptr(tau), ptr(work), lwork) == 0
    return q
