"""zml_gb300 -- GB300-native dense factor-and-solve behind zml's C ABI.

The product is the shared library zml_gb300/lib/libzml_gb300.so, whose C
entry points are declared in include/cblas.h and include/clapack.h.  This
module is the Python-side loader used by the tests and the benchmark: it
binds every declared entry point through ctypes and fails loudly when the
library has not been built (there is no CPU fallback).
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "lib", "libzml_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ROW_MAJOR, COL_MAJOR = 101, 102
NO_TRANS, TRANS, CONJ_TRANS, CONJ_NO_TRANS = 111, 112, 113, 114
UPPER, LOWER = 121, 122
NON_UNIT, UNIT = 131, 132
LEFT, RIGHT = 141, 142

i32, f64, f32, vp, ch = C.c_int, C.c_double, C.c_float, C.c_void_p, C.c_char

_SIGS = {}
for p, T in (("d", f64), ("s", f32)):
    _SIGS.update({
        "cblas_%sgemm" % p: (None, [i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32, T, vp, i32]),
        "cblas_%ssyrk" % p: (None, [i32, i32, i32, i32, i32, T, vp, i32, T, vp, i32]),
        "cblas_%strsm" % p: (None, [i32, i32, i32, i32, i32, i32, i32, T, vp, i32, vp, i32]),
        "LAPACKE_%sgetrf" % p: (i32, [i32, i32, i32, vp, i32, vp]),
        "LAPACKE_%sgetrs" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, vp, i32]),
        "LAPACKE_%sgesv" % p: (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
        "LAPACKE_%spotrf" % p: (i32, [i32, ch, i32, vp, i32]),
        "LAPACKE_%spotrs" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, i32]),
        "LAPACKE_%sposv" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, i32]),
        "LAPACKE_%slaswp" % p: (i32, [i32, i32, vp, i32, i32, i32, vp, i32]),
        "LAPACKE_%ssytrf" % p: (i32, [i32, ch, i32, vp, i32, vp]),
        "LAPACKE_%sgeqrf" % p: (i32, [i32, i32, i32, vp, i32, vp]),
        "LAPACKE_%sorgqr" % p: (i32, [i32, i32, i32, i32, vp, i32, vp]),
    })
for p, R in (("z", f64), ("c", f32)):  # complex: scalars by pointer, herk's real
    _SIGS.update({
        "cblas_%sgemm" % p: (None, [i32, i32, i32, i32, i32, i32, vp, vp, i32, vp, i32, vp, vp, i32]),
        "cblas_%sherk" % p: (None, [i32, i32, i32, i32, i32, R, vp, i32, R, vp, i32]),
        "cblas_%ssyrk" % p: (None, [i32, i32, i32, i32, i32, vp, vp, i32, vp, vp, i32]),
        "cblas_%strsm" % p: (None, [i32, i32, i32, i32, i32, i32, i32, vp, vp, i32, vp, i32]),
        "LAPACKE_%sgetrf" % p: (i32, [i32, i32, i32, vp, i32, vp]),
        "LAPACKE_%sgetrs" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, vp, i32]),
        "LAPACKE_%sgesv" % p: (i32, [i32, i32, i32, vp, i32, vp, vp, i32]),
        "LAPACKE_%spotrf" % p: (i32, [i32, ch, i32, vp, i32]),
        "LAPACKE_%spotrs" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, i32]),
        "LAPACKE_%sposv" % p: (i32, [i32, ch, i32, i32, vp, i32, vp, i32]),
        "LAPACKE_%sgeqrf" % p: (i32, [i32, i32, i32, vp, i32, vp]),
        "LAPACKE_%ssytrf" % p: (i32, [i32, ch, i32, vp, i32, vp]),
        "LAPACKE_%shetrf" % p: (i32, [i32, ch, i32, vp, i32, vp]),
    })
_SIGS.update({
    "zml_gpu_dgetrf": (i32, [i32, i32, vp, i32, vp, vp, vp]),
    "zml_gpu_dgetrs": (i32, [ch, i32, i32, vp, i32, vp, vp, i32, vp]),
    "zml_gpu_dgetrf_noalloc": (i32, [i32, i32, vp, i32, vp, vp, vp]),
    "zml_gpu_dorgqr": (i32, [i32, i32, i32, vp, i32, vp, vp]),
    "zml_gpu_dgeqrf": (i32, [i32, i32, vp, i32, vp, vp]),
    "zml_gpu_zgeqrf": (i32, [i32, i32, vp, i32, vp, vp]),
    "zml_gpu_dpotrf": (i32, [ch, i32, vp, i32, vp, vp]),
    "zml_gpu_dpotrs": (i32, [ch, i32, i32, vp, i32, vp, i32, vp]),
    "zml_gpu_dgemm": (i32, [i32, i32, i32, i32, i32, f64, vp, i32, vp, i32, f64, vp, i32, vp]),
    "zml_gpu_gemm_lowp": (i32, [i32, i32, i32, i32, f32, vp, i32, vp, i32, f32, vp, i32, vp]),
    "zml_gpu_last_error": (C.c_char_p, []),
    "zml_gpu_set_spin_limit": (i32, [C.c_longlong]),
    "zml_gpu_mixed_panel": (i32, [i32]),
    "zml_gpu_fp64_updates": (i32, [i32]),
    "zml_gpu_panel_rows": (i32, [i32]),
    "zml_gpu_dgemm_slices": (i32, [i32, i32, i32, vp, i32, vp, i32, vp, i32, i32, vp]),
    "zml_gpu_sgetrf_calu": (i32, [i32, i32, vp, i32, vp, vp, vp]),
    "zml_gpu_version": (i32, []),
})



class MpirResult(C.Structure):
    _fields_ = [("info", C.c_int), ("iters", C.c_int), ("inner_iters", C.c_int),
                ("converged", C.c_int), ("switched_f64", C.c_int), ("fp64_fallback", C.c_int),
                ("berr", C.c_double), ("factor_ms", C.c_double),
                ("berr_history", C.c_double * 32)]


_SIGS.update({
    "zml_dgesv_mpir": (i32, [i32, i32, i32, vp, i32, vp, i32, vp, i32, i32, i32, f64, i32,
                             C.POINTER(MpirResult)]),
    "LAPACKE_dsgesv": (i32, [i32, i32, i32, vp, i32, vp, vp, i32, vp, i32, vp]),
    "zml_dposv_mpir": (i32, [i32, ch, i32, i32, vp, i32, vp, i32, vp, i32, i32, i32, f64, i32,
                             C.POINTER(MpirResult)]),
    "LAPACKE_dsposv": (i32, [i32, ch, i32, i32, vp, i32, vp, i32, vp, i32, vp]),
    "zml_gpu_dposv_mpir": (i32, [ch, i32, i32, vp, i32, vp, i32, vp, i32, i32, i32, f64, i32,
                                 C.POINTER(MpirResult), vp]),
    "zml_gpu_dgesv_mpir": (i32, [i32, i32, vp, i32, vp, i32, vp, i32, i32, i32, f64, i32,
                                 C.POINTER(MpirResult), vp]),
})

_SIGS.update({
    "zml_gpu_profile": (None, [i32]),
    "zml_gpu_profile_read": (i32, [i32, C.POINTER(C.c_ulonglong), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "zml_gpu_launch_count": (C.c_ulonglong, []),
})

KERNEL_CLASSES = ["gemm_tc", "gemm_simt", "panel", "trsm_diag", "laswp", "trsv", "gemv",
                  "convert", "potf2", "vector", "batched", "qr", "mlp", "other"]


def profile_read():
    """{class: (launches, ms, flops, bytes)} accumulated since zml_gpu_profile(1)."""
    out = {}
    for t, name in enumerate(KERNEL_CLASSES):
        n, ms, fl, by = C.c_ulonglong(), C.c_double(), C.c_double(), C.c_double()
        lib().zml_gpu_profile_read(t, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by))
        if n.value:
            out[name] = (n.value, ms.value, fl.value, by.value)
    return out


_SIGS.update({
    "zml_gpu_batched_plan_create": (i32, [C.POINTER(vp), i32, vp, vp, i32, i32, i32]),
    "zml_gpu_batched_execute": (i32, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "zml_gpu_batched_run_graph": (i32, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "zml_gpu_batched_plan_destroy": (None, [vp]),
    "zml_gpu_batched_schedule": (i32, [i32, vp, vp, i32, i32]),
    "zml_gpu_batched_autotune": (i32, [i32, i32, vp, vp, vp]),
})

_SIGS.update({
    "zml_gpu_selector_features": (i32, [i32, vp, i32, vp, vp]),
    "zml_gpu_mlp_num_params": (i32, []),
    "zml_gpu_mlp_work_floats": (C.c_long, [i32]),
    "zml_gpu_mlp_forward": (i32, [i32, vp, vp, vp, vp, vp]),
    "zml_gpu_mlp_gradients": (i32, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "zml_gpu_mlp_adam": (i32, [vp, vp, vp, vp, f32, f32, f32, f32, i32, f32, vp]),
    "zml_gpu_selector_model_floats": (i32, []),
})


class AutoResult(C.Structure):
    """zml_auto_result of include/clapack.h."""
    _fields_ = [("info", C.c_int), ("predicted", C.c_int), ("used", C.c_int),
                ("attempts", C.c_int), ("converged", C.c_int), ("iters", C.c_int),
                ("berr", C.c_double), ("ms", C.c_double),
                ("features", C.c_float * 16), ("proba", C.c_float * 5), ("reserved", C.c_int)]


_SIGS.update({
    "zml_dgesv_auto": (i32, [i32, i32, i32, vp, i32, vp, i32, vp, i32, vp, f32, i32,
                             C.POINTER(AutoResult)]),
    "zml_gpu_dgesv_auto": (i32, [i32, i32, vp, i32, vp, i32, vp, i32, vp, f32, i32,
                                 C.POINTER(AutoResult), vp]),
})

class DMatrix(C.Structure):
    """zml_dmatrix of include/zml_linalg.h."""
    _fields_ = [("data", C.POINTER(C.c_double)), ("rows", C.c_int), ("cols", C.c_int),
                ("ld", C.c_int), ("layout", C.c_int), ("uplo", C.c_int), ("diag", C.c_int),
                ("owns_data", C.c_int)]

    def to_numpy(self):
        """A copy of the (rows x cols) matrix the view describes."""
        import numpy as np
        if self.rows == 0 or self.cols == 0:
            return np.zeros((self.rows, self.cols))
        if self.layout == COL_MAJOR:
            flat = np.ctypeslib.as_array(self.data, shape=(self.ld * (self.cols - 1) + self.rows,))
            idx = np.arange(self.rows)[:, None] + self.ld * np.arange(self.cols)[None, :]
        else:
            flat = np.ctypeslib.as_array(self.data, shape=(self.ld * (self.rows - 1) + self.cols,))
            idx = self.ld * np.arange(self.rows)[:, None] + np.arange(self.cols)[None, :]
        return flat[idx].copy()


ERR_INVALID_ARGUMENT, ERR_SINGULAR_MATRIX, ERR_OUT_OF_MEMORY = -2000, -2001, -2002
ERR_DIMENSION_MISMATCH = -2003
ERR_FACTORIZATION_FAILED = -2004
QR_FULL, QR_ECONOMICAL = 0, 1
_pp = C.POINTER(vp)
_SIGS.update({
    "zml_dmatrix_deinit": (None, [C.POINTER(DMatrix)]),
    "zml_plu": (i32, [i32, i32, i32, vp, i32, _pp]),
    "zml_plu_deinit": (None, [vp]),
    "zml_plu_p": (i32, [vp, vp]),
    "zml_plu_l": (DMatrix, [vp]),
    "zml_plu_u": (DMatrix, [vp]),
    "zml_plu_ipiv": (C.POINTER(C.c_int), [vp]),
    "zml_llt": (i32, [i32, ch, i32, vp, i32, _pp]),
    "zml_utu": (i32, [i32, ch, i32, vp, i32, _pp]),
    "zml_cholesky": (i32, [i32, ch, i32, vp, i32, _pp]),
    "zml_chol_deinit": (None, [vp]),
    "zml_chol_factor": (DMatrix, [vp]),
    "zml_qr": (i32, [i32, i32, i32, vp, i32, _pp]),
    "zml_qr_deinit": (None, [vp]),
    "zml_qr_q": (i32, [vp, i32, C.POINTER(DMatrix)]),
    "zml_qr_r": (DMatrix, [vp, i32]),
    "zml_qr_tau": (C.POINTER(C.c_double), [vp]),
    "zml_dmatmul": (i32, [C.POINTER(DMatrix), C.POINTER(DMatrix), C.POINTER(DMatrix)]),
    "zml_dmatvec": (i32, [C.POINTER(DMatrix), vp, i32, vp, i32]),
    "zml_dvecmat": (i32, [vp, i32, C.POINTER(DMatrix), vp, i32]),
    "zml_ldlt": (i32, [i32, ch, i32, vp, i32, _pp]),
    "zml_udut": (i32, [i32, ch, i32, vp, i32, _pp]),
    "zml_bunchkaufman": (i32, [i32, ch, i32, vp, i32, _pp, _pp]),
    "zml_ldlt_init": (i32, [i32, i32, vp, i32, vp, _pp]),
    "zml_udut_init": (i32, [i32, i32, vp, i32, vp, _pp]),
    "zml_ldlt_deinit": (None, [vp]),
    "zml_udut_deinit": (None, [vp]),
    "zml_ldlt_p": (i32, [vp, vp]),
    "zml_udut_p": (i32, [vp, vp]),
    "zml_ldlt_l": (DMatrix, [vp]),
    "zml_udut_u": (DMatrix, [vp]),
    "zml_ldlt_d": (i32, [vp, vp, vp, vp]),
    "zml_udut_d": (i32, [vp, vp, vp, vp]),
    "zml_ldlt_ipiv": (C.POINTER(C.c_int), [vp]),
    "zml_udut_ipiv": (C.POINTER(C.c_int), [vp]),
})

PREC_FP16, PREC_BF16, PREC_FP32, PREC_BF16X3 = 0, 1, 2, 3
REFINE_IR, REFINE_GMRES = 0, 1

_lib = None


class NotBuiltError(RuntimeError):
    pass


def declared_symbols():
    """Every function name declared in include/*.h."""
    names = []
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", txt, flags=re.M):
            name = m.group(1)
            if name not in ("if", "defined") and not txt[m.start():m.end()].startswith("typedef"):
                names.append(name)
    return names


def lib():
    """The loaded library with argtypes set; raises NotBuiltError if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NotBuiltError("%s missing: run python -c 'import __graft_entry__ as g; g.build()'"
                                % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _lib = L
    return _lib


def last_error():
    return lib().zml_gpu_last_error().decode()
