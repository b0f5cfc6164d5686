"""GPU parity for the complex level-3 BLAS through the C ABI (cblas_zgemm,
cblas_zherk, cblas_zsyrk and the single-precision c forms).

1. The cf64 parts of zml's own BLAS tests (tests/golden/blas_z{gemm,herk,
   syrk}.json) replayed through the C ABI: integer-valued results, exact.
2. Random shapes against the complex oracle: every transpose pair, both
   layouts, complex alpha / beta, padded leading dimensions; within
   1e-12 of the product's magnitude (binary64) or 1e-5 (binary32).  The GPU
   sums in another order than the oracle's loops.
3. beta = 0 clears C (NaNs there do not survive); herk leaves the other
   triangle untouched and the diagonal real; device pointers work.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from golden_replay import load_fixture, replay
from gpu_util import P

pytestmark = pytest.mark.gpu

TRANS = [111, 112, 113, 114]


def zcapi_call(name, args):
    """A complex fixture's call on cblas_z*: complex scalars by pointer (herk:
    real scalars by value)."""
    args = list(args)
    for pos in {"gemm": (6, 11), "syrk": (5, 8)}.get(name, ()):
        args[pos] = complex(args[pos])  # scalars by pointer, whatever the fixture's type
    keep, conv = [], []
    for a in args:
        if isinstance(a, np.ndarray):
            conv.append(P(a))
        elif isinstance(a, complex):
            v = np.array([a.real, a.imag])
            keep.append(v)
            conv.append(P(v))
        else:
            conv.append(a)
    if name == "herk":
        conv[5], conv[8] = float(args[5].real if isinstance(args[5], complex) else args[5]), \
            float(args[8].real if isinstance(args[8], complex) else args[8])
    getattr(zg.lib(), "cblas_z" + name)(*conv)


@pytest.mark.parametrize("name", ["gemm", "herk", "syrk"])
def test_reference_complex_fixtures_through_cblas(name):
    checked, failures = replay(load_fixture("z" + name), zcapi_call)
    assert checked > 0
    assert not failures, failures[:5]


def cmat(shape, rng, dtype=np.complex128):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def store(x, order, pad=0):
    """(flat storage, leading dimension) of logical matrix x in `order`, with
    `pad` unused elements after each column (col-major) or row (row-major)."""
    r, c = x.shape
    if order == 102:
        ld = max(1, r + pad)
        buf = np.zeros((c, ld), dtype=x.dtype)
        buf[:, :r] = x.T
    else:
        ld = max(1, c + pad)
        buf = np.zeros((r, ld), dtype=x.dtype)
        buf[:, :c] = x
    return buf.reshape(-1).copy(), ld


def scal(x, dtype=np.complex128):
    return np.array([x.real, x.imag], dtype=np.float64 if dtype == np.complex128 else np.float32)


@pytest.mark.parametrize("ta", TRANS)
@pytest.mark.parametrize("tb", TRANS)
@pytest.mark.parametrize("order", [101, 102])
def test_zgemm_vs_oracle(order, ta, tb):
    m, n, k = 67, 45, 33
    rng = np.random.default_rng(ta * 31 + tb * 7 + order)
    A = cmat((m, k) if ta in (111, 114) else (k, m), rng)
    B = cmat((k, n) if tb in (111, 114) else (n, k), rng)
    Cm = cmat((m, n), rng)
    a, lda = store(A, order, pad=3)
    b, ldb = store(B, order, pad=1)
    c0, ldc = store(Cm, order, pad=2)
    alpha, beta = 1.5 - 0.5j, -0.75 + 0.25j
    c_ref, c_gpu = c0.copy(), c0.copy()
    assert ol.fn("gemm", np.complex128)(order, ta, tb, m, n, k, ol.cs(alpha), ol.ptr(a), lda,
                                        ol.ptr(b), ldb, ol.cs(beta), ol.ptr(c_ref), ldc) == 0
    zg.lib().cblas_zgemm(order, ta, tb, m, n, k, P(scal(alpha)), P(a), lda, P(b), ldb,
                         P(scal(beta)), P(c_gpu), ldc)
    scale = np.abs(A).max() * np.abs(B).max() * k * 2 + np.abs(Cm).max()
    assert np.abs(c_gpu - c_ref).max() <= 1e-13 * scale
    # the padding is untouched
    np.testing.assert_array_equal(c_gpu[c0 == 0], c0[c0 == 0])


def test_zgemm_beta_zero_clears_nan_and_alpha_zero_scales():
    m, n, k = 40, 30, 20
    rng = np.random.default_rng(5)
    A, B = cmat((m, k), rng), cmat((k, n), rng)
    a, lda = store(A, 102)
    b, ldb = store(B, 102)
    c = np.full(m * n, np.nan + 1j * np.nan)
    zg.lib().cblas_zgemm(102, 111, 111, m, n, k, P(scal(1 + 0j)), P(a), lda, P(b), ldb,
                         P(scal(0j)), P(c), m)
    np.testing.assert_allclose(c.reshape(n, m).T, A @ B, rtol=1e-12, atol=1e-12)
    c2 = store(cmat((m, n), rng), 102)[0]
    want = c2 * (2 - 1j)
    zg.lib().cblas_zgemm(102, 111, 111, m, n, k, P(scal(0j)), P(a), lda, P(b), ldb,
                         P(scal(2 - 1j)), P(c2), m)
    np.testing.assert_allclose(c2, want, rtol=1e-15)


@pytest.mark.parametrize("ta,tb", [(111, 111), (113, 112), (114, 113)])
def test_cgemm_single_precision(ta, tb):
    m, n, k = 50, 40, 30
    rng = np.random.default_rng(ta + tb)
    A = cmat((m, k) if ta in (111, 114) else (k, m), rng, np.complex64)
    B = cmat((k, n) if tb in (111, 114) else (n, k), rng, np.complex64)
    Cm = cmat((m, n), rng, np.complex64)
    a, lda = store(A, 102)
    b, ldb = store(B, 102)
    c0, ldc = store(Cm, 102)
    al, be = np.complex64(0.5 + 1j), np.complex64(1 - 0.5j)
    c_ref, c_gpu = c0.copy(), c0.copy()
    assert ol.fn("gemm", np.complex64)(102, ta, tb, m, n, k, ol.cs(al, np.complex64), ol.ptr(a),
                                       lda, ol.ptr(b), ldb, ol.cs(be, np.complex64), ol.ptr(c_ref),
                                       ldc) == 0
    zg.lib().cblas_cgemm(102, ta, tb, m, n, k, P(scal(al, np.complex64)), P(a), lda, P(b), ldb,
                         P(scal(be, np.complex64)), P(c_gpu), ldc)
    assert np.abs(c_gpu - c_ref).max() <= 1e-5 * np.abs(c_ref).max()


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("order", [101, 102])
@pytest.mark.parametrize("trans_idx", [0, 1])
def test_zherk_zsyrk_vs_oracle(herm, uplo, order, trans_idx):
    n, k = 57, 23
    trans = [111, 113][trans_idx] if herm else [111, 112][trans_idx]
    rng = np.random.default_rng(n + k + uplo + order + trans + herm)
    # the logical A is n x k for no_trans; row-major herk / syrk map the
    # transpose, so the shape follows the caller's trans
    A = cmat((n, k) if trans == 111 else (k, n), rng)
    Cm = cmat((n, n), rng)
    a, lda = store(A, order, pad=2)
    c0, ldc = store(Cm, order, pad=1)
    c_ref, c_gpu = c0.copy(), c0.copy()
    if herm:
        alpha, beta = 1.25, -0.5
        assert ol.fn("herk", np.complex128)(order, uplo, trans, n, k, alpha, ol.ptr(a), lda, beta,
                                            ol.ptr(c_ref), ldc) == 0
        zg.lib().cblas_zherk(order, uplo, trans, n, k, alpha, P(a), lda, beta, P(c_gpu), ldc)
    else:
        alpha, beta = 0.5 + 1j, 2 - 1j
        assert ol.fn("syrk", np.complex128)(order, uplo, trans, n, k, ol.cs(alpha), ol.ptr(a), lda,
                                            ol.cs(beta), ol.ptr(c_ref), ldc) == 0
        zg.lib().cblas_zsyrk(order, uplo, trans, n, k, P(scal(alpha)), P(a), lda, P(scal(beta)),
                             P(c_gpu), ldc)
    scale = np.abs(A).max() ** 2 * k * 4 + np.abs(Cm).max() * 2
    assert np.abs(c_gpu - c_ref).max() <= 1e-13 * scale
    # the other triangle and the padding are untouched (the oracle leaves them)
    same = c_ref == c0
    np.testing.assert_array_equal(c_gpu[same], c0[same])
    if herm:
        g = c_gpu.reshape(n, ldc)[:, :n] if order == 101 else c_gpu.reshape(n, ldc)[:, :n].T
        assert not np.diag(g).imag.any()


def test_zgemm_device_pointers():
    import torch
    m, n, k = 64, 48, 40
    rng = np.random.default_rng(11)
    A, B = cmat((m, k), rng), cmat((k, n), rng)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # column-major storage
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    zg.lib().cblas_zgemm(102, 111, 111, m, n, k, P(scal(1 + 0j)), dA.data_ptr(), m, dB.data_ptr(),
                         k, P(scal(0j)), dC.data_ptr(), m)
    np.testing.assert_allclose(dC.cpu().numpy().T, A @ B, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("ta,tb", [(111, 111), (113, 112)])
def test_zgemm_exact_slices_path(ta, tb):
    """FP64 complex GEMM large enough (min(2m, n) >= 2048) to run as exact
    slices on the tensor cores, with K = 2 x 300 split into 256, 256 and 88,
    complex alpha and beta, and transposed / conjugated operands: within the
    error of an FP64 product of that depth."""
    import torch
    m, n, k = 1100, 2100, 300
    rng = np.random.default_rng(21)
    opA = cmat((m, k), rng)
    opB = cmat((k, n), rng)
    A = opA if ta == 111 else (opA.T if ta == 112 else opA.conj().T)  # stored op^-1(opA)
    B = opB if tb == 111 else (opB.T if tb == 112 else opB.conj().T)
    C0 = cmat((m, n), rng)
    alpha, beta = 0.75 - 0.5j, -0.25 + 1.5j
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # column-major storage
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(C0.T)).cuda()
    torch.cuda.synchronize()
    zg.lib().cblas_zgemm(102, ta, tb, m, n, k, P(scal(alpha)), dA.data_ptr(), A.shape[0],
                         dB.data_ptr(), B.shape[0], P(scal(beta)), dC.data_ptr(), m)
    torch.cuda.synchronize()
    ref = alpha * (opA @ opB) + beta * C0
    got = dC.cpu().numpy().T
    scale = np.abs(alpha) * (np.abs(opA) @ np.abs(opB)) + np.abs(beta) * np.abs(C0)
    assert (np.abs(got - ref) / scale).max() <= 64 * 2.0 ** -53
