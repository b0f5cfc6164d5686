"""GPU parity for Bunch-Kaufman (LAPACKE_dsytrf / ssytrf) against the oracle.

The GPU runs zml's unblocked pivoting step by step with every product and sum
rounded on its own (no FMA), so its factors and ipiv are the oracle's sytf2
bit for bit at every size; zml's sytrf switches to the blocked lasyf above
64 columns, against which the pivots agree and the factors to rounding.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lap

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P

pytestmark = pytest.mark.gpu


def sym(n, seed, dtype=np.float64):
    g = np.random.default_rng(seed).standard_normal((n, n))
    return np.asfortranarray(((g + g.T) / 2).astype(dtype))


def gpu_sytrf(a, uplo, layout=102):
    n = a.shape[0]
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    ipiv = np.zeros(n, dtype=np.int32)
    f = zg.lib().LAPACKE_dsytrf if a.dtype == np.float64 else zg.lib().LAPACKE_ssytrf
    info = f(layout, uplo, n, P(buf), n, P(ipiv))
    return buf, ipiv, info


def oracle_sytf2(a, ul):
    f = np.asfortranarray(a.copy())
    ipiv = np.zeros(a.shape[0], dtype=np.int32)
    info = ol.fn("sytf2", a.dtype)(102, ul, a.shape[0], ol.ptr(f), max(1, a.shape[0]), ol.ptr(ipiv))
    return f, ipiv, info


@pytest.mark.parametrize("uplo", [b"U", b"L"])
@pytest.mark.parametrize("n", [1, 2, 5, 64, 65, 130])
def test_dsytrf_bitwise_equals_oracle_sytf2(n, uplo):
    a = sym(n, seed=n * 7 + uplo[0])
    f, ipiv, info = gpu_sytrf(a, uplo)
    ul = 121 if uplo == b"U" else 122
    fr, ipr, infr = oracle_sytf2(a, ul)
    assert info == infr == 0
    np.testing.assert_array_equal(ipiv, ipr)
    tri = np.triu if uplo == b"U" else np.tril
    np.testing.assert_array_equal(tri(f), tri(fr))
    np.testing.assert_array_equal(f - tri(f), a - tri(a))  # the other triangle untouched


@pytest.mark.parametrize("uplo", [b"U", b"L"])
def test_dsytrf_vs_blocked_oracle_and_lapack_solve(uplo):
    n = 200
    a = sym(n, seed=9)
    f, ipiv, info = gpu_sytrf(a, uplo)
    ul = 121 if uplo == b"U" else 122
    fb, ipb, _ = ol.sytrf(a, ul)
    np.testing.assert_array_equal(ipiv, ipb)
    tri = np.triu if uplo == b"U" else np.tril
    assert np.abs(tri(f) - tri(fb)).max() <= 1e-10 * np.abs(fb).max()
    x = np.random.default_rng(1).standard_normal((n, 2))
    sol, inf = lap.dsytrs(f, ipiv, a @ x, lower=int(uplo == b"L"))
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-8, atol=1e-8)


def test_dsytrf_row_major_and_zero_column_info():
    a = sym(80, seed=4)
    fc, pc, _ = gpu_sytrf(a, b"L")
    fr, pr, _ = gpu_sytrf(a, b"L", layout=101)
    np.testing.assert_array_equal(pr, pc)
    np.testing.assert_array_equal(np.tril(fr), np.tril(fc))
    z = sym(30, seed=6)
    z[11, :] = 0
    z[:, 11] = 0
    for uplo, ul in ((b"U", 121), (b"L", 122)):
        _, ipiv, info = gpu_sytrf(z, uplo)
        _, ipr, infr = oracle_sytf2(z, ul)
        assert info == infr > 0
        np.testing.assert_array_equal(ipiv, ipr)


def test_ssytrf_bitwise_equals_oracle():
    a = sym(90, seed=12, dtype=np.float32)
    f, ipiv, info = gpu_sytrf(a, b"L")
    fr, ipr, infr = oracle_sytf2(a, 122)
    assert info == infr == 0
    np.testing.assert_array_equal(ipiv, ipr)
    np.testing.assert_array_equal(np.tril(f), np.tril(fr))


@pytest.mark.gpu
@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("layout", [102, 101])
def test_bunchkaufman_facade_reconstructs(uplo, layout):
    """zml_bunchkaufman: ldlt for a lower-stored matrix, udut for an upper
    one, factored on the GPU; its p / l|u / d reconstruct A."""
    import ctypes as C
    from test_api_host import _bk_unpack
    L = zg.lib()
    n = 150
    g = np.random.default_rng(5).standard_normal((n, n))
    a = (g + g.T) / 2
    ac = np.ascontiguousarray(a) if layout == 101 else np.asfortranarray(a)
    lo, up = C.c_void_p(), C.c_void_p()
    assert L.zml_bunchkaufman(layout, uplo, n, ac.ctypes.data_as(C.c_void_p), n, C.byref(lo),
                              C.byref(up)) == 0
    upper = uplo == b"U"
    h = up if upper else lo
    assert h.value and not (lo if upper else up).value
    perm, t, D = _bk_unpack(L, h, upper, n)
    (L.zml_udut_deinit if upper else L.zml_ldlt_deinit)(h)
    assert np.abs(a[np.ix_(perm, perm)] - t @ D @ t.T).max() <= 1e-10 * np.abs(a).max()


@pytest.mark.parametrize("uplo", [b"U", b"L"])
def test_dsytrf_device_pointers_n1536_bitwise(uplo):
    """Device operands at n = 1536 (every step enqueued from device state):
    still the oracle's sytf2 bit for bit."""
    import torch
    n = 1536
    a = sym(n, seed=31 + uplo[0])
    F = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # row-major storage of a^T = a
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = zg.lib().LAPACKE_dsytrf(102, uplo, n, F.data_ptr(), n, piv.data_ptr())
    ul = 121 if uplo == b"U" else 122
    fr, ipr, infr = oracle_sytf2(a, ul)
    assert info == infr == 0
    np.testing.assert_array_equal(piv.cpu().numpy(), ipr)
    f = F.cpu().numpy().T  # column-major view
    tri = np.triu if uplo == b"U" else np.tril
    np.testing.assert_array_equal(tri(f), tri(fr))


def csym(n, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return np.asfortranarray(((g + g.T) / 2).astype(dtype))  # complex symmetric, not Hermitian


def gpu_zsytrf(a, uplo, layout=102):
    n = a.shape[0]
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    ipiv = np.zeros(n, dtype=np.int32)
    f = zg.lib().LAPACKE_zsytrf if a.dtype == np.complex128 else zg.lib().LAPACKE_csytrf
    info = f(layout, uplo, n, P(buf), n, P(ipiv))
    return np.asfortranarray(buf), ipiv, info


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("uplo", [b"U", b"L"])
@pytest.mark.parametrize("n", [1, 2, 5, 64, 130, 257])
def test_zsytrf_bitwise_equals_oracle_sytf2(n, uplo, dtype):
    """Complex symmetric Bunch-Kaufman (no conjugation, |re| + |im| pivots,
    zml's fused complex products and Smith quotients): the oracle's complex
    sytf2 bit for bit, the untouched triangle left as it was."""
    a = csym(n, seed=3 * n + uplo[0], dtype=dtype)
    f, ipiv, info = gpu_zsytrf(a, uplo)
    ul = 121 if uplo == b"U" else 122
    fr, ipr, infr = oracle_sytf2(a, ul)
    assert info == infr == 0
    np.testing.assert_array_equal(ipiv, ipr)
    tri = np.triu if uplo == b"U" else np.tril
    np.testing.assert_array_equal(tri(f), tri(fr))
    np.testing.assert_array_equal(f - tri(f), a - tri(a))


def test_zsytrf_row_major_zero_column_and_lapack_solve():
    a = csym(90, seed=8)
    fc, pc, _ = gpu_zsytrf(a, b"L")
    fr, pr, _ = gpu_zsytrf(a, b"L", layout=101)
    np.testing.assert_array_equal(pr, pc)
    np.testing.assert_array_equal(np.tril(fr), np.tril(fc))
    x = np.random.default_rng(2).standard_normal((90, 2)) + 0j
    sol, inf = lap.zsytrs(fc, pc, a @ x, lower=1)
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-9, atol=1e-9)
    z = csym(30, seed=6)
    z[11, :] = 0
    z[:, 11] = 0
    for uplo, ul in ((b"U", 121), (b"L", 122)):
        f, ipiv, info = gpu_zsytrf(z, uplo)
        fr, ipr, infr = oracle_sytf2(z, ul)
        assert info == infr > 0
        np.testing.assert_array_equal(ipiv, ipr)


def herm(n, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return np.asfortranarray(((g + g.conj().T) / 2).astype(dtype))


def gpu_zhetrf(a, uplo, layout=102):
    n = a.shape[0]
    buf = np.array(a, order="F" if layout == 102 else "C", copy=True)
    ipiv = np.zeros(n, dtype=np.int32)
    f = zg.lib().LAPACKE_zhetrf if a.dtype == np.complex128 else zg.lib().LAPACKE_chetrf
    info = f(layout, uplo, n, P(buf), n, P(ipiv))
    return np.asfortranarray(buf), ipiv, info


def oracle_hetf2(a, ul):
    f = np.asfortranarray(a.copy())
    ipiv = np.zeros(a.shape[0], dtype=np.int32)
    info = ol.fn("hetf2", a.dtype)(102, ul, a.shape[0], ol.ptr(f), max(1, a.shape[0]), ol.ptr(ipiv))
    return f, ipiv, info


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 2e-5)])
@pytest.mark.parametrize("uplo", [b"U", b"L"])
@pytest.mark.parametrize("n", [1, 2, 5, 64, 130, 257])
def test_zhetrf_equals_oracle_hetf2(n, uplo, dtype, tol):
    """Hermitian Bunch-Kaufman: the oracle's hetf2 pivots exactly and its
    factors to rounding (the 2x2 step's |a_k',k| is a hypot from another
    math library), a real diagonal, the other triangle untouched."""
    a = herm(n, seed=5 * n + uplo[0], dtype=dtype)
    f, ipiv, info = gpu_zhetrf(a, uplo)
    ul = 121 if uplo == b"U" else 122
    fr, ipr, infr = oracle_hetf2(a, ul)
    assert info == infr == 0
    np.testing.assert_array_equal(ipiv, ipr)
    tri = np.triu if uplo == b"U" else np.tril
    scale = np.abs(tri(fr)).max()
    assert np.abs(tri(f) - tri(fr)).max() <= tol * scale
    assert np.all(np.diag(f).imag == 0)
    np.testing.assert_array_equal(f - tri(f), a - tri(a))


def test_zhetrf_row_major_zero_column_and_lapack_solve():
    a = herm(90, seed=12)
    fc, pc, _ = gpu_zhetrf(a, b"U")
    fr, pr, _ = gpu_zhetrf(a, b"U", layout=101)
    np.testing.assert_array_equal(pr, pc)
    np.testing.assert_array_equal(np.triu(fr), np.triu(fc))
    x = np.random.default_rng(4).standard_normal((90, 2)) + 0j
    sol, inf = lap.zhetrs(fc, pc, a @ x, lower=0)
    assert inf == 0
    np.testing.assert_allclose(sol, x, rtol=1e-9, atol=1e-9)
    z = herm(30, seed=9)
    z[7, :] = 0
    z[:, 7] = 0
    for uplo, ul in ((b"U", 121), (b"L", 122)):
        _, ipiv, info = gpu_zhetrf(z, uplo)
        _, ipr, infr = oracle_hetf2(z, ul)
        assert info == infr > 0
        np.testing.assert_array_equal(ipiv, ipr)
