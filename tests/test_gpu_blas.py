"""GPU parity for the level-3 BLAS through the C ABI (cblas_d*).

1. zml's own known-answer chains (tests/golden/blas_{gemm,trsm,syrk}.json)
   replayed through cblas_dgemm / cblas_dtrsm / cblas_dsyrk: integer-valued
   gemm/syrk results must be exact, trsm within zml's 1e-7 relative bound.
2. Random shapes against the oracle, host and device pointers.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from golden_replay import load_fixture, replay
from gpu_util import P, gaussian

pytestmark = pytest.mark.gpu


def capi_call(name, args):
    L = zg.lib()
    conv = [P(a) if isinstance(a, np.ndarray) else a for a in args]
    getattr(L, "cblas_d" + name)(*conv)


@pytest.mark.parametrize("name", ["gemm", "trsm", "syrk"])
def test_reference_fixtures_through_cblas(name):
    checked, failures = replay(load_fixture(name), capi_call)
    assert checked > 0
    assert not failures, failures[:5]


TR = [111, 112]


def store(x, order):
    """(flat storage, leading dimension) of logical matrix x in `order`."""
    if order == 102:
        return x.flatten(order="F"), max(1, x.shape[0])
    return x.flatten(order="C"), max(1, x.shape[1])


@pytest.mark.parametrize("ta", TR)
@pytest.mark.parametrize("tb", TR)
@pytest.mark.parametrize("order", [101, 102])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (65, 33, 17), (130, 257, 64), (300, 200, 129)])
def test_dgemm_vs_oracle(order, ta, tb, m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    A = rng.standard_normal((m, k) if ta == 111 else (k, m))
    B = rng.standard_normal((k, n) if tb == 111 else (n, k))
    Cm = rng.standard_normal((m, n))
    a, lda = store(A, order)
    b, ldb = store(B, order)
    c0, ldc = store(Cm, order)
    alpha, beta = 1.5, -0.75
    c_ref, c_gpu = c0.copy(), c0.copy()
    assert ol.fn("gemm")(order, ta, tb, m, n, k, alpha, P(a), lda, P(b), ldb, beta, P(c_ref), ldc) == 0
    zg.lib().cblas_dgemm(order, ta, tb, m, n, k, alpha, P(a), lda, P(b), ldb, beta, P(c_gpu), ldc)
    np.testing.assert_allclose(c_gpu, c_ref, rtol=1e-12, atol=1e-12 * k)


@pytest.mark.parametrize("side", [141, 142])
@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("ta", [111, 112])
@pytest.mark.parametrize("diag", [131, 132])
@pytest.mark.parametrize("m,n", [(70, 45), (130, 200)])
def test_dtrsm_vs_oracle(side, uplo, ta, diag, m, n):
    k = m if side == 141 else n
    rng = np.random.default_rng(k + m)
    a = np.asfortranarray(rng.standard_normal((k, k)) / k + 2 * np.eye(k))
    b0 = np.asfortranarray(rng.standard_normal((m, n)))
    b_ref, b_gpu = b0.copy(order="F"), b0.copy(order="F")
    assert ol.fn("trsm")(102, side, uplo, ta, diag, m, n, 0.5, P(a), k, P(b_ref), m) == 0
    zg.lib().cblas_dtrsm(102, side, uplo, ta, diag, m, n, 0.5, P(a), k, P(b_gpu), m)
    np.testing.assert_allclose(b_gpu, b_ref, rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("trans", [111, 112])
@pytest.mark.parametrize("order", [101, 102])
def test_dsyrk_vs_oracle(uplo, trans, order):
    n, k = 150, 70
    rng = np.random.default_rng(3)
    a, lda = store(rng.standard_normal((n, k) if trans == 111 else (k, n)), order)
    c0 = rng.standard_normal(n * n)
    c_ref, c_gpu = c0.copy(), c0.copy()
    assert ol.fn("syrk")(order, uplo, trans, n, k, -1.0, P(a), lda, 2.0, P(c_ref), n) == 0
    zg.lib().cblas_dsyrk(order, uplo, trans, n, k, -1.0, P(a), lda, 2.0, P(c_gpu), n)
    np.testing.assert_allclose(c_gpu, c_ref, rtol=1e-12, atol=1e-12 * k)


def test_device_pointer_gemm_in_place():
    import torch
    m, n, k = 257, 129, 96
    a = gaussian(m, k, seed=1)
    b = gaussian(k, n, seed=2)
    c = gaussian(m, n, seed=3)
    ref = 2.0 * a @ b + 0.5 * c
    ta = torch.from_numpy(a.T.copy()).cuda()  # row-major storage of a^T == col-major a
    tb = torch.from_numpy(b.T.copy()).cuda()
    tc = torch.from_numpy(c.T.copy()).cuda()
    zg.lib().cblas_dgemm(102, 111, 111, m, n, k, 2.0, ta.data_ptr(), m, tb.data_ptr(), k, 0.5,
                         tc.data_ptr(), m)
    np.testing.assert_allclose(tc.cpu().numpy().T, ref, rtol=1e-12, atol=1e-11)
