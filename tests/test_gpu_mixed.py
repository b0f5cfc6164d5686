"""Mixed-precision solve (zml_dgesv_mpir / LAPACKE_dsgesv) on the GPU.

Bar: the refined solution's normwise backward error
    ||b - A x||inf / (||A||inf ||x||inf + ||b||inf)
is no worse than 2x the plain FP64 LU solution's (the oracle's getrf+getrs
on the same input) plus one unit roundoff, and the forward error is within
cond(A) * u of x_true.
"""
import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import P, gaussian

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53


def berr(a, x, b):
    r = b - a @ x
    return np.abs(r).max() / (np.abs(a).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


def svd_matrix(n, kappa, seed):
    rng = np.random.default_rng(seed)
    u, _ = np.linalg.qr(rng.standard_normal((n, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = kappa ** (-np.arange(n) / (n - 1))
    return np.asfortranarray((u * s) @ v.T)


def solve(a, b, prec, mode, tol=0.0, max_iter=30):
    n = a.shape[0]
    nrhs = b.shape[1]
    x = np.zeros((n, nrhs), order="F")
    res = zg.MpirResult()
    r = zg.lib().zml_dgesv_mpir(102, n, nrhs, P(a), n, P(b), n, P(x), n, prec, mode, tol,
                                max_iter, res)
    assert r == 0, zg.last_error()
    return x, res


def fp64_berr(a, b):
    lu, ipiv, info = ol.getrf(a)
    x = ol.getrs(lu, ipiv, b)
    return berr(a, x, b)


@pytest.mark.parametrize("prec,mode", [(1, 1), (0, 1), (2, 0), (0, 0), (1, 0), (3, 0), (3, 1)])
@pytest.mark.parametrize("n", [300, 1000])
def test_mpir_reaches_fp64_backward_error(n, prec, mode):
    a = gaussian(n, seed=n + prec)
    xt = np.random.default_rng(5).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    x, res = solve(a, b, prec, mode)
    assert res.info == 0
    e = berr(a, x, b)
    e64 = fp64_berr(a, b)
    if prec == 1 and mode == 0 and not res.converged:
        pytest.skip("plain IR with BF16 factors may stall for this n (GMRES-IR covers it)")
    assert res.converged, (res.berr, list(res.berr_history[:res.iters + 1]))
    assert e <= 2 * e64 + U64, (e, e64)
    # the library's own backward error agrees with numpy's at roundoff level
    assert res.berr <= 4 * (e + U64)
    cond = np.linalg.cond(a)
    assert np.abs(x - xt).max() / np.abs(xt).max() <= 10 * cond * U64 * n


@pytest.mark.parametrize("kappa,prec", [(1e2, 1), (1e6, 3), (1e8, 2)])
def test_gmres_ir_ill_conditioned(kappa, prec):
    """GMRES-IR reaches FP64 backward error with BF16 factors at kappa 1e2,
    split BF16x3 factors at 1e6 and FP32 factors at 1e8."""
    n = 512
    a = svd_matrix(n, kappa, seed=int(np.log10(kappa)))
    xt = np.random.default_rng(7).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    x, res = solve(a, b, prec, 1)
    assert res.info == 0 and res.converged, (res.berr, list(res.berr_history[:res.iters + 1]),
                                              res.switched_f64)
    assert berr(a, x, b) <= 2 * fp64_berr(a, b) + U64


def test_mpir_multiple_rhs_and_row_major():
    n, nrhs = 400, 4
    a = gaussian(n, seed=77)
    xt = np.random.default_rng(78).uniform(-1, 1, (n, nrhs))
    b = a @ xt
    ar, br = np.ascontiguousarray(a), np.ascontiguousarray(b)
    xr = np.zeros((n, nrhs))
    res = zg.MpirResult()
    assert zg.lib().zml_dgesv_mpir(101, n, nrhs, P(ar), n, P(br), nrhs, P(xr), nrhs, 1, 1, 0.0,
                                   30, res) == 0
    assert res.converged
    np.testing.assert_allclose(xr, xt, rtol=1e-9, atol=1e-10)


def test_mpir_singular_reports_info():
    n = 300
    a = gaussian(n, seed=3)
    a[:, 100] = 0.0
    b = np.asfortranarray(np.ones((n, 1)))
    _, res = solve(a, b, 1, 1)
    assert res.info == 101


def test_dsgesv_lapack_semantics_and_fallback():
    n = 256
    a = gaussian(n, seed=12)
    xt = np.random.default_rng(13).uniform(-1, 1, (n, 2))
    b = np.asfortranarray(a @ xt)
    a0, b0 = a.copy(order="F"), b.copy(order="F")
    x = np.zeros((n, 2), order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    it = np.zeros(1, dtype=np.int32)
    assert zg.lib().LAPACKE_dsgesv(102, n, 2, P(a), n, P(ipiv), P(b), n, P(x), n, P(it)) == 0
    assert it[0] >= 0
    np.testing.assert_array_equal(a, a0)  # A untouched when refinement succeeds
    np.testing.assert_array_equal(b, b0)
    np.testing.assert_allclose(x, xt, rtol=1e-10, atol=1e-11)
    # kappa ~ 1e13: FP32 refinement cannot converge -> FP64 LU fallback
    h = svd_matrix(n, 1e13, seed=4)
    bh = np.asfortranarray(h @ xt)
    xh = np.zeros((n, 2), order="F")
    assert zg.lib().LAPACKE_dsgesv(102, n, 2, P(h), n, P(ipiv), P(bh), n, P(xh), n, P(it)) == 0
    assert it[0] < 0
    lu_ref, ipiv_ref, _ = ol.getrf(svd_matrix(n, 1e13, seed=4))
    np.testing.assert_array_equal(ipiv, ipiv_ref)


# ---- SPD systems: mixed-precision Cholesky + refinement ---------------------

def spd_matrix(n, seed, kappa=None):
    rng = np.random.default_rng(seed)
    if kappa is None:
        g = rng.standard_normal((n, n))
        return np.asfortranarray(g @ g.T / n + np.eye(n))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = kappa ** (-np.arange(n) / (n - 1))
    return np.asfortranarray((v * s) @ v.T)


def solve_spd(a, b, prec, mode, uplo=b"L"):
    n, nrhs = b.shape
    x = np.zeros((n, nrhs), order="F")
    res = zg.MpirResult()
    r = zg.lib().zml_dposv_mpir(102, uplo, n, nrhs, P(a), n, P(b), n, P(x), n, prec, mode, 0.0,
                                30, res)
    assert r == 0, zg.last_error()
    return x, res


def fp64_chol_berr(a, b):
    f, info = ol.potrf(a, 122)
    return berr(a, ol.potrs(f, b, 122), b)


@pytest.mark.parametrize("prec,mode", [(3, 1), (2, 0), (1, 1), (0, 0), (3, 0)])
@pytest.mark.parametrize("n", [300, 1100])
def test_mixed_cholesky_reaches_fp64_backward_error(n, prec, mode):
    a = spd_matrix(n, seed=n + prec)
    xt = np.random.default_rng(9).uniform(-1, 1, (n, 2))
    b = np.asfortranarray(a @ xt)
    x, res = solve_spd(a, b, prec, mode)
    assert res.info == 0
    assert res.converged, (res.berr, list(res.berr_history[:res.iters + 1]))
    assert berr(a, x, b) <= 2 * fp64_chol_berr(a, b) + U64


def test_mixed_cholesky_upper_and_ill_conditioned():
    n = 512
    a = spd_matrix(n, seed=3, kappa=1e6)
    xt = np.random.default_rng(4).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    # only the upper triangle is read: poison the strict lower one
    au = np.triu(a) + np.tril(np.full((n, n), np.nan), -1)
    x, res = solve_spd(np.asfortranarray(au), b, 3, 1, uplo=b"U")
    assert res.info == 0 and res.converged, (res.berr, list(res.berr_history[:res.iters + 1]))
    assert berr(a, x, b) <= 2 * fp64_chol_berr(a, b) + U64


def test_mixed_cholesky_not_spd_and_dsposv():
    n = 300
    a = spd_matrix(n, seed=5)
    a[200, 200] = -10.0
    b = np.asfortranarray(np.ones((n, 1)))
    _, res = solve_spd(a, b, 3, 1)
    assert res.info > 0
    good = spd_matrix(n, seed=6)
    xt = np.random.default_rng(7).uniform(-1, 1, (n, 3))
    bb = np.asfortranarray(good @ xt)
    g0 = good.copy(order="F")
    x = np.zeros((n, 3), order="F")
    it = np.zeros(1, dtype=np.int32)
    assert zg.lib().LAPACKE_dsposv(102, b"L", n, 3, P(good), n, P(bb), n, P(x), n, P(it)) == 0
    assert it[0] >= 0
    np.testing.assert_array_equal(good, g0)
    np.testing.assert_allclose(x, xt, rtol=1e-10, atol=1e-11)


def test_lookahead_factorization_is_repeatable():
    """The LU's trailing updates run on two streams beside the panels; the
    result must not depend on how they interleave: the same system solved
    three times gives bit-identical solutions and refinement histories.
    n = 20000 takes the 4-rows-a-thread panel and long overlaps."""
    torch = pytest.importorskip("torch")
    n = 20000
    g = torch.Generator(device="cuda").manual_seed(7)
    a = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    b = torch.randn(n, 1, dtype=torch.float64, device="cuda", generator=g)
    sh = torch.cuda.current_stream().cuda_stream
    runs = []
    for _ in range(3):
        x = torch.zeros(n, 1, dtype=torch.float64, device="cuda")
        res = zg.MpirResult()
        r = zg.lib().zml_gpu_dgesv_mpir(n, 1, a.data_ptr(), n, b.data_ptr(), n, x.data_ptr(), n,
                                        3, 1, 1e-14, 30, res, sh)
        torch.cuda.synchronize()
        assert r == 0, zg.last_error()
        assert res.converged
        runs.append((x.cpu().numpy(), [res.berr_history[i] for i in range(res.iters + 1)]))
    for x, hist in runs[1:]:
        assert hist == runs[0][1]
        np.testing.assert_array_equal(x, runs[0][0])


# ---- the ill-conditioned sweep: refinement, or the FP64 fallback ------------

@pytest.mark.parametrize("kappa", [1e6, 1e10])
@pytest.mark.parametrize("prec", [3, 2])  # bf16x3, fp32 factors; GMRES-IR
def test_mpir_kappa_sweep_n2048_reaches_fp64_lu(prec, kappa):
    """A = U diag(s) V^T, s_i = kappa^(-(i-1)/(n-1)).  zml_dgesv_mpir refines
    until the backward error is the FP64 LU's; where the low-precision factors
    cannot take it there (kappa u_f well above 1 leaves GMRES a spread of
    small eigenvalues that would take O(n) steps), it solves again with the
    FP64 LU and says so in fp64_fallback.  Either way the answer meets the bar."""
    n = 2048
    a = svd_matrix(n, kappa, seed=int(np.log10(kappa)) + prec)
    xt = np.random.default_rng(11).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    lu, ipiv, info = ol.getrf_mt(a)
    e64 = berr(a, ol.getrs(lu, ipiv, b), b)
    x, res = solve(a, b, prec, 1, tol=e64)
    assert res.converged, (res.berr, res.fp64_fallback, list(res.berr_history[:res.iters + 1]))
    assert berr(a, x, b) <= 2 * e64 + U64
    if prec == 2 and kappa == 1e6:
        assert not res.fp64_fallback  # FP32 factors refine this one on their own
    if res.fp64_fallback:
        assert res.info == 0


def test_mpir_fallback_when_the_low_precision_cholesky_fails():
    """BF16x3 updates of an SPD matrix with kappa 1e12 lose positive
    definiteness; zml_dposv_mpir then solves with the FP64 Cholesky."""
    n = 1024
    a = spd_matrix(n, seed=21, kappa=1e12)
    xt = np.random.default_rng(22).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    x, res = solve_spd(a, b, 3, 1)
    f, info = ol.potrf(a, 122)
    if info != 0:
        pytest.skip("not positive definite in FP64 either")
    e64 = berr(a, ol.potrs(f, b, 122), b)
    assert res.converged, (res.info, res.berr, res.fp64_fallback)
    assert berr(a, x, b) <= 2 * e64 + U64
