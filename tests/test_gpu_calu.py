"""Tournament-pivoted FP32 LU (zml_gpu_sgetrf_calu), the mixed solver's factor.

Tournament pivoting chooses each 32-column sub-panel's pivots among rows the
cluster's thread blocks nominate from their own rows, so its pivots may differ
from partial pivoting's (the oracle's getrf2); what must hold is the
factorization itself:
  * ipiv is LAPACK's form (1-based rows at or below their step, within m);
  * P A = L U to FP32 accuracy: ||PA - LU||_F / (||A||_F max(m, n) u32) < 16;
  * the multipliers stay bounded, |L| <= 16 (partial pivoting would give 1;
    tournament pivoting's are not bounded by 1 but stay small in practice);
  * a column that is zero throughout gives info = its 1-based index.
Heights cover one thread block, partly filled clusters, the 2- and
4-rows-a-thread layouts (m > 8192, m > 16384) and ragged sub-panels.  The
mixed solver must reach FP64 backward error with either panel.
"""
import numpy as np
import pytest

import zml_gb300 as zg
from gpu_util import P, gaussian, perm_from_ipiv

pytestmark = pytest.mark.gpu
EPS32 = 2.0 ** -24


def calu(a):
    import torch
    m, n = a.shape
    da = torch.from_numpy(np.asfortranarray(a.astype(np.float32)).T.copy()).cuda()
    dp = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    info = np.zeros(1, dtype=np.int32)
    rc = zg.lib().zml_gpu_sgetrf_calu(m, n, da.data_ptr(), m, dp.data_ptr(), P(info), None)
    assert rc == 0, zg.last_error()
    return da.cpu().numpy().T.astype(np.float64), dp.cpu().numpy(), int(info[0])


def check(a, lu, ipiv):
    m, n = a.shape
    k = min(m, n)
    assert np.all((ipiv >= np.arange(1, k + 1)) & (ipiv <= m))
    L = np.tril(lu[:, :k], -1) + np.eye(m, k)
    U = np.triu(lu[:k, :])
    a32 = a.astype(np.float32).astype(np.float64)
    pa = a32[perm_from_ipiv(ipiv, m)]
    be = np.linalg.norm(pa - L @ U) / (np.linalg.norm(a32) * max(m, n) * EPS32)
    assert be < 16, be
    assert np.abs(L).max() <= 16, np.abs(L).max()


@pytest.mark.parametrize("m,n", [(128, 128), (300, 200), (700, 700), (2048, 2048),
                                 (8192, 256), (9000, 130), (16384, 256), (20000, 256),
                                 (1000, 77)])
def test_calu_factorization(m, n):
    a = gaussian(m, n, seed=m + n)
    lu, ipiv, info = calu(a)
    assert info == 0
    check(a, lu, ipiv)


def test_calu_zero_column_info():
    a = gaussian(600, 300, seed=3)
    a[:, 45] = 0.0
    lu, ipiv, info = calu(a)
    assert info == 46
    assert np.all((ipiv >= 1) & (ipiv <= 600))


@pytest.mark.parametrize("tournament", [1, 0])
def test_mixed_solve_with_either_panel(tournament):
    n = 3000
    a = gaussian(n, seed=77)
    xt = np.random.default_rng(78).uniform(-1, 1, (n, 1))
    b = np.asfortranarray(a @ xt)
    L = zg.lib()
    prev = L.zml_gpu_mixed_panel(tournament)
    try:
        x = np.zeros((n, 1), order="F")
        res = zg.MpirResult()
        assert L.zml_dgesv_mpir(102, n, 1, P(a), n, P(b), n, P(x), n, 3, 1, 0.0, 30, res) == 0
    finally:
        L.zml_gpu_mixed_panel(prev)
    assert res.converged and not res.fp64_fallback, (res.berr, res.iters)
    r = b - a @ x
    berr = np.abs(r).max() / (np.abs(a).sum(1).max() * np.abs(x).max() + np.abs(b).max())
    assert berr < 64 * 2.0 ** -53
