"""zml_gpu_dgetrf_noalloc: the FP64 LU for callers that cannot allocate.

Callers inside a CUDA-graph capture, or whose device memory is owned by
another allocator, cannot let the library call cudaMalloc.  This entry point
takes its scratch from a static device array instead.  It must produce the
same factorization as zml_gpu_dgetrf (the test allows the parity tolerance of
the other LU tests, |dLU| <= 1e-9 max|LU|, identical pivots and info), on two
calls in a row -- the scratch keeps the previous call's contents, so the
second call checks that everything that must start at zero is cleared.

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu

TOL = 1e-9


def factor(entry, a):
    import torch
    m, n = a.shape
    da = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()  # column-major a
    dp = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    info = np.zeros(1, dtype=np.int32)
    rc = getattr(zg.lib(), entry)(m, n, da.data_ptr(), m, dp.data_ptr(),
                                  info.ctypes.data_as(C.c_void_p), None)
    assert rc == 0, (entry, rc, zg.last_error())
    return da.cpu().numpy().T, dp.cpu().numpy(), int(info[0])


@pytest.mark.parametrize("m,n,seed", [(700, 700, 1), (1536, 1200, 2)])
def test_noalloc_matches_dgetrf_twice(m, n, seed):
    rng = np.random.default_rng(seed)
    for call in range(2):  # two calls in a row on the shared scratch
        a = rng.standard_normal((m, n))
        if call == 1:
            a[:, 17] = 0.0  # second call: a zero pivot, so info must not leak between calls
        lu_ref, piv_ref, info_ref = factor("zml_gpu_dgetrf", a)
        lu, piv, info = factor("zml_gpu_dgetrf_noalloc", a)
        np.testing.assert_array_equal(piv, piv_ref)
        assert info == info_ref == (18 if call == 1 else 0)
        assert np.abs(lu - lu_ref).max() <= TOL * np.abs(lu_ref).max()


def test_noalloc_rejects_too_many_rows():
    m = 1 << 20  # far more rows than one panel holds in shared memory
    info = np.zeros(1, dtype=np.int32)
    rc = zg.lib().zml_gpu_dgetrf_noalloc(m, 1, None, m, None, info.ctypes.data_as(C.c_void_p),
                                         None)
    assert rc == -1005
    assert "exceeds" in zg.last_error()
