"""zml_gpu_dgetrf_noalloc: the FP64 LU for callers that cannot allocate.

Some hosts own all device memory through their own allocator (a caching pool,
or an arena reserved at start-up); a cudaMalloc from the library would
fragment or overrun it.  Some loops must not allocate after initialisation.
This entry point takes its scratch from a static device array instead.  It
runs the same panel grid, interchanges, trsm and gemm as zml_gpu_dgetrf does
below min(m, n) = 2048 (where zml_gpu_dgetrf keeps its updates on the FP64
pipe), so at the sizes here the factors must be identical bit for bit, with
identical pivots and info.
That is checked on two calls in a row: the scratch keeps the previous call's
contents, so the second call shows that everything that must start at zero is
cleared.  A third check reads the device's free memory around a call: any
cudaMalloc takes at least one 2 MiB page, and none may happen.

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu


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
        np.testing.assert_array_equal(lu, lu_ref)


def test_noalloc_takes_no_device_memory():
    import torch
    m = n = 1024
    a = np.random.default_rng(3).standard_normal((m, n))
    da = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()
    dp = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = np.zeros(1, dtype=np.int32)
    L = zg.lib()
    # a first call loads the module (its static array) and resolves the address
    assert L.zml_gpu_dgetrf_noalloc(m, n, da.data_ptr(), m, dp.data_ptr(),
                                    info.ctypes.data_as(C.c_void_p), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        da.copy_(torch.from_numpy(np.asfortranarray(a).T.copy()))
        assert L.zml_gpu_dgetrf_noalloc(m, n, da.data_ptr(), m, dp.data_ptr(),
                                        info.ctypes.data_as(C.c_void_p), None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 < 2 << 20, (free0, free1)


def test_noalloc_rejects_too_many_rows():
    m = 1 << 20  # far more rows than one panel holds in shared memory
    info = np.zeros(1, dtype=np.int32)
    rc = zg.lib().zml_gpu_dgetrf_noalloc(m, 1, None, m, None, info.ctypes.data_as(C.c_void_p),
                                         None)
    assert rc == -1005
    assert "exceeds" in zg.last_error()
