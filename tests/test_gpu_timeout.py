"""The bounded device-side waits give up, report and keep the context usable.

Every wait of the library (the cooperative panel's grid barrier, the polls of
the one-launch triangular solves) is bounded by zml_gpu_set_spin_limit's
limit.  Set to one try, the waits of a normal call run out long before the
other CTAs arrive: the call must return ZML_GPU_ERR_TIMEOUT -- no fault, no
hang, every index the kernels derive from the abandoned exchange kept inside
the matrix -- and, with the default limit restored, the next call must give
the oracle's result again.  No wait is made to run out by anything but the
limit: the waited-for work is ordinary.  The tensor-core GEMM's waits are not
driven to a timeout here (its copies and MMAs in flight would have to drain
first); neither FP64 call below uses it.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg
from gpu_util import gaussian

pytestmark = pytest.mark.gpu
ERR_TIMEOUT = -1004


@pytest.fixture
def lib():
    L = zg.lib()
    yield L
    assert L.zml_gpu_set_spin_limit(0) == 0  # the default again, whatever happened


def dev(a):
    import torch
    return torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()  # column-major on the device


def test_panel_grid_barrier_timeout_then_recovers(lib):
    """The cooperative FP64 panel's grid barrier (the no-allocation LU keeps
    that panel; zml_gpu_dgetrf takes panels of up to 8192 rows on one
    thread-block cluster, whose mbarrier waits suspend in hardware and do not
    run out at one try)."""
    import torch
    n = 1024
    a = gaussian(n, seed=41)
    info = np.zeros(1, dtype=np.int32)
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    da = dev(a)
    assert lib.zml_gpu_set_spin_limit(1) == 0
    rc = lib.zml_gpu_dgetrf_noalloc(n, n, da.data_ptr(), n, piv.data_ptr(),
                                    info.ctypes.data_as(C.c_void_p), None)
    assert rc == ERR_TIMEOUT, (rc, zg.last_error())
    assert "timed out" in zg.last_error()
    ipiv = piv.cpu().numpy()
    assert np.all((ipiv >= 1) & (ipiv <= n))  # the interchanges stayed inside the matrix
    assert lib.zml_gpu_set_spin_limit(0) == 0
    da = dev(a)
    assert lib.zml_gpu_dgetrf(n, n, da.data_ptr(), n, piv.data_ptr(),
                              info.ctypes.data_as(C.c_void_p), None) == 0
    lu_ref, ipiv_ref, info_ref = ol.getrf(a)
    assert info[0] == info_ref == 0
    np.testing.assert_array_equal(piv.cpu().numpy(), ipiv_ref)
    lu = da.cpu().numpy().T
    assert np.abs(lu - lu_ref).max() <= 1e-9 * np.abs(lu_ref).max()


def test_one_launch_solve_poll_timeout_then_recovers(lib):
    import torch
    n = 2048  # above the one-launch threshold: 16 blocks of 128 rows polling each other
    a = gaussian(n, seed=42)
    lu_ref, ipiv_ref, _ = ol.getrf(a)
    b = np.random.default_rng(43).uniform(-1, 1, (n, 1))
    dlu = dev(lu_ref)
    dp = torch.from_numpy(ipiv_ref.copy()).cuda()
    db = dev(b)
    assert lib.zml_gpu_set_spin_limit(1) == 0
    rc = lib.zml_gpu_dgetrs(b"N", n, 1, dlu.data_ptr(), n, dp.data_ptr(), db.data_ptr(), n,
                            None)
    assert rc == ERR_TIMEOUT, (rc, zg.last_error())
    assert lib.zml_gpu_set_spin_limit(0) == 0
    db = dev(b)
    assert lib.zml_gpu_dgetrs(b"N", n, 1, dlu.data_ptr(), n, dp.data_ptr(), db.data_ptr(), n,
                              None) == 0
    torch.cuda.synchronize()
    x = db.cpu().numpy().T
    x_ref = ol.getrs(lu_ref, ipiv_ref, b)
    assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max()
