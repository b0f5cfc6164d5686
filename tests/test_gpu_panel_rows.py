"""The cooperative LU panel's rows-per-block target changes its grid, not its
result: pivots and factors are bit-identical for every setting, on the FP64
pipe path (n < 2048) and on the slice-update path (n >= 2048)."""
import ctypes as C

import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [700, 2304])
def test_panel_rows_setting_leaves_factorization_unchanged(n):
    torch = pytest.importorskip("torch")
    L = zg.lib()
    g = torch.Generator(device="cuda").manual_seed(n)
    S = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    results = []
    try:
        for rows in (0, 64, 256, 100000):
            L.zml_gpu_panel_rows(rows)
            F = S.clone()
            piv = torch.zeros(n, dtype=torch.int32, device="cuda")
            info = C.c_int(-1)
            assert L.zml_gpu_dgetrf(n, n, F.data_ptr(), n, piv.data_ptr(), C.byref(info), None) == 0
            torch.cuda.synchronize()
            assert info.value == 0
            results.append((F, piv))
    finally:
        L.zml_gpu_panel_rows(-1)
    for F, piv in results[1:]:
        assert torch.equal(piv, results[0][1])
        assert torch.equal(F, results[0][0])
