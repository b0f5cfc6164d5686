"""The synchronous C entries read device operands only after the work the
caller queued before the call on the legacy default stream (PyTorch's default
stream): a matrix filled by a copy queued behind seconds-long GEMMs is
factored as filled, bit for bit the same as after an explicit synchronize."""
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu


def test_device_operands_wait_for_default_stream():
    import torch
    n = 1536
    g = torch.Generator(device="cuda").manual_seed(5)
    S = torch.randn(n, n, dtype=torch.float64, device="cuda", generator=g)
    busy = torch.randn(4096, 4096, dtype=torch.float64, device="cuda", generator=g)
    piv0 = torch.zeros(n, dtype=torch.int32, device="cuda")
    F0 = S.clone()
    torch.cuda.synchronize()
    assert zg.lib().LAPACKE_dgetrf(102, n, n, F0.data_ptr(), n, piv0.data_ptr()) == 0

    F = torch.zeros_like(S)
    piv = torch.zeros_like(piv0)
    torch.cuda.synchronize()
    for _ in range(6):  # FP64 GEMMs queued ahead of the fill, several ms each
        busy = (busy @ busy) * (1.0 / 4096)
    F.copy_(S)
    assert zg.lib().LAPACKE_dgetrf(102, n, n, F.data_ptr(), n, piv.data_ptr()) == 0
    torch.cuda.synchronize()
    assert torch.equal(piv, piv0)
    assert torch.equal(F, F0)
