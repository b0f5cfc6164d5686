"""Batched uneven small solves (zml_gpu_batched_*) against the oracle.

Every system of the batch is checked against zml's own getrf+getrs (general)
or potrf+potrs (SPD, lower) restated by the oracle on the same input:
FP64 path -- identical pivots, factors within 1e-9 max|F|, solutions within
1e-8; FP32-factor + FP64-refinement path -- normwise backward error of every
solution within 8 u (the FP64 level).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as ol
import zml_gb300 as zg

pytestmark = pytest.mark.gpu
U = 2.0 ** -53


def make_batch(sizes, seed, nrhs=4):
    rng = np.random.default_rng(seed)
    mats, rhs, spd = [], [], []
    for i, n in enumerate(sizes):
        if i % 2 == 0:
            g = rng.standard_normal((n, n))
            a = g @ g.T / n + 0.1 * np.eye(n)
            spd.append(1)
        else:
            a = rng.standard_normal((n, n))
            spd.append(0)
        mats.append(np.asfortranarray(a))
        rhs.append(np.asfortranarray(rng.uniform(-1, 1, (n, nrhs))))
    return mats, rhs, np.array(spd, dtype=np.int32)


def run(mats, rhs, spd, prec, nrhs=4, graph=False, reps=1):
    import torch
    n = np.array([m.shape[0] for m in mats], dtype=np.int32)
    A = torch.from_numpy(np.concatenate([m.ravel(order="F") for m in mats])).cuda()
    B = torch.from_numpy(np.concatenate([b.ravel(order="F") for b in rhs])).cuda()
    X = torch.zeros_like(B)
    P = torch.zeros(int(n.sum()), dtype=torch.int32, device="cuda")
    info = torch.full((len(mats),), -7, dtype=torch.int32, device="cuda")
    iters = torch.zeros(len(mats), dtype=torch.int32, device="cuda")
    L = zg.lib()
    plan = C.c_void_p()
    assert L.zml_gpu_batched_plan_create(C.byref(plan), len(mats), n.ctypes.data_as(C.c_void_p),
                                         spd.ctypes.data_as(C.c_void_p), nrhs, prec, 10) == 0
    A0 = A.clone()
    for _ in range(reps):
        A.copy_(A0)
        f = L.zml_gpu_batched_run_graph if graph else L.zml_gpu_batched_execute
        assert f(plan, A.data_ptr(), B.data_ptr(), X.data_ptr(), P.data_ptr(), info.data_ptr(),
                 iters.data_ptr(), None) == 0, zg.last_error()
    torch.cuda.synchronize()
    L.zml_gpu_batched_plan_destroy(plan)
    out = []
    oa = ob = op = 0
    for i, m in enumerate(mats):
        k = m.shape[0]
        a = A[oa:oa + k * k].cpu().numpy().reshape(k, k, order="F")
        x = X[ob:ob + k * nrhs].cpu().numpy().reshape(k, nrhs, order="F")
        p = P[op:op + k].cpu().numpy()
        out.append((a, x, p))
        oa += k * k
        ob += k * nrhs
        op += k
    return out, info.cpu().numpy(), iters.cpu().numpy()


SIZES = [1, 2, 3, 8, 23, 24, 25, 31, 32, 33, 47, 48, 63, 64, 65, 95, 96, 100, 127, 128, 129, 159,
         160, 161, 191, 192, 200, 255, 256, 256]


def test_batched_fp64_vs_oracle():
    mats, rhs, spd = make_batch(SIZES, seed=1)
    res, info, _ = run(mats, rhs, spd, prec=0)
    assert (info == 0).all()
    for i, (a0, b) in enumerate(zip(mats, rhs)):
        a, x, p = res[i]
        if spd[i]:
            f_ref, inf = ol.potrf(a0, 122)
            x_ref = ol.potrs(f_ref, b, 122)
            scale = np.abs(f_ref).max()
            assert np.abs(np.tril(a) - np.tril(f_ref)).max() <= 1e-9 * scale, i
        else:
            f_ref, p_ref, inf = ol.getrf(a0)
            x_ref = ol.getrs(f_ref, p_ref, b)
            np.testing.assert_array_equal(p, p_ref)
            assert np.abs(a - f_ref).max() <= 1e-9 * np.abs(f_ref).max(), i
        assert inf == 0
        assert np.abs(x - x_ref).max() <= 1e-8 * max(1.0, np.abs(x_ref).max()), i


def test_batched_fp32_refined_reaches_fp64_backward_error():
    rng = np.random.default_rng(3)
    sizes = list(rng.integers(8, 257, size=120))
    mats, rhs, spd = make_batch(sizes, seed=4)
    res, info, iters = run(mats, rhs, spd, prec=1)
    assert (info == 0).all()
    for i, (a0, b) in enumerate(zip(mats, rhs)):
        a, x, _ = res[i]
        np.testing.assert_array_equal(a, a0)  # A untouched
        r = b - a0 @ x
        berr = np.abs(r).max() / (np.abs(a0).sum(1).max() * np.abs(x).max() + np.abs(b).max())
        assert berr <= 8 * U, (i, sizes[i], berr, iters[i])
    assert iters.max() >= 1


def test_batched_graph_replay_and_info_isolation():
    mats, rhs, spd = make_batch([40, 41, 130, 131, 200, 201], seed=7)
    mats[1][:, 5] = 0.0          # singular general matrix: info = 6
    mats[2][50, 50] = -1e6       # not positive definite
    res_e, info_e, _ = run(mats, rhs, spd, prec=0)
    res_g, info_g, _ = run(mats, rhs, spd, prec=0, graph=True, reps=2)
    np.testing.assert_array_equal(info_e, info_g)
    assert info_e[1] == 6 and info_e[2] > 0
    assert info_e[0] == info_e[3] == info_e[4] == info_e[5] == 0
    for (a1, x1, p1), (a2, x2, p2), i in zip(res_e, res_g, range(6)):
        if info_e[i] == 0:
            np.testing.assert_array_equal(x1, x2)


def test_batched_autotune_and_schedule():
    import torch
    L = zg.lib()
    ncls = L.zml_gpu_batched_schedule(0, None, None, 0, 0)
    chosen = np.zeros(ncls, dtype=np.int32)
    ms = np.zeros(ncls)
    st = torch.cuda.current_stream().cuda_stream
    assert L.zml_gpu_batched_autotune(0, 4, chosen.ctypes.data_as(C.c_void_p),
                                      ms.ctypes.data_as(C.c_void_p), st) == 0, zg.last_error()
    assert set(chosen.tolist()) <= {1, 2, 4, 8, 16}
    got = np.zeros(ncls, dtype=np.int32)
    edges = np.zeros(ncls, dtype=np.int32)
    L.zml_gpu_batched_schedule(0, got.ctypes.data_as(C.c_void_p), edges.ctypes.data_as(C.c_void_p),
                               ncls, 0)
    np.testing.assert_array_equal(got, chosen)
    assert (np.diff(edges) > 0).all()
