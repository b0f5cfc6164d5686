"""Host-side checks of the precision selector (no GPU).

The MLP oracle's exact FP64 gradients against central finite differences,
its BF16 emulation, the matrix generator, the data sampling, checkpoint
files and the argument checks of the auto-solve entry points.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import zml_gb300 as zg

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import mlp_oracle as mo  # noqa: E402


def _batch(B=24, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((B, mo.NF))
    y = rng.integers(0, mo.NO, B)
    P = rng.standard_normal(mo.NPARAMS) * 0.3
    return X, y, P


def test_parameter_layout_matches_library():
    assert mo.NPARAMS == zg.lib().zml_gpu_mlp_num_params() == 5573
    assert zg.lib().zml_gpu_selector_model_floats() == 5573 + 32


def test_exact_gradients_match_finite_differences():
    X, y, P = _batch()
    G = mo.gradients_exact(X, y, P)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.choice(np.arange(*mo.OFF[k]), 12, replace=False)
                          if mo.OFF[k][1] - mo.OFF[k][0] > 12 else np.arange(*mo.OFF[k])
                          for k in ("W1", "b1", "W2", "b2", "W3", "b3")])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(P)
        e[i] = h
        fd = (mo.loss_exact(X, y, P + e) - mo.loss_exact(X, y, P - e)) / (2 * h)
        assert abs(fd - G[i]) <= 1e-6 + 1e-5 * abs(G[i]), (i, fd, G[i])


def test_bf16_rounding_ties_to_even():
    one = np.float32(1.0)
    v = np.array([1.0, 1 + 2.0 ** -8, 1 + 3 * 2.0 ** -8, -(1 + 2.0 ** -9), 3.14159265, 0.0],
                 dtype=np.float32)
    r = mo.bf16(v)
    assert r[0] == one and r[1] == one              # tie -> even mantissa
    assert r[2] == np.float32(1 + 2.0 ** -6)        # tie -> even (rounds up)
    assert r[3] == -one
    assert r[4] == np.float32(3.140625)
    assert r[5] == 0


def test_emulated_gradients_near_exact():
    X, y, P = _batch(B=64, seed=3)
    Ge, loss = mo.gradients_emulated(X.astype(np.float32), y, P.astype(np.float32))
    Gx = mo.gradients_exact(mo.bf16(X.astype(np.float32)), y, mo.bf16(P.astype(np.float32)))
    assert np.linalg.norm(Ge - Gx) <= 3e-2 * np.linalg.norm(Gx)
    assert abs(loss.mean() - mo.loss_exact(X, y, P)) <= 5e-2 * abs(mo.loss_exact(X, y, P))


def test_adam_oracle_first_step_is_signed_lr():
    P = np.array([1.0, -2.0, 0.5])
    G = np.array([0.3, -0.1, 0.0])
    Pn, M, V = mo.adam(P, G, np.zeros(3), np.zeros(3), 1e-2, 0.9, 0.999, 1e-12, 1, 0.0)
    assert np.allclose(Pn, P - 1e-2 * np.sign(G), atol=1e-9)


def test_features_oracle_on_known_matrix():
    A = np.array([[4.0, 1.0, 0.0], [1.0, 5.0, 2.0], [0.0, 2.0, 6.0]])
    f = mo.features(A)
    assert np.isclose(f[0], np.log2(3))
    assert f[6] == 0                                 # symmetric
    assert np.isclose(f[4], np.log10(min(4 / 1, 5 / 3, 6 / 2)), atol=1e-6)
    assert np.isclose(f[11], 0, atol=1e-6)           # ||A||_1 = ||A||_inf


def test_generator_families():
    torch = pytest.importorskip("torch")
    from zml_gb300 import selector as sel
    dev = torch.device("cpu")
    t, m = sel.generate(torch, 0, 40, 1e6, 5, dev)
    assert torch.equal(t.T, m)
    sv = np.linalg.svd(m.numpy(), compute_uv=False)
    assert np.isclose(sv[0] / sv[-1], 1e6, rtol=1e-6)
    _, s = sel.generate(torch, 1, 40, 1e6, 6, dev)
    s = s.numpy()
    assert np.allclose(s, s.T, atol=1e-14) and np.linalg.eigvalsh(s).min() > 0
    _, d = sel.generate(torch, 2, 40, 1e6, 7, dev)
    d = np.abs(d.numpy())
    assert np.all(2 * np.diag(d) >= d.sum(1) * (1 - 1e-12))  # weakly dominant rows
    _, r = sel.generate(torch, 3, 40, 1e6, 8, dev)
    rn = np.abs(r.numpy()).sum(1)
    assert rn.max() / rn.min() > 10
    # deterministic in the seed
    assert torch.equal(sel.generate(torch, 3, 40, 1e6, 8, dev)[0], sel.generate(torch, 3, 40, 1e6, 8, dev)[0])


def test_sample_specs_ranges_and_determinism():
    from zml_gb300 import selector as sel
    a = sel.sample_specs(2000, seed=1, nmin=64, nmax=2048)
    assert a == sel.sample_specs(2000, seed=1, nmin=64, nmax=2048)
    assert a != sel.sample_specs(2000, seed=2, nmin=64, nmax=2048)
    kinds, ns, kaps, seeds = zip(*a)
    assert set(kinds) == {0, 1, 2, 3}
    assert 64 <= min(ns) and max(ns) <= 2048
    assert 10 <= min(kaps) and max(kaps) <= 1e14
    assert len(set(seeds)) == len(seeds)
    # log-uniform: about half below the geometric midpoint
    assert 0.45 < np.mean(np.array(ns) < np.sqrt(64 * 2048)) < 0.55


def test_checkpoint_round_trip(tmp_path):
    from zml_gb300 import selector as sel
    st = {"params": np.arange(5.0, dtype=np.float32), "m": np.ones(5, np.float32),
          "v": np.zeros(5, np.float32), "step": 17, "epoch": 3, "mu": np.zeros(16, np.float32),
          "sd": np.ones(16, np.float32), "loss_history": np.array([1.5, 1.2, 1.0])}
    p = str(tmp_path / "ck.npz")
    sel.save_checkpoint(p, st)
    back = sel.load_checkpoint(p)
    assert int(back["step"]) == 17 and int(back["epoch"]) == 3
    for k in ("params", "m", "v", "mu", "sd", "loss_history"):
        assert np.array_equal(back[k], st[k])
    assert not os.path.exists(p + ".tmp.npz")


def test_decide_cumulative_threshold():
    from zml_gb300 import selector as sel
    pr = np.array([[0.6, 0.3, 0.05, 0.05, 0.0], [0.1, 0.1, 0.1, 0.1, 0.6], [1, 0, 0, 0, 0]])
    assert list(sel.decide(pr, 0.9)) == [1, 4, 0]
    assert list(sel.decide(pr, 0.5)) == [0, 4, 0]


def test_auto_argument_checks():
    L = zg.lib()
    a = np.zeros(16)
    ap = a.ctypes.data_as(C.c_void_p)
    model = np.zeros(L.zml_gpu_selector_model_floats(), np.float32)
    mp = model.ctypes.data_as(C.c_void_p)
    res = zg.AutoResult()
    assert L.zml_dgesv_auto(103, 4, 1, ap, 4, ap, 4, ap, 4, None, 0.9, 10, C.byref(res)) == -1
    assert L.zml_dgesv_auto(102, -1, 1, ap, 4, ap, 4, ap, 4, None, 0.9, 10, C.byref(res)) == -2
    assert L.zml_dgesv_auto(102, 4, 1, ap, 3, ap, 4, ap, 4, None, 0.9, 10, C.byref(res)) == -5
    assert L.zml_dgesv_auto(102, 4, 1, ap, 4, ap, 4, ap, 4, mp, 0.0, 10, C.byref(res)) == -11
    assert L.zml_dgesv_auto(102, 4, 1, ap, 4, ap, 4, ap, 4, mp, 1.5, 10, C.byref(res)) == -11
    assert L.zml_gpu_dgesv_auto(4, 1, ap, 4, ap, 2, ap, 4, None, 0.9, 10, C.byref(res), None) == -6
    assert L.zml_dgesv_auto(102, 0, 1, ap, 1, ap, 1, ap, 1, None, 0.9, 10, C.byref(res)) == 0
    assert C.sizeof(zg.AutoResult) == 128
