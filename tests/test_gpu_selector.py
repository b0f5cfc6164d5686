"""GPU tests of the precision selector: feature and MLP kernels against the
CPU oracle, training with checkpoint/resume, the native precision ladder,
and what the trained network gains over the ladder without it."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

import zml_gb300 as zg

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import mlp_oracle as mo  # noqa: E402

U64 = 2.0 ** -53


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no GPU")
    t.cuda.set_device(0)
    return t


@pytest.fixture(scope="module")
def sel():
    from zml_gb300 import selector
    return selector


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("kind,n", [(0, 100), (1, 257), (2, 64), (3, 130)])
def test_features_match_oracle(torch, sel, kind, n):
    dev = torch.device("cuda", 0)
    t, m = sel.generate(torch, kind, n, 1e5, 11 + kind, dev)
    f = torch.full((16,), -7.0, dtype=torch.float32, device=dev)
    assert zg.lib().zml_gpu_selector_features(n, t.data_ptr(), n, f.data_ptr(), _stream(torch)) == 0
    got = f.cpu().numpy()
    ref = mo.features(m.cpu().numpy())
    assert np.allclose(got[:12], ref[:12], rtol=1e-5, atol=1e-4), (got, ref)
    assert np.all(got[12:] == 0)


def _mlp_case(torch, B, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((B, 16)).astype(np.float32)
    y = rng.integers(0, 5, B).astype(np.int32)
    from zml_gb300 import selector
    P = (selector.init_params(seed) + 0.05 * rng.standard_normal(mo.NPARAMS)).astype(np.float32)
    return X, y, P


@pytest.mark.parametrize("B", [1, 37, 256])
def test_mlp_forward_matches_oracle(torch, B):
    X, y, P = _mlp_case(torch, B, 1)
    dev = torch.device("cuda", 0)
    Xd, Pd = torch.from_numpy(X).to(dev), torch.from_numpy(P).to(dev)
    Z = torch.zeros(B, 5, dtype=torch.float32, device=dev)
    W = torch.zeros(int(zg.lib().zml_gpu_mlp_work_floats(B)), dtype=torch.float32, device=dev)
    assert zg.lib().zml_gpu_mlp_forward(B, Xd.data_ptr(), Pd.data_ptr(), Z.data_ptr(), W.data_ptr(),
                                        _stream(torch)) == 0
    _, _, Zr = mo.forward_emulated(X, P)
    z = Z.cpu().numpy()
    assert np.max(np.abs(z - Zr)) <= 1e-3 * max(1.0, np.max(np.abs(Zr)))


@pytest.mark.parametrize("B", [5, 200])
def test_mlp_gradients_match_oracle(torch, B):
    """Gradient check: the kernels against the emulated BF16/FP32 oracle
    (tight) and against the exact FP64 gradient (BF16-level)."""
    X, y, P = _mlp_case(torch, B, 2)
    dev = torch.device("cuda", 0)
    L = zg.lib()
    Xd, yd, Pd = (torch.from_numpy(a).to(dev) for a in (X, y, P))
    G = torch.zeros(mo.NPARAMS, dtype=torch.float32, device=dev)
    loss = torch.zeros(B, dtype=torch.float32, device=dev)
    W = torch.zeros(int(L.zml_gpu_mlp_work_floats(B)), dtype=torch.float32, device=dev)
    assert L.zml_gpu_mlp_gradients(B, Xd.data_ptr(), yd.data_ptr(), Pd.data_ptr(), G.data_ptr(),
                                   loss.data_ptr(), W.data_ptr(), _stream(torch)) == 0
    g = G.cpu().numpy().astype(np.float64)
    Ge, le = mo.gradients_emulated(X, y, P)
    # a rare BF16 rounding flip of one intermediate moves one term by 2^-8
    assert np.linalg.norm(g - Ge) <= 2e-3 * np.linalg.norm(Ge)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        sl = slice(*mo.OFF[k])
        assert np.linalg.norm(g[sl] - Ge[sl]) <= 1e-2 * np.linalg.norm(Ge[sl]) + 1e-7, k
    assert np.allclose(loss.cpu().numpy(), le, rtol=1e-4, atol=1e-5)
    Gx = mo.gradients_exact(X, y, P)
    assert np.linalg.norm(g - Gx) <= 5e-2 * np.linalg.norm(Gx)


def test_adam_matches_oracle(torch):
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    n = mo.NPARAMS
    P, G = rng.standard_normal(n).astype(np.float32), rng.standard_normal(n).astype(np.float32)
    M, V = (0.1 * rng.standard_normal(n)).astype(np.float32), rng.random(n).astype(np.float32)
    d = [torch.from_numpy(a.copy()).to(dev) for a in (P, G, M, V)]
    assert zg.lib().zml_gpu_mlp_adam(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                     d[3].data_ptr(), 1e-3, 0.9, 0.999, 1e-8, 7, 1e-4,
                                     _stream(torch)) == 0
    Pr, Mr, Vr = mo.adam(P, G, M, V, 1e-3, 0.9, 0.999, 1e-8, 7, 1e-4)
    assert np.allclose(d[0].cpu().numpy(), Pr, rtol=1e-5, atol=1e-6)
    assert np.allclose(d[2].cpu().numpy(), Mr, rtol=1e-5, atol=1e-7)
    assert np.allclose(d[3].cpu().numpy(), Vr, rtol=1e-5, atol=1e-7)


def _toy_data(n=1500, seed=5):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 16)).astype(np.float32)
    y = np.clip(np.floor(X[:, 12] + X[:, 0] * 0.5 + 2.5), 0, 4).astype(np.int32)
    return X, y


def test_training_learns_and_resumes_exactly(torch, sel, tmp_path):
    dev = torch.device("cuda", 0)
    X, y = _toy_data()
    straight = sel.train(torch, X, y, dev, epochs=40, batch=256, seed=3)
    ck = str(tmp_path / "ck.npz")
    sel.train(torch, X, y, dev, epochs=20, batch=256, seed=3, checkpoint=ck, every=20)
    resumed = sel.train(torch, X, y, dev, epochs=40, batch=256, seed=3, resume=ck)
    assert int(resumed["step"]) == int(straight["step"])
    assert np.array_equal(resumed["params"], straight["params"])
    assert np.array_equal(resumed["m"], straight["m"]) and np.array_equal(resumed["v"], straight["v"])
    assert np.allclose(resumed["loss_history"], straight["loss_history"])
    h = straight["loss_history"]
    assert h[-1] < 0.5 * h[0]
    acc = np.mean(np.argmax(sel.predict_proba(torch, X, straight, dev), 1) == y)
    assert acc > 0.85


def _residual_berr(m, x, b):
    m, x, b = (a.cpu().numpy() for a in (m, x, b))
    r = b - m @ x
    return np.abs(r).max() / (np.abs(m).sum(1).max() * np.abs(x).max() + np.abs(b).max())


def test_ladder_easy_and_hard(torch, sel):
    dev = torch.device("cuda", 0)
    for kind, n, kappa, expect in ((0, 300, 10.0, 0), (0, 300, 1e14, 4), (2, 200, 1e13, None)):
        t, m = sel.generate(torch, kind, n, kappa, 99, dev)
        b = sel.rhs(torch, m, 99)
        x = torch.zeros_like(b)
        r = sel.solve_auto(torch, t, b, x, n)
        assert r.converged and r.predicted == -1
        if expect is not None:
            assert r.used == expect
        if r.used == 0:
            assert r.attempts == 1
        assert r.attempts >= 1 + (r.used >= 1) * 1
        berr = _residual_berr(m, x, b)
        assert berr <= 64 * U64 and abs(berr - r.berr) <= 0.5 * berr + 4 * U64  # roundoff level


def test_model_that_predicts_fp64_jumps_straight_there(torch, sel):
    dev = torch.device("cuda", 0)
    p = np.zeros(mo.NPARAMS, np.float32)
    p[mo.OFF["b3"][0] + 4] = 10.0                 # always class 4
    model = np.concatenate([p, np.zeros(16, np.float32), np.ones(16, np.float32)])
    t, m = sel.generate(torch, 0, 300, 1e14, 98, dev)
    b = sel.rhs(torch, m, 98)
    x = torch.zeros_like(b)
    r = sel.solve_auto(torch, t, b, x, 300, model, 0.9)
    assert r.predicted == 4 and r.used == 4 and r.attempts == 2 and r.converged
    assert abs(sum(r.proba) - 1) < 1e-5 and r.proba[4] > 0.99
    assert _residual_berr(m, x, b) <= 64 * U64
    # a model that always answers BF16 continues the probe's own refinement:
    # one factorization in all
    p[:] = 0
    p[mo.OFF["b3"][0]] = 10.0
    model = np.concatenate([p, np.zeros(16, np.float32), np.ones(16, np.float32)])
    t, m = sel.generate(torch, 0, 300, 10.0, 97, dev)
    b = sel.rhs(torch, m, 97)
    x = torch.zeros_like(b)
    r = sel.solve_auto(torch, t, b, x, 300, model, 0.9)
    assert r.predicted in (-1, 0) and r.used == 0 and r.attempts == 1 and r.converged
    assert r.iters >= 1 and _residual_berr(m, x, b) <= 64 * U64


def test_selector_gains_over_ladder(torch, sel):
    """Train on seeded matrices (n in [64, 384]), evaluate on held-out seeds:
    every solve converges (FP64 LU fallback), the network's first choice is
    at or above the label in most cases, and the guided ladder takes less
    time than the plain one."""
    dev = torch.device("cuda", 0)
    sel.warm_up(torch, dev, 384)
    X, y, _ = sel.build_dataset(torch, sel.sample_specs(800, seed=1, nmax=384), dev, workers=4)
    assert len(set(y.tolist())) >= 3
    state = sel.train(torch, X, y, dev, epochs=200)
    rec, s = sel.evaluate(torch, sel.sample_specs(200, seed=2, nmax=384), state, dev, workers=4,
                          time_sample=200)
    print(s)
    assert s["converged_guided"] == 1.0 and s["converged_ladder"] == 1.0
    assert s["choice_at_or_above_label"] >= 0.85
    assert s["speedup_vs_ladder"] > 1.0


def test_concurrent_labelling_equals_sequential(torch, sel):
    """Labels and features from several streams in flight are those of one
    stream: the library's state is per stream and its kernels deterministic."""
    dev = torch.device("cuda", 0)
    specs = sel.sample_specs(48, seed=5, nmax=512)
    X1, y1, _ = sel.build_dataset(torch, specs, dev, workers=1)
    X4, y4, _ = sel.build_dataset(torch, specs, dev, workers=6)
    np.testing.assert_array_equal(y1, y4)
    np.testing.assert_array_equal(X1, X4)


def test_condition_estimate_feature_tracks_kappa(torch, sel):
    """Feature 14, log10 of ||A||inf times ||z||inf after three steps of
    inverse iteration with the BF16 probe's factors, grows with the
    matrix's condition number and is close to it when the factors are
    accurate (kappa_2 = 10: kappa_inf lies within a factor n of it)."""
    dev = torch.device("cuda", 0)
    n = 256
    est = []
    for kappa in (1e1, 1e4, 1e8):
        t, m = sel.generate(torch, 0, n, kappa, 77, dev)
        b = sel.rhs(torch, m, 77)
        r = sel.solve_auto(torch, t, b, torch.zeros_like(b), n)
        est.append(float(np.frombuffer(r.features, dtype=np.float32)[14]))
    assert est[0] < est[1] < est[2], est
    assert 0.5 <= est[0] <= 1.0 + np.log10(n), est


def test_shipped_model_guides_heldout_solves(torch, sel):
    """The network shipped with the package (trained on 50000 matrices up to
    n = 2048) on held-out seeds: every solve converges, and where the probe
    did not settle the matrix the network's class is used."""
    dev = torch.device("cuda", 0)
    model = sel.trained_model()
    specs = sel.sample_specs(40, seed=2, nmax=512)
    consulted = 0
    for kind, n, kappa, seed in specs:
        t, m = sel.generate(torch, kind, n, kappa, seed, dev)
        b = sel.rhs(torch, m, seed)
        r = sel.solve_auto(torch, t, b, torch.zeros_like(b), n, model)
        assert r.converged
        if r.predicted >= 0:
            consulted += 1
            assert r.used >= r.predicted
    assert consulted >= 5
