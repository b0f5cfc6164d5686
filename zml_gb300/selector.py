"""Learned precision selector: data, labels, training and evaluation.

The solve itself is native: zml_gpu_dgesv_auto walks the precision ladder
BF16 -> FP16 -> BF16x3 -> FP32 (GMRES-IR, at most 10 steps each) -> FP64 LU.
Its BF16 attempt comes first and its first two refinement steps are the probe
that completes the 16 input features; given a model, the ladder resumes at
the class the network predicts instead of the next rung, and the FP64 LU is
the fallback of every path.  Without a model the call is the plain ladder:
the method without the selector, and the label generator (the class it ends
on is the lowest precision whose refinement converges within 10 steps).

This module is the host side around it:

* `generate` -- the matrix families of the selector workload: Gaussian, SPD
  (G diag(s) G^T + d I, d log-uniform in [1e-8, 1]), diagonally dominant,
  rows scaled by 10^U(-6,6); kappa log-uniform via A = U diag(s) V^T with U, V
  the orthogonal factors of seeded Gaussian matrices and
  s_i = kappa^(-(i-1)/(n-1)).
* `build_dataset` -- features and labels from the native ladder.
* `train` -- Adam on the library's own MLP forward/backward/Adam kernels
  (BF16 operands, FP32 accumulation), with checkpoint / resume.
* `evaluate` -- held-out matrices solved with and without the network.
"""
import ctypes as C
import json
import math
import os
import time

import numpy as np

from . import AutoResult, last_error, lib, shard

CLASSES = ["bf16", "fp16", "bf16x3", "fp32", "fp64"]
NF, NH, NO = 16, 64, 5
DEFAULT_CONFIDENCE = 0.9


def num_params():
    return lib().zml_gpu_mlp_num_params()


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


# ---------------------------------------------------------------------------
# matrices
def generate(torch, kind, n, kappa, seed, dev):
    """n x n FP64 matrix of family `kind` (0 Gaussian, 1 SPD, 2 diagonally
    dominant, 3 row-scaled) with singular values kappa^(-i/(n-1)) before the
    family's modification.  Returns (t, m): t's storage is the column-major
    matrix (t = m^T, row-major), m the logical matrix."""
    g = torch.Generator(device=dev).manual_seed(int(seed))
    s = float(kappa) ** (-torch.arange(n, dtype=torch.float64, device=dev) / max(1, n - 1))
    q1, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=dev, generator=g))
    if kind == 1:
        d = 10.0 ** (-8.0 * float(torch.rand(1, dtype=torch.float64, device=dev, generator=g)))
        m = (q1 * s) @ q1.T + d * torch.eye(n, dtype=torch.float64, device=dev)
    else:
        q2, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=dev, generator=g))
        m = (q1 * s) @ q2.T
        if kind == 2:
            m = m + torch.diag(m.abs().sum(1))
        elif kind == 3:
            r = 10.0 ** (12.0 * torch.rand(n, 1, dtype=torch.float64, device=dev, generator=g) - 6.0)
            m = r * m
    t = m.T.contiguous()
    return t, t.T


def sample_specs(count, seed, nmin=64, nmax=1024):
    """(kind, n, kappa, seed) per matrix: n log-uniform in [nmin, nmax], the
    four families equally likely, kappa log-uniform in [1e1, 1e14]."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(nmin), math.log(nmax), count)).astype(int)
    kind = rng.integers(0, 4, count)
    kappa = 10.0 ** rng.uniform(1, 14, count)
    return [(int(k), int(nn), float(kp), int(seed) * 1000003 + i)
            for i, (k, nn, kp) in enumerate(zip(kind, n, kappa))]


def rhs(torch, m, seed):
    """b = A x_true with x_true iid U(-1, 1) (seeded)."""
    g = torch.Generator(device=m.device).manual_seed(int(seed) + 7)
    xt = torch.rand(m.shape[0], 1, dtype=torch.float64, device=m.device, generator=g) * 2 - 1
    return (m @ xt).contiguous()


# ---------------------------------------------------------------------------
# the native ladder
def solve_auto(torch, t, b, x, n, model=None, confidence=DEFAULT_CONFIDENCE, max_iter=10):
    """zml_gpu_dgesv_auto on device tensors (t: column-major A, b, x: n x
    nrhs column-major).  model: float32 numpy array of
    zml_gpu_selector_model_floats() values, or None for the plain ladder."""
    res = AutoResult()
    mp = None
    if model is not None:
        model = np.ascontiguousarray(model, dtype=np.float32)
        mp = model.ctypes.data_as(C.c_void_p)
    r = lib().zml_gpu_dgesv_auto(n, b.shape[1] if b.dim() == 2 else 1, t.data_ptr(), n,
                                 b.data_ptr(), n, x.data_ptr(), n, mp, float(confidence),
                                 max_iter, C.byref(res), _stream(torch))
    if r != 0:
        raise RuntimeError("zml_gpu_dgesv_auto: %d %s" % (r, last_error()))
    return res


def fp64_ms(torch, t, b, n):
    """Wall time of the plain FP64 LU solve (zml_gpu_dgetrf + zml_gpu_dgetrs)."""
    a = t.clone()
    bb = b.clone()
    piv = torch.zeros(n, dtype=torch.int32, device=t.device)
    info = C.c_int(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = _stream(torch)
    if lib().zml_gpu_dgetrf(n, n, a.data_ptr(), n, piv.data_ptr(), C.byref(info), st) != 0:
        raise RuntimeError(last_error())
    if lib().zml_gpu_dgetrs(b"N", n, 1, a.data_ptr(), n, piv.data_ptr(), bb.data_ptr(), n, st) != 0:
        raise RuntimeError(last_error())
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) * 1e3


def _run_workers(torch, dev, idx, workers, fn, warm=None):
    """fn(i) for every i of idx on `workers` host threads, each with its own
    CUDA stream (the library keeps its workspaces per stream, so the solves
    of different threads share nothing).  Small solves occupy a few SMs, so
    several in flight raise throughput; the first exception is re-raised."""
    import threading
    errors = []

    def body(part):
        try:
            torch.cuda.set_device(dev)
            with torch.cuda.stream(torch.cuda.Stream(device=dev)):
                if warm is not None and part:
                    warm()
                for i in part:
                    if errors:
                        return
                    fn(i)
                torch.cuda.current_stream().synchronize()
        except Exception as e:  # noqa: BLE001 - re-raised below
            errors.append(e)

    workers = max(1, min(workers, len(idx)))
    if workers == 1:
        body(idx)
    else:
        th = [threading.Thread(target=body, args=(idx[w::workers],)) for w in range(workers)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    if errors:
        raise errors[0]


def build_dataset(torch, specs, dev, log=None, rank=0, world=1, workers=1):
    """Features (float32, len x 16), labels (int32) and the plain ladder's
    wall time (ms; inflated when workers > 1) per matrix.  With world > 1
    (an initialised process group) each rank labels its n^3-balanced
    contiguous share and every rank returns the gathered whole."""
    lo, hi = shard.shard([s[1] for s in specs], rank, world)
    X = np.zeros((len(specs), NF), dtype=np.float32)
    y = np.zeros(len(specs), dtype=np.int32)
    ms = np.zeros(len(specs))
    done = [0]

    def label(i):
        kind, n, kappa, seed = specs[i]
        t, m = generate(torch, kind, n, kappa, seed, dev)
        b = rhs(torch, m, seed)
        x = torch.zeros_like(b)
        res = solve_auto(torch, t, b, x, n)
        if not res.converged:
            raise RuntimeError("ladder did not converge: kind %d n %d kappa %.3g berr %.3g"
                               % (kind, n, kappa, res.berr))
        X[i] = np.frombuffer(res.features, dtype=np.float32)
        y[i] = res.used
        ms[i] = res.ms
        done[0] += 1
        if log and done[0] % 2500 == 0:
            log("  %d/%d matrices labelled" % (done[0], hi - lo))

    nmax = max([s[1] for s in specs[lo:hi]], default=0)
    _run_workers(torch, dev, list(range(lo, hi)), workers, label,
                 (lambda: warm_up(torch, dev, nmax)) if workers > 1 and nmax else None)
    if world > 1:
        for plo, phi, pX, py, pms in shard.gather((lo, hi, X[lo:hi], y[lo:hi], ms[lo:hi])):
            X[plo:phi], y[plo:phi], ms[plo:phi] = pX, py, pms
    return X, y, ms


# ---------------------------------------------------------------------------
# training on the library's kernels
def init_params(seed=0):
    """Glorot-uniform weights, zero biases, in the packed parameter layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((NF, NH), (NH, NH), (NH, NO)):
        lim = math.sqrt(6.0 / (fan_in + fan_out))
        parts.append(rng.uniform(-lim, lim, fan_out * fan_in).astype(np.float32))
        parts.append(np.zeros(fan_out, dtype=np.float32))
    p = np.concatenate(parts)
    assert p.size == num_params()
    return p


def normalizer(X):
    return X.mean(0).astype(np.float32), (X.std(0) + 1e-3).astype(np.float32)


def save_checkpoint(path, state):
    tmp = path + ".tmp.npz"
    np.savez(tmp, **{k: np.asarray(v) for k, v in state.items()})
    os.replace(tmp, path)


def load_checkpoint(path):
    with np.load(path) as d:
        return {k: d[k] for k in d.files}


def train(torch, X, y, dev, epochs=300, batch=256, lr=3e-3, weight_decay=1e-5, seed=0,
          checkpoint=None, every=50, resume=None):
    """Adam on zml_gpu_mlp_gradients / zml_gpu_mlp_adam.  checkpoint: path
    written every `every` epochs with the parameters, both Adam moments, the
    step and epoch counters and the feature normalisation; resume: such a
    file, from which training continues exactly (the epoch shuffles are
    replayed from `seed`)."""
    L = lib()
    rng = np.random.default_rng(seed)
    if resume:
        st = load_checkpoint(resume)
        p, m, v = st["params"], st["m"], st["v"]
        step, epoch0 = int(st["step"]), int(st["epoch"])
        mu, sd = st["mu"], st["sd"]
        hist = list(st.get("loss_history", []))
        for _ in range(epoch0):
            rng.permutation(len(X))
    else:
        p = init_params(seed)
        m = np.zeros_like(p)
        v = np.zeros_like(p)
        step, epoch0 = 0, 0
        mu, sd = normalizer(X)
        hist = []
    Xn = torch.from_numpy(((X - mu) / sd).astype(np.float32)).to(dev)
    yd = torch.from_numpy(y.astype(np.int32)).to(dev)
    P = torch.from_numpy(np.array(p, np.float32)).to(dev)
    M = torch.from_numpy(np.array(m, np.float32)).to(dev)
    V = torch.from_numpy(np.array(v, np.float32)).to(dev)
    G = torch.zeros_like(P)
    loss = torch.zeros(batch, dtype=torch.float32, device=dev)
    work = torch.zeros(int(L.zml_gpu_mlp_work_floats(batch)), dtype=torch.float32, device=dev)
    st = _stream(torch)

    def state(ep):
        return {"params": P.cpu().numpy(), "m": M.cpu().numpy(), "v": V.cpu().numpy(),
                "step": step, "epoch": ep, "mu": mu, "sd": sd,
                "loss_history": np.array(hist, dtype=np.float64)}

    for ep in range(epoch0, epochs):
        perm = torch.from_numpy(rng.permutation(len(X))).to(dev)
        tot = torch.zeros((), dtype=torch.float64, device=dev)
        for s0 in range(0, len(X), batch):
            idx = perm[s0:s0 + batch]
            B = int(idx.numel())
            xb = Xn[idx].contiguous()
            yb = yd[idx].contiguous()
            if L.zml_gpu_mlp_gradients(B, xb.data_ptr(), yb.data_ptr(), P.data_ptr(), G.data_ptr(),
                                       loss.data_ptr(), work.data_ptr(), st) != 0:
                raise RuntimeError(last_error())
            step += 1
            if L.zml_gpu_mlp_adam(P.data_ptr(), G.data_ptr(), M.data_ptr(), V.data_ptr(), lr, 0.9,
                                  0.999, 1e-8, step, weight_decay, st) != 0:
                raise RuntimeError(last_error())
            tot += loss[:B].double().sum()
        hist.append(float(tot.item()) / len(X))
        if checkpoint and (ep + 1) % every == 0:
            save_checkpoint(checkpoint, state(ep + 1))
    return state(epochs)


def trained_model():
    """The network trained at the selector workload's scale (50000 matrices,
    n log-uniform in [64, 2048], 300 epochs), as the flat array
    zml_gpu_dgesv_auto takes: parameters, feature means, feature scales."""
    path = os.path.join(os.path.dirname(__file__), "data", "selector_model.npz")
    with np.load(path) as d:
        return model_array({"params": d["params"], "mu": d["mu"], "sd": d["sd"]})


def model_array(state):
    """The flat model zml_gpu_dgesv_auto takes: parameters, means, scales."""
    a = np.concatenate([np.asarray(state["params"], np.float32), np.asarray(state["mu"], np.float32),
                        np.asarray(state["sd"], np.float32)])
    assert a.size == lib().zml_gpu_selector_model_floats()
    return a


def predict_proba(torch, X, state, dev):
    """Class probabilities of the network (zml_gpu_mlp_forward) for features X."""
    L = lib()
    Xn = torch.from_numpy(((X - state["mu"]) / state["sd"]).astype(np.float32)).to(dev)
    B = Xn.shape[0]
    P = torch.from_numpy(np.asarray(state["params"], np.float32)).to(dev)
    logits = torch.zeros(B, NO, dtype=torch.float32, device=dev)
    work = torch.zeros(int(L.zml_gpu_mlp_work_floats(B)), dtype=torch.float32, device=dev)
    if L.zml_gpu_mlp_forward(B, Xn.data_ptr(), P.data_ptr(), logits.data_ptr(), work.data_ptr(),
                             _stream(torch)) != 0:
        raise RuntimeError(last_error())
    z = logits.cpu().numpy().astype(np.float64)
    e = np.exp(z - z.max(1, keepdims=True))
    return e / e.sum(1, keepdims=True)


def decide(proba, confidence=DEFAULT_CONFIDENCE):
    """Smallest class whose cumulative probability reaches `confidence`."""
    return np.argmax(np.cumsum(proba, axis=1) >= confidence - 1e-7, axis=1)


# ---------------------------------------------------------------------------
# evaluation
def warm_up(torch, dev, nmax):
    """One hard matrix of the largest size through the whole ladder, so that
    every workspace has its final size before anything is timed."""
    t, m = generate(torch, 0, nmax, 1e14, 12345, dev)
    b = rhs(torch, m, 12345)
    solve_auto(torch, t, b, torch.zeros_like(b), nmax)
    fp64_ms(torch, t, b, nmax)


def evaluate(torch, specs, state, dev, confidence=DEFAULT_CONFIDENCE, log=None, rank=0, world=1,
             workers=1, time_sample=0):
    """Solves every held-out matrix with the plain ladder and with the ladder
    guided by the network (on `workers` concurrent streams), recording
    labels, choices and convergence.  Then `time_sample` of them, spread
    over the n range, are solved again one at a time -- ladder, guided (in
    alternating order) and the FP64 LU -- for the time comparison.  Returns
    per-matrix records and a summary (sharded like build_dataset)."""
    model = model_array(state)
    lo, hi = shard.shard([s[1] for s in specs], rank, world)
    recs = {}
    done = [0]

    def solve_both(i, timed=False):
        kind, n, kappa, seed = specs[i]
        t, m = generate(torch, kind, n, kappa, seed, dev)
        b = rhs(torch, m, seed)
        runs = {}
        for which in ((None, model) if i % 2 == 0 else (model, None)):
            x = torch.zeros_like(b)
            runs["guided" if which is not None else "ladder"] = solve_auto(
                torch, t, b, x, n, which, confidence)
        lad, gui = runs["ladder"], runs["guided"]
        r = {"kind": kind, "n": n, "kappa": kappa, "label": lad.used,
             "predicted": gui.predicted, "used": gui.used, "attempts": gui.attempts,
             "ladder_attempts": lad.attempts, "converged": bool(gui.converged),
             "ladder_converged": bool(lad.converged), "berr": gui.berr,
             "features": list(np.frombuffer(lad.features, dtype=np.float32).tolist())}
        if timed:
            r.update({"ladder_ms": lad.ms, "guided_ms": gui.ms, "fp64_ms": fp64_ms(torch, t, b, n)})
        return r

    def conv(i):
        recs[i] = solve_both(i)
        done[0] += 1
        if log and done[0] % 1000 == 0:
            log("  %d/%d held-out matrices" % (done[0], hi - lo))

    nmax = max([s[1] for s in specs[lo:hi]], default=0)
    _run_workers(torch, dev, list(range(lo, hi)), workers, conv,
                 (lambda: warm_up(torch, dev, nmax)) if workers > 1 and nmax else None)
    # the timing sample: every k-th matrix in order of n, one at a time
    order = sorted(range(lo, hi), key=lambda i: specs[i][1])
    k = max(1, len(order) // time_sample) if time_sample > 0 else 0
    for i in (order[::k][:time_sample] if k else []):
        r = solve_both(i, timed=True)
        recs[i].update({key: r[key] for key in ("ladder_ms", "guided_ms", "fp64_ms")})
    rec = [recs[i] for i in range(lo, hi)]
    if world > 1:
        rec = [r for part in shard.gather(rec) for r in part]
    return rec, summarize(rec)


BUCKETS = ((64, 128), (128, 256), (256, 512), (512, 1024), (1024, 2049))


def summarize(rec):
    lab = np.array([r["label"] for r in rec])
    pred = np.array([r["predicted"] if r["predicted"] >= 0 else r["label"] for r in rec])
    probed = np.array([r["predicted"] >= 0 for r in rec])
    timed = [r for r in rec if "guided_ms" in r]
    lad = np.array([r["ladder_ms"] for r in timed])
    gui = np.array([r["guided_ms"] for r in timed])
    f64 = np.array([r["fp64_ms"] for r in timed])
    by_n = []
    for a, b in BUCKETS:
        sel = [r for r in timed if a <= r["n"] < b]
        if sel:
            by_n.append({"n": [a, b - 1], "timed": len(sel),
                         "ladder_ms_median": float(np.median([r["ladder_ms"] for r in sel])),
                         "guided_ms_median": float(np.median([r["guided_ms"] for r in sel])),
                         "fp64_ms_median": float(np.median([r["fp64_ms"] for r in sel])),
                         "guided_ms_total": float(sum(r["guided_ms"] for r in sel)),
                         "fp64_ms_total": float(sum(r["fp64_ms"] for r in sel))})
    conv_by_n = []
    for a, b in BUCKETS:
        sel = [r for r in rec if a <= r["n"] < b]
        if sel:
            conv_by_n.append({"n": [a, b - 1], "matrices": len(sel),
                              "converged_guided": float(np.mean([r["converged"] for r in sel])),
                              "label_counts": np.bincount([r["label"] for r in sel],
                                                          minlength=NO).tolist()})
    out = {
        "matrices": len(rec),
        "label_counts": np.bincount(lab, minlength=NO).tolist(),
        "converged_guided": float(np.mean([r["converged"] for r in rec])),
        "converged_ladder": float(np.mean([r["ladder_converged"] for r in rec])),
        # among matrices the probe did not settle: the network's class is at or
        # above the label (its attempt is expected to converge) / exactly it
        "choice_at_or_above_label": float(np.mean(pred[probed] >= lab[probed])) if probed.any() else 1.0,
        "choice_exact": float(np.mean(pred[probed] == lab[probed])) if probed.any() else 1.0,
        "probe_settled": float(np.mean(~probed)),
        "attempts_ladder": float(np.mean([r["ladder_attempts"] for r in rec])),
        "attempts_guided": float(np.mean([r["attempts"] for r in rec])),
        "by_n": conv_by_n,
    }
    if timed:
        out.update({
            "timed": len(timed),
            "ladder_ms_total": float(lad.sum()),
            "guided_ms_total": float(gui.sum()),
            "fp64_ms_total": float(f64.sum()),
            "speedup_vs_ladder": float(lad.sum() / gui.sum()),
            "speedup_vs_fp64": float(f64.sum() / gui.sum()),
            "time_by_n": by_n,
        })
    return out


def main():
    import argparse
    import torch
    ap = argparse.ArgumentParser(description="train and evaluate the precision selector")
    ap.add_argument("--train", type=int, default=50000)
    ap.add_argument("--heldout", type=int, default=5000)
    ap.add_argument("--nmax", type=int, default=2048)
    ap.add_argument("--workers", type=int, default=8,
                    help="concurrent solves (threads, one CUDA stream each)")
    ap.add_argument("--time-sample", type=int, default=500,
                    help="held-out matrices timed one at a time for the time comparison")
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--confidence", type=float, default=DEFAULT_CONFIDENCE)
    ap.add_argument("--checkpoint", default=None)
    ap.add_argument("--resume", default=None)
    ap.add_argument("--out", default=None, help="model .npz to write")
    ap.add_argument("--report", default=None, help="summary JSON to write")
    a = ap.parse_args()
    # under torchrun: one rank per GPU, labelling and evaluation sharded by
    # n^3-balanced index ranges, results gathered on the host; every rank
    # trains the same network on the gathered data (deterministic kernels)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def log(s):
        if rank == 0:
            print(s, flush=True)

    t0 = time.time()
    warm_up(torch, dev, a.nmax)
    Xtr, ytr, _ = build_dataset(torch, sample_specs(a.train, seed=1, nmax=a.nmax), dev, log,
                                rank, world, a.workers)
    log("labelled %d training matrices in %.0f s, classes %s" %
        (a.train, time.time() - t0, np.bincount(ytr, minlength=NO).tolist()))
    t1 = time.time()
    state = train(torch, Xtr, ytr, dev, epochs=a.epochs, checkpoint=a.checkpoint,
                  resume=a.resume)
    log("trained %d epochs in %.1f s, loss %.4f -> %.4f" %
        (a.epochs, time.time() - t1, state["loss_history"][0], state["loss_history"][-1]))
    if a.out and rank == 0:
        save_checkpoint(a.out, state)
    t2 = time.time()
    rec, summ = evaluate(torch, sample_specs(a.heldout, seed=2, nmax=a.nmax), state, dev,
                         a.confidence, log, rank, world, a.workers, a.time_sample)
    log("evaluated %d held-out matrices in %.0f s" % (a.heldout, time.time() - t2))
    summ.update({"train": a.train, "nmax": a.nmax, "epochs": a.epochs, "workers": a.workers,
                 "label_seconds": t1 - t0, "train_seconds": t2 - t1,
                 "confidence": a.confidence, "train_label_counts":
                 np.bincount(ytr, minlength=NO).tolist(),
                 "loss_first": float(state["loss_history"][0]),
                 "loss_last": float(state["loss_history"][-1]),
                 "seconds": time.time() - t0})
    summ["ranks"] = world
    log(json.dumps(summ))
    if a.report and rank == 0:
        with open(a.report, "w") as f:
            json.dump({"summary": summ, "records": rec}, f)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
