"""CPU oracle of the precision selector's kernels (test infrastructure only).

The selector has no counterpart in the reference (zml's solve path is FP64
only), so this oracle is a restatement of the selector's own definition,
checked two ways by the tests: the exact FP64 gradients against central
finite differences of the loss, and the GPU kernels against the emulated
arithmetic below.

* MLP 16 -> 64 -> 64 -> 5, ReLU, softmax cross-entropy (mean over the batch).
  Parameters packed W1[64][16] b1[64] W2[64][64] b2[64] W3[5][64] b3[5].
* Emulated arithmetic of the kernels: operands of every product (inputs,
  weights, activations, back-propagated errors) rounded to BF16 (round to
  nearest even); dot products accumulated in FP32 by fused multiply-adds in
  index order; batch sums in sample order.  An FP32 fma(a, b, c) of FP32
  operands is emulated as round32(a * b + c) in FP64 (the product is exact;
  the sum's double rounding differs from a single rounding in rare ties).
* Features 0..11 of an n x n FP64 matrix, as defined by the feature kernels.
"""
import numpy as np

NF, NH, NO = 16, 64, 5
OFF = {}
_o = 0
for _name, _size in (("W1", NH * NF), ("b1", NH), ("W2", NH * NH), ("b2", NH),
                     ("W3", NO * NH), ("b3", NO)):
    OFF[_name] = (_o, _o + _size)
    _o += _size
NPARAMS = _o


def unpack(P):
    W1 = P[slice(*OFF["W1"])].reshape(NH, NF)
    W2 = P[slice(*OFF["W2"])].reshape(NH, NH)
    W3 = P[slice(*OFF["W3"])].reshape(NO, NH)
    return W1, P[slice(*OFF["b1"])], W2, P[slice(*OFF["b2"])], W3, P[slice(*OFF["b3"])]


def bf16(x):
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(x.shape)


def f32(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32)


def fma32(a, b, c):
    return f32(a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64))


def _dense(W, x):
    """Emulated sum_k fma(W[o, k], x[s, k]) in k order: W (O, K), x (S, K) -> (S, O)."""
    acc = np.zeros((x.shape[0], W.shape[0]), dtype=np.float32)
    for k in range(W.shape[1]):
        acc = fma32(W[None, :, k], x[:, k:k + 1], acc)
    return acc


def forward_emulated(X, P):
    W1, b1, W2, b2, W3, b3 = (bf16(t) for t in unpack(np.asarray(P, np.float32)))
    x = bf16(X)
    H1 = bf16(np.maximum(f32(_dense(W1, x) + b1), 0))
    H2 = bf16(np.maximum(f32(_dense(W2, H1) + b2), 0))
    Z = f32(_dense(W3, H2) + b3)
    return H1, H2, Z


def gradients_emulated(X, y, P):
    """(G, per-sample loss) with the kernels' rounding and summation order."""
    X = np.asarray(X, np.float32)
    B = X.shape[0]
    W1, b1, W2, b2, W3, b3 = (bf16(t) for t in unpack(np.asarray(P, np.float32)))
    x = bf16(X)
    H1, H2, Z = forward_emulated(X, P)
    m = Z.max(1, keepdims=True)
    e = np.exp(f32(Z - m))
    den = np.zeros((B, 1), np.float32)
    for o in range(NO):
        den = f32(den + e[:, o:o + 1])
    p = f32(e / den)
    onehot = np.zeros_like(p)
    onehot[np.arange(B), y] = 1
    dZ = bf16(f32(f32(p - onehot) / np.float32(B)))
    loss = -(Z[np.arange(B), y] - m[:, 0] - np.log(den[:, 0]))
    dH2 = np.where(H2 > 0, bf16(_dense(W3.T, dZ)), 0).astype(np.float32)
    dH1 = np.where(H1 > 0, bf16(_dense(W2.T, dH2)), 0).astype(np.float32)
    G = np.zeros(NPARAMS, np.float32)

    def outer_sum(d, a):  # sum over samples of d[s, o] * a[s, k] in sample order
        acc = np.zeros((d.shape[1], a.shape[1]), np.float32)
        for s in range(B):
            acc = fma32(d[s][:, None], a[s][None, :], acc)
        return acc

    def col_sum(d):
        acc = np.zeros(d.shape[1], np.float32)
        for s in range(B):
            acc = f32(acc + d[s])
        return acc

    G[slice(*OFF["W1"])] = outer_sum(dH1, x).ravel()
    G[slice(*OFF["b1"])] = col_sum(dH1)
    G[slice(*OFF["W2"])] = outer_sum(dH2, H1).ravel()
    G[slice(*OFF["b2"])] = col_sum(dH2)
    G[slice(*OFF["W3"])] = outer_sum(dZ, H2).ravel()
    G[slice(*OFF["b3"])] = col_sum(dZ)
    return G, loss.astype(np.float32)


# ---- exact FP64 network (no rounding) --------------------------------------
def loss_exact(X, y, P):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(P, np.float64))
    X = np.asarray(X, np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0)
    H2 = np.maximum(H1 @ W2.T + b2, 0)
    Z = H2 @ W3.T + b3
    m = Z.max(1, keepdims=True)
    lse = m[:, 0] + np.log(np.exp(Z - m).sum(1))
    return float(np.mean(lse - Z[np.arange(len(y)), y]))


def gradients_exact(X, y, P):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(P, np.float64))
    X = np.asarray(X, np.float64)
    B = X.shape[0]
    A1 = X @ W1.T + b1
    H1 = np.maximum(A1, 0)
    A2 = H1 @ W2.T + b2
    H2 = np.maximum(A2, 0)
    Z = H2 @ W3.T + b3
    p = np.exp(Z - Z.max(1, keepdims=True))
    p /= p.sum(1, keepdims=True)
    dZ = p.copy()
    dZ[np.arange(B), y] -= 1
    dZ /= B
    dH2 = (dZ @ W3) * (A2 > 0)
    dH1 = (dH2 @ W2) * (A1 > 0)
    G = np.zeros(NPARAMS)
    G[slice(*OFF["W1"])] = (dH1.T @ X).ravel()
    G[slice(*OFF["b1"])] = dH1.sum(0)
    G[slice(*OFF["W2"])] = (dH2.T @ H1).ravel()
    G[slice(*OFF["b2"])] = dH2.sum(0)
    G[slice(*OFF["W3"])] = (dZ.T @ H2).ravel()
    G[slice(*OFF["b3"])] = dZ.sum(0)
    return G


def adam(P, G, M, V, lr, b1, b2, eps, t, wd):
    """One Adam step with decoupled-free L2 term g + wd * p (FP64)."""
    P, G, M, V = (np.asarray(a, np.float64) for a in (P, G, M, V))
    g = G + wd * P
    M = b1 * M + (1 - b1) * g
    V = b2 * V + (1 - b2) * g * g
    mh = M / (1 - b1 ** t)
    vh = V / (1 - b2 ** t)
    return P - lr * mh / (np.sqrt(vh) + eps), M, V


# ---- features --------------------------------------------------------------
def features(A):
    """Features 0..11 of the square FP64 matrix A (logical, any layout)."""
    A = np.asarray(A, np.float64)
    n = A.shape[0]
    aA = np.abs(A)
    r1 = aA.sum(1)
    c1 = aA.sum(0)
    d = np.abs(np.diag(A))
    off = r1 - d
    F = np.sqrt((A * A).sum())
    E = aA.max()
    S = np.sqrt(((A - A.T) ** 2).sum())
    dd = d / np.maximum(off, 1e-300)
    lg = lambda v: np.log10(max(v, 1e-300))  # noqa: E731
    R, r0, Cc, c0 = r1.max(), r1.min(), c1.max(), c1.min()
    f = np.zeros(16)
    f[0] = np.log2(n)
    f[1] = lg(F / np.sqrt(n))
    f[2] = lg(R / max(r0, 1e-300))
    f[3] = lg(Cc / max(c0, 1e-300))
    f[4] = lg(dd.min())
    f[5] = np.mean(np.log10(np.maximum(dd, 1e-300)))
    f[6] = S / max(F, 1e-300)
    f[7] = lg(E * n / max(F, 1e-300))
    f[8] = lg(d.max() / max(d.min(), 1e-300))
    f[9] = lg(R / max(F, 1e-300))
    f[10] = lg(d.max() / max(R, 1e-300))
    f[11] = lg(Cc / max(R, 1e-300))
    return f.astype(np.float32)
