"""Shared helpers for the GPU parity tests."""
import ctypes as C

import numpy as np

EPS64 = 2.0 ** -53


def P(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def gaussian(m, n=None, seed=0, order="F"):
    rng = np.random.default_rng(seed)
    return np.asarray(rng.standard_normal((m, n or m)), order=order)


def spd(n, seed=0, shift=1.0):
    g = gaussian(n, seed=seed)
    return np.asfortranarray(g @ g.T / n + shift * np.eye(n))


def perm_from_ipiv(ipiv, m):
    perm = np.arange(m)
    for i, p in enumerate(ipiv):
        perm[[i, p - 1]] = perm[[p - 1, i]]
    return perm


def lu_backward_error(a, lu, ipiv):
    """||P A - L U||_F / (||A||_F * n * u)"""
    m, n = a.shape
    k = min(m, n)
    L = np.tril(lu[:, :k], -1) + np.eye(m, k)
    U = np.triu(lu[:k, :])
    pa = a[perm_from_ipiv(ipiv, m)]
    return np.linalg.norm(pa - L @ U) / (np.linalg.norm(a) * max(m, n) * EPS64)


def chol_backward_error(a, f, lower=True):
    n = a.shape[0]
    L = np.tril(f) if lower else np.triu(f).T
    return np.linalg.norm(a - L @ L.T) / (np.linalg.norm(a) * n * EPS64)


def pivot_margins(a):
    """Per-column relative gap between the chosen pivot and the runner-up,
    replayed with numpy partial pivoting (used to skip pivot comparisons
    after a near-tie, where a different summation order may flip them)."""
    a = np.array(a, dtype=np.float64, copy=True)
    m, n = a.shape
    gaps = []
    for k in range(min(m, n)):
        col = np.abs(a[k:, k])
        if col.size < 2:
            gaps.append(np.inf)
        else:
            top = np.sort(col)[-2:]
            gaps.append((top[1] - top[0]) / max(top[1], 1e-300))
        p = k + int(np.argmax(col))
        a[[k, p]] = a[[p, k]]
        if a[k, k] != 0:
            a[k + 1:, k] /= a[k, k]
            a[k + 1:, k + 1:] -= np.outer(a[k + 1:, k], a[k, k + 1:])
    return np.array(gaps)
