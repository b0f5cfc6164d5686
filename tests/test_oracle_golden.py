"""The oracle against zml's own known-answer BLAS tests (CPU only).

The fixtures in tests/golden/ are the literal expectations of zml's
test/linalg/blas/{gemm,trsm,syrk,trmm,gemv,ger,iamax,nrm2}.zig (real parts)
and of the cf64 parts and herk / geru / gerc (blas_z*.json); an oracle that
fails one of them does not restate the reference.
"""
import json
import os

import numpy as np
import pytest

import oracle_lib as ol
from golden_replay import GOLDEN, load_fixture, replay


def oracle_call(name, args):
    f = ol.fn(name)
    conv = [ol.ptr(a) if isinstance(a, np.ndarray) else a for a in args]
    r = f(*conv)
    assert r == 0, (name, args[:8], r)


@pytest.mark.parametrize("name", ["gemm", "trsm", "syrk", "trmm", "gemv", "ger"])
def test_oracle_matches_reference_fixtures(name):
    fx = load_fixture(name)
    checked, failures = replay(fx, oracle_call)
    assert checked > 0
    assert not failures, failures[:5]


def oracle_zcall(name, args):
    """A complex fixture's call on the zo_z_ routines: complex scalars go by
    value as the struct the signature names (herk's alpha / beta are real)."""
    f = ol.fn(name, np.complex128)
    conv = []
    for a, t in zip(args, f.argtypes):
        if isinstance(a, np.ndarray):
            conv.append(ol.ptr(a))
        elif t is ol.CF64:
            conv.append(ol.cs(a))
        else:
            conv.append(a)
    r = f(*conv)
    assert r == 0, (name, args[:8], r)


@pytest.mark.parametrize("name", ["gemm", "trsm", "syrk", "herk", "trmm", "gemv", "geru", "gerc"])
def test_complex_oracle_matches_reference_fixtures(name):
    """The cf64 parts of zml's BLAS tests (and its complex-only herk, geru,
    gerc tests) replayed on the complex oracle."""
    fx = load_fixture("z" + name)
    checked, failures = replay(fx, oracle_zcall)
    assert checked > 0
    assert not failures, failures[:5]


def test_oracle_iamax_and_nrm2_fixtures():
    with open(os.path.join(GOLDEN, "blas_scalars.json")) as f:
        sc = json.load(f)
    ia = sc["iamax"]
    x = np.zeros(ia["n"])
    x[ia["ones"]] = 1
    for c in ia["cases"]:
        assert ol.fn("iamax")(c["n"], ol.ptr(x), c["incx"]) == c["expect"]
    nr = sc["nrm2"]
    x = np.arange(1, nr["n"] + 1, dtype=np.float64)
    for c in nr["cases"]:
        got = ol.fn("nrm2")(c["n"], ol.ptr(x), c["incx"])
        assert abs(got - c["expect"]) <= c["rel"] * abs(c["expect"])


def test_ilaenv_and_lamch():
    lib = ol.load()
    assert lib.zo_ilaenv(1, b"DGETRF", 512, 512, -1, -1) == 64
    assert lib.zo_ilaenv(1, b"DPOTRF", 512, -1, -1, -1) == 64
    assert lib.zo_ilaenv(1, b"DGEQRF", 512, 512, -1, -1) == 32
    assert lib.zo_ilaenv(3, b"DGEQRF", 512, 512, -1, -1) == 128
    assert ol.fn("lamch")(b"e") == 2.0 ** -53
    assert ol.fn("lamch")(b"s") == np.finfo(np.float64).tiny


def test_trsm_as_written_lda_quirk():
    """zml reads b[k + j*lda] in the left/no-trans divisions; with lda != ldb
    the as-written result differs from the ldb form, with lda == ldb not."""
    lib = ol.load()
    rng = np.random.default_rng(1)
    m, n = 4, 3
    a = np.asfortranarray(np.triu(rng.standard_normal((6, m))) + 4 * np.eye(6, m))
    b0 = np.asfortranarray(rng.standard_normal((m, n)))
    out = {}
    for mode in (1, 0):
        lib.zo_set_trsm_as_written(mode)
        b = b0.copy(order="F")
        ol.fn("trsm")(102, 141, 121, 111, 131, m, n, 1.0, ol.ptr(a), 6, ol.ptr(b), m)
        out[mode] = b
    lib.zo_set_trsm_as_written(1)
    assert not np.array_equal(out[0], out[1])
    ref = np.linalg.solve(a[:m, :m], b0)
    np.testing.assert_allclose(out[0], ref, rtol=1e-12, atol=1e-12)
