"""Replays zml's BLAS known-answer chains (tests/golden/blas_*.json).

A backend is a mapping  name -> callable(*args)  where array arguments are
numpy buffers (float64, or complex128 for the complex fixtures
blas_z*.json) that the callable updates in place, and a complex scalar
argument is a Python complex.  The same fixture drives the oracle (CPU) and
the C ABI of the GPU library.
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    with open(os.path.join(GOLDEN, "blas_%s.json" % name)) as f:
        return json.load(f)


def replay(fixture, call, zero_rtol=0.0):
    """Runs every step; returns (n_checked, failures).

    zero_rtol > 0: an expectation of exactly 0 (which zml's
    expectApproxEqRel(0, x, tol) meets only with x == 0, i.e. a cancellation
    that its own loop order happens to make exact) is met when |x| is within
    zero_rtol of the largest entry of that array -- for a backend that sums
    in another order.  Every other expectation is checked as written."""
    arrays, failures, checked = {}, [], 0
    for st in fixture["steps"]:
        op = st["op"]
        if op == "alloc":
            dt = np.complex128 if st.get("complex") else np.float64
            arrays[st["name"]] = np.zeros(st["size"], dtype=dt)
        elif op == "init":
            vals = st["values"]
            if vals and isinstance(vals[0], list):
                vals = [complex(re_, im_) for re_, im_ in vals]
            arrays[st["name"]][: len(vals)] = vals
        elif op == "call":
            args = []
            for a in st["args"]:
                if isinstance(a, dict):
                    args.append(arrays[a["arr"]] if "arr" in a else complex(*a["c"]))
                else:
                    args.append(a)
            call(st["fn"], args)
        elif op == "expect":
            got = arrays[st["arr"]][st["idx"]]
            part = st.get("part")
            got = got.real if part == "re" else got.imag if part == "im" else got
            want = st["value"]
            checked += 1
            if want == 0.0 and zero_rtol > 0.0:
                ok = abs(got) <= zero_rtol * np.abs(arrays[st["arr"]]).max()
            elif "abs" in st:  # std.testing.expectApproxEqAbs
                ok = abs(got - want) <= st["abs"]
            elif st["rel"] == 0.0:
                ok = got == want
            else:  # std.testing.expectApproxEqRel
                ok = abs(got - want) <= st["rel"] * max(abs(got), abs(want)) or got == want
            if not ok:
                failures.append((st["arr"], st["idx"], want, got))
    return checked, failures
