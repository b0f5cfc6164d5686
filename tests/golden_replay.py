"""Replays zml's BLAS known-answer chains (tests/golden/blas_*.json).

A backend is a mapping  name -> callable(*args)  where array arguments are
float64 numpy buffers that the callable updates in place.  The same fixture
drives the oracle (CPU) and the C ABI of the GPU library.
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fixture(name):
    with open(os.path.join(GOLDEN, "blas_%s.json" % name)) as f:
        return json.load(f)


def replay(fixture, call):
    """Runs every step; returns (n_checked, failures)."""
    arrays, failures, checked = {}, [], 0
    for st in fixture["steps"]:
        op = st["op"]
        if op == "alloc":
            arrays[st["name"]] = np.zeros(st["size"], dtype=np.float64)
        elif op == "init":
            arrays[st["name"]][: len(st["values"])] = st["values"]
        elif op == "call":
            args = [arrays[a["arr"]] if isinstance(a, dict) else a for a in st["args"]]
            call(st["fn"], args)
        elif op == "expect":
            got = arrays[st["arr"]][st["idx"]]
            want = st["value"]
            checked += 1
            if st["rel"] == 0.0:
                ok = got == want
            else:  # std.testing.expectApproxEqRel
                ok = abs(got - want) <= st["rel"] * max(abs(got), abs(want)) or got == want
            if not ok:
                failures.append((st["arr"], st["idx"], want, got))
    return checked, failures
