#!/usr/bin/env python3
"""Generate the known-answer fixtures in tests/golden/ from zml's own BLAS tests.

zml's tests (test/linalg/blas/*.zig in srmadrid/zml) are chains of calls on
small integer-valued matrices, each call followed by literal expectations.
This script reads those Zig files as text and records, for the real (f64)
part of each test, a replayable list of steps:

    {"op": "alloc",  "name": "A", "size": 12}
    {"op": "init",   "name": "A", "values": [...]}
    {"op": "call",   "fn": "gemm", "args": [...]}      # enums as CBLAS codes,
                                                       # arrays as {"arr": name}
    {"op": "expect", "arr": "C", "idx": 0, "value": 95.0, "rel": 0.0}
    {"op": "expect_ret", "value": 127}                 # scalar results

The replay harness (tests/golden_replay.py) runs them against the oracle
and, on a GPU, against the C ABI.  The complex (cf64) parts, and the
complex-only herk / geru / gerc tests, go to blas_z<name>.json with complex
values as [re, im] pairs.  The fixtures are regenerated with

    python tests/golden/make_golden.py /path/to/zml

and the JSON is committed, because the reference tree is not available
where the GPU tests run.
"""
import json
import os
import re
import sys

ENUMS = {
    ".row_major": 101, ".col_major": 102,
    ".no_trans": 111, ".trans": 112, ".conj_trans": 113, ".conj_no_trans": 114,
    ".upper": 121, ".lower": 122,
    ".non_unit": 131, ".unit": 132,
    ".left": 141, ".right": 142,
}

# files whose real part is a literal chain of calls and expectations
CHAINED = ["gemm", "trsm", "syrk", "trmm", "gemv", "ger"]


def split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def ev(expr, consts):
    expr = expr.strip()
    expr = re.sub(r"@as\([^,]+,\s*", "(", expr)
    py = re.sub(r"(?<![/])/(?![/])", "//", expr)
    return eval(py, {"__builtins__": {}}, dict(consts))  # noqa: S307 - literal fixture arithmetic


def parse_chain(path, fn):
    text = open(path).read()
    # statements of the first test block, up to the first complex allocation
    body = text[text.index("test " + fn):]
    cut = body.find("alloc(cf64")
    if cut > 0:
        body = body[:cut]
    stmts = [s.strip() for s in re.split(r";\s*\n", body)]
    consts, steps, arrays = {}, [], set()
    for st in stmts:
        st = re.sub(r"//[^\n]*", "", st).strip()
        if not st:
            continue
        m = re.match(r"const (\w+)(?::\s*f64)? = (-?[\d.]+)$", st)
        if m:
            v = m.group(2)
            consts[m.group(1)] = float(v) if "." in v or ":" in st.split("=")[0] else int(v)
            continue
        m = re.match(r"(?:const|var) (\w+) = try a\.alloc\(f64, (.+)\)$", st)
        if m:
            arrays.add(m.group(1))
            steps.append({"op": "alloc", "name": m.group(1), "size": int(ev(m.group(2), consts))})
            continue
        m = re.match(r"@memcpy\((\w+)\.ptr, &\[_\]f64\{(.*)\}\)$", st, re.S)
        if m:
            vals = [float(x) for x in re.split(r"[,\s]+", m.group(2).strip()) if x]
            steps.append({"op": "init", "name": m.group(1), "values": vals})
            continue
        m = re.match(r"(\w+)\((.*)\) catch unreachable$", st, re.S)
        if m and m.group(1) == fn:
            args = []
            for a in split_args(m.group(2)):
                if a == ".{}":
                    continue
                if a in ENUMS:
                    args.append(ENUMS[a])
                elif a.endswith(".ptr"):
                    args.append({"arr": a[:-4]})
                else:
                    args.append(ev(a, consts))
            steps.append({"op": "call", "fn": fn, "args": args})
            continue
        m = re.match(r"try std\.testing\.expectEqual\((-?[\d.e+-]+), (\w+)\[(\d+)\]\)$", st)
        if m:
            steps.append({"op": "expect", "arr": m.group(2), "idx": int(m.group(3)),
                          "value": float(m.group(1)), "rel": 0.0})
            continue
        m = re.match(r"try std\.testing\.expectApproxEqRel\((-?[\d.e+-]+), (\w+)\[(\d+)\], ([\d.e+-]+)\)$", st)
        if m:
            steps.append({"op": "expect", "arr": m.group(2), "idx": int(m.group(3)),
                          "value": float(m.group(1)), "rel": float(m.group(4))})
            continue
    return {"name": fn, "source": "test/linalg/blas/%s.zig" % fn, "steps": steps}


# files with a complex (cf64) chain: the cf64 part of the real files above,
# and the complex-only routines
COMPLEX = ["gemm", "trsm", "syrk", "herk", "trmm", "gemv", "geru", "gerc"]

CINIT = re.compile(r"cf64\.init\(\s*([^,()]+?)\s*,\s*([^,()]+?)\s*\)")


def parse_chain_complex(path, fn):
    """The complex part of a test: every statement from the first cf64
    allocation on (constants are read from the whole test).  Complex values
    are [re, im] pairs, complex scalar arguments {"c": [re, im]}, and an
    expectation on a component carries "part": "re" | "im"."""
    text = open(path).read()
    body = text[text.index("test " + fn):]
    stmts = [re.sub(r"//[^\n]*", "", x).strip() for x in re.split(r";\s*\n", body)]
    consts, cconsts, steps, started = {}, {}, [], False
    for st in stmts:
        if not st:
            continue
        m = re.match(r"const (\w+)(?::\s*f64)? = (-?[\d.]+)$", st)
        if m:
            v = m.group(2)
            consts[m.group(1)] = float(v) if "." in v else int(v)
            continue
        m = re.match(r"const (\w+)(?::\s*cf64)? = " + CINIT.pattern + "$", st)
        if m:
            cconsts[m.group(1)] = [float(ev(m.group(2), consts)), float(ev(m.group(3), consts))]
            continue
        m = re.match(r"(?:const|var) (\w+) = try a\.alloc\((f64|cf64), (.+)\)$", st)
        if m:
            started = started or m.group(2) == "cf64"
            if started:
                steps.append({"op": "alloc", "name": m.group(1), "size": int(ev(m.group(3), consts)),
                              "complex": m.group(2) == "cf64"})
            continue
        if not started:
            continue
        m = re.match(r"@memcpy\((\w+)\.ptr, &\[_\](f64|cf64)\{(.*)\}\)$", st, re.S)
        if m:
            if m.group(2) == "cf64":
                vals = [[float(ev(x, consts)), float(ev(y, consts))] for x, y in CINIT.findall(m.group(3))]
            else:
                vals = [float(x) for x in re.split(r"[,\s]+", m.group(3).strip()) if x]
            steps.append({"op": "init", "name": m.group(1), "values": vals})
            continue
        m = re.match(r"(\w+)\((.*)\) catch unreachable$", st, re.S)
        if m and m.group(1) == fn:
            args = []
            for x in split_args(m.group(2)):
                if x == ".{}":
                    continue
                if x in ENUMS:
                    args.append(ENUMS[x])
                elif x.endswith(".ptr"):
                    args.append({"arr": x[:-4]})
                elif x in cconsts:
                    args.append({"c": cconsts[x]})
                elif CINIT.fullmatch(x):
                    mm = CINIT.fullmatch(x)
                    args.append({"c": [float(ev(mm.group(1), consts)), float(ev(mm.group(2), consts))]})
                else:
                    args.append(ev(x, consts))
            steps.append({"op": "call", "fn": fn, "args": args})
            continue
        m = re.match(r"try std\.testing\.expectEqual\((-?[\d.e+-]+), (\w+)\[(\d+)\](?:\.(re|im))?\)$", st)
        if m:
            steps.append({"op": "expect", "arr": m.group(2), "idx": int(m.group(3)),
                          "part": m.group(4), "value": float(m.group(1)), "rel": 0.0})
            continue
        m = re.match(r"try std\.testing\.expectApproxEqRel\((-?[\d.e+-]+), (\w+)\[(\d+)\](?:\.(re|im))?, "
                     r"([\d.e+-]+)\)$", st)
        if m:
            steps.append({"op": "expect", "arr": m.group(2), "idx": int(m.group(3)),
                          "part": m.group(4), "value": float(m.group(1)), "rel": float(m.group(5))})
            continue
        m = re.match(r"try std\.testing\.expectApproxEqAbs\((-?[\d.e+-]+), (\w+)\[(\d+)\](?:\.(re|im))?, "
                     r"([\d.e+-]+)\)$", st)
        if m:
            steps.append({"op": "expect", "arr": m.group(2), "idx": int(m.group(3)),
                          "part": m.group(4), "value": float(m.group(1)), "rel": 0.0,
                          "abs": float(m.group(5))})
            continue
    return {"name": "z" + fn, "source": "test/linalg/blas/%s.zig" % fn, "steps": steps}


def parse_scalar_tests(root):
    """iamax and nrm2: their expected scalars, read from the files."""
    out = {}
    t = open(os.path.join(root, "test/linalg/blas/iamax.zig")).read()
    real = re.sub(r"//[^\n]*", "", t[:t.index("alloc(cf64")])
    n = int(re.search(r"const n = (\d+);", real).group(1))
    ones = [int(x) for x in re.findall(r"x1\[(\d+)\] = 1;", real)]
    exp = [int(x) for x in re.findall(r"expectEqual\((\d+), result\d\)", real)]
    calls = re.findall(r"iamax\((n(?: / 2)?), x1\.ptr, (-?\d+), \.\{\}\) catch unreachable;\n\s*try", real)
    out["iamax"] = {"source": "test/linalg/blas/iamax.zig", "n": n, "ones": ones,
                    "cases": [{"n": ev(c[0], {"n": n}), "incx": int(c[1]), "expect": e}
                              for c, e in zip(calls, exp)]}
    t = open(os.path.join(root, "test/linalg/blas/nrm2.zig")).read()
    real = re.sub(r"//[^\n]*", "", t[:t.index("alloc(cf64")])
    calls = re.findall(r"nrm2\((n(?: / 2)?), x1\.ptr, (-?\d+), \.\{\}\) catch unreachable;\s*"
                       r"try std\.testing\.expectApproxEqRel\(([\d.e+-]+), result\d, ([\d.e+-]+)\)", real)
    n = int(re.search(r"const n = (\d+);", real).group(1))
    out["nrm2"] = {"source": "test/linalg/blas/nrm2.zig", "n": n, "x": "i+1",
                   "cases": [{"n": ev(c[0], {"n": n}), "incx": int(c[1]), "expect": float(c[2]),
                              "rel": float(c[3])} for c in calls]}
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <root of the srmadrid/zml tree>")
    root = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    for fn in CHAINED:
        fx = parse_chain(os.path.join(root, "test/linalg/blas/%s.zig" % fn), fn)
        n_calls = sum(1 for s in fx["steps"] if s["op"] == "call")
        n_exp = sum(1 for s in fx["steps"] if s["op"] == "expect")
        with open(os.path.join(here, "blas_%s.json" % fn), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        print("%-5s %3d calls %5d expectations" % (fn, n_calls, n_exp))
    for fn in COMPLEX:
        fx = parse_chain_complex(os.path.join(root, "test/linalg/blas/%s.zig" % fn), fn)
        n_calls = sum(1 for s in fx["steps"] if s["op"] == "call")
        n_exp = sum(1 for s in fx["steps"] if s["op"] == "expect")
        with open(os.path.join(here, "blas_z%s.json" % fn), "w") as f:
            json.dump(fx, f, separators=(",", ":"))
        print("z%-5s %3d calls %5d expectations" % (fn, n_calls, n_exp))
    sc = parse_scalar_tests(root)
    with open(os.path.join(here, "blas_scalars.json"), "w") as f:
        json.dump(sc, f, indent=1)
    print("iamax", sc["iamax"]["cases"], "nrm2", sc["nrm2"]["cases"])


if __name__ == "__main__":
    main()
