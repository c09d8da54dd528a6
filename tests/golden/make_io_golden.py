"""Regenerates tests/golden/io_cases.npz from the reference itself: its COO
text reader (read_G_sparse, IOfn.cpp:21-54) and its p-value code
(Calculate_Pvalue and helpers, Pvalue.cpp:85-235), both compiled unmodified
into oracle/_ref/io_harness by oracle/Makefile.

    make -C oracle && python tests/golden/make_io_golden.py

COO cases: small texts that exercise the reader's quirks (the final-line
duplicate of the feof loop, a trailing partial triplet, weights summed over
duplicates then pruned, scientific notation, CR/LF and tab separators) and
one larger seeded weighted file.  P-value cases: seeded vector pairs of
several lengths and correlations, plus the degenerate branches (length 2
and 3, identical and constant vectors).  Nothing at test time needs the
reference checkout or the harness.
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
HARNESS = ROOT / "oracle" / "_ref" / "io_harness"


def coo_cases():
    rng = np.random.default_rng(7)
    cases = [
        ("binary_trailing_newline", "1 2\n2 3\n3 3\n", 3, 3, 0),
        ("binary_no_newline", "1 2\n2 3\n3 3", 3, 3, 0),
        ("binary_partial_last", "1 2\n2 3\n3\n", 3, 3, 0),
        ("binary_duplicates", "1 1\n1 1\n2 3\n1 1\n3 2\n", 3, 3, 0),
        ("weighted_dups_prune", "1 2 0.5\n1 2 0.25\n2 1 0\n3 3 1e-20\n2 2 -1.5\n", 3, 3, 1),
        ("weighted_sci_tabs_crlf", "1\t2\t2.5e-1\r\n3 1 1E0\r\n2\t3\t7\r\n", 3, 3, 1),
        ("weighted_partial_last", "1 2 0.5\n2 3 1.5\n3 1\n", 3, 3, 1),
        ("binary_spaces_between", "  1   2 \n\n 2 1\n\t3 3  \n", 3, 3, 0),
    ]
    n1, n2, m = 400, 300, 20000
    r = rng.integers(1, n1 + 1, m)
    c = rng.integers(1, n2 + 1, m)
    v = np.round(rng.uniform(0.1, 3.0, m), 4)
    lines = "".join(f"{a} {b} {w:g}\n" for a, b, w in zip(r, c, v))
    cases.append(("weighted_large", lines, n1, n2, 1))
    r = rng.integers(1, n1 + 1, m)
    c = rng.integers(1, n2 + 1, m)
    cases.append(("binary_large", "".join(f"{a}\t{b}\n" for a, b in zip(r, c)), n1, n2, 0))
    return cases


def pvalue_cases():
    rng = np.random.default_rng(11)
    out = []
    for n, rho in ((10, 0.5), (100, 0.1), (100, -0.7), (1000, 0.02), (5000, 0.3), (25, 0.95)):
        x = rng.standard_normal(n)
        y = rho * x + np.sqrt(1 - rho * rho) * rng.standard_normal(n)
        out.append((f"gauss_n{n}_rho{rho}", x, y))
    x = np.maximum(rng.standard_normal(300), 0)  # membership-like: many zeros
    y = np.maximum(0.6 * x + 0.4 * rng.standard_normal(300), 0)
    out.append(("nonneg_n300", x, y))
    out.append(("len2", np.array([1.0, 2.0]), np.array([3.0, 1.0])))
    out.append(("len3", np.array([1.0, 2.0, 4.0]), np.array([3.0, 1.0, 2.0])))
    z = rng.standard_normal(50)
    out.append(("identical", z, z.copy()))
    out.append(("constant_x", np.full(40, 2.0), rng.standard_normal(40)))
    return out


def main():
    if not HARNESS.exists():
        raise SystemExit(f"{HARNESS} missing: run make -C oracle with the reference mounted")
    data = {}
    names = []
    with tempfile.TemporaryDirectory() as td:
        for name, text, n1, n2, dt in coo_cases():
            f = Path(td) / f"{name}.txt"
            f.write_text(text)
            res = subprocess.run([str(HARNESS), "readcoo", str(f), str(n1), str(n2), str(dt)],
                                 capture_output=True, text=True, check=True).stdout.splitlines()
            # the reference prints "reading G" first
            res = [l for l in res if not l.startswith("reading")]
            rows, cols, nnz = (int(t) for t in res[0].split())
            trip = np.array([[float(t) for t in l.split()] for l in res[1:]]).reshape(-1, 3)
            data[f"coo_{name}_text"] = np.array(text)
            data[f"coo_{name}_shape"] = np.array([n1, n2, dt])
            data[f"coo_{name}_triplets"] = trip
            names.append(name)
        pnames = []
        for name, x, y in pvalue_cases():
            f = Path(td) / f"{name}.txt"
            f.write_text("\n".join(f"{v:.17g}" for v in np.concatenate([x, y])) + "\n")
            res = subprocess.run([str(HARNESS), "pvalue", str(f), str(len(x))],
                                 capture_output=True, text=True, check=True).stdout.split()
            data[f"pv_{name}_x"] = x
            data[f"pv_{name}_y"] = y
            data[f"pv_{name}_out"] = np.array([float(t) for t in res[-3:]])
            pnames.append(name)
    data["coo_names"] = np.array(names)
    data["pv_names"] = np.array(pnames)
    np.savez_compressed(ROOT / "tests" / "golden" / "io_cases.npz", **data)
    print("wrote", len(names), "COO cases and", len(pnames), "p-value cases")


if __name__ == "__main__":
    main()
