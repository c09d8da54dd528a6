"""Regenerates the golden fixtures in this directory from the reference itself.

Run in a checkout where the reference is mounted (its path given by --ref):

    python tests/golden/make_golden.py --ref <reference checkout>

Steps per case: generate a seeded MMSB graph with this library's generator,
write it in the reference's COO text contract, run the reference's own CPU
implementation (built unmodified by oracle/Makefile into oracle/_ref with a
fixed srand seed) through oracle/ref_harness.cpp, and store graph + every
stage's output in <case>.npz.  The fixtures are what the tests compare
against; nothing at test time needs the reference checkout.
"""
from __future__ import annotations

import argparse
import importlib.util
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
PKG = ROOT / "fast-detection-of-overlapping-communities-via-online-tensor-methods_gb300"

# name: (n, k, alpha0, p_in, p_out, seed)
CASES = {
    # the reference's CPU-runnable configuration (4 x 1000 nodes, k = 10)
    "cfg1": (4000, 10, 1.0, 0.3, 0.01, 0),
    # partitions of 200 <= 20k: the full-SVD branch of SVD_symNystrom_sparse
    "fullsvd": (800, 16, 0.5, 0.3, 0.02, 1),
    # ragged partition sizes (250, 250, 250, 252), sparse, isolated nodes
    "ragged": (1002, 5, 2.0, 0.05, 0.004, 2),
}


def load_pkg():
    spec = importlib.util.spec_from_file_location("mmsb_gb300", PKG / "__init__.py",
                                                  submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["mmsb_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def read_dump(path):
    with open(path) as f:
        r, c = map(int, f.readline().split())
        data = np.loadtxt(f, ndmin=2) if r * c else np.zeros((r, c))
    return data.reshape(r, c)


def write_coo(path, blk):
    rows = np.repeat(np.arange(blk.n_rows), np.diff(blk.row_ptr))
    with open(path, "w") as f:
        f.write("".join(f"{r + 1} {c + 1}\n" for r, c in zip(rows, blk.col_idx)))


def make_case(mm, name, params, ref):
    n, k, a0, p_in, p_out, seed = params
    g = mm.generate(n, k, a0, p_in, p_out, seed)
    out = {"params": np.array([n, k, a0, p_in, p_out, seed], dtype=np.float64),
           "parts": np.array(g.parts, dtype=np.int64)}
    names = ["Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a"]
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for nm, b in zip(names, g.blocks):
            write_coo(td / f"{nm}.txt", b)
            out[f"{nm}_rp"] = b.row_ptr
            out[f"{nm}_ci"] = b.col_idx
        res = td / "out"
        nX, nA, nB, nC = g.parts
        subprocess.run([str(ROOT / "oracle" / "_ref" / "ref_harness"), str(td), str(res),
                        str(nX), str(nA), str(nB), str(nC), str(k), repr(a0)], check=True,
                       stdout=subprocess.DEVNULL)
        for nm in ["mu_a", "mu_b", "mu_c", "W", "Zb1", "Zb2", "Zc1", "Zc2", "Da", "Db", "Dc",
                   "Da_mu", "Db_mu", "Dc_mu", "phi0", "lambda", "phi", "diffloss_phi",
                   "second_term", "normprob_in", "normprob_out"]:
            out[nm] = read_dump(res / f"{nm}.txt")
        for nm in ["R_c", "R_b", "R_a"]:
            out[nm] = read_dump(res / f"{nm}.txt").astype(np.int8)
        out["pi_raw"] = read_dump(res / "pi_raw.txt").astype(np.float32)
        out["pi"] = read_dump(res / "pi.txt.dense").astype(np.float32)
        out["pi_txt_head"] = np.array((res / "pi.txt").read_text().splitlines()[:2000])
        out["white_txt"] = np.array((res / "white.txt").read_text().splitlines())
        timing = dict(l.split() for l in (res / "timing.txt").read_text().splitlines())
        out["ref_seconds"] = np.array([float(timing[s]) for s in ("whiten", "stpm", "post")])
    np.savez_compressed(Path(__file__).parent / f"{name}.npz", **out)
    print(name, g.parts, "edges", g.n_edges)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference checkout")
    ap.add_argument("cases", nargs="*", default=list(CASES))
    args = ap.parse_args()
    subprocess.run(["make", "-C", str(ROOT / "oracle"), f"REF={args.ref}"], check=True)
    mm = load_pkg()
    mm.build()
    for c in args.cases:
        make_case(mm, c, CASES[c], args.ref)


if __name__ == "__main__":
    main()
