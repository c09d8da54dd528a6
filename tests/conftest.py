"""Shared fixtures: the package (loaded from its hyphenated directory), the
FP64 oracle, and the golden fixtures produced by the reference itself."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "fast-detection-of-overlapping-communities-via-online-tensor-methods_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("cfg1", "fullsvd", "ragged")


def load_package():
    if "mmsb_gb300" in sys.modules:
        return sys.modules["mmsb_gb300"]
    spec = importlib.util.spec_from_file_location("mmsb_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["mmsb_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    if str(ROOT / "oracle") not in sys.path:
        sys.path.insert(0, str(ROOT / "oracle"))
    import mmsb_oracle
    return mmsb_oracle


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA library")


@pytest.fixture(scope="session")
def mm():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    return load_oracle()


class Golden(dict):
    """One reference fixture with convenience views."""

    def graph(self, mm):
        names = ["Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a"]
        nX, nA, nB, nC = (int(x) for x in self["parts"])
        shapes = [(nX, nA), (nX, nB), (nX, nC), (nB, nA), (nC, nA)]
        blocks = [mm.CsrBlock(r, c, self[f"{n}_rp"], self[f"{n}_ci"])
                  for n, (r, c) in zip(names, shapes)]
        return mm.Graph(blocks, (nX, nA, nB, nC))

    def scipy_blocks(self):
        import scipy.sparse as sp
        names = ["Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a"]
        nX, nA, nB, nC = (int(x) for x in self["parts"])
        shapes = [(nX, nA), (nX, nB), (nX, nC), (nB, nA), (nC, nA)]
        return [sp.csr_matrix((np.ones(len(self[f"{n}_ci"])), self[f"{n}_ci"], self[f"{n}_rp"]),
                              shape=s) for n, s in zip(names, shapes)]

    @property
    def k(self):
        return int(self["params"][1])

    @property
    def alpha0(self):
        return float(self["params"][2])

    def sketches(self):
        return tuple(self[n].astype(np.float64) for n in ("R_c", "R_b", "R_a"))

    def whitened(self):
        y = {n: self[n] for n in ("Da", "Db", "Dc")}
        for n in ("Da_mu", "Db_mu", "Dc_mu"):
            y[n] = self[n].ravel()
        return y

    def whitening(self):
        wh = {n: self[n] for n in ("W", "Zb1", "Zb2", "Zc1", "Zc2")}
        for n in ("mu_a", "mu_b", "mu_c"):
            wh[n] = self[n].ravel()
        return wh


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz") as z:
        return Golden({k: z[k] for k in z.files})


@pytest.fixture(scope="session", params=CASES)
def golden(request):
    return load_golden(request.param)


@pytest.fixture(scope="session")
def golden_cfg1():
    return load_golden("cfg1")


def align_columns(A, B):
    """Signs (and order) of B's columns matched to A's; returns aligned B."""
    s = np.sign(np.sum(A * B, axis=0))
    s[s == 0] = 1
    return B * s


def match_columns(A, B):
    """Permutation + sign of B's columns that best matches A (greedy on |cos|)."""
    An = A / np.maximum(np.linalg.norm(A, axis=0), 1e-300)
    Bn = B / np.maximum(np.linalg.norm(B, axis=0), 1e-300)
    C = np.abs(An.T @ Bn)
    perm = -np.ones(A.shape[1], dtype=int)
    used = set()
    for _ in range(A.shape[1]):
        i, j = np.unravel_index(np.argmax(C), C.shape)
        perm[i] = j
        used.add(j)
        C[i, :] = -1
        C[:, j] = -1
    Bp = B[:, perm]
    return align_columns(A, Bp), perm


def procrustes_align(A, B):
    """B Q with Q = argmin ||A - B Q|| over orthogonal Q (polar factor of B^T A)."""
    U, _, Vt = np.linalg.svd(B.T @ A)
    return B @ (U @ Vt)
