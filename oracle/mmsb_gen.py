"""Runs oracle/mmsb_gen.c (test and bench infrastructure): the library's seeded
MMSB generator restated without the GPU library.  The generator is an
executable writing the graph to a temporary file, so the CPU leg of the
benchmark runs on the same graph as the GPU leg without mapping any library
of this repository into its process."""
from __future__ import annotations

import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
EXE = HERE / "_gen" / "mmsb_gen"


def build():
    subprocess.run(["make", "-C", str(HERE), "gen"], check=True, stdout=subprocess.DEVNULL)


class Block:
    def __init__(self, n_rows, n_cols, row_ptr, col_idx):
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        self.row_ptr, self.col_idx = row_ptr, col_idx

    @property
    def nnz(self):
        return int(self.col_idx.shape[0])


class HostGraph:
    """The five blocks XA, XB, XC, BA, CA and the part sizes n_X..n_C."""

    def __init__(self, blocks, parts, n_edges):
        self.blocks, self.parts, self.n_edges = blocks, list(parts), n_edges

    @property
    def n_nodes(self):
        return int(sum(self.parts))

    def scipy_blocks(self):
        return [sp.csr_matrix((np.ones(b.nnz), b.col_idx, b.row_ptr), shape=(b.n_rows, b.n_cols))
                for b in self.blocks]


def generate(n, k, alpha0, p_in, p_out, seed=0) -> HostGraph:
    if not EXE.exists():
        build()
    fd, path = tempfile.mkstemp(suffix=".gen")
    os.close(fd)
    try:
        r = subprocess.run([str(EXE), str(int(n)), str(int(k)), repr(float(alpha0)),
                            repr(float(p_in)), repr(float(p_out)), str(int(seed)), path],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise ValueError(f"generator failed: {r.stderr.strip()}")
        raw = Path(path).read_bytes()
    finally:
        os.unlink(path)
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos).copy()
        pos += a.nbytes
        return a

    head = take(np.int64, 5)
    blocks = []
    for _ in range(5):
        nr, nc, nz = (int(x) for x in take(np.int64, 3))
        rp = take(np.int64, nr + 1)
        ci = take(np.int32, nz)
        blocks.append(Block(nr, nc, rp, ci))
    return HostGraph(blocks, head[:4].tolist(), int(head[4]))
