"""File formats of the path (CPU): the COO text reader against the
reference's own reader (read_G_sparse, IOfn.cpp:21-54, compiled unmodified;
fixtures in golden/io_cases.npz made by golden/make_io_golden.py), the
parallel reader on multi-megabyte files against the oracle's restatement of
that reader, the COO / binary CSR / write_mat / write_pi writers, and the
oracle's p-value restatement against the reference's Pvalue.cpp."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

GOLD = Path(__file__).resolve().parent / "golden" / "io_cases.npz"


@pytest.fixture(scope="module")
def io_gold():
    return np.load(GOLD)


def _triplets(m):
    m = sp.coo_matrix(m)
    return sorted(zip(m.row.tolist(), m.col.tolist(), m.data.tolist()))


def _same(got, ref, rtol=1e-6):
    return len(got) == len(ref) and all(
        g[0] == r[0] and g[1] == r[1] and abs(g[2] - r[2]) <= rtol * max(1.0, abs(r[2]))
        for g, r in zip(got, ref))


def test_oracle_reader_matches_reference(oracle, io_gold):
    for name in io_gold["coo_names"]:
        n1, n2, dt = (int(v) for v in io_gold[f"coo_{name}_shape"])
        got = _triplets(oracle.read_coo_reference(str(io_gold[f"coo_{name}_text"]), n1, n2, dt))
        ref = sorted((int(a), int(b), float(c)) for a, b, c in io_gold[f"coo_{name}_triplets"])
        assert _same(got, ref, 1e-15), name


def test_reader_compat_matches_reference(mm, io_gold, tmp_path):
    for name in io_gold["coo_names"]:
        n1, n2, dt = (int(v) for v in io_gold[f"coo_{name}_shape"])
        f = tmp_path / f"{name}.txt"
        f.write_bytes(str(io_gold[f"coo_{name}_text"]).encode())
        got = _triplets(mm.read_coo(f, n1, n2, datatype=dt, compat=True).to_scipy())
        ref = sorted((int(a), int(b), float(c)) for a, b, c in io_gold[f"coo_{name}_triplets"])
        # values are stored in FP32
        assert _same(got, ref, 1e-6), name


@pytest.mark.parametrize("weighted,trailing", [(0, True), (1, True), (1, False)])
def test_parallel_reader_on_large_files(mm, oracle, tmp_path, weighted, trailing):
    """~6 MB files are split over several threads at whitespace; duplicates,
    mixed separators and the end-of-file rule must come out as one serial
    pass of the reference reader would produce them."""
    rng = np.random.default_rng(3 + weighted)
    n1, n2, m = 3000, 2000, 400_000
    r = rng.integers(1, n1 + 1, m)
    c = rng.integers(1, n2 + 1, m)
    r[1000:1100] = r[0]  # a run of duplicates
    c[1000:1100] = c[0]
    seps = np.array([" ", "\t", "  "])[rng.integers(0, 3, m)]
    if weighted:
        v = rng.uniform(-2, 3, m).astype(np.float32)
        text = "".join(f"{a}{s}{b}{s}{w:.6g}\n" for a, b, s, w in zip(r, c, seps, v))
    else:
        text = "".join(f"{a}{s}{b}\r\n" if i % 7 == 0 else f"{a}{s}{b}\n"
                       for i, (a, b, s) in enumerate(zip(r, c, seps)))
    if not trailing:
        text = text.rstrip()
    f = tmp_path / "big.txt"
    f.write_text(text)
    assert f.stat().st_size > 3_000_000  # several 1 MB chunks
    got = mm.read_coo(f, n1, n2, datatype=weighted, compat=True).to_scipy()
    ref = oracle.read_coo_reference(text, n1, n2, weighted)
    assert got.nnz == ref.nnz
    assert abs(got - ref).max() <= 1e-5 * max(1.0, abs(ref).max())


def test_reader_strict_rules(mm, tmp_path):
    f = tmp_path / "s.txt"
    f.write_text("1 2\n2 3\n3\n")  # partial triplet
    with pytest.raises(mm.MmsbError):
        mm.read_coo(f, 3, 3)
    f.write_text("1 2\n2 x\n")  # not a number: the reference would never stop
    for compat in (False, True):
        with pytest.raises(mm.MmsbError):
            mm.read_coo(f, 3, 3, compat=compat)
    f.write_text("1 2\n1 2\n3 3\n")  # strict: duplicates collapse, no final repeat
    d = mm.read_coo(f, 3, 3).to_scipy().toarray()
    assert d[0, 1] == 1.0 and d[2, 2] == 1.0


def test_coo_writer_round_trip(mm, tmp_path):
    g = mm.generate(3000, 7, 0.5, 0.2, 0.002, seed=4)
    for b, blk in enumerate(g.blocks):
        f = tmp_path / f"b{b}.txt"
        mm.write_coo(f, blk)
        back = mm.read_coo(f, blk.n_rows, blk.n_cols)
        assert np.array_equal(back.row_ptr, blk.row_ptr) and np.array_equal(back.col_idx, blk.col_idx)
    rng = np.random.default_rng(5)
    w = sp.random(500, 400, density=0.02, format="csr", random_state=rng, dtype=np.float32)
    w.data[:] = rng.uniform(-3, 3, w.nnz).astype(np.float32)
    blk = mm.CsrBlock.from_scipy(w)
    f = tmp_path / "w.txt"
    mm.write_coo(f, blk)
    back = mm.read_coo(f, 500, 400, datatype=1)
    assert np.array_equal(back.col_idx, blk.col_idx) and np.array_equal(back.val, blk.val)


def test_binary_csr_round_trip_and_checks(mm, tmp_path):
    g = mm.generate(2000, 5, 1.0, 0.2, 0.003, seed=6)
    blk = g.blocks[0]
    f = tmp_path / "g.csr"
    mm.write_csr(f, blk)
    back = mm.read_csr(f)
    assert (back.n_rows, back.n_cols) == (blk.n_rows, blk.n_cols)
    assert np.array_equal(back.row_ptr, blk.row_ptr) and np.array_equal(back.col_idx, blk.col_idx)
    assert back.val is None
    raw = bytearray(f.read_bytes())
    bad = tmp_path / "bad.csr"
    bad.write_bytes(b"XXXXXXXX" + bytes(raw[8:]))
    with pytest.raises(mm.MmsbError):
        mm.read_csr(bad)
    col0 = 8 + 8 * 3 + 8 + 8 * (blk.n_rows + 1)  # header, row_ptr, then col_idx
    raw[col0:col0 + 4] = np.int32(blk.n_cols).tobytes()
    bad.write_bytes(bytes(raw))
    with pytest.raises(mm.MmsbError):
        mm.read_csr(bad)


def test_dense_and_triplet_writers_format(mm, tmp_path):
    rng = np.random.default_rng(8)
    m = rng.standard_normal((37, 5000))
    m[rng.random(m.shape) < 0.3] = 0.0
    f = tmp_path / "d.txt"
    mm.write_dense(f, m)
    assert f.read_text().splitlines() == ["%5.25e" % v for v in m.ravel(order="F")]
    f32 = m.astype(np.float32)
    mm.write_triplets(f, f32)
    want = ["%d\t%d\t%g" % (r + 1, c + 1, float(f32[r, c]))
            for c in range(f32.shape[1]) for r in range(f32.shape[0]) if f32[r, c] != 0]
    assert f.read_text().splitlines() == want


def test_oracle_pvalues_match_reference(oracle, io_gold):
    for name in io_gold["pv_names"]:
        got = np.array(oracle.pvalue_stats(io_gold[f"pv_{name}_x"], io_gold[f"pv_{name}_y"]))
        ref = io_gold[f"pv_{name}_out"]
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0, equal_nan=True, err_msg=name)
