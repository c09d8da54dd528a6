"""CPU-only tests: the C ABI library loads and exports every declared symbol,
the generator, the reference's file contract (COO reader, triplet writer)."""
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "mmsb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mmsb_[a-z0-9_]+)\s*\(", text)))


def test_header_and_library_exports(mm):
    names = declared_functions()
    assert len(names) >= 30
    L = mm.lib()
    for n in names:
        assert hasattr(L, n), n
    # the Python binding covers every declared function
    assert sorted(mm.exported_symbols()) == names


def test_config_defaults_match_reference_knobs(mm):
    c = mm.default_config()
    # CPU/stdafx.h:56-60 and Spectral.cpp:173
    assert (c.min_iter, c.max_iter, c.tol, c.pinv_tol) == (100, 10000, 1e-6, 1e-6)
    assert c.nystrom_rows_factor == 20 and c.normalize == 1
    assert c.stpm_method == mm.STPM_BATCH_POWER


def test_generator_deterministic_and_consistent(mm):
    g1 = mm.generate(4000, 10, 1.0, 0.3, 0.01, seed=0)
    g2 = mm.generate(4000, 10, 1.0, 0.3, 0.01, seed=0)
    g3 = mm.generate(4000, 10, 1.0, 0.3, 0.01, seed=1)
    assert g1.parts == (1000, 1000, 1000, 1000)
    for a, b in zip(g1.blocks, g2.blocks):
        assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col_idx, b.col_idx)
    assert any(a.nnz != b.nnz for a, b in zip(g1.blocks, g3.blocks))
    # E[d] = n (p + q (k-1)) / k = 4000 * 0.39 / 10 = 156
    assert abs(2 * g1.n_edges / 4000 - 156.0) < 6.0
    for b in g1.blocks:
        assert b.row_ptr[0] == 0 and b.row_ptr[-1] == b.nnz
        for r in range(0, b.n_rows, 97):
            cols = b.col_idx[b.row_ptr[r]:b.row_ptr[r + 1]]
            assert np.all(np.diff(cols) > 0)


def test_generator_ragged_and_memberships(mm):
    g = mm.generate(1003, 7, 0.5, 0.2, 0.002, seed=5, keep_pi=True)
    assert g.parts == (250, 250, 250, 253)
    assert g.pi.shape == (1003, 7)
    assert np.allclose(g.pi.sum(axis=1), 1.0, atol=1e-5)


def test_generator_rejects_bad_params(mm):
    with pytest.raises(mm.MmsbError):
        mm.generate(2, 3, 1.0, 0.1, 0.01)
    with pytest.raises(mm.MmsbError):
        mm.generate(100, 3, 1.0, 1.5, 0.01)


def test_coo_reader_reference_quirk(mm, tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("1 2\n2 1\n3 3\n")
    plain = mm.read_coo(p, 3, 3)
    assert plain.nnz == 3 and plain.val is None
    # IOfn.cpp:36-49: the trailing newline makes the feof loop push (3,3) twice
    compat = mm.read_coo(p, 3, 3, compat=True)
    dense = compat.to_scipy().toarray()
    assert dense[2, 2] == 2.0 and dense[0, 1] == 1.0
    p.write_text("1 2\n2 1\n3 3")
    assert mm.read_coo(p, 3, 3, compat=True).to_scipy().toarray()[2, 2] == 1.0


def test_coo_reader_weighted_and_errors(mm, tmp_path):
    p = tmp_path / "w.txt"
    p.write_text("1 1 0.5\n2 3 2.25\n")
    b = mm.read_coo(p, 2, 3, datatype=1)
    assert np.allclose(b.to_scipy().toarray(), [[0.5, 0, 0], [0, 0, 2.25]])
    p.write_text("1 4\n")
    with pytest.raises(mm.MmsbError):
        mm.read_coo(p, 2, 3)
    with pytest.raises(mm.MmsbError):
        mm.read_coo(tmp_path / "missing.txt", 2, 3)


def test_triplet_writer_matches_reference_format(mm, golden_cfg1, tmp_path):
    """write_pi (IOfn.cpp:57-67) output of W, byte for byte."""
    out = tmp_path / "white.txt"
    mm.write_triplets(out, golden_cfg1["W"])
    assert out.read_text().splitlines() == list(golden_cfg1["white_txt"])


def test_cli_argv_contract(mm, tmp_path):
    """The command line keeps CommunityDetection.cpp:16-40's argv: too few
    arguments or an unreadable input file exit with status 1 before any
    device work."""
    import subprocess
    cli = str(mm.CLI_PATH)
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
    missing = [str(tmp_path / f"{n}.txt") for n in ("Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a")]
    r = subprocess.run([cli, "10", "10", "10", "10", "2", "1.0", "0", *missing,
                        str(tmp_path / "pi.txt"), str(tmp_path / "white.txt")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "Gx_a" in r.stderr
    r = subprocess.run([cli, *(["1"] * 7), *missing, "a", "b", "--bogus=1"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "unknown option" in r.stderr
