"""The drop-in command line (CommunityDetection.cpp:16-149 argv and files)
against the library called directly."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write_coo(path, rp, ci):
    """Edge list as the reference's read_G_sparse reads it: 1-based "row col"."""
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp)) + 1
    with open(path, "w") as f:
        for r, c in zip(rows, ci + 1):
            f.write(f"{r}\t{c}\n")


def test_cli_matches_pipeline_and_reference(mm, golden_cfg1, tmp_path):
    g = golden_cfg1
    names = ["Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a"]
    files = []
    for n in names:
        files.append(str(tmp_path / f"{n}.txt"))
        _write_coo(files[-1], g[f"{n}_rp"], g[f"{n}_ci"])
    nX, nA, nB, nC = (int(x) for x in g["parts"])
    pi_f, white_f, lam_f = (str(tmp_path / x) for x in ("pi.txt", "white.txt", "lam.txt"))
    r = subprocess.run([str(mm.CLI_PATH), str(nX), str(nA), str(nB), str(nC), str(g.k),
                        repr(g.alpha0), "0", *files, pi_f, white_f, f"--lambda-out={lam_f}",
                        "--seed=7"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr

    # the same files through the library's reader (compat: the reference's
    # read_G_sparse, last line counted twice) and the same configuration
    blocks = [mm.read_coo(f, r, c, compat=True) for f, (r, c) in zip(
        files, [(nX, nA), (nX, nB), (nX, nC), (nB, nA), (nC, nA)])]
    with mm.Pipeline(k=g.k, alpha0=g.alpha0, seed=7) as p:
        p.upload(mm.Graph(blocks, (nX, nA, nB, nC))).whiten().stpm().postproc()
        pi, lam = p.pi(), p.lam()
        W = p.whitening()["W"]
    mm.write_triplets(tmp_path / "pi_lib.txt", pi)
    mm.write_triplets(tmp_path / "white_lib.txt", W)
    assert open(pi_f).read() == (tmp_path / "pi_lib.txt").read_text()
    assert open(white_f).read() == (tmp_path / "white_lib.txt").read_text()
    np.testing.assert_allclose(np.loadtxt(lam_f), lam, rtol=0, atol=0)

    # memberships: every node's column of the normalised Pi sums to 1 (or is empty)
    t = np.loadtxt(pi_f, ndmin=2)
    N = nX + nA + nB + nC
    colsum = np.zeros(N)
    np.add.at(colsum, t[:, 1].astype(int) - 1, t[:, 2])
    nz = colsum > 0
    assert nz.mean() > 0.9
    np.testing.assert_allclose(colsum[nz], 1.0, atol=1e-4)


def test_cli_binary_inputs_and_gpu_tree_outputs(mm, golden_cfg1, tmp_path):
    """Blocks given as binary CSR files (".csr") and --gpu-out: the same
    memberships as COO text inputs, plus the GPU tree's files."""
    g = golden_cfg1
    names = ["Gx_a", "Gx_b", "Gx_c", "Gb_a", "Gc_a"]
    nX, nA, nB, nC = (int(x) for x in g["parts"])
    shapes = [(nX, nA), (nX, nB), (nX, nC), (nB, nA), (nC, nA)]
    txt, csr = [], []
    for n, (r_, c_) in zip(names, shapes):
        blk = mm.CsrBlock(r_, c_, g[f"{n}_rp"].astype(np.int64), g[f"{n}_ci"].astype(np.int32))
        txt.append(str(tmp_path / f"{n}.txt"))
        csr.append(str(tmp_path / f"{n}.csr"))
        mm.write_coo(txt[-1], blk)
        mm.write_csr(csr[-1], blk)
    out = {}
    for kind, files in (("txt", txt), ("csr", csr)):
        pi_f, white_f = str(tmp_path / f"pi_{kind}.txt"), str(tmp_path / f"white_{kind}.txt")
        d = tmp_path / f"gpu_{kind}"
        d.mkdir()
        r = subprocess.run([str(mm.CLI_PATH), str(nX), str(nA), str(nB), str(nC), str(g.k),
                            repr(g.alpha0), "0", *files, pi_f, white_f, "--method=online",
                            "--sweeps=2", "--minibatch=100", "--seed=3", "--reader=strict",
                            f"--gpu-out={d}"], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        out[kind] = (open(pi_f).read(), d)
    assert out["txt"][0] == out["csr"][0]
    d = out["csr"][1]
    tail = f"_{g.k}_{g.alpha0:g}_1.txt"
    for name, n in (("Pi_X", nX), ("Pi_A", nA), ("Pi_B", nB), ("Pi_C", nC)):
        assert len((d / f"{name}{tail}").read_text().splitlines()) == g.k * n
    assert len((d / f"frob_norm{tail}").read_text().splitlines()) == 2
    assert (d / f"sim_info{tail}").exists() and (d / f"evals{tail}").exists()
