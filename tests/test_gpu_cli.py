"""The drop-in command line (CommunityDetection.cpp:16-149 argv and files)
against the library called directly and against the reference's outputs."""
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

    # the same configuration through the library: identical files
    with mm.Pipeline(k=g.k, alpha0=g.alpha0, seed=7) as p:
        p.upload(g.graph(mm)).whiten().stpm().postproc()
        pi, lam = p.pi(), p.lam()
        W = p.whitening()["W"]
    mm.write_triplets(tmp_path / "pi_lib.txt", pi)
    mm.write_triplets(tmp_path / "white_lib.txt", W)
    assert open(pi_f).read() == (tmp_path / "pi_lib.txt").read_text()
    assert open(white_f).read() == (tmp_path / "white_lib.txt").read_text()
    np.testing.assert_allclose(np.loadtxt(lam_f), lam, rtol=0, atol=0)

    # the whitening file spans the reference's W (write_pi of CPU/Spectral.cpp's W)
    Wf = np.zeros((nA, g.k))
    t = np.loadtxt(white_f, ndmin=2)
    Wf[t[:, 0].astype(int) - 1, t[:, 1].astype(int) - 1] = t[:, 2]
    Wr = g["W"]
    Q, _ = np.linalg.qr(Wr)
    resid = np.linalg.norm(Wf - Q @ (Q.T @ Wf)) / np.linalg.norm(Wf)
    assert resid < 1e-4
