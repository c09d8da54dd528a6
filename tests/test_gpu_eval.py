"""Ground-truth evaluation on the device (mmsb_pvalues, the test of
Pvalue.cpp for every community pair), the convergence trace and the GPU
tree's output files, through the C ABI."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solved(mm):
    g = mm.generate(4000, 10, 1.0, 0.3, 0.01, seed=0, keep_pi=True)
    p = mm.Pipeline(k=10, alpha0=1.0, stpm_method=mm.STPM_ONLINE, sweeps=6, minibatch=100, tau=0.3)
    p.upload(g).run()
    yield g, p
    p.close()


def test_pvalues_match_oracle(solved, oracle):
    g, p = solved
    truth = np.asarray(g.pi.T, dtype=np.float32)  # K x N ground truth, order [X|A|B|C]
    corr, t, pv = p.pvalues(truth)
    pi = p.pi().astype(np.float64)
    K = truth.shape[0]
    assert corr.shape == (p.k, K)
    best = []
    for i in range(p.k):
        for j in range(K):
            r_o, t_o, p_o = oracle.pvalue_stats(pi[i], truth[j].astype(np.float64))
            assert abs(corr[i, j] - r_o) < 2e-6, (i, j)
            assert abs(t[i, j] - t_o) <= 1e-5 * max(1.0, abs(t_o)), (i, j)
            # p depends on t through ~exp(-t^2/2): relative error ~ t * dt
            tol = 1e-6 + 1e-4 * p_o + p_o * min(1.0, 4.0 * abs(t_o) * 1e-5 * abs(t_o))
            assert abs(pv[i, j] - p_o) <= tol, (i, j, pv[i, j], p_o)
        best.append(int(np.argmax(corr[i])))
    # most recovered communities match a distinct true one far beyond chance
    assert len(set(best)) >= p.k - 2
    assert np.median(pv[np.arange(p.k), best]) < 1e-12


def test_convergence_traces(mm, solved):
    g, p = solved
    tr = p.convergence()
    assert tr.shape == (6,) and np.all(tr > 0) and tr[-1] < tr[0]
    with mm.Pipeline(k=10, alpha0=1.0, stpm_method=mm.STPM_BATCH_POWER, min_iter=5, max_iter=40) as q:
        q.upload(g).whiten().stpm()
        tb = q.convergence()
        assert tb.shape == (q.stats()["stpm_steps"],)
        assert abs(tb[-1] - q.stats()["stpm_last_error"]) <= 1e-12 * max(1.0, tb[-1])


def test_online_trace_matches_sweep_snapshots(mm, solved):
    """Entry s of the online trace is ||Phi after sweep s+1 - Phi after sweep s||_F:
    the same runs stopped after 4 and 5 sweeps give those two iterates (the
    schedule does not depend on the sweep count; columns aligned for the final
    lambda sign fix)."""
    g, p = solved
    tr = p.convergence()
    snaps = []
    for sweeps in (4, 5):
        with mm.Pipeline(k=10, alpha0=1.0, stpm_method=mm.STPM_ONLINE, sweeps=sweeps,
                         minibatch=100, tau=0.3) as q:
            q.upload(g).whiten().stpm()
            snaps.append(q.phi())
    a, b = snaps
    b = b * np.where(np.sum(a * b, axis=0) < 0, -1.0, 1.0)
    d = float(np.linalg.norm(b - a))
    assert abs(tr[4] - d) <= 1e-4 * d + 1e-6, (tr[4], d)


def test_gpu_tree_output_files(solved, tmp_path, oracle):
    """The GPU tree's files (GPU/post_proc.c:86-114, GPU/stpm.c:915-975): the
    Pi files hold the raw unwhitened memberships ((W evecs) diag(||lambda||_2 /
    lambda_i))^T G^T, not the normalised Pi of the CPU tree."""
    g, p = solved
    p.write_gpu_outputs(tmp_path)
    tail = f"_{p.k}_1_1.txt"
    lam, phi = p.lam().astype(np.float64), p.phi().astype(np.float64)
    Gxa, _, _, Gba, Gca = g.scipy_blocks()
    raw_o, _ = oracle.postprocess(Gxa, Gba, Gca, p.whitening(), lam, phi)
    raw_o = raw_o * np.linalg.norm(lam)
    nX, nA, nB, nC = g.parts
    off, raw = 0, []
    for name, n in (("Pi_X", nX), ("Pi_A", nA), ("Pi_B", nB), ("Pi_C", nC)):
        lines = (tmp_path / f"{name}{tail}").read_text().splitlines()
        assert len(lines) == p.k * n
        assert all(re.fullmatch(r"-?\d\.\d{25}e[+-]\d\d", l) for l in lines[:50])
        raw.append(np.array([float(l) for l in lines]).reshape(n, p.k).T)
        off += n
    raw = np.concatenate(raw, axis=1)
    assert np.abs(raw - raw_o).max() < 1e-4 * np.abs(raw_o).max()
    # normalising the raw file content column by column gives the returned Pi
    assert np.abs(oracle.norm_prob_matrix(raw) - p.pi()).max() < 1e-4
    ev = np.loadtxt(tmp_path / f"evals{tail}")
    lam = p.lam()
    np.testing.assert_allclose(ev, (1 / lam ** 2) / np.sum(1 / lam ** 2), rtol=1e-12)
    assert np.loadtxt(tmp_path / f"evecs{tail}").shape == (p.k * p.k,)
    assert np.loadtxt(tmp_path / f"frob_norm{tail}").shape == (6,)
    info = (tmp_path / f"sim_info{tail}").read_text()
    assert re.search(r"Number of nodes communities\s+= 10", info)
    assert re.search(r"Total number of Frob Norm values written to file = 6", info)
