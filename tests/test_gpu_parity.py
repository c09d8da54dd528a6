"""GPU parity: the CUDA path (through the C ABI) against the reference's outputs
(golden fixtures) and the FP64 oracle, stage by stage and end to end.

Tolerances (FP32 device arithmetic vs FP64 reference):
  SpMM                      rel 1e-5 of the output scale
  whitening W               rel 1e-4 after column-sign alignment
  whitened data             rel 1e-4
  lambda, Phi (STPM)        rel 1e-4 up to column permutation and sign
  Pi                        abs 1e-3;  community sets identical away from tau
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import align_columns, match_columns, procrustes_align

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def random_csr(rng, n_rows, n_cols, density, weighted=False, empty_rows=True):
    m = sp.random(n_rows, n_cols, density=density, format="csr", random_state=rng)
    m.data[:] = rng.uniform(0.5, 2.0, m.nnz) if weighted else 1.0
    if empty_rows:
        m = m.tolil()
        for r in range(0, n_rows, 7):
            m.rows[r] = []
            m.data[r] = []
        m = m.tocsr()
    # one heavy row
    m = m.tolil()
    m.rows[1] = list(range(0, n_cols, 2))
    m.data[1] = [1.0] * len(m.rows[1])
    return m.tocsr()


@pytest.mark.parametrize("p", [4, 20, 100, 200, 400])
@pytest.mark.parametrize("transpose", [False, True])
def test_spmm_vs_scipy(mm, p, transpose):
    rng = np.random.default_rng(p + transpose)
    G = random_csr(rng, 1501, 777, 0.01)
    blk = mm.CsrBlock.from_scipy(G)
    n_in = G.shape[0] if transpose else G.shape[1]
    P = rng.standard_normal((n_in, p)).astype(np.float32)
    Y = mm.spmm(blk, P, transpose=transpose, alpha=0.5)
    ref = 0.5 * ((G.T if transpose else G) @ P.astype(np.float64))
    assert rel(Y, ref) < 1e-5


def test_spmm_weighted_and_empty(mm):
    rng = np.random.default_rng(3)
    G = random_csr(rng, 300, 2000, 0.02, weighted=True)
    P = rng.standard_normal((2000, 36)).astype(np.float32)
    Y = mm.spmm(mm.CsrBlock.from_scipy(G), P)
    assert rel(Y, G @ P.astype(np.float64)) < 1e-5
    E = sp.csr_matrix((5, 9))
    Y0 = mm.spmm(mm.CsrBlock.from_scipy(E), rng.standard_normal((9, 8)).astype(np.float32))
    assert np.all(Y0 == 0)


@pytest.mark.parametrize("kind", ["wishart", "graded"])
@pytest.mark.parametrize("n", [6, 20, 64, 200])
def test_symeig_vs_numpy(mm, n, kind):
    """FP32 one-sided Jacobi run to convergence + three FP64 Ogita-Aishima
    refinement steps: FP64-level eigen-pairs on a Wishart spectrum and on a
    graded one spanning five decades."""
    rng = np.random.default_rng(n)
    if kind == "wishart":
        B = rng.standard_normal((n, n))
        A = B @ B.T + 0.1 * np.eye(n)
    else:
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = (Q * np.geomspace(1e3, 1e-2, n)) @ Q.T
        A = 0.5 * (A + A.T)
    ev, V = mm.symeig(A)
    ref = np.linalg.eigvalsh(A)[::-1]
    assert np.abs(V.T @ V - np.eye(n)).max() < 1e-10
    assert rel(ev, ref) < 1e-9
    assert np.abs(A @ V - V * ev).max() / np.abs(A).max() < 1e-9
    assert np.all(np.diff(ev) <= 0)


def test_whitening_matches_reference(mm, golden):
    with mm.Pipeline(k=golden.k, alpha0=golden.alpha0) as p:
        p.upload(golden.graph(mm)).whiten(golden.sketches())
        wh = p.whitening()
    for n in ("mu_a", "mu_b", "mu_c"):
        assert rel(wh[n], golden[n].ravel()) < 1e-12
    # W is defined up to rotations inside near-degenerate singular pairs
    # (cfg1: sigma 5.80 / 5.70), and the tensor power method is equivariant
    # under W -> W Q; compare after the best orthogonal alignment
    W = golden["W"]
    assert rel(procrustes_align(W, wh["W"]), W) < 1e-4
    for a, b in (("Zb1", "Zb2"), ("Zc1", "Zc2")):
        assert rel(wh[a] @ wh[b], golden[a] @ golden[b]) < 1e-4


def test_whitened_data_matches_reference(mm, golden):
    with mm.Pipeline(k=golden.k, alpha0=golden.alpha0) as p:
        p.upload(golden.graph(mm)).set_whitening(golden.whitening())
        y = p.whitened()
    for n in ("Da", "Db", "Dc"):
        assert rel(y[n], golden[n]) < 1e-4
    for n in ("Da_mu", "Db_mu", "Dc_mu"):
        assert rel(y[n], golden[n].ravel()) < 1e-4


def test_postprocess_matches_reference(mm, golden):
    with mm.Pipeline(k=golden.k, alpha0=golden.alpha0, tau=0.2) as p:
        p.upload(golden.graph(mm)).set_whitening(golden.whitening())
        p.set_phi_lambda(golden["phi"], golden["lambda"].ravel()).postproc()
        pi = p.pi()
        sets = p.sets()
    ref = golden["pi"]
    assert np.abs(pi - ref).max() < 1e-3
    away = np.abs(ref - 0.2) > 2e-3
    assert np.array_equal(sets[away], (ref > 0.2)[away])


def test_batch_power_matches_oracle(mm, oracle, golden):
    """tensorDecom_alpha0 on the reference's whitened data and Phi0, 150 iterations."""
    y = golden.whitened()
    lam_o, phi_o, it, _ = oracle.tensor_decomp_batch(y, golden.alpha0, golden["phi0"],
                                                     min_iter=100, max_iter=149)
    with mm.Pipeline(k=golden.k, alpha0=golden.alpha0, stpm_method=mm.STPM_BATCH_POWER,
                     min_iter=100, max_iter=149) as p:
        p.upload(golden.graph(mm)).set_whitened(y).stpm(golden["phi0"])
        lam, phi = p.lam(), p.phi()
        steps = p.stats()["stpm_steps"]
    assert steps == it
    assert rel(lam, lam_o) < 1e-3
    assert np.abs(phi - phi_o).max() < 1e-3


def test_online_stpm_matches_oracle(mm, oracle, golden):
    """Five sweeps of minibatch STPM against the FP64 oracle.  On the smaller
    fixtures the dynamics amplify input noise (the 1002-node ragged graph
    turns a 1e-7 relative perturbation of y into 4e-4 in Phi after five
    sweeps), so the tolerance is the larger of 1e-3 and five times the
    oracle's own response to a 1e-6 relative perturbation of y (FP32-level
    input noise)."""
    y = golden.whitened()
    lam_o, phi_o, steps_o = oracle.stpm_online(y, golden.alpha0, golden["phi0"], sweeps=5,
                                               minibatch=100)
    rng = np.random.default_rng(11)
    yp = {n: (v * (1 + 1e-6 * rng.standard_normal(v.shape)) if n in ("Da", "Db", "Dc") else v)
          for n, v in y.items()}
    lam_p, phi_p, _ = oracle.stpm_online(yp, golden.alpha0, golden["phi0"], sweeps=5,
                                         minibatch=100)
    tol_phi = max(1e-3, 5 * float(np.abs(phi_p - phi_o).max()))
    tol_lam = max(1e-3, 5 * rel(lam_p, lam_o))
    with mm.Pipeline(k=golden.k, alpha0=golden.alpha0, stpm_method=mm.STPM_ONLINE, sweeps=5,
                     minibatch=100) as p:
        p.upload(golden.graph(mm)).set_whitened(y).stpm(golden["phi0"])
        lam, phi = p.lam(), p.phi()
        assert p.stats()["stpm_steps"] == steps_o
    phi_m, perm = match_columns(phi_o, phi)
    assert np.abs(phi.T @ phi - np.eye(golden.k)).max() < 1e-4
    assert np.abs(phi_m - phi_o).max() < tol_phi
    assert rel(lam[perm], lam_o) < tol_lam


def test_adjoint_loss_and_gradient(mm, oracle, golden_cfg1):
    g = golden_cfg1
    y = g.whitened()
    rng = np.random.default_rng(1)
    phi = g["phi0"] + 0.05 * rng.standard_normal(g["phi0"].shape)
    nodes = np.arange(100, 700)
    L_o = oracle.loss_fwd(phi, y, nodes, g.alpha0, 1.0)
    dL_o = oracle.loss_bwd(phi, y, nodes, g.alpha0, 1.0)
    with mm.Pipeline(k=g.k, alpha0=g.alpha0, theta=1.0) as p:
        p.upload(g.graph(mm)).set_whitened(y)
        L = p.loss(phi, 100, 600)
        dL = p.loss_grad(phi, 100, 600)
        # FP64 central differences of the device loss are too coarse in FP32;
        # check the device gradient against FD of the FP64 oracle loss instead
        h = 1e-6
        for _ in range(10):
            d = rng.standard_normal(phi.shape)
            d /= np.linalg.norm(d)
            fd = (oracle.loss_fwd(phi + h * d, y, nodes, g.alpha0, 1.0)
                  - oracle.loss_fwd(phi - h * d, y, nodes, g.alpha0, 1.0)) / (2 * h)
            assert abs(np.sum(dL * d) - fd) < 1e-4 * max(1.0, np.abs(dL).max())
    assert abs(L - L_o) < 1e-5 * max(1.0, abs(L_o))
    assert rel(dL, dL_o) < 1e-4


def _aligned_start(W_ref, W_dev, phi0):
    """W_dev = W_ref R (+ round-off) with R orthogonal; the tensor power method
    is equivariant under that rotation, so starting from R^T phi0 reproduces
    the reference trajectory in the device's frame."""
    U, _, Vt = np.linalg.svd(W_ref.T @ W_dev)
    R = U @ Vt
    return R.T @ phi0


def test_end_to_end_batch_power_vs_reference(mm, oracle, golden):
    """The reference's own pipeline (reference sketches, tensorDecom_alpha0,
    unwhitening, normProbMatrix) end to end; 150 power iterations."""
    g = golden
    k, a0 = g.k, g.alpha0
    Gxa, _, _, Gba, Gca = g.scipy_blocks()
    lam_o, phi_o, it, _ = oracle.tensor_decomp_batch(g.whitened(), a0, g["phi0"], min_iter=100,
                                                     max_iter=149)
    _, pi_o = oracle.postprocess(Gxa, Gba, Gca, g.whitening(), lam_o, phi_o)
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_BATCH_POWER, min_iter=100,
                     max_iter=149, tau=0.3) as p:
        p.upload(g.graph(mm)).whiten(g.sketches())
        p.stpm(_aligned_start(g["W"], p.whitening()["W"], g["phi0"])).postproc()
        lam, pi, sets = p.lam(), p.pi(), p.sets()
    assert rel(lam, lam_o) < 1e-3
    assert np.abs(pi - pi_o).max() < 1e-3
    away = np.abs(pi_o - 0.3) > 2e-3
    assert np.array_equal(sets[away], (pi_o > 0.3)[away])


def test_end_to_end_online_vs_oracle(mm, oracle, golden_cfg1):
    """Whole pipeline with the online method on the reference configuration's
    graph (4 x 1000 nodes, k = 10: the FP64 dynamics there contract input
    perturbations, so FP32 and FP64 runs must agree)."""
    g = golden_cfg1
    k, a0 = g.k, g.alpha0
    Gxa, _, _, Gba, Gca = g.scipy_blocks()
    lam_o, phi_o, _ = oracle.stpm_online(g.whitened(), a0, g["phi0"], sweeps=10, minibatch=100)
    _, pi_o = oracle.postprocess(Gxa, Gba, Gca, g.whitening(), lam_o, phi_o)
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=10, minibatch=100,
                     tau=0.3) as p:
        p.upload(g.graph(mm)).whiten(g.sketches())
        p.stpm(_aligned_start(g["W"], p.whitening()["W"], g["phi0"])).postproc()
        lam, pi, sets = p.lam(), p.pi(), p.sets()
    _, perm = match_columns(pi_o.T, pi.T.astype(np.float64))
    assert rel(lam[perm], lam_o) < 1e-4
    assert np.abs(pi[perm] - pi_o).max() < 1e-3
    away = np.abs(pi_o - 0.3) > 2e-3
    assert np.array_equal(sets[perm][away], (pi_o > 0.3)[away])


def test_gaussian_sketch_whitening_vs_oracle(mm, oracle, golden_cfg1):
    """Gaussian sketch panels: W up to orthogonal alignment and the whitened
    data's invariants against the FP64 oracle fed the same panels."""
    g = golden_cfg1
    k, a0 = g.k, g.alpha0
    rng = np.random.default_rng(7)
    nX, nA, nB, nC = (int(x) for x in g["parts"])
    sk = (rng.standard_normal((nB, 2 * k)), rng.standard_normal((nC, 2 * k)),
          rng.standard_normal((nA, 2 * k)))
    Gxa, Gxb, Gxc, _, _ = g.scipy_blocks()
    wh = oracle.second_whiten(Gxa, Gxb, Gxc, k, a0, sk)
    with mm.Pipeline(k=k, alpha0=a0) as p:
        p.upload(g.graph(mm)).whiten(sk)
        W = p.whitening()["W"]
    assert rel(procrustes_align(wh["W"], W), wh["W"]) < 1e-4


def test_errors_are_status_codes(mm, golden_cfg1):
    g = golden_cfg1
    with mm.Pipeline(k=g.k, alpha0=g.alpha0) as p:
        with pytest.raises(mm.MmsbError) as e:
            p.stpm()
        assert e.value.status == 4  # call out of order
        bad = g.graph(mm)
        bad.blocks[3] = mm.CsrBlock(5, 5, np.zeros(6, np.int64), np.zeros(0, np.int32))
        with pytest.raises(mm.MmsbError) as e:
            p.upload(bad)
        assert e.value.status == 1
        # checked on the device: a column index past the block, a decreasing
        # row offset; the context stays usable
        good = g.graph(mm)
        b0 = good.blocks[0]
        ci = b0.col_idx.copy()
        ci[b0.nnz // 2] = b0.n_cols
        bad = g.graph(mm)
        bad.blocks[0] = mm.CsrBlock(b0.n_rows, b0.n_cols, b0.row_ptr, ci)
        with pytest.raises(mm.MmsbError, match="column index out of range") as e:
            p.upload(bad)
        assert e.value.status == 1
        rp = b0.row_ptr.copy()
        r = int(np.argmax(np.diff(rp) > 1))  # a row with two or more entries
        rp[r + 1] = rp[r] - 1 if rp[r] > 0 else rp[r + 2] + 1
        bad = g.graph(mm)
        bad.blocks[0] = mm.CsrBlock(b0.n_rows, b0.n_cols, rp, b0.col_idx)
        with pytest.raises(mm.MmsbError, match="decreasing row_ptr") as e:
            p.upload(bad)
        assert e.value.status == 1
        with pytest.raises(mm.MmsbError) as e:
            p.whiten()
        assert e.value.status == 4  # a failed upload leaves no graph
        p.upload(good).whiten()


def test_pinned_upload_and_download_match(mm, golden_cfg1):
    """Uploads from page-locked host arrays and downloads into a pinned
    output give the same results as plain host memory."""
    g = golden_cfg1
    graph = g.graph(mm)
    out = []
    for pinned in (False, True):
        with mm.Pipeline(k=g.k, alpha0=g.alpha0, stpm_method=mm.STPM_ONLINE, sweeps=2,
                         minibatch=100, seed=4) as p:
            if pinned:
                graph.pin()
                buf = mm.pin_host(np.empty((g.k, graph.n_nodes), np.float32, order="F"))
            p.upload(graph).run()
            out.append((p.pi(out=buf) if pinned else p.pi(), p.lam()))
            if pinned:
                graph.unpin()
                mm.unpin_host(buf)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_rank_deficient_graph(mm, oracle):
    """A graph too sparse for its k (124 X->A edges, pair operators of rank
    ~101 < 2k = 120): the eigen-solver meets exactly zero directions.  The
    pipeline must stay finite and agree with the FP64 oracle on the whitening
    subspace (W W^T, which is invariant under the free rotations)."""
    n, k, a0 = 2000, 60, 0.3
    g = mm.generate(n, k, a0, 0.02, 2e-4, seed=5)
    Gxa, Gxb, Gxc, _, _ = g.scipy_blocks()
    rng = np.random.default_rng(3)
    nX, nA, nB, nC = g.parts
    sk = (rng.standard_normal((nB, 2 * k)), rng.standard_normal((nC, 2 * k)),
          rng.standard_normal((nA, 2 * k)))
    wh = oracle.second_whiten(Gxa, Gxb, Gxc, k, a0, sk)
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=2, minibatch=128) as p:
        p.upload(g).whiten(sk)
        W = p.whitening()["W"]
        assert np.isfinite(W).all()
        P, Po = W @ W.T, wh["W"] @ wh["W"].T
        assert np.linalg.norm(P - Po) / np.linalg.norm(Po) < 1e-2
        p.stpm().postproc()
        assert np.isfinite(p.lam()).all() and np.isfinite(p.pi()).all()
