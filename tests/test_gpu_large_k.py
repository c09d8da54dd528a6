"""k above 128 (padded to 160 and 208): the contraction split into column
blocks and the single-buffer step kernel, against the FP64 oracle on the
device's own whitened data."""
import numpy as np
import pytest

from conftest import match_columns

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("k", [150, 200])
def test_large_k_contraction_and_step(mm, oracle, k):
    a0 = 0.5
    g = mm.generate(8000, k, a0, 0.2, 0.002, seed=k)
    rng = np.random.default_rng(k)
    phi0 = oracle.qr_pos(rng.standard_normal((k, k)))
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=2, minibatch=500) as p:
        p.upload(g).whiten()
        y = {n: np.asarray(v, dtype=np.float64) for n, v in p.whitened().items()}
        nx = y["Da"].shape[1]
        nodes = np.arange(0, min(1500, nx))
        # one pass of the contraction in loss and adjoint modes
        L = p.loss(phi0, 0, len(nodes))
        dL = p.loss_grad(phi0, 0, len(nodes))
        assert abs(L - oracle.loss_fwd(phi0, y, nodes, a0, 0.5)) < 1e-4 * abs(
            oracle.loss_fwd(phi0, y, nodes, a0, 0.5)) + 1e-6
        assert rel(dL, oracle.loss_bwd(phi0, y, nodes, a0, 0.5)) < 1e-4
        # online updates through the single-buffer step kernel
        p.stpm(phi0)
        lam, phi = p.lam(), p.phi()
        assert p.stats()["stpm_steps"] == 2 * -(-nx // 500)
    assert np.abs(phi.T @ phi - np.eye(k)).max() < 1e-4
    lam_o, phi_o, _ = oracle.stpm_online(y, a0, phi0, sweeps=2, minibatch=500)
    yp = {n: (v * (1 + 1e-6 * rng.standard_normal(v.shape)) if n in ("Da", "Db", "Dc") else v)
          for n, v in y.items()}
    lam_p, phi_p, _ = oracle.stpm_online(yp, a0, phi0, sweeps=2, minibatch=500)
    tol_phi = max(1e-3, 5 * float(np.abs(phi_p - phi_o).max()))
    phi_m, perm = match_columns(phi_o, phi)
    assert np.abs(phi_m - phi_o).max() < tol_phi
    assert rel(lam[perm], lam_o) < max(1e-3, 5 * rel(lam_p, lam_o))
