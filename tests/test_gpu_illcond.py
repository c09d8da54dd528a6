"""Online STPM steps whose update matrix X = Phi - beta (3 theta O - 3 G) is
ill-conditioned: on this graph (n = 200,000, k = 100, alpha0 = 1,
B = 0.05 / 5e-4) cond(X) reaches 1e4 - 4e4 in the first sweep, beyond what
an FP32 Gram can factor (cond^2 x eps >> 1).  The step kernel then restarts
the factorisation with a diagonal shift (shifted Cholesky QR); before that
change this run ended in non-finite values.  The device's first sweep is
compared with the FP64 oracle's (Householder QR, diag(R) > 0) on the
device's whitened data.  Reference: GPU/stpm.c:649-691, 774-786."""
import numpy as np
import pytest

from conftest import match_columns

pytestmark = pytest.mark.gpu


def test_online_steps_on_ill_conditioned_updates(mm, oracle):
    k, a0, mb = 100, 1.0, 4096
    g = mm.generate(200_000, k, a0, 0.05, 5e-4, seed=0)
    rng = np.random.default_rng(42)
    phi0 = oracle.qr_pos(rng.standard_normal((k, k)))
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=1, minibatch=mb) as p:
        p.upload(g).whiten()
        y = {n: np.asarray(v, np.float64) for n, v in p.whitened().items()}
        p.stpm(phi0)
        lam, phi = np.asarray(p.lam(), np.float64), np.asarray(p.phi(), np.float64)
        st = p.stats()
    assert np.isfinite(phi).all() and np.isfinite(lam).all()
    assert np.abs(phi.T @ phi - np.eye(k)).max() < 1e-5
    # the oracle's first update matrices are as ill-conditioned as stated
    nodes = oracle.stpm_minibatches(y["Da"].shape[1], mb)[0]
    X = phi0 - (1.5 * phi0 - 3.0 * oracle.online_grad_terms(phi0, y, nodes, a0))
    s = np.linalg.svd(X, compute_uv=False)
    assert s[0] / s[-1] > 1e3
    lam_o, phi_o, steps = oracle.stpm_online(y, a0, phi0, sweeps=1, minibatch=mb)
    assert st["stpm_steps"] == steps
    r = np.random.default_rng(1)
    yp = {n: (v * (1 + 1e-6 * r.standard_normal(v.shape)) if n in ("Da", "Db", "Dc") else v)
          for n, v in y.items()}
    lam_p, phi_p, _ = oracle.stpm_online(yp, a0, phi0, sweeps=1, minibatch=mb)
    pm, perm = match_columns(phi_o, phi_p)
    resp_phi = np.abs(pm - phi_o).max()
    resp_lam = np.abs(lam_p[perm] - lam_o).max() / np.abs(lam_o).max()
    dm, dperm = match_columns(phi_o, phi)
    err_phi = np.abs(dm - phi_o).max()
    err_lam = np.abs(lam[dperm] - lam_o).max() / np.abs(lam_o).max()
    print("device", err_phi, err_lam, "oracle response to 1e-6 noise", resp_phi, resp_lam)
    assert err_lam <= 10 * resp_lam + 1e-4
    assert err_phi <= 10 * resp_phi + 1e-3
