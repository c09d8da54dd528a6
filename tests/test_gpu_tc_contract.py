"""k up to 112 (padded to 64, 80 and 112 here): the online STPM's contraction runs on
the tensor cores (tcgen05, 3xTF32, Z and G in tensor memory).  Online sweeps
against the FP64 oracle on the device's own whitened data, with tolerances
set by the oracle's own response to a 1e-6 relative perturbation of y."""
import numpy as np
import pytest

from conftest import match_columns

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("k,minibatch", [(64, 500), (75, 500), (100, 700), (100, 64)])
def test_tensor_core_contraction_online_vs_oracle(mm, oracle, k, minibatch):
    a0 = 0.5
    g = mm.generate(8000, k, a0, 0.2, 0.002, seed=k + 1)
    rng = np.random.default_rng(k)
    phi0 = oracle.qr_pos(rng.standard_normal((k, k)))
    sweeps = 2 if minibatch > 100 else 1
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=sweeps,
                     minibatch=minibatch) as p:
        p.upload(g).whiten()
        y = {n: np.asarray(v, dtype=np.float64) for n, v in p.whitened().items()}
        nx = y["Da"].shape[1]
        p.stpm(phi0)
        lam, phi = p.lam(), p.phi()
        assert p.stats()["stpm_steps"] == sweeps * -(-nx // minibatch)
    assert np.abs(phi.T @ phi - np.eye(k)).max() < 1e-5
    lam_o, phi_o, _ = oracle.stpm_online(y, a0, phi0, sweeps=sweeps, minibatch=minibatch)
    yp = {n: (v * (1 + 1e-6 * rng.standard_normal(v.shape)) if n in ("Da", "Db", "Dc") else v)
          for n, v in y.items()}
    lam_p, phi_p, _ = oracle.stpm_online(yp, a0, phi0, sweeps=sweeps, minibatch=minibatch)
    tol_phi = max(1e-4, 5 * float(np.abs(phi_p - phi_o).max()))
    phi_m, perm = match_columns(phi_o, phi)
    assert np.abs(phi_m - phi_o).max() < tol_phi
    assert rel(lam[perm], lam_o) < max(1e-4, 5 * rel(lam_p, lam_o))


def _bf16(v):
    """round to the nearest BF16 (ties to even), returned as float64"""
    u = np.ascontiguousarray(v, dtype=np.float32).view(np.uint32)
    r = (u + np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.view(np.float32).astype(np.float64)


@pytest.mark.parametrize("k", [64, 75, 100])
def test_bf16_adjoint_tensor_core_vs_oracle(mm, oracle, k):
    """BF16 form of the adjoint method (tcgen05 kind::f16 contraction for all
    sweeps but the last, which refines in FP32) against the FP64 oracle; the
    tolerance is set by the oracle's own response to y rounded to BF16."""
    a0 = 0.5
    g = mm.generate(8000, k, a0, 0.2, 0.002, seed=k + 2)
    rng = np.random.default_rng(k)
    phi0 = oracle.qr_pos(rng.standard_normal((k, k)))
    out = {}
    for prec in (mm.PREC_BF16, mm.PREC_FP32):
        with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ADJOINT, sweeps=3, minibatch=500,
                         precision=prec) as p:
            p.upload(g).whiten()
            y = {n: np.asarray(v, dtype=np.float64) for n, v in p.whitened().items()}
            p.stpm(phi0)
            out[prec] = (p.lam(), p.phi())
    lam_o, phi_o, _ = oracle.stpm_online(y, a0, phi0, sweeps=3, minibatch=500, adjoint=True)
    yb = {n: (_bf16(v) if n in ("Da", "Db", "Dc") else v) for n, v in y.items()}
    lam_b, _, _ = oracle.stpm_online(yb, a0, phi0, sweeps=3, minibatch=500, adjoint=True)
    tol = max(2e-3, 5 * rel(lam_b, lam_o))
    lam, phi = out[mm.PREC_BF16]
    assert np.abs(phi.T @ phi - np.eye(k)).max() < 1e-5
    _, perm = match_columns(phi_o, phi)
    assert rel(lam[perm], lam_o) < tol
    lam32, _ = out[mm.PREC_FP32]
    assert rel(np.sort(lam), np.sort(lam32)) < tol
