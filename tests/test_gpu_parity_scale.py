"""Parity at the benchmarked size: n = 200,000 nodes in four random
partitions, k = 100, alpha0 = 0.1, B = 0.05 / 5e-4, online STPM for 20 sweeps
of 4,096-node minibatches (the GPU-at-scale configuration), device against
the FP64 oracle on the same graph and the same Gaussian sketch panels.

Stages are compared where they meet (CPU/Util.cpp:38-127 whitening,
CPU/CommunityDetection.cpp:66-139 whitened data, STPM and post-processing):
  W                   rel 1e-4 after the best orthogonal alignment
  lambda, Phi         rel 1e-4 up to column permutation and sign
  Pi                  abs 1e-3; community sets identical away from tau
once with the oracle run on the device's whitened data (the STPM and
post-processing alone) and once fully end to end (the oracle's own
whitening, the device started from the correspondingly rotated Phi0: the
method is equivariant under W -> W R for orthogonal R, QR included)."""
import os

import numpy as np
import pytest

from conftest import match_columns, procrustes_align

pytestmark = pytest.mark.gpu

WL = dict(n=200_000, k=100, alpha0=0.1, p_in=0.05, p_out=5e-4, sweeps=20, minibatch=4096, seed=0)
TAU = 0.1


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def scale_case(mm, oracle):
    oracle.FAST_GS = True
    oracle.SPMM_THREADS = os.cpu_count() or 1
    g = mm.generate(WL["n"], WL["k"], WL["alpha0"], WL["p_in"], WL["p_out"], WL["seed"])
    k, a0 = WL["k"], WL["alpha0"]
    nX, nA, nB, nC = g.parts
    rng = np.random.default_rng(42)
    sk = (rng.standard_normal((nB, 2 * k)), rng.standard_normal((nC, 2 * k)),
          rng.standard_normal((nA, 2 * k)))
    phi0 = oracle.qr_pos(rng.standard_normal((k, k)))
    Gxa, Gxb, Gxc, Gba, Gca = g.scipy_blocks()
    wh_o = oracle.second_whiten(Gxa, Gxb, Gxc, k, a0, sk)
    y_o = oracle.whitened_data(Gxa, Gxb, Gxc, wh_o)
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=WL["sweeps"],
                     minibatch=WL["minibatch"], tau=TAU) as p:
        p.upload(g).whiten(sk)
        wh_d = p.whitening()
        y_d = {n: np.asarray(v, np.float64) for n, v in p.whitened().items()}
        p.stpm(phi0).postproc()
        dev = dict(lam=np.asarray(p.lam(), np.float64), phi=np.asarray(p.phi(), np.float64),
                   pi=p.pi(), sets=p.sets(), stats=p.stats())
        # end to end: device started from the rotation of phi0 that matches
        # the oracle's whitening frame
        U, _, Vt = np.linalg.svd(wh_o["W"].T @ wh_d["W"])
        phi0_rot = (U @ Vt).T @ phi0
        p.stpm(phi0_rot).postproc()
        e2e = dict(lam=np.asarray(p.lam(), np.float64), phi=np.asarray(p.phi(), np.float64),
                   pi=p.pi(), sets=p.sets())
    return dict(g=g, blocks=(Gxa, Gba, Gca), wh_o=wh_o, y_o=y_o, wh_d=wh_d, y_d=y_d, phi0=phi0,
                dev=dev, e2e=e2e)


def _compare(oracle, case, wh, y, res, phi0, rot=None):
    k, a0 = WL["k"], WL["alpha0"]
    Gxa, Gba, Gca = case["blocks"]
    lam_o, phi_o, steps = oracle.stpm_online(y, a0, phi0, sweeps=WL["sweeps"],
                                             minibatch=WL["minibatch"])
    _, pi_o = oracle.postprocess(Gxa, Gba, Gca, wh, lam_o, phi_o)
    phi = res["phi"] if rot is None else rot @ res["phi"]
    phi_m, perm = match_columns(phi_o, phi)
    assert np.abs(phi.T @ phi - np.eye(k)).max() < 1e-5
    assert rel(phi_m, phi_o) < 1e-4
    assert rel(res["lam"][perm], lam_o) < 1e-4
    pi = res["pi"][perm].astype(np.float64)
    assert np.abs(pi - pi_o).max() < 1e-3
    away = np.abs(pi_o - TAU) > 2e-3
    assert np.array_equal(res["sets"][perm][away], (pi_o > TAU)[away])
    return steps


def test_scale_whitening_matches_oracle(scale_case):
    W_o, W_d = scale_case["wh_o"]["W"], scale_case["wh_d"]["W"]
    assert rel(procrustes_align(W_o, W_d), W_o) < 1e-4
    for n in ("Da_mu", "Db_mu", "Dc_mu"):
        # the means are invariant up to the same rotation: compare norms
        assert abs(np.linalg.norm(scale_case["y_d"][n]) - np.linalg.norm(scale_case["y_o"][n])) \
            < 1e-4 * np.linalg.norm(scale_case["y_o"][n])


def test_scale_stpm_and_post_match_oracle_on_device_whitening(oracle, scale_case):
    """The oracle's FP64 STPM + post-processing on the device's whitened data
    and whitening, same Phi0."""
    c = scale_case
    steps = _compare(oracle, c, c["wh_d"], c["y_d"], c["dev"], c["phi0"])
    assert c["dev"]["stats"]["stpm_steps"] == steps


def test_scale_end_to_end_matches_oracle(oracle, scale_case):
    """Oracle whitening -> oracle STPM -> oracle post-processing against the
    device pipeline started from the rotated Phi0."""
    c = scale_case
    U, _, Vt = np.linalg.svd(c["wh_o"]["W"].T @ c["wh_d"]["W"])
    _compare(oracle, c, c["wh_o"], c["y_o"], c["e2e"], c["phi0"], rot=U @ Vt)
