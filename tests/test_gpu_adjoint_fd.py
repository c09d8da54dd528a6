"""The adjoint form's gradient (mmsb_stpm_loss_bwd: all three partials of
the cubic form with Z recomputed per minibatch) checked on a generated
graph with k = 100 against FP64 central differences of the FP64 loss on the
device's whitened data along 100 random unit directions (step 1e-6), against
the FP64 oracle gradient, and against central differences of the device's
own FP32 loss (step 1e-2: the loss is a cubic polynomial, so the truncation
error is h^2/6 times a third derivative, while FP32 round-off of L divided by
h stays below it).  Reference semantics: Diff_Loss, CPU/Util.cpp:257-304."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_adjoint_gradient_vs_fp64_finite_differences(mm, oracle):
    k, a0 = 100, 1.0
    g = mm.generate(24_000, k, a0, 0.04, 4e-4, seed=4)
    rng = np.random.default_rng(5)
    with mm.Pipeline(k=k, alpha0=a0, stpm_method=mm.STPM_ADJOINT, theta=1.0) as p:
        p.upload(g).whiten()
        y = {n: np.asarray(v, np.float64) for n, v in p.whitened().items()}
        phi = oracle.qr_pos(rng.standard_normal((k, k))) + 0.05 * rng.standard_normal((k, k))
        b, cnt = 512, 2048
        nodes = np.arange(b, b + cnt)
        dL = p.loss_grad(phi, b, cnt)
        L = p.loss(phi, b, cnt)
        dL_o = oracle.loss_bwd(phi, y, nodes, a0, 1.0)
        L_o = oracle.loss_fwd(phi, y, nodes, a0, 1.0)
        scale = max(1.0, np.abs(dL_o).max())
        assert abs(L - L_o) <= 1e-5 * max(1.0, abs(L_o))
        assert np.abs(dL - dL_o).max() <= 1e-4 * scale
        h = 1e-6
        for _ in range(100):
            d = rng.standard_normal((k, k))
            d /= np.linalg.norm(d)
            fd = (oracle.loss_fwd(phi + h * d, y, nodes, a0, 1.0)
                  - oracle.loss_fwd(phi - h * d, y, nodes, a0, 1.0)) / (2 * h)
            assert abs(np.sum(dL * d) - fd) <= 1e-4 * scale
        hd = 1e-2
        for _ in range(10):
            d = rng.standard_normal((k, k))
            d /= np.linalg.norm(d)
            fd = (p.loss(phi + hd * d, b, cnt) - p.loss(phi - hd * d, b, cnt)) / (2 * hd)
            assert abs(np.sum(dL * d) - fd) <= 1e-3 * scale
