"""The tall-skinny Gram on the 5th-generation tensor cores (tcgen05.mma
kind::tf32 with the accumulator in tensor memory, 3xTF32 split) against FP64
numpy, and the whitening that runs its CholQR Grams on it against the FP64
oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import procrustes_align

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,pa,pb,tc", [(20000, 200, 200, True), (50000, 64, 130, True),
                                        (5000, 300, 70, True), (3000, 200, 200, False),
                                        (20000, 20, 200, False)])
def test_gram_matches_fp64(mm, n, pa, pb, tc):
    rng = np.random.default_rng(n + pa + pb)
    A = rng.standard_normal((n, pa)).astype(np.float32)
    B = (rng.standard_normal((n, pb)) * np.linspace(0.1, 10.0, pb)).astype(np.float32)
    B[::7] = 0.0  # ragged content
    S = mm.gram(A, B, alpha=0.5)
    ref = 0.5 * (A.astype(np.float64).T @ B.astype(np.float64))
    # FP32-level error: ~1e-7 per product, FP32 sums over a split's rows
    scale = 0.5 * np.sqrt(n) * np.abs(A).max() * np.abs(B).max()
    assert np.abs(S - ref).max() <= 2e-6 * scale, (n, pa, pb, tc)
    # symmetric Gram (the CholQR case) is symmetric to round-off
    G = mm.gram(A, A)
    assert np.abs(G - G.T).max() <= 1e-6 * np.abs(G).max()


def test_whitening_with_tensor_core_grams_vs_oracle(mm, oracle):
    """k = 40 (p = 80 sketch columns) and 5,000 nodes per partition: the
    CholQR Grams of both pseudo-inverse sides run on the tensor cores."""
    n, k, a0 = 20000, 40, 0.5
    g = mm.generate(n, k, a0, 0.1, 0.0005, seed=12)
    nX, nA, nB, nC = g.parts
    rng = np.random.default_rng(9)
    sk = (rng.standard_normal((nB, 2 * k)), rng.standard_normal((nC, 2 * k)),
          rng.standard_normal((nA, 2 * k)))
    Gxa, Gxb, Gxc, _, _ = g.scipy_blocks()
    wh = oracle.second_whiten(Gxa, Gxb, Gxc, k, a0, sk)
    with mm.Pipeline(k=k, alpha0=a0) as p:
        p.upload(g).whiten(sk)
        W = p.whitening()["W"]
    err = np.linalg.norm(procrustes_align(wh["W"], W) - wh["W"]) / np.linalg.norm(wh["W"])
    assert err < 1e-4
