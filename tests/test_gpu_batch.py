"""Batched solver (mmsb_batch_*): graphs of uneven n and k solved together,
against each graph solved alone through the single-graph pipeline."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (n, k, alpha0, p_in, p_out): uneven sizes, three padded sizes (32, 48, 64)
GRAPHS = [(2000, 5, 0.5, 0.3, 0.003), (6000, 17, 1.0, 0.2, 0.002), (3000, 40, 0.2, 0.25, 0.0025),
          (12000, 9, 2.0, 0.15, 0.0015), (4000, 33, 0.8, 0.2, 0.002), (8000, 60, 0.3, 0.1, 0.001)]
KW = dict(stpm_method=1, sweeps=3, minibatch=512, seed=100, tau=0.2)


def _graphs(mm):
    return [mm.generate(n, k, a0, pi, po, seed=i) for i, (n, k, a0, pi, po) in enumerate(GRAPHS)]


def _single(mm, graphs, **kw):
    out = []
    for i, ((n, k, a0, _, _), g) in enumerate(zip(GRAPHS, graphs)):
        cfg = dict(KW, **kw)
        cfg["seed"] = KW["seed"] + i
        with mm.Pipeline(k=k, alpha0=a0, **cfg) as p:
            p.upload(g).run()
            out.append((p.lam(), p.pi()))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_single_graph_pipeline(mm, precision):
    """With the contraction CTAs fixed at the single-graph grid, the batched
    launches compute exactly what the single-graph pipeline computes."""
    graphs = _graphs(mm)
    ref = _single(mm, graphs, precision=precision)
    ks = [g[1] for g in GRAPHS]
    a0 = [g[2] for g in GRAPHS]
    with mm.Batch(ks, a0, precision=precision, **KW) as b:
        b.set_contract_ctas(304)  # >= every graph's grid: each uses its single-graph grid
        for i, g in enumerate(graphs):
            b.upload(i, g)
        b.run()
        first = [(b.graph(i).lam(), b.graph(i).pi()) for i in range(len(b))]
        st = b.stats()
        assert st["graph_replayed"] == 0 and st["buckets"] == 3
        assert sorted(st["bucket_kp"]) == [32, 48, 64]
        b.run()  # replay of the captured round loop
        st2 = b.stats()
        assert st2["graph_replayed"] == 1 and st2["batched_launches"] == st["batched_launches"]
        second = [(b.graph(i).lam(), b.graph(i).pi()) for i in range(len(b))]
        lat = b.latencies()
        assert np.all(lat > 0) and np.all(lat <= st2["total_ms"] + 1e-6)
    for (lam_r, pi_r), (lam1, pi1), (lam2, pi2) in zip(ref, first, second):
        np.testing.assert_array_equal(lam1, lam_r)
        np.testing.assert_array_equal(pi1, pi_r)
        np.testing.assert_array_equal(lam2, lam1)
        np.testing.assert_array_equal(pi2, pi1)


def test_batch_autotuned_and_sequential(mm):
    graphs = _graphs(mm)
    ks = [g[1] for g in GRAPHS]
    a0 = [g[2] for g in GRAPHS]
    with mm.Batch(ks, a0, **KW) as b:
        for i, g in enumerate(graphs):
            b.upload(i, g)
        b.run_sequential()
        seq = [(b.graph(i).lam(), b.graph(i).pi()) for i in range(len(b))]
        st_seq = b.stats()
        b.run()
        st = b.stats()
        tuned = [(b.graph(i).lam(), b.graph(i).pi()) for i in range(len(b))]
    assert all(c % 8 == 0 and c >= 8 for c in st["bucket_ctas"])
    assert st_seq["rounds"] == 0 and st["rounds"] == max(
        3 * -(-g.parts[0] // 512) for g in graphs)
    for (lam_s, pi_s), (lam_t, pi_t) in zip(seq, tuned):
        # the tuned CTA count may regroup the node tiles (FP32 summation order)
        assert np.linalg.norm(lam_t - lam_s) / np.linalg.norm(lam_s) < 1e-3
        assert np.abs(pi_t - pi_s).max() < 1e-2


def test_batch_errors(mm):
    with pytest.raises(mm.MmsbError):
        mm.Batch([5, 300], **KW)  # k > 128
    with mm.Batch([5, 6], **KW) as b:
        with pytest.raises(mm.MmsbError) as e:
            b.run()  # nothing uploaded
        assert e.value.status == 4
        with pytest.raises(mm.MmsbError):
            b.set_contract_ctas(12)  # not a multiple of the cluster size
