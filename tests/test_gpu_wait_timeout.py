"""Failure detection on the device without faulting it: a bounded wait whose
barrier nothing arrives at gives up after its limit, the call returns
MMSB_ERR_TIMEOUT, and the same context then runs a whole pipeline correctly
(the flag is cleared, no kernel is left behind).  The wait limit of the STPM
kernels is a per-context setting; a limit far above any real wait changes no
result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 8


def test_bounded_wait_times_out_and_context_stays_usable(mm, golden_cfg1):
    g = golden_cfg1
    with mm.Pipeline(k=g.k, alpha0=g.alpha0, stpm_method=mm.STPM_ONLINE, sweeps=2,
                     minibatch=100, seed=3) as p:
        p.upload(g.graph(mm)).run()
        lam0, pi0 = p.lam().copy(), p.pi().copy()
        for cycles in (1000, 200000):
            assert p.diag_wait_timeout(cycles) == TIMEOUT
        assert mm.lib().mmsb_diag_wait_timeout(p._h, 0) == 1  # limit out of range
        p.run()
        np.testing.assert_array_equal(p.lam(), lam0)
        np.testing.assert_array_equal(p.pi(), pi0)
        # an explicit limit (about half a second) on the real kernels' waits
        p.set_wait_limit(1_000_000_000).run()
        np.testing.assert_array_equal(p.lam(), lam0)
        with pytest.raises(mm.MmsbError):
            p.set_wait_limit(-1)
