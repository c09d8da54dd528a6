"""The generator restated in oracle/mmsb_gen.c (used by the benchmark's CPU
leg, which must not load the GPU library) produces bit-identical blocks to
the library's own generator."""
import numpy as np
import pytest

from conftest import load_oracle


def _gen():
    load_oracle()
    import mmsb_gen
    return mmsb_gen


@pytest.mark.parametrize("n,k,a0,p,q,seed", [(4000, 10, 1.0, 0.3, 0.01, 0),
                                             (20000, 100, 0.1, 0.05, 5e-4, 0),
                                             (3001, 7, 0.5, 0.2, 0.0, 3),
                                             (1000, 40, 2.0, 0.0, 0.02, 9)])
def test_oracle_generator_matches_library(mm, n, k, a0, p, q, seed):
    g = mm.generate(n, k, a0, p, q, seed)
    h = _gen().generate(n, k, a0, p, q, seed)
    assert list(g.parts) == list(h.parts)
    assert g.n_edges == h.n_edges
    for a, b in zip(g.blocks, h.blocks):
        assert (a.n_rows, a.n_cols) == (b.n_rows, b.n_cols)
        np.testing.assert_array_equal(a.row_ptr, b.row_ptr)
        np.testing.assert_array_equal(a.col_idx, b.col_idx)


def test_oracle_generator_rejects_bad_parameters():
    with pytest.raises(ValueError):
        _gen().generate(3, 5, 1.0, 0.1, 0.01)
