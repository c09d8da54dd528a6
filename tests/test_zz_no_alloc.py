"""mmsb_op_spmm_t_noalloc: the transposed SpMM for callers that cannot
allocate device memory (code inside another framework's memory pool, or
latency-critical code that must not wait on cudaMalloc).  Its result must equal the allocating
entry point mmsb_op_spmm(transpose=1) on the same inputs, call after call,
because every call reuses the same fixed device array.

This file is collected last on purpose: if it fails, a run stopping at the
first failure has already run every other test.  The caller-owned device
buffers are made with torch, standing in for the caller's own allocator."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def make_block(rng, n_rows, n_cols, density, weighted):
    m = sp.random(n_rows, n_cols, density=density, format="csr", random_state=rng)
    m.data[:] = rng.uniform(0.5, 2.0, m.nnz) if weighted else 1.0
    m = m.tolil()
    for r in range(0, n_rows, 9):  # empty rows
        m.rows[r] = []
        m.data[r] = []
    return m.tocsr()


def test_noalloc_transposed_spmm_matches_allocating_entry(mm):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on different blocks (the second weighted and wider):
    # the shared array must be reset by each call
    for call, (n_rows, n_cols, p, weighted) in enumerate([(3000, 1200, 20, False),
                                                          (2500, 1700, 36, True)]):
        G = make_block(rng, n_rows, n_cols, 0.01, weighted)
        blk = mm.CsrBlock.from_scipy(G)
        P = rng.standard_normal((n_rows, p)).astype(np.float32)
        alpha = 0.75 + call
        ref = mm.spmm(blk, P, transpose=True, alpha=alpha)
        d_rp = torch.from_numpy(blk.row_ptr).cuda()
        d_ci = torch.from_numpy(blk.col_idx).cuda()
        d_val = torch.from_numpy(blk.val).cuda() if blk.val is not None else None
        d_P = torch.from_numpy(P).cuda()
        d_Y = torch.full((n_cols, p), float("nan"), device="cuda", dtype=torch.float32)
        st = mm.spmm_t_noalloc(d_rp.data_ptr(), d_ci.data_ptr(),
                               d_val.data_ptr() if d_val is not None else None, n_rows, n_cols,
                               blk.nnz, d_P.data_ptr(), p, alpha, d_Y.data_ptr(), stream)
        assert st == 0
        torch.cuda.synchronize()
        assert rel(d_Y.cpu().numpy(), ref) < 1e-5
    # a block whose transpose does not fit the fixed array is refused before any work
    st = mm.spmm_t_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), None, n_rows, 1_000_000, blk.nnz,
                           d_P.data_ptr(), p, 1.0, d_Y.data_ptr(), stream)
    assert st == 9  # MMSB_ERR_UNSUPPORTED
