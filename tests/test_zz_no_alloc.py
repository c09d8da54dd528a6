"""mmsb_op_spmm_t_noalloc: the transposed SpMM for callers that cannot
allocate device memory (code inside another framework's memory pool, or
latency-critical code that must not wait on cudaMalloc).  Its result must equal the allocating
entry point mmsb_op_spmm(transpose=1) on the same inputs, and G^T P in
float64, call after call, because every call reuses the same fixed device
array.

This file is collected last on purpose: if it fails, a run stopping at the
first failure has already run every other test.  The caller-owned device
buffers are made with torch, standing in for the caller's own allocator."""
import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

LIMIT = 8 << 20  # bytes of the fixed device array


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make_block(rng, n_rows, n_cols, density, weighted, used_cols=None):
    m = sp.random(n_rows, used_cols or n_cols, density=density, format="csr", random_state=rng)
    m.data[:] = rng.uniform(0.5, 2.0, m.nnz) if weighted else 1.0
    m = m.tolil()
    for r in range(0, n_rows, 9):  # empty rows
        m.rows[r] = []
        m.data[r] = []
    m = m.tocsr()
    if used_cols:  # columns past used_cols have no entries: their output rows must be 0
        m = sp.csr_matrix((m.data, m.indices, m.indptr), shape=(n_rows, n_cols))
    return m


def need_bytes(n_cols, nnz, weighted):
    a = lambda b: (b + 255) // 256 * 256
    vb = 4 if weighted else 0
    return (a(8 * (n_cols + 1)) + a((4 + vb) * nnz + 8) + a(8 * (n_cols + 1)) + a(4 * nnz + 4)
            + (a(4 * nnz + 4) if weighted else 0))


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _call(mm, torch, G, P, alpha, stream, y_offset=0):
    blk = mm.CsrBlock.from_scipy(G)
    n_rows, n_cols = G.shape
    p = P.shape[1]
    d_rp = torch.from_numpy(blk.row_ptr).cuda()
    d_ci = torch.from_numpy(blk.col_idx if blk.nnz else np.zeros(1, np.int32)).cuda()
    d_val = torch.from_numpy(blk.val).cuda() if blk.val is not None else None
    d_P = torch.from_numpy(P).cuda()
    d_Ybuf = torch.full((n_cols * p + 16,), float("nan"), device="cuda", dtype=torch.float32)
    d_Y = d_Ybuf[y_offset:y_offset + n_cols * p]
    st = mm.spmm_t_noalloc(d_rp.data_ptr(), d_ci.data_ptr(),
                           d_val.data_ptr() if d_val is not None else None, n_rows, n_cols,
                           blk.nnz, d_P.data_ptr(), p, alpha, d_Y.data_ptr(), stream)
    torch.cuda.synchronize()
    return st, d_Y.cpu().numpy().reshape(n_cols, p), blk


def test_noalloc_transposed_spmm_matches_allocating_entry(mm):
    torch = _torch()
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    # calls in a row on different blocks (weighted and wider, a block whose
    # last columns are empty, an empty block, one just under the array's
    # limit): the shared array must be reset by each call
    cases = [(3000, 1200, 20, False, 0.01, None), (2500, 1700, 36, True, 0.01, None),
             (2000, 1500, 8, False, 0.01, 1000), (700, 300, 12, True, 0.0, None)]
    # binary block: 2 * 8 (n_cols + 1) bytes of counters and offsets plus
    # 8 bytes per nonzero (staging and transposed columns), each part padded
    # to 256 bytes; nnz chosen to leave less than 1 KiB of the array unused
    n_big, c_big = 60_000, 4000
    nnz_big = (LIMIT - 2 * ((8 * (c_big + 1) + 255) // 256 * 256) - 1024) // 8
    cases.append((n_big, c_big, 4, False, nnz_big, None))
    for call, (n_rows, n_cols, p, weighted, density, used) in enumerate(cases):
        if density >= 1:  # an exact nonzero count
            G = sp.random(n_rows, n_cols, density=density / (n_rows * n_cols), format="csr",
                          random_state=rng)
            G.data[:] = 1.0
            assert LIMIT - need_bytes(n_cols, G.nnz, weighted) < 2048
        else:
            G = make_block(rng, n_rows, n_cols, density, weighted, used)
        assert need_bytes(n_cols, G.nnz, weighted) <= LIMIT
        P = rng.standard_normal((n_rows, p)).astype(np.float32)
        alpha = 0.75 + call
        st, Y, blk = _call(mm, torch, G, P, alpha, stream)
        assert st == 0
        ref = mm.spmm(blk, P, transpose=True, alpha=alpha)
        exact = alpha * (G.T @ P.astype(np.float64))
        assert rel(Y, ref) < 1e-5
        assert np.abs(Y - exact).max() <= 1e-5 * max(np.abs(exact).max(), 1.0)
        if used:
            assert np.all(Y[used:] == 0)
        if G.nnz == 0:
            assert np.all(Y == 0)


def test_noalloc_refusals(mm):
    torch = _torch()
    rng = np.random.default_rng(12)
    stream = torch.cuda.current_stream().cuda_stream
    G = make_block(rng, 500, 400, 0.02, False)
    P = rng.standard_normal((500, 8)).astype(np.float32)
    # an output view 4 bytes off a 16-byte boundary
    st, _, _ = _call(mm, torch, G, P, 1.0, stream, y_offset=1)
    assert st == 1  # MMSB_ERR_INVALID_ARG
    # a block whose transpose does not fit the fixed array is refused before any work
    blk = mm.CsrBlock.from_scipy(G)
    d_rp = torch.from_numpy(blk.row_ptr).cuda()
    d_ci = torch.from_numpy(blk.col_idx).cuda()
    d_P = torch.from_numpy(P).cuda()
    d_Y = torch.zeros((1_000_000, 8), device="cuda")
    st = mm.spmm_t_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), None, 500, 1_000_000, blk.nnz,
                           d_P.data_ptr(), 8, 1.0, d_Y.data_ptr(), stream)
    assert st == 9  # MMSB_ERR_UNSUPPORTED
    st = mm.spmm_t_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), None, 500, 400, 1 << 40,
                           d_P.data_ptr(), 8, 1.0, d_Y.data_ptr(), stream)
    assert st == 9  # no size product wraps
    # a correct call still works after the refusals
    st, Y, blk = _call(mm, torch, G, P, 2.0, stream)
    assert st == 0 and rel(Y, 2.0 * (G.T @ P.astype(np.float64))) < 1e-5
