"""Python host mirror of the GB300 MMSB tensor-method library (include/mmsb.h).

The product is the C ABI in ``lib/libmmsb.so`` (host C++ + sm_103a CUDA
kernels).  This module binds it with ctypes and mirrors the reference's
interface for the path:

  reference                                          here
  -------------------------------------------------  ---------------------------
  second_whiten(Gx_a, Gx_b, Gx_c, W, Z_B_part1, ...)  Pipeline.whiten / second_whiten
    (CommunityDetectionSoftware_CPU/.../Util.cpp:38)
  tensorDecom_alpha0(D_a, D_a_mu, ..., lambda, phi)   Pipeline.stpm / tensor_decom_alpha0
    (Util.cpp:131)
  main() post-processing + normProbMatrix             Pipeline.postproc
    (CommunityDetection.cpp:89-139)
  read_G_sparse / write_pi (IOfn.cpp:21, 57)          read_coo / write_triplets

There is no CPU fallback: if the shared library is missing, importing works but
every call raises ``LibraryNotBuilt``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libmmsb.so"
# command line with the reference executable's argv and output files
CLI_PATH = PKG_DIR / "lib" / "mmsb_cli"
CSRC = PKG_DIR / "csrc"

OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
          4: "call out of order", 5: "numerical failure", 6: "stopped on request",
          7: "I/O error", 8: "device wait timed out", 9: "unsupported configuration"}

BLOCK_XA, BLOCK_XB, BLOCK_XC, BLOCK_BA, BLOCK_CA = range(5)
STPM_BATCH_POWER, STPM_ONLINE, STPM_ADJOINT = range(3)
PREC_FP32, PREC_BF16 = range(2)


class LibraryNotBuilt(RuntimeError):
    pass


class MmsbError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("k", ctypes.c_int32), ("alpha0", ctypes.c_double),
                ("datatype", ctypes.c_int32), ("stpm_method", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("sweeps", ctypes.c_int32),
                ("minibatch", ctypes.c_int32), ("lr0", ctypes.c_double),
                ("theta", ctypes.c_double), ("min_iter", ctypes.c_int32),
                ("max_iter", ctypes.c_int32), ("tol", ctypes.c_double),
                ("pinv_tol", ctypes.c_double), ("nystrom_rows_factor", ctypes.c_int32),
                ("normalize", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("tau", ctypes.c_float), ("device", ctypes.c_int32)]


class Csr(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_int64), ("n_cols", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("row_ptr", ctypes.POINTER(ctypes.c_int64)),
                ("col_idx", ctypes.POINTER(ctypes.c_int32)),
                ("val", ctypes.POINTER(ctypes.c_float))]


class Stats(ctypes.Structure):
    _fields_ = [("whiten_ms", ctypes.c_double), ("ydata_ms", ctypes.c_double),
                ("stpm_ms", ctypes.c_double), ("post_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("spmm_ms", ctypes.c_double),
                ("spmm_bytes", ctypes.c_double), ("spmm_launches", ctypes.c_int64),
                ("stpm_steps", ctypes.c_int64), ("node_updates", ctypes.c_int64),
                ("stpm_last_error", ctypes.c_double), ("kernel_launches", ctypes.c_int64),
                ("orth_passes", ctypes.c_int64), ("contract_ms", ctypes.c_double),
                ("contract_flops", ctypes.c_double), ("contract_launches", ctypes.c_int64),
                ("step_ms", ctypes.c_double), ("step_flops", ctypes.c_double),
                ("step_launches", ctypes.c_int64), ("orth_err_max", ctypes.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchStats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("stpm_end_ms", ctypes.c_double),
                ("wall_ms", ctypes.c_double), ("latency_p50_ms", ctypes.c_double),
                ("latency_p99_ms", ctypes.c_double), ("latency_max_ms", ctypes.c_double),
                ("rounds", ctypes.c_int64), ("batched_launches", ctypes.c_int64),
                ("graph_replayed", ctypes.c_int32), ("buckets", ctypes.c_int32),
                ("bucket_kp", ctypes.c_int32 * 8), ("bucket_ctas", ctypes.c_int32 * 8),
                ("bucket_graphs", ctypes.c_int32 * 8)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v)[:self.buckets] if name.startswith("bucket_") else v
        return d


class GenParams(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("k", ctypes.c_int32), ("alpha0", ctypes.c_double),
                ("p_in", ctypes.c_double), ("p_out", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("keep_pi", ctypes.c_int32)]


_lib = None

_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_SIGS = {
    "mmsb_config_default": (None, [ctypes.POINTER(Config)]),
    "mmsb_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "mmsb_destroy": (None, [_P]),
    "mmsb_upload_graph": (ctypes.c_int, [_P, ctypes.POINTER(Csr)]),
    "mmsb_host_register": (ctypes.c_int, [_P, ctypes.c_size_t]),
    "mmsb_host_unregister": (ctypes.c_int, [_P]),
    "mmsb_whiten": (ctypes.c_int, [_P, ctypes.POINTER(_D)]),
    "mmsb_stpm": (ctypes.c_int, [_P, _D]),
    "mmsb_postproc": (ctypes.c_int, [_P]),
    "mmsb_run": (ctypes.c_int, [_P]),
    "mmsb_num_nodes": (ctypes.c_int64, [_P]),
    "mmsb_get_pi": (ctypes.c_int, [_P, _F]),
    "mmsb_get_sets": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "mmsb_get_lambda": (ctypes.c_int, [_P, _D]),
    "mmsb_get_phi": (ctypes.c_int, [_P, _D]),
    "mmsb_get_whitening": (ctypes.c_int, [_P, _D, _D, _D, _D, _D]),
    "mmsb_get_means": (ctypes.c_int, [_P, _D, _D, _D]),
    "mmsb_get_whitened": (ctypes.c_int, [_P, _F, _F, _F, _D, _D, _D]),
    "mmsb_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "mmsb_set_whitening": (ctypes.c_int, [_P, _D, _D, _D, _D, _D, _D, _D, _D]),
    "mmsb_set_whitened": (ctypes.c_int, [_P, _D, _D, _D, _D, _D, _D]),
    "mmsb_set_phi_lambda": (ctypes.c_int, [_P, _D, _D]),
    "mmsb_stpm_loss_fwd": (ctypes.c_int, [_P, _D, ctypes.c_int64, ctypes.c_int64, _D]),
    "mmsb_stpm_loss_bwd": (ctypes.c_int, [_P, _D, ctypes.c_int64, ctypes.c_int64, _D]),
    "mmsb_request_stop": (None, [_P]),
    "mmsb_last_error": (ctypes.c_char_p, [_P]),
    "mmsb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "mmsb_flush_l2": (ctypes.c_int, [_P]),
    "mmsb_synchronize": (ctypes.c_int, [_P]),
    "mmsb_op_spmm": (ctypes.c_int, [ctypes.POINTER(Csr), ctypes.c_int, _F, ctypes.c_int64,
                                    ctypes.c_float, _F]),
    "mmsb_op_symeig": (ctypes.c_int, [_D, ctypes.c_int32, _D, _D]),
    "mmsb_set_wait_limit": (ctypes.c_int, [_P, ctypes.c_int64]),
    "mmsb_diag_wait_timeout": (ctypes.c_int, [_P, ctypes.c_int64]),
    "mmsb_op_spmm_t_noalloc": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_float,
                                              _P, _P]),
    "mmsb_batch_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32), _D,
                                         ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(_P)]),
    "mmsb_batch_destroy": (None, [_P]),
    "mmsb_batch_upload": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(Csr)]),
    "mmsb_batch_run": (ctypes.c_int, [_P]),
    "mmsb_batch_run_sequential": (ctypes.c_int, [_P]),
    "mmsb_batch_count": (ctypes.c_int32, [_P]),
    "mmsb_batch_set_contract_ctas": (ctypes.c_int, [_P, ctypes.c_int32]),
    "mmsb_batch_graph": (_P, [_P, ctypes.c_int32]),
    "mmsb_batch_latencies": (ctypes.c_int, [_P, _D]),
    "mmsb_batch_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(BatchStats)]),
    "mmsb_batch_last_error": (ctypes.c_char_p, [_P]),
    "mmsb_generate": (ctypes.c_int, [ctypes.POINTER(GenParams), ctypes.POINTER(_P)]),
    "mmsb_host_graph_free": (None, [_P]),
    "mmsb_host_graph_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64),
                                            ctypes.POINTER(ctypes.c_int64)]),
    "mmsb_host_graph_block": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(Csr)]),
    "mmsb_host_graph_pi": (ctypes.c_int, [_P, _F]),
    "mmsb_read_coo": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_P)]),
    "mmsb_write_triplets_f32": (ctypes.c_int, [ctypes.c_char_p, _F, ctypes.c_int64,
                                               ctypes.c_int64]),
    "mmsb_write_triplets_f64": (ctypes.c_int, [ctypes.c_char_p, _D, ctypes.c_int64,
                                               ctypes.c_int64]),
    "mmsb_write_dense_f32": (ctypes.c_int, [ctypes.c_char_p, _F, ctypes.c_int64]),
    "mmsb_write_dense_f64": (ctypes.c_int, [ctypes.c_char_p, _D, ctypes.c_int64]),
    "mmsb_write_coo": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Csr)]),
    "mmsb_write_csr": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Csr)]),
    "mmsb_read_csr": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "mmsb_pvalues": (ctypes.c_int, [_P, _F, ctypes.c_int32, _D, _D, _D]),
    "mmsb_op_gram": (ctypes.c_int, [_F, ctypes.c_int64, ctypes.c_int32, _F, ctypes.c_int32,
                                    ctypes.c_double, _D]),
    "mmsb_get_convergence": (ctypes.c_int, [_P, _D, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "mmsb_write_gpu_outputs": (ctypes.c_int, [_P, ctypes.c_char_p]),
}


def build(jobs: int = 8, quiet: bool = True) -> Path:
    """Compile lib/libmmsb.so for sm_103a (nvcc + g++, in-tree)."""
    out = subprocess.run(["make", "-C", str(CSRC), f"-j{jobs}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("libmmsb build failed:\n" + out.stdout[-4000:] + out.stderr[-4000:])
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def lib():
    """The loaded C library; raises LibraryNotBuilt if lib/libmmsb.so is absent."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise LibraryNotBuilt(f"{LIB_PATH} is missing: run build() first (no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def _check(st, ctx=None):
    if st != OK:
        msg = lib().mmsb_last_error(ctx).decode() if ctx is not None else ""
        raise MmsbError(st, msg)


def _dptr(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _fptr(a):
    return a.ctypes.data_as(_F) if a is not None else None


def default_config(**kw) -> Config:
    c = Config()
    lib().mmsb_config_default(ctypes.byref(c))
    for k_, v in kw.items():
        if not hasattr(c, k_):
            raise KeyError(k_)
        setattr(c, k_, v)
    return c


# ---- host graphs -------------------------------------------------------------

class CsrBlock:
    """Host CSR block (numpy arrays; int64 row offsets, int32 columns)."""

    def __init__(self, n_rows, n_cols, row_ptr, col_idx, val=None):
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        self.row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        self.col_idx = np.ascontiguousarray(col_idx, dtype=np.int32)
        self.val = None if val is None else np.ascontiguousarray(val, dtype=np.float32)

    @property
    def nnz(self):
        return int(self.col_idx.size)

    def ctype(self) -> Csr:
        c = Csr()
        c.n_rows, c.n_cols, c.nnz = self.n_rows, self.n_cols, self.nnz
        c.row_ptr = self.row_ptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        c.col_idx = self.col_idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        c.val = self.val.ctypes.data_as(_F) if self.val is not None else None
        return c

    def to_scipy(self):
        import scipy.sparse as sp
        v = self.val if self.val is not None else np.ones(self.nnz)
        return sp.csr_matrix((v.astype(np.float64), self.col_idx, self.row_ptr),
                             shape=(self.n_rows, self.n_cols))

    @staticmethod
    def from_scipy(m):
        m = m.tocsr()
        m.sort_indices()
        vals = None if np.all(m.data == 1) else m.data
        return CsrBlock(m.shape[0], m.shape[1], m.indptr, m.indices, vals)


class Graph:
    """The five adjacency blocks X->A, X->B, X->C, B->A, C->A plus metadata."""

    def __init__(self, blocks, parts, n_edges=None, pi=None):
        self.blocks = list(blocks)
        self.parts = tuple(int(p) for p in parts)
        self.n_edges = n_edges
        self.pi = pi

    @property
    def n_nodes(self):
        return sum(self.parts)

    def scipy_blocks(self):
        return [b.to_scipy() for b in self.blocks]

    def _arrays(self):
        for b in self.blocks:
            for a in (b.row_ptr, b.col_idx, b.val):
                if a is not None and a.nbytes:
                    yield a

    def pin(self):
        """Page-lock the blocks' host arrays (mmsb_host_register) so that
        uploads copy them by direct DMA; undo with unpin()."""
        for a in self._arrays():
            pin_host(a)
        return self

    def unpin(self):
        for a in self._arrays():
            unpin_host(a)
        return self


def pin_host(a: np.ndarray):
    """Page-lock a contiguous host array in place (mmsb_host_register)."""
    if not a.flags["C_CONTIGUOUS"] and not a.flags["F_CONTIGUOUS"]:
        raise ValueError("pin_host needs a contiguous array")
    _check(lib().mmsb_host_register(a.ctypes.data, a.nbytes))
    return a


def unpin_host(a: np.ndarray):
    _check(lib().mmsb_host_unregister(a.ctypes.data))
    return a


def generate(n, k, alpha0, p_in, p_out, seed=0, keep_pi=False) -> Graph:
    """Seeded synthetic MMSB graph (C++ generator in the library)."""
    L = lib()
    h = _P()
    _check(L.mmsb_generate(ctypes.byref(GenParams(n, k, alpha0, p_in, p_out, seed,
                                                  int(keep_pi))), ctypes.byref(h)))
    try:
        parts = (ctypes.c_int64 * 4)()
        ne = ctypes.c_int64()
        _check(L.mmsb_host_graph_info(h, parts, ctypes.byref(ne)))
        blocks = []
        for b in range(5):
            c = Csr()
            _check(L.mmsb_host_graph_block(h, b, ctypes.byref(c)))
            rp = np.ctypeslib.as_array(c.row_ptr, (c.n_rows + 1,)).copy()
            ci = (np.ctypeslib.as_array(c.col_idx, (c.nnz,)).copy() if c.nnz
                  else np.zeros(0, np.int32))
            blocks.append(CsrBlock(c.n_rows, c.n_cols, rp, ci))
        pi = None
        if keep_pi:
            pi = np.zeros((n, k), dtype=np.float32)
            _check(L.mmsb_host_graph_pi(h, _fptr(pi)))
        return Graph(blocks, list(parts), ne.value, pi)
    finally:
        L.mmsb_host_graph_free(h)


def _block_from_handle(L, h) -> CsrBlock:
    try:
        c = Csr()
        _check(L.mmsb_host_graph_block(h, 0, ctypes.byref(c)))
        rp = np.ctypeslib.as_array(c.row_ptr, (c.n_rows + 1,)).copy()
        ci = np.ctypeslib.as_array(c.col_idx, (c.nnz,)).copy() if c.nnz else np.zeros(0, np.int32)
        val = np.ctypeslib.as_array(c.val, (c.nnz,)).copy() if (c.val and c.nnz) else None
        return CsrBlock(c.n_rows, c.n_cols, rp, ci, val)
    finally:
        L.mmsb_host_graph_free(h)


def read_coo(path, n_rows, n_cols, datatype=0, compat=False) -> CsrBlock:
    """read_G_sparse (IOfn.cpp:21-54) on up to 16 threads; compat=True
    reproduces its loop exactly (see mmsb_read_coo)."""
    L = lib()
    h = _P()
    _check(L.mmsb_read_coo(str(path).encode(), n_rows, n_cols, datatype, int(compat),
                           ctypes.byref(h)))
    return _block_from_handle(L, h)


def write_coo(path, block: CsrBlock):
    """The input contract: 1-based "row col[ value]" lines (mmsb_write_coo)."""
    c = block.ctype()
    _check(lib().mmsb_write_coo(str(path).encode(), ctypes.byref(c)))


def write_csr(path, block: CsrBlock):
    """Binary CSR container (mmsb_write_csr)."""
    c = block.ctype()
    _check(lib().mmsb_write_csr(str(path).encode(), ctypes.byref(c)))


def read_csr(path) -> CsrBlock:
    L = lib()
    h = _P()
    _check(L.mmsb_read_csr(str(path).encode(), ctypes.byref(h)))
    return _block_from_handle(L, h)


def write_dense(path, m):
    """write_mat (GPU/post_proc.c:45-59): one "%5.25e" value per line, in
    column-major order."""
    m = np.asfortranarray(m)
    if m.dtype == np.float32:
        _check(lib().mmsb_write_dense_f32(str(path).encode(), m.ctypes.data_as(_F), m.size))
    else:
        m = np.asfortranarray(m, dtype=np.float64)
        _check(lib().mmsb_write_dense_f64(str(path).encode(), m.ctypes.data_as(_D), m.size))


def write_triplets(path, m):
    """write_pi (IOfn.cpp:57-67): 1-based row/col/value of the nonzeros."""
    m = np.asfortranarray(m)
    if m.dtype == np.float32:
        _check(lib().mmsb_write_triplets_f32(str(path).encode(), m.ctypes.data_as(_F),
                                              m.shape[0], m.shape[1]))
    else:
        m = np.asfortranarray(m, dtype=np.float64)
        _check(lib().mmsb_write_triplets_f64(str(path).encode(), m.ctypes.data_as(_D),
                                              m.shape[0], m.shape[1]))


# ---- the pipeline ---------------------------------------------------------------

class Pipeline:
    """One GPU context: upload -> whiten -> stpm -> postproc (host numpy in/out)."""

    def __init__(self, config: Config | None = None, **kw):
        self.cfg = config if config is not None else default_config(**kw)
        h = _P()
        _check(lib().mmsb_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self._h = h
        self.k = self.cfg.k
        self.parts = None

    def close(self):
        if getattr(self, "_h", None) and not getattr(self, "_borrowed", False):
            lib().mmsb_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st):
        _check(st, self._h)

    def upload(self, graph: Graph):
        arr = (Csr * 5)(*[b.ctype() for b in graph.blocks])
        self._keep = graph
        self._ck(lib().mmsb_upload_graph(self._h, arr))
        self.parts = graph.parts
        return self

    def whiten(self, sketches=None):
        if sketches is None:
            self._ck(lib().mmsb_whiten(self._h, None))
        else:
            sk = [np.asfortranarray(s, dtype=np.float64) for s in sketches]
            arr = (_D * 3)(*[_dptr(s) for s in sk])
            self._ck(lib().mmsb_whiten(self._h, arr))
        return self

    def stpm(self, phi0=None):
        p = None if phi0 is None else np.asfortranarray(phi0, dtype=np.float64)
        self._ck(lib().mmsb_stpm(self._h, _dptr(p)))
        return self

    def postproc(self):
        self._ck(lib().mmsb_postproc(self._h))
        return self

    def run(self):
        self._ck(lib().mmsb_run(self._h))
        return self

    def synchronize(self):
        self._ck(lib().mmsb_synchronize(self._h))

    def flush_l2(self):
        self._ck(lib().mmsb_flush_l2(self._h))

    def set_wait_limit(self, cycles):
        """clock64 cycles a bounded device wait may take (0 = about one second)."""
        self._ck(lib().mmsb_set_wait_limit(self._h, int(cycles)))
        return self

    def diag_wait_timeout(self, cycles):
        """One bounded wait on a barrier nothing arrives at; returns the status
        (MMSB_ERR_TIMEOUT = 8 when the give-up path works)."""
        return lib().mmsb_diag_wait_timeout(self._h, int(cycles))

    def request_stop(self):
        lib().mmsb_request_stop(self._h)

    # results
    def n_nodes(self):
        return int(lib().mmsb_num_nodes(self._h))

    def pi(self, out=None):
        """Memberships, k x N (column-major); out: a preallocated float32
        array of that shape and order to fill (e.g. one pinned with pin_host)."""
        shape = (self.k, self.n_nodes())
        if out is None:
            out = np.empty(shape, dtype=np.float32, order="F")
        elif out.shape != shape or out.dtype != np.float32 or not out.flags["F_CONTIGUOUS"]:
            raise ValueError(f"out must be a float32 column-major {shape} array")
        self._ck(lib().mmsb_get_pi(self._h, _fptr(out)))
        return out

    def pvalues(self, truth):
        """Correlation, t statistic and two-sided p-value (Pvalue.cpp) of every
        (estimated, true) community pair; truth: K x N memberships in the node
        order [X|A|B|C].  Returns three k x K FP64 arrays."""
        truth = np.asfortranarray(truth, dtype=np.float32)
        K = truth.shape[0]
        if truth.shape[1] != self.n_nodes():
            raise ValueError("truth must be K x N")
        out = [np.zeros((self.k, K), dtype=np.float64, order="F") for _ in range(3)]
        self._ck(lib().mmsb_pvalues(self._h, _fptr(truth), K, *(o.ctypes.data_as(_D) for o in out)))
        return tuple(out)

    def convergence(self):
        """Convergence trace of the last stpm (mmsb_get_convergence)."""
        n = ctypes.c_int64()
        self._ck(lib().mmsb_get_convergence(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        if n.value:
            self._ck(lib().mmsb_get_convergence(self._h, out.ctypes.data_as(_D), n.value,
                                                ctypes.byref(n)))
        return out

    def write_gpu_outputs(self, directory):
        """The GPU tree's output files (mmsb_write_gpu_outputs)."""
        self._ck(lib().mmsb_write_gpu_outputs(self._h, str(directory).encode()))
        return self

    def sets(self):
        words = (self.k + 31) // 32
        out = np.zeros((self.n_nodes(), words), dtype=np.uint32)
        self._ck(lib().mmsb_get_sets(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        bits = np.unpackbits(out.view(np.uint8), axis=1, bitorder="little")[:, :self.k]
        return bits.T.astype(bool)

    def lam(self):
        out = np.zeros(self.k)
        self._ck(lib().mmsb_get_lambda(self._h, _dptr(out)))
        return out

    def phi(self):
        out = np.zeros((self.k, self.k), order="F")
        self._ck(lib().mmsb_get_phi(self._h, _dptr(out)))
        return out

    def whitening(self):
        nX, nA, nB, nC = self.parts
        k = self.k
        W, zb1, zc1 = (np.zeros((nA, k), order="F") for _ in range(3))
        zb2 = np.zeros((k, nB), order="F")
        zc2 = np.zeros((k, nC), order="F")
        self._ck(lib().mmsb_get_whitening(self._h, _dptr(W), _dptr(zb1), _dptr(zb2), _dptr(zc1),
                                          _dptr(zc2)))
        mu = [np.zeros(n) for n in (nA, nB, nC)]
        self._ck(lib().mmsb_get_means(self._h, *[_dptr(m) for m in mu]))
        return dict(W=W, Zb1=zb1, Zb2=zb2, Zc1=zc1, Zc2=zc2, mu_a=mu[0], mu_b=mu[1], mu_c=mu[2])

    def whitened(self):
        nX = self.parts[0]
        k = self.k
        ys = [np.zeros((k, nX), dtype=np.float32, order="F") for _ in range(3)]
        ms = [np.zeros(k) for _ in range(3)]
        self._ck(lib().mmsb_get_whitened(self._h, *[_fptr(y) for y in ys], *[_dptr(m) for m in ms]))
        return dict(Da=ys[0], Db=ys[1], Dc=ys[2], Da_mu=ms[0], Db_mu=ms[1], Dc_mu=ms[2])

    def stats(self):
        s = Stats()
        self._ck(lib().mmsb_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    # stage inputs
    def set_whitening(self, wh):
        arrs = [np.asfortranarray(wh[n], dtype=np.float64)
                for n in ("W", "Zb1", "Zb2", "Zc1", "Zc2", "mu_a", "mu_b", "mu_c")]
        self._ck(lib().mmsb_set_whitening(self._h, *[_dptr(a) for a in arrs]))
        return self

    def set_whitened(self, y):
        arrs = [np.asfortranarray(y[n], dtype=np.float64)
                for n in ("Da", "Db", "Dc", "Da_mu", "Db_mu", "Dc_mu")]
        self._ck(lib().mmsb_set_whitened(self._h, *[_dptr(a) for a in arrs]))
        return self

    def set_phi_lambda(self, phi, lam):
        p = np.asfortranarray(phi, dtype=np.float64)
        l_ = np.ascontiguousarray(lam, dtype=np.float64)
        self._ck(lib().mmsb_set_phi_lambda(self._h, _dptr(p), _dptr(l_)))
        return self

    # adjoint form
    def loss(self, phi, begin=0, count=0):
        p = np.asfortranarray(phi, dtype=np.float64)
        out = ctypes.c_double()
        self._ck(lib().mmsb_stpm_loss_fwd(self._h, _dptr(p), begin, count, ctypes.byref(out)))
        return out.value

    def loss_grad(self, phi, begin=0, count=0):
        p = np.asfortranarray(phi, dtype=np.float64)
        out = np.zeros((self.k, self.k), order="F")
        self._ck(lib().mmsb_stpm_loss_bwd(self._h, _dptr(p), begin, count, _dptr(out)))
        return out


# ---- reference-named convenience wrappers ----------------------------------------

class Batch:
    """Many independent graphs solved together (mmsb_batch_*): per-graph k and
    alpha0, every other setting from the keyword arguments."""

    def __init__(self, ks, alpha0s=None, minibatches=None, **kw):
        self.cfg = default_config(**kw)
        ks = np.ascontiguousarray(ks, dtype=np.int32)
        a0 = None if alpha0s is None else np.ascontiguousarray(alpha0s, dtype=np.float64)
        mbs = None if minibatches is None else np.ascontiguousarray(minibatches, dtype=np.int32)
        h = _P()
        i32 = ctypes.POINTER(ctypes.c_int32)
        st = lib().mmsb_batch_create(ctypes.byref(self.cfg), len(ks), ks.ctypes.data_as(i32),
                                     _dptr(a0), None if mbs is None else mbs.ctypes.data_as(i32),
                                     ctypes.byref(h))
        _check(st)
        self._h = h
        self.ks = ks
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            lib().mmsb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.ks)

    def _ck(self, st):
        if st != 0:
            msg = lib().mmsb_batch_last_error(self._h).decode()
            raise MmsbError(st, msg)

    def upload(self, i, graph: Graph):
        arr = (Csr * 5)(*[b.ctype() for b in graph.blocks])
        self._keep[i] = graph
        self._ck(lib().mmsb_batch_upload(self._h, i, arr))
        return self

    def set_contract_ctas(self, ctas):
        self._ck(lib().mmsb_batch_set_contract_ctas(self._h, ctas))
        return self

    def run(self):
        self._ck(lib().mmsb_batch_run(self._h))
        return self

    def run_sequential(self):
        self._ck(lib().mmsb_batch_run_sequential(self._h))
        return self

    def stats(self):
        s = BatchStats()
        self._ck(lib().mmsb_batch_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def latencies(self):
        out = np.zeros(len(self.ks))
        self._ck(lib().mmsb_batch_latencies(self._h, _dptr(out)))
        return out

    def graph(self, i):
        """Results view of graph i (a Pipeline sharing the batch's context)."""
        v = Pipeline.__new__(Pipeline)
        v._h = lib().mmsb_batch_graph(self._h, i)
        v.k = int(self.ks[i])
        v.parts = self._keep[i].parts
        v.cfg = self.cfg
        v._borrowed = True
        return v


def second_whiten(graph: Graph, k, alpha0, sketches=None, **cfg):
    """second_whiten (Util.cpp:38-127) on the GPU; returns W, Z parts and means."""
    with Pipeline(k=k, alpha0=alpha0, **cfg) as p:
        p.upload(graph).whiten(sketches)
        return p.whitening()


def spmm(block: CsrBlock, P, transpose=False, alpha=1.0):
    """Y = alpha * G P (or G^T P) through the library's CSR SpMM kernel."""
    P = np.ascontiguousarray(P, dtype=np.float32)
    n_out = block.n_cols if transpose else block.n_rows
    Y = np.zeros((n_out, P.shape[1]), dtype=np.float32)
    c = block.ctype()
    _check(lib().mmsb_op_spmm(ctypes.byref(c), int(transpose), _fptr(P), P.shape[1], alpha,
                              _fptr(Y)))
    return Y


def gram(A, B, alpha=1.0):
    """alpha A^T B for n x pa and n x pb FP32 panels (mmsb_op_gram), FP64."""
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    if A.shape[0] != B.shape[0]:
        raise ValueError("A and B need the same number of rows")
    S = np.zeros((A.shape[1], B.shape[1]), dtype=np.float64, order="F")
    _check(lib().mmsb_op_gram(_fptr(A), A.shape[0], A.shape[1], _fptr(B), B.shape[1], alpha,
                              S.ctypes.data_as(_D)))
    return S


def symeig(A):
    """Eigen-pairs (descending) of a symmetric positive semi-definite matrix."""
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    ev = np.zeros(n)
    V = np.zeros((n, n), order="F")
    _check(lib().mmsb_op_symeig(_dptr(A), n, _dptr(ev), _dptr(V)))
    return ev, V


def spmm_t_noalloc(d_row_ptr, d_col_idx, d_val, n_rows, n_cols, nnz, d_P, p, alpha, d_Y,
                   stream=0):
    """Y = alpha G^T P on caller-owned DEVICE buffers (integer addresses); the
    library allocates nothing (see include/mmsb.h).  Returns the status code."""
    return lib().mmsb_op_spmm_t_noalloc(d_row_ptr, d_col_idx, d_val or None, n_rows, n_cols, nnz,
                                        d_P, p, alpha, d_Y, stream or None)
