// Host orchestration of the pipeline on one stream: whitening chain,
// whitened data, tensor power method and unwhitening.  All arithmetic runs in
// this library's CUDA kernels; the host only sequences launches.
#include "pipeline.h"

#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "k_stpm.cuh"

using namespace mmsb;

mmsb_ctx::~mmsb_ctx() {
  if (s) cudaStreamSynchronize(s);
  if (s2) cudaStreamSynchronize(s2);
  for (auto& kv : ws) cudaFree(kv.second.first);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  for (auto& pr : spmm_pool) {
    if (pr.first) cudaEventDestroy(pr.first);
    if (pr.second) cudaEventDestroy(pr.second);
  }
  for (auto& pool : kpool)
    for (auto& pr : pool) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  if (fork_ev) cudaEventDestroy(fork_ev);
  if (join_ev) cudaEventDestroy(join_ev);
  if (s4) cudaStreamDestroy(s4);
  if (s3) cudaStreamDestroy(s3);
  if (s2) cudaStreamDestroy(s2);
  if (s) cudaStreamDestroy(s);
}

void* mmsb_ctx::buf(const std::string& name, size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  auto it = ws.find(name);
  if (it != ws.end() && it->second.second >= bytes) return it->second.first;
  if (it != ws.end()) {
    cudaStreamSynchronize(s);
    cudaFree(it->second.first);
    ws.erase(it);
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw MmsbError(e == cudaErrorMemoryAllocation ? MMSB_ERR_OUT_OF_MEMORY : MMSB_ERR_CUDA,
                    "cudaMalloc(" + name + ", " + std::to_string(bytes) + "): " +
                        cudaGetErrorString(e));
  }
  ws[name] = {p, bytes};
  return p;
}

void mmsb_ctx::free_graph() {
  for (int b = 0; b < MMSB_NUM_BLOCKS; ++b) {
    g[b] = DevCsr{};
    gt[b] = DevCsr{};
  }
  have_graph = have_white = have_y = have_phi = have_post = false;
}

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw MmsbError(MMSB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

namespace {

struct Timer {
  mmsb_ctx* c;
  int a, b;
  double* out;
  Timer(mmsb_ctx* ctx, int ia, int ib, double* o) : c(ctx), a(ia), b(ib), out(o) {
    ck(cudaEventRecord(c->ev[a], c->s), "event");
  }
  void stop() {
    ck(cudaEventRecord(c->ev[b], c->s), "event");
    ck(cudaEventSynchronize(c->ev[b]), "event sync");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]), "elapsed");
    *out = ms;
  }
};

void check_flags(mmsb_ctx* c, const char* stage) {
  unsigned f = 0;
  ck(cudaMemcpyAsync(&f, c->flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->s), "flags");
  ck(cudaStreamSynchronize(c->s), "sync");
  if (f & (kFlagNonFinite | kFlagCholeskyBreakdown)) {
    ck(cudaMemsetAsync(c->flags, 0, sizeof(unsigned), c->s), "flags");
    throw MmsbError(MMSB_ERR_NUMERICAL, std::string(stage) + ": non-finite values");
  }
  if (f & kFlagTimeout) {
    // cleared like the numerical flags: the waits that gave up have returned,
    // and the context stays usable for the next call
    ck(cudaMemsetAsync(c->flags, 0, sizeof(unsigned), c->s), "flags");
    throw MmsbError(MMSB_ERR_TIMEOUT, std::string(stage) + ": device wait timed out");
  }
}

// SpMM with timing bookkeeping (algorithmic bytes: CSR + one panel-row
// gather per nonzero + output)
void spmm(mmsb_ctx* c, const DevCsr& g, const float* P, int ld, float alpha, float* Y,
          cudaStream_t st = nullptr) {
  if (!st) st = c->s;
  const size_t slot = c->spmm_events.size();
  if (slot < c->spmm_pool.size()) {
    ck(cudaEventRecord(c->spmm_pool[slot].first, st), "event");
    ck(spmm_f32(g.rp, g.ci, g.val, g.n_rows, P, ld, alpha, Y, st, g.n_cols), "spmm");
    ck(cudaEventRecord(c->spmm_pool[slot].second, st), "event");
    c->spmm_events.push_back(slot);
  } else {
    ck(spmm_f32(g.rp, g.ci, g.val, g.n_rows, P, ld, alpha, Y, st, g.n_cols), "spmm");
  }
  c->stats.spmm_launches += 1;
  c->stats.spmm_bytes += 8.0 * (g.n_rows + 1) + 4.0 * g.nnz * (g.val ? 2 : 1) +
                         4.0 * g.nnz * ld + 4.0 * g.n_rows * ld;
}

struct Nys {
  float* U;     // n x ldk panel
  double* sig;  // k
};

}  // namespace

void check_device_flags(mmsb_ctx* c, const char* stage) { check_flags(c, stage); }

// Symmetric positive semi-definite eigen-decomposition (n <= 512), eigenvalues
// descending: FP32 one-sided Jacobi on the Cholesky factor (run to
// convergence), then three FP64 Ogita-Aishima refinement steps (quadratic
// convergence from a converged FP32 start: 1e-7 -> 1e-14 -> FP64 round-off,
// the third a margin).
void sym_eig_refined(mmsb_ctx* c, const std::string& tag, int n, const double* A, double* evals,
                     double* V, const double* factor, cudaStream_t stream, cudaStream_t aux) {
  cudaStream_t s = stream ? stream : c->s;
  double* R = c->tbuf<double>(tag + ".eR", (size_t)n * n);
  double* Y = c->tbuf<double>(tag + ".eY", (size_t)n * n);
  double* X = c->tbuf<double>(tag + ".eX", (size_t)n * n);
  double* X2 = c->tbuf<double>(tag + ".eX2", (size_t)n * n);
  double* G = c->tbuf<double>(tag + ".eG", (size_t)n * n);
  double* AX = c->tbuf<double>(tag + ".eAX", (size_t)n * n);
  double* S = c->tbuf<double>(tag + ".eS", (size_t)n * n);
  double* E = c->tbuf<double>(tag + ".eE", (size_t)n * n);
  double* lam = c->tbuf<double>(tag + ".elam", (size_t)n);
  float* work = c->tbuf<float>(tag + ".jw", (size_t)n * n);
  if (factor) {
    Y = const_cast<double*>(factor);  // A = Y Y^T given
  } else {
    ck(chol_upper_drop(n, A, n, R, 1e-300, c->flags, s), "eig chol");
    ck(transpose_f64(n, R, Y, s), "eig R^T");
  }
  ck(eig_from_factor(n, Y, lam, X, work, c->flags, s), "jacobi");
  double* dstate = c->tbuf<double>(tag + ".edelta", 4);  // delta + three maxima
  ck(cudaMemsetAsync(dstate, 0, 4 * sizeof(double), s), "delta");
  for (int step = 0; step < 3; ++step) {
    if (aux) {
      ck(cudaEventRecord(c->fork_ev, s), "fork");
      ck(cudaStreamWaitEvent(aux, c->fork_ev, 0), "fork wait");
    }
    ck(dgemm_small(true, false, n, n, n, 1.0, X, n, X, n, 0.0, G, n, aux ? aux : s), "X^T X");
    if (aux) ck(cudaEventRecord(c->join_ev, aux), "join");
    ck(dgemm_small(false, false, n, n, n, 1.0, A, n, X, n, 0.0, AX, n, s), "A X");
    ck(dgemm_small(true, false, n, n, n, 1.0, X, n, AX, n, 0.0, S, n, s), "X^T A X");
    if (aux) ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
    ck(oa_correction(n, A, G, S, E, lam, dstate, s), "oa");
    ck(cudaMemcpyAsync(X2, X, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, s), "copy");
    ck(dgemm_small(false, false, n, n, n, 1.0, X, n, E, n, 1.0, X2, n, s), "X + X E");
    std::swap(X, X2);
  }
  ck(sort_eigen(n, lam, X, evals, V, c->flags, s), "sort");
}

namespace {

// SVD_symNystrom_sparse (CPU/Spectral.cpp:169-223) of M = A B, where A is an
// n x m FP32 panel of full column rank and B an m x p FP64 matrix (B == nullptr:
// identity, m == p).  With A = Q_A R_A (CholQR2), orthogonalize_cols(M) equals
// Q_A * MGS(R_A B) because Q_A is an isometry, so the modified Gram-Schmidt and
// its drop rule run in FP64 on the small coordinate matrix P = R_A B:
//   Nystrom branch (n > 20k):  QQ = Q[0:p,:],  H = P QQ  (C = M QQ = Q_A H)
//   thin-SVD branch:           H = P
// The eigen-pairs (sigma^2, W) of H H^T give U = C V diag(1/sigma) = Q_A W
// = A R_A^{-1} W and sigma.  aux (optional, idle on entry): a second stream
// for R2^{-1} and Q_A[0:p] while the Gram-Schmidt of R_A B runs on s.
Nys svd_sym_nystrom(mmsb_ctx* c, const std::string& tag, const float* A, int lda, int m,
                    const double* B, int64_t n, cudaStream_t s, cudaStream_t aux = nullptr) {
  const int p = c->p, k = c->k, ldk = c->ldk;
  const double tol = c->cfg.pinv_tol;
  const int64_t cap = (int64_t)gram_tsk_partials(std::max<int64_t>(n, 1), m, m);
  double* part = c->tbuf<double>(tag + ".gram_part", (size_t)cap);
  double* S1 = c->tbuf<double>(tag + ".S1", (size_t)m * m);
  double* S2 = c->tbuf<double>(tag + ".S2", (size_t)m * m);
  double* R1 = c->tbuf<double>(tag + ".R1", (size_t)m * m);
  double* R2 = c->tbuf<double>(tag + ".R2", (size_t)m * m);
  double* RA = c->tbuf<double>(tag + ".RA", (size_t)m * m);
  double* T1 = c->tbuf<double>(tag + ".T1", (size_t)m * m);
  double* P = c->tbuf<double>(tag + ".P", (size_t)m * p);
  double* Hm = c->tbuf<double>(tag + ".H", (size_t)m * p);
  double* Zs = c->tbuf<double>(tag + ".Zs", (size_t)m * m);
  double* ev = c->tbuf<double>(tag + ".ev", (size_t)m);
  double* Wv = c->tbuf<double>(tag + ".W", (size_t)m * m);
  double* F = c->tbuf<double>(tag + ".F", (size_t)m * k);
  double* sig = c->tbuf<double>(tag + ".sig", (size_t)k);
  float* U = c->tbuf<float>(tag + ".U", (size_t)n * ldk);
  float* Q1 = c->tbuf<float>(tag + ".Q1", (size_t)n * round_up(m, 4));
  const int ldq = (int)round_up(m, 4);
  // CholQR2: A = Q_A R_A
  ck(gram_tsk(A, lda, m, A, lda, m, n, 1.0, S1, part, cap, s, c->flags, c->wait_limit), "gram1");
  ck(chol_upper_drop(m, S1, m, R1, 1e-300, c->flags, s), "chol1");
  ck(trinv_upper(m, R1, T1, s), "trinv1");
  ck(panel_times_small(A, lda, m, n, T1, m, m, Q1, ldq, s), "Q1");
  ck(gram_tsk(Q1, ldq, m, Q1, ldq, m, n, 1.0, S2, part, cap, s, c->flags, c->wait_limit), "gram2");
  // S2 = Q1^T Q1 is close to I: its factor needs no more than FP32 (Q1 itself is FP32)
  ck(chol_upper_drop_f32(m, S2, m, R2, c->flags, s), "chol2");
  // Q_A = Q1 R2^{-1} with R2 ~ I: products with Q_A use Q1 and T2 = R2^{-1}
  double* T2 = c->tbuf<double>(tag + ".T2", (size_t)m * m);
  const bool nystrom = n > (int64_t)c->cfg.nystrom_rows_factor * k;
  // QQ = Q[0:p, :] = Q_A[0:p, :] Q_small = Q1[0:p, :] R2^{-1} Q_small  (Spectral.cpp:185-188)
  double* Ap = nystrom ? c->tbuf<double>(tag + ".Ap", (size_t)p * m) : nullptr;
  double* QAp = nystrom ? c->tbuf<double>(tag + ".QAp", (size_t)p * m) : nullptr;
  cudaStream_t st2 = aux ? aux : s;
  if (aux) {
    ck(cudaEventRecord(c->fork_ev, s), "fork");
    ck(cudaStreamWaitEvent(aux, c->fork_ev, 0), "fork wait");
  }
  ck(trinv_upper(m, R2, T2, st2), "R2^-1");
  if (nystrom) {
    ck(panel_to_colmajor64(Q1, ldq, p, m, Ap, p, st2), "Q1[0:p]");
    ck(dgemm_small(false, false, p, m, m, 1.0, Ap, p, T2, m, 0.0, QAp, p, st2), "Q_A[0:p]");
  }
  if (aux) ck(cudaEventRecord(c->join_ev, aux), "join");
  ck(dgemm_small(false, false, m, m, m, 1.0, R2, m, R1, m, 0.0, RA, m, s), "R_A");
  // P = R_A B
  if (B)
    ck(dgemm_small(false, false, m, p, m, 1.0, RA, m, B, m, 0.0, P, m, s), "P");
  else
    ck(cudaMemcpyAsync(P, RA, sizeof(double) * m * p, cudaMemcpyDeviceToDevice, s), "P");
  if (nystrom) {
    double* Qs = c->tbuf<double>(tag + ".Qs", (size_t)m * p);
    double* QQ = c->tbuf<double>(tag + ".QQ", (size_t)p * p);
    if (B)
      ck(mgs_cols(m, p, P, m, Qs, m, tol, s), "mgs");
    else  // MGS of the upper-triangular R_A is the identity (zero where R_jj == 0)
      ck(eye_mask(m, p, P, m, Qs, m, s), "mgs(R)");
    if (aux) ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
    ck(dgemm_small(false, false, p, p, m, 1.0, QAp, p, Qs, m, 0.0, QQ, p, s), "QQ");
    ck(dgemm_small(false, false, m, p, p, 1.0, P, m, QQ, p, 0.0, Hm, m, s), "H");
  } else {
    ck(cudaMemcpyAsync(Hm, P, sizeof(double) * m * p, cudaMemcpyDeviceToDevice, s), "H");
    if (aux) ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
  }
  ck(dgemm_small(false, true, m, m, p, 1.0, Hm, m, Hm, m, 0.0, Zs, m, s), "H H^T");
  // Zs = H H^T.  The one-sided Jacobi runs on the Cholesky factor L of Zs
  // (L L^T = H H^T), not on H: L's columns are graded like the R factor of a
  // QR preconditioner, and the FP32 sweeps drop from ~13 to ~8 at p = 200,
  // more than paying for the FP64 Cholesky
  sym_eig_refined(c, tag, m, Zs, ev, Wv, nullptr, s, aux);
  // sigma = sqrt(ev_k); U = Q_A W_k diag(sigma > tol) = Q1 (R2^{-1} W_k) (masked)
  ck(sig_from_evals(k, ev, sig, s), "sig");
  ck(dgemm_small(false, false, m, k, m, 1.0, T2, m, Wv, m, 0.0, F, m, s), "F");
  ck(mask_cols(m, k, F, m, sig, tol, s), "mask");
  ck(panel_times_small(Q1, ldq, m, n, F, m, k, U, ldk, s), "U");
  return Nys{U, sig};
}

}  // namespace

// ---------------------------------------------------------------------------

void pipeline_upload(mmsb_ctx* c, const mmsb_csr* blocks) {
  const int rows_part[5] = {0, 0, 0, 2, 3};
  const int cols_part[5] = {1, 2, 3, 1, 1};
  int64_t part[4] = {-1, -1, -1, -1};
  for (int b = 0; b < MMSB_NUM_BLOCKS; ++b) {
    const mmsb_csr& m = blocks[b];
    if (m.n_rows < 0 || m.n_cols < 0 || m.nnz < 0 || (m.nnz > 0 && (!m.row_ptr || !m.col_idx)) ||
        (!m.row_ptr && m.n_rows > 0))
      throw MmsbError(MMSB_ERR_INVALID_ARG, "block " + std::to_string(b) + ": bad CSR");
    for (int side = 0; side < 2; ++side) {
      const int pp = side ? cols_part[b] : rows_part[b];
      const int64_t n = side ? m.n_cols : m.n_rows;
      if (part[pp] >= 0 && part[pp] != n)
        throw MmsbError(MMSB_ERR_INVALID_ARG, "inconsistent partition sizes across blocks");
      part[pp] = n;
    }
    if (m.n_rows > 0 && (m.row_ptr[0] != 0 || m.row_ptr[m.n_rows] != m.nnz))
      throw MmsbError(MMSB_ERR_INVALID_ARG, "block " + std::to_string(b) + ": row_ptr/nnz mismatch");
    if (m.n_cols > INT32_MAX) throw MmsbError(MMSB_ERR_INVALID_ARG, "too many columns");
  }
  c->free_graph();
  c->nX = part[0];
  c->nA = part[1];
  c->nB = part[2];
  c->nC = part[3];
  if (c->nX < 1 || c->nA < 1 || c->nB < 1 || c->nC < 1)
    throw MmsbError(MMSB_ERR_INVALID_ARG, "every partition needs at least one node");
  // copies, then the row-offset / column-index checks on the device (the
  // transposes and SpMMs index with these), before any kernel reads them
  unsigned* bad = c->tbuf<unsigned>("upload_checks", MMSB_NUM_BLOCKS);
  ck(cudaMemsetAsync(bad, 0, sizeof(unsigned) * MMSB_NUM_BLOCKS, c->s), "checks");
  for (int b = 0; b < MMSB_NUM_BLOCKS; ++b) {
    const mmsb_csr& m = blocks[b];
    DevCsr& d = c->g[b];
    const std::string t = "g" + std::to_string(b);
    d.n_rows = m.n_rows;
    d.n_cols = m.n_cols;
    d.nnz = m.nnz;
    d.rp = c->tbuf<int64_t>(t + ".rp", m.n_rows + 1);
    d.ci = c->tbuf<int32_t>(t + ".ci", m.nnz);
    d.val = m.val ? c->tbuf<float>(t + ".val", m.nnz) : nullptr;
    ck(cudaMemcpyAsync(d.rp, m.row_ptr, sizeof(int64_t) * (m.n_rows + 1), cudaMemcpyHostToDevice, c->s), "H2D rp");
    if (m.nnz) ck(cudaMemcpyAsync(d.ci, m.col_idx, sizeof(int32_t) * m.nnz, cudaMemcpyHostToDevice, c->s), "H2D ci");
    if (m.val) ck(cudaMemcpyAsync(d.val, m.val, sizeof(float) * m.nnz, cudaMemcpyHostToDevice, c->s), "H2D val");
    ck(csr_validate(d.rp, d.ci, d.n_rows, d.n_cols, d.nnz, bad + b, c->s), "checks");
  }
  unsigned hbad[MMSB_NUM_BLOCKS];
  ck(cudaMemcpyAsync(hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, c->s), "checks");
  ck(cudaStreamSynchronize(c->s), "checks");
  for (int b = 0; b < MMSB_NUM_BLOCKS; ++b) {
    if (!hbad[b]) continue;
    c->free_graph();
    throw MmsbError(MMSB_ERR_INVALID_ARG, "block " + std::to_string(b) +
                                              ((hbad[b] & 1u) ? ": decreasing row_ptr"
                                                              : ": column index out of range"));
  }
  for (int b = 0; b < MMSB_NUM_BLOCKS; ++b) {
    const mmsb_csr& m = blocks[b];
    DevCsr& d = c->g[b];
    const std::string t = "g" + std::to_string(b);
    DevCsr& e = c->gt[b];
    e.n_rows = m.n_cols;
    e.n_cols = m.n_rows;
    e.nnz = m.nnz;
    e.rp = c->tbuf<int64_t>(t + "t.rp", m.n_cols + 1);
    e.ci = c->tbuf<int32_t>(t + "t.ci", m.nnz);
    e.val = m.val ? c->tbuf<float>(t + "t.val", m.nnz) : nullptr;
    int32_t* scratch = c->tbuf<int32_t>("transpose_scratch", 2 * (m.n_cols + 1) + 2 * m.nnz + 2);
    ck(csr_transpose(d.rp, d.ci, d.val, d.n_rows, d.n_cols, d.nnz, e.rp, e.ci, e.val, scratch, c->s),
       "transpose");
  }
  ck(cudaStreamSynchronize(c->s), "upload sync");
  c->have_graph = true;
}

static void alloc_results(mmsb_ctx* c) {
  const int k = c->k, ldk = c->ldk;
  c->W = c->tbuf<float>("W", (size_t)c->nA * ldk);
  c->Zb1 = c->tbuf<float>("Zb1", (size_t)c->nA * ldk);
  c->Zc1 = c->tbuf<float>("Zc1", (size_t)c->nA * ldk);
  c->mu = c->tbuf<double>("mu", (size_t)(c->nA + c->nB + c->nC));
  for (int q = 0; q < 3; ++q) c->y[q] = c->tbuf<float>("y" + std::to_string(q), (size_t)c->nX * ldk);
  c->ymu = c->tbuf<float>("ymu", 3 * (size_t)k);
  c->ymu64 = c->tbuf<double>("ymu64", 3 * (size_t)k);
  c->phi = c->tbuf<float>("phi", (size_t)k * k);
  c->lambda = c->tbuf<double>("lambda", (size_t)k);
}

// whitened data and means from W, Zb1, Ub, Zc1, Uc (CommunityDetection.cpp:66-68)
void pipeline_ydata(mmsb_ctx* c) {
  const int k = c->k, ldk = c->ldk;
  cudaStream_t s = c->s;
  double* part = c->tbuf<double>("gram_part_y", gram_tsk_partials(std::max(c->nA, std::max(c->nB, c->nC)), k, k));
  const int64_t cap = (int64_t)gram_tsk_partials(std::max(c->nA, std::max(c->nB, c->nC)), k, k);
  double* ZW = c->tbuf<double>("ZW", (size_t)k * k);
  float* Wb = c->tbuf<float>("Wb_eff", (size_t)c->nB * ldk);
  float* Wc = c->tbuf<float>("Wc_eff", (size_t)c->nC * ldk);
  float* mu32 = c->tbuf<float>("mu32", (size_t)(c->nA + c->nB + c->nC) * 4);
  const double* mu_a = c->mu;
  const double* mu_b = c->mu + c->nA;
  const double* mu_c = c->mu + c->nA + c->nB;
  // Wb_eff = Ub (Zb1^T W), Wc_eff = Uc (Zc1^T W).  The C side (its own
  // Gram workspace) runs on the second stream beside the A and B sides.
  cudaStream_t s2 = c->s2;
  double* part2 = c->tbuf<double>("gram_part_y2", (size_t)cap);
  double* ZW2 = c->tbuf<double>("ZW2", (size_t)k * k);
  ck(cudaEventRecord(c->fork_ev, s), "fork");
  ck(cudaStreamWaitEvent(s2, c->fork_ev, 0), "fork wait");
  ck(gram_tsk(c->Zc1, ldk, k, c->W, ldk, k, c->nA, 1.0, ZW2, part2, cap, s2), "Zc1^T W");
  ck(panel_times_small(c->Uc, ldk, k, c->nC, ZW2, k, k, Wc, ldk, s2), "Wc");
  spmm(c, c->g[MMSB_BLOCK_XC], Wc, ldk, 1.f, c->y[2], s2);
  ck(cudaEventRecord(c->join_ev, s2), "join");
  ck(gram_tsk(c->Zb1, ldk, k, c->W, ldk, k, c->nA, 1.0, ZW, part, cap, s), "Zb1^T W");
  ck(panel_times_small(c->Ub, ldk, k, c->nB, ZW, k, k, Wb, ldk, s), "Wb");
  spmm(c, c->g[MMSB_BLOCK_XA], c->W, ldk, 1.f, c->y[0]);
  spmm(c, c->g[MMSB_BLOCK_XB], Wb, ldk, 1.f, c->y[1]);
  ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
  // whitened means: W_P^T mu_P (mu as an n x 1 panel, ld 4)
  ck(colmajor64_to_panel(mu_a, c->nA, 1, c->nA, mu32, 4, s), "mu32a");
  ck(gram_tsk(c->W, ldk, k, mu32, 4, 1, c->nA, 1.0, c->ymu64, part, cap, s), "ymu_a");
  ck(colmajor64_to_panel(mu_b, c->nB, 1, c->nB, mu32, 4, s), "mu32b");
  ck(gram_tsk(Wb, ldk, k, mu32, 4, 1, c->nB, 1.0, c->ymu64 + k, part, cap, s), "ymu_b");
  ck(colmajor64_to_panel(mu_c, c->nC, 1, c->nC, mu32, 4, s), "mu32c");
  ck(gram_tsk(Wc, ldk, k, mu32, 4, 1, c->nC, 1.0, c->ymu64 + 2 * k, part, cap, s), "ymu_c");
  ck(f64_to_f32(c->ymu64, c->ymu, 3 * k, s), "ymu32");
  c->have_y = true;
}

// sums the device time of the SpMM launches recorded since the last call
void collect_spmm_time(mmsb_ctx* c) {
  double ms = 0.0;
  for (size_t slot : c->spmm_events) {
    ck(cudaEventSynchronize(c->spmm_pool[slot].second), "event sync");
    float t = 0.f;
    ck(cudaEventElapsedTime(&t, c->spmm_pool[slot].first, c->spmm_pool[slot].second), "elapsed");
    ms += t;
  }
  c->stats.spmm_ms += ms;
  c->spmm_events.clear();
}

void pipeline_whiten(mmsb_ctx* c, const double* const* sketches, bool finish) {
  if (!c->have_graph) throw MmsbError(MMSB_ERR_STATE, "whiten before upload_graph");
  c->spmm_events.clear();
  const int k = c->k, p = c->p, ldp = c->ldp, ldk = c->ldk;
  cudaStream_t s = c->s;
  alloc_results(c);
  const double inv = c->cfg.normalize ? 1.0 / (double)c->nX : 1.0;
  const double tol = c->cfg.pinv_tol;
  const DevCsr &XB = c->g[1], &XC = c->g[2];
  const DevCsr &XAt = c->gt[0], &XBt = c->gt[1], &XCt = c->gt[2];
  const int64_t nmax = std::max(std::max(c->nX, c->nA), std::max(c->nB, c->nC));
  float* R[3];
  const int64_t rn[3] = {c->nB, c->nC, c->nA};
  const bool upload = sketches && (sketches[0] || sketches[1] || sketches[2]);
  // generated sketches: R[0] here and R[1] on the second stream as each side
  // starts, R[2] and the means after side zc (the W step is their first
  // reader); uploaded ones share one staging buffer, so all come first
  for (int q = 0; q < 3; ++q) R[q] = c->tbuf<float>("R" + std::to_string(q), (size_t)rn[q] * ldp);
  auto make_sketch = [&](int q, cudaStream_t st) {
    if (sketches && sketches[q]) {
      double* tmp = c->tbuf<double>("sketch_upload", (size_t)rn[q] * p);
      ck(cudaMemcpyAsync(tmp, sketches[q], sizeof(double) * rn[q] * p, cudaMemcpyHostToDevice, st), "H2D sketch");
      ck(colmajor64_to_panel(tmp, rn[q], p, rn[q], R[q], ldp, st), "sketch panel");
    } else {
      ck(gaussian_panel(R[q], rn[q], p, ldp, c->cfg.seed, 11 + q, st), "gaussian");
    }
  };
  // partition means (Util.cpp:48-51): column sums of G_XP = row sums of G_XP^T
  auto means = [&]() {
    ck(row_sums_f64(XAt.rp, XAt.val, c->nA, inv, c->mu, s), "mu_a");
    ck(row_sums_f64(XBt.rp, XBt.val, c->nB, inv, c->mu + c->nA, s), "mu_b");
    ck(row_sums_f64(XCt.rp, XCt.val, c->nC, inv, c->mu + c->nA + c->nB, s), "mu_c");
  };
  if (upload) {
    for (int q = 0; q < 3; ++q) make_sketch(q, s);
    means();
  }

  double* Linv_c = c->tbuf<double>("Linv_c", (size_t)k);
  double* Linv_b = c->tbuf<double>("Linv_b", (size_t)k);
  c->Ub = c->tbuf<float>("Ub", (size_t)c->nB * ldk);
  c->Uc = c->tbuf<float>("Uc", (size_t)c->nC * ldk);
  float* Vc = c->tbuf<float>("Vc", (size_t)c->nB * ldk);
  float* Vb = c->tbuf<float>("Vb", (size_t)c->nC * ldk);

  // pinv_Nystrom_sparse_component (Spectral.cpp:296-315) of
  //   Zc_den = inv Gx_c^T Gx_b (n_C x n_B), sketch R_c (n_B x 2k)
  //   Zb_den = inv Gx_b^T Gx_c (n_B x n_C), sketch R_b (n_C x 2k)
  // The two sides are independent: each runs on its own stream with its own
  // workspace (their small latency-bound factorisations overlap).
  struct Side {
    const DevCsr *Gin, *Gout_t, *Gout, *Gin_t;
    int64_t n_in, n_out;
    float* Rk;
    float* V;
    float* U;
    double* Linv;
    const char* tag;
    cudaStream_t st, aux;  // aux: the side's helper stream in its Nystrom step
  } sides[2] = {
      {&XB, &XCt, &XC, &XBt, c->nB, c->nC, R[0], Vc, c->Uc, Linv_c, "zc", s, c->s3},
      {&XC, &XBt, &XB, &XCt, c->nC, c->nB, R[1], Vb, c->Ub, Linv_b, "zb", c->s2, c->s4},
  };
  ck(cudaEventRecord(c->fork_ev, s), "fork");
  ck(cudaStreamWaitEvent(c->s2, c->fork_ev, 0), "fork wait");
  if (!upload) {
    make_sketch(0, s);
    make_sketch(1, c->s2);
  }
  for (auto& sd : sides) {
    const std::string t = sd.tag;
    cudaStream_t st = sd.st;
    float* T1 = c->tbuf<float>(t + ".T1", (size_t)c->nX * ldp);
    float* XR = c->tbuf<float>(t + ".XR", (size_t)sd.n_out * ldp);
    float* Gram = c->tbuf<float>(t + ".Gram", (size_t)sd.n_in * ldp);
    float* T3 = c->tbuf<float>(t + ".T3", (size_t)c->nX * ldk);
    float* VL = c->tbuf<float>(t + ".VL", (size_t)sd.n_in * ldk);
    double* Linv_sqrt = c->tbuf<double>(t + ".Linv_sqrt", (size_t)k);
    // X = inv Gout^T Gin  (n_out x n_in):  XR = X R ; Gram = X^T XR
    spmm(c, *sd.Gin, sd.Rk, ldp, 1.f, T1, st);                  // Gin R       (n_X x p)
    spmm(c, *sd.Gout_t, T1, ldp, (float)inv, XR, st);           // X R         (n_out x p)
    spmm(c, *sd.Gout, XR, ldp, 1.f, T1, st);                    // Gout XR     (n_X x p)
    spmm(c, *sd.Gin_t, T1, ldp, (float)inv, Gram, st);          // X^T X R     (n_in x p)
    Nys ny = svd_sym_nystrom(c, sd.tag, Gram, ldp, p, nullptr, sd.n_in, st, sd.aux);  // V, sigma
    ck(cudaMemcpyAsync(sd.V, ny.U, sizeof(float) * sd.n_in * ldk, cudaMemcpyDeviceToDevice, st), "V");
    // U = X V diag(sqrt(pinv(sigma)));  Linv = pinv(sqrt(sigma))  (Spectral.cpp:235-244, 307)
    ck(sqrt_pinv(k, ny.sig, tol, Linv_sqrt, sd.Linv, st), "Linv");
    ck(cudaMemcpyAsync(VL, sd.V, sizeof(float) * sd.n_in * ldk, cudaMemcpyDeviceToDevice, st), "VL");
    ck(panel_scale_cols(VL, ldk, sd.n_in, k, Linv_sqrt, st), "VL scale");
    spmm(c, *sd.Gin, VL, ldk, 1.f, T3, st);
    spmm(c, *sd.Gout_t, T3, ldk, (float)inv, sd.U, st);
  }
  if (!upload) {  // after side zc on this stream
    make_sketch(2, s);
    means();
  }
  ck(cudaEventRecord(c->join_ev, c->s2), "join");
  ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
  float* T3 = c->tbuf<float>("zc.T3", (size_t)c->nX * ldk);
  float* VL = c->tbuf<float>("VL", (size_t)nmax * ldk);
  double* Linv_sqrt = c->tbuf<double>("Linv_sqrt", (size_t)k);
  float* T4 = c->tbuf<float>("T4", (size_t)c->nX * ldk);
  double* core = c->tbuf<double>("core", (size_t)k * k);
  const int64_t cap = (int64_t)gram_tsk_partials(nmax, std::max(k, p), p);
  double* part = c->tbuf<double>("gram_part_w", (size_t)cap);
  const int m2 = k + 1, ldm2 = (int)round_up(m2, 4);
  double* Q1 = c->tbuf<double>("ZbR", (size_t)k * p);
  double* ma = c->tbuf<double>("muR", (size_t)p);
  double* Bm = c->tbuf<double>("M2B", (size_t)m2 * p);
  float* mu32 = c->tbuf<float>("mu32", (size_t)(c->nA + c->nB + c->nC) * 4);
  float* Am = c->tbuf<float>("M2A", (size_t)c->nA * ldm2);
  {
    // the B side (Z_B_part1 and its sketch products) on the second stream,
    // with the side's own panels and Gram workspace, beside the C side and
    // the core on this one
    cudaStream_t s2 = c->s2;
    float* T3b = c->tbuf<float>("zb.T3", (size_t)c->nX * ldk);
    float* VLb = c->tbuf<float>("zb.VL", (size_t)c->nC * ldk);
    double* part2 = c->tbuf<double>("gram_part_w2", (size_t)cap);
    ck(cudaEventRecord(c->fork_ev, s), "fork");
    ck(cudaStreamWaitEvent(s2, c->fork_ev, 0), "fork wait");
    // Z_B_part1 = Zb_num V_b diag(Linv_b), Zb_num = inv Gx_a^T Gx_c (Util.cpp:96-97)
    ck(cudaMemcpyAsync(VLb, Vb, sizeof(float) * c->nC * ldk, cudaMemcpyDeviceToDevice, s2), "VL");
    ck(panel_scale_cols(VLb, ldk, c->nC, k, Linv_b, s2), "Vb scale");
    spmm(c, XC, VLb, ldk, 1.f, T3b, s2);
    spmm(c, XAt, T3b, ldk, (float)inv, c->Zb1, s2);
    ck(gram_tsk(c->Zb1, ldk, k, R[2], ldp, p, c->nA, 1.0, Q1, part2, cap, s2), "Zb1^T R");
    ck(colmajor64_to_panel(c->mu, c->nA, 1, c->nA, mu32, 4, s2), "mu32");
    ck(gram_tsk(mu32, 4, 1, R[2], ldp, p, c->nA, 1.0, ma, part2, cap, s2), "mu^T R");
    ck(cudaEventRecord(c->join_ev, s2), "join");
  }
  // Z_C_part1 = Zc_num V_c diag(Linv_c), Zc_num = inv Gx_a^T Gx_b (Util.cpp:83-84)
  ck(cudaMemcpyAsync(VL, Vc, sizeof(float) * c->nB * ldk, cudaMemcpyDeviceToDevice, s), "VL");
  ck(panel_scale_cols(VL, ldk, c->nB, k, Linv_c, s), "Vc scale");
  spmm(c, XB, VL, ldk, 1.f, T3);
  spmm(c, XAt, T3, ldk, (float)inv, c->Zc1);
  // core = U_c^T Zc_den U_b = inv (Gx_c U_c)^T (Gx_b U_b)  (Util.cpp:90-94)
  spmm(c, XC, c->Uc, ldk, 1.f, T3);
  spmm(c, XB, c->Ub, ldk, 1.f, T4);
  ck(gram_tsk(T3, ldk, k, T4, ldk, k, c->nX, inv, core, part, cap, s), "core");
  ck(diag_guard(k, core, s), "core guard");
  ck(cudaStreamWaitEvent(s, c->join_ev, 0), "join wait");
  // M2 sketch = (a0+1) Zc1 core (Zb1^T R_a) - a0 mu_a (mu_a^T R_a)  (Util.cpp:103-113),
  // kept factored as M2 = [Zc1 | mu_a] B with B = [(a0+1) core Zb1^T R_a ; -a0 mu_a^T R_a]
  // (rank <= k+1, so its Gram-Schmidt must see FP64 round-off, not FP32)
  ck(dgemm_small(false, false, k, p, k, c->cfg.alpha0 + 1.0, core, k, Q1, k, 0.0, Bm, m2, s), "B");
  ck(set_row_scaled(m2, p, Bm, m2, k, -c->cfg.alpha0, ma, s), "B shift row");
  ck(panel_copy(c->Zc1, ldk, c->nA, k, Am, ldm2, s), "A_M");
  ck(panel_set_col(Am, ldm2, c->nA, k, c->mu, s), "A_M mu");
  // W = U_w diag(pinv(sqrt(sigma_w)))  (Util.cpp:116-123)
  Nys nw = svd_sym_nystrom(c, "w", Am, ldm2, m2, Bm, c->nA, s, c->s2);
  ck(sqrt_pinv(k, nw.sig, tol, nullptr, Linv_sqrt, s), "Lw");
  ck(cudaMemcpyAsync(c->W, nw.U, sizeof(float) * c->nA * ldk, cudaMemcpyDeviceToDevice, s), "W");
  ck(panel_scale_cols(c->W, ldk, c->nA, k, Linv_sqrt, s), "W scale");
  c->have_white = true;
  pipeline_ydata(c);
  if (finish) pipeline_whiten_finish(c);
}

void pipeline_whiten_finish(mmsb_ctx* c) {
  check_flags(c, "whitening");
  collect_spmm_time(c);
}

// ---------------------------------------------------------------------------

struct PartialOut {
  float* gpart;
  int grid;
  int64_t stride;
};

// event pair around one STPM kernel launch (which: 0 contraction, 1 step);
// summed by collect_kernel_times after the STPM loop
template <typename F>
static void timed_launch(mmsb_ctx* c, int which, F&& launch) {
  ++c->klaunched[which];
  if (!c->ksample) {
    // untimed: nothing between this launch and its neighbours, so that the
    // STPM kernels' programmatic serialization can overlap them
    launch();
    return;
  }
  auto& pool = c->kpool[which];
  if (c->kused[which] == pool.size()) {
    std::pair<cudaEvent_t, cudaEvent_t> pr{};
    ck(cudaEventCreate(&pr.first), "event");
    ck(cudaEventCreate(&pr.second), "event");
    pool.push_back(pr);
  }
  auto& pr = pool[c->kused[which]++];
  ck(cudaEventRecord(pr.first, c->s), "event");
  launch();
  ck(cudaEventRecord(pr.second, c->s), "event");
}

static void collect_kernel_times(mmsb_ctx* c) {
  double* out[2] = {&c->stats.contract_ms, &c->stats.step_ms};
  int64_t* cnt[2] = {&c->stats.contract_launches, &c->stats.step_launches};
  for (int w = 0; w < 2; ++w) {
    double ms = 0.0;
    for (size_t i = 0; i < c->kused[w]; ++i) {
      ck(cudaEventSynchronize(c->kpool[w][i].second), "event sync");
      float t = 0.f;
      ck(cudaEventElapsedTime(&t, c->kpool[w][i].first, c->kpool[w][i].second), "elapsed");
      ms += t;
    }
    // timed launches are a sample of all (every 8th minibatch step): scale
    // their mean to every launch
    if (c->kused[w] > 0) ms *= (double)c->klaunched[w] / (double)c->kused[w];
    *out[w] += ms;
    *cnt[w] += c->klaunched[w];
    c->kused[w] = 0;
    c->klaunched[w] = 0;
  }
  c->ksample = true;
}

StpmPartialArgs stpm_partial_args(mmsb_ctx* c, int q1, int q2, int q3, int64_t begin,
                                  int64_t count, double c0, double c2, bool bf16, float* gpart,
                                  int64_t stride, int nblocks) {
  const int k = c->k;
  StpmPartialArgs a{};
  a.y1 = c->y[q1];
  a.y2 = c->y[q2];
  a.y3 = c->y[q3];
  a.ldy = c->ldk;
  if (bf16) {
    a.yh1 = c->yh[q1];
    a.yh2 = c->yh[q2];
    a.yh3 = c->yh[q3];
    a.ldyh = c->ldkh;
  }
  a.phi = c->phi;
  a.mu1 = c->ymu + q1 * k;
  a.mu2 = c->ymu + q2 * k;
  a.mu3 = c->ymu + q3 * k;
  a.begin = begin;
  a.count = count;
  a.k = k;
  a.c0 = (float)c0;
  a.c2 = (float)c2;
  a.gpart = gpart;
  a.part_stride = stride;
  a.nblocks = nblocks;
  a.flags = c->flags;
  a.wait_limit = c->wait_limit;
  return a;
}

// per-CTA partial contractions over nodes [begin, begin+count)
static PartialOut stpm_partials(mmsb_ctx* c, int mode, int q1, int q2, int q3, int64_t begin,
                                int64_t count, double c0, double c2, bool bf16 = false,
                                const void* phi_img = nullptr) {
  const int k = c->k;
  const int grid = stpm_partial_grid(count, bf16);
  const int64_t stride = (int64_t)k * k + 3 * k + 4;
  float* gpart = c->tbuf<float>("gpart", (size_t)grid * stride);
  StpmPartialArgs a = stpm_partial_args(c, q1, q2, q3, begin, count, c0, c2, bf16, gpart, stride, grid);
  a.phi_img = phi_img;
  timed_launch(c, 0, [&]() { ck(stpm_partial(mode, a, grid, bf16, c->s), "stpm_partial"); });
  const int products = mode == kModePlain ? 3 : mode == kModeAdjoint ? 6 : 3;
  c->stats.contract_flops += 2.0 * k * k * (double)count * products;
  return PartialOut{gpart, grid / stpm_partial_cluster(), stride};
}

static void stpm_pass(mmsb_ctx* c, int mode, int q1, int q2, int q3, int64_t begin, int64_t count,
                      double c0, double c1, double c2, double scale, float* G, double* loss) {
  const int k = c->k;
  PartialOut po = stpm_partials(c, mode, q1, q2, q3, begin, count, c0, c2);
  StpmReduceArgs r{};
  r.mode = mode;
  r.k = k;
  r.gpart = po.gpart;
  r.part_stride = po.stride;
  r.nparts = po.grid;
  r.phi = c->phi;
  r.mu1 = c->ymu + q1 * k;
  r.mu2 = c->ymu + q2 * k;
  r.mu3 = c->ymu + q3 * k;
  r.mu_out = r.mu3;
  r.c1 = c1;
  r.c2 = c2;
  r.scale = scale;
  r.count = (double)count;
  r.G = G;
  r.loss_out = loss;
  ck(stpm_reduce(r, c->s), "stpm_reduce");
}

static StpmUpdateArgs step_args(mmsb_ctx* c, int step_mode, bool counted) {
  StpmUpdateArgs u{};
  u.k = c->k;
  u.step_mode = step_mode;
  u.phi = c->phi;
  u.theta3 = (float)(3.0 * c->cfg.theta);
  u.max_passes = 4;
  u.flags = c->flags;
  if (counted) {
    u.orth_passes = c->tbuf<int>("orth_passes", 4);
    u.orth_err = c->tbuf<float>("orth_err", 4);
  }
  const int kp = stpm_step_kp(c->k);
  if (kp > 128) u.xstash = c->tbuf<float>("xstash", (size_t)kp * kp);
  u.wait_limit = c->wait_limit;
  u.active = 1;
  return u;
}

// Q of the QR factorisation of Phi (diag(R) > 0), in place
static void qr_only(mmsb_ctx* c) {
  StpmUpdateArgs u = step_args(c, kStepQR, false);
  ck(stpm_update(u, c->s), "stpm_qr");
}

void* stpm_phi_image(mmsb_ctx* c) {
  const size_t bytes = stpm_phi_image_bytes(c->k);
  return bytes ? c->buf("phi_img", bytes) : nullptr;
}

StpmUpdateArgs stpm_online_update_args(mmsb_ctx* c, const OnlineRound& rd, float* gpart,
                                       int64_t stride, int nparts) {
  const int k = c->k;
  StpmUpdateArgs u = step_args(c, kStepOnline, true);
  u.mode = rd.mode;
  u.gpart = gpart;
  u.part_stride = stride;
  u.nparts = nparts;
  u.mu1 = c->ymu;
  u.mu2 = c->ymu + k;
  u.mu3 = c->ymu + 2 * k;
  u.c1 = rd.c1;
  u.c2 = rd.c2;
  u.scale = rd.scale;
  u.count = (double)rd.cnt;
  u.beta = (float)rd.beta;
  u.gscale = (float)rd.gscale;
  u.phi_general = rd.r == 0 ? 1 : 0;
  u.phi_img = stpm_phi_image(c);
  return u;
}

// minibatch schedule of the online / adjoint methods: update r of
// sweeps x ceil(n_X / b) covers nodes [x0, x0 + cnt) of sweep r / steps with
// beta_r = lr0 / (1 + r); the BF16 form's last sweep is FP32
bool stpm_online_round(const mmsb_ctx* c, int64_t r, OnlineRound* out) {
  const int64_t nx = c->nX;
  const int64_t b = std::max<int64_t>(1, std::min<int64_t>(c->cfg.minibatch, nx));
  const int64_t per = (nx + b - 1) / b;
  if (r < 0 || r >= per * c->cfg.sweeps) return false;
  const double a0 = c->cfg.alpha0;
  const double p0 = (a0 + 1.0) * (a0 + 2.0) / 2.0, p1 = a0 * a0, p2 = -a0 * (a0 + 1.0) / 2.0;
  const int64_t sw = r / per;
  out->r = r;
  out->x0 = (r % per) * b;
  out->cnt = std::min<int64_t>(b, nx - out->x0);
  out->beta = c->cfg.lr0 / (1.0 + (double)r);
  out->bf16 = c->cfg.precision == MMSB_PREC_BF16 && sw + 1 < c->cfg.sweeps;
  if (c->cfg.stpm_method == MMSB_STPM_ADJOINT) {
    // dT (column i = d That_i / d phi_i); step = 3 theta O - dT
    out->mode = kModeAdjoint;
    out->c0 = p0;
    out->c1 = p1;
    out->c2 = p2;
    out->scale = 1.0 / (double)out->cnt;
    out->gscale = 1.0;
  } else {
    // G = mean of The_second_term; step = 3 theta O - 3 G
    out->mode = kModePlain;
    out->c0 = p0 / (double)out->cnt;
    out->c1 = p1;
    out->c2 = p2 / (double)out->cnt;
    out->scale = 1.0;
    out->gscale = 3.0;
  }
  return true;
}

int64_t stpm_online_rounds(const mmsb_ctx* c) {
  const int64_t nx = c->nX;
  const int64_t b = std::max<int64_t>(1, std::min<int64_t>(c->cfg.minibatch, nx));
  return ((nx + b - 1) / b) * c->cfg.sweeps;
}

// one minibatch update: partial contractions, then the fused reduction +
// Phi - beta (3 theta O - gscale G) + QR re-orthonormalisation on one cluster
static void stpm_step(mmsb_ctx* c, const OnlineRound& rd, bool timed = true,
                      float* trace_snap = nullptr, double* trace_out = nullptr) {
  c->ksample = timed;
  // the previous step of the run wrote Phi's operand image for the
  // tensor-core contraction of the plain FP32 form
  void* img = stpm_phi_image(c);
  const bool use_img = img && rd.r > 0 && rd.mode == kModePlain && !rd.bf16;
  PartialOut po = stpm_partials(c, rd.mode, 0, 1, 2, rd.x0, rd.cnt, rd.c0, rd.c2, rd.bf16,
                                use_img ? img : nullptr);
  StpmUpdateArgs u = stpm_online_update_args(c, rd, po.gpart, po.stride, po.grid);
  u.trace_snap = trace_snap;
  u.trace_out = trace_out;
  timed_launch(c, 1, [&]() { ck(stpm_update(u, c->s), "stpm_step"); });
}

// Phi0 (host FP64, or the Q factor of a seeded Gaussian matrix), counters
// and, for the BF16 form, the BF16 copies of y
void stpm_prepare(mmsb_ctx* c, const double* phi0) {
  if (!c->have_y) throw MmsbError(MMSB_ERR_STATE, "stpm before whitening");
  const int k = c->k;
  if (stpm_kp(k) < 0) throw MmsbError(MMSB_ERR_UNSUPPORTED, "STPM kernels support k <= 208");
  cudaStream_t s = c->s;
  ck(cudaMemsetAsync(c->tbuf<int>("orth_passes", 4), 0, sizeof(int), s), "orth counter");
  ck(cudaMemsetAsync(c->tbuf<float>("orth_err", 4), 0, sizeof(float), s), "orth error");
  if (phi0) {
    double* tmp = c->tbuf<double>("phi64", (size_t)k * k);
    ck(cudaMemcpyAsync(tmp, phi0, sizeof(double) * k * k, cudaMemcpyHostToDevice, s), "H2D phi0");
    ck(f64_to_f32(tmp, c->phi, (int64_t)k * k, s), "phi0");
  } else {
    // orthonormal start: Q of a seeded Gaussian matrix, as the GPU tree's
    // random start (GPU/stpm.c:1041-1064)
    ck(gaussian_panel(c->phi, k, k, k, c->cfg.seed, 7, s), "phi0");
    qr_only(c);  // (not counted: the statistics cover the minibatch steps)
  }
  c->stats.stpm_steps = 0;
  c->stats.contract_ms = c->stats.step_ms = c->stats.contract_flops = c->stats.step_flops = 0.0;
  c->stats.contract_launches = c->stats.step_launches = 0;
  c->kused[0] = c->kused[1] = 0;
  if (c->cfg.stpm_method != MMSB_STPM_BATCH_POWER && c->cfg.precision == MMSB_PREC_BF16) {
    const int64_t nx = c->nX;
    c->ldkh = (int)round_up(k, 8);
    for (int q = 0; q < 3; ++q) {
      c->yh[q] = c->buf("yh" + std::to_string(q), sizeof(uint16_t) * (size_t)nx * c->ldkh);
      ck(panel_to_bf16(c->y[q], c->ldk, nx, k, c->yh[q], c->ldkh, s), "y bf16");
    }
  }
}

// The final orthonormalisation of the BF16 form in FP64: two Cholesky QR
// passes on the k x k Phi (FP64 Gram, Cholesky, triangular inverse and
// products), the same Q as the per-step QR (diag(R) > 0).  Returns the FP64
// Phi (device) and leaves its FP32 rounding in c->phi.
static double* final_qr_f64(mmsb_ctx* c) {
  const int k = c->k;
  cudaStream_t s = c->s;
  double* Pa = c->tbuf<double>("fq.Pa", (size_t)k * k);
  double* Pb = c->tbuf<double>("fq.Pb", (size_t)k * k);
  double* S = c->tbuf<double>("fq.S", (size_t)k * k);
  double* R = c->tbuf<double>("fq.R", (size_t)k * k);
  double* T = c->tbuf<double>("fq.T", (size_t)k * k);
  ck(f32_to_f64(c->phi, Pa, (int64_t)k * k, s), "phi64");
  for (int pass = 0; pass < 2; ++pass) {
    ck(dgemm_small(true, false, k, k, k, 1.0, Pa, k, Pa, k, 0.0, S, k, s), "Phi^T Phi");
    ck(chol_upper_drop(k, S, k, R, 1e-300, c->flags, s), "chol");
    ck(trinv_upper(k, R, T, s), "R^-1");
    ck(dgemm_small(false, false, k, k, k, 1.0, Pa, k, T, k, 0.0, Pb, k, s), "Phi R^-1");
    std::swap(Pa, Pb);
  }
  ck(f64_to_f32(Pa, c->phi, (int64_t)k * k, s), "phi32");
  return Pa;
}

// lambda_i = That(phi_i, phi_i, phi_i) over all of X, sign fixed so lambda > 0
// (queued on the context's stream).  The BF16 form first re-orthonormalises
// Phi in FP64 and takes the final dot products phi_i . T(I, phi_i, phi_i)
// with the FP64 Phi.
void stpm_lambda_pass(mmsb_ctx* c) {
  const int k = c->k;
  const int64_t nx = c->nX;
  const double a0 = c->cfg.alpha0;
  const double p0 = (a0 + 1.0) * (a0 + 2.0) / 2.0, p1 = a0 * a0, p2 = -a0 * (a0 + 1.0) / 2.0;
  double* phi64 = nullptr;
  if (c->cfg.precision == MMSB_PREC_BF16 && c->cfg.stpm_method != MMSB_STPM_BATCH_POWER)
    phi64 = final_qr_f64(c);
  float* G = c->tbuf<float>("G", (size_t)k * k);
  stpm_pass(c, kModePlain, 0, 1, 2, 0, nx, p0 / nx, p1, p2 / nx, 1.0, G, nullptr);
  ck(stpm_tensor_values(k, c->phi, G, c->lambda, c->s, phi64), "lambda");
}

// statistics and device flags of an online / adjoint run (waits for the stream)
void stpm_online_stats(mmsb_ctx* c, int64_t steps) {
  const int k = c->k;
  c->stats.stpm_steps = steps;
  c->stats.node_updates = c->nX * c->cfg.sweeps;
  int passes = 0;
  float oerr = 0.f;
  ck(cudaMemcpyAsync(&passes, c->tbuf<int>("orth_passes", 4), sizeof(int), cudaMemcpyDeviceToHost,
                     c->s), "orth counter");
  ck(cudaMemcpyAsync(&oerr, c->tbuf<float>("orth_err", 4), sizeof(float), cudaMemcpyDeviceToHost,
                     c->s), "orth error");
  ck(cudaStreamSynchronize(c->s), "sync");
  c->stats.orth_passes = passes;
  c->stats.orth_err_max = oerr;
  // per online update 4 k^3 (the Gram Phi^T Phi and the product with its
  // square) and 3 k^3 for the first-order pass (Gram, triangular product);
  // per exact Cholesky QR pass 2 k^3 (Gram) + k^3 (triangular product) +
  // k^3 / 3 (Cholesky) + k^3 / 3 (triangular inverse)
  const double kkk = (double)k * k * k;
  c->stats.step_flops = kkk * (7.0 * (double)steps + 11.0 / 3.0 * (double)passes);
  check_flags(c, "stpm");
  collect_kernel_times(c);
  c->have_phi = true;
}

void stpm_finish_online(mmsb_ctx* c, int64_t steps) {
  stpm_lambda_pass(c);
  stpm_online_stats(c, steps);
}

void pipeline_stpm(mmsb_ctx* c, const double* phi0) {
  stpm_prepare(c, phi0);
  const int k = c->k;
  cudaStream_t s = c->s;
  const int64_t nx = c->nX;
  if (c->cfg.stpm_method == MMSB_STPM_BATCH_POWER) {
    // tensorDecom_alpha0 (Util.cpp:131-184)
    const double a0 = c->cfg.alpha0;
    const double p0 = (a0 + 1.0) * (a0 + 2.0) / 2.0, p1 = a0 * a0, p2 = -a0 * (a0 + 1.0) / 2.0;
    const double inv_x = 1.0 / (double)nx;
    const double p_main = p0 * inv_x, p_s1 = p2 * inv_x, p_s0 = p1;
    float* G = c->tbuf<float>("G", (size_t)k * k);
    double err = 0.0;
    // ||Phi - Phi_old||_F of every iteration (the GPU tree's frob_norm file,
    // GPU/stpm.c:743), up to its buffer size
    constexpr int64_t kConvCap = 100000;
    c->conv = c->tbuf<double>("conv", kConvCap);
    c->conv_count = 0;
    for (int64_t it = 1;; ++it) {
      if (c->stop.load()) throw MmsbError(MMSB_ERR_STOPPED, "stop requested");
      stpm_pass(c, kModePlain, 1, 2, 0, 0, nx, p_main, p_s0, p_s1, 1.0, G, nullptr);
      ck(stpm_batch_update(k, c->phi, G, c->lambda, c->dscalar, s), "batch update");
      if (c->conv_count < kConvCap)
        ck(cudaMemcpyAsync(c->conv + c->conv_count++, c->dscalar, sizeof(double),
                           cudaMemcpyDeviceToDevice, s), "trace");
      c->stats.stpm_steps = it;
      if (it >= c->cfg.min_iter) {
        ck(cudaMemcpyAsync(&err, c->dscalar, sizeof(double), cudaMemcpyDeviceToHost, s), "err");
        ck(cudaStreamSynchronize(s), "sync");
        if (err < c->cfg.tol || it > c->cfg.max_iter) break;
      }
    }
    c->stats.stpm_last_error = err;
    c->stats.node_updates = nx * c->stats.stpm_steps;
    check_flags(c, "stpm");
    collect_kernel_times(c);
    c->have_phi = true;
    return;
  }
  const int64_t rounds = stpm_online_rounds(c);
  const int64_t per = std::max<int64_t>(1, rounds / std::max(1, c->cfg.sweeps));
  // ||Phi - Phi at the previous sweep's end||_F after every sweep: the step
  // kernel that ends a sweep writes one partial per CTA (at most 16), summed
  // once after the loop
  constexpr int kTraceStride = 16;
  const int64_t ntrace = rounds / per;
  float* snap = c->tbuf<float>("phi_snap", (size_t)k * k);
  double* tparts = c->tbuf<double>("conv_parts", (size_t)std::max<int64_t>(1, ntrace) * kTraceStride);
  c->conv = c->tbuf<double>("conv", (size_t)std::max<int64_t>(1, ntrace));
  c->conv_count = 0;
  ck(cudaMemcpyAsync(snap, c->phi, sizeof(float) * k * k, cudaMemcpyDeviceToDevice, s), "trace");
  ck(cudaMemsetAsync(tparts, 0, sizeof(double) * std::max<int64_t>(1, ntrace) * kTraceStride, s),
     "trace");
  OnlineRound rd;
  for (int64_t r = 0; r < rounds; ++r) {
    if (c->stop.load()) throw MmsbError(MMSB_ERR_STOPPED, "stop requested");
    stpm_online_round(c, r, &rd);
    const bool ends_sweep = (r + 1) % per == 0 && c->conv_count < ntrace;
    stpm_step(c, rd, r % 8 == 0, ends_sweep ? snap : nullptr,
              ends_sweep ? tparts + c->conv_count * kTraceStride : nullptr);
    if (ends_sweep) ++c->conv_count;
  }
  ck(conv_sum(tparts, (int)c->conv_count, kTraceStride, kTraceStride, c->conv, s), "trace");
  stpm_finish_online(c, rounds);
}

void pipeline_post(mmsb_ctx* c) {
  if (!c->have_phi || !c->have_white) throw MmsbError(MMSB_ERR_STATE, "postproc before stpm");
  const int k = c->k, ldk = c->ldk;
  cudaStream_t s = c->s;
  const int64_t N = c->nX + c->nA + c->nB + c->nC;
  const int words = (k + 31) / 32;
  c->pi = c->tbuf<float>("pi", (size_t)N * k);
  c->bits = c->tbuf<uint32_t>("bits", (size_t)N * words);
  double* F = c->tbuf<double>("postF", (size_t)k * k);
  double* ZP = c->tbuf<double>("postZP", (size_t)k * k);
  float* PA = c->tbuf<float>("PA", (size_t)c->nA * ldk);
  float* PA2 = c->tbuf<float>("PA2", (size_t)c->nB * ldk);
  const int64_t cap = (int64_t)gram_tsk_partials(c->nA, k, k);
  double* part = c->tbuf<double>("gram_part_post", (size_t)cap);
  // P_A = W Phi diag(pinv(lambda)) = (diag(pinv lambda) Phi^T W^T)^T  (CommunityDetection.cpp:98-100)
  ck(phi_scaled(k, c->phi, c->lambda, c->cfg.pinv_tol, F, s), "F");
  ck(panel_times_small(c->W, ldk, k, c->nA, F, k, k, PA, ldk, s), "PA");
  // pi_a needs Z_B_part2^T (Z_B_part1^T P_A) (CommunityDetection.cpp:101)
  ck(gram_tsk(c->Zb1, ldk, k, PA, ldk, k, c->nA, 1.0, ZP, part, cap, s), "Zb1^T PA");
  ck(panel_times_small(c->Ub, ldk, k, c->nB, ZP, k, k, PA2, ldk, s), "PA2");
  const float tau = c->cfg.tau;
  const DevCsr &XA = c->g[0], &BA = c->g[3], &CA = c->g[4], &BAt = c->gt[3];
  ck(unwhiten_normprob(XA.rp, XA.ci, XA.val, XA.n_rows, PA, ldk, k, tau, 0, c->pi, c->bits, s), "pi_x");
  ck(unwhiten_normprob(BAt.rp, BAt.ci, BAt.val, BAt.n_rows, PA2, ldk, k, tau, c->nX, c->pi, c->bits, s), "pi_a");
  ck(unwhiten_normprob(BA.rp, BA.ci, BA.val, BA.n_rows, PA, ldk, k, tau, c->nX + c->nA, c->pi, c->bits, s), "pi_b");
  ck(unwhiten_normprob(CA.rp, CA.ci, CA.val, CA.n_rows, PA, ldk, k, tau, c->nX + c->nA + c->nB, c->pi, c->bits, s), "pi_c");
  c->have_post = true;
}

// The GPU tree's raw memberships (GPU/post_proc.c:86-106: Pi = ((W evecs)
// inv_evals)^T G^T with inv_evals = diag(||lambda||_2 / lambda_i), the
// pinv threshold applied, GPU/wrappers.cu genInvEvalMat): ||lambda||_2 times
// the unnormalised Pi of pipeline_post, node-major N x k into `out` (device).
void pipeline_post_raw(mmsb_ctx* c, double lambda_norm, float* out) {
  if (!c->have_post) throw MmsbError(MMSB_ERR_STATE, "raw memberships before postproc");
  const int k = c->k, ldk = c->ldk;
  cudaStream_t s = c->s;
  float* PA = c->tbuf<float>("PA", (size_t)c->nA * ldk);
  float* PA2 = c->tbuf<float>("PA2", (size_t)c->nB * ldk);
  const float sc = (float)lambda_norm;
  const DevCsr &XA = c->g[0], &BA = c->g[3], &CA = c->g[4], &BAt = c->gt[3];
  ck(unwhiten_normprob(XA.rp, XA.ci, XA.val, XA.n_rows, PA, ldk, k, 0.f, 0, out, nullptr, s, sc), "raw pi_x");
  ck(unwhiten_normprob(BAt.rp, BAt.ci, BAt.val, BAt.n_rows, PA2, ldk, k, 0.f, c->nX, out, nullptr, s, sc), "raw pi_a");
  ck(unwhiten_normprob(BA.rp, BA.ci, BA.val, BA.n_rows, PA, ldk, k, 0.f, c->nX + c->nA, out, nullptr, s, sc), "raw pi_b");
  ck(unwhiten_normprob(CA.rp, CA.ci, CA.val, CA.n_rows, PA, ldk, k, 0.f, c->nX + c->nA + c->nB, out, nullptr, s, sc), "raw pi_c");
}

// ---------------------------------------------------------------------------
// Adjoint form: L(Phi) = theta sum_ij (phi_i.phi_j)^3 - 2 sum_i That(phi_i,phi_i,phi_i)

namespace {

struct PhiSwap {
  mmsb_ctx* c;
  float* saved;
  double* phi64;
  PhiSwap(mmsb_ctx* ctx, const double* phi_host) : c(ctx), saved(ctx->phi) {
    const int k = c->k;
    phi64 = c->tbuf<double>("loss_phi64", (size_t)k * k);
    c->phi = c->tbuf<float>("loss_phi32", (size_t)k * k);
    ck(cudaMemcpyAsync(phi64, phi_host, sizeof(double) * k * k, cudaMemcpyHostToDevice, c->s), "H2D phi");
    ck(f64_to_f32(phi64, c->phi, (int64_t)k * k, c->s), "phi32");
  }
  ~PhiSwap() { c->phi = saved; }
};

void check_range(mmsb_ctx* c, int64_t& begin, int64_t& count) {
  if (!c->have_y) throw MmsbError(MMSB_ERR_STATE, "loss needs whitened data");
  if (stpm_kp(c->k) < 0) throw MmsbError(MMSB_ERR_UNSUPPORTED, "STPM kernels support k <= 208");
  if (count <= 0) {
    begin = 0;
    count = c->nX;
  }
  if (begin < 0 || begin + count > c->nX) throw MmsbError(MMSB_ERR_INVALID_ARG, "node range");
}

}  // namespace

double pipeline_loss(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count) {
  check_range(c, begin, count);
  const int k = c->k;
  const double a0 = c->cfg.alpha0;
  const double p0 = (a0 + 1.0) * (a0 + 2.0) / 2.0, p1 = a0 * a0, p2 = -a0 * (a0 + 1.0) / 2.0;
  PhiSwap sw(c, phi);
  float* G = c->tbuf<float>("G", (size_t)k * k);
  double* S = c->tbuf<double>("loss_S", (size_t)k * k);
  stpm_pass(c, kModeLoss, 0, 1, 2, begin, count, p0, p1, p2, 1.0, G, c->dscalar + 1);
  ck(dgemm_small(true, false, k, k, k, 1.0, sw.phi64, k, sw.phi64, k, 0.0, S, k, c->s), "S");
  ck(cube_sum(k * k, S, c->cfg.theta, c->dscalar + 2, c->s), "cube");
  double h[2] = {0, 0};
  ck(cudaMemcpyAsync(h, c->dscalar + 1, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->s), "D2H");
  ck(cudaStreamSynchronize(c->s), "sync");
  return h[1] - 2.0 * h[0];
}

void pipeline_loss_grad(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count,
                        double* dphi) {
  check_range(c, begin, count);
  const int k = c->k;
  const double a0 = c->cfg.alpha0;
  const double p0 = (a0 + 1.0) * (a0 + 2.0) / 2.0, p1 = a0 * a0, p2 = -a0 * (a0 + 1.0) / 2.0;
  PhiSwap sw(c, phi);
  float* G = c->tbuf<float>("G", (size_t)k * k);
  double* S = c->tbuf<double>("loss_S", (size_t)k * k);
  double* S2 = c->tbuf<double>("loss_S2", (size_t)k * k);
  double* out = c->tbuf<double>("loss_grad", (size_t)k * k);
  double* dT = c->tbuf<double>("loss_dT", (size_t)k * k);
  // dT: column i = d That_i / d phi_i (three partials of the cubic form)
  stpm_pass(c, kModeAdjoint, 0, 1, 2, begin, count, p0, p1, p2, 1.0 / (double)count, G, nullptr);
  ck(f32_to_f64(G, dT, (int64_t)k * k, c->s), "dT");
  // 6 theta Phi (S o S) - 2 dT
  ck(dgemm_small(true, false, k, k, k, 1.0, sw.phi64, k, sw.phi64, k, 0.0, S, k, c->s), "S");
  ck(hadamard_square((int64_t)k * k, S, S2, c->s), "S2");
  ck(dgemm_small(false, false, k, k, k, 6.0 * c->cfg.theta, sw.phi64, k, S2, k, 0.0, out, k, c->s), "O");
  ck(axpy_f64((int64_t)k * k, -2.0, dT, out, c->s), "grad");
  ck(cudaMemcpyAsync(dphi, out, sizeof(double) * k * k, cudaMemcpyDeviceToHost, c->s), "D2H");
  ck(cudaStreamSynchronize(c->s), "sync");
}
