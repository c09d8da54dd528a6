// Shared declarations of the device kernels (launchers) and small helpers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#define MMSB_CUDA_TRY(expr)                       \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return e_;             \
  } while (0)

namespace mmsb {

constexpr int kNumSMs = 152;

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// Device-side status word shared by kernels that can fail (non-finite
// values, bounded waits).  Bit flags, OR-ed with atomicOr.
enum DeviceFlag : unsigned {
  kFlagNonFinite = 1u,
  kFlagCholeskyBreakdown = 2u,
  kFlagNoConvergence = 4u,
  kFlagTimeout = 8u,
};

// A bounded device wait on a barrier nothing arrives at: sets kFlagTimeout
// after `limit` clock64 cycles (the failure path of every bounded wait).
cudaError_t wait_probe(unsigned* flags, long long limit, cudaStream_t s);

// Counts launches of this library's kernels (reported in mmsb_stats).
extern thread_local int64_t g_launch_count;

// ---- sparse (k_sparse.cu) ---------------------------------------------------

// Y[n_rows x ld] (row-major) = alpha * G * P[n_cols x ld]; ld % 4 == 0.
// p_rows (rows of P, i.e. columns of G), when given, lets panels far larger
// than L2 run as column slices that stay L2-resident.
cudaError_t spmm_f32(const int64_t* rp, const int32_t* ci, const float* val, int64_t n_rows,
                     const float* P, int ld, float alpha, float* Y, cudaStream_t s,
                     int64_t p_rows = 0);
// Checks an uploaded block: ORs 1 into *bad for a decreasing row offset, 2
// for a column index outside [0, n_cols).
cudaError_t csr_validate(const int64_t* rp, const int32_t* ci, int64_t n_rows, int64_t n_cols,
                         int64_t nnz, unsigned* bad, cudaStream_t s);
// Transposed CSR (deterministic: columns sorted within each row).
cudaError_t csr_transpose(const int64_t* rp, const int32_t* ci, const float* val, int64_t n_rows,
                          int64_t n_cols, int64_t nnz, int64_t* rpT, int32_t* ciT, float* valT,
                          int32_t* scratch_cnt, cudaStream_t s);
// out[r] = scale * sum of row r of G (row count for binary)
cudaError_t row_sums_f64(const int64_t* rp, const float* val, int64_t n_rows, double scale,
                         double* out, cudaStream_t s);

// Fused unwhitening + normProbMatrix + threshold over one CSR block:
// raw[r,:] = G[r,:] * P (ld = ldp, first k columns), normalised per row,
// written to pi[(row_offset + r) * k + i] and set bits.  raw_scale > 0:
// raw_scale * raw written instead (no normalisation, bits untouched).
cudaError_t unwhiten_normprob(const int64_t* rp, const int32_t* ci, const float* val,
                              int64_t n_rows, const float* P, int ldp, int k, float tau,
                              int64_t row_offset, float* pi, uint32_t* bits, cudaStream_t s,
                              float raw_scale = 0.f);

// ---- dense (k_dense.cu) -----------------------------------------------------

// S[pa x pb] (column-major FP64) = alpha * A^T B, A: n x pa (lda), B: n x pb (ldb),
// row-major FP32; FP32 partial sums over row chunks, FP64 across chunks.
// (tensor cores, tcgen05 kind::tf32 with the 3xTF32 split, when both sides
// have >= 64 columns and n >= 4096; flags receives a timeout of its bounded
// waits)
cudaError_t gram_tsk(const float* A, int lda, int pa, const float* B, int ldb, int pb, int64_t n,
                     double alpha, double* S, double* partials, int64_t partials_cap,
                     cudaStream_t s, unsigned* flags = nullptr, long long wait_limit = 0);
inline bool gram_use_tc(int64_t n, int pa, int pb) { return pa >= 64 && pb >= 64 && n >= 4096; }
int gram_tc_nsplit(int64_t n, int pa, int pb);
cudaError_t gram_tc_partial(const float* A, int lda, int pa, const float* B, int ldb, int pb,
                            int64_t n, double* partials, int nsplit, unsigned* flags,
                            cudaStream_t s, long long wait_limit = 0);
size_t gram_tsk_partials(int64_t n, int pa, int pb);
// Y[n x ldy] (row-major FP32) = M[n x ldm] (first p cols) * F (p x q, column-major FP64, ldf);
// columns q..ldy-1 of Y are zeroed.
cudaError_t panel_times_small(const float* M, int ldm, int p, int64_t n, const double* F, int ldf,
                              int q, float* Y, int ldy, cudaStream_t s);
// C (m x n) = alpha * op(A) op(B) + beta * C, FP64 column-major, small sizes.
cudaError_t dgemm_small(bool ta, bool tb, int m, int n, int k, double alpha, const double* A,
                        int lda, const double* B, int ldb, double beta, double* C, int ldc,
                        cudaStream_t s);
// Upper Cholesky S = R^T R with drop tolerance: a pivot <= drop2 zeroes row j of R.
cudaError_t chol_upper_drop(int p, const double* S, int lds, double* R, double drop2,
                            unsigned* flags, cudaStream_t s);
// The same factorisation computed in FP32 (R stored as FP64), for a
// well-conditioned S such as the Gram of an already orthonormalised panel;
// pivots <= 0 are dropped.
cudaError_t chol_upper_drop_f32(int p, const double* S, int lds, double* R, unsigned* flags,
                                cudaStream_t s);
// T = R^{-1} for upper triangular R (rows with R_jj == 0 -> zero rows/cols of T).
cudaError_t trinv_upper(int p, const double* R, double* T, cudaStream_t s);
// Eigen-decomposition of Z = Y Y^T from Y (p x p, column-major FP64): one-sided
// Jacobi on Y; eigenvalues descending, eigenvectors column-major p x p.
cudaError_t eig_from_factor(int p, const double* Y, double* evals, double* evecs,
                            float* work, unsigned* flags, cudaStream_t s);
// Modified Gram-Schmidt of the columns of an m x p FP64 matrix (reference drop rule).
cudaError_t mgs_cols(int m, int p, const double* P, int ldp, double* Q, int ldq, double tol,
                     cudaStream_t s);
// Ogita-Aishima eigen refinement pieces (see k_dense.cu); delta_state holds 4
// doubles (the cluster threshold, then scratch for its three maxima).
cudaError_t oa_correction(int n, const double* A, const double* XtX, const double* S, double* E,
                          double* lam, double* delta_state, cudaStream_t s);
cudaError_t sort_eigen(int n, const double* lam, const double* X, double* evals, double* evecs,
                       unsigned* flags, cudaStream_t s);
cudaError_t panel_set_col(float* P, int ld, int64_t rows, int col, const double* v,
                          cudaStream_t s);
cudaError_t panel_copy(const float* src, int lds, int64_t rows, int q, float* dst, int ldd,
                       cudaStream_t s);
// Philox-4x32-10 standard normal panel, row-major n x ld (first q columns).
cudaError_t gaussian_panel(float* P, int64_t n, int q, int ld, uint64_t seed, uint64_t stream,
                           cudaStream_t s);
// Column-major FP64 (rows x cols, ld) <-> row-major FP32 panel conversions.
cudaError_t colmajor64_to_panel(const double* A, int64_t rows, int cols, int64_t lda, float* P,
                                int ldp, cudaStream_t s);
cudaError_t panel_to_colmajor64(const float* P, int ldp, int64_t rows, int cols, double* A,
                                int64_t lda, cudaStream_t s);
// Scale columns: P[:, j] *= d[j] (row-major panel, FP64 factors).
cudaError_t panel_scale_cols(float* P, int ldp, int64_t n, int q, const double* d,
                             cudaStream_t s);
cudaError_t fill_f32(float* p, int64_t n, float v, cudaStream_t s);
cudaError_t fill_f64(double* p, int64_t n, double v, cudaStream_t s);
// dst[j] = src[j] (FP64 vector ops on device, tiny)
cudaError_t axpy_f64(int64_t n, double a, const double* x, double* y, cudaStream_t s);

// ---- small element-wise helpers (k_misc.cu) -----------------------------------
// conv[i] = sqrt of the sum of parts[i * stride + 0 .. used - 1] (the step
// kernel's per-CTA trace partials), for i < count
cudaError_t conv_sum(const double* parts, int count, int stride, int used, double* conv,
                     cudaStream_t s);

cudaError_t sig_from_evals(int k, const double* ev, double* sig, cudaStream_t s);
cudaError_t scale_cols_pinv(int rows, int k, double* F, int ldf, const double* sig, double tol,
                            cudaStream_t s);
cudaError_t sqrt_pinv(int k, const double* sig, double tol, double* a, double* b, cudaStream_t s);
cudaError_t diag_guard(int k, double* core, cudaStream_t s);
cudaError_t panel_rank1(float* P, int ld, int64_t n, int q, double alpha, const double* u,
                        const double* v, cudaStream_t s);
cudaError_t f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s);
cudaError_t f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t s);
// row-major rows x cols FP32 panel (stride ld) -> BF16 panel (stride ldh >= cols, zero padded)
cudaError_t panel_to_bf16(const float* src, int64_t ld, int64_t rows, int cols, void* dst,
                          int64_t ldh, cudaStream_t s);
cudaError_t phi_scaled(int k, const float* phi, const double* lambda, double tol, double* F,
                       cudaStream_t s);
cudaError_t transpose_f64(int p, const double* A, double* At, cudaStream_t s);
cudaError_t cube_sum(int n, const double* S, double a, double* out, cudaStream_t s);
cudaError_t hadamard_square(int64_t n, const double* a, double* b, cudaStream_t s);
cudaError_t mask_cols(int rows, int k, double* F, int ldf, const double* sig, double tol,
                      cudaStream_t s);
cudaError_t set_row_scaled(int rows, int cols, double* B, int ldb, int row, double alpha,
                           const double* v, cudaStream_t s);
cudaError_t eye_mask(int m, int p, const double* R, int ldr, double* Q, int ldq, cudaStream_t s);

// ---- ground-truth evaluation (k_eval.cu) --------------------------------------

// Mean and population variance of each of the m columns of a node-major
// n x m FP32 panel (ld), FP64; part holds colstats_partials(n, m) doubles.
size_t colstats_partials(int64_t n, int m);
cudaError_t column_stats(const float* X, int ld, int m, int64_t n, double* part, double* mean,
                         double* var, cudaStream_t s);
// Y (n x m, ld m) = X - mean per column, FP32.
cudaError_t center_columns(const float* X, int ld, int m, int64_t n, const double* mean, float* Y,
                           cudaStream_t s);
// Correlation, t statistic and two-sided p-value (Pvalue.cpp:85-235) of every
// pair from C = A_c^T B_c (k x K, column-major), n and the variances.
cudaError_t pair_pvalues(const double* C, int k, int K, int64_t n, const double* va,
                         const double* vb, double* corr, double* tstat, double* pval,
                         unsigned* flags, cudaStream_t s);

}  // namespace mmsb
