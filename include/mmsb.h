/*
 * mmsb.h -- C ABI of the GB300-native MMSB tensor-method pipeline.
 *
 * The pipeline is the reference's community-detection path
 *   whitening  ->  whitened data y = W^T G^T  ->  tensor power method  ->
 *   unwhitening + normalisation,
 * i.e. CommunityDetectionSoftware_CPU/CommunityDetection/CommunityDetection.cpp:16-149
 * (CPU tree) and CommunityDetectionSoftware_GPU/stpm.c:132-1015 (GPU tree).
 *
 * Conventions
 *   - every call returns mmsb_status (MMSB_OK == 0); nothing calls exit();
 *     the reference exits with 1 on file errors (IOfn.cpp:30-34,
 *     GPU/pre_proc.c:54-58) and 2 on library errors (GPU/pre_proc.c:96-109);
 *   - dense matrices are column-major, like Eigen's default and CULA;
 *   - all pointers passed to the API are HOST pointers; the library owns the
 *     device copies and the CUDA streams of a context (a main stream, on
 *     which every call's work is ordered, and helper streams that the
 *     whitening forks from it and joins back before it returns);
 *   - a context is not thread-safe, except mmsb_request_stop();
 *   - graph blocks are CSR with int64 row offsets and int32 column indices,
 *     0-based (the text readers convert the reference's 1-based COO).
 */
#ifndef MMSB_H_
#define MMSB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMSB_ABI_VERSION 1

typedef enum mmsb_status {
  MMSB_OK = 0,
  MMSB_ERR_INVALID_ARG = 1,
  MMSB_ERR_CUDA = 2,
  MMSB_ERR_OUT_OF_MEMORY = 3,
  MMSB_ERR_STATE = 4,      /* call out of order (e.g. stpm before whiten) */
  MMSB_ERR_NUMERICAL = 5,  /* NaN/Inf or a factorisation that broke down */
  MMSB_ERR_STOPPED = 6,    /* mmsb_request_stop() was honoured */
  MMSB_ERR_IO = 7,
  MMSB_ERR_TIMEOUT = 8,    /* a bounded device-side wait gave up */
  MMSB_ERR_UNSUPPORTED = 9
} mmsb_status;

/* The five adjacency blocks the reference reads (CommunityDetection.cpp:30-34,
 * 47-49, 94-95): rows x cols. */
enum {
  MMSB_BLOCK_XA = 0, /* n_X x n_A  (Gx_a) */
  MMSB_BLOCK_XB = 1, /* n_X x n_B  (Gx_b) */
  MMSB_BLOCK_XC = 2, /* n_X x n_C  (Gx_c) */
  MMSB_BLOCK_BA = 3, /* n_B x n_A  (Gb_a) */
  MMSB_BLOCK_CA = 4, /* n_C x n_A  (Gc_a) */
  MMSB_NUM_BLOCKS = 5
};

typedef enum mmsb_stpm_method {
  /* tensorDecom_alpha0 (CPU/Util.cpp:131-184): full-batch power iteration,
   * lambda = ||T(I,phi,phi)||^3, column normalisation, MINITER/MAXITER/TOLERANCE */
  MMSB_STPM_BATCH_POWER = 0,
  /* minibatch stochastic update with the Diff_Loss gradient (CPU/Util.cpp:257-304)
   * and re-orthonormalisation after every step (GPU/stpm.c:774-786) */
  MMSB_STPM_ONLINE = 1,
  /* the same schedule driven by the exact adjoint of the implicit tensor loss
   * L(Phi) = theta*sum_ij (phi_i.phi_j)^3 - 2*sum_i T(phi_i,phi_i,phi_i) */
  MMSB_STPM_ADJOINT = 2
} mmsb_stpm_method;

typedef enum mmsb_precision {
  MMSB_PREC_FP32 = 0, /* y, Phi and every bulk product in FP32 */
  MMSB_PREC_BF16 = 1  /* y and Phi in BF16 on the tensor cores, FP32 accumulation */
} mmsb_precision;

typedef struct mmsb_config {
  int32_t k;              /* KHID: number of communities */
  double alpha0;          /* Dirichlet concentration */
  int32_t datatype;       /* DATATYPE: 0 binary, 1 weighted (IOfn.cpp:40-49) */
  int32_t stpm_method;    /* mmsb_stpm_method */
  int32_t precision;      /* mmsb_precision */
  int32_t sweeps;         /* online/adjoint: passes over the X partition */
  int32_t minibatch;      /* online/adjoint: nodes per update */
  double lr0;             /* online/adjoint: beta_t = lr0 / (1 + t) */
  double theta;           /* weight of the orthogonality term of the loss */
  int32_t min_iter;       /* batch power: MINITER  (CPU/stdafx.h:57) */
  int32_t max_iter;       /* batch power: MAXITER  (CPU/stdafx.h:58) */
  double tol;             /* batch power: TOLERANCE (CPU/stdafx.h:59) */
  double pinv_tol;        /* pinv threshold, TOLERANCE in CPU/Spectral.cpp:44-68 */
  int32_t nystrom_rows_factor; /* Nystrom branch iff rows > factor*k (Spectral.cpp:173) */
  int32_t normalize;      /* NORMALIZE (CPU/stdafx.h:60): moments scaled by 1/n_X */
  uint64_t seed;          /* Gaussian sketch panel and initial Phi */
  float tau;              /* community-set threshold on normalised Pi */
  int32_t device;         /* CUDA device ordinal */
} mmsb_config;

/* One CSR block (host memory).  val == NULL means binary (all ones). */
typedef struct mmsb_csr {
  int64_t n_rows;
  int64_t n_cols;
  int64_t nnz;
  const int64_t* row_ptr; /* n_rows + 1 */
  const int32_t* col_idx; /* nnz */
  const float* val;       /* nnz or NULL */
} mmsb_csr;

/* Device time of each stage of the last call, milliseconds (CUDA events on
 * the context's stream), plus iteration counters. */
typedef struct mmsb_stats {
  double whiten_ms;
  double ydata_ms;
  double stpm_ms;
  double post_ms;
  double total_ms;
  double spmm_ms;          /* summed time of the whitening SpMM launches */
  double spmm_bytes;       /* algorithmic bytes of those launches */
  int64_t spmm_launches;
  int64_t stpm_steps;      /* minibatch updates (online/adjoint) or iterations (batch) */
  int64_t node_updates;    /* n_X * sweeps (online/adjoint) or n_X * iterations */
  double stpm_last_error;  /* batch power: last ||Phi - Phi_old||_F */
  int64_t kernel_launches; /* launches of this library's kernels by the last call */
  int64_t orth_passes;     /* exact Cholesky QR passes summed over the STPM steps */
  /* STPM kernels of the last mmsb_stpm, timed with CUDA events around each
   * launch; flops are algorithmic (k, not the padded tile size):
   * contraction 2 k^2 per node per Z and per G product, step 7 k^3 per
   * online update (its Grams and products, the first-order QR pass) plus
   * 11/3 k^3 per exact Cholesky QR pass */
  double contract_ms;
  double contract_flops;
  int64_t contract_launches;
  double step_ms;
  double step_flops;
  int64_t step_launches;
  /* largest max_ij |Q1^T Q1 - I| over the steps, Q1 the result of the exact
   * Cholesky QR passes of a step before its first-order pass (the returned
   * Phi is orthonormal to about the square of this, or FP32 round-off) */
  double orth_err_max;
} mmsb_stats;

typedef struct mmsb_ctx mmsb_ctx;

/* ---- configuration and lifetime ---------------------------------------- */

/* Fills the reference's defaults: alpha0 1, binary, batch power with
 * MINITER 100 / MAXITER 10000 / TOLERANCE 1e-6 (CPU/stdafx.h:56-60),
 * pinv tolerance 1e-6, Nystrom factor 20, NORMALIZE on; online schedule
 * 10 sweeps, minibatch 100, beta_t = 1/(1+t), theta 1/2 (the weight
 * 1 - 3 theta beta_t of Phi in the online step is then never 0). */
void mmsb_config_default(mmsb_config* cfg);

/* Replaces the reference's globals NX..KHID/alpha0/DATATYPE
 * (CPU/CommunityDetection.cpp:9-26) and the GPU tree's device choice
 * (GPU/stpm.c:1111-1118). */
mmsb_status mmsb_create(const mmsb_config* cfg, mmsb_ctx** out);
void mmsb_destroy(mmsb_ctx* ctx);

/* Copies the five blocks to the device, checks them there (row offsets
 * non-decreasing, column indices inside the block) and builds their
 * transposes.  A block that fails a check returns MMSB_ERR_INVALID_ARG and
 * leaves the context without a graph.  Host buffers pinned with
 * mmsb_host_register are copied at full link speed.
 * Replaces read_G_sparse x5 (CPU/IOfn.cpp:21-54; CommunityDetection.cpp:47-49,94-95)
 * and read_G (GPU/pre_proc.c:49-80). */
mmsb_status mmsb_upload_graph(mmsb_ctx* ctx, const mmsb_csr blocks[MMSB_NUM_BLOCKS]);

/* Page-locks (unlocks) an existing host buffer so that uploads from it and
 * result downloads into it run as direct DMA instead of through staging
 * copies.  No counterpart in the reference (its host path never leaves the
 * CPU); a thin wrapper of cudaHostRegister / cudaHostUnregister. */
mmsb_status mmsb_host_register(void* ptr, size_t bytes);
mmsb_status mmsb_host_unregister(void* ptr);

/* ---- pipeline stages ------------------------------------------------------ */

/* second_whiten (CPU/Util.cpp:38-127) plus the whitened data and means
 * (CommunityDetection.cpp:66-68); GPU tree: pre_proc (GPU/pre_proc.c:112-372).
 * sketches == NULL: Gaussian sketch panels N(0,1) drawn on the device from
 * cfg.seed.  Otherwise sketches[0..2] are R_c (n_B x 2k), R_b (n_C x 2k) and
 * R_a (n_A x 2k), column-major, used where random_embedding_mat
 * (CPU/Spectral.cpp:118-134) is called. */
mmsb_status mmsb_whiten(mmsb_ctx* ctx, const double* const* sketches);

/* Tensor decomposition: tensorDecom_alpha0 (CPU/Util.cpp:131-184) or the
 * GPU tree's STPM loop (GPU/stpm.c:497-809), per cfg.stpm_method.
 * phi0 == NULL: orthonormal start drawn from cfg.seed; else k x k column-major. */
mmsb_status mmsb_stpm(mmsb_ctx* ctx, const double* phi0);

/* Unwhitening, concatenation [X|A|B|C], normProbMatrix and the community-set
 * threshold: CommunityDetection.cpp:98-139 / GPU/post_proc.c:62-119. */
mmsb_status mmsb_postproc(mmsb_ctx* ctx);

/* mmsb_whiten(NULL) + mmsb_stpm(NULL) + mmsb_postproc on the uploaded graph. */
mmsb_status mmsb_run(mmsb_ctx* ctx);

/* ---- results (host buffers) --------------------------------------------- */

int64_t mmsb_num_nodes(const mmsb_ctx* ctx); /* n_X + n_A + n_B + n_C */

/* Normalised memberships, k x N column-major over the node order [X|A|B|C]
 * (CommunityDetection.cpp:121-139). */
mmsb_status mmsb_get_pi(mmsb_ctx* ctx, float* pi);
/* Ground-truth evaluation (CPU/Pvalue.cpp:85-235, the hypothesis test the
 * reference ships for matching recovered to true communities): for every
 * pair (i, j) of an estimated community i (row of Pi) and a true community j
 * (row j of truth, a k_true x N column-major host array in the node order
 * [X|A|B|C], e.g. data/Pi_true_*), the Pearson correlation over the N nodes,
 * t = r sqrt((N-2)/(1-r^2)) and the two-sided p-value from the incomplete
 * beta function with the reference's branch rules.  Outputs are k x k_true
 * column-major FP64 (entry i + j k); any may be NULL.  Requires
 * mmsb_postproc. */
mmsb_status mmsb_pvalues(mmsb_ctx* ctx, const float* truth, int32_t k_true, double* corr,
                         double* tstat, double* pval);
/* Convergence trace of the last mmsb_stpm: batch power, ||Phi - Phi_old||_F
 * of every iteration (the GPU tree's frob_norm values, GPU/stpm.c:743, up to
 * 100000); online/adjoint, ||Phi - Phi at the previous sweep's end||_F after
 * every sweep.  Copies min(cap, count) values; *count gets the total. */
mmsb_status mmsb_get_convergence(mmsb_ctx* ctx, double* out, int64_t cap, int64_t* count);
/* The GPU tree's output files (GPU/post_proc.c:110-114, GPU/stpm.c:915-963)
 * into directory dir, named <name>_<k>_<alpha0>_<lr0>.txt as GPU/stpm.h:82-91:
 * Pi_X, Pi_A, Pi_B, Pi_C (normalised Pi, k x n_P column-major), evecs (Phi,
 * k x k column-major), evals (Dirichlet weights lambda^-2 / sum lambda^-2),
 * frob_norm (the convergence trace) -- one "%5.25e" value per line -- and
 * sim_info (sizes, parameters and stage times). */
mmsb_status mmsb_write_gpu_outputs(mmsb_ctx* ctx, const char* dir);

/* Community sets {i : pi(i,node) > tau}: N words of ceil(k/32) uint32 each. */
mmsb_status mmsb_get_sets(mmsb_ctx* ctx, uint32_t* bits);
mmsb_status mmsb_get_lambda(mmsb_ctx* ctx, double* lambda);  /* k */
mmsb_status mmsb_get_phi(mmsb_ctx* ctx, double* phi);        /* k x k */
/* W (n_A x k), Z_B_part1 (n_A x k), Z_B_part2 (k x n_B), Z_C_part1 (n_A x k),
 * Z_C_part2 (k x n_C); any pointer may be NULL (CPU/Util.cpp:38-40 outputs). */
mmsb_status mmsb_get_whitening(mmsb_ctx* ctx, double* W, double* zb1, double* zb2,
                               double* zc1, double* zc2);
mmsb_status mmsb_get_means(mmsb_ctx* ctx, double* mu_a, double* mu_b, double* mu_c);
/* Whitened data k x n_X column-major (Data_a_G/Data_b_G/Data_c_G) and the
 * whitened means (k each); any pointer may be NULL. */
mmsb_status mmsb_get_whitened(mmsb_ctx* ctx, float* ya, float* yb, float* yc,
                              double* ymu_a, double* ymu_b, double* ymu_c);
mmsb_status mmsb_get_stats(const mmsb_ctx* ctx, mmsb_stats* out);

/* ---- stage inputs (stage-wise parity with the reference) ---------------- */

/* Installs W, Z_B_part1/2, Z_C_part1/2 and the means (same shapes as the
 * getters) and computes the whitened data from them on the device. */
mmsb_status mmsb_set_whitening(mmsb_ctx* ctx, const double* W, const double* zb1,
                               const double* zb2, const double* zc1, const double* zc2,
                               const double* mu_a, const double* mu_b, const double* mu_c);
/* Installs whitened data (k x n_X column-major) and whitened means. */
mmsb_status mmsb_set_whitened(mmsb_ctx* ctx, const double* ya, const double* yb,
                              const double* yc, const double* ymu_a, const double* ymu_b,
                              const double* ymu_c);
/* Installs Phi (k x k) and lambda (k) for mmsb_postproc. */
mmsb_status mmsb_set_phi_lambda(mmsb_ctx* ctx, const double* phi, const double* lambda);

/* ---- adjoint form ------------------------------------------------------- */

/* Implicit tensor loss over the whitened nodes [node_begin, node_begin+count)
 * (count <= 0: all of X):
 *   L(Phi) = theta * sum_ij (phi_i . phi_j)^3 - 2 * sum_i That(phi_i, phi_i, phi_i),
 *   That(u,u,u) = mean_x [p0 (u.a)(u.b)(u.c) + p2((u.a)(u.b)(u.mc) + (u.a)(u.mb)(u.c)
 *                 + (u.ma)(u.b)(u.c))] + p1 (u.ma)(u.mb)(u.mc),
 * p0 = (a0+1)(a0+2)/2, p1 = a0^2, p2 = -a0(a0+1)/2 (CPU/Util.cpp:289-291).
 * This is ||T - sum phi^{x3}||^2 - ||T||^2 for theta = 1.  Forward returns L;
 * backward returns dL/dPhi (k x k column-major), recomputing Z = Phi^T y. */
mmsb_status mmsb_stpm_loss_fwd(mmsb_ctx* ctx, const double* phi, int64_t node_begin,
                               int64_t count, double* loss);
mmsb_status mmsb_stpm_loss_bwd(mmsb_ctx* ctx, const double* phi, int64_t node_begin,
                               int64_t count, double* dphi);

/* ---- control ------------------------------------------------------------ */

/* Thread-safe; mirrors forceExit_flag (GPU/stpm.c:61,754-758).  The STPM loop
 * stops at the next step boundary and the call returns MMSB_ERR_STOPPED. */
void mmsb_request_stop(mmsb_ctx* ctx);
const char* mmsb_last_error(const mmsb_ctx* ctx);

/* Failure detection of the device side.  The reference has no device-side
 * waits to bound (its CULA calls block, GPU/stpm.c:497-809); here every wait
 * of the STPM kernels and of the tensor-core Grams on a barrier, a copy or a
 * peer CTA gives up after a limit of clock64 cycles, sets a device flag and
 * the call returns MMSB_ERR_TIMEOUT with the context still usable.
 * mmsb_set_wait_limit: that limit for the kernels of this context
 * (0 = about one second).  mmsb_diag_wait_timeout: one bounded wait, of the
 * same helper, on a barrier that nothing arrives at, with a limit of `cycles`
 * (1 .. 2e9): returns MMSB_ERR_TIMEOUT when the give-up path works. */
mmsb_status mmsb_set_wait_limit(mmsb_ctx* ctx, int64_t cycles);
mmsb_status mmsb_diag_wait_timeout(mmsb_ctx* ctx, int64_t cycles);
const char* mmsb_status_string(mmsb_status st);
/* Writes a buffer larger than L2 on the context's stream (benchmark hygiene). */
mmsb_status mmsb_flush_l2(mmsb_ctx* ctx);
mmsb_status mmsb_synchronize(mmsb_ctx* ctx);

/* ---- single operators (tests and kernel benchmarks) ----------------------- */

/* Y (n_rows x p, row-major) = alpha * G * P (P: n_cols x p, row-major);
 * with transpose != 0, Y (n_cols x p) = alpha * G^T * P (P: n_rows x p). */
mmsb_status mmsb_op_spmm(const mmsb_csr* g, int transpose, const float* P, int64_t p,
                         float alpha, float* Y);
/* Symmetric eigen-decomposition of an n x n positive semi-definite matrix
 * (column-major, n <= 512), eigenvalues descending; vectors column-major n x n. */
/* S (pa x pb, column-major FP64) = alpha A^T B for node-major FP32 panels A
 * (n x pa) and B (n x pb), host arrays: the tall-skinny Gram of the Nystrom
 * chain (X^T (X R) products of CPU/Spectral.cpp:228-246 and the CholQR
 * Grams), on the tensor cores (tcgen05, 3xTF32) when pa, pb >= 64. */
mmsb_status mmsb_op_gram(const float* A, int64_t n, int32_t pa, const float* B, int32_t pb,
                         double alpha, double* S);
mmsb_status mmsb_op_symeig(const double* A, int32_t n, double* evals, double* evecs);

/* No counterpart in the reference.  Y = alpha * G^T * P for callers that
 * cannot allocate device memory (code inside another framework's memory pool,
 * which owns every device allocation, or latency-critical code that must not
 * wait on cudaMalloc, which can synchronize the device): same result as
 * mmsb_op_spmm with
 * transpose != 0, but every pointer is a DEVICE pointer the caller owns and
 * the call allocates nothing.  G: n_rows x n_cols CSR (d_val NULL = binary)
 * with row_ptr[0] == 0, non-decreasing offsets, row_ptr[n_rows] == nnz and
 * 0 <= col < n_cols (not checked: a block breaking them gives a wrong Y, but
 * no access outside the buffers and the array); P: n_rows x p row-major,
 * Y: n_cols x p row-major, p a multiple of 4, both 16-byte aligned
 * (MMSB_ERR_INVALID_ARG otherwise).  The transposed copy of G is built in a
 * fixed 8 MiB device array compiled into the library (held on every GPU that
 * loads it until exit): blocks needing more (about 16 * (n_cols + 1 + nnz)
 * bytes) return MMSB_ERR_UNSUPPORTED before any work.  All calls share that
 * array, so calls that overlap on the GPU race; serialise them.  The first
 * call in a CUDA context looks the array up (this can load the module): make
 * it before any stream capture; after a device reset the next call looks it
 * up again.  stream: a cudaStream_t (NULL = default stream). */
mmsb_status mmsb_op_spmm_t_noalloc(const int64_t* d_row_ptr, const int32_t* d_col_idx,
                                   const float* d_val, int64_t n_rows, int64_t n_cols,
                                   int64_t nnz, const float* d_P, int64_t p, float alpha,
                                   float* d_Y, void* stream);

/* ---- synthetic MMSB graphs ---------------------------------------------- */

typedef struct mmsb_gen_params {
  int64_t n;        /* nodes, split uniformly at random into X, A, B, C */
  int32_t k;        /* communities */
  double alpha0;    /* Dirichlet(alpha0/k * 1) memberships */
  double p_in;      /* B diagonal */
  double p_out;     /* B off-diagonal */
  uint64_t seed;
  int32_t keep_pi;  /* keep the ground-truth memberships */
} mmsb_gen_params;

typedef struct mmsb_host_graph mmsb_host_graph;

mmsb_status mmsb_generate(const mmsb_gen_params* params, mmsb_host_graph** out);
void mmsb_host_graph_free(mmsb_host_graph* g);
/* part sizes n_X, n_A, n_B, n_C; undirected edge count */
mmsb_status mmsb_host_graph_info(const mmsb_host_graph* g, int64_t part_sizes[4],
                                 int64_t* n_edges);
/* Borrowed view of one block, valid until mmsb_host_graph_free. */
mmsb_status mmsb_host_graph_block(const mmsb_host_graph* g, int which, mmsb_csr* out);
/* Ground-truth memberships k x N column-major in [X|A|B|C] order (keep_pi). */
mmsb_status mmsb_host_graph_pi(const mmsb_host_graph* g, float* pi);

/* ---- file contract (CPU/IOfn.cpp:21-67) ----------------------------------- */

/* Reads a 1-based COO text block ("row col" or "row col value", any
 * whitespace, datatype 0/1), parsed on up to 16 threads.  compat != 0
 * reproduces the reference reader (read_G_sparse, IOfn.cpp:21-54) exactly:
 * its while(!feof) loop pushes the last triplet a second time unless the last
 * number ends the file, completes a trailing partial triplet with the
 * previous values, sums duplicates and prunes |v| <= 1e-18 (prune(1e-6)).
 * compat == 0: no extra triplet, a partial triplet is an error, the last
 * duplicate wins, nothing is pruned.  A non-number token is an error (the
 * reference would loop forever).  The block is owned by a host graph handle
 * freed with mmsb_host_graph_free. */
mmsb_status mmsb_read_coo(const char* path, int64_t n_rows, int64_t n_cols,
                          int32_t datatype, int32_t compat, mmsb_host_graph** out);
/* Writes "row\tcol\tvalue" 1-based triplets of the nonzeros of a column-major
 * rows x cols matrix in column order, values with 6 significant digits,
 * as write_pi (IOfn.cpp:57-67) prints them. */
mmsb_status mmsb_write_triplets_f32(const char* path, const float* m, int64_t rows,
                                    int64_t cols);
mmsb_status mmsb_write_triplets_f64(const char* path, const double* m, int64_t rows,
                                    int64_t cols);
/* write_mat (GPU/post_proc.c:45-59): count values, one "%5.25e" per line. */
mmsb_status mmsb_write_dense_f32(const char* path, const float* m, int64_t count);
mmsb_status mmsb_write_dense_f64(const char* path, const double* m, int64_t count);
/* A block in the input contract read by mmsb_read_coo: 1-based "row col"
 * lines (val == NULL) or "row col value" (9 significant digits), row by row.
 * No counterpart in the reference (it only reads this format). */
mmsb_status mmsb_write_coo(const char* path, const mmsb_csr* m);
/* Binary CSR container, no counterpart in the reference: "MMSBCSR" + version
 * byte 1, int64 n_rows, n_cols, nnz, int32 has_values, int32 0, int64
 * row_ptr[n_rows + 1], int32 col_idx[nnz], float val[nnz] if has_values,
 * little-endian.  mmsb_read_csr checks the structure (offsets 0..nnz,
 * non-decreasing, columns in range) and returns a host graph of one block. */
mmsb_status mmsb_write_csr(const char* path, const mmsb_csr* m);
mmsb_status mmsb_read_csr(const char* path, mmsb_host_graph** out);

/* ---- batched solver (many independent graphs) ----------------------------
 * No counterpart in the reference, which solves one graph per process.  Each
 * graph has its own context (k, alpha0 and seed base->seed + index; every
 * other field from base, online or adjoint method, minibatch optionally per
 * graph); the whitening chains of
 * all graphs are queued concurrently, and the STPM minibatch updates of all
 * graphs advance together: per round one contraction launch and one step
 * launch per group of graphs with the same padded k, the whole round loop
 * captured in a CUDA graph on the first run and replayed afterwards.  The
 * contraction's CTAs per graph are chosen per group by timing candidates on
 * the first run.  Results of graph i: the mmsb_get_* functions on
 * mmsb_batch_graph(b, i). */
typedef struct mmsb_batch mmsb_batch;

typedef struct mmsb_batch_stats {
  double total_ms;        /* last run: start to the last graph's results (device events) */
  double stpm_end_ms;     /* batched run: start to the end of the STPM rounds */
  double wall_ms;         /* host wall clock of the last run */
  double latency_p50_ms;  /* per-graph latency: start to the graph's results */
  double latency_p99_ms;
  double latency_max_ms;
  int64_t rounds;           /* batched minibatch rounds (the longest schedule) */
  int64_t batched_launches; /* kernel launches of the STPM round loop */
  int32_t graph_replayed;   /* 1: the round loop ran as a CUDA graph replay */
  int32_t buckets;          /* groups of graphs with the same padded k */
  int32_t bucket_kp[8];
  int32_t bucket_ctas[8];   /* tuned contraction CTAs per graph */
  int32_t bucket_graphs[8];
} mmsb_batch_stats;

/* k[count] required; alpha0[count] and minibatch[count] optional (NULL: base's) */
mmsb_status mmsb_batch_create(const mmsb_config* base, int32_t count, const int32_t* k,
                              const double* alpha0, const int32_t* minibatch, mmsb_batch** out);
void mmsb_batch_destroy(mmsb_batch* b);
/* upload graph `graph` (all before the first run) */
mmsb_status mmsb_batch_upload(mmsb_batch* b, int32_t graph, const mmsb_csr blocks[MMSB_NUM_BLOCKS]);
/* whitening, STPM and post-processing of every graph, batched */
mmsb_status mmsb_batch_run(mmsb_batch* b);
/* the same work graph by graph, each through the single-graph pipeline */
mmsb_status mmsb_batch_run_sequential(mmsb_batch* b);
int32_t mmsb_batch_count(const mmsb_batch* b);
/* contraction CTAs per graph: 0 (default) lets the first run choose by
 * timing; a positive multiple of 8 fixes it (before the first run) */
mmsb_status mmsb_batch_set_contract_ctas(mmsb_batch* b, int32_t ctas);
mmsb_ctx* mmsb_batch_graph(mmsb_batch* b, int32_t graph);
/* per-graph latency (ms) of the last run, count values */
mmsb_status mmsb_batch_latencies(const mmsb_batch* b, double* ms);
mmsb_status mmsb_batch_get_stats(const mmsb_batch* b, mmsb_batch_stats* out);
const char* mmsb_batch_last_error(const mmsb_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* MMSB_H_ */
