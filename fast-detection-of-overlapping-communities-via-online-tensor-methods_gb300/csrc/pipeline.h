// Pipeline stages behind the C ABI (host C++; all arithmetic in CUDA kernels).
#pragma once
#include <stdexcept>
#include <string>

#include "context.h"
#include "k_stpm.cuh"

struct MmsbError : std::runtime_error {
  mmsb_status status;
  MmsbError(mmsb_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

void ck(cudaError_t e, const char* what);

// eigen-pairs (descending) of a symmetric PSD n x n device matrix (n <= 512)
// factor: optional Y with A = Y Y^T (skips the Cholesky)
// Reads and clears the device flag word; throws on a set flag (stage names it).
void check_device_flags(mmsb_ctx* c, const char* stage);
// aux (optional, idle on entry): a second stream for X^T X beside A X and
// X^T A X in each refinement step
void sym_eig_refined(mmsb_ctx* c, const std::string& tag, int n, const double* A, double* evals,
                     double* V, const double* factor = nullptr, cudaStream_t stream = nullptr,
                     cudaStream_t aux = nullptr);

void pipeline_upload(mmsb_ctx* c, const mmsb_csr* blocks);
// finish == false leaves the device work queued on the context's streams;
// pipeline_whiten_finish then waits and checks the device flags
void pipeline_whiten(mmsb_ctx* c, const double* const* sketches, bool finish = true);
void pipeline_whiten_finish(mmsb_ctx* c);
void pipeline_ydata(mmsb_ctx* c);
void pipeline_stpm(mmsb_ctx* c, const double* phi0);
void pipeline_post(mmsb_ctx* c);
// ||lambda||_2 * Lambda^-1 Phi^T W^T G^T (the GPU tree's raw Pi), N x k device
void pipeline_post_raw(mmsb_ctx* c, double lambda_norm, float* out);

// pieces of the online / adjoint STPM shared with the batched solver
struct OnlineRound {
  int mode;                    // kModePlain (online) or kModeAdjoint
  int64_t r;                   // update index within the run
  int64_t x0, cnt;             // minibatch nodes
  double beta;                 // step size lr0 / (1 + r)
  bool bf16;                   // BF16 contraction (BF16 form, all sweeps but the last)
  double c0, c1, c2, scale, gscale;
};
void stpm_prepare(mmsb_ctx* c, const double* phi0);
int64_t stpm_online_rounds(const mmsb_ctx* c);
bool stpm_online_round(const mmsb_ctx* c, int64_t r, OnlineRound* out);
mmsb::StpmPartialArgs stpm_partial_args(mmsb_ctx* c, int q1, int q2, int q3, int64_t begin,
                                  int64_t count, double c0, double c2, bool bf16, float* gpart,
                                  int64_t stride, int nblocks);
mmsb::StpmUpdateArgs stpm_online_update_args(mmsb_ctx* c, const OnlineRound& rd, float* gpart,
                                       int64_t stride, int nparts);
// the context's buffer for the step kernel's operand image of Phi (null
// where the tensor-core contraction does not exist for k)
void* stpm_phi_image(mmsb_ctx* c);
void stpm_lambda_pass(mmsb_ctx* c);
void stpm_online_stats(mmsb_ctx* c, int64_t steps);
void stpm_finish_online(mmsb_ctx* c, int64_t steps);
// L(Phi) and dL/dPhi over a node range (adjoint form); phi: k x k column-major host FP64
double pipeline_loss(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count);
void pipeline_loss_grad(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count,
                        double* dphi);
