// Pipeline stages behind the C ABI (host C++; all arithmetic in CUDA kernels).
#pragma once
#include <stdexcept>
#include <string>

#include "context.h"

struct MmsbError : std::runtime_error {
  mmsb_status status;
  MmsbError(mmsb_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

void ck(cudaError_t e, const char* what);

// eigen-pairs (descending) of a symmetric PSD n x n device matrix (n <= 512)
// factor: optional Y with A = Y Y^T (skips the Cholesky)
void sym_eig_refined(mmsb_ctx* c, const std::string& tag, int n, const double* A, double* evals,
                     double* V, const double* factor = nullptr, cudaStream_t stream = nullptr);

void pipeline_upload(mmsb_ctx* c, const mmsb_csr* blocks);
void pipeline_whiten(mmsb_ctx* c, const double* const* sketches);
void pipeline_ydata(mmsb_ctx* c);
void pipeline_stpm(mmsb_ctx* c, const double* phi0);
void pipeline_post(mmsb_ctx* c);
// L(Phi) and dL/dPhi over a node range (adjoint form); phi: k x k column-major host FP64
double pipeline_loss(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count);
void pipeline_loss_grad(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count,
                        double* dphi);
