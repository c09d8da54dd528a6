// Argument blocks and launchers of the tensor-power-method kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mmsb {

enum StpmMode : int {
  kModePlain = 0,    // one contraction with (Y1, Y2 -> Yout)
  kModeAdjoint = 1,  // exact gradient of the cubic form: three contractions
  kModeLoss = 2,     // forward value of the cubic form only
};

enum StpmStep : int {
  kStepOnline = 0,  // Phi - beta (3 theta O - gscale G), then QR (diag(R) > 0)
  kStepQR = 1,      // Q of the QR factorisation of Phi only
};

struct StpmPartialArgs {
  const float* y1;
  const float* y2;
  const float* y3;  // plain: Yout
  int64_t ldy;      // row stride of the node-major y arrays (multiple of 4)
  const void* yh1;  // BF16 copies of y1..y3 (BF16 form), row stride ldyh (multiple of 8)
  const void* yh2;
  const void* yh3;
  int64_t ldyh;
  const float* phi; // k x k column-major
  const float* mu1;
  const float* mu2;
  const float* mu3;
  int64_t begin, count;  // node range
  int k;
  float c0, c2;          // plain: C = c0 Z1Z2 + c2(Z1 m2 + m1 Z2); adjoint/loss: p0, p2
  float* gpart;          // [grid][part_stride]: k*k partial G, then 3k d-sums (+1 loss)
  int64_t part_stride;
  int nblocks;           // batched launches: CTAs of this graph (multiple of the cluster size)
  unsigned* flags;       // device flag word (MMSB_ERR_TIMEOUT of a bounded wait), may be null
  long long wait_limit;  // clock64 cycles a bounded wait may take (0: about one second)
  // tensor-core plain FP32 form (KP <= 112): Phi already split into its TF32
  // hi / lo operand image, followed by Phi^T mu1 | Phi^T mu2 (2 KP floats),
  // as the previous step kernel wrote it (stpm_phi_image_bytes); null: the
  // contraction stages Phi itself
  const void* phi_img;
};

// bytes of the operand image of Phi that the step kernel writes for the
// tensor-core contraction (0 where that form does not exist for k)
size_t stpm_phi_image_bytes(int k);

struct StpmReduceArgs {
  int mode;
  int k;
  const float* gpart;
  int64_t part_stride;
  int nparts;
  const float* phi;
  const float* mu1;
  const float* mu2;
  const float* mu3;
  const float* mu_out;  // plain mode
  double c1, c2;        // plain: d = c1 m1 m2 + c2 sum Z1Z2; adjoint/loss: p1, p2
  double scale;         // multiplies the contraction (adjoint: 1/count)
  double count;         // nodes in the pass
  float* G;             // k x k column-major output
  double* loss_out;     // loss mode: sum_i That(phi_i,phi_i,phi_i)
};

struct StpmUpdateArgs {
  int k;
  int step_mode;
  float* phi;           // in/out, k x k column-major
  const float* G;       // unused by the fused step (kept for the batch path)
  // fused reduction of the partial kernel's output (online/adjoint steps)
  int mode;             // kModePlain or kModeAdjoint
  const float* gpart;
  int64_t part_stride;
  int nparts;
  const float* mu1;
  const float* mu2;
  const float* mu3;     // plain: mu_out
  double c1, c2, scale, count;
  float beta;
  float theta3;         // 3 * theta
  float gscale;         // 3 (plain) or 1 (adjoint: G already holds dT)
  int max_passes;        // exact Cholesky QR passes per step at most
  unsigned* flags;
  int* orth_passes;      // accumulates the exact Cholesky QR passes (may be null)
  float* orth_err;       // max |Q1^T Q1 - I| before the first-order pass, max over steps (may be null)
  float* xstash;         // KP x KP scratch in global memory (KP > 128 only)
  long long wait_limit;  // clock64 cycles a bounded wait may take (0: about one second)
  int active;            // batched launches: 0 = no update for this graph in this round
  // online steps: 1 = form Phi (Phi^T Phi)^.2 literally (the first step of a
  // run, whose Phi0 need not be orthonormal); 0 = Phi is the previous step's
  // Q (orthonormal to ~1e-7), so the diagonal of (Phi^T Phi)^.2 suffices
  int phi_general;
  // the contraction's operand image of the new Phi (stpm_phi_image_bytes), or
  // null
  void* phi_img;
  // convergence trace (may be null): CTA q writes sum over its columns of
  // (Phi_new - trace_snap)^2 to trace_out[q] and sets trace_snap = Phi_new there
  float* trace_snap;
  double* trace_out;
};

int stpm_kp(int k);
int stpm_step_kp(int k);
// grid of the partial kernel (a multiple of its cluster size); partial
// blocks written = grid / stpm_partial_cluster()
int stpm_partial_grid(int64_t count, bool bf16);
int stpm_partial_cluster();
// bf16: y read from yh1..yh3 and Phi rounded to BF16 (FP32 accumulation);
// otherwise FP32 operands through the 3xTF32 split
cudaError_t stpm_partial(int mode, const StpmPartialArgs& a, int grid, bool bf16, cudaStream_t s);
cudaError_t stpm_reduce(const StpmReduceArgs& a, cudaStream_t s);
// batched forms over `graphs` graphs of one padded size KP: args are device
// arrays indexed by graph; the contraction runs `grid` CTAs per graph (a
// multiple of stpm_partial_cluster(); each graph uses its args.nblocks of
// them), the step one cluster per graph (args.active == 0 skips a graph)
cudaError_t stpm_partial_batched(int mode, int KP, const StpmPartialArgs* args, int graphs,
                                 int grid, bool bf16, cudaStream_t s);
cudaError_t stpm_update_batched(int KP, const StpmUpdateArgs* args, int graphs, cudaStream_t s);
cudaError_t stpm_update(const StpmUpdateArgs& a, cudaStream_t s);
cudaError_t stpm_batch_update(int k, float* phi, const float* G, double* lambda, double* err,
                              cudaStream_t s);
// lambda_i = phi_i . G_i in FP64 (phi64: an FP64 copy of Phi to use for the
// dot product, may be null), sign fixed so lambda_i > 0 (both copies flipped)
cudaError_t stpm_tensor_values(int k, float* phi, const float* G, double* lambda, cudaStream_t s,
                               double* phi64 = nullptr);

}  // namespace mmsb
