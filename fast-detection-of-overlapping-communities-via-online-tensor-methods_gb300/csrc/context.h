// Context of one pipeline instance: configuration, stream, device-resident
// graph and results, and a grow-only workspace of named device buffers.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"
#include "mmsb.h"

struct DevCsr {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  int64_t* rp = nullptr;
  int32_t* ci = nullptr;
  float* val = nullptr;
};

struct mmsb_ctx {
  mmsb_config cfg{};
  cudaStream_t s = nullptr;
  // second stream: the two independent pseudo-inverse sides of the whitening
  cudaStream_t s2 = nullptr;
  cudaStream_t s3 = nullptr, s4 = nullptr;  // helpers of the two whitening sides
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  std::string err;
  std::atomic<bool> stop{false};
  mmsb_stats stats{};

  int64_t nX = 0, nA = 0, nB = 0, nC = 0;
  DevCsr g[MMSB_NUM_BLOCKS];   // as uploaded
  DevCsr gt[MMSB_NUM_BLOCKS];  // transposes
  bool have_graph = false, have_white = false, have_y = false, have_phi = false,
       have_post = false;

  int k = 0, p = 0, ldk = 0, ldp = 0;

  // device results
  float* W = nullptr;    // n_A x ldk   (row-major panel)
  float* Zb1 = nullptr;  // n_A x ldk
  float* Ub = nullptr;   // n_B x ldk   (Z_B_part2 = Ub^T)
  float* Zc1 = nullptr;  // n_A x ldk
  float* Uc = nullptr;   // n_C x ldk   (Z_C_part2 = Uc^T)
  double* mu = nullptr;  // mu_a | mu_b | mu_c (n_A + n_B + n_C)
  float* y[3] = {nullptr, nullptr, nullptr};  // n_X x ldk each
  void* yh[3] = {nullptr, nullptr, nullptr};  // BF16 copies, n_X x ldkh (BF16 form)
  int ldkh = 0;                               // round_up(k, 8)
  float* ymu = nullptr;                       // 3 x k (FP32)
  double* ymu64 = nullptr;                    // 3 x k
  float* phi = nullptr;                       // k x k column-major
  double* lambda = nullptr;                   // k
  float* pi = nullptr;                        // N x k
  uint32_t* bits = nullptr;                   // N x words
  unsigned* flags = nullptr;                  // device status word
  double* conv = nullptr;                     // convergence trace of the last mmsb_stpm
  int64_t conv_count = 0;
  double* dscalar = nullptr;                  // device scalars (errors, losses)

  std::map<std::string, std::pair<void*, size_t>> ws;
  cudaEvent_t ev[8] = {};
  // event pairs around whitening SpMM launches (roofline timing)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spmm_pool;
  std::vector<size_t> spmm_events;
  // event pairs around the STPM contraction (0) and step (1) launches
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> kpool[2];
  size_t kused[2] = {0, 0};
  int64_t klaunched[2] = {0, 0};  // launches since the last collect (timed or not)
  bool ksample = true;             // time the next STPM launches with events
  // clock64 cycles a bounded device wait of the STPM kernels may take
  // (0: about one second); mmsb_set_wait_limit
  long long wait_limit = 0;

  ~mmsb_ctx();
  // grow-only named workspace buffer of at least `bytes` bytes
  void* buf(const std::string& name, size_t bytes);
  template <typename T>
  T* tbuf(const std::string& name, size_t count) {
    return static_cast<T*>(buf(name, count * sizeof(T)));
  }
  void free_graph();
};
