// C ABI (include/mmsb.h).  Every entry point converts exceptions into a
// status code and records the message in the context; nothing exits.
#include <cmath>
#include <cstdio>
#include <string>
#include <algorithm>
#include <functional>
#include <cstring>
#include <memory>
#include <vector>

#include "mmsb.h"
#include "pipeline.h"

using namespace mmsb;

namespace {

thread_local std::string g_last_global_error;

template <typename F>
mmsb_status guard(mmsb_ctx* c, F&& f) {
  try {
    f();
    return MMSB_OK;
  } catch (const MmsbError& e) {
    if (c) c->err = e.what();
    g_last_global_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    if (c) c->err = "host allocation failed";
    g_last_global_error = "host allocation failed";
    return MMSB_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    if (c) c->err = e.what();
    g_last_global_error = e.what();
    return MMSB_ERR_CUDA;
  }
}

void timed(mmsb_ctx* c, double* out_ms, const std::function<void()>& body) {
  ck(cudaEventRecord(c->ev[0], c->s), "event");
  body();
  ck(cudaEventRecord(c->ev[1], c->s), "event");
  ck(cudaEventSynchronize(c->ev[1]), "event sync");
  float ms = 0.f;
  ck(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]), "elapsed");
  *out_ms = ms;
}

void d2h(mmsb_ctx* c, void* dst, const void* src, size_t bytes) {
  ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->s), "D2H");
}

// row-major FP32 panel (n x ld) -> column-major FP64 host (n x q) or its transpose
void panel_to_host(mmsb_ctx* c, const float* P, int ld, int64_t n, int q, double* out,
                   bool transpose) {
  std::vector<float> h((size_t)n * ld);
  d2h(c, h.data(), P, h.size() * sizeof(float));
  ck(cudaStreamSynchronize(c->s), "sync");
  for (int64_t r = 0; r < n; ++r)
    for (int j = 0; j < q; ++j) {
      const double v = h[(size_t)r * ld + j];
      if (transpose) out[(size_t)r * q + j] = v;  // q x n column-major
      else out[(size_t)j * n + r] = v;            // n x q column-major
    }
}

void host_to_panel(mmsb_ctx* c, const double* A, int64_t n, int q, bool transposed, float* P,
                   int ld) {
  std::vector<float> h((size_t)n * ld, 0.f);
  for (int64_t r = 0; r < n; ++r)
    for (int j = 0; j < q; ++j)
      h[(size_t)r * ld + j] = (float)(transposed ? A[(size_t)r * q + j] : A[(size_t)j * n + r]);
  ck(cudaMemcpyAsync(P, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->s), "H2D");
  ck(cudaStreamSynchronize(c->s), "sync");
}

}  // namespace

extern "C" {

void mmsb_config_default(mmsb_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->k = 10;
  cfg->alpha0 = 1.0;
  cfg->datatype = 0;
  cfg->stpm_method = MMSB_STPM_BATCH_POWER;
  cfg->precision = MMSB_PREC_FP32;
  cfg->sweeps = 10;
  cfg->minibatch = 100;
  cfg->lr0 = 1.0;
  // 1/2: the Phi term's weight 1 - 3 theta beta_t = 1 - 1.5 / (1 + t) of the
  // online step is -1/2, 1/4, 1/2, ... and never 0; at theta = 1 it is 0 at
  // t = 2, where the step becomes the bare minibatch gradient, singular
  // whenever the minibatch's whitened data miss a direction, with a QR
  // factor that is not unique.  (theta = 1/4 avoids the zero too, but on the
  // reference configuration its iterates have not settled after 10 sweeps:
  // BF16 rounding of y moved the FP64 oracle's lambda by 3e-2, against 3e-4
  // at theta = 1/2 and 1.)
  cfg->theta = 0.5;
  cfg->min_iter = 100;
  cfg->max_iter = 10000;
  cfg->tol = 1e-6;
  cfg->pinv_tol = 1e-6;
  cfg->nystrom_rows_factor = 20;
  cfg->normalize = 1;
  cfg->seed = 0;
  cfg->tau = 0.1f;
  cfg->device = 0;
}

const char* mmsb_status_string(mmsb_status st) {
  switch (st) {
    case MMSB_OK: return "ok";
    case MMSB_ERR_INVALID_ARG: return "invalid argument";
    case MMSB_ERR_CUDA: return "CUDA error";
    case MMSB_ERR_OUT_OF_MEMORY: return "out of memory";
    case MMSB_ERR_STATE: return "call out of order";
    case MMSB_ERR_NUMERICAL: return "numerical failure";
    case MMSB_ERR_STOPPED: return "stopped on request";
    case MMSB_ERR_IO: return "I/O error";
    case MMSB_ERR_TIMEOUT: return "device wait timed out";
    case MMSB_ERR_UNSUPPORTED: return "unsupported configuration";
  }
  return "unknown status";
}

mmsb_status mmsb_create(const mmsb_config* cfg, mmsb_ctx** out) {
  if (!cfg || !out) return MMSB_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->k < 1 || cfg->k > 256 || !(cfg->alpha0 >= 0) || cfg->sweeps < 0 || cfg->minibatch < 1 ||
      cfg->stpm_method < 0 || cfg->stpm_method > 2 || cfg->precision < 0 || cfg->precision > 1 ||
      cfg->nystrom_rows_factor < 1 || !(cfg->pinv_tol >= 0) || cfg->max_iter < 0)
    return MMSB_ERR_INVALID_ARG;
  std::unique_ptr<mmsb_ctx> c(new mmsb_ctx());
  mmsb_status st = guard(c.get(), [&]() {
    c->cfg = *cfg;
    ck(cudaSetDevice(cfg->device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&c->s3, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&c->s4, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming), "event");
    for (auto& e : c->ev) ck(cudaEventCreate(&e), "event");
    c->spmm_pool.resize(64);
    for (auto& pr : c->spmm_pool) {
      ck(cudaEventCreate(&pr.first), "event");
      ck(cudaEventCreate(&pr.second), "event");
    }
    c->k = cfg->k;
    c->p = 2 * cfg->k;
    c->ldk = (int)round_up(c->k, 4);
    c->ldp = (int)round_up(c->p, 4);
    c->flags = c->tbuf<unsigned>("flags", 4);
    c->dscalar = c->tbuf<double>("dscalar", 8);
    ck(cudaMemsetAsync(c->flags, 0, 16, c->s), "flags");
    ck(cudaStreamSynchronize(c->s), "sync");
  });
  if (st != MMSB_OK) return st;
  *out = c.release();
  return MMSB_OK;
}

void mmsb_destroy(mmsb_ctx* ctx) { delete ctx; }

mmsb_status mmsb_upload_graph(mmsb_ctx* c, const mmsb_csr blocks[MMSB_NUM_BLOCKS]) {
  if (!c || !blocks) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() { pipeline_upload(c, blocks); });
}

mmsb_status mmsb_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return MMSB_ERR_INVALID_ARG;
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e == cudaSuccess) return MMSB_OK;
  cudaGetLastError();
  return e == cudaErrorInvalidValue || e == cudaErrorHostMemoryAlreadyRegistered
             ? MMSB_ERR_INVALID_ARG
             : MMSB_ERR_CUDA;
}

mmsb_status mmsb_host_unregister(void* ptr) {
  if (!ptr) return MMSB_ERR_INVALID_ARG;
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e == cudaSuccess) return MMSB_OK;
  cudaGetLastError();
  return e == cudaErrorHostMemoryNotRegistered ? MMSB_ERR_INVALID_ARG : MMSB_ERR_CUDA;
}

mmsb_status mmsb_whiten(mmsb_ctx* c, const double* const* sketches) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    c->stats = mmsb_stats{};
    g_launch_count = 0;
    timed(c, &c->stats.whiten_ms, [&]() { pipeline_whiten(c, sketches); });
    c->stats.kernel_launches = g_launch_count;
  });
}

mmsb_status mmsb_stpm(mmsb_ctx* c, const double* phi0) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    c->stop.store(false);
    const int64_t l0 = g_launch_count;
    timed(c, &c->stats.stpm_ms, [&]() { pipeline_stpm(c, phi0); });
    c->stats.kernel_launches += g_launch_count - l0;
  });
}

mmsb_status mmsb_postproc(mmsb_ctx* c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    const int64_t l0 = g_launch_count;
    timed(c, &c->stats.post_ms, [&]() { pipeline_post(c); });
    c->stats.kernel_launches += g_launch_count - l0;
  });
}

mmsb_status mmsb_run(mmsb_ctx* c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    c->stats = mmsb_stats{};
    c->stop.store(false);
    g_launch_count = 0;
    double total = 0;
    timed(c, &total, [&]() {
      timed(c, &c->stats.whiten_ms, [&]() { pipeline_whiten(c, nullptr); });
      timed(c, &c->stats.stpm_ms, [&]() { pipeline_stpm(c, nullptr); });
      timed(c, &c->stats.post_ms, [&]() { pipeline_post(c); });
    });
    c->stats.total_ms = c->stats.whiten_ms + c->stats.stpm_ms + c->stats.post_ms;
    c->stats.kernel_launches = g_launch_count;
  });
}

int64_t mmsb_num_nodes(const mmsb_ctx* c) { return c ? c->nX + c->nA + c->nB + c->nC : 0; }

mmsb_status mmsb_get_pi(mmsb_ctx* c, float* pi) {
  if (!c || !pi) return MMSB_ERR_INVALID_ARG;
  if (!c->have_post) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    d2h(c, pi, c->pi, sizeof(float) * (size_t)mmsb_num_nodes(c) * c->k);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_pvalues(mmsb_ctx* c, const float* truth, int32_t k_true, double* corr,
                         double* tstat, double* pval) {
  if (!c || !truth || k_true < 1) return MMSB_ERR_INVALID_ARG;
  if (!c->have_post) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    const int k = c->k, K = k_true;
    const int64_t N = mmsb_num_nodes(c);
    if (N < 1) throw MmsbError(MMSB_ERR_STATE, "no nodes");
    cudaStream_t s = c->s;
    float* T = c->tbuf<float>("eval.truth", (size_t)N * K);
    ck(cudaMemcpyAsync(T, truth, sizeof(float) * (size_t)N * K, cudaMemcpyHostToDevice, s), "H2D truth");
    const int mx = std::max(k, K);
    double* part = c->tbuf<double>("eval.part", colstats_partials(N, mx));
    double* mean = c->tbuf<double>("eval.mean", (size_t)k + K);
    double* var = c->tbuf<double>("eval.var", (size_t)k + K);
    ck(column_stats(c->pi, k, k, N, part, mean, var, s), "stats");
    ck(column_stats(T, K, K, N, part, mean + k, var + k, s), "stats");
    float* Ac = c->tbuf<float>("eval.ac", (size_t)N * k);
    float* Bc = c->tbuf<float>("eval.bc", (size_t)N * K);
    ck(center_columns(c->pi, k, k, N, mean, Ac, s), "centre");
    ck(center_columns(T, K, K, N, mean + k, Bc, s), "centre");
    double* C = c->tbuf<double>("eval.c", (size_t)k * K);
    const int64_t cap = (int64_t)gram_tsk_partials(N, k, K);
    double* gp = c->tbuf<double>("eval.gram", (size_t)cap);
    ck(gram_tsk(Ac, k, k, Bc, K, K, N, 1.0, C, gp, cap, s), "cross products");
    double* out = c->tbuf<double>("eval.out", (size_t)3 * k * K);
    const size_t kk = (size_t)k * K;
    ck(pair_pvalues(C, k, K, N, var, var + k, out, out + kk, out + 2 * kk, c->flags, s), "p-values");
    if (corr) d2h(c, corr, out, sizeof(double) * kk);
    if (tstat) d2h(c, tstat, out + kk, sizeof(double) * kk);
    if (pval) d2h(c, pval, out + 2 * kk, sizeof(double) * kk);
    ck(cudaStreamSynchronize(s), "sync");
    check_device_flags(c, "p-values");
  });
}

mmsb_status mmsb_get_convergence(mmsb_ctx* c, double* out, int64_t cap, int64_t* count) {
  if (!c || (cap > 0 && !out)) return MMSB_ERR_INVALID_ARG;
  if (!c->have_phi) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    if (count) *count = c->conv_count;
    const int64_t n = std::min<int64_t>(std::max<int64_t>(cap, 0), c->conv_count);
    if (n > 0) d2h(c, out, c->conv, sizeof(double) * (size_t)n);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_write_gpu_outputs(mmsb_ctx* c, const char* dir) {
  if (!c || !dir) return MMSB_ERR_INVALID_ARG;
  if (!c->have_post) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    const int k = c->k;
    const int64_t N = mmsb_num_nodes(c);
    std::vector<float> pi((size_t)N * k), phi((size_t)k * k);
    std::vector<double> lam(k), conv((size_t)c->conv_count);
    d2h(c, phi.data(), c->phi, sizeof(float) * phi.size());
    d2h(c, lam.data(), c->lambda, sizeof(double) * k);
    if (!conv.empty()) d2h(c, conv.data(), c->conv, sizeof(double) * conv.size());
    ck(cudaStreamSynchronize(c->s), "sync");
    // Pi files hold the raw unwhitened memberships scaled by ||lambda||_2
    // (GPU/post_proc.c:86-114), not the normalised Pi of the CPU tree
    double lnorm = 0.0;
    for (int i = 0; i < k; ++i) lnorm += lam[i] * lam[i];
    lnorm = std::sqrt(lnorm);
    float* raw = c->tbuf<float>("pi_raw", (size_t)N * k);
    pipeline_post_raw(c, lnorm, raw);
    d2h(c, pi.data(), raw, sizeof(float) * pi.size());
    ck(cudaStreamSynchronize(c->s), "sync");
    // file names of GPU/stpm.h:82-91: <name>_<NCOM>_<ALPHA_0>_<LEARN_RATE>.txt
    char tail[96];
    std::snprintf(tail, sizeof(tail), "_%d_%g_%g.txt", k, c->cfg.alpha0, c->cfg.lr0);
    auto path = [&](const char* name) { return std::string(dir) + "/" + name + tail; };
    auto io = [&](mmsb_status st, const std::string& f) {
      if (st != MMSB_OK) throw MmsbError(MMSB_ERR_IO, "writing " + f);
    };
    // Pi_X, Pi_A, Pi_B, Pi_C: k x n_P column-major slices of Pi (write_mat,
    // GPU/post_proc.c:110-114)
    const char* names[4] = {"Pi_X", "Pi_A", "Pi_B", "Pi_C"};
    const int64_t part[4] = {c->nX, c->nA, c->nB, c->nC};
    int64_t off = 0;
    for (int q = 0; q < 4; ++q) {
      const std::string f = path(names[q]);
      io(mmsb_write_dense_f32(f.c_str(), pi.data() + off * k, part[q] * k), f);
      off += part[q];
    }
    // evecs: Phi column-major; evals: the Dirichlet weights
    // lambda_i^-2 / sum_j lambda_j^-2 (GPU/stpm.c:848-870)
    {
      const std::string f = path("evecs");
      io(mmsb_write_dense_f32(f.c_str(), phi.data(), (int64_t)k * k), f);
    }
    std::vector<double> alpha(k);
    double sum = 0.0;
    for (int i = 0; i < k; ++i) {
      alpha[i] = 1.0 / (lam[i] * lam[i]);
      sum += alpha[i];
    }
    for (int i = 0; i < k; ++i) alpha[i] /= sum;
    {
      const std::string f = path("evals");
      io(mmsb_write_dense_f64(f.c_str(), alpha.data(), k), f);
    }
    {
      const std::string f = path("frob_norm");
      io(mmsb_write_dense_f64(f.c_str(), conv.data(), (int64_t)conv.size()), f);
    }
    // sim_info (GPU/stpm.c:944-963), times in seconds of this library's stages
    const std::string f = path("sim_info");
    FILE* fp = std::fopen(f.c_str(), "w");
    if (!fp) throw MmsbError(MMSB_ERR_IO, "writing " + f);
    const bool online = c->cfg.stpm_method != MMSB_STPM_BATCH_POWER;
    const int64_t per = online ? std::max<int64_t>(1, c->stats.stpm_steps / std::max(1, c->cfg.sweeps)) : 1;
    const double pre = c->stats.whiten_ms / 1e3, stpm = c->stats.stpm_ms / 1e3, post = c->stats.post_ms / 1e3;
    std::fprintf(fp, "Total number of nodes          = %d\n", (int)N);
    std::fprintf(fp, "Number of nodes in partition X = %d\n", (int)c->nX);
    std::fprintf(fp, "Number of nodes in partition A = %d\n", (int)c->nA);
    std::fprintf(fp, "Number of nodes in partition B = %d\n", (int)c->nB);
    std::fprintf(fp, "Number of nodes in partition C = %d\n", (int)c->nC);
    std::fprintf(fp, "Number of nodes communities    = %d\n", k);
    std::fprintf(fp, "Alpha_0 (Dirichlet parameter)  = %5.25e\n", c->cfg.alpha0);
    std::fprintf(fp, "Learning rate = %5.25e\n", c->cfg.lr0);
    std::fprintf(fp, "Threshold for STPM convergence    = %5.25e\n", c->cfg.tol);
    std::fprintf(fp, "Pseudoinverse numerical tolerance = %5.25e\n", c->cfg.pinv_tol);
    std::fprintf(fp, "Total number of Frob Norm values written to file = %d\n", (int)conv.size());
    std::fprintf(fp, "Number of iterations between convergence test    = %d\n", (int)per);
    std::fprintf(fp, "Maximum number of stochastic iterations allowed  = %d\n",
                 (int)(online ? c->stats.stpm_steps : c->cfg.max_iter));
    std::fprintf(fp, "Exec Time Pre Proc  = %5.25e (Seconds)\n", pre);
    std::fprintf(fp, "Exec Time STPM      = %5.25e (Seconds)\n", stpm);
    std::fprintf(fp, "Exec Time Post Proc = %5.25e (Seconds)\n", post);
    std::fprintf(fp, "Total Exec Time     = %5.25e (Seconds)\n", pre + stpm + post);
    if (std::fclose(fp) != 0) throw MmsbError(MMSB_ERR_IO, "writing " + f);
  });
}

mmsb_status mmsb_get_sets(mmsb_ctx* c, uint32_t* bits) {
  if (!c || !bits) return MMSB_ERR_INVALID_ARG;
  if (!c->have_post) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    d2h(c, bits, c->bits, sizeof(uint32_t) * (size_t)mmsb_num_nodes(c) * ((c->k + 31) / 32));
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_get_lambda(mmsb_ctx* c, double* lambda) {
  if (!c || !lambda) return MMSB_ERR_INVALID_ARG;
  if (!c->have_phi) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    d2h(c, lambda, c->lambda, sizeof(double) * c->k);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_get_phi(mmsb_ctx* c, double* phi) {
  if (!c || !phi) return MMSB_ERR_INVALID_ARG;
  if (!c->have_phi) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    std::vector<float> h((size_t)c->k * c->k);
    d2h(c, h.data(), c->phi, h.size() * sizeof(float));
    ck(cudaStreamSynchronize(c->s), "sync");
    for (size_t i = 0; i < h.size(); ++i) phi[i] = h[i];
  });
}

mmsb_status mmsb_get_whitening(mmsb_ctx* c, double* W, double* zb1, double* zb2, double* zc1,
                               double* zc2) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  if (!c->have_white) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    if (W) panel_to_host(c, c->W, c->ldk, c->nA, c->k, W, false);
    if (zb1) panel_to_host(c, c->Zb1, c->ldk, c->nA, c->k, zb1, false);
    if (zb2) panel_to_host(c, c->Ub, c->ldk, c->nB, c->k, zb2, true);
    if (zc1) panel_to_host(c, c->Zc1, c->ldk, c->nA, c->k, zc1, false);
    if (zc2) panel_to_host(c, c->Uc, c->ldk, c->nC, c->k, zc2, true);
  });
}

mmsb_status mmsb_get_means(mmsb_ctx* c, double* mu_a, double* mu_b, double* mu_c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  if (!c->have_white) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    if (mu_a) d2h(c, mu_a, c->mu, sizeof(double) * c->nA);
    if (mu_b) d2h(c, mu_b, c->mu + c->nA, sizeof(double) * c->nB);
    if (mu_c) d2h(c, mu_c, c->mu + c->nA + c->nB, sizeof(double) * c->nC);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_get_whitened(mmsb_ctx* c, float* ya, float* yb, float* yc, double* ymu_a,
                              double* ymu_b, double* ymu_c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  if (!c->have_y) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    float* outs[3] = {ya, yb, yc};
    std::vector<float> h((size_t)c->nX * c->ldk);
    for (int q = 0; q < 3; ++q) {
      if (!outs[q]) continue;
      d2h(c, h.data(), c->y[q], h.size() * sizeof(float));
      ck(cudaStreamSynchronize(c->s), "sync");
      for (int64_t x = 0; x < c->nX; ++x)
        std::memcpy(outs[q] + x * c->k, h.data() + x * c->ldk, sizeof(float) * c->k);
    }
    std::vector<float> m(3 * (size_t)c->k);
    d2h(c, m.data(), c->ymu, m.size() * sizeof(float));
    std::vector<double> m64(3 * (size_t)c->k);
    d2h(c, m64.data(), c->ymu64, m64.size() * sizeof(double));
    ck(cudaStreamSynchronize(c->s), "sync");
    double* mo[3] = {ymu_a, ymu_b, ymu_c};
    for (int q = 0; q < 3; ++q)
      if (mo[q])
        for (int i = 0; i < c->k; ++i) mo[q][i] = m64[(size_t)q * c->k + i];
  });
}

mmsb_status mmsb_get_stats(const mmsb_ctx* c, mmsb_stats* out) {
  if (!c || !out) return MMSB_ERR_INVALID_ARG;
  *out = c->stats;
  return MMSB_OK;
}

mmsb_status mmsb_set_whitening(mmsb_ctx* c, const double* W, const double* zb1, const double* zb2,
                               const double* zc1, const double* zc2, const double* mu_a,
                               const double* mu_b, const double* mu_c) {
  if (!c || !W || !zb1 || !zb2 || !zc1 || !zc2 || !mu_a || !mu_b || !mu_c)
    return MMSB_ERR_INVALID_ARG;
  if (!c->have_graph) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    const int k = c->k, ldk = c->ldk;
    c->W = c->tbuf<float>("W", (size_t)c->nA * ldk);
    c->Zb1 = c->tbuf<float>("Zb1", (size_t)c->nA * ldk);
    c->Zc1 = c->tbuf<float>("Zc1", (size_t)c->nA * ldk);
    c->Ub = c->tbuf<float>("Ub", (size_t)c->nB * ldk);
    c->Uc = c->tbuf<float>("Uc", (size_t)c->nC * ldk);
    c->mu = c->tbuf<double>("mu", (size_t)(c->nA + c->nB + c->nC));
    for (int q = 0; q < 3; ++q) c->y[q] = c->tbuf<float>("y" + std::to_string(q), (size_t)c->nX * ldk);
    c->ymu = c->tbuf<float>("ymu", 3 * (size_t)k);
    c->ymu64 = c->tbuf<double>("ymu64", 3 * (size_t)k);
    c->phi = c->tbuf<float>("phi", (size_t)k * k);
    c->lambda = c->tbuf<double>("lambda", (size_t)k);
    host_to_panel(c, W, c->nA, k, false, c->W, ldk);
    host_to_panel(c, zb1, c->nA, k, false, c->Zb1, ldk);
    host_to_panel(c, zc1, c->nA, k, false, c->Zc1, ldk);
    host_to_panel(c, zb2, c->nB, k, true, c->Ub, ldk);
    host_to_panel(c, zc2, c->nC, k, true, c->Uc, ldk);
    ck(cudaMemcpyAsync(c->mu, mu_a, sizeof(double) * c->nA, cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaMemcpyAsync(c->mu + c->nA, mu_b, sizeof(double) * c->nB, cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaMemcpyAsync(c->mu + c->nA + c->nB, mu_c, sizeof(double) * c->nC, cudaMemcpyHostToDevice, c->s), "H2D");
    c->have_white = true;
    pipeline_ydata(c);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

mmsb_status mmsb_set_whitened(mmsb_ctx* c, const double* ya, const double* yb, const double* yc,
                              const double* ymu_a, const double* ymu_b, const double* ymu_c) {
  if (!c || !ya || !yb || !yc || !ymu_a || !ymu_b || !ymu_c) return MMSB_ERR_INVALID_ARG;
  if (!c->have_graph) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    const int k = c->k, ldk = c->ldk;
    const double* ys[3] = {ya, yb, yc};
    for (int q = 0; q < 3; ++q) {
      c->y[q] = c->tbuf<float>("y" + std::to_string(q), (size_t)c->nX * ldk);
      host_to_panel(c, ys[q], c->nX, k, true, c->y[q], ldk);  // k x n_X column-major = n_X rows
    }
    c->ymu = c->tbuf<float>("ymu", 3 * (size_t)k);
    c->ymu64 = c->tbuf<double>("ymu64", 3 * (size_t)k);
    c->phi = c->tbuf<float>("phi", (size_t)k * k);
    c->lambda = c->tbuf<double>("lambda", (size_t)k);
    std::vector<double> m(3 * (size_t)k);
    std::vector<float> m32(3 * (size_t)k);
    std::memcpy(m.data(), ymu_a, sizeof(double) * k);
    std::memcpy(m.data() + k, ymu_b, sizeof(double) * k);
    std::memcpy(m.data() + 2 * k, ymu_c, sizeof(double) * k);
    for (size_t i = 0; i < m.size(); ++i) m32[i] = (float)m[i];
    ck(cudaMemcpyAsync(c->ymu64, m.data(), m.size() * sizeof(double), cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaMemcpyAsync(c->ymu, m32.data(), m32.size() * sizeof(float), cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaStreamSynchronize(c->s), "sync");
    c->have_y = true;
  });
}

mmsb_status mmsb_set_phi_lambda(mmsb_ctx* c, const double* phi, const double* lambda) {
  if (!c || !phi || !lambda) return MMSB_ERR_INVALID_ARG;
  if (!c->have_white) return MMSB_ERR_STATE;
  return guard(c, [&]() {
    const int k = c->k;
    c->phi = c->tbuf<float>("phi", (size_t)k * k);
    c->lambda = c->tbuf<double>("lambda", (size_t)k);
    std::vector<float> h((size_t)k * k);
    for (size_t i = 0; i < h.size(); ++i) h[i] = (float)phi[i];
    ck(cudaMemcpyAsync(c->phi, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaMemcpyAsync(c->lambda, lambda, sizeof(double) * k, cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaStreamSynchronize(c->s), "sync");
    c->have_phi = true;
  });
}

mmsb_status mmsb_stpm_loss_fwd(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count,
                               double* loss) {
  if (!c || !phi || !loss) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() { *loss = pipeline_loss(c, phi, begin, count); });
}

mmsb_status mmsb_stpm_loss_bwd(mmsb_ctx* c, const double* phi, int64_t begin, int64_t count,
                               double* dphi) {
  if (!c || !phi || !dphi) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() { pipeline_loss_grad(c, phi, begin, count, dphi); });
}

void mmsb_request_stop(mmsb_ctx* c) {
  if (c) c->stop.store(true);
}

const char* mmsb_last_error(const mmsb_ctx* c) {
  return c ? c->err.c_str() : g_last_global_error.c_str();
}

mmsb_status mmsb_flush_l2(mmsb_ctx* c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    const size_t bytes = (size_t)256 << 20;
    float* f = c->tbuf<float>("l2_flush", bytes / sizeof(float));
    ck(fill_f32(f, (int64_t)(bytes / sizeof(float)), 1.f, c->s), "flush");
  });
}

mmsb_status mmsb_set_wait_limit(mmsb_ctx* c, int64_t cycles) {
  if (!c || cycles < 0) return MMSB_ERR_INVALID_ARG;
  c->wait_limit = (long long)cycles;
  return MMSB_OK;
}

mmsb_status mmsb_diag_wait_timeout(mmsb_ctx* c, int64_t cycles) {
  if (!c || cycles < 1 || cycles > 2000000000LL) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() {
    ck(wait_probe(c->flags, (long long)cycles, c->s), "wait probe");
    check_device_flags(c, "wait probe");
  });
}

mmsb_status mmsb_synchronize(mmsb_ctx* c) {
  if (!c) return MMSB_ERR_INVALID_ARG;
  return guard(c, [&]() { ck(cudaStreamSynchronize(c->s), "sync"); });
}

// ---- single operators ------------------------------------------------------

mmsb_status mmsb_op_spmm(const mmsb_csr* g, int transpose, const float* P, int64_t p, float alpha,
                         float* Y) {
  if (!g || !P || !Y || p < 1 || p > 4096) return MMSB_ERR_INVALID_ARG;
  mmsb_config cfg;
  mmsb_config_default(&cfg);
  mmsb_ctx* c = nullptr;
  mmsb_status st = mmsb_create(&cfg, &c);
  if (st != MMSB_OK) return st;
  std::unique_ptr<mmsb_ctx> own(c);
  return guard(c, [&]() {
    const int ld = (int)round_up(p, 4);
    const int64_t n_in = transpose ? g->n_rows : g->n_cols;
    const int64_t n_out = transpose ? g->n_cols : g->n_rows;
    DevCsr d;
    d.n_rows = g->n_rows;
    d.n_cols = g->n_cols;
    d.nnz = g->nnz;
    d.rp = c->tbuf<int64_t>("rp", g->n_rows + 1);
    d.ci = c->tbuf<int32_t>("ci", g->nnz);
    d.val = g->val ? c->tbuf<float>("val", g->nnz) : nullptr;
    ck(cudaMemcpyAsync(d.rp, g->row_ptr, sizeof(int64_t) * (g->n_rows + 1), cudaMemcpyHostToDevice, c->s), "H2D");
    if (g->nnz) ck(cudaMemcpyAsync(d.ci, g->col_idx, sizeof(int32_t) * g->nnz, cudaMemcpyHostToDevice, c->s), "H2D");
    if (g->val) ck(cudaMemcpyAsync(d.val, g->val, sizeof(float) * g->nnz, cudaMemcpyHostToDevice, c->s), "H2D");
    DevCsr use = d;
    if (transpose) {
      use.n_rows = g->n_cols;
      use.n_cols = g->n_rows;
      use.rp = c->tbuf<int64_t>("rpT", g->n_cols + 1);
      use.ci = c->tbuf<int32_t>("ciT", g->nnz);
      use.val = g->val ? c->tbuf<float>("valT", g->nnz) : nullptr;
      int32_t* scratch = c->tbuf<int32_t>("scratch", 2 * (g->n_cols + 1) + 2 * g->nnz + 2);
      ck(csr_transpose(d.rp, d.ci, d.val, d.n_rows, d.n_cols, d.nnz, use.rp, use.ci, use.val, scratch, c->s), "transpose");
    }
    std::vector<float> hp((size_t)n_in * ld, 0.f), hy((size_t)n_out * ld);
    for (int64_t r = 0; r < n_in; ++r) std::memcpy(&hp[(size_t)r * ld], P + r * p, sizeof(float) * p);
    float* dP = c->tbuf<float>("P", hp.size());
    float* dY = c->tbuf<float>("Y", hy.size());
    ck(cudaMemcpyAsync(dP, hp.data(), hp.size() * sizeof(float), cudaMemcpyHostToDevice, c->s), "H2D");
    ck(spmm_f32(use.rp, use.ci, use.val, use.n_rows, dP, ld, alpha, dY, c->s), "spmm");
    d2h(c, hy.data(), dY, hy.size() * sizeof(float));
    ck(cudaStreamSynchronize(c->s), "sync");
    for (int64_t r = 0; r < n_out; ++r) std::memcpy(Y + r * p, &hy[(size_t)r * ld], sizeof(float) * p);
  });
}

mmsb_status mmsb_op_gram(const float* A, int64_t n, int32_t pa, const float* B, int32_t pb,
                         double alpha, double* S) {
  if (!A || !B || !S || n < 1 || pa < 1 || pb < 1 || pa > 4096 || pb > 4096)
    return MMSB_ERR_INVALID_ARG;
  mmsb_config cfg;
  mmsb_config_default(&cfg);
  mmsb_ctx* c = nullptr;
  mmsb_status st = mmsb_create(&cfg, &c);
  if (st != MMSB_OK) return st;
  std::unique_ptr<mmsb_ctx> own(c);
  return guard(c, [&]() {
    float* dA = c->tbuf<float>("A", (size_t)n * pa);
    float* dB = c->tbuf<float>("B", (size_t)n * pb);
    double* dS = c->tbuf<double>("S", (size_t)pa * pb);
    const int64_t cap = (int64_t)gram_tsk_partials(n, pa, pb);
    double* part = c->tbuf<double>("part", (size_t)cap);
    ck(cudaMemcpyAsync(dA, A, sizeof(float) * n * pa, cudaMemcpyHostToDevice, c->s), "H2D");
    ck(cudaMemcpyAsync(dB, B, sizeof(float) * n * pb, cudaMemcpyHostToDevice, c->s), "H2D");
    ck(gram_tsk(dA, pa, pa, dB, pb, pb, n, alpha, dS, part, cap, c->s, c->flags), "gram");
    d2h(c, S, dS, sizeof(double) * pa * pb);
    ck(cudaStreamSynchronize(c->s), "sync");
    check_device_flags(c, "gram");
  });
}

mmsb_status mmsb_op_symeig(const double* A, int32_t n, double* evals, double* evecs) {
  if (!A || !evals || !evecs || n < 1 || n > 512) return MMSB_ERR_INVALID_ARG;
  mmsb_config cfg;
  mmsb_config_default(&cfg);
  mmsb_ctx* c = nullptr;
  mmsb_status st = mmsb_create(&cfg, &c);
  if (st != MMSB_OK) return st;
  std::unique_ptr<mmsb_ctx> own(c);
  return guard(c, [&]() {
    double* dA = c->tbuf<double>("A", (size_t)n * n);
    double* ev = c->tbuf<double>("ev", (size_t)n);
    double* V = c->tbuf<double>("V", (size_t)n * n);
    ck(cudaMemcpyAsync(dA, A, sizeof(double) * n * n, cudaMemcpyHostToDevice, c->s), "H2D");
    sym_eig_refined(c, "op", n, dA, ev, V);
    d2h(c, evals, ev, sizeof(double) * n);
    d2h(c, evecs, V, sizeof(double) * n * n);
    ck(cudaStreamSynchronize(c->s), "sync");
  });
}

}  // extern "C"
