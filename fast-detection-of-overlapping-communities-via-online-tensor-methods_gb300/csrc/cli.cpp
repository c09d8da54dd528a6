// Drop-in command line for the reference's driver
// (CommunityDetectionSoftware_CPU/CommunityDetection/CommunityDetection.cpp:16-149):
//
//   mmsb_cli NX NA NB NC KHID alpha0 DATATYPE Gx_a Gx_b Gx_c Gb_a Gc_a PI_OUT WHITE_OUT
//            [--method=batch|online|adjoint] [--sweeps=N] [--minibatch=N] [--seed=N]
//            [--tau=X] [--lambda-out=FILE] [--reader=compat|strict] [--device=N]
//            [--gpu-out=DIR]
//
// Same positional arguments and output files as the reference: PI_OUT gets the
// normalised memberships as 1-based "community<TAB>node<TAB>value" triplets of
// the nonzeros over the node order [X|A|B|C] and WHITE_OUT the whitening
// matrix (write_pi, IOfn.cpp:57-67).  The reference's own reader is
// reproduced by default (--reader=compat); a block file ending in ".csr" is
// read as this library's binary CSR container instead.  --gpu-out=DIR also
// writes the GPU tree's output files (Pi_X/A/B/C, evecs, evals, frob_norm,
// sim_info).  Errors print a message and exit with 1 (file) or 2 (device),
// like the reference's exit codes.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mmsb.h"

namespace {

int fail(const char* what, mmsb_status st, const mmsb_ctx* ctx) {
  std::fprintf(stderr, "%s failed: %s (%s)\n", what, mmsb_status_string(st),
               ctx ? mmsb_last_error(ctx) : "");
  return st == MMSB_ERR_IO ? 1 : 2;
}

bool opt(const char* arg, const char* name, std::string* value) {
  const size_t n = std::strlen(name);
  if (std::strncmp(arg, name, n) == 0 && arg[n] == '=') {
    *value = arg + n + 1;
    return true;
  }
  return false;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 15) {
    std::fprintf(stderr,
                 "usage: %s NX NA NB NC KHID alpha0 DATATYPE Gx_a Gx_b Gx_c Gb_a Gc_a PI_OUT "
                 "WHITE_OUT [--method=batch|online|adjoint] [--sweeps=N] [--minibatch=N] "
                 "[--seed=N] [--tau=X] [--lambda-out=FILE] [--reader=compat|strict] "
                 "[--device=N] [--gpu-out=DIR]\n",
                 argv[0]);
    return 1;
  }
  const int64_t n[4] = {std::atoll(argv[1]), std::atoll(argv[2]), std::atoll(argv[3]),
                        std::atoll(argv[4])};
  mmsb_config cfg;
  mmsb_config_default(&cfg);
  cfg.k = std::atoi(argv[5]);
  cfg.alpha0 = std::atof(argv[6]);
  cfg.datatype = std::atoi(argv[7]);
  const char* files[5] = {argv[8], argv[9], argv[10], argv[11], argv[12]};
  const char* pi_out = argv[13];
  const char* white_out = argv[14];
  std::string lambda_out, gpu_out;
  int compat = 1;
  for (int i = 15; i < argc; ++i) {
    std::string v;
    if (opt(argv[i], "--method", &v)) {
      cfg.stpm_method = v == "online" ? MMSB_STPM_ONLINE
                        : v == "adjoint" ? MMSB_STPM_ADJOINT
                                         : MMSB_STPM_BATCH_POWER;
    } else if (opt(argv[i], "--sweeps", &v)) {
      cfg.sweeps = std::atoi(v.c_str());
    } else if (opt(argv[i], "--minibatch", &v)) {
      cfg.minibatch = std::atoi(v.c_str());
    } else if (opt(argv[i], "--seed", &v)) {
      cfg.seed = std::strtoull(v.c_str(), nullptr, 10);
    } else if (opt(argv[i], "--tau", &v)) {
      cfg.tau = (float)std::atof(v.c_str());
    } else if (opt(argv[i], "--lambda-out", &v)) {
      lambda_out = v;
    } else if (opt(argv[i], "--reader", &v)) {
      compat = v != "strict";
    } else if (opt(argv[i], "--device", &v)) {
      cfg.device = std::atoi(v.c_str());
    } else if (opt(argv[i], "--gpu-out", &v)) {
      gpu_out = v;
    } else {
      std::fprintf(stderr, "unknown option %s\n", argv[i]);
      return 1;
    }
  }
  // blocks: rows x cols = X x A, X x B, X x C, B x A, C x A  (CommunityDetection.cpp:47-49,94-95)
  const int rows_part[5] = {0, 0, 0, 2, 3};
  const int cols_part[5] = {1, 2, 3, 1, 1};
  mmsb_host_graph* h[5] = {};
  mmsb_csr blocks[5];
  for (int b = 0; b < 5; ++b) {
    const size_t len = std::strlen(files[b]);
    const bool bin = len > 4 && std::strcmp(files[b] + len - 4, ".csr") == 0;
    mmsb_status st = bin ? mmsb_read_csr(files[b], &h[b])
                         : mmsb_read_coo(files[b], n[rows_part[b]], n[cols_part[b]], cfg.datatype,
                                         compat, &h[b]);
    if (st == MMSB_OK && bin) {
      mmsb_csr c;
      mmsb_host_graph_block(h[b], 0, &c);
      if (c.n_rows != n[rows_part[b]] || c.n_cols != n[cols_part[b]]) st = MMSB_ERR_IO;
    }
    if (st != MMSB_OK) {
      std::fprintf(stderr, "reading %s failed\n", files[b]);
      return 1;
    }
    mmsb_host_graph_block(h[b], 0, &blocks[b]);
  }
  mmsb_ctx* ctx = nullptr;
  mmsb_status st = mmsb_create(&cfg, &ctx);
  if (st != MMSB_OK) return fail("mmsb_create", st, nullptr);
  int rc = 0;
  if ((st = mmsb_upload_graph(ctx, blocks)) != MMSB_OK) rc = fail("upload", st, ctx);
  else if ((st = mmsb_whiten(ctx, nullptr)) != MMSB_OK) rc = fail("whitening", st, ctx);
  else if ((st = mmsb_stpm(ctx, nullptr)) != MMSB_OK) rc = fail("tensor decomposition", st, ctx);
  else if ((st = mmsb_postproc(ctx)) != MMSB_OK) rc = fail("post-processing", st, ctx);
  if (rc == 0) {
    const int64_t N = mmsb_num_nodes(ctx);
    std::vector<float> pi((size_t)cfg.k * N);
    std::vector<double> W((size_t)n[1] * cfg.k), lam(cfg.k);
    mmsb_get_pi(ctx, pi.data());
    mmsb_get_whitening(ctx, W.data(), nullptr, nullptr, nullptr, nullptr);
    mmsb_get_lambda(ctx, lam.data());
    if (mmsb_write_triplets_f32(pi_out, pi.data(), cfg.k, N) != MMSB_OK ||
        mmsb_write_triplets_f64(white_out, W.data(), n[1], cfg.k) != MMSB_OK) {
      std::fprintf(stderr, "writing results failed\n");
      rc = 1;
    }
    if (rc == 0 && !lambda_out.empty()) {
      FILE* f = std::fopen(lambda_out.c_str(), "w");
      if (!f) {
        rc = 1;
      } else {
        for (int i = 0; i < cfg.k; ++i) std::fprintf(f, "%.17g\n", lam[i]);
        std::fclose(f);
      }
    }
    if (rc == 0 && !gpu_out.empty() && mmsb_write_gpu_outputs(ctx, gpu_out.c_str()) != MMSB_OK) {
      std::fprintf(stderr, "writing the GPU-tree outputs to %s failed\n", gpu_out.c_str());
      rc = 1;
    }
    mmsb_stats s;
    mmsb_get_stats(ctx, &s);
    std::printf("whitening %.3f ms, tensor decomposition %.3f ms (%lld steps), post-processing "
                "%.3f ms\n",
                s.whiten_ms, s.stpm_ms, (long long)s.stpm_steps, s.post_ms);
  }
  mmsb_destroy(ctx);
  for (auto* g : h) mmsb_host_graph_free(g);
  return rc;
}
