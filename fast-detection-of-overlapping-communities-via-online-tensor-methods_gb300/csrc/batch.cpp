// Batched solver: many independent graphs of uneven size and k.
//
// Whitening: every graph has its own context (streams, workspace); a pool of
// host threads queues the graphs' whitening chains, whose small latency-bound
// kernels then run concurrently across the GPU.
// STPM: the online / adjoint minibatch updates of all graphs advance together
// in rounds.  Graphs are grouped by padded size KP; per round and group one
// launch of the contraction covers every graph of the group (blockIdx.y =
// graph, its own node range, CTAs and partial buffer) and one launch of the
// step kernel gives each graph its own cluster.  Graphs whose schedule is
// shorter sit out the remaining rounds.  The whole round loop is captured
// once in a CUDA graph and replayed by later runs.  The contraction's CTAs
// per graph are chosen per group by timing candidate counts on the first run
// (the autotuner).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "pipeline.h"

using namespace mmsb;

namespace {

constexpr int kMaxBuckets = 8;

struct Bucket {
  int KP = 0;
  int mode = kModePlain;
  std::vector<int> graphs;  // indices into mmsb_batch::g
  int ctas = 0;             // tuned contraction CTAs per graph (multiple of 8)
  // device argument arrays: contraction [round][precision][slot], step [round][slot]
  StpmPartialArgs* d_pargs = nullptr;
  StpmUpdateArgs* d_uargs = nullptr;
  size_t pcap = 0, ucap = 0;  // capacities (elements) of the argument arrays
  std::vector<uint8_t> has_prec[2];  // per round: some graph uses this precision
};

template <typename F>
void parallel_for(int n, int threads, int device, F&& f) {
  std::vector<std::thread> pool;
  std::mutex m;
  std::exception_ptr err;
  const int T = std::max(1, std::min(threads, n));
  for (int t = 0; t < T; ++t)
    pool.emplace_back([&, t]() {
      try {
        ck(cudaSetDevice(device), "cudaSetDevice");
        for (int i = t; i < n; i += T) f(i);
      } catch (...) {
        std::lock_guard<std::mutex> lock(m);
        if (!err) err = std::current_exception();
      }
    });
  for (auto& th : pool) th.join();
  if (err) std::rethrow_exception(err);
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t lo = (size_t)std::floor(pos), hi = std::min(v.size() - 1, lo + 1);
  return v[lo] + (v[hi] - v[lo]) * (pos - (double)lo);
}

}  // namespace

struct mmsb_batch {
  mmsb_config base{};
  std::vector<mmsb_ctx*> g;
  std::vector<cudaEvent_t> ready_ev, done_ev;
  cudaStream_t bs = nullptr;
  cudaEvent_t start_ev = nullptr, stpm_ev = nullptr;
  std::vector<Bucket> buckets;
  int64_t rounds = 0;
  bool planned = false;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_launches = 0;
  int fixed_ctas = 0;  // 0: autotune the contraction CTAs per graph
  mmsb_batch_stats stats{};
  std::vector<double> latency;
  std::string err;

  ~mmsb_batch() {
    if (bs) cudaStreamSynchronize(bs);
    if (exec) cudaGraphExecDestroy(exec);
    for (auto& b : buckets) {
      cudaFree(b.d_pargs);
      cudaFree(b.d_uargs);
    }
    for (auto e : ready_ev) cudaEventDestroy(e);
    for (auto e : done_ev) cudaEventDestroy(e);
    if (start_ev) cudaEventDestroy(start_ev);
    if (stpm_ev) cudaEventDestroy(stpm_ev);
    for (auto* c : g) mmsb_destroy(c);
    if (bs) cudaStreamDestroy(bs);
  }
};

namespace {

// partial buffer of graph c for up to `ctas` contraction CTAs
float* batch_gpart(mmsb_ctx* c, int ctas, int64_t* stride) {
  *stride = (int64_t)c->k * c->k + 3 * c->k + 4;
  return c->tbuf<float>("gpart_batch", (size_t)(ctas / stpm_partial_cluster()) * (size_t)*stride);
}

// writes the argument arrays of bucket b for contraction CTA cap `ctas`
void fill_args(mmsb_batch* B, Bucket& b, int ctas, int64_t rounds) {
  const size_t G = b.graphs.size();
  std::vector<StpmPartialArgs> pa((size_t)rounds * 2 * G);
  std::vector<StpmUpdateArgs> ua((size_t)rounds * G);
  b.has_prec[0].assign((size_t)rounds, 0);
  b.has_prec[1].assign((size_t)rounds, 0);
  for (size_t slot = 0; slot < G; ++slot) {
    mmsb_ctx* c = B->g[(size_t)b.graphs[slot]];
    int64_t stride = 0;
    float* gp = batch_gpart(c, ctas, &stride);
    OnlineRound rd;
    for (int64_t r = 0; r < rounds; ++r) {
      StpmPartialArgs* p = &pa[((size_t)r * 2) * G + slot];
      StpmUpdateArgs& u = ua[(size_t)r * G + slot];
      // inactive defaults: no nodes, no update
      p[0] = StpmPartialArgs{};
      p[G] = StpmPartialArgs{};
      u = StpmUpdateArgs{};
      if (!stpm_online_round(c, r, &rd)) continue;
      const int need = stpm_partial_grid(rd.cnt, rd.bf16);
      const int nb = std::min(ctas, need);
      p[rd.bf16 ? G : 0] =
          stpm_partial_args(c, 0, 1, 2, rd.x0, rd.cnt, rd.c0, rd.c2, rd.bf16, gp, stride, nb);
      // rounds after the first read the operand image of Phi that the
      // graph's previous step wrote (plain FP32 tensor-core form)
      if (r > 0 && rd.mode == kModePlain && !rd.bf16) p[0].phi_img = stpm_phi_image(c);
      b.has_prec[rd.bf16 ? 1 : 0][(size_t)r] = 1;
      u = stpm_online_update_args(c, rd, gp, stride, nb / stpm_partial_cluster());
      u.active = 1;
    }
  }
  if (pa.size() > b.pcap) {
    ck(cudaFree(b.d_pargs), "batch args");
    b.d_pargs = nullptr;
    ck(cudaMalloc(&b.d_pargs, sizeof(StpmPartialArgs) * pa.size()), "batch args");
    b.pcap = pa.size();
  }
  if (ua.size() > b.ucap) {
    ck(cudaFree(b.d_uargs), "batch args");
    b.d_uargs = nullptr;
    ck(cudaMalloc(&b.d_uargs, sizeof(StpmUpdateArgs) * ua.size()), "batch args");
    b.ucap = ua.size();
  }
  ck(cudaMemcpy(b.d_pargs, pa.data(), sizeof(StpmPartialArgs) * pa.size(), cudaMemcpyHostToDevice),
     "batch args");
  ck(cudaMemcpy(b.d_uargs, ua.data(), sizeof(StpmUpdateArgs) * ua.size(), cudaMemcpyHostToDevice),
     "batch args");
}

// one round of one bucket: contraction launch(es), then the step launch
void launch_round(mmsb_batch* B, Bucket& b, int64_t r) {
  const int G = (int)b.graphs.size();
  for (int prec = 0; prec < 2; ++prec) {
    if (!b.has_prec[prec][(size_t)r]) continue;
    ck(stpm_partial_batched(b.mode, b.KP, b.d_pargs + ((size_t)r * 2 + prec) * G, G, b.ctas,
                            prec == 1, B->bs), "batched contraction");
    ++B->graph_launches;
  }
  ck(stpm_update_batched(b.KP, b.d_uargs + (size_t)r * G, G, B->bs), "batched step");
  ++B->graph_launches;
}

// contraction CTAs per graph for bucket b: the candidate with the shortest
// first-round contraction (median of three timed launches each)
void autotune(mmsb_batch* B, Bucket& b) {
  int need = 8;
  OnlineRound rd;
  for (int gi : b.graphs)
    if (stpm_online_round(B->g[(size_t)gi], 0, &rd)) need = std::max(need, stpm_partial_grid(rd.cnt, rd.bf16));
  std::vector<int> cand;
  for (int c = 8; c < need; c *= 2) cand.push_back(c);
  cand.push_back(need);
  if (cand.size() == 1) {
    b.ctas = need;
    return;
  }
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  double best = 1e30;
  for (int c : cand) {
    fill_args(B, b, c, 1);
    const int prec = b.has_prec[1][0] ? 1 : 0;
    std::vector<float> t;
    for (int rep = 0; rep < 4; ++rep) {
      ck(cudaEventRecord(e0, B->bs), "event");
      ck(stpm_partial_batched(b.mode, b.KP, b.d_pargs + (size_t)prec * b.graphs.size(),
                              (int)b.graphs.size(), c, prec == 1, B->bs), "tune");
      ck(cudaEventRecord(e1, B->bs), "event");
      ck(cudaEventSynchronize(e1), "event sync");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
      if (rep > 0) t.push_back(ms);  // first launch warms up
    }
    std::sort(t.begin(), t.end());
    if (t[1] < best) {
      best = t[1];
      b.ctas = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the tuning launches wrote partial buffers sized for up to `need` CTAs
  for (int gi : b.graphs) {
    int64_t stride;
    batch_gpart(B->g[(size_t)gi], need, &stride);
  }
}

void plan(mmsb_batch* B) {
  std::map<int, std::vector<int>> by_kp;
  B->rounds = 0;
  for (size_t i = 0; i < B->g.size(); ++i) {
    by_kp[stpm_kp(B->g[i]->k)].push_back((int)i);
    B->rounds = std::max(B->rounds, stpm_online_rounds(B->g[i]));
  }
  if (by_kp.size() > (size_t)kMaxBuckets)
    throw MmsbError(MMSB_ERR_UNSUPPORTED, "too many distinct padded sizes in one batch");
  const int mode = B->base.stpm_method == MMSB_STPM_ADJOINT ? kModeAdjoint : kModePlain;
  for (auto& kv : by_kp) {
    Bucket b;
    b.KP = kv.first;
    b.mode = mode;
    b.graphs = kv.second;
    B->buckets.push_back(std::move(b));
  }
  for (auto& b : B->buckets) {
    if (B->fixed_ctas > 0)
      b.ctas = B->fixed_ctas;
    else
      autotune(B, b);
    // partial buffers at their final size before the arguments point at them
    for (int gi : b.graphs) {
      int64_t stride;
      batch_gpart(B->g[(size_t)gi], b.ctas, &stride);
    }
    fill_args(B, b, b.ctas, B->rounds);
  }
  ck(cudaStreamSynchronize(B->bs), "sync");
  B->planned = true;
}

void run_rounds(mmsb_batch* B) {
  for (int64_t r = 0; r < B->rounds; ++r)
    for (auto& b : B->buckets) launch_round(B, b, r);
}

void batch_run(mmsb_batch* B) {
  const auto t0 = std::chrono::steady_clock::now();
  const int G = (int)B->g.size();
  for (auto* c : B->g)
    if (!c->have_graph) throw MmsbError(MMSB_ERR_STATE, "batch run before every graph is uploaded");
  ck(cudaEventRecord(B->start_ev, B->bs), "event");
  for (auto* c : B->g) ck(cudaStreamWaitEvent(c->s, B->start_ev, 0), "wait");
  // whitening and Phi0 of every graph, queued from a pool of host threads
  parallel_for(G, 16, B->base.device, [&](int i) {
    mmsb_ctx* c = B->g[(size_t)i];
    c->stats = mmsb_stats{};
    pipeline_whiten(c, nullptr, false);
    stpm_prepare(c, nullptr);
    ck(cudaEventRecord(B->ready_ev[(size_t)i], c->s), "event");
  });
  for (int i = 0; i < G; ++i) ck(cudaStreamWaitEvent(B->bs, B->ready_ev[(size_t)i], 0), "wait");
  // batched STPM rounds: planned (and tuned) once, replayed as a CUDA graph
  if (!B->planned) plan(B);
  B->graph_launches = 0;
  if (B->exec) {
    ck(cudaGraphLaunch(B->exec, B->bs), "graph launch");
    for (int64_t r = 0; r < B->rounds; ++r)
      for (auto& b : B->buckets) B->graph_launches += 1 + b.has_prec[0][(size_t)r] + b.has_prec[1][(size_t)r];
    B->stats.graph_replayed = 1;
  } else {
    run_rounds(B);
    B->stats.graph_replayed = 0;
    // capture the same launches for the next runs
    cudaGraph_t graph = nullptr;
    const int64_t launches = B->graph_launches;
    ck(cudaStreamSynchronize(B->bs), "sync");
    ck(cudaStreamBeginCapture(B->bs, cudaStreamCaptureModeThreadLocal), "capture");
    run_rounds(B);
    ck(cudaStreamEndCapture(B->bs, &graph), "capture");
    ck(cudaGraphInstantiate(&B->exec, graph, 0), "instantiate");
    cudaGraphDestroy(graph);
    B->graph_launches = launches;
  }
  ck(cudaEventRecord(B->stpm_ev, B->bs), "event");
  // lambda and unwhitening per graph
  for (int i = 0; i < G; ++i) {
    mmsb_ctx* c = B->g[(size_t)i];
    ck(cudaStreamWaitEvent(c->s, B->stpm_ev, 0), "wait");
    stpm_lambda_pass(c);
    c->have_phi = true;
    pipeline_post(c);
    ck(cudaEventRecord(B->done_ev[(size_t)i], c->s), "event");
  }
  B->latency.assign((size_t)G, 0.0);
  double last = 0.0;
  for (int i = 0; i < G; ++i) {
    mmsb_ctx* c = B->g[(size_t)i];
    try {
      pipeline_whiten_finish(c);
      stpm_online_stats(c, stpm_online_rounds(c));
    } catch (const MmsbError& e) {
      throw MmsbError(e.status, "graph " + std::to_string(i) + ": " + e.what());
    }
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, B->start_ev, B->done_ev[(size_t)i]), "elapsed");
    B->latency[(size_t)i] = ms;
    last = std::max(last, (double)ms);
  }
  float stpm_ms = 0.f;
  ck(cudaEventElapsedTime(&stpm_ms, B->start_ev, B->stpm_ev), "elapsed");
  const auto t1 = std::chrono::steady_clock::now();
  B->stats.total_ms = last;
  B->stats.stpm_end_ms = stpm_ms;
  B->stats.wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  B->stats.rounds = B->rounds;
  B->stats.batched_launches = B->graph_launches;
}

void batch_run_sequential(mmsb_batch* B) {
  const auto t0 = std::chrono::steady_clock::now();
  const int G = (int)B->g.size();
  B->latency.assign((size_t)G, 0.0);
  double sum = 0.0;
  for (int i = 0; i < G; ++i) {
    mmsb_ctx* c = B->g[(size_t)i];
    if (!c->have_graph) throw MmsbError(MMSB_ERR_STATE, "batch run before every graph is uploaded");
    c->stats = mmsb_stats{};
    ck(cudaEventRecord(B->ready_ev[(size_t)i], c->s), "event");
    pipeline_whiten(c, nullptr);
    pipeline_stpm(c, nullptr);
    pipeline_post(c);
    ck(cudaEventRecord(B->done_ev[(size_t)i], c->s), "event");
    ck(cudaEventSynchronize(B->done_ev[(size_t)i]), "sync");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, B->ready_ev[(size_t)i], B->done_ev[(size_t)i]), "elapsed");
    B->latency[(size_t)i] = ms;
    sum += ms;
  }
  const auto t1 = std::chrono::steady_clock::now();
  B->stats.total_ms = sum;
  B->stats.stpm_end_ms = 0.0;
  B->stats.wall_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  B->stats.rounds = 0;
  B->stats.batched_launches = 0;
  B->stats.graph_replayed = 0;
}

void finish_stats(mmsb_batch* B) {
  B->stats.latency_p50_ms = percentile(B->latency, 0.5);
  B->stats.latency_p99_ms = percentile(B->latency, 0.99);
  B->stats.latency_max_ms = percentile(B->latency, 1.0);
  B->stats.buckets = (int32_t)B->buckets.size();
  for (size_t i = 0; i < B->buckets.size() && i < (size_t)kMaxBuckets; ++i) {
    B->stats.bucket_kp[i] = B->buckets[i].KP;
    B->stats.bucket_ctas[i] = B->buckets[i].ctas;
    B->stats.bucket_graphs[i] = (int32_t)B->buckets[i].graphs.size();
  }
}

template <typename F>
mmsb_status bguard(mmsb_batch* B, F&& f) {
  try {
    f();
    return MMSB_OK;
  } catch (const MmsbError& e) {
    if (B) B->err = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    if (B) B->err = "host allocation failed";
    return MMSB_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    if (B) B->err = e.what();
    return MMSB_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

mmsb_status mmsb_batch_create(const mmsb_config* base, int32_t count, const int32_t* k,
                              const double* alpha0, const int32_t* minibatch, mmsb_batch** out) {
  if (!base || !out || count < 1 || count > 65535 || !k) return MMSB_ERR_INVALID_ARG;
  *out = nullptr;
  if (base->stpm_method == MMSB_STPM_BATCH_POWER) return MMSB_ERR_UNSUPPORTED;
  std::unique_ptr<mmsb_batch> B(new mmsb_batch());
  B->base = *base;
  mmsb_status st = bguard(B.get(), [&]() {
    ck(cudaSetDevice(base->device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&B->bs, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreate(&B->start_ev), "event");
    ck(cudaEventCreate(&B->stpm_ev), "event");
    for (int32_t i = 0; i < count; ++i) {
      mmsb_config cfg = *base;
      cfg.k = k[i];
      if (alpha0) cfg.alpha0 = alpha0[i];
      if (minibatch) cfg.minibatch = minibatch[i];
      cfg.seed = base->seed + (uint64_t)i;
      if (cfg.k < 1 || cfg.k > 128) throw MmsbError(MMSB_ERR_UNSUPPORTED, "batch graphs need 1 <= k <= 128");
      mmsb_ctx* c = nullptr;
      const mmsb_status s = mmsb_create(&cfg, &c);
      if (s != MMSB_OK) throw MmsbError(s, "graph context " + std::to_string(i));
      B->g.push_back(c);
      cudaEvent_t e0, e1;
      ck(cudaEventCreate(&e0), "event");
      ck(cudaEventCreate(&e1), "event");
      B->ready_ev.push_back(e0);
      B->done_ev.push_back(e1);
    }
  });
  if (st != MMSB_OK) return st;
  *out = B.release();
  return MMSB_OK;
}

void mmsb_batch_destroy(mmsb_batch* b) { delete b; }

mmsb_status mmsb_batch_upload(mmsb_batch* b, int32_t graph, const mmsb_csr blocks[MMSB_NUM_BLOCKS]) {
  if (!b || !blocks || graph < 0 || graph >= (int32_t)b->g.size()) return MMSB_ERR_INVALID_ARG;
  if (b->planned) return MMSB_ERR_STATE;  // the captured plan points at the graphs' buffers
  const mmsb_status s = mmsb_upload_graph(b->g[(size_t)graph], blocks);
  if (s != MMSB_OK) b->err = mmsb_last_error(b->g[(size_t)graph]);
  return s;
}

mmsb_status mmsb_batch_run(mmsb_batch* b) {
  if (!b) return MMSB_ERR_INVALID_ARG;
  return bguard(b, [&]() {
    ck(cudaSetDevice(b->base.device), "cudaSetDevice");
    batch_run(b);
    finish_stats(b);
  });
}

mmsb_status mmsb_batch_run_sequential(mmsb_batch* b) {
  if (!b) return MMSB_ERR_INVALID_ARG;
  return bguard(b, [&]() {
    ck(cudaSetDevice(b->base.device), "cudaSetDevice");
    batch_run_sequential(b);
    finish_stats(b);
  });
}

int32_t mmsb_batch_count(const mmsb_batch* b) { return b ? (int32_t)b->g.size() : 0; }

mmsb_status mmsb_batch_set_contract_ctas(mmsb_batch* b, int32_t ctas) {
  if (!b || ctas < 0 || ctas % stpm_partial_cluster() != 0) return MMSB_ERR_INVALID_ARG;
  if (b->planned) return MMSB_ERR_STATE;
  b->fixed_ctas = ctas;
  return MMSB_OK;
}

mmsb_ctx* mmsb_batch_graph(mmsb_batch* b, int32_t graph) {
  if (!b || graph < 0 || graph >= (int32_t)b->g.size()) return nullptr;
  return b->g[(size_t)graph];
}

mmsb_status mmsb_batch_latencies(const mmsb_batch* b, double* ms) {
  if (!b || !ms) return MMSB_ERR_INVALID_ARG;
  if (b->latency.size() != b->g.size()) return MMSB_ERR_STATE;
  std::copy(b->latency.begin(), b->latency.end(), ms);
  return MMSB_OK;
}

mmsb_status mmsb_batch_get_stats(const mmsb_batch* b, mmsb_batch_stats* out) {
  if (!b || !out) return MMSB_ERR_INVALID_ARG;
  *out = b->stats;
  return MMSB_OK;
}

const char* mmsb_batch_last_error(const mmsb_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
