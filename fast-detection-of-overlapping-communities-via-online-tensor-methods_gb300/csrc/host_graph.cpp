// Host-side graph handling: seeded MMSB generator and the CSR container (the
// file formats live in io.cpp).
//
// Generator (synthetic stand-in for the reference's data/ graphs):
//   pi_i ~ Dirichlet(alpha0/k * 1);  B = q*J + (p-q)*I;
//   undirected A_ij ~ Bernoulli(pi_i^T B pi_j), i != j.
// It is sampled in O(n*k + edges) as the union of an Erdos-Renyi(q) layer
// (geometric skipping over the n(n-1)/2 pairs) and, per community c, an
// inhomogeneous rank-1 layer with pair probability (p-q) pi_ic pi_jc
// (sorted-weight skipping, Miller & Hagberg 2011).  The union's edge
// probability is 1-(1-q)prod_c(1-(p-q)pi_ic pi_jc) = pi_i^T B pi_j - O(p^2).
// Nodes are split into X, A, B, C by a uniformly random permutation.
#include "host_graph.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>

mmsb_csr HostCsr::view() const {
  mmsb_csr v;
  v.n_rows = n_rows;
  v.n_cols = n_cols;
  v.nnz = nnz();
  v.row_ptr = row_ptr.data();
  v.col_idx = col.data();
  v.val = val.empty() ? nullptr : val.data();
  return v;
}

HostCsr csr_from_triplets(int64_t n_rows, int64_t n_cols, std::vector<int64_t>& rows,
                          std::vector<int32_t>& cols, std::vector<float>* vals,
                          bool sum_dups) {
  HostCsr m;
  m.n_rows = n_rows;
  m.n_cols = n_cols;
  const size_t n = rows.size();
  std::vector<int64_t> cnt(n_rows + 1, 0);
  for (size_t i = 0; i < n; ++i) cnt[rows[i] + 1]++;
  for (int64_t r = 0; r < n_rows; ++r) cnt[r + 1] += cnt[r];
  std::vector<int32_t> c(n);
  std::vector<float> v(vals ? n : 0);
  std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
  for (size_t i = 0; i < n; ++i) {
    int64_t p = pos[rows[i]]++;
    c[p] = cols[i];
    if (vals) v[p] = (*vals)[i];
  }
  m.row_ptr.assign(n_rows + 1, 0);
  m.col.reserve(n);
  if (vals) m.val.reserve(n);
  std::vector<std::pair<int32_t, float>> tmp;
  for (int64_t r = 0; r < n_rows; ++r) {
    tmp.clear();
    for (int64_t p = cnt[r]; p < cnt[r + 1]; ++p) tmp.emplace_back(c[p], vals ? v[p] : 1.0f);
    std::stable_sort(tmp.begin(), tmp.end(),
                     [](const std::pair<int32_t, float>& a, const std::pair<int32_t, float>& b) {
                       return a.first < b.first;
                     });
    for (size_t i = 0; i < tmp.size();) {
      size_t j = i;
      float s = 0.f;
      while (j < tmp.size() && tmp[j].first == tmp[i].first) {
        s = sum_dups ? s + tmp[j].second : tmp[j].second;
        ++j;
      }
      m.col.push_back(tmp[i].first);
      if (vals) m.val.push_back(s);
      i = j;
    }
    m.row_ptr[r + 1] = (int64_t)m.col.size();
  }
  return m;
}

namespace {

// xoshiro256** (Blackman & Vigna 2018) seeded through splitmix64.
struct Rng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed, uint64_t stream = 0) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
    for (int i = 0; i < 4; ++i) s[i] = splitmix(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform in the open interval (0, 1)
  double uniform() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  // standard normal, Marsaglia polar method
  double normal() {
    for (;;) {
      double u = 2.0 * uniform() - 1.0, v = 2.0 * uniform() - 1.0;
      double s2 = u * u + v * v;
      if (s2 > 0.0 && s2 < 1.0) return u * std::sqrt(-2.0 * std::log(s2) / s2);
    }
  }
};

// log of a Gamma(a, 1) draw (Marsaglia & Tsang 2000; a < 1 via the
// U^(1/a) boost, kept in log space so tiny shapes do not underflow).
double log_gamma_draw(Rng& r, double a) {
  double boost = 0.0;
  if (a < 1.0) {
    boost = std::log(r.uniform()) / a;
    a += 1.0;
  }
  const double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
  for (;;) {
    double x = r.normal();
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = r.uniform();
    if (std::log(u) < 0.5 * x * x + d - d * v + d * std::log(v)) return std::log(d * v) + boost;
  }
}

void er_layer(int64_t n, double q, Rng& r, std::vector<uint64_t>& out) {
  if (q <= 0.0 || n < 2) return;
  if (q >= 1.0) {
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = i + 1; j < n; ++j) out.push_back((uint64_t)i * n + j);
    return;
  }
  const double lq = std::log1p(-q);
  int64_t i = 0, j = 0;  // (i, j): last visited pair, j in (i, n)
  for (;;) {
    double skip = std::floor(std::log(r.uniform()) / lq);
    if (skip > 9e18) break;
    j += 1 + (int64_t)skip;
    while (j >= n && i < n - 1) {
      int64_t over = j - n;
      ++i;
      j = i + 1 + over;
    }
    if (i >= n - 1) break;
    out.push_back((uint64_t)i * n + j);
  }
}

// pairs (u, v) with probability min(1, s * w_u * w_v)
void rank1_layer(int64_t n, const std::vector<std::pair<double, int64_t>>& sorted_w, double s,
                 Rng& r, std::vector<uint64_t>& out) {
  const int64_t m = (int64_t)sorted_w.size();
  for (int64_t u = 0; u + 1 < m; ++u) {
    const double wu = sorted_w[u].first;
    int64_t v = u + 1;
    double p = std::min(1.0, s * wu * sorted_w[v].first);
    while (v < m && p > 0.0) {
      if (p < 1.0) {
        double skip = std::floor(std::log(r.uniform()) / std::log1p(-p));
        if (skip >= (double)(m - v)) break;
        v += (int64_t)skip;
      }
      if (v >= m) break;
      double q = std::min(1.0, s * wu * sorted_w[v].first);
      if (r.uniform() < q / p) {
        int64_t a = sorted_w[u].second, b = sorted_w[v].second;
        if (a > b) std::swap(a, b);
        out.push_back((uint64_t)a * n + b);
      }
      p = q;
      ++v;
    }
  }
}

}  // namespace

extern "C" mmsb_status mmsb_generate(const mmsb_gen_params* P, mmsb_host_graph** out) {
  if (!P || !out || P->n < 4 || P->k < 1 || !(P->alpha0 > 0) || P->p_in < 0 || P->p_out < 0 ||
      P->p_in > 1 || P->p_out > 1)
    return MMSB_ERR_INVALID_ARG;
  *out = nullptr;
  const int64_t n = P->n;
  const int k = P->k;
  const double q = P->p_out, s = std::max(0.0, P->p_in - P->p_out);
  std::unique_ptr<mmsb_host_graph> g(new mmsb_host_graph());
  g->k = k;

  // memberships, node-major n x k
  std::vector<float> pi((size_t)n * k);
  {
    Rng r(P->seed, 1);
    std::vector<double> lg(k);
    const double a = P->alpha0 / k;
    for (int64_t i = 0; i < n; ++i) {
      double mx = -1e300;
      for (int c = 0; c < k; ++c) {
        lg[c] = log_gamma_draw(r, a);
        mx = std::max(mx, lg[c]);
      }
      double sum = 0.0;
      for (int c = 0; c < k; ++c) sum += (lg[c] = std::exp(lg[c] - mx));
      for (int c = 0; c < k; ++c) pi[(size_t)i * k + c] = (float)(lg[c] / sum);
    }
  }

  // layers: index 0 is Erdos-Renyi, 1..k the community layers
  std::vector<std::vector<uint64_t>> layer_edges(k + 1);
  auto run_layer = [&](int L) {
    Rng r(P->seed, 100 + (uint64_t)L);
    if (L == 0) {
      er_layer(n, q, r, layer_edges[0]);
      return;
    }
    const int c = L - 1;
    if (s <= 0.0) return;
    std::vector<std::pair<double, int64_t>> w;
    double wmax = 0.0;
    for (int64_t i = 0; i < n; ++i) wmax = std::max(wmax, (double)pi[(size_t)i * k + c]);
    const double wmin = wmax > 0 ? 1e-13 / (s * wmax) : 1.0;
    for (int64_t i = 0; i < n; ++i) {
      double wi = pi[(size_t)i * k + c];
      if (wi > wmin) w.emplace_back(wi, i);
    }
    std::sort(w.begin(), w.end(), [](const std::pair<double, int64_t>& a,
                                     const std::pair<double, int64_t>& b) {
      return a.first > b.first || (a.first == b.first && a.second < b.second);
    });
    rank1_layer(n, w, s, r, layer_edges[L]);
  };
  {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
      th.emplace_back([&, t]() {
        for (int L = (int)t; L <= k; L += (int)nt) run_layer(L);
      });
    for (auto& t : th) t.join();
  }
  std::vector<uint64_t> edges;
  {
    size_t tot = 0;
    for (auto& e : layer_edges) tot += e.size();
    edges.reserve(tot);
    for (auto& e : layer_edges) {
      edges.insert(edges.end(), e.begin(), e.end());
      std::vector<uint64_t>().swap(e);
    }
  }
  std::sort(edges.begin(), edges.end());
  edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
  g->n_edges = (int64_t)edges.size();

  // random partition X, A, B, C (sizes n/4, n/4, n/4, rest)
  std::vector<int64_t> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  {
    Rng r(P->seed, 2);
    for (int64_t i = n - 1; i > 0; --i) {
      int64_t j = (int64_t)(r.next() % (uint64_t)(i + 1));
      std::swap(perm[i], perm[j]);
    }
  }
  const int64_t q4 = n / 4;
  g->part[0] = q4;
  g->part[1] = q4;
  g->part[2] = q4;
  g->part[3] = n - 3 * q4;
  const int64_t off[4] = {0, q4, 2 * q4, 3 * q4};
  std::vector<int8_t> part_of(n);
  std::vector<int32_t> local_of(n);
  for (int64_t pos = 0; pos < n; ++pos) {
    int p = pos < off[1] ? 0 : pos < off[2] ? 1 : pos < off[3] ? 2 : 3;
    part_of[perm[pos]] = (int8_t)p;
    local_of[perm[pos]] = (int32_t)(pos - off[p]);
  }

  // blocks: XA, XB, XC (rows X), BA (rows B), CA (rows C); columns A/B/C
  enum { X = 0, A = 1, B = 2, C = 3 };
  std::vector<int64_t> br[5];
  std::vector<int32_t> bc[5];
  for (uint64_t e : edges) {
    int64_t u = (int64_t)(e / (uint64_t)n), v = (int64_t)(e % (uint64_t)n);
    int pu = part_of[u], pv = part_of[v];
    if (pu > pv) {
      std::swap(u, v);
      std::swap(pu, pv);
    }
    int blk = -1;
    int64_t r = 0;
    int32_t c = 0;
    if (pu == X && pv != X) {
      blk = pv - 1;  // XA=0, XB=1, XC=2
      r = local_of[u];
      c = local_of[v];
    } else if (pu == A && pv == B) {
      blk = MMSB_BLOCK_BA;
      r = local_of[v];
      c = local_of[u];
    } else if (pu == A && pv == C) {
      blk = MMSB_BLOCK_CA;
      r = local_of[v];
      c = local_of[u];
    }
    if (blk >= 0) {
      br[blk].push_back(r);
      bc[blk].push_back(c);
    }
  }
  const int rows_part[5] = {X, X, X, B, C};
  const int cols_part[5] = {A, B, C, A, A};
  for (int b = 0; b < 5; ++b) {
    g->blocks[b] = csr_from_triplets(g->part[rows_part[b]], g->part[cols_part[b]], br[b], bc[b],
                                     nullptr, false);
  }
  g->n_blocks = 5;
  if (P->keep_pi) {
    g->pi.resize((size_t)n * k);
    for (int64_t pos = 0; pos < n; ++pos)
      std::memcpy(&g->pi[(size_t)pos * k], &pi[(size_t)perm[pos] * k], sizeof(float) * k);
  }
  *out = g.release();
  return MMSB_OK;
}

extern "C" void mmsb_host_graph_free(mmsb_host_graph* g) { delete g; }

extern "C" mmsb_status mmsb_host_graph_info(const mmsb_host_graph* g, int64_t part_sizes[4],
                                            int64_t* n_edges) {
  if (!g) return MMSB_ERR_INVALID_ARG;
  if (part_sizes)
    for (int i = 0; i < 4; ++i) part_sizes[i] = g->part[i];
  if (n_edges) *n_edges = g->n_edges;
  return MMSB_OK;
}

extern "C" mmsb_status mmsb_host_graph_block(const mmsb_host_graph* g, int which, mmsb_csr* out) {
  if (!g || !out || which < 0 || which >= g->n_blocks) return MMSB_ERR_INVALID_ARG;
  *out = g->blocks[which].view();
  return MMSB_OK;
}

extern "C" mmsb_status mmsb_host_graph_pi(const mmsb_host_graph* g, float* pi) {
  if (!g || !pi || g->pi.empty()) return MMSB_ERR_INVALID_ARG;
  std::memcpy(pi, g->pi.data(), g->pi.size() * sizeof(float));
  return MMSB_OK;
}
