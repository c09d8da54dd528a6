/*
 * Seeded synthetic MMSB graphs for the CPU side of the benchmark -- TEST AND
 * BENCH INFRASTRUCTURE, like the rest of oracle/.
 *
 * bench.py's reference arm times the oracle port of the reference path on the
 * host cores and must not load the GPU library, yet it has to run on the very
 * graph the GPU arm runs on.  This file restates the library's generator
 * (mmsb_generate) step by step, so that both arms see bit-identical CSR blocks
 * for the same parameters (tests/test_oracle_gen.py asserts it):
 *
 *   pi_i ~ Dirichlet(alpha0/k * 1) (log-space Gamma draws, Marsaglia-Tsang,
 *   a < 1 boosted by U^(1/a)); undirected edges = union of an Erdos-Renyi(q)
 *   layer (geometric skipping) and per community c a rank-1 layer of pair
 *   probability (p - q) pi_ic pi_jc (sorted-weight skipping, Miller &
 *   Hagberg 2011); nodes split into X, A, B, C by a uniformly random
 *   permutation (Fisher-Yates); blocks XA, XB, XC, BA, CA as CSR with sorted
 *   unique columns.  Random numbers: xoshiro256** (Blackman & Vigna 2018)
 *   seeded through splitmix64, one stream per purpose (1: memberships,
 *   2: permutation, 100 + L: layer L).
 *
 * Build: cc -O2 -ffp-contract=off -DMMSB_GEN_MAIN mmsb_gen.c -lm, an executable
 * (oracle/Makefile target gen, also run by __graft_entry__.build()) that
 * writes the graph to a file, so the timed CPU process maps no library of
 * this repository.  The library is built with -ffp-contract=off as well, so
 * no fused multiply-add changes a draw.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  uint64_t s[4];
} rng_t;

static uint64_t splitmix(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void rng_init(rng_t* r, uint64_t seed, uint64_t stream) {
  uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull);
  for (int i = 0; i < 4; ++i) r->s[i] = splitmix(&x);
}

static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(rng_t* r) {
  uint64_t* s = r->s;
  const uint64_t out = rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return out;
}

/* uniform in (0, 1) */
static double uniform(rng_t* r) {
  return ((double)(rng_next(r) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

/* standard normal, Marsaglia's polar method */
static double normal(rng_t* r) {
  for (;;) {
    double u = 2.0 * uniform(r) - 1.0, v = 2.0 * uniform(r) - 1.0;
    double s2 = u * u + v * v;
    if (s2 > 0.0 && s2 < 1.0) return u * sqrt(-2.0 * log(s2) / s2);
  }
}

static double log_gamma_draw(rng_t* r, double a) {
  double boost = 0.0;
  if (a < 1.0) {
    boost = log(uniform(r)) / a;
    a += 1.0;
  }
  const double d = a - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
  for (;;) {
    double x = normal(r);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = uniform(r);
    if (log(u) < 0.5 * x * x + d - d * v + d * log(v)) return log(d * v) + boost;
  }
}

typedef struct {
  uint64_t* e;
  size_t n, cap;
} vec_u64;

static int push(vec_u64* v, uint64_t x) {
  if (v->n == v->cap) {
    size_t cap = v->cap ? 2 * v->cap : 1024;
    uint64_t* p = (uint64_t*)realloc(v->e, cap * sizeof(uint64_t));
    if (!p) return -1;
    v->e = p;
    v->cap = cap;
  }
  v->e[v->n++] = x;
  return 0;
}

static int er_layer(int64_t n, double q, rng_t* r, vec_u64* out) {
  if (q <= 0.0 || n < 2) return 0;
  if (q >= 1.0) {
    for (int64_t i = 0; i < n; ++i)
      for (int64_t j = i + 1; j < n; ++j)
        if (push(out, (uint64_t)i * n + j)) return -1;
    return 0;
  }
  const double lq = log1p(-q);
  int64_t i = 0, j = 0;
  for (;;) {
    double skip = floor(log(uniform(r)) / lq);
    if (skip > 9e18) break;
    j += 1 + (int64_t)skip;
    while (j >= n && i < n - 1) {
      int64_t over = j - n;
      ++i;
      j = i + 1 + over;
    }
    if (i >= n - 1) break;
    if (push(out, (uint64_t)i * n + j)) return -1;
  }
  return 0;
}

typedef struct {
  double w;
  int64_t i;
} wnode;

static int wnode_cmp(const void* pa, const void* pb) {
  const wnode* a = (const wnode*)pa;
  const wnode* b = (const wnode*)pb;
  if (a->w > b->w) return -1;
  if (a->w < b->w) return 1;
  return a->i < b->i ? -1 : a->i > b->i ? 1 : 0;
}

static int rank1_layer(int64_t n, const wnode* w, int64_t m, double s, rng_t* r, vec_u64* out) {
  for (int64_t u = 0; u + 1 < m; ++u) {
    const double wu = w[u].w;
    int64_t v = u + 1;
    double p = fmin(1.0, s * wu * w[v].w);
    while (v < m && p > 0.0) {
      if (p < 1.0) {
        double skip = floor(log(uniform(r)) / log1p(-p));
        if (skip >= (double)(m - v)) break;
        v += (int64_t)skip;
      }
      if (v >= m) break;
      double q = fmin(1.0, s * wu * w[v].w);
      if (uniform(r) < q / p) {
        int64_t a = w[u].i, b = w[v].i;
        if (a > b) {
          int64_t t = a;
          a = b;
          b = t;
        }
        if (push(out, (uint64_t)a * n + b)) return -1;
      }
      p = q;
      ++v;
    }
  }
  return 0;
}

static int u64_cmp(const void* pa, const void* pb) {
  uint64_t a = *(const uint64_t*)pa, b = *(const uint64_t*)pb;
  return a < b ? -1 : a > b ? 1 : 0;
}

/* One generated graph: part sizes, undirected edge count, the five blocks
 * (row offsets int64, sorted unique columns int32). */
typedef struct {
  int64_t part[4];
  int64_t n_edges;
  int64_t n_rows[5], n_cols[5], nnz[5];
  int64_t* row_ptr[5];
  int32_t* col[5];
} gen_graph;

void gen_free(gen_graph* g) {
  if (!g) return;
  for (int b = 0; b < 5; ++b) {
    free(g->row_ptr[b]);
    free(g->col[b]);
  }
  free(g);
}

/* Returns NULL on invalid parameters or allocation failure. */
gen_graph* gen_generate(int64_t n, int32_t k, double alpha0, double p_in, double p_out,
                        uint64_t seed) {
  if (n < 4 || k < 1 || !(alpha0 > 0) || p_in < 0 || p_out < 0 || p_in > 1 || p_out > 1)
    return NULL;
  const double q = p_out, s = fmax(0.0, p_in - p_out);
  gen_graph* g = (gen_graph*)calloc(1, sizeof(gen_graph));
  float* pi = (float*)malloc(sizeof(float) * (size_t)n * k);
  double* lg = (double*)malloc(sizeof(double) * k);
  vec_u64 edges = {0};
  if (!g || !pi || !lg) goto fail;
  {
    rng_t r;
    rng_init(&r, seed, 1);
    const double a = alpha0 / k;
    for (int64_t i = 0; i < n; ++i) {
      double mx = -1e300;
      for (int c = 0; c < k; ++c) {
        lg[c] = log_gamma_draw(&r, a);
        mx = fmax(mx, lg[c]);
      }
      double sum = 0.0;
      for (int c = 0; c < k; ++c) sum += (lg[c] = exp(lg[c] - mx));
      for (int c = 0; c < k; ++c) pi[(size_t)i * k + c] = (float)(lg[c] / sum);
    }
  }
  {
    rng_t r;
    rng_init(&r, seed, 100);
    if (er_layer(n, q, &r, &edges)) goto fail;
  }
  if (s > 0.0) {
    wnode* w = (wnode*)malloc(sizeof(wnode) * (size_t)n);
    if (!w) goto fail;
    for (int c = 0; c < k; ++c) {
      rng_t r;
      rng_init(&r, seed, 100 + (uint64_t)(c + 1));
      double wmax = 0.0;
      for (int64_t i = 0; i < n; ++i) wmax = fmax(wmax, (double)pi[(size_t)i * k + c]);
      const double wmin = wmax > 0 ? 1e-13 / (s * wmax) : 1.0;
      int64_t m = 0;
      for (int64_t i = 0; i < n; ++i) {
        double wi = pi[(size_t)i * k + c];
        if (wi > wmin) {
          w[m].w = wi;
          w[m].i = i;
          ++m;
        }
      }
      qsort(w, (size_t)m, sizeof(wnode), wnode_cmp);
      if (rank1_layer(n, w, m, s, &r, &edges)) {
        free(w);
        goto fail;
      }
    }
    free(w);
  }
  qsort(edges.e, edges.n, sizeof(uint64_t), u64_cmp);
  {
    size_t u = 0;
    for (size_t i = 0; i < edges.n; ++i)
      if (i == 0 || edges.e[i] != edges.e[i - 1]) edges.e[u++] = edges.e[i];
    edges.n = u;
  }
  g->n_edges = (int64_t)edges.n;
  {
    int64_t* perm = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int8_t* part_of = (int8_t*)malloc((size_t)n);
    int32_t* local_of = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!perm || !part_of || !local_of) {
      free(perm);
      free(part_of);
      free(local_of);
      goto fail;
    }
    for (int64_t i = 0; i < n; ++i) perm[i] = i;
    rng_t r;
    rng_init(&r, seed, 2);
    for (int64_t i = n - 1; i > 0; --i) {
      int64_t j = (int64_t)(rng_next(&r) % (uint64_t)(i + 1));
      int64_t t = perm[i];
      perm[i] = perm[j];
      perm[j] = t;
    }
    const int64_t q4 = n / 4;
    g->part[0] = g->part[1] = g->part[2] = q4;
    g->part[3] = n - 3 * q4;
    const int64_t off[4] = {0, q4, 2 * q4, 3 * q4};
    for (int64_t pos = 0; pos < n; ++pos) {
      int p = pos < off[1] ? 0 : pos < off[2] ? 1 : pos < off[3] ? 2 : 3;
      part_of[perm[pos]] = (int8_t)p;
      local_of[perm[pos]] = (int32_t)(pos - off[p]);
    }
    /* blocks XA, XB, XC (rows X), BA (rows B), CA (rows C) */
    static const int rows_part[5] = {0, 0, 0, 2, 3}, cols_part[5] = {1, 2, 3, 1, 1};
    int64_t* cnt[5] = {0};
    int ok = 1;
    for (int b = 0; b < 5; ++b) {
      g->n_rows[b] = g->part[rows_part[b]];
      g->n_cols[b] = g->part[cols_part[b]];
      cnt[b] = (int64_t*)calloc((size_t)g->n_rows[b] + 1, sizeof(int64_t));
      if (!cnt[b]) ok = 0;
    }
    /* two passes over the edges: count per row, then scatter */
    for (int pass = 0; pass < 2 && ok; ++pass) {
      if (pass == 1) {
        for (int b = 0; b < 5; ++b) {
          for (int64_t rr = 0; rr < g->n_rows[b]; ++rr) cnt[b][rr + 1] += cnt[b][rr];
          g->nnz[b] = cnt[b][g->n_rows[b]];
          g->row_ptr[b] = (int64_t*)malloc(sizeof(int64_t) * ((size_t)g->n_rows[b] + 1));
          g->col[b] = (int32_t*)malloc(sizeof(int32_t) * ((size_t)g->nnz[b] + 1));
          if (!g->row_ptr[b] || !g->col[b]) ok = 0;
          else memcpy(g->row_ptr[b], cnt[b], sizeof(int64_t) * ((size_t)g->n_rows[b] + 1));
        }
        if (!ok) break;
      }
      for (size_t i = 0; i < edges.n; ++i) {
        int64_t u = (int64_t)(edges.e[i] / (uint64_t)n), v = (int64_t)(edges.e[i] % (uint64_t)n);
        int pu = part_of[u], pv = part_of[v];
        if (pu > pv) {
          int64_t t = u;
          u = v;
          v = t;
          int tp = pu;
          pu = pv;
          pv = tp;
        }
        int blk = -1;
        int64_t rr = 0;
        int32_t cc = 0;
        if (pu == 0 && pv != 0) {
          blk = pv - 1;
          rr = local_of[u];
          cc = local_of[v];
        } else if (pu == 1 && pv == 2) {
          blk = 3;
          rr = local_of[v];
          cc = local_of[u];
        } else if (pu == 1 && pv == 3) {
          blk = 4;
          rr = local_of[v];
          cc = local_of[u];
        }
        if (blk < 0) continue;
        if (pass == 0) cnt[blk][rr + 1]++;
        else g->col[blk][cnt[blk][rr]++] = cc;
      }
    }
    /* columns sorted within each row (edges are unique, so no duplicates) */
    for (int b = 0; b < 5 && ok; ++b)
      for (int64_t rr = 0; rr < g->n_rows[b]; ++rr) {
        int32_t* c = g->col[b] + g->row_ptr[b][rr];
        int64_t len = g->row_ptr[b][rr + 1] - g->row_ptr[b][rr];
        for (int64_t x = 1; x < len; ++x) { /* insertion sort: rows are short */
          int32_t v = c[x];
          int64_t y = x - 1;
          while (y >= 0 && c[y] > v) {
            c[y + 1] = c[y];
            --y;
          }
          c[y + 1] = v;
        }
      }
    for (int b = 0; b < 5; ++b) free(cnt[b]);
    free(perm);
    free(part_of);
    free(local_of);
    if (!ok) goto fail;
  }
  free(pi);
  free(lg);
  free(edges.e);
  return g;
fail:
  free(pi);
  free(lg);
  free(edges.e);
  gen_free(g);
  return NULL;
}

#ifdef MMSB_GEN_MAIN
#include <stdio.h>
/* mmsb_gen N K ALPHA0 P_IN P_OUT SEED OUT: writes the graph to OUT as
 * int64 part[4], int64 n_edges, then per block int64 n_rows, n_cols, nnz,
 * int64 row_ptr[n_rows + 1], int32 col[nnz] (host byte order). */
int main(int argc, char** argv) {
  if (argc != 8) {
    fprintf(stderr, "usage: %s N K ALPHA0 P_IN P_OUT SEED OUT\n", argv[0]);
    return 2;
  }
  gen_graph* g = gen_generate(strtoll(argv[1], NULL, 10), (int32_t)strtol(argv[2], NULL, 10),
                              strtod(argv[3], NULL), strtod(argv[4], NULL), strtod(argv[5], NULL),
                              strtoull(argv[6], NULL, 10));
  if (!g) {
    fprintf(stderr, "invalid parameters or out of memory\n");
    return 1;
  }
  FILE* f = fopen(argv[7], "wb");
  if (!f) {
    gen_free(g);
    return 1;
  }
  int ok = fwrite(g->part, sizeof(int64_t), 4, f) == 4 &&
           fwrite(&g->n_edges, sizeof(int64_t), 1, f) == 1;
  for (int b = 0; b < 5 && ok; ++b) {
    int64_t hdr[3] = {g->n_rows[b], g->n_cols[b], g->nnz[b]};
    ok = fwrite(hdr, sizeof(int64_t), 3, f) == 3 &&
         fwrite(g->row_ptr[b], sizeof(int64_t), (size_t)g->n_rows[b] + 1, f) ==
             (size_t)g->n_rows[b] + 1 &&
         fwrite(g->col[b], sizeof(int32_t), (size_t)g->nnz[b], f) == (size_t)g->nnz[b];
  }
  ok = (fclose(f) == 0) && ok;
  gen_free(g);
  return ok ? 0 : 1;
}
#endif
