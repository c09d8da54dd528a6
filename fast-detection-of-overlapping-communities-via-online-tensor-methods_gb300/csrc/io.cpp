// File formats of the path, parsed and formatted on up to 16 host threads:
//   * the reference's COO text input (read_G_sparse, CPU/IOfn.cpp:21-54),
//   * its triplet output (write_pi, CPU/IOfn.cpp:57-67),
//   * the GPU tree's dense outputs (write_mat, GPU/post_proc.c:45-59: one
//     "%5.25e" value per line, column-major),
//   * COO text output of a block (the input contract, for producing files),
//   * a binary CSR container of this library (no counterpart in the
//     reference): "MMSBCSR" + version byte, int64 n_rows, n_cols, nnz, int32
//     has_values, int32 0, then int64 row_ptr[n_rows + 1], int32
//     col_idx[nnz] and, if has_values, float val[nnz]; little-endian.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "host_graph.h"

namespace {

// host threads for parsing and formatting: up to 16, or MMSB_IO_THREADS
unsigned io_threads(size_t work, size_t min_per_thread) {
  static const unsigned cap = []() {
    const char* e = std::getenv("MMSB_IO_THREADS");
    const long v = e ? std::strtol(e, nullptr, 10) : 0;
    return v > 0 ? (unsigned)std::min<long>(v, 256) : 16u;
  }();
  const unsigned hw = std::max(1u, std::min(cap, std::thread::hardware_concurrency()));
  const size_t want = std::max<size_t>(1, work / std::max<size_t>(1, min_per_thread));
  return (unsigned)std::min<size_t>(hw, want);
}

// f(t) for t in [0, nt) on nt threads (the calling thread runs t = 0)
template <typename F>
void parallel_for(unsigned nt, F&& f) {
  std::vector<std::thread> th;
  th.reserve(nt > 0 ? nt - 1 : 0);
  for (unsigned t = 1; t < nt; ++t) th.emplace_back([&f, t]() { f(t); });
  f(0);
  for (auto& x : th) x.join();
}

inline bool is_space(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

// One number at p (the strtod grammar that fscanf("%lf") accepts), p at a
// non-space character of a NUL-terminated buffer.  Returns the end, or p if
// no number starts there.  Plain integers take a fast path with the same
// (correctly rounded) value.
inline const char* parse_number(const char* p, double* x) {
  const char* q = p;
  const bool neg = *q == '-';
  if (*q == '-' || *q == '+') ++q;
  const char* d0 = q;
  uint64_t v = 0;
  while (*q >= '0' && *q <= '9' && q - d0 < 18) v = v * 10 + (uint64_t)(*q++ - '0');
  if (q > d0 && (*q == '\0' || is_space(*q))) {
    *x = neg ? -(double)v : (double)v;
    return q;
  }
  char* end = nullptr;
  const double r = std::strtod(p, &end);
  if (end == p) return p;
  *x = r;
  return end;
}

struct TokenChunk {
  std::vector<double> tok;
  size_t last_end = 0;  // offset just past the chunk's last number
  bool bad = false;     // a non-number stopped the chunk
};

// Splits buf[0, len) at whitespace into up to nt chunks and parses each on
// its own thread.  buf[len] must be '\0'.
std::vector<TokenChunk> tokenize(const char* buf, size_t len) {
  const unsigned nt = io_threads(len, 1 << 20);
  std::vector<size_t> b(nt + 1, len);
  b[0] = 0;
  for (unsigned t = 1; t < nt; ++t) {
    size_t x = std::max(b[t - 1], len / nt * t);
    while (x < len && !is_space(buf[x])) ++x;
    b[t] = x;
  }
  std::vector<TokenChunk> ch(nt);
  parallel_for(nt, [&](unsigned t) {
    TokenChunk& c = ch[t];
    c.tok.reserve((b[t + 1] - b[t]) / 4 + 16);
    const char* p = buf + b[t];
    const char* e = buf + b[t + 1];
    for (;;) {
      while (p < e && is_space(*p)) ++p;
      if (p >= e) break;
      double v;
      const char* q = parse_number(p, &v);
      if (q == p) {
        c.bad = true;
        break;
      }
      c.tok.push_back(v);
      c.last_end = (size_t)(q - buf);
      p = q;
    }
  });
  return ch;
}

// CSR from triplets in input order: counting sort by row (stable), then per
// row a stable sort by column; duplicates summed in FP64 (sum) or the last
// one kept; entries with |v| <= prune dropped when prune >= 0.  Rows are
// split over threads.
HostCsr build_csr(int64_t n_rows, int64_t n_cols, const std::vector<int64_t>& rows,
                  const std::vector<int32_t>& cols, const std::vector<float>& vals, bool sum,
                  double prune) {
  const size_t n = rows.size();
  const unsigned nt = io_threads(n, 1 << 18);
  // per-thread row counts over contiguous triplet ranges
  std::vector<std::vector<int64_t>> cnt(nt, std::vector<int64_t>(n_rows, 0));
  auto range = [&](unsigned t, size_t total) {
    return std::make_pair(total / nt * t, t + 1 == nt ? total : total / nt * (t + 1));
  };
  parallel_for(nt, [&](unsigned t) {
    auto rg = range(t, n);
    for (size_t i = rg.first; i < rg.second; ++i) cnt[t][rows[i]]++;
  });
  std::vector<int64_t> start(n_rows + 1, 0);
  for (int64_t r = 0; r < n_rows; ++r) {
    int64_t s = start[r];
    for (unsigned t = 0; t < nt; ++t) {
      const int64_t c = cnt[t][r];
      cnt[t][r] = s;  // this thread's first slot in row r
      s += c;
    }
    start[r + 1] = s;
  }
  std::vector<int32_t> c(n);
  std::vector<float> v(n);
  parallel_for(nt, [&](unsigned t) {
    auto rg = range(t, n);
    for (size_t i = rg.first; i < rg.second; ++i) {
      const int64_t p = cnt[t][rows[i]]++;
      c[p] = cols[i];
      v[p] = vals[i];
    }
  });
  std::vector<std::vector<int64_t>>().swap(cnt);
  // per row: sort, merge duplicates, prune; kept counts into keep[r]
  std::vector<int64_t> keep(n_rows + 1, 0);
  const unsigned rt = io_threads((size_t)n_rows + n, 1 << 16);
  parallel_for(rt, [&](unsigned t) {
    const int64_t r0 = n_rows / rt * t, r1 = t + 1 == rt ? n_rows : n_rows / rt * (t + 1);
    std::vector<std::pair<int32_t, float>> tmp;
    for (int64_t r = r0; r < r1; ++r) {
      tmp.clear();
      for (int64_t p = start[r]; p < start[r + 1]; ++p) tmp.emplace_back(c[p], v[p]);
      std::stable_sort(tmp.begin(), tmp.end(),
                       [](const std::pair<int32_t, float>& a, const std::pair<int32_t, float>& b) {
                         return a.first < b.first;
                       });
      int64_t w = start[r];
      for (size_t i = 0; i < tmp.size();) {
        size_t j = i;
        double s = 0.0;
        while (j < tmp.size() && tmp[j].first == tmp[i].first) {
          s = sum ? s + (double)tmp[j].second : (double)tmp[j].second;
          ++j;
        }
        if (prune < 0.0 || std::fabs(s) > prune) {
          c[w] = tmp[i].first;
          v[w] = (float)s;
          ++w;
        }
        i = j;
      }
      keep[r + 1] = w - start[r];
    }
  });
  HostCsr m;
  m.n_rows = n_rows;
  m.n_cols = n_cols;
  m.row_ptr.assign(n_rows + 1, 0);
  for (int64_t r = 0; r < n_rows; ++r) m.row_ptr[r + 1] = m.row_ptr[r] + keep[r + 1];
  m.col.resize(m.row_ptr[n_rows]);
  m.val.resize(m.row_ptr[n_rows]);
  parallel_for(rt, [&](unsigned t) {
    const int64_t r0 = n_rows / rt * t, r1 = t + 1 == rt ? n_rows : n_rows / rt * (t + 1);
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t k = keep[r + 1];
      std::memcpy(&m.col[m.row_ptr[r]], &c[start[r]], sizeof(int32_t) * k);
      std::memcpy(&m.val[m.row_ptr[r]], &v[start[r]], sizeof(float) * k);
    }
  });
  if (std::all_of(m.val.begin(), m.val.end(), [](float x) { return x == 1.0f; }))
    std::vector<float>().swap(m.val);
  return m;
}

bool read_file(const char* path, std::string* out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    return false;
  }
  out->resize((size_t)sz);
  const size_t got = sz ? std::fread(&(*out)[0], 1, (size_t)sz, f) : 0;
  std::fclose(f);
  return got == (size_t)sz;
}

// Writes items [0, n) formatted by fmt(i0, i1, std::string&) on up to 16
// threads: contiguous item ranges, each formatted into its own string, the
// strings written in order; in rounds of about 64 MiB of text per thread.
template <typename F>
mmsb_status write_ranges(const char* path, int64_t n, size_t bytes_per_item, F&& fmt) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return MMSB_ERR_IO;
  const size_t bpi = std::max<size_t>(1, bytes_per_item);
  const unsigned nt = io_threads((size_t)std::max<int64_t>(n, 0) * bpi, 1 << 20);
  const int64_t per_round = std::max<int64_t>(1, (int64_t)(((size_t)nt << 26) / bpi));
  std::vector<std::string> piece(nt);
  bool ok = true;
  for (int64_t base = 0; base < n && ok; base += per_round) {
    const int64_t m = std::min(per_round, n - base);
    parallel_for(nt, [&](unsigned t) {
      const int64_t i0 = base + m / nt * t, i1 = base + (t + 1 == nt ? m : m / nt * (t + 1));
      piece[t].clear();
      piece[t].reserve((size_t)(i1 - i0) * bpi);
      fmt(i0, i1, piece[t]);
    });
    for (unsigned t = 0; t < nt && ok; ++t)
      ok = std::fwrite(piece[t].data(), 1, piece[t].size(), f) == piece[t].size();
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? MMSB_OK : MMSB_ERR_IO;
}

// write_pi: the nonzeros of a column-major rows x cols matrix in column
// order as "row\tcol\tvalue", the value as std::ostream prints a double by
// default (%g, 6 significant digits); one item per column
template <typename T>
mmsb_status write_triplets(const char* path, const T* m, int64_t rows, int64_t cols) {
  if (!path || rows < 0 || cols < 0 || (!m && rows * cols > 0)) return MMSB_ERR_INVALID_ARG;
  return write_ranges(path, cols, (size_t)rows * 12, [&](int64_t c0, int64_t c1, std::string& s) {
    char line[96];
    for (int64_t c = c0; c < c1; ++c)
      for (int64_t r = 0; r < rows; ++r) {
        const double v = (double)m[c * rows + r];
        if (v == 0.0) continue;
        const int len = std::snprintf(line, sizeof(line), "%lld\t%lld\t%g\n", (long long)(r + 1),
                                      (long long)(c + 1), v);
        s.append(line, (size_t)len);
      }
  });
}

// write_mat: one "%5.25e" value per line
template <typename T>
mmsb_status write_dense(const char* path, const T* m, int64_t count) {
  if (!path || count < 0 || (!m && count > 0)) return MMSB_ERR_INVALID_ARG;
  return write_ranges(path, count, 34, [&](int64_t i0, int64_t i1, std::string& s) {
    char line[64];
    for (int64_t i = i0; i < i1; ++i) {
      const int len = std::snprintf(line, sizeof(line), "%5.25e\n", (double)m[i]);
      s.append(line, (size_t)len);
    }
  });
}

struct BinHeader {
  char magic[8];
  int64_t n_rows, n_cols, nnz;
  int32_t has_val, zero;
};
constexpr char kBinMagic[8] = {'M', 'M', 'S', 'B', 'C', 'S', 'R', 1};

}  // namespace

// ---------------------------------------------------------------------------

extern "C" mmsb_status mmsb_read_coo(const char* path, int64_t n_rows, int64_t n_cols,
                                     int32_t datatype, int32_t compat, mmsb_host_graph** out) {
  if (!path || !out || n_rows < 0 || n_cols < 0 || n_rows > INT32_MAX || n_cols > INT32_MAX)
    return MMSB_ERR_INVALID_ARG;
  *out = nullptr;
  std::string buf;
  if (!read_file(path, &buf)) return MMSB_ERR_IO;
  std::vector<TokenChunk> ch = tokenize(buf.c_str(), buf.size());
  // the token stream ends at the first non-number: the reference's fscanf
  // loop would retry it forever, so the file is rejected
  std::vector<size_t> off(ch.size() + 1, 0);
  size_t last_end = 0;
  for (size_t t = 0; t < ch.size(); ++t) {
    if (ch[t].bad) return MMSB_ERR_IO;
    off[t + 1] = off[t] + ch[t].tok.size();
    if (!ch[t].tok.empty()) last_end = ch[t].last_end;
  }
  const size_t ntok = off.back();
  const int per = datatype == 1 ? 3 : 2;
  auto token = [&](size_t i) {
    const size_t t = (size_t)(std::upper_bound(off.begin(), off.end(), i) - off.begin()) - 1;
    return ch[t].tok[i - off[t]];
  };
  const size_t full = ntok / per, rem = ntok % per;
  // read_G_sparse loops while(!feof): after the last complete triplet one
  // more pass runs unless the last number ended the file; its failed reads
  // leave the previous values, so that pass pushes the last triplet again
  // (or a partial one completed by the previous values).
  size_t extra = 0;
  if (compat) {
    if (ntok < (size_t)per) return MMSB_ERR_IO;  // the reference would push unset fields
    extra = rem > 0 ? 1 : (last_end < buf.size() ? 1 : 0);
  } else if (rem != 0) {
    return MMSB_ERR_IO;
  }
  const size_t nt_trip = full + extra;
  std::vector<int64_t> rows(nt_trip);
  std::vector<int32_t> cols(nt_trip);
  std::vector<float> vals(nt_trip);
  std::vector<int> bad_range(16, 0);
  const unsigned nt = io_threads(full, 1 << 16);
  auto put = [&](size_t i, double r, double c, double v) {
    // Triplet<double>(r_idx - 1, c_idx - 1, val): indices truncated to int
    const int64_t ri = (int64_t)(r - 1.0), ci = (int64_t)(c - 1.0);
    if (!(r - 1.0 >= -1.0 && r - 1.0 < (double)INT32_MAX && c - 1.0 >= -1.0 &&
          c - 1.0 < (double)INT32_MAX) ||
        ri < 0 || ri >= n_rows || ci < 0 || ci >= n_cols)
      return false;
    rows[i] = ri;
    cols[i] = (int32_t)ci;
    vals[i] = datatype == 1 ? (float)v : 1.0f;
    return true;
  };
  parallel_for(nt, [&](unsigned t) {
    const size_t a = full / nt * t, b = t + 1 == nt ? full : full / nt * (t + 1);
    for (size_t i = a; i < b; ++i) {
      const size_t k = i * per;
      if (!put(i, token(k), token(k + 1), per == 3 ? token(k + 2) : 1.0)) {
        bad_range[t] = 1;
        return;
      }
    }
  });
  for (unsigned t = 0; t < nt; ++t)
    if (bad_range[t]) return MMSB_ERR_IO;
  if (extra) {
    double f[3];
    for (int j = 0; j < per; ++j)
      f[j] = (size_t)j < rem ? token(full * per + j) : token((full - 1) * per + j);
    if (!put(full, f[0], f[1], per == 3 ? f[2] : 1.0)) return MMSB_ERR_IO;
  }
  std::unique_ptr<mmsb_host_graph> g(new mmsb_host_graph());
  // compat: setFromTriplets sums duplicates, then prune(1e-6) keeps
  // |v| > 1e-6 * 1e-12 (Eigen's dummy precision); otherwise the last
  // duplicate wins and nothing is pruned
  g->blocks[0] = build_csr(n_rows, n_cols, rows, cols, vals, compat != 0, compat ? 1e-18 : -1.0);
  g->n_blocks = 1;
  *out = g.release();
  return MMSB_OK;
}

extern "C" mmsb_status mmsb_write_triplets_f32(const char* path, const float* m, int64_t rows,
                                               int64_t cols) {
  return write_triplets(path, m, rows, cols);
}

extern "C" mmsb_status mmsb_write_triplets_f64(const char* path, const double* m, int64_t rows,
                                               int64_t cols) {
  return write_triplets(path, m, rows, cols);
}

extern "C" mmsb_status mmsb_write_dense_f32(const char* path, const float* m, int64_t count) {
  return write_dense(path, m, count);
}

extern "C" mmsb_status mmsb_write_dense_f64(const char* path, const double* m, int64_t count) {
  return write_dense(path, m, count);
}

extern "C" mmsb_status mmsb_write_coo(const char* path, const mmsb_csr* m) {
  if (!path || !m || m->n_rows < 0 || (m->n_rows > 0 && !m->row_ptr) ||
      (m->nnz > 0 && !m->col_idx))
    return MMSB_ERR_INVALID_ARG;
  // the input contract: "row col" (binary) or "row col value" lines, 1-based,
  // row by row; weights with 9 significant digits read back to the same float
  const size_t per_row = 16 * (size_t)std::max<int64_t>(1, m->nnz / std::max<int64_t>(1, m->n_rows)) + 1;
  return write_ranges(path, m->n_rows, per_row, [&](int64_t r0, int64_t r1, std::string& s) {
    char line[96];
    for (int64_t r = r0; r < r1; ++r)
      for (int64_t p = m->row_ptr[r]; p < m->row_ptr[r + 1]; ++p) {
        const int len =
            m->val ? std::snprintf(line, sizeof(line), "%lld %lld %.9g\n", (long long)(r + 1),
                                   (long long)m->col_idx[p] + 1, (double)m->val[p])
                   : std::snprintf(line, sizeof(line), "%lld %lld\n", (long long)(r + 1),
                                   (long long)m->col_idx[p] + 1);
        s.append(line, (size_t)len);
      }
  });
}

extern "C" mmsb_status mmsb_write_csr(const char* path, const mmsb_csr* m) {
  if (!path || !m || m->n_rows < 0 || m->n_cols < 0 || m->nnz < 0 || !m->row_ptr ||
      (m->nnz > 0 && !m->col_idx))
    return MMSB_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return MMSB_ERR_IO;
  BinHeader h;
  std::memcpy(h.magic, kBinMagic, 8);
  h.n_rows = m->n_rows;
  h.n_cols = m->n_cols;
  h.nnz = m->nnz;
  h.has_val = m->val ? 1 : 0;
  h.zero = 0;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  ok = ok && std::fwrite(m->row_ptr, sizeof(int64_t), (size_t)m->n_rows + 1, f) == (size_t)m->n_rows + 1;
  if (m->nnz > 0) {
    ok = ok && std::fwrite(m->col_idx, sizeof(int32_t), (size_t)m->nnz, f) == (size_t)m->nnz;
    if (m->val) ok = ok && std::fwrite(m->val, sizeof(float), (size_t)m->nnz, f) == (size_t)m->nnz;
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? MMSB_OK : MMSB_ERR_IO;
}

extern "C" mmsb_status mmsb_read_csr(const char* path, mmsb_host_graph** out) {
  if (!path || !out) return MMSB_ERR_INVALID_ARG;
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return MMSB_ERR_IO;
  BinHeader h;
  std::unique_ptr<mmsb_host_graph> g(new mmsb_host_graph());
  HostCsr& m = g->blocks[0];
  auto fail = [&]() {
    std::fclose(f);
    return MMSB_ERR_IO;
  };
  if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kBinMagic, 8) != 0 ||
      h.n_rows < 0 || h.n_cols < 0 || h.nnz < 0 || h.n_rows > INT32_MAX || h.n_cols > INT32_MAX ||
      (h.has_val != 0 && h.has_val != 1))
    return fail();
  m.n_rows = h.n_rows;
  m.n_cols = h.n_cols;
  m.row_ptr.resize((size_t)h.n_rows + 1);
  m.col.resize((size_t)h.nnz);
  if (std::fread(m.row_ptr.data(), sizeof(int64_t), m.row_ptr.size(), f) != m.row_ptr.size())
    return fail();
  if (h.nnz > 0 && std::fread(m.col.data(), sizeof(int32_t), m.col.size(), f) != m.col.size())
    return fail();
  if (h.has_val) {
    m.val.resize((size_t)h.nnz);
    if (h.nnz > 0 && std::fread(m.val.data(), sizeof(float), m.val.size(), f) != m.val.size())
      return fail();
  }
  std::fclose(f);
  // structure checks: offsets from 0 to nnz, non-decreasing; columns in range
  if (m.row_ptr[0] != 0 || m.row_ptr[(size_t)h.n_rows] != h.nnz) return MMSB_ERR_IO;
  for (int64_t r = 0; r < h.n_rows; ++r)
    if (m.row_ptr[r + 1] < m.row_ptr[r]) return MMSB_ERR_IO;
  for (int32_t c : m.col)
    if (c < 0 || (int64_t)c >= h.n_cols) return MMSB_ERR_IO;
  g->n_blocks = 1;
  *out = g.release();
  return MMSB_OK;
}
