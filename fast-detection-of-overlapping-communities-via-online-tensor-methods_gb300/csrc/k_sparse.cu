// Sparse kernels: CSR x dense-panel products (the whitening workhorse), the
// device-side CSR transpose, row sums (partition means) and the fused
// unwhitening + normProbMatrix + threshold epilogue.
//
// Panels are row-major with a leading dimension that is a multiple of 4, so
// every panel row is gathered as 16-byte vectors.  One group of G lanes owns
// one output row; each lane keeps up to two float4 accumulators, and four
// nonzeros are in flight per lane to cover gather latency.
#include <cstdlib>
#include "common.cuh"

#include <cfloat>

namespace mmsb {

thread_local int64_t g_launch_count = 0;

namespace {

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

__device__ __forceinline__ void fma4(float4& a, float v, const float4& x) {
  a.x = fmaf(v, x.x, a.x);
  a.y = fmaf(v, x.y, a.y);
  a.z = fmaf(v, x.z, a.z);
  a.w = fmaf(v, x.w, a.w);
}

// G lanes per row; every lane accumulates chunks (base + gl) and (base + G + gl)
// of the 16-byte column chunks [cb, ce) (rows of P and Y have c4 chunks).
template <int G>
__global__ void __launch_bounds__(256) spmm_rows_kernel(
    const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, int64_t n_rows, const float4* __restrict__ P, int c4,
    float alpha, float4* __restrict__ Y, int cb, int ce) {
  const int lane = threadIdx.x & 31;
  const int gl = lane % G;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  if (row >= n_rows) return;
  const int64_t beg = rp[row], end = rp[row + 1];
  for (int base = cb; base < ce; base += 2 * G) {
    const int ch0 = base + gl, ch1 = base + G + gl;
    const bool h0 = ch0 < ce, h1 = ch1 < ce;
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    int64_t j = beg;
    for (; j + 4 <= end; j += 4) {
      const int64_t c_0 = ci[j], c_1 = ci[j + 1], c_2 = ci[j + 2], c_3 = ci[j + 3];
      float v0 = 1.f, v1 = 1.f, v2 = 1.f, v3 = 1.f;
      if (val) {
        v0 = val[j];
        v1 = val[j + 1];
        v2 = val[j + 2];
        v3 = val[j + 3];
      }
      if (h0) {
        float4 x0 = ldg4(P + c_0 * c4 + ch0), x1 = ldg4(P + c_1 * c4 + ch0);
        float4 x2 = ldg4(P + c_2 * c4 + ch0), x3 = ldg4(P + c_3 * c4 + ch0);
        fma4(a0, v0, x0);
        fma4(a0, v1, x1);
        fma4(a0, v2, x2);
        fma4(a0, v3, x3);
      }
      if (h1) {
        float4 x0 = ldg4(P + c_0 * c4 + ch1), x1 = ldg4(P + c_1 * c4 + ch1);
        float4 x2 = ldg4(P + c_2 * c4 + ch1), x3 = ldg4(P + c_3 * c4 + ch1);
        fma4(a1, v0, x0);
        fma4(a1, v1, x1);
        fma4(a1, v2, x2);
        fma4(a1, v3, x3);
      }
    }
    for (; j < end; ++j) {
      const int64_t c = ci[j];
      const float v = val ? val[j] : 1.f;
      if (h0) fma4(a0, v, ldg4(P + c * c4 + ch0));
      if (h1) fma4(a1, v, ldg4(P + c * c4 + ch1));
    }
    if (h0) Y[row * c4 + ch0] = make_float4(alpha * a0.x, alpha * a0.y, alpha * a0.z, alpha * a0.w);
    if (h1) Y[row * c4 + ch1] = make_float4(alpha * a1.x, alpha * a1.y, alpha * a1.z, alpha * a1.w);
  }
}

template <int G>
cudaError_t launch_spmm(const int64_t* rp, const int32_t* ci, const float* val, int64_t n_rows,
                        const float* P, int c4, float alpha, float* Y, cudaStream_t s,
                        int cb = 0, int ce = -1) {
  const int threads = 256;
  const int64_t blocks = ceil_div(n_rows * G, threads);
  spmm_rows_kernel<G><<<(unsigned)blocks, threads, 0, s>>>(
      rp, ci, val, n_rows, reinterpret_cast<const float4*>(P), c4, alpha,
      reinterpret_cast<float4*>(Y), cb, ce < 0 ? c4 : ce);
  ++g_launch_count;
  return cudaGetLastError();
}

// ---- transpose -----------------------------------------------------------

// (entries with a column index outside [0, n_cols) are skipped here and in
// scatter_kernel, and row ranges are clipped to [0, nnz): a malformed block
// gives a wrong transpose but no access outside the buffers)
__global__ void count_cols_kernel(const int32_t* __restrict__ ci, int64_t nnz, int64_t n_cols,
                                  unsigned long long* __restrict__ cnt) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = ci[j];
    if (c >= 0 && (int64_t)c < n_cols) atomicAdd(&cnt[c + 1], 1ull);
  }
}

// Inclusive scan in place over n+1 entries, one CTA of 1024 threads: with
// entry 0 == 0 and entry c + 1 == the count of column c on input, entry c is
// then the offset of column c.  Groups of kScanTiles coalesced tiles of 1024
// entries are loaded together (one memory latency per group), then scanned
// tile by tile: a warp scan by shuffles, a scan of the 32 warp totals, and a
// carry across tiles.
constexpr int kScanTiles = 16;

__global__ void __launch_bounds__(1024) scan_kernel(unsigned long long* __restrict__ a, int64_t n1) {
  __shared__ unsigned long long wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned long long carry = 0ull;
  for (int64_t group = 0; group < n1; group += (int64_t)kScanTiles * 1024) {
    unsigned long long v[kScanTiles];
#pragma unroll
    for (int q = 0; q < kScanTiles; ++q) {
      const int64_t i = group + (int64_t)q * 1024 + t;
      v[q] = i < n1 ? a[i] : 0ull;
    }
#pragma unroll
    for (int q = 0; q < kScanTiles; ++q) {
      const int64_t i = group + (int64_t)q * 1024 + t;
      unsigned long long x = v[q];
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
      }
      if (lane == 31) wsum[w] = x;
      __syncthreads();
      if (w == 0) {
        unsigned long long u = wsum[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const unsigned long long y = __shfl_up_sync(0xffffffffu, u, off);
          if (lane >= off) u += y;
        }
        wsum[lane] = u;
      }
      __syncthreads();
      if (i < n1) a[i] = carry + (w ? wsum[w - 1] : 0ull) + x;
      carry += wsum[31];
      __syncthreads();  // wsum is rewritten by the next tile
    }
  }
}

__global__ void scatter_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                               const float* __restrict__ val, int64_t n_rows, int64_t n_cols,
                               int64_t nnz, unsigned long long* __restrict__ cursor,
                               int32_t* __restrict__ ciT, float* __restrict__ valT) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rp[r] > 0 ? rp[r] : 0, e = rp[r + 1] < nnz ? rp[r + 1] : nnz;
    for (int64_t j = b; j < e; ++j) {
      const int32_t c = ci[j];
      if (c < 0 || (int64_t)c >= n_cols) continue;
      unsigned long long pos = atomicAdd(&cursor[c], 1ull);
      if (pos >= (unsigned long long)nnz) continue;
      ciT[pos] = (int32_t)r;
      if (valT) valT[pos] = val[j];
    }
  }
}

// Sorts every row segment of the transposed CSR by column (rank sort, one
// warp per segment; equal columns, from duplicate entries of the input, keep
// their input order, so the ranks always form a permutation).
constexpr int kSegStage = 512;  // segment entries a warp stages in shared memory

__global__ void __launch_bounds__(256) segment_sort_kernel(const int64_t* __restrict__ rpT,
                                                           int64_t n_rowsT,
                                                           const int32_t* __restrict__ in_c,
                                                           const float* __restrict__ in_v,
                                                           int32_t* __restrict__ out_c,
                                                           float* __restrict__ out_v) {
  __shared__ int32_t seg[8][kSegStage];
  const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= n_rowsT) return;  // warp-uniform
  const int64_t b = rpT[w], e = rpT[w + 1];
  const int64_t L = e - b;
  if (L <= kSegStage) {
    // the segment in shared memory: the rank loop reads broadcast words
    int32_t* sg = seg[wb];
    for (int64_t i = lane; i < L; i += 32) sg[i] = in_c[b + i];
    __syncwarp();
    for (int64_t i = lane; i < L; i += 32) {
      const int32_t x = sg[i];
      int rank = 0;
      for (int j = 0; j < (int)L; ++j) {
        const int32_t y = sg[j];
        rank += (y < x) || (y == x && j < i);
      }
      out_c[b + rank] = x;
      if (out_v) out_v[b + rank] = in_v[b + i];
    }
    return;
  }
  for (int64_t i = lane; i < L; i += 32) {
    const int32_t x = in_c[b + i];
    int64_t rank = 0;
    for (int64_t j = 0; j < L; ++j) {
      const int32_t y = in_c[b + j];
      rank += (y < x) || (y == x && j < i);
    }
    out_c[b + rank] = x;
    if (out_v) out_v[b + rank] = in_v[b + i];
  }
}

__global__ void u64_to_i64_kernel(const unsigned long long* __restrict__ a, int64_t n,
                                  int64_t* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (int64_t)a[i];
}

__global__ void row_sums_kernel(const int64_t* __restrict__ rp, const float* __restrict__ val,
                                int64_t n_rows, double scale, double* __restrict__ out) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows;
       r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    if (val) {
      for (int64_t j = rp[r]; j < rp[r + 1]; ++j) s += (double)val[j];
    } else {
      s = (double)(rp[r + 1] - rp[r]);
    }
    out[r] = scale * s;
  }
}

// ---- unwhitening + normProbVector + threshold ------------------------------

__global__ void __launch_bounds__(256) unwhiten_normprob_kernel(
    const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
    const float* __restrict__ val, int64_t n_rows, const float4* __restrict__ P, int c4, int k,
    float tau, int64_t row_offset, float* __restrict__ pi, uint32_t* __restrict__ bits,
    float raw_scale) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= n_rows) return;
  const int64_t beg = rp[row], end = rp[row + 1];
  const int ch0 = lane, ch1 = lane + 32;
  const bool h0 = ch0 < c4, h1 = ch1 < c4;
  float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
  for (int64_t j = beg; j < end; ++j) {
    const int64_t c = ci[j];
    const float v = val ? val[j] : 1.f;
    if (h0) fma4(a0, v, ldg4(P + c * c4 + ch0));
    if (h1) fma4(a1, v, ldg4(P + c * c4 + ch1));
  }
  float x[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
  // entries beyond k (panel padding) do not take part
  float pos = 0.f, neg = 0.f;
  bool nz = false;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int idx = (e < 4 ? 4 * ch0 : 4 * ch1) + (e & 3);
    if (idx >= k) x[e] = 0.f;
    if (x[e] > 0.f) pos += x[e];
    else neg += x[e];
    nz |= x[e] != 0.f;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    pos += __shfl_xor_sync(0xffffffffu, pos, off);
    neg += __shfl_xor_sync(0xffffffffu, neg, off);
  }
  nz = __any_sync(0xffffffffu, nz);
  if (raw_scale > 0.f) {
    // raw unwhitened memberships (the GPU tree's Pi files), no normalisation
    // and no set bits
    float* out = pi + (row_offset + row) * (int64_t)k;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = (e < 4 ? 4 * ch0 : 4 * ch1) + (e & 3);
      if (idx < k) out[idx] = x[e] * raw_scale;
    }
    return;
  }
  if (nz) {
    // Probability.cpp:45-55: the larger-magnitude mass fixes sign and scale
    const bool flip = fabsf(pos) < fabsf(neg);
    const float inv = flip ? -1.f / fabsf(neg) : 1.f / fabsf(pos);
#pragma unroll
    for (int e = 0; e < 8; ++e) x[e] = fmaxf(x[e] * inv, 0.f);
  }
  float* out = pi + (row_offset + row) * (int64_t)k;
  unsigned nib0 = 0, nib1 = 0;
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int idx = (e < 4 ? 4 * ch0 : 4 * ch1) + (e & 3);
    if (idx < k) {
      out[idx] = x[e];
      if (x[e] > tau) {
        if (e < 4) nib0 |= 1u << (e & 3);
        else nib1 |= 1u << (e & 3);
      }
    }
  }
  // 8 lanes x 4 entries form one 32-bit word of the membership bit set
  unsigned w0 = nib0 << (4 * (lane & 7)), w1 = nib1 << (4 * (lane & 7));
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    w0 |= __shfl_xor_sync(0xffffffffu, w0, off);
    w1 |= __shfl_xor_sync(0xffffffffu, w1, off);
  }
  const int words = (k + 31) / 32;
  uint32_t* brow = bits + (row_offset + row) * (int64_t)words;
  if ((lane & 7) == 0) {
    const int wi0 = lane >> 3, wi1 = 4 + (lane >> 3);
    if (wi0 < words) brow[wi0] = w0;
    if (wi1 < words) brow[wi1] = w1;
  }
}

}  // namespace

cudaError_t spmm_f32(const int64_t* rp, const int32_t* ci, const float* val, int64_t n_rows,
                     const float* P, int ld, float alpha, float* Y, cudaStream_t s,
                     int64_t p_rows) {
  if (ld % 4 != 0) return cudaErrorInvalidValue;
  if (n_rows == 0) return cudaSuccess;
  const int c4 = ld / 4;
  // a panel far larger than L2 (129 MB): column slices of <= 64 MB, one pass
  // over the CSR each, so that every slice's gathered rows stay L2-resident
  // MMSB_SPMM_SLICE_MB overrides the 64 MB slice (a tuning override)
  static const double slice = []() {
    const char* e = std::getenv("MMSB_SPMM_SLICE_MB");
    const double v = e ? std::strtod(e, nullptr) : 0.0;
    return v >= 1.0 ? v * 1e6 : 64e6;
  }();
  if (p_rows > 0 && (double)p_rows * ld * sizeof(float) > 1.5 * slice) {
    int w4 = (int)std::min<int64_t>(c4, std::max<int64_t>(8, (int64_t)(slice / (16.0 * p_rows))));
    w4 = std::max(8, w4 / 8 * 8);
    for (int cb = 0; cb < c4; cb += w4) {
      const int ce = std::min(c4, cb + w4);
      cudaError_t e = w4 >= 64   ? launch_spmm<32>(rp, ci, val, n_rows, P, c4, alpha, Y, s, cb, ce)
                      : w4 >= 32 ? launch_spmm<16>(rp, ci, val, n_rows, P, c4, alpha, Y, s, cb, ce)
                      : w4 >= 16 ? launch_spmm<8>(rp, ci, val, n_rows, P, c4, alpha, Y, s, cb, ce)
                                 : launch_spmm<4>(rp, ci, val, n_rows, P, c4, alpha, Y, s, cb, ce);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  if (c4 <= 2) return launch_spmm<1>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
  if (c4 <= 4) return launch_spmm<2>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
  if (c4 <= 8) return launch_spmm<4>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
  if (c4 <= 16) return launch_spmm<8>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
  if (c4 <= 32) return launch_spmm<16>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
  return launch_spmm<32>(rp, ci, val, n_rows, P, c4, alpha, Y, s);
}

// Input checks of an uploaded block (the transposes and SpMMs index with
// these): bit 1 = a decreasing row offset, bit 2 = a column index outside
// [0, n_cols).  Grid-stride over rows and nonzeros.
__global__ void csr_validate_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                    int64_t n_rows, int64_t n_cols, int64_t nnz,
                                    unsigned* __restrict__ bad) {
  unsigned f = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += stride)
    if (rp[r + 1] < rp[r]) f |= 1u;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += stride) {
    const int32_t c = ci[j];
    if (c < 0 || (int64_t)c >= n_cols) f |= 2u;
  }
  f = __reduce_or_sync(0xffffffffu, f);
  if (f && (threadIdx.x & 31) == 0) atomicOr(bad, f);
}

cudaError_t csr_validate(const int64_t* rp, const int32_t* ci, int64_t n_rows, int64_t n_cols,
                         int64_t nnz, unsigned* bad, cudaStream_t s) {
  const int T = 256;
  const int64_t work = std::max(n_rows, nnz);
  const unsigned G = (unsigned)std::max<int64_t>(1, std::min<int64_t>(kNumSMs * 8, ceil_div(work, T)));
  csr_validate_kernel<<<G, T, 0, s>>>(rp, ci, n_rows, n_cols, nnz, bad);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t csr_transpose(const int64_t* rp, const int32_t* ci, const float* val, int64_t n_rows,
                          int64_t n_cols, int64_t nnz, int64_t* rpT, int32_t* ciT, float* valT,
                          int32_t* scratch, cudaStream_t s) {
  // scratch: (n_cols + 1) u64 counters followed by nnz int32 (+ nnz float)
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(scratch);
  int32_t* tmp_c = reinterpret_cast<int32_t*>(cnt + (n_cols + 1));
  float* tmp_v = val ? reinterpret_cast<float*>(tmp_c + nnz) : nullptr;
  MMSB_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (n_cols + 1), s));
  const int T = 256;
  const unsigned G = (unsigned)std::min<int64_t>(4 * kNumSMs * 8, std::max<int64_t>(1, ceil_div(nnz, T)));
  if (nnz > 0) {
    count_cols_kernel<<<G, T, 0, s>>>(ci, nnz, n_cols, cnt);
    ++g_launch_count;
  }
  scan_kernel<<<1, 1024, 0, s>>>(cnt, n_cols + 1);
  ++g_launch_count;
  u64_to_i64_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(1024, ceil_div(n_cols + 1, T))), T, 0, s>>>(cnt, n_cols + 1, rpT);
  ++g_launch_count;
  if (nnz > 0) {
    const unsigned GR = (unsigned)std::max<int64_t>(1, std::min<int64_t>(4096, ceil_div(n_rows, T)));
    // row 0 in every slot first: a malformed block (row ranges that overlap
    // or skip entries) then leaves valid row indices, never stale words
    MMSB_CUDA_TRY(cudaMemsetAsync(tmp_c, 0, sizeof(int32_t) * nnz, s));
    scatter_kernel<<<GR, T, 0, s>>>(rp, ci, val, n_rows, n_cols, nnz, cnt, tmp_c, tmp_v);
    ++g_launch_count;
    segment_sort_kernel<<<(unsigned)ceil_div(n_cols * 32, T), T, 0, s>>>(rpT, n_cols, tmp_c, tmp_v,
                                                                          ciT, valT);
    ++g_launch_count;
  }
  return cudaGetLastError();
}

cudaError_t row_sums_f64(const int64_t* rp, const float* val, int64_t n_rows, double scale,
                         double* out, cudaStream_t s) {
  if (n_rows == 0) return cudaSuccess;
  const int T = 256;
  row_sums_kernel<<<(unsigned)std::min<int64_t>(4096, ceil_div(n_rows, T)), T, 0, s>>>(
      rp, val, n_rows, scale, out);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t unwhiten_normprob(const int64_t* rp, const int32_t* ci, const float* val,
                              int64_t n_rows, const float* P, int ldp, int k, float tau,
                              int64_t row_offset, float* pi, uint32_t* bits, cudaStream_t s,
                              float raw_scale) {
  if (ldp % 4 != 0 || k > 256 || k > ldp) return cudaErrorInvalidValue;
  if (n_rows == 0) return cudaSuccess;
  const int T = 256;
  unwhiten_normprob_kernel<<<(unsigned)ceil_div(n_rows * 32, T), T, 0, s>>>(
      rp, ci, val, n_rows, reinterpret_cast<const float4*>(P), ldp / 4, k, tau, row_offset, pi,
      bits, raw_scale);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
