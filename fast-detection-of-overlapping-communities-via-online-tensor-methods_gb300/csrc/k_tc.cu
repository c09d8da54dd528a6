// Tall-skinny Gram S = A^T B (A: n x pa, B: n x pb, FP32 node-major panels)
// on the 5th-generation tensor cores: tcgen05.mma kind::tf32 with the
// accumulator in tensor memory, FP32 accuracy by the 3xTF32 split
// (a = hi + lo, hi rounded to TF32; D += Ahi Bhi + Ahi Blo + Alo Bhi).
//
// CTA tile: 128 columns of A (the MMA's M, one TMEM lane each) x 128 columns
// of B (N, one TMEM column each) over a contiguous range of rows (the MMA's
// K).  Rows are staged 32 at a time into shared memory, split into hi / lo
// and written in the canonical K-major layout without swizzle: 8 x 16-byte
// core matrices (8 M-rows x 4 K-elements, 128 contiguous bytes), the next
// core along K at +128 B (leading byte offset), the next along M at
// +1024 B (stride byte offset).  Two stages: while the tensor core reads one,
// the threads fill the other; one elected thread issues the 12 MMAs of a stage
// (4 K-steps of 8 x 3 products) and commits them to that stage's mbarrier.
// The FP32 accumulator is read back with tcgen05.ld and written as this
// split's FP64 partial, summed over splits by gram_reduce.
#include "common.cuh"

namespace mmsb {
namespace {

constexpr int kTcM = 128, kTcN = 128, kTcK = 32;  // tile edge, rows per stage
constexpr int kTcThreads = 512;  // 16 warps: the staging is issue-bound
constexpr uint32_t kStageBytes = 4u * (2 * kTcM * kTcK + 2 * kTcN * kTcK);  // Ahi Alo Bhi Blo
constexpr uint32_t kTcSmem = 2 * kStageBytes + 1024;  // + alignment slack

__device__ __forceinline__ uint32_t sm_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait_limited(uint32_t bar, uint32_t parity, long long limit) {
  const long long start = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - start > limit) return false;
  }
}

// shared memory matrix descriptor, K-major, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100-class tensor cores
  return d;               // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor: kind::tf32, D in FP32, A and B TF32 and K-major
__host__ __device__ constexpr uint32_t tf32_idesc(int m, int n) {
  return (1u << 4)                      // D format: F32
         | (2u << 7)                    // A format: TF32
         | (2u << 10)                   // B format: TF32
         | ((uint32_t)(n >> 3) << 17)   // N / 8
         | ((uint32_t)(m >> 4) << 24);  // M / 16
}

// byte offset of element (r, k) of a 128 x 32 K-major tile
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)((r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__global__ void __launch_bounds__(kTcThreads, 1)
gram_tc_kernel(const float* __restrict__ A, int lda, int pa, const float* __restrict__ B, int ldb,
               int pb, int64_t n, int64_t rows_per_split, double* __restrict__ partials,
               unsigned* flags, long long wait_limit) {
  const long long wl = wait_limit > 0 ? wait_limit : 2000000000LL;
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  // 1024-byte aligned stage area
  unsigned char* base = tc_raw + ((1024 - (sm_addr(tc_raw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTcM, n0 = blockIdx.y * kTcN;
  const int64_t r0 = (int64_t)blockIdx.z * rows_per_split;
  const int64_t r1 = min(n, r0 + rows_per_split);
  const int64_t span = r1 > r0 ? r1 - r0 : 0;
  const int nchunks = (int)((span + kTcK - 1) / kTcK);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sm_addr(&tmem_slot)),
                 "r"(kTcN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  constexpr uint32_t idesc = tf32_idesc(kTcM, kTcN);
  uint32_t phase[2] = {0u, 0u};
  bool timed_out = false;
  int issued[2] = {0, 0};  // commits outstanding per stage (0 or 1)
  // Staging: thread task u (8 per thread) = one M-row m of A or B and four
  // consecutive rows 4 kq .. 4 kq + 3 of the chunk: four coalesced loads
  // (lanes along m), then one 16-byte store each of hi and lo into the core
  // matrix row (m, 4 kq .. 4 kq + 3).  The next chunk's loads are issued
  // before this chunk's barrier and MMAs, so their latency overlaps them.
  constexpr int kTasks = 2 * kTcM * (kTcK / 4) / kTcThreads;  // 4
  float v[kTasks][4];
  auto load_chunk = [&](int c) {
    const int64_t rb = r0 + (int64_t)c * kTcK;
#pragma unroll
    for (int u = 0; u < kTasks; ++u) {
      const int e = tid + kTcThreads * u;
      const bool isA = e < kTcM * (kTcK / 4);
      const int w = isA ? e : e - kTcM * (kTcK / 4);
      const int kq = w / kTcM, m = w % kTcM;
      const int col = (isA ? m0 : n0) + m;
      const bool cok = col < (isA ? pa : pb);
      const float* X = isA ? A : B;
      const int ld = isA ? lda : ldb;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t row = rb + 4 * kq + i;
        v[u][i] = (cok && row < r1) ? __ldg(X + row * ld + col) : 0.f;
      }
    }
  };
  if (nchunks > 0) load_chunk(0);
  for (int c = 0; c < nchunks; ++c) {
    const int st = c & 1;
    unsigned char* stage = base + st * kStageBytes;
    // the MMAs that last read this stage (chunk c - 2) must be done
    if (issued[st]) {
      if (!mbar_wait_limited(sm_addr(&bars[st]), phase[st], wl)) timed_out = true;
      phase[st] ^= 1u;
      issued[st] = 0;
    }
    if (__syncthreads_or(timed_out)) {
      timed_out = true;
      break;
    }
    unsigned char* Ahi = stage;
    unsigned char* Alo = stage + 4 * kTcM * kTcK;
    unsigned char* Bhi = stage + 8 * kTcM * kTcK;
    unsigned char* Blo = Bhi + 4 * kTcN * kTcK;
#pragma unroll
    for (int u = 0; u < kTasks; ++u) {
      const int e = tid + kTcThreads * u;
      const bool isA = e < kTcM * (kTcK / 4);
      const int w = isA ? e : e - kTcM * (kTcK / 4);
      const int kq = w / kTcM, m = w % kTcM;
      uint32_t h[4];
      float l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h[i]) : "f"(v[u][i]));
        l[i] = v[u][i] - __uint_as_float(h[i]);
      }
      const uint32_t off = tile_off(m, 4 * kq);
      *reinterpret_cast<uint4*>((isA ? Ahi : Bhi) + off) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<float4*>((isA ? Alo : Blo) + off) = make_float4(l[0], l[1], l[2], l[3]);
    }
    if (c + 1 < nchunks) load_chunk(c + 1);
    // generic-proxy stores -> visible to the tensor core's async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      const uint32_t a_hi = sm_addr(Ahi), a_lo = sm_addr(Alo), b_hi = sm_addr(Bhi),
                     b_lo = sm_addr(Blo);
#pragma unroll
      for (int ks = 0; ks < kTcK / 8; ++ks) {
        const uint32_t koff = (uint32_t)ks * 256u;  // two 16-byte core matrices per K-step of 8
        const uint64_t dah = smem_desc(a_hi + koff, 128, 1024), dal = smem_desc(a_lo + koff, 128, 1024);
        const uint64_t dbh = smem_desc(b_hi + koff, 128, 1024), dbl = smem_desc(b_lo + koff, 128, 1024);
        const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(dah), "l"(dbh), "r"(idesc), "r"(acc0)
            : "memory");
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(dah), "l"(dbl), "r"(idesc), "r"(1u)
            : "memory");
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
            "l"(dal), "l"(dbh), "r"(idesc), "r"(1u)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       sm_addr(&bars[st]))
                   : "memory");
    }
    issued[st] = 1;
  }
  // wait for every outstanding commit (also after a timeout, bounded)
  for (int st = 0; st < 2; ++st)
    if (issued[st]) {
      if (!mbar_wait_limited(sm_addr(&bars[st]), phase[st], wl)) timed_out = true;
      phase[st] ^= 1u;
    }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (rows m), columns
  // [kCols (w / 4), +kCols) (n), 16 at a time
  if (!timed_out && nchunks > 0) {
    constexpr int kGroups = kTcThreads / 128, kCols = kTcN / kGroups;  // column groups of warps
    const int q = warp & 3, half = warp >> 2;
    const int m = m0 + 32 * q + lane;
    double* out = partials + (int64_t)blockIdx.z * pa * pb;
    for (int cb = 0; cb < kCols; cb += 16) {
      const int col = kCols * half + cb;
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (m < pa) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int nn = n0 + col + j;
          if (nn < pb) out[(int64_t)nn * pa + m] = (double)__uint_as_float(v[j]);
        }
      }
    }
  } else if (nchunks == 0) {
    double* out = partials + (int64_t)blockIdx.z * pa * pb;
    for (int e = tid; e < kTcM * kTcN; e += kTcThreads) {
      const int m = m0 + e % kTcM, nn = n0 + e / kTcM;
      if (m < pa && nn < pb) out[(int64_t)nn * pa + m] = 0.0;
    }
  }
  if (timed_out && tid == 0 && flags) atomicOr(flags, kFlagTimeout);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcN)
                 : "memory");
}

}  // namespace

int gram_tc_nsplit(int64_t n, int pa, int pb) {
  const int64_t tiles = ceil_div(pa, kTcM) * ceil_div(pb, kTcN);
  int64_t want = ceil_div(kNumSMs, tiles);
  want = std::min<int64_t>(want, ceil_div(n, 8 * kTcK));
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, 256));
}

cudaError_t gram_tc_partial(const float* A, int lda, int pa, const float* B, int ldb, int pb,
                            int64_t n, double* partials, int nsplit, unsigned* flags,
                            cudaStream_t s, long long wait_limit) {
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kTcSmem));
    set = true;
  }
  const int64_t rows = round_up(ceil_div(n, nsplit), kTcK);
  dim3 grid((unsigned)ceil_div(pa, kTcM), (unsigned)ceil_div(pb, kTcN), (unsigned)nsplit);
  gram_tc_kernel<<<grid, kTcThreads, kTcSmem, s>>>(A, lda, pa, B, ldb, pb, n, rows, partials, flags,
                                                   wait_limit);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
