// Tensor power method kernels (FP32 path).
//
// The reference's STPM (GPU/stpm.c:497-790) issues ~2k+10 tiny library calls
// per sample; tensorDecom_alpha0 (CPU/Util.cpp:131-184) runs k sparse
// mat-vecs per column per iteration.  Both reduce to one contraction shape,
// computed here per tile of T nodes:
//
//   Z1 = Y1 Phi, Z2 = Y2 Phi                      (T x k, Phi resident in smem)
//   C  = c0 Z1.Z2 + c2 (Z1 diag(m2) + diag(m1) Z2) (alpha0 correction terms)
//   G += Yout^T C ,  d += colsum(Z1.Z2)            (k x k partial per CTA)
//
// with m1 = Phi^T mu1, m2 = Phi^T mu2.  The online update (Diff_Loss,
// Util.cpp:257-304) uses (Y1,Y2,Yout) = (y_A,y_B,y_C); the batch power
// iteration (tensor_form_main/shift1/shift0, Util.cpp:187-206) uses
// (y_B,y_C,y_A).  The adjoint mode computes all three partial derivatives of
// the cubic form (three Z's, three coefficient matrices, one stacked
// contraction) and the loss.
//
// Partials are reduced deterministically by stpm_reduce; the k x k update
// (orthogonality term, step, Newton-Schulz polar orthonormalisation) runs on
// one 8-CTA cluster exchanging column blocks through distributed shared memory.
#include "common.cuh"
#include "k_stpm.cuh"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

namespace mmsb {

namespace {

constexpr int TN = 32;  // nodes per tile
constexpr int kPartialCluster = 8;  // CTAs whose partials are summed through DSMEM

__device__ __forceinline__ int64_t ceil_div_dev(int64_t a, int64_t b) { return (a + b - 1) / b; }

// dynamic smem layout helpers
__host__ __device__ constexpr int ys_ld(int KP) { return KP + 1; }

template <int KP, int MODE>
__global__ void __launch_bounds__(256) stpm_partial_kernel(StpmPartialArgs a) {
  constexpr int NZ = MODE == kModeAdjoint || MODE == kModeLoss ? 3 : 2;
  constexpr int NY = 3;
  constexpr int LD = ys_ld(KP);
  constexpr int PT = KP / 16;  // contraction patch edge
  constexpr int ZC = KP / 8;   // Z columns per thread
  extern __shared__ float sm[];
  float* Phis = sm;                          // KP x KP, row j = component j (Phis[j*KP+i] = Phi_ji)
  float* Ys = Phis + KP * KP;                // NY tiles, each TN x LD
  float* Cs = Ys + NY * TN * LD;             // NZ coefficient tiles (TN x LD) [plain: 1]
  float* mv = Cs + (MODE == kModePlain ? 1 : 3) * TN * LD;  // m1, m2, m3 (KP each)
  float* dsum = mv + 3 * KP;                 // 3 x KP accumulators of sum Z_a Z_b
  const int tid = threadIdx.x;
  const int k = a.k;

  for (int e = tid; e < KP * KP; e += 256) {
    const int j = e / KP, i = e % KP;
    Phis[e] = (i < k && j < k) ? a.phi[(int64_t)i * k + j] : 0.f;
  }
  // stage mu_1..3 in dsum (zeroed again below)
  for (int e = tid; e < 3 * KP; e += 256) {
    const int which = e / KP, j = e % KP;
    const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
    dsum[e] = (mu && j < k) ? mu[j] : 0.f;
  }
  __syncthreads();
  // m_P = Phi^T mu_P
  for (int e = tid; e < 3 * KP; e += 256) {
    const int which = e / KP, i = e % KP;
    const float* mu = dsum + which * KP;
    float s0 = 0.f, s1 = 0.f;
    if (i < k) {
      int j = 0;
      for (; j + 1 < k; j += 2) {
        s0 = fmaf(Phis[j * KP + i], mu[j], s0);
        s1 = fmaf(Phis[(j + 1) * KP + i], mu[j + 1], s1);
      }
      if (j < k) s0 = fmaf(Phis[j * KP + i], mu[j], s0);
    }
    mv[e] = s0 + s1;
  }
  __syncthreads();
  for (int e = tid; e < 3 * KP; e += 256) dsum[e] = 0.f;
  __syncthreads();

  const int pj = tid / 16, pi = tid % 16;  // contraction patch (rows j, cols i)
  float acc[PT][PT];
#pragma unroll
  for (int r = 0; r < PT; ++r)
#pragma unroll
    for (int c = 0; c < PT; ++c) acc[r][c] = 0.f;
  float tsum = 0.f;  // loss mode: sum of t over this thread's entries
  float dloc[3][ZC];
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int c = 0; c < ZC; ++c) dloc[q][c] = 0.f;

  const int x_lane = tid % TN, grp = tid / TN;
  const int64_t ntiles = ceil_div_dev(a.count, TN);
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t x0 = a.begin + tile * TN;
    const int64_t left = a.begin + a.count - x0;
    const int nvalid = left < TN ? (int)left : TN;
    // load the node tiles (row-major y, ld = a.ldy)
    for (int q = 0; q < NY; ++q) {
      const float* Y = q == 0 ? a.y1 : q == 1 ? a.y2 : a.y3;
      float* dst = Ys + q * TN * LD;
      for (int e = tid; e < TN * KP; e += 256) {
        const int xx = e / KP, j = e % KP;
        dst[xx * LD + j] = (xx < nvalid && j < k) ? Y[(x0 + xx) * a.ldy + j] : 0.f;
      }
    }
    __syncthreads();
    // Z = Y Phi for this thread's node and columns
    float z[NZ][ZC];
#pragma unroll
    for (int q = 0; q < NZ; ++q)
#pragma unroll
      for (int c = 0; c < ZC; ++c) z[q][c] = 0.f;
    {
      const float* y0 = Ys + 0 * TN * LD + x_lane * LD;
      const float* y1 = Ys + 1 * TN * LD + x_lane * LD;
      const float* y2 = Ys + 2 * TN * LD + x_lane * LD;
      for (int j = 0; j < KP; ++j) {
        const float v0 = y0[j], v1 = y1[j];
        const float v2 = NZ == 3 ? y2[j] : 0.f;
        const float* ph = Phis + j * KP + grp;
#pragma unroll
        for (int c = 0; c < ZC; ++c) {
          const float f = ph[8 * c];
          z[0][c] = fmaf(v0, f, z[0][c]);
          z[1][c] = fmaf(v1, f, z[1][c]);
          if (NZ == 3) z[NZ - 1][c] = fmaf(v2, f, z[NZ - 1][c]);
        }
      }
    }
    const bool valid = x_lane < nvalid;
#pragma unroll
    for (int c = 0; c < ZC; ++c) {
      const int i = grp + 8 * c;
      const float m1 = mv[i], m2 = mv[KP + i];
      if (MODE == kModePlain) {
        const float z1 = z[0][c], z2 = z[1][c];
        const float cf = a.c0 * z1 * z2 + a.c2 * (z1 * m2 + m1 * z2);
        Cs[x_lane * LD + i] = valid ? cf : 0.f;
        if (valid) dloc[0][c] = fmaf(z1, z2, dloc[0][c]);
      } else {
        const float m3 = mv[2 * KP + i];
        const float z1 = z[0][c], z2 = z[1][c], z3 = z[2][c];
        const float p0 = a.c0, p2 = a.c2;
        if (MODE == kModeAdjoint) {
          Cs[0 * TN * LD + x_lane * LD + i] = valid ? p0 * z2 * z3 + p2 * (z2 * m3 + m2 * z3) : 0.f;
          Cs[1 * TN * LD + x_lane * LD + i] = valid ? p0 * z1 * z3 + p2 * (z1 * m3 + m1 * z3) : 0.f;
          Cs[2 * TN * LD + x_lane * LD + i] = valid ? p0 * z1 * z2 + p2 * (z1 * m2 + m1 * z2) : 0.f;
        }
        if (valid) {
          dloc[0][c] = fmaf(z2, z3, dloc[0][c]);
          dloc[1][c] = fmaf(z1, z3, dloc[1][c]);
          dloc[2][c] = fmaf(z1, z2, dloc[2][c]);
          if (MODE == kModeLoss && i < k)
            tsum += p0 * z1 * z2 * z3 + p2 * (z1 * z2 * m3 + z1 * m2 * z3 + m1 * z2 * z3);
        }
      }
    }
    __syncthreads();
    if (MODE != kModeLoss) {
      // G[j, i] += sum_x Yout[x, j] C[x, i]   (adjoint: sum over the three pairs)
      constexpr int NPAIR = MODE == kModePlain ? 1 : 3;
#pragma unroll
      for (int q = 0; q < NPAIR; ++q) {
        const float* Yo = Ys + (MODE == kModePlain ? 2 : q) * TN * LD;
        const float* Cq = Cs + q * TN * LD;
        for (int xx = 0; xx < TN; ++xx) {
          float yv[PT], cv[PT];
#pragma unroll
          for (int r = 0; r < PT; ++r) yv[r] = Yo[xx * LD + pj * PT + r];
#pragma unroll
          for (int c = 0; c < PT; ++c) cv[c] = Cq[xx * LD + pi * PT + c];
#pragma unroll
          for (int r = 0; r < PT; ++r)
#pragma unroll
            for (int c = 0; c < PT; ++c) acc[r][c] = fmaf(yv[r], cv[c], acc[r][c]);
        }
      }
    }
    __syncthreads();
  }
  // d sums: reduce over the 32 node lanes of each group via smem atomics
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int c = 0; c < ZC; ++c) {
      float v = dloc[q][c];
#pragma unroll
      for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (x_lane == 0 && (q == 0 || MODE != kModePlain)) dsum[q * KP + grp + 8 * c] = v;
    }
  if (MODE == kModeLoss) {
#pragma unroll
    for (int off = 16; off; off >>= 1) tsum += __shfl_xor_sync(0xffffffffu, tsum, off);
  }
  __syncthreads();
  // cluster reduction: every CTA stages its partial (k x k column-major
  // contraction, 3 d-sums, loss) in shared memory; CTA r of the cluster sums a
  // 1/CLP slice over the cluster's CTAs through DSMEM and writes it out.
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank();
  constexpr int CLP = kPartialCluster;
  constexpr int STAGE = KP * KP + 3 * KP + 4;
  float* stage = sm;  // Phi, y and C tiles are dead from here on
  {
    // dsum lives after the stage area (see layout), copy it in place first
    float dtmp[3 * KP / 256 + 1];
    int cnt = 0;
    for (int e = tid; e < 3 * KP; e += 256) dtmp[cnt++] = dsum[e];
    __shared__ float tred[8];
    if (MODE == kModeLoss) {
      if (x_lane == 0) tred[grp] = tsum;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PT; ++r)
#pragma unroll
      for (int c = 0; c < PT; ++c) stage[(pi * PT + c) * KP + pj * PT + r] = acc[r][c];
    cnt = 0;
    for (int e = tid; e < 3 * KP; e += 256) stage[KP * KP + e] = dtmp[cnt++];
    if (tid == 0) {
      float t = 0.f;
      if (MODE == kModeLoss)
        for (int g8 = 0; g8 < 8; ++g8) t += tred[g8];
      stage[KP * KP + 3 * KP] = t;
    }
  }
  cluster.sync();
  float* gp = a.gpart + (int64_t)(blockIdx.x / CLP) * a.part_stride;
  const int slice = (STAGE + CLP - 1) / CLP;
  for (int e = crank * slice + tid; e < min(STAGE, (crank + 1) * slice); e += 256) {
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < CLP; ++q) v += cluster.map_shared_rank(stage, q)[e];
    if (e < KP * KP) {
      const int i = e / KP, j = e % KP;
      if (i < k && j < k && MODE != kModeLoss) gp[(int64_t)i * k + j] = v;
    } else if (e < KP * KP + 3 * KP) {
      const int q = (e - KP * KP) / KP, i = (e - KP * KP) % KP;
      if (i < k) gp[(int64_t)k * k + q * k + i] = v;
    } else if (e == KP * KP + 3 * KP) {
      gp[(int64_t)k * k + 3 * k] = v;
    }
  }
  cluster.sync();  // keep shared memory alive until every remote read is done
}

// G = sum_parts gpart + mu-terms; d-vectors folded in (see stpm_reduce doc).
__global__ void stpm_reduce_kernel(StpmReduceArgs a) {
  const int k = a.k;
  const int64_t kk = (int64_t)k * k;
  extern __shared__ double mred[];  // m1, m2, m3, dsum(3k)
  double* m = mred;
  double* ds = mred + 3 * k;
  for (int e = threadIdx.x; e < 3 * k; e += blockDim.x) {
    const int which = e / k, i = e % k;
    const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
    double s = 0.0;
    if (mu)
      for (int j = 0; j < k; ++j) s += (double)a.phi[(int64_t)i * k + j] * (double)mu[j];
    m[e] = s;
    double d = 0.0;
    for (int p = 0; p < a.nparts; ++p) d += (double)a.gpart[(int64_t)p * a.part_stride + kk + e];
    ds[e] = d;
  }
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < kk;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % k), i = (int)(e / k);
    double s = 0.0;
    if (a.mode != kModeLoss)
      for (int p = 0; p < a.nparts; ++p) s += (double)a.gpart[(int64_t)p * a.part_stride + e];
    s *= a.scale;
    if (a.mode == kModePlain) {
      // mu_out * (c1 m1 m2 + c2 sum Z1 Z2)
      const double d = a.c1 * m[i] * m[k + i] + a.c2 * ds[i];
      s += (double)a.mu_out[j] * d;
    } else if (a.mode == kModeAdjoint) {
      const double dm1 = a.c2 * ds[i] / a.count + a.c1 * m[k + i] * m[2 * k + i];
      const double dm2 = a.c2 * ds[k + i] / a.count + a.c1 * m[i] * m[2 * k + i];
      const double dm3 = a.c2 * ds[2 * k + i] / a.count + a.c1 * m[i] * m[k + i];
      s += (double)a.mu1[j] * dm1 + (double)a.mu2[j] * dm2 + (double)a.mu3[j] * dm3;
    }
    a.G[e] = (float)s;
  }
  if (a.mode == kModeLoss && blockIdx.x == 0 && threadIdx.x == 0) {
    double t = 0.0;
    for (int p = 0; p < a.nparts; ++p) t += (double)a.gpart[(int64_t)p * a.part_stride + kk + 3 * k];
    double that = t / a.count;
    for (int i = 0; i < k; ++i) that += a.c1 * m[i] * m[k + i] * m[2 * k + i];
    a.loss_out[0] = that;  // sum_i That(phi_i, phi_i, phi_i)
  }
}

// ---- k x k step on one thread-block cluster -------------------------------------
//
// Every CTA of the cluster holds the whole current matrix X (column-major,
// leading dimension KP + 4) and owns NB = 8 or 16 of its columns.  The
// products X^T X[:, blk] and X B[:, blk] run on the tensor cores as warp-level
// m16n8k8 TF32 MMAs with the 3xTF32 split (a = a_hi + a_lo; hi*hi + hi*lo +
// lo*hi accumulated in FP32, relative error ~1e-6 per product), one warp per
// 16 x 8 output tile.  The new column block is staged in shared memory and
// sent to every CTA's next buffer by bulk asynchronous copies
// (cp.async.bulk shared::cta -> shared::cluster), which complete on the
// receiver's mbarrier; a CTA proceeds once all CL blocks of the next
// iterate have arrived, so the data exchange itself is the per-iteration
// synchronisation.  A block sent at broadcast n is rewritten only at
// broadcast n + 2, after every receiver has finished waiting for broadcast
// n (two staging buffers alternate).

// scaled Newton-Schulz: first guess of the smallest singular value after
// the initial scaling, the error below which the plain step is used, and a
// cap on the scale that keeps f(a sigma) > 0 for sigma slightly above 1
constexpr float kNsLowerGuess = 2e-2f;
constexpr float kNsPlainBelow = 0.1f;
constexpr float kNsMaxScale = 1.7f;
__device__ __forceinline__ float ns_poly(float y) { return y * (1.5f - 0.5f * y * y); }

// column stride of X, B and the output tile: KP + 4 (== 4 mod 8 for KP a
// multiple of 16) makes the fragment loads of the Gram product conflict-free
__host__ __device__ constexpr int step_xld(int KP) { return KP + 4; }

// NB = 8 (one n-tile) when the cluster has KP / 8 CTAs, else 16
template <int KP, int CL>
struct StepSmem {
  static constexpr int NB = KP / CL, XLD = step_xld(KP), MT = KP / 16, NT = NB / 8;
  static constexpr int TILES = MT * NT, KS = TILES <= 8 ? 2 : 1;  // K split over warps
  static constexpr size_t floats = (size_t)2 * KP * XLD    // X, next X
                                   + (size_t)4 * NB * XLD  // B (Ab), G block, 2 output tiles
                                   + (size_t)TILES * 128   // K-split partial tiles
                                   + 4 * KP + 3 * CL + 3 * NB + 2 * NB + 8;
};

__device__ __forceinline__ uint32_t tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// waits for the phase with the given parity to complete; false after about
// one second (then the caller reports kFlagTimeout instead of hanging)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  const long long start = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - start > 2000000000LL) return false;
  }
}

// bulk copy of `bytes` (multiple of 16, 16-byte aligned) from this CTA's
// shared memory to the same offset as dst_local in cluster rank `rank`,
// completing on that rank's copy of the mbarrier at bar_local
__device__ __forceinline__ void bulk_copy_to_rank(const void* dst_local, const void* src,
                                                  uint32_t bytes, uint64_t* bar_local,
                                                  uint32_t rank) {
  uint32_t dst, bar;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(dst) : "r"(smem_addr(dst_local)), "r"(rank));
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(bar) : "r"(smem_addr(bar_local)), "r"(rank));
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "r"(smem_addr(src)), "r"(bytes), "r"(bar)
      : "memory");
}

// One warp: acc = sum over k in [kb, ke) of A(m, k) B(k, n) for the 16 x 8
// tile at pa = &A(0, 0) of the tile, pb = &B(0, 0) of the tile, with
// A(m, k) = pa[m AM + k AK] and B(k, n) = pb[k BK + n BN].  Fragments of
// m16n8k8 (g = lane / 4, t = lane % 4): a = A(g|g+8, t|t+4), b = B(t|t+4, g),
// acc = C(g|g+8, 2t|2t+1).
template <int AM, int AK, int BK, int BN>
__device__ __forceinline__ void warp_tile_3xtf32(const float* __restrict__ pa,
                                                 const float* __restrict__ pb, int kb, int ke,
                                                 float (&acc)[4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f}, c2[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
  for (int k0 = kb; k0 < ke; k0 += 8) {
    const float av[4] = {pa[g * AM + (k0 + t) * AK], pa[(g + 8) * AM + (k0 + t) * AK],
                         pa[g * AM + (k0 + t + 4) * AK], pa[(g + 8) * AM + (k0 + t + 4) * AK]};
    const float bv[2] = {pb[(k0 + t) * BK + g * BN], pb[(k0 + t + 4) * BK + g * BN]};
    uint32_t ah[4], al[4], bh[2], bl[2];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      ah[q] = tf32_round(av[q]);
      al[q] = tf32_round(av[q] - __uint_as_float(ah[q]));
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      bh[q] = tf32_round(bv[q]);
      bl[q] = tf32_round(bv[q] - __uint_as_float(bh[q]));
    }
    mma_tf32(c0, ah, bh);
    mma_tf32(c1, ah, bl);
    mma_tf32(c2, al, bh);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = c0[q] + (c1[q] + c2[q]);
}

// Tile products of the step.  Warp w < TILES * KS owns tile w % TILES and
// half w / TILES of the K range (KS = 2); the halves meet in `part`.
// kProdGram:  A_blk = X^T X[:, c0 .. c0+NB)   (A(m=i, k=r) = X[i XLD + r])
// kProdTimes: P_blk = X B_blk                 (A(m=r, k=i) = X[i XLD + r])
enum StepProd : int { kProdGram = 0, kProdTimes = 1 };

template <int KP, int CL, int PROD>
__device__ __forceinline__ bool step_product(const float* __restrict__ X, const float* __restrict__ Bm,
                                             int c0, float* __restrict__ part, float (&acc)[4],
                                             int& m0, int& n0) {
  using S = StepSmem<KP, CL>;
  constexpr int XLD = S::XLD;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = warp % S::TILES, ks = warp / S::TILES;
  const bool active = warp < S::TILES * S::KS;
  m0 = (tile % S::MT) * 16;
  n0 = (tile / S::MT) * 8;
  const int kb = ks * (KP / S::KS), ke = kb + KP / S::KS;
  if (active) {
    if (PROD == kProdGram)
      warp_tile_3xtf32<XLD, 1, 1, XLD>(X + m0 * XLD, X + (c0 + n0) * XLD, kb, ke, acc);
    else
      warp_tile_3xtf32<1, XLD, 1, XLD>(X + m0, Bm + n0 * XLD, kb, ke, acc);
    if (S::KS == 2 && ks == 1) {
#pragma unroll
      for (int q = 0; q < 4; ++q) part[tile * 128 + q * 32 + lane] = acc[q];
    }
  }
  __syncthreads();
  if (!active || ks != 0) return false;
  if (S::KS == 2) {
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] += part[tile * 128 + q * 32 + lane];
  }
  return true;
}

template <int KP, int CL>
__global__ void __launch_bounds__(512, 1) stpm_step_kernel(StpmUpdateArgs a) {
  using S = StepSmem<KP, CL>;
  constexpr int NB = S::NB, XLD = S::XLD;
  static_assert(NB == 8 || NB == 16, "column block of 8 or 16");
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) float sm[];
  float* Xa = sm;
  float* Xb = Xa + KP * XLD;
  float* Ab = Xb + KP * XLD;      // B (or A) block, column jb at Ab + jb * XLD
  float* Gb = Ab + NB * XLD;      // G block (online step)
  float* Ot = Gb + NB * XLD;      // 2 staging tiles of the cluster broadcast
  float* part = Ot + 2 * NB * XLD;    // K-split partial tiles
  float* mv = part + S::TILES * 128;  // m1, m2, m3 (+ pad) for this block
  float* red = mv + 4 * KP;       // initial statistics of the CL ranks (3 x CL)
  float* dcol = red + 3 * CL;     // 3 * NB d-sums (online step)
  float* colabs = dcol + 3 * NB;  // NB column abs sums (+ NB spare)
  __shared__ float s_abs, s_err, s_fro;
  __shared__ __align__(8) uint64_t s_full[2];  // "next iterate arrived" for Xa / Xb
  const int k = a.k;
  const int c0 = rank * NB;
  const int tid = threadIdx.x, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
  for (int e = tid; e < KP * XLD; e += blockDim.x) {
    const int r = e % XLD, c = e / XLD;
    Xa[e] = (r < k && c < k) ? a.phi[(int64_t)c * k + r] : 0.f;
    Xb[e] = 0.f;
  }
  for (int e = tid; e < 2 * NB * XLD; e += blockDim.x) Ot[e] = 0.f;
  if (tid == 0) {
    mbar_init(&s_full[0], 1);
    mbar_init(&s_full[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  cluster.sync();  // Phi read and barriers initialised everywhere before any copy
  uint32_t parity[2] = {0u, 0u};
  int nbcast = 0;
  bool timed_out = false;

  float* X = Xa;   // current iterate
  float* dn = Xb;  // next iterate (the same offset in every CTA of the cluster)
  auto swap_buffers = [&]() {
    float* tt = X;
    X = dn;
    dn = tt;
  };
  // P = alpha X B_blk + beta_self X[:, blk] + gamma Gb, zero outside k x k,
  // staged (with this CTA's statistics s_abs, s_err, s_fro in the padding
  // rows KP.. of its first column) and sent to every rank's next buffer;
  // returns once the whole next iterate has arrived (false on a timeout)
  auto times_and_broadcast = [&](float alpha, float beta_self, const float* Gsrc, float gamma) {
    float* Otc = Ot + (nbcast & 1) * NB * XLD;
    ++nbcast;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    int m0, n0;
    if (step_product<KP, CL, kProdTimes>(X, Ab, c0, part, acc, m0, n0)) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        float v = alpha * acc[q] + beta_self * X[col * XLD + r];
        if (Gsrc) v += gamma * Gsrc[jb * XLD + r];
        Otc[jb * XLD + r] = (r < k && col < k) ? v : 0.f;
      }
    }
    if (tid == 0) {
      Otc[KP] = s_abs;
      Otc[KP + 1] = s_err;
      Otc[KP + 2] = s_fro;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // staging -> async proxy
    __syncthreads();
    const int bi = dn == Xa ? 0 : 1;
    if (tid < CL)
      bulk_copy_to_rank(dn + c0 * XLD, Otc, (uint32_t)(sizeof(float) * NB * XLD), &s_full[bi],
                        (uint32_t)tid);
    if (tid == 0) mbar_arrive_expect_tx(&s_full[bi], (uint32_t)(sizeof(float) * KP * XLD));
    const bool ok = mbar_wait_bounded(&s_full[bi], parity[bi]);
    parity[bi] ^= 1u;
    return !__syncthreads_or(!ok);
  };
  if (a.step_mode == kStepOnline) {
    // G block (columns c0 .. c0+NB) from the per-CTA partials, plus the mean
    // terms phi_i . mu (a warp per dot product, lanes along the k entries)
    for (int e = tid / 32; e < 3 * NB; e += blockDim.x / 32) {
      const int which = e / NB, jb = e % NB, i = c0 + jb;
      const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
      float sv = 0.f;
      if (i < k && mu)
        for (int j = lane; j < k; j += 32) sv = fmaf(X[i * XLD + j], mu[j], sv);
#pragma unroll
      for (int off = 16; off; off >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, off);
      if (lane == 0) mv[which * KP + jb] = sv;
    }
    __syncthreads();
    // per-column sums of the d partials (3 x NB), then the contraction block
    for (int e = tid / 32; e < 3 * NB; e += blockDim.x / 32) {
      const int which = e / NB, jb = e % NB, i = c0 + jb;
      float sd = 0.f;
      if (i < k && (which == 0 || a.mode == kModeAdjoint))
        for (int pp = tid % 32; pp < a.nparts; pp += 32)
          sd += a.gpart[(int64_t)pp * a.part_stride + (int64_t)k * k + which * k + i];
#pragma unroll
      for (int off = 16; off; off >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, off);
      if ((tid & 31) == 0) dcol[e] = sd;
    }
    __syncthreads();
    for (int e = tid; e < NB * KP; e += blockDim.x) {
      const int jb = e / KP, j = e % KP, i = c0 + jb;
      float gval = 0.f;
      if (i < k && j < k) {
        const float* gp = a.gpart + (int64_t)i * k + j;
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int pp = 0;
        for (; pp + 4 <= a.nparts; pp += 4) {
          s0 += gp[(int64_t)pp * a.part_stride];
          s1 += gp[(int64_t)(pp + 1) * a.part_stride];
          s2 += gp[(int64_t)(pp + 2) * a.part_stride];
          s3 += gp[(int64_t)(pp + 3) * a.part_stride];
        }
        for (; pp < a.nparts; ++pp) s0 += gp[(int64_t)pp * a.part_stride];
        float gv = ((s0 + s1) + (s2 + s3)) * (float)a.scale;
        const float m1 = mv[jb], m2 = mv[KP + jb], m3 = mv[2 * KP + jb];
        const float c1 = (float)a.c1, c2 = (float)a.c2;
        if (a.mode == kModePlain) {
          gv += a.mu3[j] * (c1 * m1 * m2 + c2 * dcol[jb]);
        } else {
          const float ic = (float)(1.0 / a.count);
          gv += a.mu1[j] * (c2 * dcol[jb] * ic + c1 * m2 * m3) +
                a.mu2[j] * (c2 * dcol[NB + jb] * ic + c1 * m1 * m3) +
                a.mu3[j] * (c2 * dcol[2 * NB + jb] * ic + c1 * m1 * m2);
        }
        gval = gv;
      }
      Gb[jb * XLD + j] = gval;
    }
    // Phi' = Phi - beta (3 theta Phi (Phi^T Phi)^.2 - gscale G)   (Util.cpp:259-272)
    {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      int m0, n0;
      if (step_product<KP, CL, kProdGram>(X, nullptr, c0, part, acc, m0, n0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1);
          Ab[jb * XLD + i] = acc[q] * acc[q];
        }
      }
      __syncthreads();
    }
    if (!times_and_broadcast(-a.beta * a.theta3, 1.f, Gb, a.beta * a.gscale)) timed_out = true;
    swap_buffers();
  }
  // Scaled Newton-Schulz polar iteration X <- X (3 a I - a^3 X^T X) / 2.
  // After the first scaling every singular value of X lies in [l, 1]; with
  // f(y) = 3y/2 - y^3/2 the step maps sigma to f(a sigma), and
  // a = sqrt(3 / (1 + l + l^2)) makes f(a l) = f(a), so the lower end grows by
  // up to sqrt(3) * 3/2 ~ 2.6x per iteration instead of 3/2 (the scaled
  // Newton-Schulz iteration; l starts from the guess kNsLowerGuess and is
  // tightened by sigma_min^2 >= 1 - ||X^T X - I||_F).  Once max|X^T X - I|
  // < kNsPlainBelow the plain step (a = 1) takes over: with X^T X = I + E the
  // next error is -3/4 E^2 + E^3/4, so after |E| < 1e-3 one more iteration
  // reaches the FP32 floor and the loop stops there.
  // One exchange per iteration: the statistics of A_t = X_t^T X_t travel
  // with the broadcast of X_{t+1}; if they show X_t had already converged,
  // X_{t+1} is discarded.  The scale of step t therefore uses
  // the statistics of A_{t-1}; every CTA derives the same a from the same
  // exchanged numbers.
  //
  // gram_stats: A_blk = X^T X[:, blk] with its statistics (max column abs
  // sum, max |A - I|, ||A - I||_F^2 over the block) in s_abs, s_err, s_fro,
  // and Ab = d0 I + d1 A_blk.
  auto gram_stats = [&](float d0, float d1) {
    if (tid < NB) colabs[tid] = 0.f;
    if (tid == 0) {
      s_err = 0.f;
      s_fro = 0.f;
    }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    int m0, n0;
    // (step_product's barrier also orders the resets above before the atomics)
    const bool own = step_product<KP, CL, kProdGram>(X, nullptr, c0, part, acc, m0, n0);
    if (own) {
      float er = 0.f, fr = 0.f, ca[2] = {0.f, 0.f};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        const float v = acc[q];
        const bool diag = i == col;
        if (i < k && col < k) {
          const float d = v - (diag ? 1.f : 0.f);
          er = fmaxf(er, fabsf(d));
          fr = fmaf(d, d, fr);
          ca[q & 1] += fabsf(v);
        }
        Ab[jb * XLD + i] = (diag ? d0 : 0.f) + d1 * v;
      }
#pragma unroll
      for (int off = 4; off < 32; off <<= 1) {  // over g: lanes with the same t4
        ca[0] += __shfl_xor_sync(0xffffffffu, ca[0], off);
        ca[1] += __shfl_xor_sync(0xffffffffu, ca[1], off);
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        er = fmaxf(er, __shfl_xor_sync(0xffffffffu, er, off));
        fr += __shfl_xor_sync(0xffffffffu, fr, off);
      }
      if (g == 0) {
        atomicAdd(&colabs[n0 + 2 * t4], ca[0]);
        atomicAdd(&colabs[n0 + 2 * t4 + 1], ca[1]);
      }
      if (lane == 0) {
        atomicMax(reinterpret_cast<int*>(&s_err), __float_as_int(er));
        atomicAdd(&s_fro, fr);
      }
    }
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      for (int jb = 0; jb < NB; ++jb) m = fmaxf(m, colabs[jb]);
      s_abs = m;
    }
    __syncthreads();
  };
  // initial statistics: rank q's [abs sum | max error | Frobenius^2] go to
  // red[q], red[CL + q], red[2 CL + q] of every rank
  auto post_stats = [&]() {
    if (tid < CL) {
      float* r = cluster.map_shared_rank(red, tid);
      r[rank] = s_abs;
      r[CL + rank] = s_err;
      r[2 * CL + rank] = s_fro;
    }
  };
  auto reduce_stats = [&](const float* src, int stride, float& gabs, float& gerr, float& gfro) {
    gabs = 0.f;
    gerr = 0.f;
    gfro = 0.f;
    for (int q = 0; q < CL; ++q) {
      gabs = fmaxf(gabs, src[q * stride]);
      gerr = fmaxf(gerr, src[q * stride + 1]);
      gfro += src[q * stride + 2];
    }
  };
  // initial scaling: sigma_max^2 <= ||X^T X||_1
  gram_stats(0.f, 1.f);
  post_stats();
  cluster.sync();
  int it = 0;
  bool done = timed_out, last = false;
  if (!done) {
    float gabs = 0.f, gerr = 0.f, gfro = 0.f;
    for (int q = 0; q < CL; ++q) {
      gabs = fmaxf(gabs, red[q]);
      gerr = fmaxf(gerr, red[CL + q]);
      gfro += red[2 * CL + q];
    }
    if (!(gerr == gerr) || !(gabs == gabs)) {
      if (tid == 0 && rank == 0) atomicOr(a.flags, kFlagNonFinite);
      done = true;
    } else if (gerr < a.ns_tol) {
      done = true;
    } else if (gabs > 0.f) {
      const float sc = rsqrtf(gabs);
      for (int e = tid; e < KP * XLD; e += blockDim.x) X[e] *= sc;
      __syncthreads();
    }
  }
  cluster.sync();  // every CTA has read the statistics slots
  float lo = kNsLowerGuess;  // lower bound (guess at first) on sigma(X_t)
  float prev_err = 1e30f;    // max|A_{t-1} - I|
  for (; !done && it < a.max_ns; ++it) {
    const float al = prev_err < kNsPlainBelow ? 1.f : fminf(sqrtf(3.f / (1.f + lo + lo * lo)), kNsMaxScale);
    // A_t, its statistics and the speculative B_t in one pass
    gram_stats(1.5f * al, -0.5f * al * al * al);
    if (!times_and_broadcast(1.f, 0.f, nullptr, 0.f)) {
      timed_out = true;
      break;
    }
    float gabs, gerr, gfro;
    reduce_stats(dn + KP, NB * XLD, gabs, gerr, gfro);  // A_t's statistics, from every rank
    if (!(gerr == gerr) || !(gabs == gabs) || !(gfro == gfro)) {
      if (tid == 0 && rank == 0) atomicOr(a.flags, kFlagNonFinite);
      done = true;
      break;
    }
    if (gerr < a.ns_tol) {  // X_t was converged: keep it, drop X_{t+1}
      done = true;
      break;
    }
    // bound for X_{t+1}: [lb, 1] -> [min(f(a lb), f(a)), 1]
    const float lb = fmaxf(lo, sqrtf(fmaxf(0.f, 1.f - sqrtf(gfro))));
    lo = al > 1.f ? fminf(ns_poly(al * lb), ns_poly(al)) : ns_poly(lb);
    prev_err = gerr;
    swap_buffers();
    if (last) {
      done = true;
      ++it;
      break;
    }
    if (gerr < 1e-3f) last = true;
  }
  if (timed_out) {
    if (tid == 0) atomicOr(a.flags, kFlagTimeout);
  } else if (!done && rank == 0 && tid == 0) {
    atomicOr(a.flags, kFlagNoConvergence);
  }
  if (rank == 0 && tid == 0 && a.ns_iters) atomicAdd(a.ns_iters, it);
  for (int e = tid; e < KP * NB; e += blockDim.x) {
    const int r = e % KP, col = c0 + e / KP;
    if (r < k && col < k) a.phi[(int64_t)col * k + r] = X[col * XLD + r];
  }
  cluster.sync();  // keep shared memory alive until remote writers are done
  if (timed_out) __nanosleep(100000);  // let copies a stalled exchange left in flight land
}

// batch power: Phi_new = G (already includes the shift terms), lambda = ||col||^3,
// column normalisation, error = ||Phi_new - Phi_old||_F
__global__ void __launch_bounds__(1024) batch_update_kernel(int k, float* __restrict__ phi,
                                                            const float* __restrict__ G,
                                                            double* __restrict__ lambda,
                                                            double* __restrict__ err_out) {
  __shared__ double nrm[256];
  __shared__ double errsum;
  const int tid = threadIdx.x;
  if (tid == 0) errsum = 0.0;
  for (int i = tid; i < k; i += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += (double)G[(int64_t)i * k + j] * G[(int64_t)i * k + j];
    nrm[i] = sqrt(s);
    lambda[i] = s * sqrt(s);
  }
  __syncthreads();
  double e = 0.0;
  for (int idx = tid; idx < k * k; idx += blockDim.x) {
    const int i = idx / k;
    const double v = (double)G[idx] / nrm[i];
    const double d = v - (double)phi[idx];
    e += d * d;
    phi[idx] = (float)v;
  }
  atomicAdd(&errsum, e);
  __syncthreads();
  if (tid == 0) err_out[0] = sqrt(errsum);
}

// lambda_i = phi_i . G_i (tensor value); sign fix so lambda_i > 0
__global__ void tensor_value_kernel(int k, float* __restrict__ phi, const float* __restrict__ G,
                                    double* __restrict__ lambda) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (i >= k) return;
  double s = 0.0;
  for (int j = lane; j < k; j += 32) s += (double)phi[(int64_t)i * k + j] * G[(int64_t)i * k + j];
#pragma unroll
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  const bool flip = s < 0.0;
  if (lane == 0) lambda[i] = flip ? -s : s;
  if (flip)
    for (int j = lane; j < k; j += 32) phi[(int64_t)i * k + j] = -phi[(int64_t)i * k + j];
}

template <int KP, int MODE>
cudaError_t launch_partial_t(const StpmPartialArgs& a, int grid, cudaStream_t s) {
  const size_t smem = stpm_partial_smem(KP, MODE);
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_partial_kernel<KP, MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3(256, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kPartialCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_partial_kernel<KP, MODE>, a));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_partial_m(int KP, const StpmPartialArgs& a, int grid, cudaStream_t s) {
  switch (KP) {
    case 32: return launch_partial_t<32, MODE>(a, grid, s);
    case 48: return launch_partial_t<48, MODE>(a, grid, s);
    case 64: return launch_partial_t<64, MODE>(a, grid, s);
    case 80: return launch_partial_t<80, MODE>(a, grid, s);
    case 96: return launch_partial_t<96, MODE>(a, grid, s);
    case 112: return launch_partial_t<112, MODE>(a, grid, s);
    case 128: return launch_partial_t<128, MODE>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int KP, int CL>
cudaError_t launch_step_t(const StpmUpdateArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(float) * StepSmem<KP, CL>::floats;
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_step_kernel<KP, CL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (CL > 8)
      MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_step_kernel<KP, CL>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL, 1, 1);
  cfg.blockDim = dim3(512, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_step_kernel<KP, CL>, a));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int KP>
cudaError_t launch_step_k(const StpmUpdateArgs& a, cudaStream_t s) {
  // KP / 8 CTAs (8 columns each; up to 16, a non-portable cluster size) where
  // the device can co-schedule them, else KP / 16 CTAs of 16 columns
  static int wide = -1;
  if (wide != 0) {
    cudaError_t e = launch_step_t<KP, KP / 8>(a, s);
    if (e == cudaSuccess) {
      wide = 1;
      return e;
    }
    if (wide == 1) return e;
    cudaGetLastError();
    wide = 0;
  }
  return launch_step_t<KP, KP / 16>(a, s);
}

}  // namespace

int stpm_partial_cluster() { return kPartialCluster; }

int stpm_kp(int k) { return (int)round_up(k, 16) < 32 ? 32 : (int)round_up(k, 16); }

size_t stpm_partial_smem(int KP, int mode) {
  const int LD = ys_ld(KP);
  const int ncs = mode == kModePlain ? 1 : 3;
  return sizeof(float) * ((size_t)KP * KP + (size_t)3 * TN * LD + (size_t)ncs * TN * LD + 3 * KP +
                          3 * KP);
}

int stpm_partial_grid(int64_t count) {
  const int64_t tiles = ceil_div(count, TN);
  const int64_t g = std::max<int64_t>(1, std::min<int64_t>(tiles, 2 * kNumSMs));
  return (int)round_up(g, kPartialCluster);
}

cudaError_t stpm_partial(int mode, const StpmPartialArgs& a, int grid, cudaStream_t s) {
  const int KP = stpm_kp(a.k);
  if (KP > 128) return cudaErrorInvalidValue;
  switch (mode) {
    case kModePlain: return launch_partial_m<kModePlain>(KP, a, grid, s);
    case kModeAdjoint: return launch_partial_m<kModeAdjoint>(KP, a, grid, s);
    case kModeLoss: return launch_partial_m<kModeLoss>(KP, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t stpm_reduce(const StpmReduceArgs& a, cudaStream_t s) {
  const int64_t kk = (int64_t)a.k * a.k;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(2 * kNumSMs, ceil_div(kk, 256)));
  stpm_reduce_kernel<<<grid, 256, sizeof(double) * 6 * a.k, s>>>(a);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t stpm_update(const StpmUpdateArgs& a, cudaStream_t s) {
  switch (stpm_step_kp(a.k)) {
    case 32: return launch_step_k<32>(a, s);
    case 48: return launch_step_k<48>(a, s);
    case 64: return launch_step_k<64>(a, s);
    case 80: return launch_step_k<80>(a, s);
    case 96: return launch_step_k<96>(a, s);
    case 112: return launch_step_k<112>(a, s);
    case 128: return launch_step_k<128>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

int stpm_step_kp(int k) { return k <= 32 ? 32 : (int)round_up(k, 16); }

cudaError_t stpm_batch_update(int k, float* phi, const float* G, double* lambda, double* err,
                              cudaStream_t s) {
  batch_update_kernel<<<1, 1024, 0, s>>>(k, phi, G, lambda, err);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t stpm_tensor_values(int k, float* phi, const float* G, double* lambda, cudaStream_t s) {
  tensor_value_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, s>>>(k, phi, G, lambda);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
