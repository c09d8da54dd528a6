// Tensor power method kernels (FP32 form and BF16 form).
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
// The contraction runs on the tensor cores (stpm_contract_kernel); partials
// of 8-CTA clusters are summed through distributed shared memory and reduced
// deterministically by stpm_reduce or by the step kernel.  The k x k update
// (orthogonality term, step, Newton-Schulz polar orthonormalisation) runs on
// one cluster of KP / 8 CTAs exchanging column blocks by bulk copies.
#include "common.cuh"

#include <cstdlib>
#include "k_stpm.cuh"
#include "tc_util.cuh"

#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <type_traits>

namespace cg = cooperative_groups;

namespace mmsb {

namespace {

constexpr int kPartialCluster = 8;  // CTAs whose partials are summed through DSMEM

__device__ __forceinline__ int64_t ceil_div_dev(int64_t a, int64_t b) { return (a + b - 1) / b; }

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
    for (int p = 0; p < a.nparts; ++p)  // one loss slot per contraction column block
      for (int sl = 0; sl < 4; ++sl) t += (double)a.gpart[(int64_t)p * a.part_stride + kk + 3 * k + sl];
    double that = t / a.count;
    for (int i = 0; i < k; ++i) that += a.c1 * m[i] * m[k + i] * m[2 * k + i];
    a.loss_out[0] = that;  // sum_i That(phi_i, phi_i, phi_i)
  }
}

// ---- k x k step on one thread-block cluster -------------------------------------
//
// The update of one minibatch step (Diff_Loss, CPU/Util.cpp:257-284, as the
// GPU tree applies it at GPU/stpm.c:649-691, then its re-orthonormalisation
// by culaDeviceDgeqrfp + culaDeviceDorgqr, GPU/stpm.c:783-784):
//
//   X   = Phi - beta (3 theta Phi (Phi^T Phi)^.2 - gscale G)
//   Phi = Q  of  X = Q R  with R upper triangular, diag(R) > 0
//
// Q is computed by Cholesky QR: A = X^T X = R1^T R1 (Cholesky), Q1 = X R1^-1,
// then E = Q1^T Q1 - I and Q = Q1 (I - F) with F upper triangular,
// F + F^T = E (F = strict upper part of E plus half its diagonal), which is
// the second Cholesky QR pass to first order in E.  Every factor applied to X
// from the right is upper triangular with a positive diagonal, so Q is the
// Q of the QR factorisation with diag(R) > 0 (it is unique), the factor the
// reference forms.  When a pivot of the Cholesky shows that X's columns are
// far from independent (R_jj^2 / A_jj below kQrExactBelow; the loss of
// orthogonality of one pass grows like eps / that ratio), further exact
// Cholesky QR passes run on Q1 before the first-order step.  When a pivot
// has lost (nearly) all its digits (ratio below kShiftBelow: the FP32 Gram
// squares cond(X), which reaches 1e4 - 2e5 in the first sweep of the
// benchmarked workloads, beyond 1 / sqrt(eps)), the Gram is formed again
// and factored with a diagonal shift s = kShiftScale trace(A) (shifted
// Cholesky QR, Fukaya et al., SIAM J. Sci. Comput. 42 (2020)): A + s I is
// safely positive definite, Q1 = X R_s^-1 has cond ~ sqrt(s) / sigma_min, and
// the plain passes that follow orthonormalise it.  Every CTA of the cluster
// computes the same Cholesky from the same data, so the pass count needs no
// vote.
//
// Layout: every CTA holds whole k x k matrices (column-major, leading
// dimension KP + 4) and owns NB = 8 or 16 columns.  The products
// X^T Y[:, blk] (Gram) and X B_blk (times) run on the tensor cores as
// warp-level m16n8k8 TF32 MMAs with the 3xTF32 split (a = a_hi + a_lo;
// hi*hi + hi*lo + lo*hi accumulated in FP32, relative error ~1e-6 per
// product; the first-order correction M F, |F| <= ~1e-5, as one TF32
// product), one warp per 16 x 8 output tile.  A CTA's new column block is
// staged in shared memory and sent to every CTA by bulk asynchronous copies
// (cp.async.bulk shared::cta -> shared::cluster) that complete on the
// receiver's per-block mbarrier; a CTA proceeds once all CL blocks have
// arrived.  A staging tile used for broadcast n is rewritten at broadcast
// n + 2 only, after every receiver has waited for broadcast n + 1 (sent by
// each rank after it received all of broadcast n).
//
// Hardware barriers of the step kernel's CTA: 0 = __syncthreads (whole CTA),
// 1 = the four panel warps of inverse_columns (128 threads), 2 = the block-row
// release of chol_blocked (warp 0 arrives, the other warps sync; whole CTA).
// The three are never in use at the same time.

// pivot ratio R_jj^2 / A_jj below which one more exact Cholesky QR pass runs
// (one pass leaves Q1^T Q1 - I of about eps / ratio times a small constant, and
// the first-order pass squares it), the floor a pivot below FP32 round-off of
// A_jj is raised to (a column numerically dependent on the ones before it:
// the floor keeps R^-1 bounded, the next pass orthonormalises); the largest
// number of plain exact passes per step is StpmUpdateArgs::max_passes
constexpr float kQrExactBelow = 1e-2f;
constexpr float kPivotFloor = 1e-7f;
// shifted restarts: below this pivot ratio the factorisation is redone with
// the shift kShiftScale trace(A) (times 100 for each further restart, at
// most kMaxShifts)
constexpr float kShiftBelow = 1e-5f;
constexpr float kShiftScale = 1e-5f;
constexpr int kMaxShifts = 3;

// column stride of the k x k matrices: KP + 4 (== 4 mod 8 for KP a multiple
// of 16) makes the fragment loads of the Gram product conflict-free
__host__ __device__ constexpr int step_xld(int KP) { return KP + 4; }

// NB = 8 (one n-tile) when the cluster has KP / 8 CTAs, else 16.  Above
// KP = 128 two FP32 copies of a k x k matrix no longer fit one SM (SB: a
// single buffer, refilled after a cluster barrier, one staging tile, the
// second tile holding the G block and then the inverse diagonal blocks of
// the Cholesky factor; a matrix still needed after the buffer is refilled
// is kept in global memory, StpmUpdateArgs::xstash).
template <int KP, int CL>
struct StepSmem {
  static constexpr int NB = KP / CL, XLD = step_xld(KP), MT = KP / 16, NT = NB / 8;
  static constexpr int TILES = MT * NT, KS = TILES <= 8 ? 2 : 1;  // K split over warps
  static constexpr bool SB = KP > 128;
  static constexpr int NBK = KP / 8;  // 8-column blocks of the Cholesky factor
  static constexpr size_t full = (size_t)(SB ? 1 : 2) * KP * XLD;
  static constexpr size_t tiles = (size_t)4 * NB * XLD;  // B block, 2 staging tiles, G block
  static constexpr size_t kpart = KS == 2 ? (size_t)TILES * 128 : 0;
  // mean terms, d-sums, |phi_i|^2, mu1..3, tmp
  static constexpr size_t small = 6 * KP + 4 * NB + 128 + 8;
  // inverse diagonal blocks and superblock corners (SB: in the G block's tile)
  static constexpr size_t tinv = SB ? 0 : (size_t)64 * NBK + 64 * (KP / 16);
  static constexpr size_t floats = full + tiles - (SB ? NB * XLD : 0) + kpart + small + tinv +
                                   2 * KP;  // original diagonal, 1 / R_jj
  static_assert(!SB || (size_t)64 * NBK + 64 * (KP / 16) <= (size_t)NB * XLD,
                "inverse blocks in the G tile");
  static_assert(floats * sizeof(float) <= 227 * 1024 - 2048, "step kernel shared memory");
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

// waits for the phase with the given parity to complete; false after `limit`
// clock64 cycles (then the caller reports kFlagTimeout instead of hanging)
// global -> this CTA's shared memory, completing on `bar` (16-byte aligned
// addresses, bytes a multiple of 16)
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  long long limit) {
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
    if (clock64() - start > limit) return false;
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
// acc = C(g|g+8, 2t|2t+1).  SPLIT = false: one TF32 product (for a small
// correction term whose relative error may be ~1e-3).
template <int AM, int AK, int BK, int BN, bool SPLIT = true>
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
      al[q] = __float_as_uint(av[q] - __uint_as_float(ah[q]));  // the MMA reads its top 19 bits
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      bh[q] = tf32_round(bv[q]);
      bl[q] = __float_as_uint(bv[q] - __uint_as_float(bh[q]));
    }
    mma_tf32(c0, ah, bh);
    if (SPLIT) {
      mma_tf32(c1, ah, bl);
      mma_tf32(c2, al, bh);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = SPLIT ? c0[q] + (c1[q] + c2[q]) : c0[q];
}

// Tile products of the step.  Warp w < TILES * KS owns tile w % TILES and
// half w / TILES of the K range (KS = 2); the halves meet in `part`.
// kProdGram:  C_blk = X^T Y[:, c0 .. c0+NB)   (A(m=i, k=r) = X[i XLD + r], B = Y block)
// kProdTimes: C_blk = X B_blk                 (A(m=r, k=i) = X[i XLD + r])
// epi(acc, m0, n0) receives each finished 16 x 8 tile.
enum StepProd : int { kProdGram = 0, kProdTimes = 1 };

template <int KP, int CL, int PROD, bool SPLIT = true, typename Epi>
__device__ __forceinline__ void step_tiles(const float* __restrict__ X, const float* __restrict__ Bm,
                                           float* part, Epi&& epi) {
  using S = StepSmem<KP, CL>;
  constexpr int XLD = S::XLD;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  auto product = [&](int tile, int kb, int ke, float (&acc)[4]) {
    const int m0 = (tile % S::MT) * 16, n0 = (tile / S::MT) * 8;
    if (PROD == kProdGram)
      warp_tile_3xtf32<XLD, 1, 1, XLD, SPLIT>(X + m0 * XLD, Bm + n0 * XLD, kb, ke, acc);
    else
      warp_tile_3xtf32<1, XLD, 1, XLD, SPLIT>(X + m0, Bm + n0 * XLD, kb, ke, acc);
  };
  if (S::KS == 2) {
    const int tile = warp % S::TILES, ks = warp / S::TILES;
    const bool active = warp < S::TILES * S::KS;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    if (active) {
      product(tile, ks * (KP / 2), ks * (KP / 2) + KP / 2, acc);
      if (ks == 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) part[tile * 128 + q * 32 + lane] = acc[q];
      }
    }
    __syncthreads();
    if (!active || ks != 0) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] += part[tile * 128 + q * 32 + lane];
    epi(acc, (tile % S::MT) * 16, (tile / S::MT) * 8);
  } else {
    for (int tile = warp; tile < S::TILES; tile += nw) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      product(tile, 0, KP, acc);
      epi(acc, (tile % S::MT) * 16, (tile / S::MT) * 8);
    }
  }
}

// ---- Cholesky factor and its inverse on one CTA ----------------------------------
//
// A (KP x KP symmetric, column-major, leading dimension XLD, upper triangle
// read) = R^T R with R upper triangular, blocked by 8 columns (right-looking,
// one block of look-ahead).  Per block J: every thread forms one column of
// the block row R_J = R_JJ^-T A_J by forward substitution; then warp 0,
// which formed the block row's first 8 columns itself, goes straight on to
// update the next 8 x 8 diagonal block, and one thread factors it in
// registers (no shuffles on the pivot chain), while the other warps wait at
// a named barrier for the whole block row and update the rest of the
// trailing upper triangle with 3xTF32 tensor-core tiles (a rank-8 update is
// one k-step); one CTA barrier closes the block.  R overwrites A's upper
// triangle, 1 / R_jj goes to rd; the inverses T_JJ = R_JJ^-1 of the diagonal
// blocks (tinv, 8 x 8 column-major each) are formed afterwards, one block per
// thread, off the pivot chain.  Rows and columns >= k must hold the identity
// (the caller sets their diagonal to 1; X's padding columns are zero).

// One thread: the (already updated) 8 x 8 diagonal block at (j0, j0).  A
// pivot that is not above kPivotFloor * dg (breakdown, or NaN) is raised to
// it and counted as ratio 0.  Returns the smallest ratio R_jj^2 / dg[j] over
// the live columns j0 + j < k.
template <int XLD>
__device__ __forceinline__ float factor_diag8(float* A, int j0, int k, float* rd, const float* dg) {
  float a[8][8];
#pragma unroll
  for (int l = 0; l < 8; ++l)
#pragma unroll
    for (int i = 0; i <= l; ++i) a[i][l] = A[(j0 + i) + (j0 + l) * XLD];
  float rmin = 1.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float d = a[j][j];
    const float d0 = dg[j0 + j];
    float ratio = __fdividef(d, d0);
    if (!(d > kPivotFloor * d0)) {
      d = kPivotFloor * d0;
      ratio = 0.f;
    }
    if (j0 + j < k) rmin = fminf(rmin, ratio);
    const float ri = rsqrtf(d);
    rd[j0 + j] = ri;
    a[j][j] = d * ri;
#pragma unroll
    for (int l = j + 1; l < 8; ++l) a[j][l] *= ri;
#pragma unroll
    for (int i = j + 1; i < 8; ++i)
#pragma unroll
      for (int l = i; l < 8; ++l) a[i][l] = fmaf(-a[j][i], a[j][l], a[i][l]);
  }
#pragma unroll
  for (int l = 0; l < 8; ++l)
#pragma unroll
    for (int i = 0; i <= l; ++i) A[(j0 + i) + (j0 + l) * XLD] = a[i][l];
  return rmin;
}

// One thread: T = R_JJ^-1 (upper, 8 x 8 column-major into tb) of the
// diagonal block at (j0, j0), column by column: T(j, j) = 1 / R_jj,
// T(m, j) = -(sum_{m <= i < j} T(m, i) R(i, j)) / R(j, j).
template <int XLD>
__device__ __forceinline__ void invert_diag8(const float* A, int j0, const float* rd, float* tb) {
  float r[8][8], t[8][8];
#pragma unroll
  for (int l = 0; l < 8; ++l)
#pragma unroll
    for (int i = 0; i < l; ++i) r[i][l] = A[(j0 + i) + (j0 + l) * XLD];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float rv = rd[j0 + j];
    t[j][j] = rv;
#pragma unroll
    for (int m = 0; m < j; ++m) {
      float s = 0.f;
#pragma unroll
      for (int i = m; i < j; ++i) s = fmaf(t[m][i], r[i][j], s);
      t[m][j] = -s * rv;
    }
  }
#pragma unroll
  for (int l = 0; l < 8; ++l)
#pragma unroll
    for (int i = 0; i < 8; ++i) tb[i + 8 * l] = i <= l ? t[i][l] : 0.f;
}

// Whole CTA.  Returns the smallest pivot ratio (the same value in every
// thread: every CTA of a cluster factors the same matrix the same way).
// (No __restrict__ on these shared-memory pointers: other threads write what
// a thread reads after each barrier, and the ratio decides the control flow
// of the whole CTA, so no load may be moved across a barrier.  With
// __restrict__ the compiler did move the read of the ratio above the
// barrier: warps left the pass loop apart and the kernel hung.)
template <int KP>
__device__ float chol_blocked(float* A, int k, float* tinv, float* rd, float* dg,
                              volatile float* s_ratio, float shift = 0.f) {
  constexpr int XLD = step_xld(KP), NBK = KP / 8;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
  const int nw = blockDim.x >> 5;
  for (int i = tid; i < KP; i += blockDim.x) {
    float d = A[i + i * XLD] + shift;
    if (i >= k) d = 1.f;
    A[i + i * XLD] = d;
    dg[i] = fmaxf(d, 1e-30f);
  }
  __syncthreads();
  float rmin = 1.f;
  if (tid == 0) rmin = factor_diag8<XLD>(A, 0, k, rd, dg);
  __syncthreads();
  for (int J = 0; J + 1 < NBK; ++J) {
    const int j0 = 8 * J, rest = KP - j0 - 8;
    // block row: R(j0 + a, c) = (A(j0 + a, c) - sum_{b < a} R(j0 + b, j0 + a)
    // R(j0 + b, c)) / R(j0 + a, j0 + a), c >= j0 + 8 (a thread per column)
    for (int e = tid; e < rest; e += blockDim.x) {
      const int c = j0 + 8 + e;
      float x[8];
#pragma unroll
      for (int b = 0; b < 8; ++b) x[b] = A[(j0 + b) + c * XLD];
#pragma unroll
      for (int aa = 0; aa < 8; ++aa) {
        float s = x[aa];
#pragma unroll
        for (int b = 0; b < aa; ++b) s = fmaf(-A[(j0 + b) + (j0 + aa) * XLD], x[b], s);
        x[aa] = s * rd[j0 + aa];
      }
#pragma unroll
      for (int b = 0; b < 8; ++b) A[(j0 + b) + c * XLD] = x[b];
    }
    // trailing update of the upper triangle, A(c, c') -= sum_b R(j0+b, c)
    // R(j0+b, c') for j0 + 8 <= c <= c'
    const int n0 = j0 + 8;
    if (warp == 0) {
      // the next diagonal block needs only the block row's columns n0 ..
      // n0+7, which lanes 0-7 of this warp formed: the other warps are
      // released through barrier 2 (arrive: release), and this warp goes on
      // with the diagonal block and its factorisation at once
      asm volatile("bar.arrive 2, %0;" ::"r"(nw * 32) : "memory");
      __syncwarp();
      float sv[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int e = lane + 32 * h, i = e & 7, l = e >> 3;
        sv[h] = A[(n0 + i) + (n0 + l) * XLD];
#pragma unroll
        for (int b = 0; b < 8; ++b)
          sv[h] = fmaf(-A[(j0 + b) + (n0 + i) * XLD], A[(j0 + b) + (n0 + l) * XLD], sv[h]);
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int e = lane + 32 * h, i = e & 7, l = e >> 3;
        if (i <= l) A[(n0 + i) + (n0 + l) * XLD] = sv[h];
      }
      __syncwarp();
      if (lane == 0) rmin = fminf(rmin, factor_diag8<XLD>(A, n0, k, rd, dg));
    } else {
      asm volatile("bar.sync 2, %0;" ::"r"(nw * 32) : "memory");  // every block-row column
    }
    if (warp != 0 && rest > 8) {
      // columns c' >= n0 + 8 in 8-wide tiles, rows c in [n0, c'] in 16-row
      // tiles from mb; a last tile that would pass KP is computed at KP - 16
      // (rows below mb not written), so no read leaves the matrix
      const int mt = (rest + 15) / 16, ntl = (rest - 8) / 8;
      for (int tl = warp - 1; tl < mt * ntl; tl += nw - 1) {
        const int mb = n0 + 16 * (tl % mt), nc0 = n0 + 8 + 8 * (tl / mt);
        if (mb > nc0 + 7) continue;  // entirely below the diagonal
        const int m0 = min(mb, KP - 16);
        float acc[4];
        warp_tile_3xtf32<XLD, 1, 1, XLD>(A + j0 + m0 * XLD, A + j0 + nc0 * XLD, 0, 8, acc);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = m0 + g + ((q & 2) ? 8 : 0), c = nc0 + 2 * t4 + (q & 1);
          if (r >= mb && r <= c) A[r + c * XLD] -= acc[q];
        }
      }
    }
    __syncthreads();
  }
  // the inverses of the diagonal blocks, one block per thread
  for (int J = tid; J < NBK; J += blockDim.x) invert_diag8<XLD>(A, 8 * J, rd, tinv + 64 * J);
  if (tid == 0) *s_ratio = rmin;
  __syncthreads();
  return *s_ratio;
}

// Columns c0 .. c0+NB of W = R^-1 (NB = 8 or 16: whole 8-column blocks) into
// Wb (column jb at Wb + jb * XLD, rows past the diagonal block zero), by
// block back substitution per 8-column block K: W_KK = T_KK, then upwards in
// levels of 16 rows aligned to 16 (one 8-row level first when K is odd):
// W_Q = -T_Q S_Q with S_Q = sum over the rows P below Q of R_QP W_PK, where
// for a 16-row superblock Q = (a, b) of 8-row blocks T_Q = [T_a X; 0 T_b],
// X = -T_a R_ab T_b (x16, 8 x 8 column-major per superblock, formed here
// first).  One barrier per level: warps 0-3 add the last term of S_Q and
// apply -T_Q (a named barrier between the two), while the other warps add
// R_rP W_PK of the last level into the partial sums of the rows above
// (held in Wb until their level).  The levels of the last column block are
// about KP / 16 instead of KP / 8, which is what the cluster waits for.
// Blocks that lie wholly in the padding (8K >= k: R is the identity there)
// get unit columns.  tmp: 128 floats.  Whole CTA of at least 5 warps; ends
// with a barrier.
template <int KP, int NB>
__device__ void inverse_columns(const float* R, const float* tinv, float* x16, int c0, int k,
                                float* Wb, float* tmp) {
  constexpr int XLD = step_xld(KP), NSB = KP / 16;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < NB * XLD; e += nt) Wb[e] = 0.f;
  // X(a, b) = -sum_i T_2m(a, i) sum_j R(16m + i, 16m + 8 + j) T_2m+1(j, b)
  // (the T blocks hold explicit zeros below their diagonals; the R reads of
  // a warp are broadcasts)
  for (int e = tid; e < NSB * 64; e += nt) {
    const int m = e >> 6, aa = e & 7, b = (e >> 3) & 7, r0 = 16 * m;
    const float* ta = tinv + 64 * (2 * m);
    const float* tb = ta + 64;
    float tv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) tv[j] = tb[j + 8 * b];
    float x = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float y = 0.f;
#pragma unroll
      for (int j = 0; j < 8; ++j) y = fmaf(R[(r0 + i) + (r0 + 8 + j) * XLD], tv[j], y);
      x = fmaf(ta[aa + 8 * i], y, x);
    }
    x16[e] = -x;
  }
#pragma unroll 1
  for (int sb = 0; sb < NB / 8; ++sb) {
    const int K = c0 / 8 + sb;
    float* W = Wb + 8 * sb * XLD;
    __syncthreads();  // zero fill, X and the previous column block done
    if (8 * K >= k) {
      if (tid < 8) W[8 * K + tid + tid * XLD] = 1.f;
      continue;
    }
    for (int e = tid; e < 64; e += nt) {
      const int aa = e & 7, jb = e >> 3;
      W[8 * K + aa + jb * XLD] = tinv[64 * K + e];  // W_KK = T_KK (column-major)
    }
    __syncthreads();
    int lo = 8 * K, h = 8;  // rows [lo, lo + h) were the last level
    while (lo > 0) {
      const int hn = (lo & 15) ? 8 : 16, nlo = lo - hn;
      if (tid < 128) {
        // S_Q (row i, column jb) = partial sum + R(nlo + i, lo ..) W(lo .., jb)
        const int i = tid & 15, jb = tid >> 4;
        if (i < hn) {
          float sv = W[nlo + i + jb * XLD];
#pragma unroll
          for (int b = 0; b < 8; ++b) sv = fmaf(R[(nlo + i) + (lo + b) * XLD], W[lo + b + jb * XLD], sv);
          if (h == 16) {
#pragma unroll
            for (int b = 8; b < 16; ++b) sv = fmaf(R[(nlo + i) + (lo + b) * XLD], W[lo + b + jb * XLD], sv);
          }
          tmp[i + 16 * jb] = sv;
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (i < hn) {
          const float* s = tmp + 16 * jb;
          float w = 0.f;
          // T rows from the diagonal on (zeros below it are stored)
          const int ii = i & 7;
          const float* t = tinv + 64 * (nlo / 8 + (i >> 3));
          const float* sv = s + (i & 8);
#pragma unroll
          for (int b = 0; b < 8; ++b) w = fmaf(t[ii + 8 * b], sv[b], w);
          if (hn == 16 && i < 8) {
            const float* x = x16 + 64 * (nlo / 16) + i;
#pragma unroll
            for (int j = 0; j < 8; ++j) w = fmaf(x[8 * j], s[8 + j], w);
          }
          W[nlo + i + jb * XLD] = -w;
        }
      } else {
        // rows above the level accumulate R(r, lo ..) W(lo .., jb)
        for (int e = tid - 128; e < nlo * 8; e += nt - 128) {
          const int r = e % nlo, jb = e / nlo;
          float sv = W[r + jb * XLD];
#pragma unroll
          for (int b = 0; b < 8; ++b) sv = fmaf(R[r + (lo + b) * XLD], W[lo + b + jb * XLD], sv);
          if (h == 16) {
#pragma unroll
            for (int b = 8; b < 16; ++b) sv = fmaf(R[r + (lo + b) * XLD], W[lo + b + jb * XLD], sv);
          }
          W[r + jb * XLD] = sv;
        }
      }
      __syncthreads();
      h = hn;
      lo = nlo;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint64_t* bar, uint32_t parity,
                                                          long long limit) {
  const long long start = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - start > limit) return false;
  }
}

template <int KP>
struct ContractTc;  // the tensor-core contraction's shared-memory layout (below)

template <int KP, int CL>
__device__ __forceinline__ void step_body(const StpmUpdateArgs& a) {
  using S = StepSmem<KP, CL>;
  constexpr int NB = S::NB, XLD = S::XLD;
  static_assert(NB == 8 || NB == 16, "column block of 8 or 16");
  // one warp of the 512 threads issues the copy to each rank
  static_assert(CL <= 16 && S::TILES <= 32, "cluster or tile count");
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) float sm[];
  float* Xa = sm;
  float* Xb = S::SB ? Xa : Xa + KP * XLD;
  float* Ab = Xa + S::full;                       // B block of the products, column jb at Ab + jb * XLD
  float* Ot = Ab + NB * XLD;                      // staging tile(s) of the broadcasts
  float* Gb = Ot + (S::SB ? 1 : 2) * NB * XLD;    // G block (online step)
  float* part = Gb + NB * XLD;                    // K-split partial tiles
  float* mv = part + S::kpart;                    // m1, m2, m3 of this block
  float* dcol = mv + 3 * KP;                      // 3 * NB d-sums
  float* nn = dcol + 3 * NB;                      // |phi_i|^2 of this block
  float* mus = nn + NB;                           // mu1, mu2, mu3 (KP each)
  float* tmp = mus + 3 * KP;                      // 128 (inverse columns)
  float* tinv = S::SB ? Gb : tmp + 128 + 8;       // 8 x 8 inverse diagonal blocks
  float* x16 = tinv + 64 * S::NBK;                // corners of the 16 x 16 inverse blocks
  float* dg = (S::SB ? tmp + 128 + 8 : x16 + 64 * (KP / 16));  // original diagonal
  float* rd = dg + KP;                            // 1 / R_jj
  __shared__ float s_ratio;
  __shared__ float s_emax[16];
  __shared__ __align__(8) uint64_t s_blk[2][16];  // block q of Xa / Xb arrived
  __shared__ __align__(8) uint64_t s_csync;       // bounded cluster barrier
  const int k = a.k;
  const int c0 = rank * NB;
  const int tid = threadIdx.x, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
  const long long wl = tc::wait_limit_or_default(a.wait_limit);
  {
    // Phi: loads issued in batches of 8 per thread so that their latencies overlap
    constexpr int N = KP * XLD, B = 8;
    for (int e0 = tid; e0 < N; e0 += 512 * B) {
      float v[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int e = e0 + 512 * u, r = e % XLD, c = e / XLD;
        v[u] = (e < N && r < k && c < k) ? __ldg(a.phi + (int64_t)c * k + r) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (e0 + 512 * u < N) {
          Xa[e0 + 512 * u] = v[u];
          if (!S::SB) Xb[e0 + 512 * u] = 0.f;
        }
    }
  }
  for (int e = tid; e < (S::SB ? 1 : 2) * NB * XLD; e += blockDim.x) Ot[e] = 0.f;
  if (tid < 2 * CL) mbar_init(&s_blk[tid / CL][tid % CL], 1);
  if (tid == 2 * CL) mbar_init(&s_csync, CL);
  if (tid <= 2 * CL) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  if (a.step_mode == kStepOnline) {
    // mu1..3 for the G block below, and the mean terms phi_i . mu and
    // |phi_i|^2 of this block's columns (a warp per dot product, lanes along
    // the k entries): Phi and mu only, so before the wait
    for (int e = tid; e < 3 * KP; e += blockDim.x) {
      const int which = e / KP, j = e % KP;
      const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
      mus[e] = (mu && j < k) ? __ldg(mu + j) : 0.f;
    }
    for (int e = tid / 32; e < 4 * NB; e += blockDim.x / 32) {
      const int which = e / NB, jb = e % NB, i = c0 + jb;
      const float* col = Xa + i * XLD;
      const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : which == 2 ? a.mu3 : col;
      float sv = 0.f;
      if (i < k && mu)
        for (int j = lane; j < k; j += 32) sv = fmaf(col[j], mu[j], sv);
#pragma unroll
      for (int off = 16; off; off >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, off);
      if (lane == 0) {
        if (which < 3) mv[which * KP + jb] = sv; else nn[jb] = sv;
      }
    }
  }
  cluster.sync();  // Phi read and barriers initialised everywhere before any copy
  // launched with programmatic serialization after the contraction, the
  // prologue above overlapped its tail (Phi is final: the contraction lets
  // this kernel start only after its own wait on the previous step); from
  // here on its partials are read, so wait for it to complete, and let the
  // next contraction be scheduled (it waits for this kernel in turn)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  uint32_t parity = 0u;  // bit b: phase parity awaited on the barriers of buffer b
  uint32_t csync_parity = 0u;
  int nbcast = 0;
  bool timed_out = false;
  constexpr uint32_t kBlockBytes = sizeof(float) * NB * XLD;
  auto buf_of = [&](const float* b) { return b == Xa ? 0 : 1; };
  // staging tile of the next broadcast (or of the final block)
  auto stage_next = [&]() -> float* {
    float* p = S::SB ? Ot : Ot + (nbcast & 1) * NB * XLD;
    ++nbcast;
    return p;
  };
  // bounded cluster barrier: every thread of every CTA has passed the
  // __syncthreads before its rank's arrival (remote mbarrier arrives with
  // release semantics, waited for with acquire); false after a timeout
  auto csync_arrive = [&]() {
    __syncthreads();
    if (tid < CL) {
      uint32_t remote;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(smem_addr(&s_csync)), "r"(tid));
      asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(remote) : "memory");
    }
  };
  auto csync_wait = [&]() -> bool {
    bool ok = true;
    if (tid == 0) ok = mbar_wait_cluster_bounded(&s_csync, csync_parity, wl);
    csync_parity ^= 1u;
    return !__syncthreads_or(!ok);
  };
  auto csync = [&]() -> bool {
    csync_arrive();
    return csync_wait();
  };
  // the staged block Otc (this CTA's columns) into `dst` of every rank,
  // own copy included; sync_first: a cluster barrier first, because some
  // rank may still be reading its `dst`
  auto broadcast = [&](float* Otc, float* dst, bool sync_first) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // staging -> async proxy
    if (sync_first) {
      if (!csync()) timed_out = true;
    } else {
      __syncthreads();
    }
    float* own = dst + c0 * XLD;
    for (int e = tid; e < NB * XLD; e += blockDim.x) own[e] = Otc[e];
    const int bi = buf_of(dst), w = tid >> 5;
    // one issuing thread per warp (copies issued by lanes of one warp
    // serialise); rank q sends to q+1, q+2, ... first, so every rank receives
    // its blocks spread over the exchange
    if (lane == 0 && w < CL - 1)
      bulk_copy_to_rank(own, Otc, kBlockBytes, &s_blk[bi][rank], (uint32_t)((rank + 1 + w) % CL));
    if (tid < CL && tid != rank) mbar_arrive_expect_tx(&s_blk[bi][tid], kBlockBytes);
  };
  // every block of `buf` has arrived (false after a timeout of any wait);
  // SB: then a cluster barrier, after which every copy of the broadcast has
  // landed everywhere (the single staging tile and the G tile are free)
  auto wait_buf = [&](const float* buf) -> bool {
    const int bi = buf_of(buf);
    bool ok = true;
    if (tid < CL && tid != rank) ok = mbar_wait_bounded(&s_blk[bi][tid], (parity >> bi) & 1u, wl);
    parity ^= 1u << bi;
    ok = !__syncthreads_or(!ok);
    if (S::SB) ok = csync() && ok;
    return ok;
  };
  // Gram block C = P^T P[:, c0 .. c0+NB) into the staging tile, zero outside
  // k x k; a non-finite entry raises kFlagNonFinite
  auto gram_stage = [&](const float* P, float* Otc) {
    bool bad = false;
    step_tiles<KP, CL, kProdGram>(P, P + c0 * XLD, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        const float v = acc[q];
        if (!isfinite(v)) bad = true;
        Otc[jb * XLD + i] = (i < k && col < k) ? v : 0.f;
      }
    });
    if (bad) atomicOr(a.flags, kFlagNonFinite);
  };

  float* M = Xa;               // the matrix to orthonormalise (full in every CTA)
  float* F = S::SB ? Xa : Xb;  // the other buffer
  if (a.step_mode == kStepOnline) {
    // G block (columns c0 .. c0+NB) from the per-CTA partials.  The first 8
    // partials of this thread's (up to) two G entries are loaded together
    // with the d-sum partials, so that one round trip covers them all.
    constexpr int kPre = 2, kPreParts = 8;
    float gpre[kPre][kPreParts];
#pragma unroll
    for (int h = 0; h < kPre; ++h) {
      const int e = tid + h * (int)blockDim.x, jb = e / KP, j = e % KP, i = c0 + jb;
      const bool live = e < NB * KP && i < k && j < k;
#pragma unroll
      for (int u = 0; u < kPreParts; ++u)
        gpre[h][u] = (live && u < a.nparts)
                         ? __ldg(a.gpart + (int64_t)u * a.part_stride + (int64_t)i * k + j)
                         : 0.f;
    }
    // per-column sums of the d partials (3 x NB)
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
        const int h = (e - tid) / (int)blockDim.x;  // 0 or 1 for the preloaded entries
        if (h < kPre) {
#pragma unroll
          for (int h2 = 0; h2 < kPre; ++h2)
            if (h2 == h) {
              s0 += gpre[h2][0] + gpre[h2][4];
              s1 += gpre[h2][1] + gpre[h2][5];
              s2 += gpre[h2][2] + gpre[h2][6];
              s3 += gpre[h2][3] + gpre[h2][7];
            }
          pp = kPreParts;
        }
        for (; pp + 8 <= a.nparts; pp += 8) {
          float v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) v[u] = __ldg(gp + (int64_t)(pp + u) * a.part_stride);
          s0 += v[0] + v[4];
          s1 += v[1] + v[5];
          s2 += v[2] + v[6];
          s3 += v[3] + v[7];
        }
        for (; pp < a.nparts; ++pp) s0 += __ldg(gp + (int64_t)pp * a.part_stride);
        float gv = ((s0 + s1) + (s2 + s3)) * (float)a.scale;
        const float m1 = mv[jb], m2 = mv[KP + jb], m3 = mv[2 * KP + jb];
        const float c1 = (float)a.c1, c2 = (float)a.c2;
        if (a.mode == kModePlain) {
          gv += mus[2 * KP + j] * (c1 * m1 * m2 + c2 * dcol[jb]);
        } else {
          const float ic = (float)(1.0 / a.count);
          gv += mus[j] * (c2 * dcol[jb] * ic + c1 * m2 * m3) +
                mus[KP + j] * (c2 * dcol[NB + jb] * ic + c1 * m1 * m3) +
                mus[2 * KP + j] * (c2 * dcol[2 * NB + jb] * ic + c1 * m1 * m2);
        }
        gval = gv;
      }
      Gb[jb * XLD + j] = gval;
    }
    // X = Phi - beta (3 theta Phi (Phi^T Phi)^.2 - gscale G)   (Util.cpp:259-272)
    float* Otc;
    const float alpha = -a.beta * a.theta3, gamma = a.beta * a.gscale;
    if (a.phi_general) {
      // the literal product (first step of a run: Phi0 need not be orthonormal)
      step_tiles<KP, CL, kProdGram>(M, M + c0 * XLD, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1);
          Ab[jb * XLD + i] = acc[q] * acc[q];
        }
      });
      __syncthreads();
      Otc = stage_next();
      step_tiles<KP, CL, kProdTimes>(M, Ab, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
          const float v = alpha * acc[q] + M[col * XLD + r] + gamma * Gb[jb * XLD + r];
          Otc[jb * XLD + r] = (r < k && col < k) ? v : 0.f;
        }
      });
    } else {
      // Phi is the previous step's Q: Phi^T Phi = I to ~1e-7, so
      // (Phi^T Phi)^.2 = diag(|phi_i|^4) + O(1e-14) and Phi times it is
      // phi_i |phi_i|^4, column by column
      __syncthreads();
      Otc = stage_next();
      for (int e = tid; e < NB * XLD; e += blockDim.x) {
        const int r = e % XLD, jb = e / XLD, col = c0 + jb;
        const float n2 = nn[jb] * nn[jb];
        Otc[e] = (r < k && col < k) ? M[col * XLD + r] * (1.f + alpha * n2) + gamma * Gb[e] : 0.f;
      }
    }
    broadcast(Otc, F, S::SB);
    if (!wait_buf(F)) timed_out = true;
    float* t = M;
    M = F;
    F = t;
  }
  // Cholesky QR passes on M: A = M^T M gathered into F, R = chol(A) and the
  // columns of R^-1 this CTA needs (computed by every CTA from the same A),
  // M R^-1 gathered into F, which becomes M.  (SB: M is kept in global
  // memory while its buffer holds A.)
  int passes = 0, shifts = 0, plain_left = a.max_passes;
  float shift = 0.f;
  bool resync = false;  // a rank may still be factoring the last Gram in F
  __shared__ float s_shift;
  // SB: the buffer (R, read by no one now) gets M back from the stash
  // (written before the barrier of the last broadcast)
  auto restore_m = [&]() {
    for (int e = tid; e < KP * KP; e += blockDim.x) {
      const int r = e % KP, c = e / KP;
      M[c * XLD + r] = __ldcg(a.xstash + (int64_t)c * KP + r);
    }
    __syncthreads();
  };
  while (!timed_out) {
    float* Otc = stage_next();
    gram_stage(M, Otc);
    if (S::SB) {
      // M's own columns to the stash (every rank's are read back below)
      for (int e = tid; e < NB * KP; e += blockDim.x) {
        const int r = e % KP, jb = e / KP;
        a.xstash[(int64_t)(c0 + jb) * KP + r] = M[(c0 + jb) * XLD + r];
      }
    }
    broadcast(Otc, F, S::SB || resync);
    resync = false;
    if (!wait_buf(F)) {
      timed_out = true;
      break;
    }
    const float ratio = chol_blocked<KP>(F, k, tinv, rd, dg, &s_ratio, shift);
    if (__syncthreads_or(ratio < kShiftBelow) && shifts < kMaxShifts) {
      // near breakdown: the Gram again, factored with a diagonal shift
      if (tid == 0) {
        float tr = 0.f;
        for (int i = 0; i < k; ++i) tr += dg[i];
        s_shift = shift > 0.f ? 100.f * shift : kShiftScale * tr;
      }
      __syncthreads();
      shift = s_shift;
      ++shifts;
      if (S::SB) restore_m();
      resync = true;
      continue;
    }
    inverse_columns<KP, NB>(F, tinv, x16, c0, k, Ab, tmp);
    ++passes;
    if (S::SB) restore_m();
    Otc = stage_next();
    step_tiles<KP, CL, kProdTimes>(M, Ab, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        Otc[jb * XLD + r] = (r < k && col < k) ? acc[q] : 0.f;
      }
    });
    // every rank has finished its Cholesky in F (and, SB, its product on M)
    // before any block of M R^-1 is written there
    broadcast(Otc, F, true);
    if (!wait_buf(F)) {
      timed_out = true;
      break;
    }
    float* t = M;
    M = F;
    F = S::SB ? M : t;
    if (shift > 0.f) {
      // Q1 of a shifted factor is well conditioned, not orthonormal: plain
      // passes follow
      shift = 0.f;
      plain_left = a.max_passes;
      continue;
    }
    --plain_left;
    // the decision is taken by the whole CTA together (a barrier OR), so
    // every warp leaves or repeats the loop
    const bool again = __syncthreads_or(ratio < kQrExactBelow) != 0;
    if (!again || plain_left <= 0) {
      if (again && rank == 0 && tid == 0) atomicOr(a.flags, kFlagNoConvergence);
      break;
    }
  }
  // every copy of the last exchange has landed in this CTA, and each rank
  // sent its blocks only after the barrier that opened that exchange, so
  // every rank's phase of that barrier is complete: this CTA's arrival at
  // the closing barrier (no remote access follows) goes out now, its wait
  // comes at the end
  const bool early_arrive = !timed_out;
  if (early_arrive) csync_arrive();
  // first-order second pass: E = M^T M - I, F = strict upper part of E plus
  // half its diagonal (this CTA's columns, in Ab), Phi = M (I - F)
  float emax = 0.f;
  if (!timed_out) {
    step_tiles<KP, CL, kProdGram>(M, M + c0 * XLD, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        const bool live = i < k && col < k;
        const float e = live ? acc[q] - (i == col ? 1.f : 0.f) : 0.f;
        emax = fmaxf(emax, fabsf(e));
        Ab[jb * XLD + i] = i < col ? e : i == col ? 0.5f * e : 0.f;
      }
    });
#pragma unroll
    for (int off = 16; off; off >>= 1) emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if (lane == 0) s_emax[tid >> 5] = emax;
    __syncthreads();
    float* Otc = stage_next();
    // |F| is at most ~1e-5 here (an exact pass left M orthonormal to u times
    // at most 1 / the pivot ratio bound), so a single TF32 product keeps
    // M F to ~1e-9, below the FP32 resolution of Phi's entries
    step_tiles<KP, CL, kProdTimes, false>(M, Ab, part, [&](const float (&acc)[4], int m0, int n0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = m0 + g + ((q & 2) ? 8 : 0), jb = n0 + 2 * t4 + (q & 1), col = c0 + jb;
        Otc[jb * XLD + r] = (r < k && col < k) ? M[col * XLD + r] - acc[q] : 0.f;
      }
    });
    __syncthreads();
    if (tid == 0) {
      float m = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, s_emax[w]);
      if (a.orth_err) atomicMax(reinterpret_cast<int*>(a.orth_err), __float_as_int(m));
    }
    for (int e = tid; e < KP * NB; e += blockDim.x) {
      const int r = e % KP, jb = e / KP, col = c0 + jb;
      if (r < k && col < k) a.phi[(int64_t)col * k + r] = Otc[jb * XLD + r];
    }
    if constexpr (KP <= 112) {
      if (a.phi_img) {
        // the next contraction's operand image of this CTA's columns i (rows
        // of its A operand, K = j): TF32 hi / lo in the core-matrix layout,
        // then Phi^T mu1, Phi^T mu2 of the columns
        using CT = ContractTc<KP>;
        unsigned char* img = static_cast<unsigned char*>(a.phi_img);
        for (int e = tid; e < NB * (KP / 4); e += blockDim.x) {
          const int jb = e / (KP / 4), jq = e % (KP / 4), i = c0 + jb;
          float v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) v[u] = Otc[jb * XLD + 4 * jq + u];  // zero past k
          uint4 h;
          float4 l;
          tc::split4(v, h, l);
          const uint32_t off = tc::kmajor_off(i, 4 * jq, CT::SBOJ);
          *reinterpret_cast<uint4*>(img + CT::PH + off) = h;
          *reinterpret_cast<float4*>(img + CT::PL + off) = l;
        }
        float* mimg = reinterpret_cast<float*>(img + 2 * CT::PSZ);
        for (int e = tid >> 5; e < 2 * NB; e += blockDim.x >> 5) {
          const int which = e / NB, jb = e % NB, i = c0 + jb;
          const float* mu = which == 0 ? a.mu1 : a.mu2;
          float sv = 0.f;
          if (mu && i < k)
            for (int j = lane; j < k; j += 32) sv = fmaf(Otc[jb * XLD + j], mu[j], sv);
#pragma unroll
          for (int off = 16; off; off >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, off);
          if (lane == 0) mimg[which * KP + i] = sv;
        }
      }
    }
    if (a.trace_out) {  // ||Phi_new - snapshot||_F^2 over this CTA's columns, fixed order
      double d2 = 0.0;
      for (int e = tid; e < KP * NB; e += blockDim.x) {
        const int r = e % KP, jb = e / KP, col = c0 + jb;
        if (r < k && col < k) {
          const float v = Otc[jb * XLD + r];
          const double d = (double)v - (double)a.trace_snap[(int64_t)col * k + r];
          d2 = fma(d, d, d2);
          a.trace_snap[(int64_t)col * k + r] = v;
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, off);
      __shared__ double tpart[16];
      if (lane == 0) tpart[tid >> 5] = d2;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += tpart[w];
        a.trace_out[rank] = t;
      }
    }
  }
  if (timed_out) {
    if (tid == 0) atomicOr(a.flags, kFlagTimeout);
  }
  if (rank == 0 && tid == 0 && a.orth_passes) atomicAdd(a.orth_passes, passes);
  // keep shared memory alive until remote writers are done (bounded: after a
  // timeout the ranks may stand at different barriers)
  if (!(early_arrive ? csync_wait() : csync())) {
    if (tid == 0) atomicOr(a.flags, kFlagTimeout);
    __nanosleep(100000);  // let copies a stalled exchange left in flight land
  }
}

template <int KP, int CL>
__global__ void __launch_bounds__(512, 1) stpm_step_kernel(StpmUpdateArgs a) {
  step_body<KP, CL>(a);
}

// one cluster per graph: blockIdx.y selects the graph's arguments; graphs
// with no update in this round (active == 0) leave at once
template <int KP, int CL>
__global__ void __launch_bounds__(512, 1) stpm_step_batched(const StpmUpdateArgs* __restrict__ args) {
  const StpmUpdateArgs a = args[blockIdx.y];
  if (!a.active) return;
  step_body<KP, CL>(a);
}

// ---- partial contractions on the tensor cores -----------------------------------
//
// Per tile of TM nodes, with Phi resident in shared memory:
//   Z_q^T = Phi^T Y_q^T           (k x TM, m16n8k8 3xTF32 or m16n8k16 BF16 MMAs;
//                                  both operands contiguous along j)
//   C = c0 Z1.Z2 + c2 (Z1 m2 + m1 Z2)   (on the Z fragments; stored i-major)
//   G += Yout^T C                 (k x k, accumulated in registers over the
//                                  CTA's tiles; the Yout operand is read
//                                  transposed: strided loads in FP32,
//                                  ldmatrix.trans in BF16)
//   d_i += sum_x Z1 Z2            (per column i)
// The FP32 form keeps FP32 accuracy through the 3xTF32 split; the BF16 form
// reads y rounded to BF16, Phi as a BF16 pair (hi + lo: Z = hi^T y + lo^T y,
// two MMAs), the coefficients C rounded to BF16, and accumulates in FP32.
// Tensor-core form of the plain FP32 contraction (tcgen05.mma kind::tf32,
// 3xTF32: D += Ahi Bhi + Ahi Blo + Alo Bhi), for KP in [32, 112].  Per tile
// of TM = 32 nodes:
//   [Z1 Z2] = Phi^T [y1 y2]      A = Phi  (M = i, K = j), B = y1 | y2 (N = 2 TM, K = j)
//   C   = c0 Z1 Z2 + c2 (Z1 m2 + m1 Z2)   (TMEM -> registers -> shared)
//   G  += y3^T C                 A = y3   (M = j, K = x), B = C   (N = i, K = x)
// Z1, Z2 and G live in tensor memory (columns [0, TM), [TM, 2 TM),
// [2 TM, 2 TM + KP)); G accumulates over the CTA's tiles.  Operands are
// staged hi / lo in shared memory, K-major without swizzle; y3 is staged
// transposed (node index along K).  An M = 128 operand of KP < 128 rows
// reads its rows past KP from the buffer after it: their products land in
// TMEM lanes that are never read.
template <int KP>
struct ContractTc {
  static constexpr int TM = 32;
  static constexpr uint32_t SBOJ = (KP / 4) * 128u;  // 8-row groups of a K = j operand
  static constexpr uint32_t SBOX = (TM / 4) * 128u;  // 8-row groups of a K = x operand
  static constexpr uint32_t PSZ = 4u * KP * KP, TSZ = 4u * TM * KP;
  static constexpr uint32_t PH = 0, PL = PSZ;                                   // Phi, KP rows i
  // y1 hi | y2 hi | y1 lo | y2 lo (TM rows x each): y1 and y2 stack into one
  // operand of N = 2 TM rows, so one MMA makes Z1 and Z2 side by side
  static constexpr uint32_t Y1H = 2 * PSZ, Y2H = Y1H + TSZ, Y1L = Y2H + TSZ, Y2L = Y1L + TSZ;
  static constexpr uint32_t Y3H = Y2L + TSZ, Y3L = Y3H + TSZ;                   // KP rows j
  static constexpr uint32_t CH = Y3L + TSZ, CLO = CH + TSZ;                     // KP rows i
  static constexpr uint32_t END = CLO + TSZ;
  static constexpr uint32_t READ_END =  // furthest byte read by an M = 128 operand
      (Y3L + 16 * SBOX > PL + 16 * SBOJ) ? Y3L + 16 * SBOX : PL + 16 * SBOJ;
  static constexpr uint32_t STAGE = 4u * (KP * KP + 3 * KP + 1);  // partial for the cluster sum
  static constexpr uint32_t REGION0 = END > READ_END ? END : READ_END;
  static constexpr uint32_t REGION = ((REGION0 > STAGE ? REGION0 : STAGE) + 127) / 128 * 128;
  // alignment slack, m1 | m2, d-sums of the 4 node groups
  static constexpr size_t smem = 1024 + REGION + sizeof(float) * (2 * KP + 4 * KP);
  static constexpr uint32_t TMEM_COLS = 256;
  static_assert(KP % 16 == 0 && KP >= 32 && KP <= 112, "tensor-core contraction: KP in [32, 112]");
  static_assert(smem <= 227 * 1024, "tensor-core contraction shared memory");
};

// BF16 tensor-core form of the adjoint contraction (tcgen05.mma kind::f16,
// BF16 operands, FP32 accumulation), for KP in [32, 112]: per tile of TM = 64
// nodes
//   [Z1 Z2 Z3] = Phi^T [y1 y2 y3]  A = Phi as a BF16 hi / lo pair (M = i, K = j),
//                                  B = y1 | y2 | y3 (N = 3 TM, K = j)
//   C_1..3 (alpha0 terms of the Z pairs, BF16)       TMEM -> registers -> shared
//   G += sum_c y_c^T C_c           A = y_c staged transposed (M = j, K = x),
//                                  B = C_c (N = i, K = x)
// Z in TMEM columns [0, 3 TM), G in [3 TM, 3 TM + KP).  16-bit operands: a
// core matrix is 8 rows x 8 elements, one MMA consumes K = 16.
template <int KP>
struct ContractTcBf {
  static constexpr int TM = 64;
  static constexpr uint32_t SBOJ = (KP / 8) * 128u;  // 8-row groups of a K = j operand
  static constexpr uint32_t SBOX = (TM / 8) * 128u;  // 8-row groups of a K = x operand
  static constexpr uint32_t PSZ = 2u * KP * KP, TSZ = 2u * TM * KP;
  static constexpr uint32_t PH = 0, PL = PSZ;   // Phi hi / lo, KP rows i
  static constexpr uint32_t YB = 2 * PSZ;       // y1 | y2 | y3, TM rows x each
  static constexpr uint32_t YT = YB + 3 * TSZ;  // y_c transposed, KP rows j each
  static constexpr uint32_t CB = YT + 3 * TSZ;  // C_c, KP rows i each
  static constexpr uint32_t END = CB + 3 * TSZ;
  static constexpr uint32_t READ_END =  // furthest byte an M = 128 operand reads (Phi lo, y3^T)
      (YT + 2 * TSZ + 16 * SBOX > PL + 16 * SBOJ) ? YT + 2 * TSZ + 16 * SBOX : PL + 16 * SBOJ;
  static constexpr uint32_t STAGE = 4u * (KP * KP + 3 * KP + 1);
  static constexpr uint32_t REGION0 = END > READ_END ? END : READ_END;
  static constexpr uint32_t REGION = ((REGION0 > STAGE ? REGION0 : STAGE) + 127) / 128 * 128;
  // alignment slack, m1 | m2 | m3, d-sums (3 pairs x 4 node groups)
  static constexpr size_t smem = 1024 + REGION + sizeof(float) * (3 * KP + 12 * KP);
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert(KP % 16 == 0 && KP >= 32 && KP <= 112, "BF16 tensor-core contraction: KP in [32, 112]");
  static_assert(3 * TM + KP <= 512, "tensor memory columns");
  static_assert(smem <= 227 * 1024, "BF16 tensor-core contraction shared memory");
};

template <int KP, bool TC, bool TCBF>
constexpr size_t contract_smem(size_t cuda_core_form) {
  if constexpr (TC)
    return ContractTc<KP>::smem;
  else if constexpr (TCBF)
    return ContractTcBf<KP>::smem;
  else
    return cuda_core_form;
}

template <int KP, int MODE, bool BF>
struct Contract {
  static constexpr bool TC = MODE == kModePlain && !BF && KP <= 112;
  static constexpr bool TCBF = MODE == kModeAdjoint && BF && KP <= 112;
  using T = typename std::conditional<BF, __nv_bfloat16, float>::type;
  static constexpr int TM = BF ? 64 : 32;  // nodes per tile
  static constexpr int NZ = MODE == kModePlain ? 2 : 3;
  static constexpr int NC = MODE == kModePlain ? 1 : MODE == kModeAdjoint ? 3 : 0;
  // columns i of Phi handled by one CTA: all of them up to KP = 128, above
  // that blocks of 64 (blockIdx.y), so that Phi's block, the G accumulators
  // and the staged partial fit one SM; Z, C, G and the d-sums are separable
  // by column
  static constexpr int IB = KP <= 128 ? KP : 64;
  static constexpr int NBC = (KP + IB - 1) / IB;  // column blocks (<= 4: one loss slot each)
  static constexpr int PAD = BF ? 8 : 4;   // row strides == 4 words mod 8: conflict-free fragments
  static constexpr int PLD = KP + PAD, LDY = KP + PAD, LDC = TM + PAD;
  static constexpr int MTI = IB / 16, NTX = TM / 8;        // Z^T tiles: i (16) x nodes (8)
  static constexpr int MTJ = KP / 16, NTI = IB / 8;        // G tiles: j (16) x i (8)
  static constexpr int NW = 16, NT = 32 * NW;               // warps, threads per CTA
  static constexpr int GT = MTJ * NTI, GPW = (GT + NW - 1) / NW;  // G tiles, per warp
  static constexpr int KSTEP = BF ? 16 : 8;
  // the BF16 form keeps Phi as a pair of BF16 arrays (hi + lo): rounding Phi
  // itself to BF16 would bias every product Phi^T y of a step the same way
  static constexpr int NPHI = BF ? 2 : 1;
  static constexpr size_t tile_bytes =
      sizeof(T) * ((size_t)NPHI * IB * PLD + (size_t)3 * TM * LDY + (size_t)NC * IB * LDC);
  static constexpr size_t stage_bytes = sizeof(float) * ((size_t)KP * IB + 3 * IB + 4);
  static constexpr size_t region = ((tile_bytes > stage_bytes ? tile_bytes : stage_bytes) + 15) / 16 * 16;
  static constexpr size_t smem_mma = region + sizeof(float) * (3 * IB + NW + NW * 3 * IB);
  static constexpr size_t smem = contract_smem<KP, TC, TCBF>(smem_mma);
  static_assert(NBC <= 4, "one loss slot per column block");
};

template <typename T>
__device__ __forceinline__ T to_elem(float v);
template <>
__device__ __forceinline__ float to_elem<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 to_elem<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ uint32_t ld_b32(const void* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p)));
}

// v = hi + lo with hi rounded to TF32; lo is passed as full FP32 bits: a TF32
// MMA reads only the top 19 bits of an operand, so lo enters truncated to
// TF32 (|error| <= 2^-10 |lo| <= 2^-21 |v|) without a second conversion
__device__ __forceinline__ void split_tf32(float v, uint32_t& hi, uint32_t& lo) {
  hi = tf32_round(v);
  lo = __float_as_uint(v - __uint_as_float(hi));
}

// The cluster's CTAs staged their partials (column block cb: G block, 3
// d-sums, loss) at the same shared-memory offset `stage`; CTA r sums a 1/CLP
// slice over the cluster through DSMEM and writes it out.  Column block cb
// writes loss slot cb of the 4 spare floats of the partial row (block 0 also
// clears the unused slots).
template <int KP, int IB, int NBC, int MODE>
__device__ __forceinline__ void partial_cluster_sum(const StpmPartialArgs& a, float* stage, int cb,
                                                    int i0) {
  cg::cluster_group cluster = cg::this_cluster();
  const int crank = (int)cluster.block_rank(), tid = threadIdx.x, NT = blockDim.x, k = a.k;
  constexpr int CLP = kPartialCluster;
  constexpr int STAGE = KP * IB + 3 * IB + 1;
  // 16-byte slices: the staging areas have room past STAGE (the tile region
  // they overlay is larger), and KP, IB are multiples of 4, so the 4 entries
  // of a vector share their row i of G
  constexpr int STAGE4 = (STAGE + 3) / 4;
  static_assert(KP % 4 == 0 && IB % 4 == 0, "16-byte slices");
  cluster.sync();
  float* gp = a.gpart + (int64_t)(blockIdx.x / CLP) * a.part_stride;
  const int slice4 = (STAGE4 + CLP - 1) / CLP;
  auto put = [&](int e, float v) {
    if (e < KP * IB) {
      const int i = i0 + e / KP, j = e % KP;
      if (i < k && j < k && MODE != kModeLoss) gp[(int64_t)i * k + j] = v;
    } else if (e < KP * IB + 3 * IB) {
      const int q = (e - KP * IB) / IB, i = i0 + (e - KP * IB) % IB;
      if (i < k) gp[(int64_t)k * k + q * k + i] = v;
    } else if (e < STAGE) {
      gp[(int64_t)k * k + 3 * k + cb] = v;
    }
  };
  for (int e4 = crank * slice4 + tid; e4 < min(STAGE4, (crank + 1) * slice4); e4 += NT) {
    float4 r[CLP];
#pragma unroll
    for (int q = 0; q < CLP; ++q) r[q] = reinterpret_cast<const float4*>(cluster.map_shared_rank(stage, q))[e4];
    float4 v = r[0];
#pragma unroll
    for (int q = 1; q < CLP; ++q) {
      v.x += r[q].x;
      v.y += r[q].y;
      v.z += r[q].z;
      v.w += r[q].w;
    }
    put(4 * e4, v.x);
    put(4 * e4 + 1, v.y);
    put(4 * e4 + 2, v.z);
    put(4 * e4 + 3, v.w);
  }
  if (cb == 0 && crank == 0 && tid < 4 && tid >= NBC) gp[(int64_t)k * k + 3 * k + tid] = 0.f;
  cluster.sync();  // keep shared memory alive until every remote read is done
}

// The tensor-core contraction of one CTA (plain mode, FP32): stages this
// CTA's partial -- G column-major (stage[i KP + j]), the d-sums d1 (then
// d2 = d3 = 0) and a zero loss -- at `stage`, as the CUDA-core form does.
template <int KP>
__device__ __forceinline__ void contract_tc(const StpmPartialArgs& a, int nblocks,
                                            unsigned char* smraw, float* stage) {
  using C = ContractTc<KP>;
  constexpr int TM = C::TM, NT = 512, NQ = KP / 4;
  __shared__ __align__(8) uint64_t bars[3];  // Z products done | G products done | Phi image
  __shared__ uint32_t tmem_slot;
  unsigned char* base = smraw + ((1024 - (tc::sm_addr(smraw) & 1023)) & 1023);
  float* mv = reinterpret_cast<float*>(base + C::REGION);  // m1 | m2
  float* dsum = mv + 2 * KP;                               // d1 per node group (4 x KP)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k = a.k;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, C::TMEM_COLS);
  if (tid == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // Staging tasks are laid out so that the 8 lanes of a quarter-warp write
  // one whole core matrix (8 consecutive rows x 16 bytes, 128 contiguous
  // bytes: no bank conflicts), and the global loads of a warp still cover
  // whole 32-byte sectors.  y1, y2 (row x, 16-byte chunks along j): lane l
  // takes row 8 g + (l & 7) and chunk 4 h + (l >> 3) of warp-task (g, h); y3
  // (transposed: row j, 4 nodes along K): lane = j, four scalar loads.
  // A tile's loads go to registers one tile ahead.
  constexpr int T12 = 2 * TM * NQ, S12 = (T12 + NT - 1) / NT;
  constexpr int T3 = KP * (TM / 4), S3 = (T3 + NT - 1) / NT;
  static_assert(NQ % 4 == 0 && TM % 8 == 0, "warp-task shape");
  uint4 p12[S12];
  float p3[S3][4];
  auto task12 = [&](int e, int& q, int& x, int& jq) {
    const int l = e & 31, w = e >> 5;
    x = 8 * (w % (TM / 8)) + (l & 7);
    jq = 4 * ((w / (TM / 8)) % (NQ / 4)) + (l >> 3);
    q = w / ((TM / 8) * (NQ / 4));
  };
  auto tile_nodes = [&](int64_t tile, int64_t& x0) {
    x0 = a.begin + tile * TM;
    const int64_t left = a.begin + a.count - x0;
    return left < TM ? (int)left : TM;
  };
  auto load_tile = [&](int64_t tile) {
    int64_t x0;
    const int nv = tile_nodes(tile, x0);
#pragma unroll
    for (int s = 0; s < S12; ++s) {
      const int e = tid + NT * s;
      p12[s] = make_uint4(0u, 0u, 0u, 0u);
      if (e < T12) {
        int q, x, jq;
        task12(e, q, x, jq);
        const float* Y = q == 0 ? a.y1 : a.y2;
        if (x < nv && 4 * jq < a.ldy)
          p12[s] = __ldg(reinterpret_cast<const uint4*>(Y + (x0 + x) * a.ldy + 4 * jq));
      }
    }
#pragma unroll
    for (int s = 0; s < S3; ++s) {
      const int e = tid + NT * s, j = e % KP, xq = e / KP;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = 4 * xq + u;
        p3[s][u] = (e < T3 && x < nv && j < a.ldy) ? __ldg(a.y3 + (x0 + x) * a.ldy + j) : 0.f;
      }
    }
  };
  auto store_tile = [&]() {
#pragma unroll
    for (int s = 0; s < S12; ++s) {
      const int e = tid + NT * s;
      if (e < T12) {
        int q, x, jq;
        task12(e, q, x, jq);
        const float v[4] = {__uint_as_float(p12[s].x), __uint_as_float(p12[s].y),
                            __uint_as_float(p12[s].z), __uint_as_float(p12[s].w)};
        uint4 h;
        float4 l;
        tc::split4(v, h, l);
        const uint32_t off = tc::kmajor_off(x, 4 * jq, C::SBOJ);
        *reinterpret_cast<uint4*>(base + (q == 0 ? C::Y1H : C::Y2H) + off) = h;
        *reinterpret_cast<float4*>(base + (q == 0 ? C::Y1L : C::Y2L) + off) = l;
      }
    }
#pragma unroll
    for (int s = 0; s < S3; ++s) {
      const int e = tid + NT * s, j = e % KP, xq = e / KP;
      if (e < T3) {
        uint4 h;
        float4 l;
        tc::split4(p3[s], h, l);
        const uint32_t off = tc::kmajor_off(j, 4 * xq, C::SBOX);
        *reinterpret_cast<uint4*>(base + C::Y3H + off) = h;
        *reinterpret_cast<float4*>(base + C::Y3L + off) = l;
      }
    }
  };
  const int64_t ntiles = ceil_div_dev(a.count, TM);
  float* mus = mv;  // mu_1 | mu_2 staged in mv
  // Launched as a programmatic dependent of the step that writes Phi: all
  // that does not read Phi -- TMEM, barriers, mu and the whole first node
  // tile -- is done before the wait and overlaps that kernel's tail.
  const bool first_staged = (int64_t)blockIdx.x < ntiles;
  if (first_staged) load_tile(blockIdx.x);
  for (int e = tid; e < 2 * KP; e += NT) {
    const float* mu = e < KP ? a.mu1 : a.mu2;
    const int j = e % KP;
    mus[e] = (mu && j < k) ? mu[j] : 0.f;
  }
  for (int e = tid; e < 4 * KP; e += NT) dsum[e] = 0.f;
  if (first_staged) store_tile();
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // Phi hi / lo (operand row i = column i of Phi, contiguous in j), all of
  // a thread's loads issued together; the partial dot products of its
  // chunks with mu_1, mu_2 go to part[] (in the C area, free until the first
  // epilogue) and are summed per column in a fixed order: m_q = Phi^T mu_q
  constexpr int PT = (KP * NQ + NT - 1) / NT;
  auto task_phi = [&](int e, int& i, int& jq) {  // 8 rows i x 4 chunks per warp
    const int l = e & 31, w = e >> 5;
    i = 8 * (w % (KP / 8)) + (l & 7);
    jq = 4 * (w / (KP / 8)) + (l >> 3);
  };
  float* part = reinterpret_cast<float*>(base + C::CH);  // [q][i][jq]
  static_assert(2 * KP * NQ * 4 <= 2 * C::TSZ, "partials fit the C area");
  bool img_timed_out = false;
  if (a.phi_img) {
    // the previous step kernel wrote Phi's operand image and Phi^T mu1|2:
    // bulk copies of the hi | lo image (in 4 pieces) and plain loads of m
    __syncthreads();  // every thread past its first-tile stores (the barrier init is ordered)
    if (tid == 0) {
      constexpr uint32_t bytes = 2 * C::PSZ, piece = bytes / 4;
      static_assert(bytes % 64 == 0, "16-byte pieces");
      mbar_arrive_expect_tx(&bars[2], bytes);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        bulk_copy_g2s(base + C::PH + q * piece, static_cast<const unsigned char*>(a.phi_img) + q * piece,
                      piece, &bars[2]);
    }
    const float* mimg = reinterpret_cast<const float*>(static_cast<const unsigned char*>(a.phi_img) +
                                                       2 * C::PSZ);
    float m = 0.f;
    if (tid < 2 * KP) m = mimg[tid];
    __syncthreads();  // every read of mus done (mv and mus share storage)
    if (tid < 2 * KP) mv[tid] = m;
    if (!tc::mbar_wait(&bars[2], 0u, tc::wait_limit_or_default(a.wait_limit))) img_timed_out = true;
  } else {
    float v[PT][4];
#pragma unroll
    for (int t = 0; t < PT; ++t) {
      int i, jq;
      task_phi(tid + NT * t, i, jq);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = 4 * jq + u;
        v[t][u] = (tid + NT * t < KP * NQ && i < k && j < k) ? __ldg(a.phi + (int64_t)i * k + j) : 0.f;
      }
    }
    __syncthreads();  // mus staged
#pragma unroll
    for (int t = 0; t < PT; ++t) {
      const int e = tid + NT * t;
      int i, jq;
      task_phi(e, i, jq);
      if (e < KP * NQ) {
        uint4 h;
        float4 l;
        tc::split4(v[t], h, l);
        const uint32_t off = tc::kmajor_off(i, 4 * jq, C::SBOJ);
        *reinterpret_cast<uint4*>(base + C::PH + off) = h;
        *reinterpret_cast<float4*>(base + C::PL + off) = l;
        float p1 = 0.f, p2 = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          p1 = fmaf(v[t][u], mus[4 * jq + u], p1);
          p2 = fmaf(v[t][u], mus[KP + 4 * jq + u], p2);
        }
        part[i * NQ + jq] = p1;
        part[KP * NQ + i * NQ + jq] = p2;
      }
    }
    __syncthreads();
    float m = 0.f;
    if (tid < 2 * KP) {
      const float* pp = part + (tid / KP) * KP * NQ + (tid % KP) * NQ;
#pragma unroll 4
      for (int jq = 0; jq < NQ; ++jq) m += pp[jq];
    }
    __syncthreads();  // every read of mus done
    if (tid < 2 * KP) mv[tid] = m;
  }

  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot, sbase = tc::sm_addr(base);
  const float cc0 = a.c0, cc2 = a.c2;
  uint32_t ph_z = 0u, ph_g = 0u;
  bool g_pending = false, timed_out = img_timed_out, any = false;
  int64_t tile = blockIdx.x;
  for (; tile < ntiles; tile += nblocks) {
    // the G products of the previous tile read y3 and C
    if (g_pending) {
      if (!tc::mbar_wait(&bars[1], ph_g, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
      ph_g ^= 1u;
      g_pending = false;
    }
    if (__syncthreads_or(timed_out)) {
      timed_out = true;
      break;
    }
    if (tile != (int64_t)blockIdx.x) store_tile();  // the first tile was staged before the wait
    int64_t x0;
    const int nv = tile_nodes(tile, x0);
    if (tile + nblocks < ntiles) load_tile(tile + nblocks);  // in flight during the MMAs
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      // K-step ks starts 256 B further: + 16 in the descriptor's address field
      constexpr uint32_t iz = tc::tf32_idesc(128, 2 * TM);
      const uint64_t dph = tc::smem_desc(sbase + C::PH, 128, C::SBOJ);
      const uint64_t dpl = tc::smem_desc(sbase + C::PL, 128, C::SBOJ);
      const uint64_t dyh = tc::smem_desc(sbase + C::Y1H, 128, C::SBOJ);
      const uint64_t dyl = tc::smem_desc(sbase + C::Y1L, 128, C::SBOJ);
#pragma unroll
      for (int ks = 0; ks < KP / 8; ++ks) {
        const uint64_t ko = 16u * ks;
        tc::mma_tf32(tmem, dph + ko, dyh + ko, iz, ks > 0 ? 1u : 0u);
        tc::mma_tf32(tmem, dph + ko, dyl + ko, iz, 1u);
        tc::mma_tf32(tmem, dpl + ko, dyh + ko, iz, 1u);
      }
      tc::commit(&bars[0]);
    }
    if (!tc::mbar_wait(&bars[0], ph_z, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
    ph_z ^= 1u;
    tc::fence_after_sync();
    {
      // warp w: TMEM lanes (rows i) 32 (w % 4) .., nodes 8 (w / 4) .. + 7
      const int sub = warp & 3, xg = warp >> 2, i = 32 * sub + lane;
      const uint32_t lb = tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(8 * xg);
      float z1[8], z2[8];
      tc::tmem_ld8(lb, z1);
      tc::tmem_ld8(lb + TM, z2);
      if (i < KP) {
        const float m1 = mv[i], m2 = mv[KP + i];
        float cv[8], d = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const bool valid = 8 * xg + u < nv && i < k;
          cv[u] = valid ? cc0 * z1[u] * z2[u] + cc2 * (z1[u] * m2 + m1 * z2[u]) : 0.f;
          if (valid) d = fmaf(z1[u], z2[u], d);
        }
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          const float v[4] = {cv[4 * h2], cv[4 * h2 + 1], cv[4 * h2 + 2], cv[4 * h2 + 3]};
          uint4 h;
          float4 l;
          tc::split4(v, h, l);
          const uint32_t off = tc::kmajor_off(i, 8 * xg + 4 * h2, C::SBOX);
          *reinterpret_cast<uint4*>(base + C::CH + off) = h;
          *reinterpret_cast<float4*>(base + C::CLO + off) = l;
        }
        dsum[xg * KP + i] += d;
      }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      constexpr uint32_t ig = tc::tf32_idesc(128, KP);
      const uint32_t d = tmem + (uint32_t)(2 * TM);
      const uint64_t dah = tc::smem_desc(sbase + C::Y3H, 128, C::SBOX);
      const uint64_t dal = tc::smem_desc(sbase + C::Y3L, 128, C::SBOX);
      const uint64_t dbh = tc::smem_desc(sbase + C::CH, 128, C::SBOX);
      const uint64_t dbl = tc::smem_desc(sbase + C::CLO, 128, C::SBOX);
#pragma unroll
      for (int ks = 0; ks < TM / 8; ++ks) {
        const uint64_t ko = 16u * ks;
        tc::mma_tf32(d, dah + ko, dbh + ko, ig, (any || ks > 0) ? 1u : 0u);
        tc::mma_tf32(d, dah + ko, dbl + ko, ig, 1u);
        tc::mma_tf32(d, dal + ko, dbh + ko, ig, 1u);
      }
      tc::commit(&bars[1]);
    }
    g_pending = true;
    any = true;
  }
  if (g_pending) {
    if (!tc::mbar_wait(&bars[1], ph_g, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
    ph_g ^= 1u;
  }
  tc::fence_after_sync();
  const bool ok = !__syncthreads_or(timed_out);
  // the tiles are dead: stage the partial over them (stage <= base)
  {
    const int sub = warp & 3, cg4 = warp >> 2, j = 32 * sub + lane;
    for (int c4 = 0; c4 < NQ; c4 += 4) {
      const int ic = cg4 * NQ + c4;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (ok && any) tc::tmem_ld4(tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(2 * TM + ic), v);
      if (j < KP)
#pragma unroll
        for (int u = 0; u < 4; ++u) stage[(ic + u) * KP + j] = v[u];
    }
  }
  for (int e = tid; e < 3 * KP + 1; e += NT)
    stage[KP * KP + e] = e < KP ? ((dsum[e] + dsum[KP + e]) + (dsum[2 * KP + e] + dsum[3 * KP + e])) : 0.f;
  if (!ok && tid == 0 && a.flags) atomicOr(a.flags, kFlagTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

// The BF16 tensor-core adjoint contraction of one CTA: stages this CTA's
// partial (G column-major at stage[i KP + j], the three d-sums, a zero loss)
// at `stage`, as the CUDA-core form does.
template <int KP>
__device__ __forceinline__ void contract_tc_bf(const StpmPartialArgs& a, int nblocks,
                                               unsigned char* smraw, float* stage) {
  using C = ContractTcBf<KP>;
  constexpr int TM = C::TM, NT = 512, NJ = KP / 8;  // 16-byte chunks (8 elements) along j
  __shared__ __align__(8) uint64_t bars[2];  // Z products done | G products done
  __shared__ uint32_t tmem_slot;
  unsigned char* base = smraw + ((1024 - (tc::sm_addr(smraw) & 1023)) & 1023);
  float* mv = reinterpret_cast<float*>(base + C::REGION);  // m1 | m2 | m3
  float* dsum = mv + 3 * KP;                               // [pair][node group][i]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k = a.k;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, C::TMEM_COLS);
  if (tid == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // Node tiles, one tile ahead in registers.  Row form (B of the Z product):
  // task (q, x, chunk) = one 16-byte load of y_q's row x; the 8 lanes of a
  // quarter-warp take 8 consecutive rows, so they write one whole core matrix.
  // Transposed form (A of the G product): task (c, j, node chunk) = 8 scalar
  // loads of column j (lanes along j: coalesced) packed into one 16-byte row.
  constexpr int TR = 3 * TM * NJ, SR = (TR + NT - 1) / NT;
  constexpr int TT = 3 * KP * (TM / 8), ST = (TT + NT - 1) / NT;
  uint4 pr[SR], pt[ST];
  auto yh = [&](int q) {
    return static_cast<const unsigned short*>(q == 0 ? a.yh1 : q == 1 ? a.yh2 : a.yh3);
  };
  auto task_row = [&](int e, int& q, int& x, int& jc) {
    const int grp = e >> 3, rest = grp / (TM / 8);
    x = 8 * (grp % (TM / 8)) + (e & 7);
    jc = rest % NJ;
    q = rest / NJ;
  };
  auto tile_nodes = [&](int64_t tile, int64_t& x0) {
    x0 = a.begin + tile * TM;
    const int64_t left = a.begin + a.count - x0;
    return left < TM ? (int)left : TM;
  };
  auto load_tile = [&](int64_t tile) {
    int64_t x0;
    const int nv = tile_nodes(tile, x0);
#pragma unroll
    for (int s = 0; s < SR; ++s) {
      const int e = tid + NT * s;
      pr[s] = make_uint4(0u, 0u, 0u, 0u);
      if (e < TR) {
        int q, x, jc;
        task_row(e, q, x, jc);
        if (x < nv && 8 * jc < a.ldyh)
          pr[s] = __ldg(reinterpret_cast<const uint4*>(yh(q) + (x0 + x) * a.ldyh + 8 * jc));
      }
    }
#pragma unroll
    for (int s = 0; s < ST; ++s) {
      const int e = tid + NT * s, j = e % KP, rest = e / KP, xc = rest % (TM / 8), c = rest / (TM / 8);
      uint32_t w[4] = {0u, 0u, 0u, 0u};
      if (e < TT && j < a.ldyh) {
        const unsigned short* Yc = yh(c);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int x = 8 * xc + u;
          const uint32_t v = x < nv ? (uint32_t)__ldg(Yc + (x0 + x) * a.ldyh + j) : 0u;
          w[u >> 1] |= v << (16 * (u & 1));
        }
      }
      pt[s] = make_uint4(w[0], w[1], w[2], w[3]);
    }
  };
  auto store_tile = [&]() {
#pragma unroll
    for (int s = 0; s < SR; ++s) {
      const int e = tid + NT * s;
      if (e < TR) {
        int q, x, jc;
        task_row(e, q, x, jc);
        *reinterpret_cast<uint4*>(base + C::YB + q * C::TSZ + tc::kmajor16_off(x, 8 * jc, C::SBOJ)) = pr[s];
      }
    }
#pragma unroll
    for (int s = 0; s < ST; ++s) {
      const int e = tid + NT * s, j = e % KP, rest = e / KP, xc = rest % (TM / 8), c = rest / (TM / 8);
      if (e < TT)
        *reinterpret_cast<uint4*>(base + C::YT + c * C::TSZ + tc::kmajor16_off(j, 8 * xc, C::SBOX)) = pt[s];
    }
  };
  const int64_t ntiles = ceil_div_dev(a.count, TM);
  float* mus = mv;  // mu_1 | mu_2 | mu_3 staged in mv
  // everything that does not read Phi happens before the dependency wait
  const bool first_staged = (int64_t)blockIdx.x < ntiles;
  if (first_staged) load_tile(blockIdx.x);
  for (int e = tid; e < 3 * KP; e += NT) {
    const float* mu = e < KP ? a.mu1 : e < 2 * KP ? a.mu2 : a.mu3;
    const int j = e % KP;
    mus[e] = (mu && j < k) ? mu[j] : 0.f;
  }
  for (int e = tid; e < 12 * KP; e += NT) dsum[e] = 0.f;
  if (first_staged) store_tile();
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // Phi as a BF16 pair (hi = bf16(Phi), lo = bf16(Phi - hi)); the partial dot
  // products of each chunk with mu_1..3 (FP32 Phi) go to part[] in the C
  // area and are summed per column in a fixed order: m_q = Phi^T mu_q
  constexpr int PT = (KP * NJ + NT - 1) / NT;
  float* part = reinterpret_cast<float*>(base + C::CB);  // [q][i][jc]
  static_assert(3 * KP * NJ * 4 <= 3 * C::TSZ, "partials fit the C area");
  {
    float v[PT][8];
#pragma unroll
    for (int t = 0; t < PT; ++t) {
      const int e = tid + NT * t, grp = e >> 3, i = 8 * (grp % (KP / 8)) + (e & 7), jc = grp / (KP / 8);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = 8 * jc + u;
        v[t][u] = (e < KP * NJ && i < k && j < k) ? __ldg(a.phi + (int64_t)i * k + j) : 0.f;
      }
    }
    __syncthreads();  // mus staged
#pragma unroll
    for (int t = 0; t < PT; ++t) {
      const int e = tid + NT * t, grp = e >> 3, i = 8 * (grp % (KP / 8)) + (e & 7), jc = grp / (KP / 8);
      if (e < KP * NJ) {
        uint32_t h[4] = {0u, 0u, 0u, 0u}, l[4] = {0u, 0u, 0u, 0u};
        float p1 = 0.f, p2 = 0.f, p3 = 0.f;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const __nv_bfloat16 hb = __float2bfloat16_rn(v[t][u]);
          const __nv_bfloat16 lb = __float2bfloat16_rn(v[t][u] - __bfloat162float(hb));
          h[u >> 1] |= (uint32_t)__bfloat16_as_ushort(hb) << (16 * (u & 1));
          l[u >> 1] |= (uint32_t)__bfloat16_as_ushort(lb) << (16 * (u & 1));
          p1 = fmaf(v[t][u], mus[8 * jc + u], p1);
          p2 = fmaf(v[t][u], mus[KP + 8 * jc + u], p2);
          p3 = fmaf(v[t][u], mus[2 * KP + 8 * jc + u], p3);
        }
        const uint32_t off = tc::kmajor16_off(i, 8 * jc, C::SBOJ);
        *reinterpret_cast<uint4*>(base + C::PH + off) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(base + C::PL + off) = make_uint4(l[0], l[1], l[2], l[3]);
        part[i * NJ + jc] = p1;
        part[KP * NJ + i * NJ + jc] = p2;
        part[2 * KP * NJ + i * NJ + jc] = p3;
      }
    }
    __syncthreads();
    float m = 0.f;
    if (tid < 3 * KP) {
      const float* pp = part + (tid / KP) * KP * NJ + (tid % KP) * NJ;
#pragma unroll 2
      for (int jc = 0; jc < NJ; ++jc) m += pp[jc];
    }
    __syncthreads();  // every read of mus done
    if (tid < 3 * KP) mv[tid] = m;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot, sbase = tc::sm_addr(base);
  const float cc0 = a.c0, cc2 = a.c2;
  uint32_t ph_z = 0u, ph_g = 0u;
  bool g_pending = false, timed_out = false, any = false;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += nblocks) {
    if (g_pending) {  // the G products of the previous tile read y^T and C
      if (!tc::mbar_wait(&bars[1], ph_g, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
      ph_g ^= 1u;
      g_pending = false;
    }
    if (__syncthreads_or(timed_out)) {
      timed_out = true;
      break;
    }
    if (tile != (int64_t)blockIdx.x) store_tile();
    int64_t x0;
    const int nv = tile_nodes(tile, x0);
    if (tile + nblocks < ntiles) load_tile(tile + nblocks);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      constexpr uint32_t iz = tc::bf16_idesc(128, 3 * TM);
      const uint64_t dph = tc::smem_desc(sbase + C::PH, 128, C::SBOJ);
      const uint64_t dpl = tc::smem_desc(sbase + C::PL, 128, C::SBOJ);
      const uint64_t dy = tc::smem_desc(sbase + C::YB, 128, C::SBOJ);
#pragma unroll
      for (int ks = 0; ks < KP / 16; ++ks) {
        const uint64_t ko = 16u * ks;  // 256 bytes: two core matrices along K
        tc::mma_bf16(tmem, dph + ko, dy + ko, iz, ks > 0 ? 1u : 0u);
        tc::mma_bf16(tmem, dpl + ko, dy + ko, iz, 1u);
      }
      tc::commit(&bars[0]);
    }
    if (!tc::mbar_wait(&bars[0], ph_z, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
    ph_z ^= 1u;
    tc::fence_after_sync();
    {
      // warp w: TMEM lanes (rows i) 32 (w % 4) .., nodes 16 (w / 4) .. + 15
      const int sub = warp & 3, xg = warp >> 2, i = 32 * sub + lane;
      const uint32_t lb = tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(16 * xg);
      const float m1 = i < KP ? mv[i] : 0.f, m2 = i < KP ? mv[KP + i] : 0.f,
                  m3 = i < KP ? mv[2 * KP + i] : 0.f;
      float d0 = 0.f, d1 = 0.f, d2 = 0.f;
#pragma unroll
      for (int h2 = 0; h2 < 2; ++h2) {  // 8 nodes at a time (warp-wide TMEM loads)
        float z1[8], z2[8], z3[8];
        tc::tmem_ld8(lb + 8 * h2, z1);
        tc::tmem_ld8(lb + TM + 8 * h2, z2);
        tc::tmem_ld8(lb + 2 * TM + 8 * h2, z3);
        if (i < KP) {
          uint32_t w0[4] = {0u, 0u, 0u, 0u}, w1[4] = {0u, 0u, 0u, 0u}, w2[4] = {0u, 0u, 0u, 0u};
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const bool valid = 16 * xg + 8 * h2 + u < nv && i < k;
            const float a1 = z1[u], a2 = z2[u], a3 = z3[u];
            const float v0 = valid ? cc0 * a2 * a3 + cc2 * (a2 * m3 + m2 * a3) : 0.f;
            const float v1 = valid ? cc0 * a1 * a3 + cc2 * (a1 * m3 + m1 * a3) : 0.f;
            const float v2 = valid ? cc0 * a1 * a2 + cc2 * (a1 * m2 + m1 * a2) : 0.f;
            if (valid) {
              d0 = fmaf(a2, a3, d0);
              d1 = fmaf(a1, a3, d1);
              d2 = fmaf(a1, a2, d2);
            }
            const int sh = 16 * (u & 1);
            w0[u >> 1] |= (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v0)) << sh;
            w1[u >> 1] |= (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v1)) << sh;
            w2[u >> 1] |= (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v2)) << sh;
          }
          const uint32_t off = tc::kmajor16_off(i, 16 * xg + 8 * h2, C::SBOX);
          *reinterpret_cast<uint4*>(base + C::CB + off) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
          *reinterpret_cast<uint4*>(base + C::CB + C::TSZ + off) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
          *reinterpret_cast<uint4*>(base + C::CB + 2 * C::TSZ + off) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
        }
      }
      if (i < KP) {
        dsum[(0 * 4 + xg) * KP + i] += d0;
        dsum[(1 * 4 + xg) * KP + i] += d1;
        dsum[(2 * 4 + xg) * KP + i] += d2;
      }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      constexpr uint32_t ig = tc::bf16_idesc(128, KP);
      const uint32_t d = tmem + (uint32_t)(3 * TM);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const uint64_t da = tc::smem_desc(sbase + C::YT + c * C::TSZ, 128, C::SBOX);
        const uint64_t db = tc::smem_desc(sbase + C::CB + c * C::TSZ, 128, C::SBOX);
#pragma unroll
        for (int ks = 0; ks < TM / 16; ++ks)
          tc::mma_bf16(d, da + 16u * ks, db + 16u * ks, ig, (any || c > 0 || ks > 0) ? 1u : 0u);
      }
      tc::commit(&bars[1]);
    }
    g_pending = true;
    any = true;
  }
  if (g_pending) {
    if (!tc::mbar_wait(&bars[1], ph_g, tc::wait_limit_or_default(a.wait_limit))) timed_out = true;
    ph_g ^= 1u;
  }
  tc::fence_after_sync();
  const bool ok = !__syncthreads_or(timed_out);
  {
    const int sub = warp & 3, cg4 = warp >> 2, j = 32 * sub + lane;
    constexpr int NQ = KP / 4;
    for (int c4 = 0; c4 < NQ; c4 += 4) {
      const int ic = cg4 * NQ + c4;
      float v[4] = {0.f, 0.f, 0.f, 0.f};
      if (ok && any)
        tc::tmem_ld4(tmem + ((uint32_t)(32 * sub) << 16) + (uint32_t)(3 * TM + ic), v);
      if (j < KP)
#pragma unroll
        for (int u = 0; u < 4; ++u) stage[(ic + u) * KP + j] = v[u];
    }
  }
  for (int e = tid; e < 3 * KP + 1; e += NT) {
    float v = 0.f;
    if (e < 3 * KP) {
      const float* ds = dsum + (e / KP) * 4 * KP + e % KP;
      v = (ds[0] + ds[KP]) + (ds[2 * KP] + ds[3 * KP]);
    }
    stage[KP * KP + e] = v;
  }
  if (!ok && tid == 0 && a.flags) atomicOr(a.flags, kFlagTimeout);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

template <int KP, int MODE, bool BF>
__device__ __forceinline__ void contract_body(const StpmPartialArgs& a, int nblocks) {
  using Cfg = Contract<KP, MODE, BF>;
  using T = typename Cfg::T;
  constexpr int TM = Cfg::TM, NZ = Cfg::NZ, NC = Cfg::NC, PLD = Cfg::PLD, LDY = Cfg::LDY,
                LDC = Cfg::LDC;
  constexpr int IB = Cfg::IB;
  static_assert(KP % 16 == 0 && KP <= 256, "KP");
  extern __shared__ __align__(16) unsigned char smraw[];
  if constexpr (Cfg::TC) {  // waits for the previous kernel itself, after its own prologue
    static_assert(Cfg::NT == 512 && Cfg::NBC == 1, "tensor-core contraction launch shape");
    float* stage = reinterpret_cast<float*>(smraw);
    contract_tc<KP>(a, nblocks, smraw, stage);
    partial_cluster_sum<KP, IB, Cfg::NBC, MODE>(a, stage, 0, 0);
    return;
  } else if constexpr (Cfg::TCBF) {  // likewise
    static_assert(Cfg::NT == 512 && Cfg::NBC == 1, "tensor-core contraction launch shape");
    float* stage = reinterpret_cast<float*>(smraw);
    contract_tc_bf<KP>(a, nblocks, smraw, stage);
    partial_cluster_sum<KP, IB, Cfg::NBC, MODE>(a, stage, 0, 0);
    return;
  }
  // programmatic serialization: wait for the previous kernel (the step that
  // wrote Phi), then let the next one be scheduled early
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  // this CTA's columns of Phi: i0 + ii, ii < IB (i local below)
  const int cb = (Cfg::NBC > 1) ? (int)blockIdx.y : 0, i0 = cb * IB;
  T* Phis = reinterpret_cast<T*>(smraw);  // Phis[ii PLD + j] = Phi_j,i0+ii (column i0+ii of Phi)
  T* Ys = Phis + IB * PLD;                // 3 node-major tiles: Ys[q TM LDY + x LDY + j]
  T* CT = Ys + 3 * TM * LDY;              // NC coefficient tiles, i-major: CT[c IB LDC + ii LDC + x]
  T* PhiLo = CT + NC * IB * LDC;          // BF16 form: Phi - hi(Phi), same layout as Phis
  float* mv = reinterpret_cast<float*>(smraw + Cfg::region);  // m1 | m2 | m3 (IB each)
  constexpr int NW = Cfg::NW, NT = Cfg::NT;
  float* tred = mv + 3 * IB;                                  // NW loss partials
  float* dw = tred + NW;  // per-warp d-sums (3 IB each), summed in a fixed order at the end
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t4 = lane & 3;
  const int k = a.k;

  // Phi: loads issued in batches of 8 per thread so that their latencies overlap
  {
    constexpr int N = IB * PLD, B = 8;
    for (int e0 = tid; e0 < N; e0 += NT * B) {
      float v[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int e = e0 + NT * u, i = i0 + e / PLD, j = e % PLD;
        v[u] = (e < N && i < k && j < k) ? __ldg(a.phi + (int64_t)i * k + j) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (e0 + NT * u < N) {
          const T hi = to_elem<T>(v[u]);
          Phis[e0 + NT * u] = hi;
          if (BF) PhiLo[e0 + NT * u] = to_elem<T>(v[u] - to_f32(hi));
        }
    }
  }
  // m_P = Phi^T mu_P with Phi as staged (mu_1..3 staged in dw, which is
  // free until the d-sums start)
  for (int e = tid; e < 3 * KP; e += NT) {
    const int which = e / KP, j = e % KP;
    const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
    dw[e] = (mu && j < k) ? mu[j] : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < 3 * IB; e += NT) {
    const float* mu = dw + (e / IB) * KP;
    const T* ph = Phis + (e % IB) * PLD;
    const T* pl = PhiLo + (e % IB) * PLD;
    float s0 = 0.f, s1 = 0.f;
#pragma unroll 4
    for (int j = 0; j < KP; j += 2) {
      float p0 = to_f32(ph[j]), p1 = to_f32(ph[j + 1]);
      if (BF) {
        p0 += to_f32(pl[j]);
        p1 += to_f32(pl[j + 1]);
      }
      s0 = fmaf(p0, mu[j], s0);
      s1 = fmaf(p1, mu[j + 1], s1);
    }
    mv[e] = s0 + s1;
  }
  __syncthreads();
  for (int e = tid; e < NW * 3 * IB; e += NT) dw[e] = 0.f;
  if (tid < NW) tred[tid] = 0.f;
  __syncthreads();

  float gacc[Cfg::GPW][4];
#pragma unroll
  for (int u = 0; u < Cfg::GPW; ++u)
#pragma unroll
    for (int q = 0; q < 4; ++q) gacc[u][q] = 0.f;
  float tsum = 0.f;
  const float cc0 = a.c0, cc2 = a.c2;

  const int64_t ntiles = ceil_div_dev(a.count, TM);
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += nblocks) {
    const int64_t x0 = a.begin + tile * TM;
    const int64_t left = a.begin + a.count - x0;
    const int nvalid = left < TM ? (int)left : TM;
    // node tiles, 16-byte chunks; columns past the stored row are zero
    constexpr int CH = 16 / (int)sizeof(T), NCH = KP / CH;
    {
      constexpr int N = 3 * TM * NCH, B = 4;
      for (int e0 = tid; e0 < N; e0 += NT * B) {
        uint4 v[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int e = e0 + NT * u;
          const int q = e / (TM * NCH), rem = e % (TM * NCH), xx = rem / NCH, c = rem % NCH;
          v[u] = make_uint4(0u, 0u, 0u, 0u);
          if (e < N) {
            if (BF) {
              const T* Y = static_cast<const T*>(q == 0 ? a.yh1 : q == 1 ? a.yh2 : a.yh3);
              if (xx < nvalid && c * CH < a.ldyh)
                v[u] = __ldg(reinterpret_cast<const uint4*>(Y + (x0 + xx) * a.ldyh + c * CH));
            } else {
              const float* Y = q == 0 ? a.y1 : q == 1 ? a.y2 : a.y3;
              if (xx < nvalid && c * CH < a.ldy)
                v[u] = __ldg(reinterpret_cast<const uint4*>(Y + (x0 + xx) * a.ldy + c * CH));
            }
          }
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
          const int e = e0 + NT * u;
          if (e >= N) break;
          const int q = e / (TM * NCH), rem = e % (TM * NCH), xx = rem / NCH, c = rem % NCH;
          *reinterpret_cast<uint4*>(Ys + q * TM * LDY + xx * LDY + c * CH) = v[u];
        }
      }
    }
    __syncthreads();

    // ---- Z^T tiles (16 i x 8 x), C and the d-sums
    for (int p = warp; p < Cfg::MTI * Cfg::NTX; p += NW) {
      const int m0 = (p % Cfg::MTI) * 16, n0 = (p / Cfg::MTI) * 8;
      float z[NZ][4];
#pragma unroll
      for (int q = 0; q < NZ; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) z[q][r] = 0.f;
      if (BF) {
#pragma unroll 2
        for (int k0 = 0; k0 < KP; k0 += 16) {
          const T* pa = Phis + m0 * PLD + k0 + 2 * t4;
          const T* pl = PhiLo + m0 * PLD + k0 + 2 * t4;
          const uint32_t af[4] = {ld_b32(pa + g * PLD), ld_b32(pa + (g + 8) * PLD),
                                  ld_b32(pa + g * PLD + 8), ld_b32(pa + (g + 8) * PLD + 8)};
          const uint32_t afl[4] = {ld_b32(pl + g * PLD), ld_b32(pl + (g + 8) * PLD),
                                   ld_b32(pl + g * PLD + 8), ld_b32(pl + (g + 8) * PLD + 8)};
#pragma unroll
          for (int q = 0; q < NZ; ++q) {
            const T* pb = Ys + q * TM * LDY + (n0 + g) * LDY + k0 + 2 * t4;
            const uint32_t bf[2] = {ld_b32(pb), ld_b32(pb + 8)};
            mma_bf16(z[q], af, bf);
            mma_bf16(z[q], afl, bf);
          }
        }
      } else {
        float zc[NZ][4];
#pragma unroll
        for (int q = 0; q < NZ; ++q)
#pragma unroll
          for (int r = 0; r < 4; ++r) zc[q][r] = 0.f;
#pragma unroll 2
        for (int k0 = 0; k0 < KP; k0 += 8) {
          const float* pa = reinterpret_cast<const float*>(Phis) + m0 * PLD + k0 + t4;
          uint32_t ah[4], al[4];
          split_tf32(pa[g * PLD], ah[0], al[0]);
          split_tf32(pa[(g + 8) * PLD], ah[1], al[1]);
          split_tf32(pa[g * PLD + 4], ah[2], al[2]);
          split_tf32(pa[(g + 8) * PLD + 4], ah[3], al[3]);
#pragma unroll
          for (int q = 0; q < NZ; ++q) {
            const float* pb = reinterpret_cast<const float*>(Ys) + q * TM * LDY + (n0 + g) * LDY + k0 + t4;
            uint32_t bh[2], bl[2];
            split_tf32(pb[0], bh[0], bl[0]);
            split_tf32(pb[4], bh[1], bl[1]);
            mma_tf32(z[q], ah, bh);
            mma_tf32(zc[q], ah, bl);
            mma_tf32(zc[q], al, bh);
          }
        }
#pragma unroll
        for (int q = 0; q < NZ; ++q)
#pragma unroll
          for (int r = 0; r < 4; ++r) z[q][r] += zc[q][r];
      }
      // epilogue: fragment r holds (i = m0 + g + 8 (r >> 1), x = n0 + 2 t4 + (r & 1))
      float dl[3][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      float cv[3][4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = m0 + g + 8 * (r >> 1), x = n0 + 2 * t4 + (r & 1);
        const bool valid = x < nvalid && i0 + i < k;
        const float m1 = mv[i], m2 = mv[IB + i];
        const float z1 = z[0][r], z2 = z[1][r];
        if (MODE == kModePlain) {
          cv[0][r] = valid ? cc0 * z1 * z2 + cc2 * (z1 * m2 + m1 * z2) : 0.f;
          if (valid) dl[0][r >> 1] = fmaf(z1, z2, dl[0][r >> 1]);
        } else {
          const float m3 = mv[2 * IB + i], z3 = z[NZ - 1][r];
          if (MODE == kModeAdjoint) {
            cv[0][r] = valid ? cc0 * z2 * z3 + cc2 * (z2 * m3 + m2 * z3) : 0.f;
            cv[1][r] = valid ? cc0 * z1 * z3 + cc2 * (z1 * m3 + m1 * z3) : 0.f;
            cv[2][r] = valid ? cc0 * z1 * z2 + cc2 * (z1 * m2 + m1 * z2) : 0.f;
          }
          if (valid) {
            dl[0][r >> 1] = fmaf(z2, z3, dl[0][r >> 1]);
            dl[1][r >> 1] = fmaf(z1, z3, dl[1][r >> 1]);
            dl[2][r >> 1] = fmaf(z1, z2, dl[2][r >> 1]);
            if (MODE == kModeLoss)
              tsum += cc0 * z1 * z2 * z3 + cc2 * (z1 * z2 * m3 + z1 * m2 * z3 + m1 * z2 * z3);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          T* dst = CT + c * IB * LDC + (m0 + g + 8 * h) * LDC + n0 + 2 * t4;
          if (BF) {
            *reinterpret_cast<__nv_bfloat162*>(dst) = __floats2bfloat162_rn(cv[c][2 * h], cv[c][2 * h + 1]);
          } else {
            *reinterpret_cast<float2*>(dst) = make_float2(cv[c][2 * h], cv[c][2 * h + 1]);
          }
        }
#pragma unroll
      for (int qd = 0; qd < 3; ++qd) {
        if (MODE == kModePlain && qd > 0) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float v = dl[qd][h];
          v += __shfl_xor_sync(0xffffffffu, v, 1);
          v += __shfl_xor_sync(0xffffffffu, v, 2);
          if (t4 == 0) dw[warp * 3 * IB + qd * IB + m0 + g + 8 * h] += v;
        }
      }
    }
    __syncthreads();

    // ---- G (16 j x 8 i tiles) += Yout^T C over this tile's nodes
    if (NC > 0) {
#pragma unroll
      for (int k0 = 0; k0 < TM; k0 += Cfg::KSTEP) {
#pragma unroll
        for (int u = 0; u < Cfg::GPW; ++u) {
          const int tt = warp + NW * u;
          if (tt >= Cfg::GT) continue;
          const int m0 = (tt % Cfg::MTJ) * 16, n0 = (tt / Cfg::MTJ) * 8;
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            const T* Yo = Ys + (MODE == kModePlain ? 2 : c) * TM * LDY;
            const T* Cc = CT + c * IB * LDC;
            if (BF) {
              uint32_t af[4];
              const int q = lane >> 3, rr = lane & 7;
              ldsm_x4_trans(af, Yo + (k0 + (q >> 1) * 8 + rr) * LDY + m0 + (q & 1) * 8);
              const T* pb = Cc + (n0 + g) * LDC + k0 + 2 * t4;
              const uint32_t bf[2] = {ld_b32(pb), ld_b32(pb + 8)};
              mma_bf16(gacc[u], af, bf);
            } else {
              const float* pa = reinterpret_cast<const float*>(Yo) + (k0 + t4) * LDY + m0 + g;
              uint32_t ah[4], al[4];
              split_tf32(pa[0], ah[0], al[0]);
              split_tf32(pa[8], ah[1], al[1]);
              split_tf32(pa[4 * LDY], ah[2], al[2]);
              split_tf32(pa[4 * LDY + 8], ah[3], al[3]);
              const float* pb = reinterpret_cast<const float*>(Cc) + (n0 + g) * LDC + k0 + t4;
              uint32_t bh[2], bl[2];
              split_tf32(pb[0], bh[0], bl[0]);
              split_tf32(pb[4], bh[1], bl[1]);
              mma_tf32(gacc[u], ah, bh);
              mma_tf32(gacc[u], ah, bl);
              mma_tf32(gacc[u], al, bh);
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (MODE == kModeLoss) {
#pragma unroll
    for (int off = 16; off; off >>= 1) tsum += __shfl_xor_sync(0xffffffffu, tsum, off);
    if (lane == 0) tred[warp] = tsum;
  }
  // cluster reduction: every CTA stages its partial (this column block of
  // the k x k column-major contraction, its 3 d-sums, loss) in shared memory;
  // CTA r of the cluster sums a 1/CLP slice over the cluster's CTAs through
  // DSMEM and writes it out.  Column block cb writes loss slot cb of the 4
  // spare floats of the partial row (block 0 also clears the unused slots).
  float* stage = reinterpret_cast<float*>(smraw);  // tiles are dead from here on
  if (NC > 0) {
#pragma unroll
    for (int u = 0; u < Cfg::GPW; ++u) {
      const int tt = warp + NW * u;
      if (tt >= Cfg::GT) continue;
      const int m0 = (tt % Cfg::MTJ) * 16, n0 = (tt / Cfg::MTJ) * 8;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int j = m0 + g + 8 * (r >> 1), i = n0 + 2 * t4 + (r & 1);
        stage[i * KP + j] = gacc[u][r];
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < 3 * IB; e += NT) {
    float v = 0.f;
#pragma unroll
    for (int w = 0; w < NW; ++w) v += dw[w * 3 * IB + e];
    stage[KP * IB + e] = v;
  }
  if (tid == 0) {
    float t = 0.f;
    if (MODE == kModeLoss)
      for (int w = 0; w < NW; ++w) t += tred[w];
    stage[KP * IB + 3 * IB] = t;
  }
  partial_cluster_sum<KP, IB, Cfg::NBC, MODE>(a, stage, cb, i0);
}

template <int KP, int MODE, bool BF>
__global__ void __launch_bounds__(Contract<KP, MODE, BF>::NT) stpm_contract_kernel(StpmPartialArgs a) {
  contract_body<KP, MODE, BF>(a, gridDim.x);
}

// blockIdx.y selects the graph; its first a.nblocks CTAs (a multiple of the
// cluster size) work, the rest and graphs without nodes this round leave
template <int KP, int MODE, bool BF>
__global__ void __launch_bounds__(Contract<KP, MODE, BF>::NT) stpm_contract_batched(const StpmPartialArgs* __restrict__ args) {
  const StpmPartialArgs a = args[blockIdx.y];
  if ((int)blockIdx.x >= a.nblocks || a.count <= 0) return;
  contract_body<KP, MODE, BF>(a, a.nblocks);
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
                                    double* __restrict__ lambda, double* __restrict__ phi64) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (i >= k) return;
  double s = 0.0;
  for (int j = lane; j < k; j += 32)
    s += (phi64 ? phi64[(int64_t)i * k + j] : (double)phi[(int64_t)i * k + j]) * G[(int64_t)i * k + j];
#pragma unroll
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  const bool flip = s < 0.0;
  if (lane == 0) lambda[i] = flip ? -s : s;
  if (flip)
    for (int j = lane; j < k; j += 32) {
      phi[(int64_t)i * k + j] = -phi[(int64_t)i * k + j];
      if (phi64) phi64[(int64_t)i * k + j] = -phi64[(int64_t)i * k + j];
    }
}

template <int KP, int MODE, bool BF>
cudaError_t launch_partial_t(const StpmPartialArgs& a, int grid, cudaStream_t s) {
  const size_t smem = Contract<KP, MODE, BF>::smem;
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_contract_kernel<KP, MODE, BF>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, (unsigned)Contract<KP, MODE, BF>::NBC, 1);
  cfg.blockDim = dim3(Contract<KP, MODE, BF>::NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kPartialCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // see contract_body
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_contract_kernel<KP, MODE, BF>, a));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int MODE, bool BF>
cudaError_t launch_partial_m(int KP, const StpmPartialArgs& a, int grid, cudaStream_t s) {
  switch (KP) {
    case 32: return launch_partial_t<32, MODE, BF>(a, grid, s);
    case 48: return launch_partial_t<48, MODE, BF>(a, grid, s);
    case 64: return launch_partial_t<64, MODE, BF>(a, grid, s);
    case 80: return launch_partial_t<80, MODE, BF>(a, grid, s);
    case 96: return launch_partial_t<96, MODE, BF>(a, grid, s);
    case 112: return launch_partial_t<112, MODE, BF>(a, grid, s);
    case 128: return launch_partial_t<128, MODE, BF>(a, grid, s);
    case 160: return launch_partial_t<160, MODE, BF>(a, grid, s);
    case 208: return launch_partial_t<208, MODE, BF>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <bool BF>
cudaError_t launch_partial_p(int mode, int KP, const StpmPartialArgs& a, int grid, cudaStream_t s) {
  switch (mode) {
    case kModePlain: return launch_partial_m<kModePlain, BF>(KP, a, grid, s);
    case kModeAdjoint: return launch_partial_m<kModeAdjoint, BF>(KP, a, grid, s);
    case kModeLoss: return launch_partial_m<kModeLoss, BF>(KP, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int KP, int MODE, bool BF>
cudaError_t launch_partial_batched_t(const StpmPartialArgs* args, int graphs, int grid,
                                     cudaStream_t s) {
  const size_t smem = Contract<KP, MODE, BF>::smem;
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_contract_batched<KP, MODE, BF>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, (unsigned)graphs, 1);
  cfg.blockDim = dim3(Contract<KP, MODE, BF>::NT, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kPartialCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_contract_batched<KP, MODE, BF>, args));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int MODE, bool BF>
cudaError_t launch_partial_batched_m(int KP, const StpmPartialArgs* args, int graphs, int grid,
                                     cudaStream_t s) {
  switch (KP) {
    case 32: return launch_partial_batched_t<32, MODE, BF>(args, graphs, grid, s);
    case 48: return launch_partial_batched_t<48, MODE, BF>(args, graphs, grid, s);
    case 64: return launch_partial_batched_t<64, MODE, BF>(args, graphs, grid, s);
    case 80: return launch_partial_batched_t<80, MODE, BF>(args, graphs, grid, s);
    case 96: return launch_partial_batched_t<96, MODE, BF>(args, graphs, grid, s);
    case 112: return launch_partial_batched_t<112, MODE, BF>(args, graphs, grid, s);
    case 128: return launch_partial_batched_t<128, MODE, BF>(args, graphs, grid, s);
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
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;  // see step_body
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_step_kernel<KP, CL>, a));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int KP>
cudaError_t launch_step_k(const StpmUpdateArgs& a, cudaStream_t s) {
  // KP / 8 CTAs (8 columns each; up to 16, a non-portable cluster size) where
  // the device can co-schedule them, else KP / 16 CTAs of 16 columns; above
  // KP = 128 always KP / 16 (a cluster holds at most 16 CTAs)
  if constexpr (KP > 128) {
    return launch_step_t<KP, KP / 16>(a, s);
  } else {
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
}

template <int KP, int CL>
cudaError_t launch_step_batched_t(const StpmUpdateArgs* args, int graphs, cudaStream_t s) {
  const size_t smem = sizeof(float) * StepSmem<KP, CL>::floats;
  static bool set = false;
  if (!set) {
    MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_step_batched<KP, CL>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (CL > 8)
      MMSB_CUDA_TRY(cudaFuncSetAttribute(stpm_step_batched<KP, CL>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL, (unsigned)graphs, 1);
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
  MMSB_CUDA_TRY(cudaLaunchKernelEx(&cfg, stpm_step_batched<KP, CL>, args));
  ++g_launch_count;
  return cudaGetLastError();
}

template <int KP>
cudaError_t launch_step_batched_k(const StpmUpdateArgs* args, int graphs, cudaStream_t s) {
  static int wide = -1;
  if (wide != 0) {
    cudaError_t e = launch_step_batched_t<KP, KP / 8>(args, graphs, s);
    if (e == cudaSuccess) {
      wide = 1;
      return e;
    }
    if (wide == 1) return e;
    cudaGetLastError();
    wide = 0;
  }
  return launch_step_batched_t<KP, KP / 16>(args, graphs, s);
}

}  // namespace

int stpm_partial_cluster() { return kPartialCluster; }

// padded k of the STPM kernels: multiples of 16 from 32 to 128, then 160 and
// 208 (k <= 208); -1 beyond
int stpm_kp(int k) {
  const int r = (int)round_up(k, 16);
  if (r <= 32) return 32;
  if (r <= 128) return r;
  if (r <= 160) return 160;
  if (r <= 208) return 208;
  return -1;
}

int stpm_partial_grid(int64_t count, bool bf16) {
  // at least 64 nodes per CTA (two FP32 tiles, one BF16 tile): measured on
  // 4,096-node minibatches at k = 100, 64 CTAs beat 128 (44 vs 53 us in FP32;
  // staging Phi and the cluster reduction are per-CTA costs)
  (void)bf16;
  // MMSB_CONTRACT_NODES overrides the 64 nodes per CTA (a tuning override)
  static const int64_t per_cta = []() {
    const char* e = std::getenv("MMSB_CONTRACT_NODES");
    const long v = e ? std::strtol(e, nullptr, 10) : 0;
    return v >= 16 ? (int64_t)v : (int64_t)64;
  }();
  const int64_t tiles = ceil_div(count, per_cta);
  // MMSB_CONTRACT_CTAS caps the contraction CTAs of single-graph runs (a
  // tuning override; default 2 per SM)
  static const int64_t cap = []() {
    const char* e = std::getenv("MMSB_CONTRACT_CTAS");
    const long v = e ? std::strtol(e, nullptr, 10) : 0;
    return v > 0 ? (int64_t)v : (int64_t)2 * kNumSMs;
  }();
  const int64_t g = std::max<int64_t>(1, std::min<int64_t>(tiles, cap));
  return (int)round_up(g, kPartialCluster);
}

cudaError_t stpm_partial(int mode, const StpmPartialArgs& a, int grid, bool bf16, cudaStream_t s) {
  const int KP = stpm_kp(a.k);
  if (KP < 0) return cudaErrorInvalidValue;
  if (bf16 && (!a.yh1 || !a.yh2 || !a.yh3 || a.ldyh % 8 != 0)) return cudaErrorInvalidValue;
  if (!bf16 && a.ldy % 4 != 0) return cudaErrorInvalidValue;
  return bf16 ? launch_partial_p<true>(mode, KP, a, grid, s)
              : launch_partial_p<false>(mode, KP, a, grid, s);
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
    case 160: return launch_step_k<160>(a, s);
    case 208: return launch_step_k<208>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

int stpm_step_kp(int k) { return stpm_kp(k); }

size_t stpm_phi_image_bytes(int k) {
  const int kp = stpm_kp(k);
  if (kp < 32 || kp > 112) return 0;
  return (size_t)8 * kp * kp + (size_t)8 * kp;  // hi | lo (ContractTc<KP>::PSZ each), m1 | m2
}

cudaError_t stpm_partial_batched(int mode, int KP, const StpmPartialArgs* args, int graphs,
                                 int grid, bool bf16, cudaStream_t s) {
  if (KP > 128 || grid % kPartialCluster != 0 || graphs < 1 || graphs > 65535)
    return cudaErrorInvalidValue;
  switch (mode) {
    case kModePlain:
      return bf16 ? launch_partial_batched_m<kModePlain, true>(KP, args, graphs, grid, s)
                  : launch_partial_batched_m<kModePlain, false>(KP, args, graphs, grid, s);
    case kModeAdjoint:
      return bf16 ? launch_partial_batched_m<kModeAdjoint, true>(KP, args, graphs, grid, s)
                  : launch_partial_batched_m<kModeAdjoint, false>(KP, args, graphs, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t stpm_update_batched(int KP, const StpmUpdateArgs* args, int graphs, cudaStream_t s) {
  if (graphs < 1 || graphs > 65535) return cudaErrorInvalidValue;
  switch (KP) {
    case 32: return launch_step_batched_k<32>(args, graphs, s);
    case 48: return launch_step_batched_k<48>(args, graphs, s);
    case 64: return launch_step_batched_k<64>(args, graphs, s);
    case 80: return launch_step_batched_k<80>(args, graphs, s);
    case 96: return launch_step_batched_k<96>(args, graphs, s);
    case 112: return launch_step_batched_k<112>(args, graphs, s);
    case 128: return launch_step_batched_k<128>(args, graphs, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t stpm_batch_update(int k, float* phi, const float* G, double* lambda, double* err,
                              cudaStream_t s) {
  batch_update_kernel<<<1, 1024, 0, s>>>(k, phi, G, lambda, err);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t stpm_tensor_values(int k, float* phi, const float* G, double* lambda, cudaStream_t s,
                               double* phi64) {
  tensor_value_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, s>>>(k, phi, G, lambda, phi64);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
