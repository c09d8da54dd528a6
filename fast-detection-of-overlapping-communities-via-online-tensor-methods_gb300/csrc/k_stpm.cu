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
  for (int e = tid; e < 3 * KP; e += 256) dsum[e] = 0.f;
  __syncthreads();
  // m_P = Phi^T mu_P
  for (int e = tid; e < 3 * KP; e += 256) {
    const int which = e / KP, i = e % KP;
    const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
    float s = 0.f;
    if (i < k && mu)
      for (int j = 0; j < k; ++j) s = fmaf(Phis[j * KP + i], mu[j], s);
    mv[e] = s;
  }
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
// leading dimension KP + 4) and owns NB = KP / CL of its columns.  Products
// X^T X[:, blk] and X B[:, blk] are formed locally; the new column block is
// written into every CTA's next buffer through distributed shared memory,
// followed by one cluster barrier per iteration.

// leading dimension: multiple of 4 (float4) with an odd float4 stride
__host__ __device__ constexpr int step_xld(int KP) { return ((KP / 4) % 2) ? KP + 8 : KP + 4; }

template <int KP, int CL>
struct StepSmem {
  static constexpr int NB = KP / CL;
  static constexpr size_t floats = (size_t)2 * KP * step_xld(KP) + (size_t)2 * NB * KP + 4 * KP + 6 * CL + 3 * NB + 8;
};

// Ab[jb * KP + i] = X[:, i] . X[:, c0 + jb]
template <int KP, int CL>
__device__ __forceinline__ void step_gram(const float* __restrict__ X, int c0, float* __restrict__ Ab) {
  constexpr int NB = KP / CL, XLD = step_xld(KP), IG = KP / 4;
  for (int t = threadIdx.x; t < IG * NB; t += blockDim.x) {
    // columns t, t+IG, t+2IG, t+3IG: neighbouring threads read neighbouring
    // columns, whose float4 addresses differ by XLD/4 (odd) -> no bank conflicts
    const int i0 = t % IG, jb = t / IG;
    const float* xj = X + (c0 + jb) * XLD;
    float4 acc[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int r = 0; r < KP; r += 4) {
      const float4 b = *reinterpret_cast<const float4*>(xj + r);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 a = *reinterpret_cast<const float4*>(X + (i0 + q * IG) * XLD + r);
        acc[q].x = fmaf(a.x, b.x, acc[q].x);
        acc[q].y = fmaf(a.y, b.y, acc[q].y);
        acc[q].z = fmaf(a.z, b.z, acc[q].z);
        acc[q].w = fmaf(a.w, b.w, acc[q].w);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      Ab[jb * KP + i0 + q * IG] = (acc[q].x + acc[q].y) + (acc[q].z + acc[q].w);
  }
}

// value(r, c0+jb) = beta_self X[r, c0+jb] + alpha (X B)[r, jb] + gamma Gb[jb*KP + r],
// zero outside k x k, written to every cluster rank's buffer
template <int KP, int CL>
__device__ __forceinline__ void step_times(const float* __restrict__ X, const float* __restrict__ B,
                                           int c0, float alpha, float beta_self,
                                           const float* __restrict__ Gb, float gamma, int k,
                                           float* const* dst) {
  constexpr int NB = KP / CL, XLD = step_xld(KP), RG = KP / 4;
  for (int t = threadIdx.x; t < RG * NB; t += blockDim.x) {
    const int r0 = 4 * (t % RG), jb = t / RG;
    const float* b = B + jb * KP;
    float4 acc2[2];
    acc2[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    acc2[1] = acc2[0];
#pragma unroll 2
    for (int i = 0; i < KP; i += 4) {
      const float4 bb = *reinterpret_cast<const float4*>(b + i);
      const float bv[4] = {bb.x, bb.y, bb.z, bb.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 x = *reinterpret_cast<const float4*>(X + (i + q) * XLD + r0);
        float4& ac = acc2[q & 1];
        ac.x = fmaf(x.x, bv[q], ac.x);
        ac.y = fmaf(x.y, bv[q], ac.y);
        ac.z = fmaf(x.z, bv[q], ac.z);
        ac.w = fmaf(x.w, bv[q], ac.w);
      }
    }
    const float4 acc = make_float4(acc2[0].x + acc2[1].x, acc2[0].y + acc2[1].y,
                                   acc2[0].z + acc2[1].z, acc2[0].w + acc2[1].w);
    const int col = c0 + jb;
    const float4 self = *reinterpret_cast<const float4*>(X + col * XLD + r0);
    float v[4] = {beta_self * self.x + alpha * acc.x, beta_self * self.y + alpha * acc.y,
                  beta_self * self.z + alpha * acc.z, beta_self * self.w + alpha * acc.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (Gb) v[q] += gamma * Gb[jb * KP + r0 + q];
      if (r0 + q >= k || col >= k) v[q] = 0.f;
    }
    const float4 out = make_float4(v[0], v[1], v[2], v[3]);
#pragma unroll
    for (int q = 0; q < CL; ++q) *reinterpret_cast<float4*>(dst[q] + col * XLD + r0) = out;
  }
}

template <int KP, int CL>
__global__ void __launch_bounds__(512) stpm_step_kernel(StpmUpdateArgs a) {
  constexpr int NB = KP / CL, XLD = step_xld(KP);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) float sm[];
  float* Xa = sm;
  float* Xb = Xa + KP * XLD;
  float* Ab = Xb + KP * XLD;
  float* Gb = Ab + NB * KP;
  float* mv = Gb + NB * KP;     // m1, m2, m3 (+ pad) for this block
  float* red = mv + 4 * KP;     // 3 x 2*CL statistics slots (initial, even, odd)
  __shared__ float s_abs, s_err;
  const int k = a.k;
  const int c0 = rank * NB;
  const int tid = threadIdx.x;
  for (int e = tid; e < KP * XLD; e += blockDim.x) {
    const int r = e % XLD, c = e / XLD;
    Xa[e] = (r < k && c < k) ? a.phi[(int64_t)c * k + r] : 0.f;
    Xb[e] = 0.f;
  }
  float* dstA[CL];
  float* dstB[CL];
#pragma unroll
  for (int q = 0; q < CL; ++q) {
    dstA[q] = cluster.map_shared_rank(Xa, q);
    dstB[q] = cluster.map_shared_rank(Xb, q);
  }
  __syncthreads();
  cluster.sync();  // every CTA has read Phi before anyone writes it back

  float* X = Xa;
  float* const* dn = dstB;
  float* const* dc = dstA;
  auto swap_buffers = [&]() {
    X = (X == Xa) ? Xb : Xa;
    float* const* td = dc;
    dc = dn;
    dn = td;
  };
  if (a.step_mode == kStepOnline) {
    // G block (columns c0 .. c0+NB) from the per-CTA partials, plus the mean terms
    for (int e = tid; e < 3 * NB; e += blockDim.x) {
      const int which = e / NB, jb = e % NB, i = c0 + jb;
      const float* mu = which == 0 ? a.mu1 : which == 1 ? a.mu2 : a.mu3;
      float sv = 0.f;
      if (i < k && mu)
        for (int j = 0; j < k; ++j) sv = fmaf(X[i * XLD + j], mu[j], sv);
      mv[which * KP + jb] = sv;
    }
    __syncthreads();
    // per-column sums of the d partials (3 x NB), then the contraction block
    float* dcol = red + 6 * CL;  // 3 * NB floats
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
      float g = 0.f;
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
        g = gv;
      }
      Gb[e] = g;
    }
    // Phi' = Phi - beta (3 theta Phi (Phi^T Phi)^.2 - gscale G)   (Util.cpp:259-272)
    step_gram<KP, CL>(X, c0, Ab);
    __syncthreads();
    for (int e = tid; e < KP * NB; e += blockDim.x) Ab[e] = Ab[e] * Ab[e];
    __syncthreads();
    step_times<KP, CL>(X, Ab, c0, -a.beta * a.theta3, 1.f, Gb, a.beta * a.gscale, k, dn);
    cluster.sync();
    swap_buffers();
  }
  // Newton-Schulz polar iteration X <- X (3 I - X^T X) / 2.  With
  // X^T X = I + E the next error is -3/4 E^2 + E^3/4, so once |E| < 1e-3 one
  // more iteration reaches the FP32 floor; the loop stops there.
  // One cluster barrier per iteration: the statistics of A_t = X_t^T X_t
  // travel with the broadcast of X_{t+1}; if they show X_t had already
  // converged, X_{t+1} is discarded.
  auto block_stats = [&]() {
    if (tid == 0) {
      s_abs = 0.f;
      s_err = 0.f;
    }
    __syncthreads();
    for (int jb = tid / 32; jb < NB; jb += blockDim.x / 32) {
      const int col = c0 + jb;
      float cs = 0.f, er = 0.f;
      for (int i = tid % 32; i < KP; i += 32) {
        const float v = Ab[jb * KP + i];
        if (i < k && col < k) {
          cs += fabsf(v);
          er = fmaxf(er, fabsf(v - (i == col ? 1.f : 0.f)));
        }
      }
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        cs += __shfl_xor_sync(0xffffffffu, cs, off);
        er = fmaxf(er, __shfl_xor_sync(0xffffffffu, er, off));
      }
      if ((tid & 31) == 0) {
        atomicMax(reinterpret_cast<int*>(&s_abs), __float_as_int(cs));
        atomicMax(reinterpret_cast<int*>(&s_err), __float_as_int(er));
      }
    }
    __syncthreads();
  };
  auto cluster_stats = [&](float& gabs, float& gerr) {
    gabs = 0.f;
    gerr = 0.f;
    for (int q = 0; q < CL; ++q) {
      gabs = fmaxf(gabs, red[q]);
      gerr = fmaxf(gerr, red[CL + q]);
    }
  };
  // initial scaling: sigma_max^2 <= ||X^T X||_1
  step_gram<KP, CL>(X, c0, Ab);
  block_stats();
  if (tid < CL) {
    float* r = cluster.map_shared_rank(red, tid);
    r[rank] = s_abs;
    r[CL + rank] = s_err;
  }
  cluster.sync();
  int it = 0;
  bool done = false, last = false;
  {
    float gabs, gerr;
    cluster_stats(gabs, gerr);
    if (!(gerr == gerr) || !(gabs == gabs)) {
      if (tid == 0 && rank == 0) atomicOr(a.flags, kFlagNonFinite);
      done = true;
    } else if (gerr < a.ns_tol) {
      done = true;
    } else if (gabs > 0.f) {
      const float sc = rsqrtf(gabs);
      for (int e = tid; e < KP * NB; e += blockDim.x) Ab[e] *= sc * sc;
      for (int e = tid; e < KP * XLD; e += blockDim.x) X[e] *= sc;
      __syncthreads();
    }
  }
  cluster.sync();  // every CTA has read the statistics slots
  for (; !done && it < a.max_ns; ++it) {
    if (it > 0) {
      step_gram<KP, CL>(X, c0, Ab);
      block_stats();
    } else {
      // A_0 of the scaled X is already in Ab; its error decides below
      block_stats();
    }
    // speculative next iterate from A_t, broadcast together with A_t's statistics
    for (int e = tid; e < KP * NB; e += blockDim.x) {
      const int i = e % KP, jb = e / KP;
      Ab[e] = ((i == c0 + jb) ? 1.5f : 0.f) - 0.5f * Ab[e];
    }
    __syncthreads();
    step_times<KP, CL>(X, Ab, c0, 1.f, 0.f, nullptr, 0.f, k, dn);
    if (tid < CL) {
      float* r = cluster.map_shared_rank(red, tid) + 2 * CL * (1 + (it & 1));
      r[rank] = s_abs;
      r[CL + rank] = s_err;
    }
    cluster.sync();
    float gabs = 0.f, gerr = 0.f;
    for (int q = 0; q < CL; ++q) {
      const float* rr = red + 2 * CL * (1 + (it & 1));
      gabs = fmaxf(gabs, rr[q]);
      gerr = fmaxf(gerr, rr[CL + q]);
    }
    if (!(gerr == gerr) || !(gabs == gabs)) {
      if (tid == 0 && rank == 0) atomicOr(a.flags, kFlagNonFinite);
      done = true;
      break;
    }
    if (gerr < a.ns_tol) {  // X_t was converged: keep it, drop X_{t+1}
      done = true;
      break;
    }
    swap_buffers();
    if (last) {
      done = true;
      ++it;
      break;
    }
    if (gerr < 1e-3f) last = true;
  }
  if (!done && rank == 0 && tid == 0) atomicOr(a.flags, kFlagNoConvergence);
  if (rank == 0 && tid == 0 && a.ns_iters) atomicAdd(a.ns_iters, it);
  for (int e = tid; e < KP * NB; e += blockDim.x) {
    const int r = e % KP, col = c0 + e / KP;
    if (r < k && col < k) a.phi[(int64_t)col * k + r] = X[col * XLD + r];
  }
  cluster.sync();  // keep shared memory alive until remote writers are done
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
  static int use16 = -1;  // 16-CTA clusters where the device allows them
  if (use16 != 0) {
    cudaError_t e = launch_step_t<KP, 16>(a, s);
    if (e == cudaSuccess) {
      use16 = 1;
      return e;
    }
    if (use16 == 1) return e;
    cudaGetLastError();
    use16 = 0;
  }
  return launch_step_t<KP, 8>(a, s);
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
