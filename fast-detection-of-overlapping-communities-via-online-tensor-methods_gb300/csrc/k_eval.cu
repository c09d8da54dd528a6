// Ground-truth evaluation: correlation, t statistic and p-value of every
// (estimated community, true community) pair of membership rows, the
// hypothesis test of the reference's Pvalue.cpp (Calculate_Correlation,
// Calculate_Tstat, Calculate_Pvalue, Pvalue.cpp:85-235) for all pairs at once.
//
//   column statistics (FP64):  mean and population variance of every
//                              membership row over the N nodes
//   centred copies (FP32):     a - mean, so the cross products carry no
//                              E[ab] - E[a]E[b] cancellation
//   cross products:            C = A_c^T B_c (k x K) by the Gram kernel
//                              (FP32 within 256-row chunks, FP64 across)
//   pairs (FP64):              r = C / (N sa sb), t = r sqrt((N-2)/(1-r^2)),
//                              p by the incomplete beta function
//
// The incomplete beta follows the published Numerical Recipes method the
// reference uses (continued fraction by the modified Lentz method, stop at
// |del - 1| <= 3e-7; Lanczos log-gamma with NR's six coefficients), with the
// reference's branch order for the p-value.
#include "common.cuh"

namespace mmsb {
namespace {

// per column j of a node-major n x m panel (ld): partial sum and sum of
// squares over row chunk blockIdx.y, written to part[(y * m + j) * 2 + 0/1]
__global__ void __launch_bounds__(256) colstats_partial_kernel(const float* __restrict__ X, int ld,
                                                               int m, int64_t n, int64_t rows,
                                                               double* __restrict__ part) {
  __shared__ double s1[8][33], s2[8][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  const int64_t r0 = (int64_t)blockIdx.y * rows, r1 = min(n, r0 + rows);
  double a = 0.0, b = 0.0;
  if (j < m)
    for (int64_t r = r0 + w; r < r1; r += 8) {
      const double v = X[r * ld + j];
      a += v;
      b = fma(v, v, b);
    }
  s1[w][lane] = a;
  s2[w][lane] = b;
  __syncthreads();
  if (w == 0 && j < m) {
    double x = 0.0, y = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      x += s1[q][lane];
      y += s2[q][lane];
    }
    part[((int64_t)blockIdx.y * m + j) * 2 + 0] = x;
    part[((int64_t)blockIdx.y * m + j) * 2 + 1] = y;
  }
}

// mean and centred second moment (population variance) per column, the
// splits summed in order
__global__ void colstats_final_kernel(const double* __restrict__ part, int m, int splits, int64_t n,
                                      double* __restrict__ mean, double* __restrict__ var) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  double a = 0.0, b = 0.0;
  for (int q = 0; q < splits; ++q) {
    a += part[((int64_t)q * m + j) * 2 + 0];
    b += part[((int64_t)q * m + j) * 2 + 1];
  }
  const double mu = a / (double)n;
  mean[j] = mu;
  var[j] = fmax(0.0, b / (double)n - mu * mu);
}

__global__ void center_kernel(const float* __restrict__ X, int ld, int m, int64_t n,
                              const double* __restrict__ mean, float* __restrict__ Y) {
  const int64_t total = n * (int64_t)m;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / m;
    const int j = (int)(e % m);
    Y[e] = (float)((double)X[r * ld + j] - mean[j]);
  }
}

__device__ double nr_gammln(double xx) {
  const double cof[6] = {76.18009173, -86.50532033, 24.01409822, -1.231739516, 0.120858003e-2,
                         -0.536382e-5};
  double x = xx - 1.0;
  double tmp = x + 5.5;
  tmp -= (x + 0.5) * log(tmp);
  double ser = 1.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    x += 1.0;
    ser += cof[j] / x;
  }
  return -tmp + log(2.50662827465 * ser);
}

// continued fraction, modified Lentz; *ok = false if it did not converge in
// max_it rounds
__device__ double nr_betacf(double a, double b, double x, int max_it, bool* ok) {
  const double fpmin = 1e-30, eps = 3e-7;
  const double qab = a + b, qap = a + 1.0, qam = a - 1.0;
  double c = 1.0, d = 1.0 - qab * x / qap;
  if (fabs(d) < fpmin) d = fpmin;
  d = 1.0 / d;
  double h = d;
  for (int m = 1; m <= max_it; ++m) {
    const double m2 = 2.0 * m;
    double aa = m * (b - m) * x / ((qam + m2) * (a + m2));
    d = 1.0 + aa * d;
    if (fabs(d) < fpmin) d = fpmin;
    c = 1.0 + aa / c;
    if (fabs(c) < fpmin) c = fpmin;
    d = 1.0 / d;
    h *= d * c;
    aa = -(a + m) * (qab + m) * x / ((a + m2) * (qap + m2));
    d = 1.0 + aa * d;
    if (fabs(d) < fpmin) d = fpmin;
    c = 1.0 + aa / c;
    if (fabs(c) < fpmin) c = fpmin;
    d = 1.0 / d;
    const double del = d * c;
    h *= del;
    if (fabs(del - 1.0) <= eps) return h;
  }
  *ok = false;
  return h;
}

__device__ double nr_betainc(double a, double b, double x, bool* ok) {
  double bt = 0.0;
  if (!(x == 0.0 || x == 1.0))
    bt = exp(nr_gammln(a + b) - nr_gammln(a) - nr_gammln(b) + a * log(x) + b * log(1.0 - x));
  if (x < (a + 1.0) / (a + b + 2.0)) return bt * nr_betacf(a, b, x, 100000, ok) / a;
  return 1.0 - bt * nr_betacf(b, a, 1.0 - x, 100000, ok) / b;
}

// one thread per pair (i, j): outputs column-major k x K (entry i + j k)
__global__ void pvalue_kernel(const double* __restrict__ C, int k, int K, int64_t n,
                              const double* __restrict__ va, const double* __restrict__ vb,
                              double* __restrict__ corr, double* __restrict__ tstat,
                              double* __restrict__ pval, unsigned* flags) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)k * K) return;
  const int i = (int)(e % k), j = (int)(e / k);
  const double cov = C[(int64_t)j * k + i] / (double)n;
  const double r = cov / (sqrt(va[i]) * sqrt(vb[j]));
  const double t_raw = r * sqrt((double)(n - 2) / (1.0 - r * r));
  const double t = -fabs(t_raw);
  const double dof = (double)(n - 2);
  double p = 0.5;
  const bool nans = isnan(t) || dof <= 0.0;
  if (dof != 1.0 && dof <= 1e7 && !nans) {
    bool ok = true;
    p = 0.5 * nr_betainc(0.5 * dof, 0.5, dof / (dof + t * t), &ok);
    if (t > 0) p = 1.0 - p;
    if (!ok) atomicOr(flags, kFlagNoConvergence);
  }
  corr[e] = r;
  tstat[e] = t_raw;
  pval[e] = 2.0 * p;
}

constexpr int64_t kStatRows = 8192;

}  // namespace

size_t colstats_partials(int64_t n, int m) {
  return (size_t)2 * (size_t)m * (size_t)std::max<int64_t>(1, ceil_div(n, kStatRows));
}

cudaError_t column_stats(const float* X, int ld, int m, int64_t n, double* part, double* mean,
                         double* var, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaErrorInvalidValue;
  const int splits = (int)std::max<int64_t>(1, ceil_div(n, kStatRows));
  colstats_partial_kernel<<<dim3((unsigned)ceil_div(m, 32), (unsigned)splits), 256, 0, s>>>(
      X, ld, m, n, kStatRows, part);
  colstats_final_kernel<<<(unsigned)ceil_div(m, 256), 256, 0, s>>>(part, m, splits, n, mean, var);
  g_launch_count += 2;
  return cudaGetLastError();
}

cudaError_t center_columns(const float* X, int ld, int m, int64_t n, const double* mean, float* Y,
                           cudaStream_t s) {
  const int64_t total = n * (int64_t)m;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(8 * kNumSMs, ceil_div(total, 256)));
  center_kernel<<<grid, 256, 0, s>>>(X, ld, m, n, mean, Y);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t pair_pvalues(const double* C, int k, int K, int64_t n, const double* va,
                         const double* vb, double* corr, double* tstat, double* pval,
                         unsigned* flags, cudaStream_t s) {
  const int64_t pairs = (int64_t)k * K;
  if (pairs == 0) return cudaSuccess;
  pvalue_kernel<<<(unsigned)ceil_div(pairs, 128), 128, 0, s>>>(C, k, K, n, va, vb, corr, tstat,
                                                               pval, flags);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
