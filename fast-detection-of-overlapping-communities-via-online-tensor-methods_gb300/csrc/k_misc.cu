// Small element-wise kernels on k- and p-sized data of the whitening and
// post-processing chains (pinv thresholds, scaling, guards, conversions).
#include "common.cuh"

#include <cuda_bf16.h>

#include "tc_util.cuh"

#include <algorithm>

namespace mmsb {

namespace {

__global__ void sig_from_evals_kernel(int k, const double* __restrict__ ev, double* __restrict__ sig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) sig[i] = sqrt(fmax(ev[i], 0.0));
}

// F[:, j] *= pinv(sig_j)  (pinv_vector, CPU/Spectral.cpp:50-57)
__global__ void scale_cols_pinv_kernel(int rows, int k, double* __restrict__ F, int ldf,
                                       const double* __restrict__ sig, double tol) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * k) return;
  const int r = e % rows, j = e / rows;
  const double s = sig[j];
  F[(int64_t)j * ldf + r] *= fabs(s) > tol ? 1.0 / s : 0.0;
}

// a = sqrt(pinv(sig)) (Spectral.cpp:235-236), b = pinv(sqrt(sig)) (Spectral.cpp:307, Util.cpp:118)
__global__ void sqrt_pinv_kernel(int k, const double* __restrict__ sig, double tol,
                                 double* __restrict__ a, double* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  const double s = sig[i];
  if (a) a[i] = fabs(s) > tol ? sqrt(1.0 / s) : 0.0;
  if (b) {
    const double r = sqrt(s);
    b[i] = fabs(r) > tol ? 1.0 / r : 0.0;
  }
}

// term_k_k.nonZeros() < KHID -> diagonal set to one (CPU/Util.cpp:91-94)
__global__ void diag_guard_kernel(int k, double* __restrict__ core) {
  __shared__ int nnz;
  if (threadIdx.x == 0) nnz = 0;
  __syncthreads();
  int local = 0;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) local += core[e] != 0.0;
  atomicAdd(&nnz, local);
  __syncthreads();
  if (nnz < k)
    for (int i = threadIdx.x; i < k; i += blockDim.x) core[(int64_t)i * k + i] = 1.0;
}

__global__ void panel_rank1_kernel(float* __restrict__ P, int ld, int64_t n, int q, double alpha,
                                   const double* __restrict__ u, const double* __restrict__ v) {
  const int64_t total = n * q;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / q;
    const int j = (int)(e % q);
    P[r * ld + j] = (float)((double)P[r * ld + j] + alpha * u[r] * v[j]);
  }
}

__global__ void f64_to_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    b[e] = (float)a[e];
}

__global__ void f32_to_f64_kernel(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    b[e] = (double)a[e];
}

// dst[r, c] = bf16(src[r, c]) for c < cols, 0 for cols <= c < ldh
__global__ void panel_to_bf16_kernel(const float* __restrict__ src, int64_t ld, int64_t rows,
                                     int cols, __nv_bfloat16* __restrict__ dst, int64_t ldh) {
  const int64_t n = rows * ldh;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ldh;
    const int c = (int)(e % ldh);
    dst[e] = __float2bfloat16_rn(c < cols ? src[r * ld + c] : 0.f);
  }
}

// F[:, i] = phi[:, i] * pinv(lambda_i)   (CommunityDetection.cpp:98-99)
__global__ void phi_scaled_kernel(int k, const float* __restrict__ phi,
                                  const double* __restrict__ lambda, double tol,
                                  double* __restrict__ F) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= k * k) return;
  const int i = e / k;
  const double l = lambda[i];
  F[e] = (double)phi[e] * (fabs(l) > tol ? 1.0 / l : 0.0);
}

__global__ void transpose_f64_kernel(int p, const double* __restrict__ A, double* __restrict__ At) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p * p) return;
  const int r = e % p, c = e / p;
  At[(int64_t)r * p + c] = A[e];
}

// out = a * sum_ij (S_ij)^3  (loss orthogonality term, S = Phi^T Phi)
__global__ void cube_sum_kernel(int n, const double* __restrict__ S, double a,
                                double* __restrict__ out) {
  __shared__ double red[32];
  double v = 0.0;
  for (int e = threadIdx.x; e < n; e += blockDim.x) v += S[e] * S[e] * S[e];
#pragma unroll
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    out[0] = a * s;
  }
}

__global__ void hadamard_square_kernel(int64_t n, const double* __restrict__ a,
                                       double* __restrict__ b) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    b[e] = a[e] * a[e];
}


// F[:, j] = 0 where sig_j <= tol (pinv_vector semantics, CPU/Spectral.cpp:50-57)
__global__ void mask_cols_kernel(int rows, int k, double* __restrict__ F, int ldf,
                                 const double* __restrict__ sig, double tol) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * k) return;
  const int r = e % rows, j = e / rows;
  if (!(fabs(sig[j]) > tol)) F[(int64_t)j * ldf + r] = 0.0;
}

// B[row, j] = alpha * v[j]
__global__ void set_row_scaled_kernel(int cols, double* __restrict__ B, int ldb, int row,
                                      double alpha, const double* __restrict__ v) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < cols) B[(int64_t)j * ldb + row] = alpha * v[j];
}

// Q = MGS of an upper-triangular R with non-negative diagonal: e_j, or 0 where R_jj == 0
__global__ void eye_mask_kernel(int m, int p, const double* __restrict__ R, int ldr,
                                double* __restrict__ Q, int ldq) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * p) return;
  const int i = e % m, j = e / m;
  Q[(int64_t)j * ldq + i] = (i == j && j < m && R[(int64_t)j * ldr + j] != 0.0) ? 1.0 : 0.0;
}

unsigned blocks(int64_t n, int T = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(8 * kNumSMs, ceil_div(n, T)));
}

// ||Phi - snap||_F (FP64) into *out, then snap = Phi (one CTA): the
// convergence trace of the online methods, one value per sweep
// conv[i] = sqrt(sum_q parts[i * stride + q]), q < used (fixed order)
__global__ void conv_sum_kernel(const double* __restrict__ parts, int count, int stride, int used,
                                double* __restrict__ conv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  double t = 0.0;
  for (int q = 0; q < used; ++q) t += parts[(int64_t)i * stride + q];
  conv[i] = sqrt(t);
}

}  // namespace

cudaError_t conv_sum(const double* parts, int count, int stride, int used, double* conv,
                     cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  conv_sum_kernel<<<(unsigned)ceil_div((int64_t)count, 128), 128, 0, s>>>(parts, count, stride, used, conv);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t sig_from_evals(int k, const double* ev, double* sig, cudaStream_t s) {
  sig_from_evals_kernel<<<blocks(k), 256, 0, s>>>(k, ev, sig);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t scale_cols_pinv(int rows, int k, double* F, int ldf, const double* sig, double tol,
                            cudaStream_t s) {
  scale_cols_pinv_kernel<<<(unsigned)ceil_div((int64_t)rows * k, 256), 256, 0, s>>>(rows, k, F, ldf, sig, tol);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t sqrt_pinv(int k, const double* sig, double tol, double* a, double* b, cudaStream_t s) {
  sqrt_pinv_kernel<<<blocks(k), 256, 0, s>>>(k, sig, tol, a, b);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t diag_guard(int k, double* core, cudaStream_t s) {
  diag_guard_kernel<<<1, 256, 0, s>>>(k, core);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t panel_rank1(float* P, int ld, int64_t n, int q, double alpha, const double* u,
                        const double* v, cudaStream_t s) {
  panel_rank1_kernel<<<blocks(n * q), 256, 0, s>>>(P, ld, n, q, alpha, u, v);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t f64_to_f32(const double* a, float* b, int64_t n, cudaStream_t s) {
  f64_to_f32_kernel<<<blocks(n), 256, 0, s>>>(a, b, n);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t panel_to_bf16(const float* src, int64_t ld, int64_t rows, int cols, void* dst,
                          int64_t ldh, cudaStream_t s) {
  panel_to_bf16_kernel<<<blocks(rows * ldh), 256, 0, s>>>(src, ld, rows, cols,
                                                          static_cast<__nv_bfloat16*>(dst), ldh);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t f32_to_f64(const float* a, double* b, int64_t n, cudaStream_t s) {
  f32_to_f64_kernel<<<blocks(n), 256, 0, s>>>(a, b, n);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t phi_scaled(int k, const float* phi, const double* lambda, double tol, double* F,
                       cudaStream_t s) {
  phi_scaled_kernel<<<(unsigned)ceil_div((int64_t)k * k, 256), 256, 0, s>>>(k, phi, lambda, tol, F);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t transpose_f64(int p, const double* A, double* At, cudaStream_t s) {
  transpose_f64_kernel<<<(unsigned)ceil_div((int64_t)p * p, 256), 256, 0, s>>>(p, A, At);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t cube_sum(int n, const double* S, double a, double* out, cudaStream_t s) {
  cube_sum_kernel<<<1, 1024, 0, s>>>(n, S, a, out);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t hadamard_square(int64_t n, const double* a, double* b, cudaStream_t s) {
  hadamard_square_kernel<<<blocks(n), 256, 0, s>>>(n, a, b);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t mask_cols(int rows, int k, double* F, int ldf, const double* sig, double tol,
                      cudaStream_t s) {
  mask_cols_kernel<<<(unsigned)ceil_div((int64_t)rows * k, 256), 256, 0, s>>>(rows, k, F, ldf, sig, tol);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t set_row_scaled(int rows, int cols, double* B, int ldb, int row, double alpha,
                           const double* v, cudaStream_t s) {
  (void)rows;
  set_row_scaled_kernel<<<(unsigned)ceil_div(cols, 256), 256, 0, s>>>(cols, B, ldb, row, alpha, v);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t eye_mask(int m, int p, const double* R, int ldr, double* Q, int ldq, cudaStream_t s) {
  eye_mask_kernel<<<(unsigned)ceil_div((int64_t)m * p, 256), 256, 0, s>>>(m, p, R, ldr, Q, ldq);
  ++g_launch_count;
  return cudaGetLastError();
}

// One CTA waits, through the bounded mbarrier wait of the tensor-core
// kernels (tc::mbar_wait), on a barrier that nothing ever arrives at; the
// wait gives up after `limit` clock64 cycles and reports kFlagTimeout, the
// same path a stalled wait of a real kernel takes.  No copy or MMA is in
// flight, so the kernel leaves cleanly.
__global__ void wait_probe_kernel(unsigned* __restrict__ flags, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(&bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  bool ok = true;
  if (threadIdx.x == 0) ok = tc::mbar_wait(&bar, 0u, limit);
  if (!ok) atomicOr(flags, kFlagTimeout);
}

cudaError_t wait_probe(unsigned* flags, long long limit, cudaStream_t s) {
  wait_probe_kernel<<<1, 32, 0, s>>>(flags, limit);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace mmsb
