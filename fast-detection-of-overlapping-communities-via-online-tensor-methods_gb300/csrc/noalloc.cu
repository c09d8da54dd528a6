// Transposed CSR SpMM for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc: code running inside another
// framework's memory pool (which owns every device allocation and would be
// bypassed or fragmented by a raw cudaMalloc), or latency-critical code that
// must not wait on cudaMalloc, which can synchronize the device.  Such a
// caller already owns its input and output device buffers; the only extra
// memory this operation needs -- the transposed copy of the CSR block -- lives
// here in a fixed, file-scope device array instead.
//
// The array (kNoAllocScratchBytes, 8 MiB) stays resident on every GPU
// that loads this library until the process exits.  All calls share it: two
// calls that overlap on the GPU (different streams, or different host threads)
// race on it and must be serialised by the caller.  Each call clears the part
// that must start at zero (the per-column counters) itself.  The first call
// in a CUDA context looks the array's device address up (see below); make that
// first call before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "mmsb.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Device address of the scratch array in the current context.  The address
// is looked up once per context and cached under the context's unique ID
// (cuCtxGetId, reached through the runtime's driver entry point, so no link
// to the driver library is needed): a device reset or a framework that
// destroys and recreates the primary context gets a new ID and so a fresh
// lookup instead of a stale pointer.
cudaError_t scratch_for_current_context(void** out) {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static std::mutex mu;
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static unsigned long long cached_id = ~0ull;
  static void* cached_addr = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  cudaError_t e = cudaFree(nullptr);  // makes the device's primary context current (no allocation)
  if (e != cudaSuccess) return e;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess || q2 != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
    get_current = reinterpret_cast<GetCurrent>(f1);
    get_id = reinterpret_cast<GetId>(f2);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return cudaErrorContextIsDestroyed;
  if (id != cached_id || !cached_addr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    cached_addr = p;
    cached_id = id;
  }
  *out = cached_addr;
  return cudaSuccess;
}

}  // namespace

extern "C" mmsb_status mmsb_op_spmm_t_noalloc(const int64_t* d_row_ptr, const int32_t* d_col_idx,
                                              const float* d_val, int64_t n_rows, int64_t n_cols,
                                              int64_t nnz, const float* d_P, int64_t p, float alpha,
                                              float* d_Y, void* stream) {
  if (!d_row_ptr || (nnz > 0 && !d_col_idx) || !d_P || !d_Y || n_rows < 0 || n_cols < 0 ||
      nnz < 0 || p < 4 || p % 4 != 0 || n_cols > INT32_MAX || n_rows > INT32_MAX ||
      (n_rows == 0 && nnz > 0))
    return MMSB_ERR_INVALID_ARG;
  // the panels are read and written as 16-byte vectors
  if (((uintptr_t)d_P | (uintptr_t)d_Y) & 15u) return MMSB_ERR_INVALID_ARG;
  // sizes beyond the array are refused before any product that could wrap
  if ((size_t)nnz > kNoAllocScratchBytes / 8 || (size_t)n_cols > kNoAllocScratchBytes / 16)
    return MMSB_ERR_UNSUPPORTED;
  // scratch layout: column counters (u64, n_cols+1) | transposed row offsets
  // (i64, n_cols+1) | staging columns (i32, nnz) [+ staging values (f32, nnz)]
  // | transposed columns (i32, nnz) [+ transposed values (f32, nnz)]
  const size_t vbytes = d_val ? 4 : 0;
  const size_t counters = align256(sizeof(uint64_t) * (size_t)(n_cols + 1));
  const size_t staging = align256((4 + vbytes) * (size_t)nnz + 8);
  const size_t rpT = align256(sizeof(int64_t) * (size_t)(n_cols + 1));
  const size_t ciT = align256(4 * (size_t)nnz + 4);
  const size_t valT = d_val ? align256(4 * (size_t)nnz + 4) : 0;
  const size_t need = counters + staging + rpT + ciT + valT;
  if (need > kNoAllocScratchBytes) return MMSB_ERR_UNSUPPORTED;  // block too large for the array
  void* base = nullptr;
  cudaError_t e = scratch_for_current_context(&base);
  if (e != cudaSuccess) return MMSB_ERR_CUDA;
  unsigned char* s = static_cast<unsigned char*>(base);
  int32_t* work = reinterpret_cast<int32_t*>(s);  // counters, then staging (csr_transpose layout)
  int64_t* rp_t = reinterpret_cast<int64_t*>(s + counters + staging);
  int32_t* ci_t = reinterpret_cast<int32_t*>(s + counters + staging + rpT);
  float* val_t = d_val ? reinterpret_cast<float*>(s + counters + staging + rpT + ciT) : nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  e = mmsb::csr_transpose(d_row_ptr, d_col_idx, d_val, n_rows, n_cols, nnz, rp_t, ci_t, val_t,
                          work, st);
  if (e == cudaSuccess)
    e = mmsb::spmm_f32(rp_t, ci_t, val_t, n_cols, d_P, (int)p, alpha, d_Y, st);
  return e == cudaSuccess ? MMSB_OK : MMSB_ERR_CUDA;
}
