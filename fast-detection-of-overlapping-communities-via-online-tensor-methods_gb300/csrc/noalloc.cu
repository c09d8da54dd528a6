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
// on a device looks the array's device address up once (see below); make that
// first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "mmsb.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Device address of the scratch array for the current device.  The first
// call on a device looks the symbol up (this may load the module); later
// calls reuse the cached address.
cudaError_t scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" mmsb_status mmsb_op_spmm_t_noalloc(const int64_t* d_row_ptr, const int32_t* d_col_idx,
                                              const float* d_val, int64_t n_rows, int64_t n_cols,
                                              int64_t nnz, const float* d_P, int64_t p, float alpha,
                                              float* d_Y, void* stream) {
  if (!d_row_ptr || (nnz > 0 && !d_col_idx) || !d_P || !d_Y || n_rows < 0 || n_cols < 0 ||
      nnz < 0 || p < 4 || p % 4 != 0 || n_cols > INT32_MAX || n_rows > INT32_MAX)
    return MMSB_ERR_INVALID_ARG;
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
  cudaError_t e = scratch_for_current_device(&base);
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
