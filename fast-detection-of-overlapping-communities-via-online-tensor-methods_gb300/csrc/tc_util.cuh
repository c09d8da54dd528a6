// Helpers for the 5th-generation tensor cores (tcgen05, sm_100-class):
// shared-memory matrix descriptors, the kind::tf32 instruction descriptor,
// MMA issue and commit, tensor-memory allocation and loads, bounded
// mbarrier waits.
//
// Operand layout used throughout: K-major, no swizzle.  A core matrix is 8
// rows x 16 bytes (4 TF32 elements along K), 128 contiguous bytes; the next
// core along K is at +128 B (leading byte offset), the next 8-row group at
// +SBO (stride byte offset) = (K / 4) * 128 B for a tile K elements deep.
// One MMA consumes K = 8, i.e. two cores along K: the descriptor of K-step
// ks starts at +256 * ks.
#pragma once
#include <cstdint>

namespace mmsb {
namespace tc {

__device__ __forceinline__ uint32_t sm_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) of a K-major tile whose 8-row groups are
// sbo bytes apart
__device__ __forceinline__ uint32_t kmajor_off(int r, int k, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 2) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 3) * 4u;
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

// instruction descriptor: kind::f16 with A and B in BF16 (format 1; both
// operands of one MMA must have the same 16-bit type), D in FP32, K-major
__host__ __device__ constexpr uint32_t bf16_idesc(int m, int n) {
  return (1u << 4)                      // D format: F32
         | (1u << 7)                    // A format: BF16
         | (1u << 10)                   // B format: BF16
         | ((uint32_t)(n >> 3) << 17)   // N / 8
         | ((uint32_t)(m >> 4) << 24);  // M / 16
}

// byte offset of element (r, k) of a K-major 16-bit tile (a core matrix is 8
// rows x 8 elements) whose 8-row groups are sbo bytes apart
__device__ __forceinline__ uint32_t kmajor16_off(int r, int k, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 3) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}

// D (+)= A B with BF16 operands (K = 16 per instruction), one elected thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D (+)= A B, one elected thread; accumulate = 0 overwrites D
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

// the MMAs issued so far by this thread arrive on the mbarrier when done
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   sm_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sm_addr(bar)), "r"(count)
               : "memory");
}

// clock64 cycles a bounded wait gives up after by default (about one second)
constexpr long long kWaitLimitDefault = 2000000000LL;
__device__ __forceinline__ long long wait_limit_or_default(long long v) {
  return v > 0 ? v : kWaitLimitDefault;
}

// waits for the phase with the given parity; false after `limit` clock64
// cycles (the caller then reports kFlagTimeout instead of hanging)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          long long limit = kWaitLimitDefault) {
  const uint32_t b = sm_addr(bar);
  const long long start = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(b), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - start > limit) return false;
  }
}

// warp-wide: allocate ncols (a power of two >= 32) tensor-memory columns,
// address written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   sm_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory stores -> visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// warp-wide: 8 consecutive columns of this warp's 32 lanes (lane = row)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 4; ++j) v[j] = __uint_as_float(r[j]);
}

// v = hi + lo: hi rounded to TF32, lo the FP32 remainder (a TF32 MMA reads
// the top 19 bits of lo)
__device__ __forceinline__ void split4(const float (&v)[4], uint4& hi, float4& lo) {
  uint32_t h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h[i]) : "f"(v[i]));
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_float4(v[0] - __uint_as_float(h[0]), v[1] - __uint_as_float(h[1]),
                   v[2] - __uint_as_float(h[2]), v[3] - __uint_as_float(h[3]));
}

}  // namespace tc
}  // namespace mmsb
