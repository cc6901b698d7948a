// f3d_tc.cuh -- fifth-generation tensor core (tcgen05) building blocks for
// the DFT-matmul form: tensor memory allocation, shared-memory matrix
// descriptors, the f16 MMA with fp32 accumulation, mbarrier waits with a time
// limit, tensor-memory loads and bulk shared->global copies. Inline PTX only
// (sm_100 family, compiled for sm_103a).
//
// Operand layouts (K-major, 16-bit elements):
//  - INTERLEAVE (no swizzle): 8x8 "core matrices" of 128 contiguous bytes
//    (row r of the core matrix at r*16 bytes). The core matrix holding
//    (row, k) starts at (row/8)*SBO + (k/8)*LBO; here LBO = 128 (K-adjacent
//    core matrices are contiguous) and SBO = (K/8)*128.
//  - SWIZZLE_128B: rows of 64 elements (128 bytes); 8-row atoms of 1024 bytes,
//    the 16-byte chunk c of row r stored at chunk position c ^ (r % 8). Atoms
//    are SBO = 1024 bytes apart and the tile base is 1024-byte aligned.
// Each MMA instruction consumes K = 16 elements: the descriptor start
// advances by 2*LBO per step for INTERLEAVE and by 32 bytes inside the
// 128-byte row for SWIZZLE_128B.
#pragma once

#include <cuda_fp16.h>
#include <cstdint>

namespace f3d {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- tensor memory -------------------------------------------------------
// Allocation and release are warp-wide (.sync.aligned): call from one full warp.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Ordering of tensor-core operations around thread barriers.
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the
// async proxy (tensor core operand reads, bulk copies).
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive 32-bit columns of this thread's tensor-memory lane (the warp
// reads lanes 32*(warp%4) .. +31), waited for inside the same statement so
// that no use of the registers can be scheduled before the data arrives.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive 32-bit columns of this thread's tensor-memory lane, as
// tmem_ld32.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
// M (16 or 32) consecutive columns.
template <int M>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[M]) {
  static_assert(M == 16 || M == 32, "tensor-memory load width");
  if constexpr (M == 32) tmem_ld32(taddr, v);
  else tmem_ld16(taddr, v);
}

// ---- MMA -----------------------------------------------------------------
enum : uint32_t { LAYOUT_INTERLEAVE = 0, LAYOUT_SW128 = 2 };

// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (16-byte units, 14 bits each), the fixed version field 0b001 at bit 46,
// base offset 0 (atoms 1024-byte aligned) and the layout at bits 61-63.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (static_cast<uint64_t>(layout) << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulator (bits 4-5 = 1), A and
// B fp16 (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N/8 at bits
// 17-22 and M/16 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by a single thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// Arrives on the mbarrier once every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---- mbarrier ----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase with this parity to complete; gives up after
// `limit_ns` nanoseconds and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const uint32_t a = smem_u32(bar);
  uint64_t t0 = 0;
  for (uint32_t i = 0;; i++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i == 0) t0 = global_ns();
    else if ((i & 63) == 0 && global_ns() - t0 > limit_ns) return false;
  }
}

// Arrival that also announces `bytes` of bulk-copy data for the phase.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// ---- bulk copies -------------------------------------------------------------
// Global -> shared, completing on the mbarrier; 16-byte aligned, size a
// multiple of 16.
__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(sdst)),
               "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Shared -> global, 16-byte aligned addresses, size a multiple of 16.
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(ssrc)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Waits until the committed bulk stores have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Waits until the committed bulk stores are complete.
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Starts pulling `bytes` (a multiple of 16, 16-byte aligned) into L2.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// ---- operand packing ---------------------------------------------------------
// (a, b) -> fp16 pairs hi + lo with hi = fp16(x), lo = fp16(x - hi): the pair
// carries about 22 significant bits.
__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 hf = __half22float2(h);
#if __CUDA_ARCH__ >= 1000
  // Both residuals in one packed op: hf * -1 + (a, b), rounded once per lane
  // like the scalar subtraction.
  const float2 r = __ffma2_rn(hf, make_float2(-1.0f, -1.0f), make_float2(a, b));
  const __half2 l = __floats2half2_rn(r.x, r.y);
#else
  const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
#endif
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Byte offset of element (row, k) in an INTERLEAVE K-major tile with K columns.
__host__ __device__ constexpr uint32_t off_il(int row, int k, int K) {
  return static_cast<uint32_t>((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
// Byte offset of element (row, k) in a SWIZZLE_128B K-major tile (K = 64).
__host__ __device__ constexpr uint32_t off_sw128(int row, int k) {
  return static_cast<uint32_t>((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 3) ^ (row & 7)) & 7) << 4) +
                               (k & 7) * 2);
}

}  // namespace tc
}  // namespace f3d
