// tc_util.cuh -- Blackwell (sm_103a) tensor-core helpers in inline PTX:
// shared-memory matrix descriptors, tcgen05.mma (kind::f16, BF16 inputs, FP32
// accumulation in tensor memory), tcgen05.commit to an mbarrier, tensor
// memory allocation and loads, and bounded mbarrier waits.
//
// Operand layout (no swizzle, K-major, the canonical "interleaved" form): a
// tile of R rows x K columns of 16-bit elements is stored as 8 x 8 core
// matrices of 128 contiguous bytes (8 rows of 16 bytes).  Core matrices that
// are adjacent along K are 128 bytes apart (the descriptor's leading byte
// offset); groups of 8 rows are K*16 bytes apart (its stride byte offset).
// Element (r, k) therefore lives at byte
//     (r / 8) * K * 16 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace umt {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of a K-column operand tile
__host__ __device__ __forceinline__ uint32_t km_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * K * 16 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, each >> 4 in 14 bits; bits 46-48 = 0b001
// (descriptor version of this GPU family); base offset 0; no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9 = 1, bits 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T, issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(tmem_d), "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

// Arrive on the mbarrier once every tcgen05.mma issued so far by this thread
// has completed (its shared-memory reads and tensor-memory writes).
__device__ __forceinline__ void umma_commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok) : "r"(smem_u32(m)), "r"(parity) : "memory");
  return ok != 0;
}

// Wait for the mbarrier phase with the given parity to complete; gives up
// after about 2^24 polls (a few seconds) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *m, uint32_t parity) {
  for (int i = 0; i < (1 << 24); ++i) {
    if (mbar_test(m, parity)) return true;
    if (i >= 32) __nanosleep(64);
  }
  return false;
}

// Tensor memory: allocated and released by one whole warp.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               ::"r"(smem_u32(slot)), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the tensor cores' reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane (32x32b
// shape: warp w of the CTA reads lanes 32w..32w+31, one lane per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  // the registers are written asynchronously: wait, with every register tied
  // to the wait so that no use can be scheduled before it
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Issue D = A[128 x K] * B[N x K]^T as K/16 MMAs (one thread) and commit.
// A and B are K-major canonical tiles at shared addresses sa, sb.
__device__ __forceinline__ void umma_tile(uint32_t tmem_d, uint32_t sa, uint32_t sb, int N, int K,
                                          uint64_t *mbar, bool accumulate) {
  const uint32_t idesc = umma_idesc_bf16(128, N);
  const uint32_t sbo = (uint32_t)K * 16u;
  for (int kk = 0; kk < K / 16; ++kk) {
    const uint64_t da = umma_desc(sa + kk * 256u, 128u, sbo);
    const uint64_t db = umma_desc(sb + kk * 256u, 128u, sbo);
    umma_bf16(tmem_d, da, db, idesc, (accumulate || kk > 0) ? 1u : 0u);
  }
  umma_commit(mbar);
}

// Copy a row-major [R x K] BF16 matrix (global, 16-byte aligned rows) into a
// K-major canonical tile in shared memory, 16 bytes per thread step.
__device__ __forceinline__ void load_tile_km(unsigned char *dst, const __nv_bfloat16 *src, int R, int K, int ld,
                                             int tid, int nthreads) {
  const int c8 = K >> 3;
  for (int q = tid; q < R * c8; q += nthreads) {
    const int r = q / c8, k8 = q - r * c8;
    const uint4 v = *reinterpret_cast<const uint4 *>(src + (size_t)r * ld + k8 * 8);
    *reinterpret_cast<uint4 *>(dst + (r >> 3) * K * 16 + k8 * 128 + (r & 7) * 16) = v;
  }
}

}  // namespace umt
