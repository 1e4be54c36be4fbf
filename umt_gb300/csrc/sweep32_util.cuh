// sweep32_util.cuh -- device helpers shared by the FP32 sweep kernels
// (sweep32.cu, sweep32p.cu, rz.cu): team lane masks, asynchronous
// global->shared copies, programmatic dependent launch, the approximate
// reciprocal, and group-pair (float2) loads and stores for the paired FP32
// instructions (FFMA2/FMUL2/FADD2) of sm_100-class GPUs.
#pragma once
#include <cuda_runtime.h>

namespace umt {

// Lanes of the calling thread's team (GT consecutive lanes of one warp).
__device__ __forceinline__ unsigned team_mask(int GT, int tid) {
  return (GT == 32) ? 0xffffffffu : (((1u << GT) - 1u) << ((tid & 31) / GT * GT));
}

__device__ __forceinline__ void cp_async(void *smem, const void *gmem, int bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (bytes == 16)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
  else if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
// An L2 cache policy under which the lines a copy brings in are the first to
// be evicted: for data a sweep reads exactly once (the previous flux, the zone
// programs), so that it does not push out of L2 the rows that later work
// items read again (upwind flux written by the previous stage, the source).
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
  unsigned long long pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol));
  return pol;
}
// cp_async with an L2 cache policy; the 16-byte .cg form also bypasses L1
// (for data read once per block).
__device__ __forceinline__ void cp_async_pol(void *smem, const void *gmem, int bytes, unsigned long long pol) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (bytes == 16)
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "l"(pol));
  else if (bytes == 8)
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "l"(pol));
  else
    asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "l"(pol));
}
__device__ __forceinline__ void cp_async16_cg_pol(void *smem, const void *gmem, unsigned long long pol) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "l"(pol));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Bulk (TMA 1-D) copies global -> shared completing on an mbarrier: one
// thread moves a whole contiguous range (16-byte aligned, a multiple of 16
// bytes) and the team waits on the barrier's first phase.
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init_one(uint64_t *b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(b)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy_pol(void *dst, const void *src, uint32_t bytes, uint64_t *b,
                                              unsigned long long pol) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b)), "l"(pol) : "memory");
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b)) : "memory");
}
// Wait for the barrier's phase 0; gives up after 2^22 polls and returns false.
__device__ __forceinline__ bool mbar_wait_phase0(uint64_t *b) {
  for (int i = 0; i < (1 << 22); ++i) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok) : "r"(smem_addr(b)) : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

// Programmatic dependent launch: allow the next kernel of the stream to start
// launching its blocks, and (in that next kernel) wait until the previous
// kernel has completed and its memory writes are visible.  Without a
// programmatic dependency the wait returns at once.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// 1/x for positive, normal x: the hardware reciprocal approximation
// (rcp.approx.ftz.f32, max. 1 ulp).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <int NP>
__device__ __forceinline__ void ld2(const float *p, float2 (&v)[NP]) {
  if constexpr (NP == 2) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = make_float2(t.x, t.y); v[1] = make_float2(t.z, t.w);
  } else {
    v[0] = *reinterpret_cast<const float2 *>(p);
  }
}
template <int NP>
__device__ __forceinline__ void st2(float *p, const float2 (&v)[NP]) {
  if constexpr (NP == 2)
    *reinterpret_cast<float4 *>(p) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
  else
    *reinterpret_cast<float2 *>(p) = v[0];
}

// Let a kernel use all the shared memory its static arrays leave free
// (sweep32.cu).
int allow_dynamic_smem(const void *fn);

}  // namespace umt
