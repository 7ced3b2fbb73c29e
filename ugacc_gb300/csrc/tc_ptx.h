// PTX building blocks of the tcgen05 / TMA / mbarrier kernels (sm_103a): shared by the
// tensor-core GEMMs (tc_gemm.cu) and the fused guess-network kernel (mlp.cu).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

namespace ucc {
namespace tc {

constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s per bounded wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(n));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false if the deadline passed or another warp raised the error flag.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* err,
                                          unsigned long long limit_ns = WAIT_NS) {
  if (mbar_test(b, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_test(b, parity)) return true;
    if ((it & 255u) == 0) {
      if (*(volatile int*)err) return false;
      if (gtimer() - t0 > limit_ns) {
        atomicExch(err, 1);
        return false;
      }
    }
  }
}
// Bounded wait that ignores the error flag (used to drain in-flight copies).
__device__ __forceinline__ void mbar_wait_deadline(uint64_t* b, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (!mbar_test(b, parity))
    if (gtimer() - t0 > WAIT_NS) return;
}
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
// the same load into the same shared-memory offset of every CTA in cta_mask (cluster
// multicast; complete_tx lands on the barrier at the same offset in each of them)
__device__ __forceinline__ void tma_load_mc(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y,
                                            uint16_t cta_mask) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar)), "h"(cta_mask)
      : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// every thread of every CTA of the cluster
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// shared-memory matrix descriptor: K-major, 128B swizzle, 8-row core groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(const void* p) {
  const uint64_t a = smem_u32(p);
  return ((a & 0x3FFFFull) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}
__device__ __forceinline__ void mma_i(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// arrive on the barrier at this offset in every CTA of cta_mask once this thread's MMAs complete
__device__ __forceinline__ void mma_commit_mc(uint64_t* bar, uint16_t cta_mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(cta_mask)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// shared-memory stores of ordinary instructions made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// FP32 -> FP64 by moving the bit fields (integer pipe, GB300 has few FP64 units); zero,
// subnormal, infinite and NaN inputs take the converting instruction
__device__ __forceinline__ double f32_bits_to_f64(uint32_t fb) {
  const uint32_t e = (fb >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)__uint_as_float(fb);
  const unsigned long long sgn = (unsigned long long)(fb >> 31) << 63;
  const unsigned long long ex = (unsigned long long)(e + 896u) << 52;
  const unsigned long long mt = (unsigned long long)(fb & 0x7FFFFFu) << 29;
  return __longlong_as_double((long long)(sgn | ex | mt));
}

// FP64 -> FP32 truncated toward zero by moving the bit fields (relative error below 2^-23,
// integer pipe); zeros keep their sign, values outside FP32's normal range take the
// converting instruction
__device__ __forceinline__ float f64_to_f32_trunc(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
  if ((b << 1) == 0ull) return __uint_as_float(sgn);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < -126 || e > 127) return (float)v;
  return __uint_as_float(sgn | ((uint32_t)(e + 127) << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}


}  // namespace tc
}  // namespace ucc
