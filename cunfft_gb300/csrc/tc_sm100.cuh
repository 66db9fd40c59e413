// tc_sm100.cuh -- inline-PTX wrappers for the 5th-generation tensor cores (tcgen05),
// tensor memory and mbarriers on sm_100-family GPUs (GB300: sm_103a).
//
// Operand layout used throughout: both operands K-major without swizzle.  The
// unit is the core matrix, 8 rows x 16 bytes (8 x 4 tf32 values along K), stored
// as 128 contiguous bytes.  Element (r, k) of an operand tile sits at byte
//     (r / 8) * SBO + (k / 4) * LBO + (r % 8) * 16 + (k % 4) * 4
// with LBO the step between core matrices along K and SBO the step between
// 8-row groups.  The shared-memory matrix descriptor carries start >> 4, LBO >> 4,
// SBO >> 4, the descriptor version (1 for tcgen05) and the layout (0 = no swizzle).
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace cg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- shared-memory matrix descriptor (K-major, no swizzle) ----
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// K-major operand in the 128-byte swizzled layout written by a TMA load with
// CU_TENSOR_MAP_SWIZZLE_128B: rows of 128 bytes (32 TF32 K values), 8-row atoms of
// 1024 bytes (SBO), the 16-byte chunks of row r XOR-permuted by r mod 8.  The leading
// byte offset is unused (K fits one atom), the layout type 2 (128-byte swizzle) sits
// in bits 61-63.  The atoms must start on 1024-byte boundaries; the k-th group of 8
// K values starts 32 k bytes into the row (the hardware applies the XOR).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// K-major operand in the 64-byte swizzled layout of a TMA load with
// CU_TENSOR_MAP_SWIZZLE_64B: rows of 64 bytes (32 FP16 K values), 8-row atoms of
// 512 bytes (SBO), layout type 4 (64-byte swizzle) in bits 61-63; atoms on 512-byte
// boundaries, the k-th group of 16 K values 32 k bytes into the row.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(512u >> 4) << 32) | (1ull << 46) |
         (4ull << 61);
}

// ---- instruction descriptor: kind::tf32, FP32 accumulator, A and B K-major ----
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                        // D format: F32
         | (2u << 7)                      // A format: TF32
         | (2u << 10)                     // B format: TF32
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// ---- instruction descriptor: kind::f16 with FP16 A and B (same type), FP32 accumulator, K-major ----
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4)                        // D format: F32
         | (0u << 7)                      // A format: F16
         | (0u << 10)                     // B format: F16
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// try_wait that may suspend the thread for up to hint_ns nanoseconds (woken early
// when the phase completes), so a waiting thread does not spin on issue slots
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.  Returns false
// after max_polls unsuccessful polls, each of which suspends the thread for at
// most 1 microsecond.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i)
    if (mbar_try_wait_sleep(bar, parity, 1000u)) return true;
  return false;
}
// The same, after first spinning on the non-blocking test for `spin` polls: a phase that
// completes within a few hundred cycles is seen at once instead of after the suspended
// thread wakes up.  For latency-bound hand-offs where the waiting warp has nothing else to do.
__device__ __forceinline__ bool mbar_wait_spin(uint64_t* bar, uint32_t parity, uint32_t max_polls, uint32_t spin) {
  for (uint32_t i = 0; i < spin; ++i)
    if (mbar_test_wait(bar, parity)) return true;
  return mbar_wait_bounded(bar, parity, max_polls);
}

// arrive (release) on the mbarrier once
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// Arrival that also announces `bytes` of asynchronous (TMA) transactions on the barrier.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// 5-D tiled TMA load of one box into shared memory, completing `bar`'s transactions.
// c0 (the innermost coordinate) times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_5d(void* dst, const void* tmap, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
      : "memory");
}

// Bulk reduction global[0, bytes) += shared[0, bytes) as FP32 adds, performed by the
// bulk-copy engine and L2.  Both addresses 16-byte aligned, bytes a multiple of 16.
// Completion is tracked by this thread's bulk groups.
__device__ __forceinline__ void bulk_reduce_add_f32(void* gdst, uint32_t ssrc, uint32_t bytes) {
  asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.f32 [%0], [%1], %2;\n" ::"l"(gdst), "r"(ssrc),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// this thread's bulk operations have finished reading their shared-memory sources
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// this thread's bulk operations are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// Warp-wide hand-offs on an mbarrier whose count is in warps: one arrival or one
// poller per (converged) warp instead of 32 same-address operations, which the
// shared-memory pipe would serialise.  __syncwarp orders every lane's earlier
// shared-memory writes before lane 0's release, and lane 0's acquire before every
// lane's later accesses.
__device__ __forceinline__ void mbar_arrive_warp(uint64_t* bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
}
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, uint32_t max_polls,
                                               uint32_t spin = 0) {
  uint32_t ok = 1;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait_spin(bar, parity, max_polls, spin) ? 1u : 0u;
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

// named barrier among `count` threads (a multiple of 32) of the CTA
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t count) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
}

// named barrier that also returns, to every participating thread, whether any of them
// passed cond = true (barrier.red.or): a decision all of them take the same way
__device__ __forceinline__ bool named_sync_or(uint32_t id, uint32_t count, bool cond) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %3, 0;\n barrier.cta.red.or.pred q, %1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(id), "r"(count), "r"((uint32_t)cond)
      : "memory");
  return r != 0;
}

// ---- proxy and tcgen05 ordering fences ----
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// ---- tensor memory allocation (one full warp executes these) ----
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- MMA: D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread ----
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// D (+)= A B^T, A and B FP16 (K = 16 per instruction), FP32 accumulator in tensor memory
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// ---- MMA with A in tensor memory: D[tmem] (+)= A[tmem] * B[smem]^T ----
// A (M = 128 rows, K = 16 FP16) occupies lanes 0..127 of 8 columns from tmem_a: row m
// in lane m, elements 2c and 2c + 1 in the low and high halves of column c.
__device__ __forceinline__ void mma_f16_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
      "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on the mbarrier once every previously issued tcgen05 op of this thread completes
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// ---- tensor memory -> registers: 32 lanes x 16 consecutive 32-bit columns ----
// Warp w may access TMEM lanes 32 (w % 4) .. 32 (w % 4) + 31; taddr = base + (lane << 16) + column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// ---- registers -> tensor memory: 32 lanes x 8 consecutive 32-bit columns ----
// Same lane rule as the loads; thread t writes lane (taddr lane) + t.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n" ::"r"(taddr), "r"(r[0]),
               "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
               : "memory");
}
// 32 lanes x 16 consecutive 32-bit columns
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

// ---- FP32 -> (hi, lo) split for 3xTF32 products ----
// hi = tf32(v) rounded to nearest (low 13 mantissa bits zero), lo = v - hi exactly.
__device__ __forceinline__ float tf32_round(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

}  // namespace tc

// (hi, lo) 3xTF32 parts of four values
__device__ __forceinline__ void tc_split4(float4 v, float4& hi, float4& lo) {
  hi.x = tc::tf32_round(v.x);
  hi.y = tc::tf32_round(v.y);
  hi.z = tc::tf32_round(v.z);
  hi.w = tc::tf32_round(v.w);
  lo.x = v.x - hi.x;
  lo.y = v.y - hi.y;
  lo.z = v.z - hi.z;
  lo.w = v.w - hi.w;
}

// Window tap at y = fr + m - l, the FP32 tap of WeightMath<float>::taps, zero outside
// the window 0 <= l < W.  The tap is evaluated for every l and then selected: lanes
// hold different windows, and a branch around it would diverge on every tap.
template <int WIN>
__device__ __forceinline__ float tc_tap(float fr, float mf, int l, int W, TapK k) {
  const float e = win_tap<WIN>(fr + (mf - (float)l), k);
  return (unsigned)l < (unsigned)W ? e : 0.f;
}

}  // namespace cg
