// Inline-PTX helpers for mbarrier pipelines fed by bulk asynchronous copies
// (cp.async.bulk, the non-tensor form of TMA).  All waits are bounded: after
// BF_SPIN_LIMIT polls the waiter records an error and gives up, so a broken
// protocol can never hang the GPU.
#pragma once

#include <cstdint>

namespace bfg {

constexpr long long BF_SPIN_LIMIT = 1ll << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
          bar),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait until the phase with the given parity of barrier `bar` has completed.
// Returns false after `limit` polls (setting *err), or as soon as another
// thread has set *err, so that every waiter leaves promptly once one of them
// has given up.  The default limit is about a second of polling; the plain
// path's bulk-copy kernel takes it from the operator, so that a test can make
// its waits run out (bf_op_set_wait_limit).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err,
                                          long long limit = BF_SPIN_LIMIT) {
  for (long long it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 32) {
      __nanosleep(64);
      if ((it & 63) == 0 && *(volatile int*)err) return false;
    }
  }
  atomicExch(err, 1);
  return false;
}

// Bounded wait that ignores *err: used to let the block's own bulk copies
// land before it exits.  Its limit is always the default one: copies that
// were issued do complete, and the block must not exit before they have.
__device__ __forceinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity, int* err) {
  for (long long it = 0; it < BF_SPIN_LIMIT; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 32) __nanosleep(64);
  }
  atomicExch(err, 2);
  return false;
}

// order earlier generic-proxy shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// global -> shared bulk copy completing `bytes` of transaction count on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// barrier among the first `nthreads` threads of the block (named barrier 1)
__device__ __forceinline__ void named_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

}  // namespace bfg
