// bulk.cuh -- inline-PTX helpers for bulk global->shared copies
// (cp.async.bulk, completion counted on an mbarrier) used by the SpMV
// kernels, and the step-epilogue trait that names their per-row vectors.
#pragma once

#include <stdint.h>

#include <type_traits>

namespace pdlp {

// Limit of every mbarrier wait: ~2 s at 2 GHz, after which the waiting
// kernel records an error flag and carries on without the data.
constexpr long long kBulkWaitCycles = 4000000000LL;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// L2 policy for data read once per sweep (the tile streams): evicted first,
// so the gathered iterate vectors (8-80 MB) stay resident in the 129 MB L2
// while ~0.5 GB of matrix streams through it every iteration.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint "
      "[%0], [%1], %2, [%3], %4;" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}
// Bounded wait on an mbarrier phase: false after kBulkWaitCycles without completion.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > kBulkWaitCycles) return false;
  return true;
}

// Epilogues that stage per-row vectors declare NV, vec_t, vecs and make_pre;
// the others read their vectors from global memory in row().
template <class E, class = void>
struct step_vectors {
  static constexpr int NV = 0;
  using vec_t = double;
};
template <class E>
struct step_vectors<E, std::void_t<decltype(E::NV)>> {
  static constexpr int NV = E::NV;
  using vec_t = typename E::vec_t;
};

}  // namespace pdlp
