// mbarrier helpers shared by the tensor-core kernels and the wait self-test.
//
// Every wait in this library's device code is bounded by %globaltimer: after
// the budget a wait returns false and its caller records QD_ERR_TIMEOUT in the
// device status word, which the host reads after the launch; the context stays
// usable.  (No trap, no endless spin.)
#pragma once
#include <cstdint>

namespace qd {

constexpr uint64_t WAIT_NS = 1000000000ull;   // default budget of one wait: 1 s

__device__ inline uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ inline uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ inline void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ inline bool mbar_try_wait(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ inline void mbar_arrive(uint32_t a) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(a) : "memory");
}

// waits for the phase of the given parity to complete; false after budget_ns
__device__ inline bool mbar_wait_bounded(uint32_t a, uint32_t parity, uint64_t budget_ns = WAIT_NS) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(a, parity))
    if (globaltimer() - t0 > budget_ns) return false;
  return true;
}

}  // namespace qd
