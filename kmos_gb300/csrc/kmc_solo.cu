// kmc_solo.cu -- the solo kernel's variants (kmc_run.cuh): one per process count
// 1..SOLO_PMAX, each with the program and tables on chip or in device memory.  A
// separate translation unit so that they compile in parallel with the rest of the engine.
#define KMC_DEFINE_SOLO_KERNEL
#include "kmc_run.cuh"

namespace kmc_host {
const void *solo_kernel(int P, bool onchip) {
  using kmc::kmc_solo_kernel;
#define KMC_SOLO_CASE(N) \
  case N:                \
    return onchip ? (const void *)kmc_solo_kernel<N, true> : (const void *)kmc_solo_kernel<N, false>;
  switch (P) {
    KMC_SOLO_CASE(1) KMC_SOLO_CASE(2) KMC_SOLO_CASE(3) KMC_SOLO_CASE(4)
    KMC_SOLO_CASE(5) KMC_SOLO_CASE(6) KMC_SOLO_CASE(7) KMC_SOLO_CASE(8)
    default: return nullptr;
  }
#undef KMC_SOLO_CASE
}
}  // namespace kmc_host
