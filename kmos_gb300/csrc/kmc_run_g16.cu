// kmc_run_g16.cu -- the step kernel's two-trajectories-per-warp variants (16 lanes per
// trajectory, kmc_run.cuh), for models of up to 64 processes: 1, 2 or 4 processes per
// lane, 3 or 4 rounds of fast-stream edits.  A separate translation unit so that the
// variants compile in parallel with the rest of the engine.
#include "kmc_run.cuh"

namespace kmc_host {
const void *run_kernel_g16(int np, int r) {
  using kmc::kmc_run_kernel;
  switch (np * 10 + r) {
    case 13: return (const void *)kmc_run_kernel<1, 3, 16>;
    case 14: return (const void *)kmc_run_kernel<1, 4, 16>;
    case 23: return (const void *)kmc_run_kernel<2, 3, 16>;
    case 24: return (const void *)kmc_run_kernel<2, 4, 16>;
    case 43: return (const void *)kmc_run_kernel<4, 3, 16>;
    case 44: return (const void *)kmc_run_kernel<4, 4, 16>;
    default: return nullptr;
  }
}
}  // namespace kmc_host
