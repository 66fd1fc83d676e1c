#pragma once
// Body of nav_queue_all.cu / nav_queue_core.cu: the persistent work-queue step kernel in its
// four register budgets, fused (configurations 1-4) or split in two kernels (5-8), for the
// shape set of the including unit.
#include "nav_mixed_kernels.cuh"

namespace vg {
namespace VG_NAV_SET {

cudaError_t launch_step_mixed_queue(const DevGeom &g, const StepArgs &a, unsigned long long *counter,
                                    int blocks_per_sm, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  if (blocks_per_sm > 4 && !a.reloc) blocks_per_sm -= 4; // no relocation buffer: the fused kernel
  if (blocks_per_sm == 8) return launch_queue_split<128, 5>(g, a, counter, s);
  if (blocks_per_sm == 7) return launch_queue_split<128, 3>(g, a, counter, s);
  if (blocks_per_sm == 6) return launch_queue_split<256, 2>(g, a, counter, s);
  if (blocks_per_sm == 5) return launch_queue_split<256, 1>(g, a, counter, s);
  cudaError_t e;
  if (blocks_per_sm == 4)
    e = launch_queue<128, 5>(g, a, counter, s);
  else if (blocks_per_sm == 3)
    e = launch_queue<128, 3>(g, a, counter, s);
  else
    e = blocks_per_sm == 2 ? launch_queue<256, 2>(g, a, counter, s) : launch_queue<256, 1>(g, a, counter, s);
  if (e == cudaSuccess && a.steps_done) e = cudaEventRecord(a.steps_done, s);
  return e;
}

} // namespace VG_NAV_SET
} // namespace vg
