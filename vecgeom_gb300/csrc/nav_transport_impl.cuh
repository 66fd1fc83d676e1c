#pragma once
// Body of nav_transport_all.cu / nav_transport_core.cu: the transport-stream iteration and
// tail kernels, for the shape set of the including unit.
#include "nav_mixed_kernels.cuh"

namespace vg {
namespace VG_NAV_SET {

cudaError_t launch_transport_iter(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                  int blocks_per_sm, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  if (!mixed) return launch_transport<false, 256, 1>(g, a, counter, s);
  blocks_per_sm = (blocks_per_sm - 1) % 4 + 1; // split configurations: the fused kernel of the same budget
  if (blocks_per_sm == 4) return launch_transport<true, 128, 5>(g, a, counter, s);
  if (blocks_per_sm == 3) return launch_transport<true, 128, 3>(g, a, counter, s);
  return blocks_per_sm == 2 ? launch_transport<true, 256, 2>(g, a, counter, s)
                            : launch_transport<true, 256, 1>(g, a, counter, s);
}

cudaError_t launch_transport_drain(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                   cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  static int resident[2] = {0, 0};
  int &r = resident[mixed ? 1 : 0];
  if (r == 0) {
    int v = 0;
    const cudaError_t e = mixed ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_transport_drain<true>, 256, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_transport_drain<false>, 256, 0);
    if (e != cudaSuccess) return e;
    r = v > 0 ? v : 1;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  size_t blocks = (size_t)sms * r, need = (a.n + 255) / 256;
  if (blocks > need) blocks = need;
  if (mixed)
    k_transport_drain<true><<<(unsigned)blocks, 256, 0, s>>>(g, a, counter);
  else
    k_transport_drain<false><<<(unsigned)blocks, 256, 0, s>>>(g, a, counter);
  return cudaGetLastError();
}

} // namespace VG_NAV_SET
} // namespace vg
