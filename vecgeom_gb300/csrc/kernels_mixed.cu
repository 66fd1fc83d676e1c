// Unsorted mixed-precision step, locate and step + safety (every shape type), and the
// launchers of the scheduled kernels: each picks the build of the navigation kernels for
// the geometry's shape set (nav_queue_*.cu, nav_transport_*.cu).
#define VG_NAV_SET set_all
#define VG_NAV_UNSCHEDULED_KERNELS
#include "nav_mixed_kernels.cuh"

namespace vg {

cudaError_t launch_step_mixed(const DevGeom &g, const StepArgs &a, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  set_all::k_step_mixed<<<set_all::grid_for(a.n, 256), 256, 0, s>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_step_mixed_queue(const DevGeom &g, const StepArgs &a, unsigned long long *counter,
                                    int blocks_per_sm, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  return core_shapes_only(g) ? set_core::launch_step_mixed_queue(g, a, counter, blocks_per_sm, s)
                             : set_all::launch_step_mixed_queue(g, a, counter, blocks_per_sm, s);
}

cudaError_t launch_step_safety(const DevGeom &g, const StepArgs &a, double *safety, bool mixed, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  const unsigned grid = set_all::grid_for(a.n, 256);
  if (mixed)
    set_all::k_step_safety<true><<<grid, 256, 0, s>>>(g, a, safety);
  else
    set_all::k_step_safety<false><<<grid, 256, 0, s>>>(g, a, safety);
  return cudaGetLastError();
}

cudaError_t launch_transport_iter(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                  int blocks_per_sm, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  return core_shapes_only(g) ? set_core::launch_transport_iter(g, a, mixed, counter, blocks_per_sm, s)
                             : set_all::launch_transport_iter(g, a, mixed, counter, blocks_per_sm, s);
}

cudaError_t launch_transport_drain(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                   cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  return core_shapes_only(g) ? set_core::launch_transport_drain(g, a, mixed, counter, s)
                             : set_all::launch_transport_drain(g, a, mixed, counter, s);
}

cudaError_t launch_transport_init(const NavState *st, size_t n, int32_t *nsteps, int32_t *status, uint32_t *list,
                                  unsigned int *count, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  set_all::k_transport_init<<<set_all::grid_for(n, 256), 256, 0, s>>>(st, n, nsteps, status, list, count);
  return cudaGetLastError();
}

cudaError_t launch_locate_mixed(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                                NavState *out, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  set_all::k_locate_mixed<<<set_all::grid_for(n, 256), 256, 0, s>>>(g, x, y, z, n, out);
  return cudaGetLastError();
}

} // namespace vg
