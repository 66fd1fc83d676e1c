// Plain-FP64 navigation kernels: one thread per track, LocatePoint, ApproachNextDaughter and
// the launcher of ComputeStepAndPropagatedState (nav_fp64_step_impl.cuh, one build per shape set). Compiled with --fmad=false. These divergent kernels are
// latency-bound, so FP64 compares stay on the FP64 pipe and the exact shortcuts are off
// (VG_FP64_INT_COMPARE 0, VG_FP64_SHORTCUTS 0, see fp64_int.cuh).
#define VG_FP64_INT_COMPARE 0
#define VG_FP64_SHORTCUTS 0
#define VG_INLINE_CONTAINS 1
#include "launch.h"
#include "nav_fp64.cuh"
#define VG_NAV_SET set_all
#include "nav_fp64_step_impl.cuh"

namespace vg {
namespace {

using f64::V3;

inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

__global__ void __launch_bounds__(256) k_locate(const DevGeom g, const double *__restrict__ x,
                                                const double *__restrict__ y, const double *__restrict__ z, size_t n,
                                                NavState *__restrict__ out)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    NavState s{0u, 0u, 0, {0, 0, 0}};
    int status = 0;
    f64::locate_global_point(g, g.world_pv, V3{__ldg(x + i), __ldg(y + i), __ldg(z + i)}, s.navInd, true, status);
    out[i] = s;
  }
}

// BVH::ApproachNextDaughter (source/BVH.cpp:394-449) in the frame of each track's volume,
// with the state's last-exited volume as `last`, as the step passes it to
// CheckDaughterIntersections.
__global__ void __launch_bounds__(256) k_approach(const DevGeom g, const double *__restrict__ x,
                                                  const double *__restrict__ y, const double *__restrict__ z,
                                                  const double *__restrict__ dx, const double *__restrict__ dy,
                                                  const double *__restrict__ dz, const NavState *__restrict__ in,
                                                  double *__restrict__ step, int32_t *__restrict__ status, size_t n)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const NavState s = in[i];
    int st           = kTrackErrState;
    if (s.navInd != 0) {
      const Xform m = f64::nav_top_matrix(g, s.navInd);
      const int lv  = g.pv_lv[f64::nav_top(g, s.navInd)];
      double t      = step[i];
      st            = kTrackOk;
      if (g.lv_nd[lv] > 0)
        st = f64::bvh_approach_next_daughter(g, lv, f64::to_local(m, V3{__ldg(x + i), __ldg(y + i), __ldg(z + i)}),
                                             f64::rotate(m, V3{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)}), t,
                                             f64::nav_top(g, s.lastExited));
      if (st == kTrackOk) step[i] = t;
    }
    if (status) status[i] = st;
  }
}

} // namespace

cudaError_t launch_approach_fp64(const DevGeom &g, const double *x, const double *y, const double *z,
                                 const double *dx, const double *dy, const double *dz, const NavState *in,
                                 double *step, int32_t *status, size_t n, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  k_approach<<<grid_for(n, 256), 256, 0, s>>>(g, x, y, z, dx, dy, dz, in, step, status, n);
  return cudaGetLastError();
}

cudaError_t launch_locate_fp64(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                               NavState *out, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  k_locate<<<grid_for(n, 256), 256, 0, s>>>(g, x, y, z, n, out);
  return cudaGetLastError();
}

cudaError_t launch_step_fp64(const DevGeom &g, const StepArgs &a, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  return core_shapes_only(g) ? set_core::launch_step_fp64(g, a, s) : set_all::launch_step_fp64(g, a, s);
}

} // namespace vg
