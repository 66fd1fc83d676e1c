#pragma once
// Plain-FP64 ComputeStepAndPropagatedState, one thread per track, for the shape set of the
// including unit (VG_NAV_SET, VG_SHAPE_MASK; kernels_nav_fp64.cu, nav_step_fp64_core.cu).
// The unit defines the FP64 compile switches of the plain navigator before including it.
#ifndef VG_NAV_SET
#error "define VG_NAV_SET before including nav_fp64_step_impl.cuh"
#endif
#include "launch.h"
#include "nav_fp64.cuh"

namespace vg {
namespace VG_NAV_SET {
namespace {

__global__ void __launch_bounds__(256) k_step(const DevGeom g, const StepArgs a)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const size_t t   = a.order ? (size_t)__ldg(a.order + i) : i;
    const NavState s = a.in[t];
    NavState o;
    int st = 0, nv = 0;
    const double lim = a.limit ? __ldg(a.limit + t) : kInfLength;
    a.step[t] = f64::compute_step(g, f64::V3{__ldg(a.x + t), __ldg(a.y + t), __ldg(a.z + t)},
                                  f64::V3{__ldg(a.dx + t), __ldg(a.dy + t), __ldg(a.dz + t)}, lim, s, o, st,
                                  a.nvisited ? &nv : nullptr);
    a.out[t] = o;
    if (a.status) a.status[t] = st;
    if (a.nvisited) a.nvisited[t] = nv;
  }
}

} // namespace

cudaError_t launch_step_fp64(const DevGeom &g, const StepArgs &a, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  size_t blocks = (a.n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_step<<<(unsigned)blocks, 256, 0, s>>>(g, a);
  return cudaGetLastError();
}

} // namespace VG_NAV_SET
} // namespace vg
