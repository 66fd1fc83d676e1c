// Kernel launchers shared between the C-ABI (capi.cpp) and the CUDA translation units.
#pragma once
#include "vg_types.h"
#include <cstddef>
#include <cuda_runtime.h>

namespace vg {

struct QueryArgs {
  const double *x, *y, *z, *dx, *dy, *dz;
  size_t n;
  void *out;
};

struct StepArgs {
  const double *x, *y, *z, *dx, *dy, *dz, *limit;
  const NavState *in;
  NavState *out;
  double *step;
  int32_t *status;
  int32_t *nvisited;
  size_t n;
};

cudaError_t launch_shape_query_fp64(int type, const double *rec, const Xform &xf, int apply_xf, int q,
                                    const QueryArgs &a, cudaStream_t s);
cudaError_t launch_shape_query_dyn_fp64(const DevGeom &g, int shape, const Xform &xf, int q, const QueryArgs &a,
                                        cudaStream_t s);
cudaError_t launch_locate_fp64(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                               NavState *out, cudaStream_t s);
cudaError_t launch_step_fp64(const DevGeom &g, const StepArgs &a, cudaStream_t s);
cudaError_t launch_step_mixed(const DevGeom &g, const StepArgs &a, cudaStream_t s);
cudaError_t launch_locate_mixed(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                                NavState *out, cudaStream_t s);
// flags: VG_PREC_FP64 (0) or VG_PREC_MIXED (1)
inline cudaError_t launch_step(const DevGeom &g, const StepArgs &a, uint32_t flags, cudaStream_t s)
{
  return (flags & 1u) ? launch_step_mixed(g, a, s) : launch_step_fp64(g, a, s);
}

} // namespace vg
