// Run-time shape dispatch for the navigator (one switch per query on the shape tag of
// the flattened record). The per-shape SoA kernels do not use it: they are instantiated
// per shape type.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {
namespace f64 {

#define VG_SHAPE_CASES(FN, ...)                                                     \
  switch (g.shape_type[shape]) {                                                    \
  case kShapeBox: return box_##FN(rec<BoxRec>(g, shape), __VA_ARGS__);              \
  case kShapeTube: return tube_##FN(rec<TubeRec>(g, shape), __VA_ARGS__);           \
  case kShapeCone: return cone_##FN(rec<ConeRec>(g, shape), __VA_ARGS__);           \
  default: break;                                                                   \
  }

__device__ inline bool shape_contains(const DevGeom &g, int shape, V3 p)
{
  VG_SHAPE_CASES(contains, p)
  return false;
}
__device__ inline int shape_inside(const DevGeom &g, int shape, V3 p)
{
  VG_SHAPE_CASES(inside, p)
  return kOutside;
}
__device__ inline double shape_dist_in(const DevGeom &g, int shape, V3 p, V3 d)
{
  VG_SHAPE_CASES(dist_in, p, d)
  return kInfLength;
}
__device__ inline double shape_dist_out(const DevGeom &g, int shape, V3 p, V3 d)
{
  VG_SHAPE_CASES(dist_out, p, d)
  return -1.;
}
__device__ inline double shape_safety_in(const DevGeom &g, int shape, V3 p)
{
  VG_SHAPE_CASES(safety_in, p)
  return kInfLength;
}
__device__ inline double shape_safety_out(const DevGeom &g, int shape, V3 p)
{
  VG_SHAPE_CASES(safety_out, p)
  return -1.;
}
#undef VG_SHAPE_CASES

} // namespace f64
} // namespace vg
