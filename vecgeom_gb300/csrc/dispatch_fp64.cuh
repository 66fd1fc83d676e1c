// Run-time shape dispatch (one switch per query on the shape tag of the flattened record)
// used by the navigator and by the SoA kernel of variable-length shapes, plus the boolean
// subtraction, whose operands are placed primitive shapes.
#pragma once
#include "shapes_fp64.cuh"
#include "shapes_more_fp64.cuh"
#include "shapes_torus_fp64.cuh"
#include "shapes_polyhedron_fp64.cuh"
#include "shapes_sphere_fp64.cuh"
#include "shapes_gentrap_fp64.cuh"
#include "shapes_hype_fp64.cuh"

namespace vg {


// Shape types compiled into this translation unit's dispatch (bit t set: shape type t). A
// unit built for a subset serves only geometries whose shape types all lie in it; the
// host selects it from the geometry's type mask (DevGeom::type_mask).
#ifndef VG_SHAPE_MASK
#define VG_SHAPE_MASK 0xffffffffu
#endif
#define VG_HAS_SHAPE(t) (((VG_SHAPE_MASK) >> (t)) & 1u)

#ifndef VG_INLINE_CONTAINS
#define VG_INLINE_CONTAINS 0
#endif

namespace f64 {

// Shapes are addressed either by id (shape) or by (type, off), the tag and record offset
// the caller already holds (PvRec, LeafRec); both reach the same kernels.
template <class R>
__device__ __forceinline__ const R &rec_at(const DevGeom &g, int off)
{
  return *reinterpret_cast<const R *>(g.shape_data + off);
}
#define VG_PRIM_CASES(FN, ...)                                                                  \
  switch (type) {                                                                               \
  case kShapeBox: if (VG_HAS_SHAPE(kShapeBox)) return box_##FN(rec_at<BoxRec>(g, off), __VA_ARGS__); break; \
  case kShapeTube: if (VG_HAS_SHAPE(kShapeTube)) return tube_##FN(rec_at<TubeRec>(g, off), __VA_ARGS__); break; \
  case kShapeCone: if (VG_HAS_SHAPE(kShapeCone)) return cone_##FN(rec_at<ConeRec>(g, off), __VA_ARGS__); break; \
  case kShapeTrd: if (VG_HAS_SHAPE(kShapeTrd)) return trd_##FN(rec_at<TrdRec>(g, off), __VA_ARGS__); break; \
  case kShapeTrap: if (VG_HAS_SHAPE(kShapeTrap)) return trap_##FN(rec_at<TrapRec>(g, off), __VA_ARGS__); break; \
  case kShapeCutTube: if (VG_HAS_SHAPE(kShapeCutTube)) return cuttube_##FN(rec_at<CutTubeRec>(g, off), __VA_ARGS__); break; \
  case kShapeSphere: if (VG_HAS_SHAPE(kShapeSphere)) return sphere_##FN(rec_at<SphereRec>(g, off), __VA_ARGS__); break; \
  case kShapeGenTrap: if (VG_HAS_SHAPE(kShapeGenTrap)) return gentrap_##FN(rec_at<GenTrapRec>(g, off), __VA_ARGS__); break; \
  case kShapeHype: if (VG_HAS_SHAPE(kShapeHype)) return hype_##FN(rec_at<HypeRec>(g, off), __VA_ARGS__); break; \
  case kShapePolycone: if (VG_HAS_SHAPE(kShapePolycone)) return polycone_##FN(rec_at<PolyconeRec>(g, off), __VA_ARGS__); break; \
  case kShapePolyhedron: if (VG_HAS_SHAPE(kShapePolyhedron)) return polyhedron_##FN(rec_at<PolyhedronRec>(g, off), __VA_ARGS__); break; \
  case kShapeTorus2: if (VG_HAS_SHAPE(kShapeTorus2)) return torus_##FN(rec_at<TorusRec>(g, off), __VA_ARGS__); break; \
  default: break;                                                                               \
  }

__device__ inline bool prim_contains_to(const DevGeom &g, int type, int off, V3 p)
{
  VG_PRIM_CASES(contains, p)
  return false;
}
__device__ inline bool prim_contains(const DevGeom &g, int shape, V3 p)
{
  return prim_contains_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline int prim_inside_to(const DevGeom &g, int type, int off, V3 p)
{
  VG_PRIM_CASES(inside, p)
  return kOutside;
}
__device__ inline int prim_inside(const DevGeom &g, int shape, V3 p)
{
  return prim_inside_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline double prim_dist_in_to(const DevGeom &g, int type, int off, V3 p, V3 d)
{
  VG_PRIM_CASES(dist_in, p, d)
  return kInfLength;
}
__device__ inline double prim_dist_in(const DevGeom &g, int shape, V3 p, V3 d)
{
  return prim_dist_in_to(g, g.shape_type[shape], g.shape_off[shape], p, d);
}
__device__ inline double prim_dist_out_to(const DevGeom &g, int type, int off, V3 p, V3 d)
{
  VG_PRIM_CASES(dist_out, p, d)
  return -1.;
}
__device__ inline double prim_dist_out(const DevGeom &g, int shape, V3 p, V3 d)
{
  return prim_dist_out_to(g, g.shape_type[shape], g.shape_off[shape], p, d);
}
__device__ inline double prim_safety_in_to(const DevGeom &g, int type, int off, V3 p)
{
  VG_PRIM_CASES(safety_in, p)
  return kInfLength;
}
__device__ inline double prim_safety_in(const DevGeom &g, int shape, V3 p)
{
  return prim_safety_in_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline double prim_safety_out_to(const DevGeom &g, int type, int off, V3 p)
{
  VG_PRIM_CASES(safety_out, p)
  return -1.;
}
__device__ inline double prim_safety_out(const DevGeom &g, int shape, V3 p)
{
  return prim_safety_out_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
#undef VG_PRIM_CASES

// ---------------------------------------------------------------- boolean subtraction
// Placed-operand helpers (SpecializedPlacedVolImplHelper.h:98-170): mother-frame input.
struct Operand {
  const Xform *xf;
  int shape;
  __device__ Operand(const DevGeom &g, double pv) : xf(&g.pv_xf[(int)pv]), shape(g.lv_shape[g.pv_lv[(int)pv]]) {}
  __device__ bool contains(const DevGeom &g, V3 p) const { return prim_contains(g, shape, to_local(*xf, p)); }
  __device__ int inside(const DevGeom &g, V3 p) const { return prim_inside(g, shape, to_local(*xf, p)); }
  __device__ double dist_in(const DevGeom &g, V3 p, V3 d) const
  {
    return prim_dist_in(g, shape, to_local(*xf, p), rotate(*xf, d));
  }
  __device__ double placed_dist_out(const DevGeom &g, V3 p, V3 d) const
  {
    return prim_dist_out(g, shape, to_local(*xf, p), rotate(*xf, d));
  }
};

// BooleanImplementation.h:64-72
__device__ inline bool boolminus_contains(const DevGeom &g, const BoolRec &b, V3 p)
{
  if (!Operand(g, b.left_pv).contains(g, p)) return false;
  return !Operand(g, b.right_pv).contains(g, p);
}
// BooleanImplementation.h:73-107
__device__ inline int boolminus_inside(const DevGeom &g, const BoolRec &b, V3 p)
{
  const int a = Operand(g, b.left_pv).inside(g, p);
  if (a == kOutside) return kOutside;
  const int c = Operand(g, b.right_pv).inside(g, p);
  if (a == kInside && c == kOutside) return kInside;
  if ((a == kInside && c == kSurface) || (c == kOutside && a == kSurface)) return kSurface;
  return kOutside;
}
// BooleanImplementation.h:108-147 (push loop bounded by kBoolMaxPush; a track that hits the
// bound gets kInfLength)
__device__ inline double boolminus_dist_in(const DevGeom &g, const BoolRec &b, V3 p, V3 dir)
{
  const Operand L(g, b.left_pv), R(g, b.right_pv);
  double snxt = 0.;
  V3 hit      = p;
  bool inR    = R.contains(g, p);
  for (int it = 0; it < kBoolMaxPush; ++it) {
    if (inR) {
      const double d1 = R.placed_dist_out(g, hit, dir);
      const bool okd  = dge(d1, 0.) && dlt(d1, kInfLength);
      snxt += okd ? (d1 + kPushTolerance) : 0.;
      const double s = okd ? (d1 + kPushTolerance) : 0.;
      hit            = V3{hit.x + s * dir.x, hit.y + s * dir.y, hit.z + s * dir.z};
      if (L.contains(g, hit) && dgt(L.placed_dist_out(g, hit, dir), kPushTolerance)) return snxt;
    }
    double d2 = L.dist_in(g, hit, dir);
    d2        = dmax(d2, 0.);
    if (deq(d2, kInfLength)) return kInfLength;
    const double d1 = R.dist_in(g, hit, dir);
    if (dlt(d2, d1 - kTolerance)) return snxt + (d2 + kPushTolerance);
    const bool okd = dge(d1, 0.) && dlt(d1, kInfLength);
    snxt += okd ? d1 + kPushTolerance : 0.;
    const double s = okd ? (d1 + kPushTolerance) : kPushTolerance;
    hit            = V3{hit.x + s * dir.x, hit.y + s * dir.y, hit.z + s * dir.z};
    inR            = true;
  }
  return kInfLength;
}
// BooleanImplementation.h:148-157
__device__ inline double boolminus_dist_out(const DevGeom &g, const BoolRec &b, V3 p, V3 d)
{
  const double dl = Operand(g, b.left_pv).placed_dist_out(g, p, d);
  const double dr = Operand(g, b.right_pv).dist_in(g, p, d);
  return dmin(dl, dr);
}
// BooleanImplementation.h:158-170
__device__ inline double boolminus_safety_in(const DevGeom &g, const BoolRec &b, V3 p)
{
  const Operand L(g, b.left_pv), R(g, b.right_pv);
  if (L.contains(g, p) && R.contains(g, p)) return prim_safety_out(g, R.shape, to_local(*R.xf, p));
  return prim_safety_in(g, L.shape, to_local(*L.xf, p));
}
// BooleanImplementation.h:171-178 (left operand queried in the boolean's frame)
__device__ inline double boolminus_safety_out(const DevGeom &g, const BoolRec &b, V3 p)
{
  const Operand L(g, b.left_pv), R(g, b.right_pv);
  const double sl = prim_safety_out(g, L.shape, p);
  const double sr = prim_safety_in(g, R.shape, to_local(*R.xf, p));
  return dmin(sl, sr);
}

// ---------------------------------------------------------------- full dispatch
// Out of line by default: the scheduled step kernels call it from several places (relocation,
// Contains fallbacks) and inlining every copy costs them instruction-cache misses (3.6 %
// slower); the plain-FP64 navigator unit sets VG_INLINE_CONTAINS, where inlining is faster.
#if VG_INLINE_CONTAINS
__device__ inline bool shape_contains_to(const DevGeom &g, int type, int off, V3 p)
#else
static __device__ __noinline__ bool shape_contains_to(const DevGeom &g, int type, int off, V3 p)
#endif
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_contains(g, rec_at<BoolRec>(g, off), p);
  return prim_contains_to(g, type, off, p);
}
__device__ inline bool shape_contains(const DevGeom &g, int shape, V3 p)
{
  return shape_contains_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline int shape_inside_to(const DevGeom &g, int type, int off, V3 p)
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_inside(g, rec_at<BoolRec>(g, off), p);
  return prim_inside_to(g, type, off, p);
}
__device__ inline int shape_inside(const DevGeom &g, int shape, V3 p)
{
  return shape_inside_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline double shape_dist_in_to(const DevGeom &g, int type, int off, V3 p, V3 d)
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_dist_in(g, rec_at<BoolRec>(g, off), p, d);
  return prim_dist_in_to(g, type, off, p, d);
}
__device__ inline double shape_dist_in(const DevGeom &g, int shape, V3 p, V3 d)
{
  return shape_dist_in_to(g, g.shape_type[shape], g.shape_off[shape], p, d);
}
__device__ inline double shape_dist_out_to(const DevGeom &g, int type, int off, V3 p, V3 d)
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_dist_out(g, rec_at<BoolRec>(g, off), p, d);
  return prim_dist_out_to(g, type, off, p, d);
}
__device__ inline double shape_dist_out(const DevGeom &g, int shape, V3 p, V3 d)
{
  return shape_dist_out_to(g, g.shape_type[shape], g.shape_off[shape], p, d);
}
__device__ inline double shape_safety_in_to(const DevGeom &g, int type, int off, V3 p)
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_safety_in(g, rec_at<BoolRec>(g, off), p);
  return prim_safety_in_to(g, type, off, p);
}
__device__ inline double shape_safety_in(const DevGeom &g, int shape, V3 p)
{
  return shape_safety_in_to(g, g.shape_type[shape], g.shape_off[shape], p);
}
__device__ inline double shape_safety_out_to(const DevGeom &g, int type, int off, V3 p)
{
  if (VG_HAS_SHAPE(kShapeBoolMinus) && type == kShapeBoolMinus) return boolminus_safety_out(g, rec_at<BoolRec>(g, off), p);
  return prim_safety_out_to(g, type, off, p);
}
__device__ inline double shape_safety_out(const DevGeom &g, int shape, V3 p)
{
  return shape_safety_out_to(g, g.shape_type[shape], g.shape_off[shape], p);
}

} // namespace f64
} // namespace vg
