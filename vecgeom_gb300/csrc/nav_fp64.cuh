// Plain-FP64 BVH navigation on the flattened device geometry: NavIndex state operations,
// BVH traversals, GlobalLocator and the BVHNavigator step with relocation. Every loop is
// bounded; when a bound is hit the track gets an error status instead of trapping.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {

// Per-track status codes (also VG_TRACK_* in the C-ABI).
constexpr int32_t kTrackOk       = 0;
constexpr int32_t kTrackErrStack = 1; // BVH stack would overflow
constexpr int32_t kTrackErrIter  = 2; // a relocation/locate loop exceeded its bound
constexpr int32_t kTrackErrState = 3; // input state is outside the world or not a table node

namespace f64 {

// ---------------------------------------------------------------- shape dispatch
template <class R>
__device__ __forceinline__ const R &rec(const DevGeom &g, int shape)
{
  return *reinterpret_cast<const R *>(g.shape_data + g.shape_off[shape]);
}

} // namespace f64
} // namespace vg
#include "dispatch_fp64.cuh"
namespace vg {
namespace f64 {

__device__ __forceinline__ int pv_shape(const DevGeom &g, int pv) { return g.lv_shape[g.pv_lv[pv]]; }

// ---------------------------------------------------------------- NavIndex table (NavStateIndex.h:172-265)
__device__ __forceinline__ uint32_t nav_pop(const DevGeom &g, uint32_t n) { return n > 0 ? __ldg(&g.nav[n]) : 0u; }
__device__ __forceinline__ uint32_t nav_push(const DevGeom &g, uint32_t n, int pv)
{
  return n > 0 ? __ldg(&g.nav[n + 3 + g.pv_child[pv]]) : 1u;
}
__device__ __forceinline__ int nav_top(const DevGeom &g, uint32_t n) { return n > 0 ? (int)__ldg(&g.nav[n + 1]) : -1; }
__device__ __forceinline__ uint32_t nav_meta(const DevGeom &g, uint32_t n) { return __ldg(&g.nav[n + 2]); }

// TopMatrixImpl (NavStateIndex.h:232-265). Tables built by this library cache the global
// matrix of every node (has-matrix bit 0x04 set), so the matrix is read directly; absent
// translation or rotation parts stay at their identity values.
__device__ __forceinline__ Xform nav_top_matrix(const DevGeom &g, uint32_t n)
{
  Xform t;
  for (int i = 0; i < 3; ++i) t.t[i] = 0.;
  for (int i = 0; i < 9; ++i) t.r[i] = (i % 4 == 0) ? 1. : 0.;
  if (n == 0) return t;
  const uint32_t meta = nav_meta(g, n);
  const bool hasTrans = (meta & 0x200u) != 0, hasRot = (meta & 0x100u) != 0;
  if (!(meta & 0x400u) || (!hasTrans && !hasRot)) return t;
  const uint32_t nd = meta >> 16;
  uint32_t w        = n + 3 + nd + ((nd + 1) & 1);
  w += (w & 1u);
  const double *m = reinterpret_cast<const double *>(g.nav + w);
  if (hasTrans)
    for (int i = 0; i < 3; ++i) t.t[i] = __ldg(m + i);
  if (hasRot)
    for (int i = 0; i < 9; ++i) t.r[i] = __ldg(m + 3 + i);
  return t;
}

// ---------------------------------------------------------------- boxes (VecGeom/base/AABB.h)
__device__ __forceinline__ bool aabb_contains(const double *b, V3 p)
{
  return dge(p.x, __ldg(b)) && dle(p.x, __ldg(b + 3)) && dge(p.y, __ldg(b + 1)) && dle(p.y, __ldg(b + 4)) &&
         dge(p.z, __ldg(b + 2)) && dle(p.z, __ldg(b + 5));
}
__device__ __forceinline__ void aabb_slab(const double *b, V3 p, V3 inv, double &tmin, double &tmax)
{
  double t0x = (__ldg(b) - p.x) * inv.x, t1x = (__ldg(b + 3) - p.x) * inv.x;
  double t0y = (__ldg(b + 1) - p.y) * inv.y, t1y = (__ldg(b + 4) - p.y) * inv.y;
  double t0z = (__ldg(b + 2) - p.z) * inv.z, t1z = (__ldg(b + 5) - p.z) * inv.z;
  if (dgt(t0x, t1x)) { double s = t0x; t0x = t1x; t1x = s; }
  if (dgt(t0y, t1y)) { double s = t0y; t0y = t1y; t1y = s; }
  if (dgt(t0z, t1z)) { double s = t0z; t0z = t1z; t1z = s; }
  tmin = max3(t0x, t0y, t0z);
  tmax = min3(t1x, t1y, t1z) * (1. + 2 * kEpsilon);
}

// ---------------------------------------------------------------- placed volumes
__device__ __forceinline__ double pv_dist_in(const DevGeom &g, int pv, V3 p, V3 d)
{
  const Xform &m = g.pv_xf[pv];
  return shape_dist_in(g, pv_shape(g, pv), to_local(m, p), rotate(m, d));
}
__device__ __forceinline__ bool pv_contains(const DevGeom &g, int pv, V3 p, V3 &lp)
{
  lp = to_local(g.pv_xf[pv], p);
  return shape_contains(g, pv_shape(g, pv), lp);
}

// BVH::CheckDaughterIntersections (VecGeom/base/BVH.h:96-146)
__device__ __forceinline__ int bvh_check_daughters(const DevGeom &g, int lv, V3 lp, V3 ld, double &step, int last_pv,
                                                   int &hit_pv, int *nvisited)
{
  const int b = g.lv_bvh[lv];
  if (b < 0) return kTrackOk;
  const int node0 = g.bvh_node0[b];
  const int dbase = g.lv_dstart[lv];
  const V3 inv{1.0 / nonzero(ld.x), 1.0 / nonzero(ld.y), 1.0 / nonzero(ld.z)};
  unsigned stack[32];
  int sp     = 1;
  stack[0]   = 0;
  int visits = 0;
  do {
    const unsigned id = stack[--sp];
    ++visits;
    const int nc = __ldg(&g.node_nchild[node0 + id]);
    if (nc >= 0) {
      const int off = __ldg(&g.node_offset[node0 + id]);
      for (int i = 0; i < nc; ++i) {
        const int prim = __ldg(&g.prim_id[off + i]);
        double tmin, tmax;
        aabb_slab(g.prim_box + 6 * (size_t)(dbase + prim), lp, inv, tmin, tmax);
        if (dle(tmin, tmax) && dge(tmax, 0.0) && dlt(tmin, step)) {
          const int vol     = __ldg(&g.daughters[dbase + prim]);
          const double dist = pv_dist_in(g, vol, lp, ld);
          if (dlt(dist, step) && !(dle(dist, 0.0) && vol == last_pv)) step = dist, hit_pv = vol;
        }
      }
    } else {
      const unsigned cl = 2 * id + 1, cr = 2 * id + 2;
      double tminL, tmaxL, tminR, tmaxR;
      aabb_slab(g.node_box + 6 * (size_t)(node0 + cl), lp, inv, tminL, tmaxL);
      aabb_slab(g.node_box + 6 * (size_t)(node0 + cr), lp, inv, tminR, tmaxR);
      const bool tl = dle(tminL, tmaxL) && dge(tmaxL, 0.0) && dlt(tminL, step);
      const bool tr = dle(tminR, tmaxR) && dge(tmaxR, 0.0) && dlt(tminR, step);
      if (sp + 2 > 32) {
        if (nvisited) *nvisited = visits;
        return kTrackErrStack;
      }
      if (dlt(tminR, tminL)) {
        if (tr) stack[sp++] = cr;
        if (tl) stack[sp++] = cl;
      } else {
        if (tl) stack[sp++] = cl;
        if (tr) stack[sp++] = cr;
      }
    }
  } while (sp > 0);
  if (nvisited) *nvisited = visits;
  return kTrackOk;
}

// VUnplacedVolume::ApproachSolid (UnplacedVolume.h:272-280): BoxImplementation::
// IntersectCachedKernel2 (BoxImplementation.h:324-368) on the shape's bounding box `bb`
// (lo xyz, hi xyz) with t0 = 0, t1 = kInfLength; kInfLength on a miss.
__device__ __forceinline__ double approach_solid(const double *bb, V3 p, V3 inv)
{
  const int sx = dlt(inv.x, 0.) ? 3 : 0, sy = dlt(inv.y, 0.) ? 3 : 0, sz = dlt(inv.z, 0.) ? 3 : 0;
  double tmin        = (__ldg(bb + sx) - p.x) * inv.x;
  const double tymax = (__ldg(bb + 4 - sy) - p.y) * inv.y;
  if (dgt(tmin, tymax)) return kInfLength;
  double tmax        = (__ldg(bb + 3 - sx) - p.x) * inv.x;
  const double tymin = (__ldg(bb + 1 + sy) - p.y) * inv.y;
  if (dgt(tymin, tmax)) return kInfLength;
  tmin               = dmax(tmin, tymin);
  tmax               = dmin(tmax, tymax);
  const double tzmin = (__ldg(bb + 2 + sz) - p.z) * inv.z;
  const double tzmax = (__ldg(bb + 5 - sz) - p.z) * inv.z;
  if (dgt(tmin, tzmax) || dgt(tzmin, tmax)) return kInfLength;
  tmin = dmax(tmin, tzmin);
  tmax = dmin(tmax, tzmax);
  if (!(dle(tmin, kInfLength + kTolerance) && dgt(tmax, 0. - kTolerance))) return kInfLength;
  return tmin;
}

// BVH::ApproachNextDaughter (source/BVH.cpp:394-449): the traversal of
// CheckDaughterIntersections with each candidate's bounding-box approach distance (in its own
// frame) in place of its DistanceToIn; lowers `step` to the first box the ray reaches.
__device__ __forceinline__ int bvh_approach_next_daughter(const DevGeom &g, int lv, V3 lp, V3 ld, double &step,
                                                          int last_pv)
{
  const int b = g.lv_bvh[lv];
  if (b < 0) return kTrackOk;
  const int node0 = g.bvh_node0[b];
  const int dbase = g.lv_dstart[lv];
  const V3 inv{1.0 / nonzero(ld.x), 1.0 / nonzero(ld.y), 1.0 / nonzero(ld.z)};
  unsigned stack[32];
  int sp   = 1;
  stack[0] = 0;
  do {
    const unsigned id = stack[--sp];
    const int nc      = __ldg(&g.node_nchild[node0 + id]);
    if (nc >= 0) {
      const int off = __ldg(&g.node_offset[node0 + id]);
      for (int i = 0; i < nc; ++i) {
        const int prim = __ldg(&g.prim_id[off + i]);
        double tmin, tmax;
        aabb_slab(g.prim_box + 6 * (size_t)(dbase + prim), lp, inv, tmin, tmax);
        if (dle(tmin, tmax) && dge(tmax, 0.0) && dlt(tmin, step)) {
          const int vol  = __ldg(&g.daughters[dbase + prim]);
          const Xform &m = g.pv_xf[vol];
          const V3 d     = rotate(m, ld);
          const V3 dinv{1.0 / nonzero(d.x), 1.0 / nonzero(d.y), 1.0 / nonzero(d.z)};
          const double dist = approach_solid(g.shape_bbox + 6 * (size_t)pv_shape(g, vol), to_local(m, lp), dinv);
          if (dlt(dist, step) && !(dle(dist, 0.0) && vol == last_pv)) step = dist;
        }
      }
    } else {
      const unsigned cl = 2 * id + 1, cr = 2 * id + 2;
      double tminL, tmaxL, tminR, tmaxR;
      aabb_slab(g.node_box + 6 * (size_t)(node0 + cl), lp, inv, tminL, tmaxL);
      aabb_slab(g.node_box + 6 * (size_t)(node0 + cr), lp, inv, tminR, tmaxR);
      const bool tl = dle(tminL, tmaxL) && dge(tmaxL, 0.0) && dlt(tminL, step);
      const bool tr = dle(tminR, tmaxR) && dge(tmaxR, 0.0) && dlt(tminR, step);
      if (sp + 2 > 32) return kTrackErrStack;
      if (dlt(tminR, tminL)) {
        if (tr) stack[sp++] = cr;
        if (tl) stack[sp++] = cl;
      } else {
        if (tl) stack[sp++] = cl;
        if (tr) stack[sp++] = cr;
      }
    }
  } while (sp > 0);
  return kTrackOk;
}

// BVH::LevelLocate, excluded-volume variant (BVH.h:236-285)
__device__ __forceinline__ bool bvh_level_locate(const DevGeom &g, int lv, int excl_pv, V3 lp, int &pv, V3 &dlp,
                                                 int &status)
{
  const int b     = g.lv_bvh[lv];
  const int node0 = g.bvh_node0[b];
  const int dbase = g.lv_dstart[lv];
  unsigned stack[32];
  int sp   = 1;
  stack[0] = 0;
  do {
    const unsigned id = stack[--sp];
    const int nc      = __ldg(&g.node_nchild[node0 + id]);
    if (nc >= 0) {
      const int off = __ldg(&g.node_offset[node0 + id]);
      for (int i = 0; i < nc; ++i) {
        const int prim = __ldg(&g.prim_id[off + i]);
        if (aabb_contains(g.prim_box + 6 * (size_t)(dbase + prim), lp)) {
          const int vol = __ldg(&g.daughters[dbase + prim]);
          if (vol != excl_pv && pv_contains(g, vol, lp, dlp)) {
            pv = vol;
            return true;
          }
        }
      }
    } else {
      if (sp + 2 > 32) {
        status = kTrackErrStack;
        return false;
      }
      const unsigned cl = 2 * id + 1, cr = 2 * id + 2;
      if (aabb_contains(g.node_box + 6 * (size_t)(node0 + cl), lp)) stack[sp++] = cl;
      if (aabb_contains(g.node_box + 6 * (size_t)(node0 + cr), lp)) stack[sp++] = cr;
    }
  } while (sp > 0);
  return false;
}

// GlobalLocator::LocateGlobalPoint (GlobalLocator.h:35-82); returns the located pv or -1.
__device__ __forceinline__ int locate_global_point(const DevGeom &g, int vol, V3 p, uint32_t &nav, bool top,
                                                   int &status)
{
  int cand = vol;
  if (top) cand = shape_contains(g, pv_shape(g, vol), p) ? vol : -1;
  if (cand < 0) return -1;
  nav    = nav_push(g, nav, cand);
  int lv = g.pv_lv[cand];
  for (int level = 0; level < 256; ++level) {
    if (g.lv_nd[lv] == 0) return nav_top(g, nav);
    int pv = -1;
    V3 tp;
    if (!bvh_level_locate(g, lv, -1, p, pv, tp, status)) return nav_top(g, nav);
    nav  = nav_push(g, nav, pv);
    cand = nav_top(g, nav);
    lv   = g.pv_lv[cand];
    p    = tp;
  }
  status = kTrackErrIter;
  return nav_top(g, nav);
}

// GlobalLocator::LocateGlobalPointExclVolume with top = false (GlobalLocator.h:88-135)
__device__ __forceinline__ void locate_excl(const DevGeom &g, int vol, int excl, V3 p, uint32_t &nav, int &status)
{
  int cand = vol;
  nav      = nav_push(g, nav, cand);
  int lv   = g.pv_lv[cand];
  for (int level = 0; level < 256; ++level) {
    if (g.lv_nd[lv] == 0) return;
    V3 tp;
    if (!bvh_level_locate(g, lv, excl, p, cand, tp, status)) return;
    lv  = g.pv_lv[cand];
    p   = tp;
    nav = nav_push(g, nav, cand);
  }
  status = kTrackErrIter;
}

// GlobalLocator::RelocatePointFromPathForceDifferent (GlobalLocator.h:171-200)
__device__ __forceinline__ void relocate_force_different(const DevGeom &g, V3 lp, uint32_t &nav, int &status)
{
  int cur         = nav_top(g, nav);
  const int entry = cur;
  if (cur < 0) return;
  for (int level = 0; level < 256 && cur >= 0; ++level) {
    if (cur == entry || !shape_contains(g, pv_shape(g, cur), lp)) {
      nav = nav_pop(g, nav);
      lp  = to_master(g.pv_xf[cur], lp);
      cur = nav_top(g, nav);
    } else {
      nav = nav_pop(g, nav);
      locate_excl(g, cur, entry, lp, nav, status);
      return;
    }
  }
}

// AABB::Safety (VecGeom/base/AABB.h:81): max over axes of |p - centre| - half size, with
// centre = 0.5 (max + min) and half size = 0.5 (max - min) as the reference forms them.
__device__ __forceinline__ double aabb_safety(const double *b, V3 p)
{
  const double cx = 0.5 * (__ldg(b + 3) + __ldg(b)), cy = 0.5 * (__ldg(b + 4) + __ldg(b + 1));
  const double cz = 0.5 * (__ldg(b + 5) + __ldg(b + 2));
  const double hx = 0.5 * (__ldg(b + 3) - __ldg(b)), hy = 0.5 * (__ldg(b + 4) - __ldg(b + 1));
  const double hz = 0.5 * (__ldg(b + 5) - __ldg(b + 2));
  return max3(fabs(p.x - cx) - hx, fabs(p.y - cy) - hy, fabs(p.z - cz) - hz);
}

// BVH::ComputeSafety (VecGeom/base/BVH.h:172-209): minimum of `safety` and the SafetyToIn of
// every daughter whose box is closer than the current minimum.
__device__ __forceinline__ double bvh_compute_safety(const DevGeom &g, int lv, V3 lp, double safety, int &status)
{
  const int b     = g.lv_bvh[lv];
  const int node0 = g.bvh_node0[b];
  const int dbase = g.lv_dstart[lv];
  unsigned stack[32];
  int sp   = 1;
  stack[0] = 0;
  do {
    const unsigned id = stack[--sp];
    const int nch     = __ldg(&g.node_nchild[node0 + id]);
    if (nch >= 0) {
      const int off = __ldg(&g.node_offset[node0 + id]);
      for (int i = 0; i < nch; ++i) {
        const int prim = __ldg(&g.prim_id[off + i]);
        if (dlt(aabb_safety(g.prim_box + 6 * (size_t)(dbase + prim), lp), safety)) {
          const int vol     = __ldg(&g.daughters[dbase + prim]);
          const double dist = shape_safety_in(g, pv_shape(g, vol), to_local(g.pv_xf[vol], lp));
          if (dlt(dist, safety)) safety = dist;
        }
      }
    } else {
      if (sp + 2 > 32) {
        status = kTrackErrStack;
        return safety;
      }
      const unsigned cl = 2 * id + 1, cr = 2 * id + 2;
      const double sl = aabb_safety(g.node_box + 6 * (size_t)(node0 + cl), lp);
      const double sr = aabb_safety(g.node_box + 6 * (size_t)(node0 + cr), lp);
      const bool tl = dlt(sl, safety), tr = dlt(sr, safety);
      if (dlt(sr, sl)) {
        if (tr) stack[sp++] = cr;
        if (tl) stack[sp++] = cl;
      } else {
        if (tl) stack[sp++] = cl;
        if (tr) stack[sp++] = cr;
      }
    }
  } while (sp > 0);
  return safety;
}

// Safety part of ComputeStepAndSafetyAndPropagatedState (VNavigator.h:1014-1064) with
// BVHSafetyEstimator::ComputeSafetyForLocalPoint (BVHSafetyEstimator.h:38-46): the mother's
// SafetyToOut, lowered by the daughters' SafetyToIn when positive.
__device__ __forceinline__ double safety_of_state(const DevGeom &g, V3 gp, uint32_t navInd, int &status)
{
  if (navInd == 0) {
    status = kTrackErrState;
    return 0.;
  }
  const Xform m = nav_top_matrix(g, navInd);
  const V3 lp   = to_local(m, gp);
  const int lv  = g.pv_lv[nav_top(g, navInd)];
  double safety = shape_safety_out(g, g.lv_shape[lv], lp);
  if (dgt(safety, 0.0) && g.lv_nd[lv] > 0) safety = bvh_compute_safety(g, lv, lp, safety, status);
  return safety;
}

// VNavigatorHelper<BVHNavigator<false>>::ComputeStepAndPropagatedState (VNavigator.h:436-492)
__device__ __forceinline__ double compute_step(const DevGeom &g, V3 gp, V3 gd, double limit, NavState const &in,
                                               NavState &out, int &status, int *nvisited)
{
  out    = in;
  status = kTrackOk;
  if (in.navInd == 0) {
    status = kTrackErrState;
    return 0.;
  }
  const Xform m = nav_top_matrix(g, in.navInd);
  const V3 lp   = to_local(m, gp);
  const V3 ld   = rotate(m, gd);
  const int pv  = nav_top(g, in.navInd);
  const int lv  = g.pv_lv[pv];
  double step   = shape_dist_out(g, g.lv_shape[lv], lp, ld);
  if (dlt(step, 0.)) step = 0.;
  int hit = -1;
  if (g.lv_nd[lv] > 0) {
    const int last = nav_top(g, in.lastExited);
    status         = bvh_check_daughters(g, lv, lp, ld, step, last, hit, nvisited);
    if (status != kTrackOk) return 0.;
  }
  // PrepareOutState (VNavigator.h:192-235)
  if (deq(step, kInfLength) && dgt(limit, 0.)) {
    out.onBoundary = 1;
    out.navInd     = nav_pop(g, out.navInd);
    return kTolerance;
  }
  if (dgt(step, limit)) {
    out.onBoundary = 0;
    return limit;
  }
  out.onBoundary = 1;
  out.lastExited = out.navInd;
  if (hit >= 0) out.navInd = nav_push(g, out.navInd, hit);
  if (dlt(step, 0.)) step = 0.;
  // Relocate(MovePointAfterBoundary(...)) (VNavigator.h:168-173, 1070-1091)
  const double s = step + 1E-6;
  const V3 after{lp.x + s * ld.x, lp.y + s * ld.y, lp.z + s * ld.z};
  if (hit < 0) {
    relocate_force_different(g, after, out.navInd, status);
  } else {
    out.navInd = nav_pop(g, out.navInd);
    locate_global_point(g, hit, to_local(g.pv_xf[hit], after), out.navInd, false, status);
  }
  return step;
}

} // namespace f64
} // namespace vg
