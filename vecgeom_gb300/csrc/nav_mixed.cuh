// Mixed-precision navigator (VG_PREC_MIXED). The reference algorithm and its FP64
// arithmetic decide every result: the global-to-local transform, the mother's
// DistanceToOut, the DistanceToIn of every daughter that can still win, and every
// relocation Contains that is not certain. FP32 is used only to prune work that cannot
// change the result:
//   * BVH node and daughter boxes are tested in FP32 against copies inflated by kBoxPad
//     (rounded outward), so a box the FP64 test enters is always entered;
//   * each daughter surviving the box test gets an FP32 lower bound of its DistanceToIn
//     from a conservative descriptor of its shape (bounding box, or cylindrical shell for
//     tubes/cones/polycones/tori); only daughters whose bound is below the current step get
//     the exact FP64 DistanceToIn, lowest bound first, so the step shrinks as early as it can;
//   * Contains in relocation is decided in FP32 when the point is farther than kBoxPad from
//     the descriptor's boundary, else in FP64.
// A lower bound never exceeds the FP64 distance and a certain decision never disagrees
// with FP64, so out-states and steps equal the FP64 path's; only exact ties between two
// daughters could resolve differently (both sides keep the first one they evaluate).
#pragma once
#include "nav_fp64.cuh"

namespace vg {
namespace mixed {

#if VG_FP64_INT_COMPARE // (otherwise these names are macros)
using f64::deq;
using f64::dgt;
using f64::dle;
using f64::dlt;
#endif

using f64::V3;

// Pad (mm) added to every FP32 box/descriptor on each side. FP32 rounding of coordinates
// up to 4 m is <= 2.4e-4 mm, and slab parameters carry <= ~1e-6 relative error, so a 4 um
// pad keeps every FP32 inclusion test a superset of the FP64 one.
constexpr float kBoxPad = 4e-3f;
// Relative shrink applied to every FP32 lower bound (covers the FP32 rounding of the
// quotient and square-root chains; 2^-16 is ~500 FP32 ulps).
constexpr float kLbRel = 1.52587890625e-5f;

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(V3 v) { return F3{(float)v.x, (float)v.y, (float)v.z}; }

// Descriptor of a shape for FP32 bounds (host-built, 8 floats):
//   kind 0: box lo[3], hi[3] (extent, local frame), flag: box is the shape itself
//   kind 1: cylindrical shell rmin, rmax, zlo, zhi (local frame), flag: shell is the shape
struct ShapeLB {
  float kind, flag, a0, a1, a2, a3, a4, a5;
};

__device__ __forceinline__ float inv_dir(float d) { return 1.0f / (d + copysignf(1e-30f, d)); }

// FP32 slab interval of a box padded by kBoxPad.
__device__ __forceinline__ void slab_f(const float *lo, const float *hi, F3 p, F3 inv, float &tmin, float &tmax)
{
  float t0x = (lo[0] - kBoxPad - p.x) * inv.x, t1x = (hi[0] + kBoxPad - p.x) * inv.x;
  float t0y = (lo[1] - kBoxPad - p.y) * inv.y, t1y = (hi[1] + kBoxPad - p.y) * inv.y;
  float t0z = (lo[2] - kBoxPad - p.z) * inv.z, t1z = (hi[2] + kBoxPad - p.z) * inv.z;
  tmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
  tmax = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
}
__device__ __forceinline__ bool box_contains_f(const float *lo, const float *hi, F3 p)
{
  return p.x >= lo[0] - kBoxPad && p.x <= hi[0] + kBoxPad && p.y >= lo[1] - kBoxPad && p.y <= hi[1] + kBoxPad &&
         p.z >= lo[2] - kBoxPad && p.z <= hi[2] + kBoxPad;
}

// Lower bound of DistanceToIn for a shell rmin <= r <= rmax, zlo <= z <= zhi (already
// padded) from p along unit d; +inf when the ray certainly misses.
__device__ __forceinline__ float shell_lb(float rmin, float rmax, float zlo, float zhi, F3 p, F3 d)
{
  // z slab
  float tz = 0.f;
  if (p.z < zlo) {
    if (d.z <= 0.f) return INFINITY;
    tz = (zlo - p.z) / d.z;
  } else if (p.z > zhi) {
    if (d.z >= 0.f) return INFINITY;
    tz = (zhi - p.z) / d.z;
  }
  // radial
  const float a  = fmaf(d.x, d.x, d.y * d.y);
  const float b  = fmaf(p.x, d.x, p.y * d.y);
  const float r2 = fmaf(p.x, p.x, p.y * p.y);
  float tr       = 0.f;
  if (r2 > rmax * rmax) {
    const float c   = r2 - rmax * rmax;
    const float err = (r2 + rmax * rmax) * 1e-6f + 1e-6f;
    if (b >= 0.f && c > err) return INFINITY; // outside and not approaching the axis
    const float disc = fmaf(b, b, -a * c);
    const float derr = (b * b + a * (r2 + rmax * rmax)) * 1e-6f + 1e-12f;
    if (disc + derr < 0.f) return INFINITY;
    if (a <= 0.f) return 0.f;
    tr = (-b - sqrtf(disc + derr)) / (a * (1.f + 1e-6f));
  } else if (rmin > 0.f && r2 < rmin * rmin) {
    const float c    = r2 - rmin * rmin; // < 0
    const float disc = fmaf(b, b, -a * c);
    const float derr = (b * b + a * (r2 + rmin * rmin)) * 1e-6f + 1e-12f;
    const float dl   = fmaxf(disc - derr, 0.f);
    if (a <= 1e-30f) return INFINITY;
    tr = (-b + sqrtf(dl)) / (a * (1.f + 1e-6f));
  }
  return fmaxf(fmaxf(tz, tr), 0.f) * (1.f - kLbRel) - kBoxPad;
}

// Lower bound of DistanceToIn of a placed daughter (p, d in the mother frame). The
// daughter's frame offset (p - t) is formed in FP64, the rotation in FP32.
//
// `ub` receives an upper bound of the FP64 DistanceToIn when one is certain, else +inf. It
// is given for daughters whose shape is their box: if the FP32 ray crosses the box shrunk
// by 2 kBoxPad over a parameter interval [t0, t1] with t0 > 0, then the FP64 ray (within
// kBoxPad of the FP32 one) is strictly inside the box at t0, so the box's DistanceToIn is a
// hit (entry before exit, exit ahead, the far planes ahead by more than kHalfTolerance) at a
// distance <= t0; the bound adds the FP32 rounding of t0 and 1 um.
// The record of a prim slot: box and placed volume (first 32 bytes).
__device__ __forceinline__ void leaf_box(const LeafRec *rp, float lo[3], float hi[3], int &pv)
{
  const float4 a = __ldg(reinterpret_cast<const float4 *>(rp));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(rp) + 1);
  lo[0] = a.x, lo[1] = a.y, lo[2] = a.z, hi[0] = a.w, hi[1] = b.x, hi[2] = b.y;
  pv = __float_as_int(b.z);
}
__device__ __forceinline__ ShapeLB leaf_lb(const LeafRec *rp)
{
  const float4 a = __ldg(reinterpret_cast<const float4 *>(rp) + 2);
  const float4 b = __ldg(reinterpret_cast<const float4 *>(rp) + 3);
  return ShapeLB{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}
// The daughter-frame point and direction in FP32: pf - t and the rotation in FP32 from the
// FP32 mother-frame point pf and direction df (each converted once per traversal: a
// double/float conversion takes an FP64-pipe slot on GB300). With |p|, |t| <= kMaxCoord
// (4 m) the FP32 rounding of pf, t and the difference is at most 3 * 2^-24 * 4000 mm =
// 7.2e-4 mm per component and the FP32 rotation adds at most ~1.2e-3 mm, within kBoxPad.
__device__ __forceinline__ F3 leaf_local_point(const LeafRec *rp, F3 pf)
{
  const F3 q{pf.x - __ldg(&rp->t[0]), pf.y - __ldg(&rp->t[1]), pf.z - __ldg(&rp->t[2])};
  const float *r = rp->r;
  return F3{fmaf(q.x, __ldg(r + 0), fmaf(q.y, __ldg(r + 3), q.z * __ldg(r + 6))),
            fmaf(q.x, __ldg(r + 1), fmaf(q.y, __ldg(r + 4), q.z * __ldg(r + 7))),
            fmaf(q.x, __ldg(r + 2), fmaf(q.y, __ldg(r + 5), q.z * __ldg(r + 8)))};
}
__device__ __forceinline__ F3 leaf_local_dir(const LeafRec *rp, F3 dd)
{
  const float *r = rp->r;
  return F3{fmaf(dd.x, __ldg(r + 0), fmaf(dd.y, __ldg(r + 3), dd.z * __ldg(r + 6))),
            fmaf(dd.x, __ldg(r + 1), fmaf(dd.y, __ldg(r + 4), dd.z * __ldg(r + 7))),
            fmaf(dd.x, __ldg(r + 2), fmaf(dd.y, __ldg(r + 5), dd.z * __ldg(r + 8)))};
}
__device__ __forceinline__ bool f32_coord_ok(F3 l)
{
  return fabsf(l.x) <= 4000.f && fabsf(l.y) <= 4000.f && fabsf(l.z) <= 4000.f;
}

// The record of placed volume pv (two 16-byte loads).
__device__ __forceinline__ PvRec pv_rec(const DevGeom &g, int pv)
{
  const int4 a = __ldg(reinterpret_cast<const int4 *>(g.pv_rec + pv));
  const int4 b = __ldg(reinterpret_cast<const int4 *>(g.pv_rec + pv) + 1);
  return PvRec{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

__device__ __forceinline__ float daughter_lb(const LeafRec *rp, F3 pf, F3 df, float &ub)
{
  ub = INFINITY;
  if (__ldg(&rp->exact_only)) return -INFINITY;
  const F3 lp     = leaf_local_point(rp, pf);
  const F3 ld     = leaf_local_dir(rp, df);
  const ShapeLB s = leaf_lb(rp);
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    const F3 inv{inv_dir(ld.x), inv_dir(ld.y), inv_dir(ld.z)};
    float tmin, tmax;
    slab_f(lo, hi, lp, inv, tmin, tmax);
    if (!(tmin <= tmax) || tmax < 0.f) return INFINITY;
    if (tmin <= 0.f) return -INFINITY; // inside the padded box: the distance may be <= 0
    if (s.flag != 0.f) {
      // slab of the box shrunk by 2 kBoxPad (slab_f pads by kBoxPad, so shrink by 3 kBoxPad)
      const float ls[3] = {lo[0] + 3.f * kBoxPad, lo[1] + 3.f * kBoxPad, lo[2] + 3.f * kBoxPad};
      const float hs[3] = {hi[0] - 3.f * kBoxPad, hi[1] - 3.f * kBoxPad, hi[2] - 3.f * kBoxPad};
      if (ls[0] < hs[0] && ls[1] < hs[1] && ls[2] < hs[2]) {
        float t0, t1;
        slab_f(ls, hs, lp, inv, t0, t1);
        const float u = fmaf(t0, 1.f + 2.f * kLbRel, 1e-3f);
        if (t0 > 0.f && t1 * (1.f - 2.f * kLbRel) > u) ub = u;
      }
    }
    return tmin * (1.f - kLbRel) - kBoxPad;
  }
  const float rmin = fmaxf(s.a0 - kBoxPad, 0.f), rmax = s.a1 + kBoxPad;
  const float zlo = s.a2 - kBoxPad, zhi = s.a3 + kBoxPad;
  const float r2  = fmaf(lp.x, lp.x, lp.y * lp.y);
  if (lp.z >= zlo && lp.z <= zhi && r2 <= rmax * rmax && r2 >= rmin * rmin) return -INFINITY;
  return shell_lb(rmin, rmax, zlo, zhi, lp, ld);
}

// Contains with an FP32 certain-outside / certain-inside test before the FP64 one.
// Returns the daughter-local FP64 point in `lp` when it returns true.
__device__ __forceinline__ bool pv_contains_mixed(const DevGeom &g, const LeafRec *rp, int pv, V3 p, F3 pf, V3 &lp)
{
  const Xform &m = g.pv_xf[pv];
  if (__ldg(&rp->exact_only)) {
    lp = f64::to_local(m, p);
    return f64::shape_contains_to(g, __ldg(&rp->type), __ldg(&rp->off), lp);
  }
  const F3 l      = leaf_local_point(rp, pf);
  const ShapeLB s = leaf_lb(rp);
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    if (!box_contains_f(lo, hi, l)) return false;
    if (s.flag != 0.f && l.x > lo[0] + kBoxPad && l.x < hi[0] - kBoxPad && l.y > lo[1] + kBoxPad &&
        l.y < hi[1] - kBoxPad && l.z > lo[2] + kBoxPad && l.z < hi[2] - kBoxPad) {
      lp = f64::to_local(m, p);
      return true;
    }
  } else {
    const float r2 = fmaf(l.x, l.x, l.y * l.y);
    const float ro = s.a1 + kBoxPad, ri = fmaxf(s.a0 - kBoxPad, 0.f);
    if (l.z < s.a2 - kBoxPad || l.z > s.a3 + kBoxPad || r2 > ro * ro || r2 < ri * ri) return false;
    const float ro_in = s.a1 - kBoxPad, ri_in = s.a0 + kBoxPad;
    if (s.flag != 0.f && l.z > s.a2 + kBoxPad && l.z < s.a3 - kBoxPad && r2 < ro_in * ro_in && r2 > ri_in * ri_in) {
      lp = f64::to_local(m, p);
      return true;
    }
  }
  lp = f64::to_local(m, p);
  return f64::shape_contains_to(g, __ldg(&rp->type), __ldg(&rp->off), lp);
}

// Out-of-line FP64 fallbacks for points beyond the FP32 range (rare: keeps their code out of
// the hot loop).
static __device__ __noinline__ int check_daughters_far(const DevGeom &g, int lv, V3 lp, V3 ld, double &step,
                                                       int last_pv, int &hit_pv, int *nvisited)
{
  return f64::bvh_check_daughters(g, lv, lp, ld, step, last_pv, hit_pv, nvisited);
}
static __device__ __noinline__ bool level_locate_far(const DevGeom &g, int lv, int excl_pv, V3 lp, int &pv, V3 &dlp,
                                                     int &status)
{
  return f64::bvh_level_locate(g, lv, excl_pv, lp, pv, dlp, status);
}

// Second pass of check_daughters_mixed (rare, out of line to keep the step kernel's body
// small): traverses the whole tree again under the current bound and evaluates in FP64, at
// once, every candidate whose lower bound lies from `floor_lb` (the lowest bound the first
// pass left out of its full buffer; every lower bound the first pass kept and evaluated is
// at most that) up to the bound. A kept candidate with a bound equal to floor_lb is
// evaluated again, which cannot change the result.
static __device__ __noinline__ int check_daughters_second_pass(const DevGeom &g, int node0, V3 lp, V3 ld, F3 pf, F3 ldf,
                                                              F3 inv, float floor_lb, int last_pv, double &step,
                                                              float &bound, int &hit_pv, int &visits)
{
  unsigned stack[32];
  int sp   = 1;
  stack[0] = 0;
  do {
    const unsigned id = stack[--sp];
    ++visits;
    const NodeF nd = g.node_f[node0 + id];
    if (nd.nchild >= 0) {
      for (int i = 0; i < nd.nchild; ++i) {
        const int slot    = nd.offset + i;
        const LeafRec *rp = g.leaf_rec + slot;
        float blo[3], bhi[3];
        int vol;
        leaf_box(rp, blo, bhi, vol);
        float tmin, tmax;
        slab_f(blo, bhi, pf, inv, tmin, tmax);
        if (!(tmin <= tmax && tmax >= 0.f && tmin < bound)) continue;
        float ub;
        const float lb = daughter_lb(rp, pf, ldf, ub);
        if (!(lb < bound) || lb < floor_lb) continue;
        const Xform &m    = g.pv_xf[vol];
        const double dist =
            f64::shape_dist_in_to(g, __ldg(&rp->type), __ldg(&rp->off), f64::to_local(m, lp), f64::rotate(m, ld));
        if (dlt(dist, step) && !(dle(dist, 0.0) && vol == last_pv)) {
          step   = dist;
          hit_pv = vol;
          bound  = fminf(bound, __double2float_ru(step));
        }
      }
    } else {
      const unsigned cl_ = 2 * id + 1, cr_ = 2 * id + 2;
      const NodeF L = g.node_f[node0 + cl_], R = g.node_f[node0 + cr_];
      float tminL, tmaxL, tminR, tmaxR;
      slab_f(L.lo, L.hi, pf, inv, tminL, tmaxL);
      slab_f(R.lo, R.hi, pf, inv, tminR, tmaxR);
      if (sp + 2 > 32) return kTrackErrStack;
      if (tminL <= tmaxL && tmaxL >= 0.f && tminL < bound) stack[sp++] = cl_;
      if (tminR <= tmaxR && tmaxR >= 0.f && tminR < bound) stack[sp++] = cr_;
    }
  } while (sp > 0);
  return kTrackOk;
}

// BVH::CheckDaughterIntersections with FP32 pruning (see file comment). Candidates wait in
// a small buffer sorted by lower bound and are evaluated in FP64 at the end of the
// traversal, lowest bound first, each evaluation tightening the step and dropping every
// candidate that can no longer win. A full buffer keeps the kCandBuf lowest bounds and
// remembers the lowest bound it left out; if that one is still below the step once the
// buffer is evaluated, a second traversal evaluates every candidate from there up to the
// step directly. (Evaluating the lowest buffered candidate as soon as the buffer filled, as
// before, ran FP64 evaluations of far candidates in the middle of the traversal for tracks
// whose daughters' boxes all contain them, such as the world volume's nested layers.)
constexpr int kCandBuf = 8;

__device__ __forceinline__ int check_daughters_mixed(const DevGeom &g, int lv, int node0, V3 lp, V3 ld, double &step,
                                                     int last_pv, int &hit_pv, int *nvisited, int first = -1)
{
  const F3 pf = f3(lp);
  // beyond the range the FP32 pad covers, the exact FP64 traversal decides alone
  if (!f32_coord_ok(pf)) return check_daughters_far(g, lv, lp, ld, step, last_pv, hit_pv, nvisited);
  const F3 ldf    = f3(ld);
  const F3 inv{inv_dir(ldf.x), inv_dir(ldf.y), inv_dir(ldf.z)};
  float bound = __double2float_ru(step);
  float cl[kCandBuf] = {};
  int cp[kCandBuf]   = {}; // prim slots of the candidates
  int nc = 0;
  auto evaluate = [&](int slot) {
    const LeafRec *rp = g.leaf_rec + slot;
    const int vol     = __ldg(&rp->pv);
    const Xform &m    = g.pv_xf[vol];
    const double dist =
        f64::shape_dist_in_to(g, __ldg(&rp->type), __ldg(&rp->off), f64::to_local(m, lp), f64::rotate(m, ld));
    if (dlt(dist, step) && !(dle(dist, 0.0) && vol == last_pv)) {
      step   = dist;
      hit_pv = vol;
      bound  = fminf(bound, __double2float_ru(step));
      while (nc > 0 && cl[nc - 1] >= bound) --nc;
    }
  };
  auto evaluate_first = [&]() {
    const float lb = cl[0];
    const int slot = cp[0];
    for (int k = 1; k < nc; ++k) cl[k - 1] = cl[k], cp[k - 1] = cp[k];
    --nc;
    if (lb >= bound) {
      nc = 0;
      return;
    }
    evaluate(slot);
  };
  float dropped = INFINITY; // lowest lower bound left out of the full buffer
  auto add = [&](float lb, int slot) {
    if (!(lb < bound)) return;
    if (nc == kCandBuf) {
      if (lb >= cl[nc - 1]) {
        dropped = fminf(dropped, lb);
        return;
      }
      dropped = fminf(dropped, cl[nc - 1]);
      --nc;
    }
    int k = nc++;
    while (k > 0 && cl[k - 1] > lb) cl[k] = cl[k - 1], cp[k] = cp[k - 1], --k;
    cl[k] = lb, cp[k] = slot;
  };
  unsigned stack[32];
  int sp     = 1;
  stack[0]   = 0;
  int visits = 0;
  // Learned proposal: explore depth-3 subtree `first` before the rest (and not again), so
  // the upper bounds of its daughters tighten the bound for the remaining traversal. Exact
  // FP64 evaluations still wait for the end of the traversal, where the lanes of a warp
  // reach them together.
  unsigned skip = 0xffffffffu;
  if (first >= 0) {
    skip     = 7u + (unsigned)first;
    stack[1] = skip;
    sp       = 2;
  }
  do {
    const unsigned id = stack[--sp];
    ++visits;
    const NodeF nd = g.node_f[node0 + id];
    if (nd.nchild >= 0) {
      for (int i = 0; i < nd.nchild; ++i) {
        const int slot    = nd.offset + i;
        const LeafRec *rp = g.leaf_rec + slot;
        float blo[3], bhi[3];
        int vol;
        leaf_box(rp, blo, bhi, vol);
        float tmin, tmax;
        slab_f(blo, bhi, pf, inv, tmin, tmax);
        if (tmin <= tmax && tmax >= 0.f && tmin < bound) {
          float ub;
          const float lb = daughter_lb(rp, pf, ldf, ub);
          add(lb, slot);
          // a certain upper bound of this daughter's distance bounds the step: whatever
          // starts beyond it can no longer be the first hit
          if (ub < bound && vol != last_pv) {
            bound = ub;
            while (nc > 0 && cl[nc - 1] >= bound) --nc;
          }
        }
      }
    } else {
      const unsigned cl_ = 2 * id + 1, cr_ = 2 * id + 2;
      const NodeF L = g.node_f[node0 + cl_], R = g.node_f[node0 + cr_];
      float tminL, tmaxL, tminR, tmaxR;
      slab_f(L.lo, L.hi, pf, inv, tminL, tmaxL);
      slab_f(R.lo, R.hi, pf, inv, tminR, tmaxR);
      const bool tl = tminL <= tmaxL && tmaxL >= 0.f && tminL < bound && cl_ != skip;
      const bool tr = tminR <= tmaxR && tmaxR >= 0.f && tminR < bound && cr_ != skip;
      if (sp + 2 > 32) {
        if (nvisited) *nvisited = visits;
        return kTrackErrStack;
      }
      if (tminR < tminL) {
        if (tr) stack[sp++] = cr_;
        if (tl) stack[sp++] = cl_;
      } else {
        if (tl) stack[sp++] = cl_;
        if (tr) stack[sp++] = cr_;
      }
    }
  } while (sp > 0);
  while (nc > 0) evaluate_first();
  if (dropped < bound) { // the candidates left out of the full buffer may still win
    const int st = check_daughters_second_pass(g, node0, lp, ld, pf, ldf, inv, dropped, last_pv, step, bound, hit_pv,
                                               visits);
    if (st != kTrackOk) {
      if (nvisited) *nvisited = visits;
      return st;
    }
  }
  if (nvisited) *nvisited = visits;
  return kTrackOk;
}

// BVH::LevelLocate with FP32 box tests (padded) and mixed Contains.
__device__ __forceinline__ bool level_locate_mixed(const DevGeom &g, int lv, int node0, int excl_pv, V3 lp, int &pv,
                                                   V3 &dlp, int &status)
{
  const F3 pf = f3(lp);
  if (!f32_coord_ok(pf)) return level_locate_far(g, lv, excl_pv, lp, pv, dlp, status);
  unsigned stack[32];
  int sp   = 1;
  stack[0] = 0;
  do {
    const unsigned id = stack[--sp];
    const NodeF nd    = g.node_f[node0 + id];
    if (nd.nchild >= 0) {
      for (int i = 0; i < nd.nchild; ++i) {
        const LeafRec *rp = g.leaf_rec + (nd.offset + i);
        float blo[3], bhi[3];
        int vol;
        leaf_box(rp, blo, bhi, vol);
        if (box_contains_f(blo, bhi, pf)) {
          if (vol != excl_pv && pv_contains_mixed(g, rp, vol, lp, pf, dlp)) {
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
      const NodeF L = g.node_f[node0 + cl], R = g.node_f[node0 + cr];
      if (box_contains_f(L.lo, L.hi, pf)) stack[sp++] = cl;
      if (box_contains_f(R.lo, R.hi, pf)) stack[sp++] = cr;
    }
  } while (sp > 0);
  return false;
}

// Contains of placed volume `pv`'s own shape (mother frame of its daughters) with the FP32
// certain-outside / certain-inside tests first.
__device__ __forceinline__ bool shape_contains_mixed(const DevGeom &g, const ShapeLB *lbs, const PvRec &r, V3 p)
{
  const ShapeLB s = lbs[r.shape];
  const F3 l      = f3(p);
  if (!f32_coord_ok(l)) return f64::shape_contains_to(g, r.type, r.off, p);
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    if (!box_contains_f(lo, hi, l)) return false;
    if (s.flag != 0.f && l.x > lo[0] + kBoxPad && l.x < hi[0] - kBoxPad && l.y > lo[1] + kBoxPad &&
        l.y < hi[1] - kBoxPad && l.z > lo[2] + kBoxPad && l.z < hi[2] - kBoxPad)
      return true;
  } else {
    const float r2 = fmaf(l.x, l.x, l.y * l.y);
    const float ro = s.a1 + kBoxPad, ri = fmaxf(s.a0 - kBoxPad, 0.f);
    if (l.z < s.a2 - kBoxPad || l.z > s.a3 + kBoxPad || r2 > ro * ro || r2 < ri * ri) return false;
    const float ro_in = s.a1 - kBoxPad, ri_in = s.a0 + kBoxPad;
    if (s.flag != 0.f && l.z > s.a2 + kBoxPad && l.z < s.a3 - kBoxPad && r2 < ro_in * ro_in && r2 > ri_in * ri_in)
      return true;
  }
  return f64::shape_contains_to(g, r.type, r.off, p);
}

// NavIndex push with the child index already known (NavStateIndex::PushImpl)
__device__ __forceinline__ uint32_t nav_push_child(const DevGeom &g, uint32_t n, int child)
{
  return n > 0 ? __ldg(&g.nav[n + 3 + child]) : 1u;
}

__device__ __forceinline__ int locate_global_point_mixed(const DevGeom &g, const ShapeLB *lbs, int vol, V3 p,
                                                         uint32_t &nav, bool top, int &status)
{
  int cand  = vol;
  PvRec rec = pv_rec(g, vol);
  if (top) cand = shape_contains_mixed(g, lbs, rec, p) ? vol : -1;
  if (cand < 0) return -1;
  nav = nav_push_child(g, nav, rec.child);
  for (int level = 0; level < 256; ++level) {
    if (rec.nd == 0) return f64::nav_top(g, nav);
    int pv = -1;
    V3 tp;
    if (!level_locate_mixed(g, rec.lv, rec.node0, -1, p, pv, tp, status)) return f64::nav_top(g, nav);
    rec = pv_rec(g, pv);
    nav = nav_push_child(g, nav, rec.child);
    p   = tp;
  }
  status = kTrackErrIter;
  return f64::nav_top(g, nav);
}

__device__ __forceinline__ void locate_excl_mixed(const DevGeom &g, int vol, int excl, V3 p, uint32_t &nav,
                                                  int &status)
{
  PvRec rec = pv_rec(g, vol);
  nav       = nav_push_child(g, nav, rec.child);
  for (int level = 0; level < 256; ++level) {
    if (rec.nd == 0) return;
    V3 tp;
    int cand = -1;
    if (!level_locate_mixed(g, rec.lv, rec.node0, excl, p, cand, tp, status)) return;
    rec = pv_rec(g, cand);
    p   = tp;
    nav = nav_push_child(g, nav, rec.child);
  }
  status = kTrackErrIter;
}

__device__ __forceinline__ void relocate_force_different_mixed(const DevGeom &g, const ShapeLB *lbs, V3 lp,
                                                               uint32_t &nav, int &status)
{
  int cur         = f64::nav_top(g, nav);
  const int entry = cur;
  if (cur < 0) return;
  for (int level = 0; level < 256 && cur >= 0; ++level) {
    if (cur == entry || !shape_contains_mixed(g, lbs, pv_rec(g, cur), lp)) {
      nav = f64::nav_pop(g, nav);
      lp  = f64::to_master(g.pv_xf[cur], lp);
      cur = f64::nav_top(g, nav);
    } else {
      nav = f64::nav_pop(g, nav);
      locate_excl_mixed(g, cur, entry, lp, nav, status);
      return;
    }
  }
}

// What a step leaves to its relocation (ComputeStepAndPropagatedState's last part): nothing,
// the exit through the mother (RelocatePoint), or the entry into the daughter pushed on the
// state (LocateGlobalPoint from it).
enum { kRelocNone = 0, kRelocExit = 1, kRelocEnter = 2 };

// ComputeStepAndPropagatedState with FP32 pruning (same control flow as f64::compute_step),
// up to the relocation: the returned step and `out` are final unless `reloc` is set, in
// which case relocate_after_step_mixed completes `out` (and may set `status`).
__device__ __forceinline__ double step_before_relocation_mixed(const DevGeom &g, V3 lp, V3 ld, double limit,
                                                               NavState const &in, NavState &out, int &status,
                                                               int *nvisited, int proposal, int &reloc)
{
  reloc           = kRelocNone;
  const int pv    = f64::nav_top(g, in.navInd);
  const PvRec rec = pv_rec(g, pv);
  double step     = f64::shape_dist_out_to(g, rec.type, rec.off, lp, ld);
  if (dlt(step, 0.)) step = 0.;
  int hit = -1;
  if (rec.nd > 0) {
    const int last = f64::nav_top(g, in.lastExited);
    int first = -1; // the proposal applies to BVHs of depth >= 3 whose depth-3 node is reachable
    if (proposal >= 0 && proposal < 8 && rec.depth >= 3) {
      int n   = 7 + proposal;
      bool ok = true;
      for (int d = 0; d < 3; ++d) {
        n  = (n - 1) >> 1;
        ok = ok && __ldg(&g.node_nchild[rec.node0 + n]) < 0;
      }
      if (ok) first = proposal;
    }
    status = check_daughters_mixed(g, rec.lv, rec.node0, lp, ld, step, last, hit, nvisited, first);
    if (status != kTrackOk) return 0.;
  }
  if (deq(step, kInfLength) && dgt(limit, 0.)) {
    out.onBoundary = 1;
    out.navInd     = f64::nav_pop(g, out.navInd);
    return kTolerance;
  }
  if (dgt(step, limit)) {
    out.onBoundary = 0;
    return limit;
  }
  out.onBoundary = 1;
  out.lastExited = out.navInd;
  if (hit >= 0) out.navInd = f64::nav_push(g, out.navInd, hit);
  if (dlt(step, 0.)) step = 0.;
  reloc = hit < 0 ? kRelocExit : kRelocEnter;
  return step;
}

// The point a step's relocation starts from: lp, ld and step as step_before_relocation_mixed
// saw and returned them (VNavigator.h:478-490, the point pushed 1e-6 mm past the boundary).
__device__ __forceinline__ V3 relocation_point(V3 lp, V3 ld, double step)
{
  const double s = step + 1E-6;
  return V3{lp.x + s * ld.x, lp.y + s * ld.y, lp.z + s * ld.z};
}

// The relocation of a step from its relocation point, `out` as step_before_relocation_mixed
// left it.
__device__ __forceinline__ void relocate_from_point_mixed(const DevGeom &g, const ShapeLB *lbs, V3 after, int reloc,
                                                          NavState &out, int &status)
{
  if (reloc == kRelocExit) {
    relocate_force_different_mixed(g, lbs, after, out.navInd, status);
  } else {
    const int hit = f64::nav_top(g, out.navInd);
    out.navInd    = f64::nav_pop(g, out.navInd);
    locate_global_point_mixed(g, lbs, hit, f64::to_local(g.pv_xf[hit], after), out.navInd, false, status);
  }
}

__device__ __forceinline__ void relocate_after_step_mixed(const DevGeom &g, const ShapeLB *lbs, V3 lp, V3 ld,
                                                          double step, int reloc, NavState &out, int &status)
{
  relocate_from_point_mixed(g, lbs, relocation_point(lp, ld, step), reloc, out, status);
}

__device__ __forceinline__ double compute_step_mixed(const DevGeom &g, const ShapeLB *lbs, V3 gp, V3 gd, double limit,
                                                     NavState const &in, NavState &out, int &status, int *nvisited,
                                                     int proposal = -1)
{
  out    = in;
  status = kTrackOk;
  if (in.navInd == 0) {
    status = kTrackErrState;
    return 0.;
  }
  const Xform m = f64::nav_top_matrix(g, in.navInd);
  const V3 lp   = f64::to_local(m, gp);
  const V3 ld   = f64::rotate(m, gd);
  int reloc;
  const double step = step_before_relocation_mixed(g, lp, ld, limit, in, out, status, nvisited, proposal, reloc);
  if (reloc != kRelocNone) relocate_after_step_mixed(g, lbs, lp, ld, step, reloc, out, status);
  return step;
}

} // namespace mixed
} // namespace vg
