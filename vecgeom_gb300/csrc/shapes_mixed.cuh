// Mixed-precision SoA shape queries (VG_PREC_MIXED on the vg_placed_* entry points). FP32
// on the shape's conservative descriptor (box or cylindrical shell, see nav_mixed.cuh)
// settles the cases it can prove, FP64 the rest:
//   * Inside / Contains: certainly outside the padded descriptor -> kOutside / false;
//     certainly inside a descriptor that is the shape itself, farther than the pad from its
//     boundary -> kInside / true (the surface band is 5e-10 mm, the pad 4e-3 mm);
//   * DistanceToIn: a point outside the padded descriptor box whose ray certainly misses
//     it -> kInfLength, the FP64 kernels' miss value;
//   * SafetyToIn / SafetyToOut of a Box: computed in FP32 and lowered by a proven bound of
//     its rounding error, so the result never exceeds the FP64 safety and lies at most
//     2^-21 (max|p| + max half-length) mm below it;
//   * everything else, and any point with a local coordinate beyond kMaxCoord, in FP64.
// Inside, Contains and the distances therefore equal the FP64 results exactly; only Box
// safeties differ, downwards, by a stated bound.
#pragma once
#include "nav_mixed.cuh"

namespace vg {
namespace mixed {

constexpr float kMaxCoord = 4000.f; // the pad covers FP32 rounding of coordinates up to 4 m

__device__ __forceinline__ bool in_range(F3 l)
{
  return fabsf(l.x) <= kMaxCoord && fabsf(l.y) <= kMaxCoord && fabsf(l.z) <= kMaxCoord;
}

// kOutside: certainly outside; kInside: certainly inside (and away from the surface);
// 0: undecided.
__device__ __forceinline__ int lb_classify(const ShapeLB &s, V3 p)
{
  const F3 l = f3(p);
  if (!in_range(l)) return 0;
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    if (!box_contains_f(lo, hi, l)) return kOutside;
    if (s.flag != 0.f && l.x > lo[0] + kBoxPad && l.x < hi[0] - kBoxPad && l.y > lo[1] + kBoxPad &&
        l.y < hi[1] - kBoxPad && l.z > lo[2] + kBoxPad && l.z < hi[2] - kBoxPad)
      return kInside;
    return 0;
  }
  const float r2 = fmaf(l.x, l.x, l.y * l.y);
  const float ro = s.a1 + kBoxPad, ri = fmaxf(s.a0 - kBoxPad, 0.f);
  if (l.z < s.a2 - kBoxPad || l.z > s.a3 + kBoxPad || r2 > ro * ro || r2 < ri * ri) return kOutside;
  const float ro_in = s.a1 - kBoxPad, ri_in = s.a0 + kBoxPad;
  if (s.flag != 0.f && l.z > s.a2 + kBoxPad && l.z < s.a3 - kBoxPad && r2 < ro_in * ro_in && r2 > ri_in * ri_in)
    return kInside;
  return 0;
}

// True when p lies outside the padded descriptor box and its ray certainly misses it.
__device__ __forceinline__ bool lb_certain_miss(const ShapeLB &s, V3 p, V3 d)
{
  const F3 l = f3(p);
  if (!in_range(l)) return false;
  float lo[3], hi[3];
  if (s.kind == 0.f) {
    lo[0] = s.a0, lo[1] = s.a1, lo[2] = s.a2, hi[0] = s.a3, hi[1] = s.a4, hi[2] = s.a5;
  } else {
    lo[0] = lo[1] = -s.a1, hi[0] = hi[1] = s.a1, lo[2] = s.a2, hi[2] = s.a3;
  }
  if (box_contains_f(lo, hi, l)) return false;
  const F3 dd = f3(d);
  const F3 inv{inv_dir(dd.x), inv_dir(dd.y), inv_dir(dd.z)};
  float tmin, tmax;
  slab_f(lo, hi, l, inv, tmin, tmax);
  return !(tmin <= tmax) || tmax < 0.f;
}

// ---------------------------------------------------------------- exact-shape FP32 tests
// Classification of a point (FP32, in the shape's frame, within kBoxPad / 2 of the exact
// FP64 local point) against the shape itself, not its descriptor: kInside when the point
// is farther than kBoxPad inside every surface, kOutside when it is farther than kBoxPad
// outside one of them, 0 otherwise. Every FP64 Inside/Contains decision of the reference
// uses tolerance bands of at most ~1e-8 mm, so a certain FP32 answer is the FP64 answer.
// The FP32 rounding of the compared quantities (radii from squares, linear profiles) is
// below 1e-3 mm for coordinates up to kMaxCoord, inside the pad.
__device__ __forceinline__ int f32_classify_desc(const ShapeLB &s, F3 l)
{
  if (!in_range(l)) return 0;
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    if (!box_contains_f(lo, hi, l)) return kOutside;
    if (s.flag != 0.f && l.x > lo[0] + kBoxPad && l.x < hi[0] - kBoxPad && l.y > lo[1] + kBoxPad &&
        l.y < hi[1] - kBoxPad && l.z > lo[2] + kBoxPad && l.z < hi[2] - kBoxPad)
      return kInside;
    return 0;
  }
  const float r2 = fmaf(l.x, l.x, l.y * l.y);
  const float ro = s.a1 + kBoxPad, ri = fmaxf(s.a0 - kBoxPad, 0.f);
  if (l.z < s.a2 - kBoxPad || l.z > s.a3 + kBoxPad || r2 > ro * ro || r2 < ri * ri) return kOutside;
  const float ro_in = s.a1 - kBoxPad, ri_in = s.a0 + kBoxPad;
  if (s.flag != 0.f && l.z > s.a2 + kBoxPad && l.z < s.a3 - kBoxPad && r2 < ro_in * ro_in && r2 > ri_in * ri_in)
    return kInside;
  return 0;
}
// phi wedge from its two along-vectors: signed distances to the two half-planes
__device__ __forceinline__ int f32_wedge(double dphi, double a1x, double a1y, double a2x, double a2y, F3 l)
{
  // the reference's sector tests switch form at dphi = pi (< in one place, <= in another):
  // an opening within 1e-12 of pi is left undecided
  if (fabs(dphi - kPi) < 1e-12) return 0;
  const float s1 = fmaf(-l.x, (float)a1y, l.y * (float)a1x);
  const float s2 = fmaf(-(float)a2x, l.y, (float)a2y * l.x);
  if (dphi <= kPi) {
    if (s1 > kBoxPad && s2 > kBoxPad) return kInside;
    if (s1 < -kBoxPad || s2 < -kBoxPad) return kOutside;
  } else {
    if (s1 > kBoxPad || s2 > kBoxPad) return kInside;
    if (s1 < -kBoxPad && s2 < -kBoxPad) return kOutside;
  }
  return 0;
}
// radial / z test of r against [rmin, rmax] (rmin 0: solid), |z| against dz
__device__ __forceinline__ int f32_rz(float r, float rmin, float rmax, float az, float dz)
{
  if (az > dz + kBoxPad || r > rmax + kBoxPad || (rmin > 0.f && r < rmin - kBoxPad)) return kOutside;
  if (az < dz - kBoxPad && r < rmax - kBoxPad && (rmin <= 0.f || r > rmin + kBoxPad)) return kInside;
  return 0;
}
template <class R>
__device__ __forceinline__ int f32_classify(const R &, const ShapeLB &s, F3 l)
{
  return f32_classify_desc(s, l);
}
__device__ __forceinline__ int f32_classify(const TubeRec &t, const ShapeLB &, F3 l)
{
  if (!in_range(l)) return 0;
  const int c = f32_rz(sqrtf(fmaf(l.x, l.x, l.y * l.y)), (float)t.rmin, (float)t.rmax, fabsf(l.z), (float)t.z);
  if (c == kOutside || t.dphi >= kTwoPi) return c;
  const int w = f32_wedge(t.dphi, t.a1x, t.a1y, t.a2x, t.a2y, l);
  if (w == kOutside) return kOutside;
  return (c == kInside && w == kInside) ? kInside : 0;
}
__device__ __forceinline__ int f32_classify(const ConeRec &c, const ShapeLB &, F3 l)
{
  if (!in_range(l)) return 0;
  // radii at z from the reference's linear profiles (ConeUtilities.h:113-131)
  const float rmax = c.origRmax1 == c.origRmax2 ? (float)c.origRmax1
                                                : fmaf((float)c.outerSlope, l.z, (float)c.outerOffset);
  const bool hasmin = c.rmin1 > 0 || c.rmin2 > 0;
  const float rmin  = !hasmin ? 0.f : (c.rmin1 == c.rmin2 ? (float)c.rmin1 : fmaf((float)c.innerSlope, l.z, (float)c.innerOffset));
  // a conical surface is closer than the radial difference; scale the pad by 1/cos of its
  // half-angle (|slope| <= 1e3 keeps the bound meaningful, steeper profiles stay undecided)
  const float so = fabsf((float)c.outerSlope), si = hasmin ? fabsf((float)c.innerSlope) : 0.f;
  if (so > 1e3f || si > 1e3f) return 0;
  const float k   = sqrtf(1.f + fmaxf(so, si) * fmaxf(so, si));
  const float r   = sqrtf(fmaf(l.x, l.x, l.y * l.y));
  const float az  = fabsf(l.z);
  const float pr  = kBoxPad * k;
  int cr;
  if (az > (float)c.dz + kBoxPad || r > rmax + pr || (hasmin && r < rmin - pr))
    cr = kOutside;
  else if (az < (float)c.dz - kBoxPad && r < rmax - pr && (!hasmin || r > rmin + pr))
    cr = kInside;
  else
    cr = 0;
  if (cr == kOutside || c.dphi >= kTwoPi) return cr;
  const int w = f32_wedge(c.dphi, c.a1x, c.a1y, c.a2x, c.a2y, l);
  if (w == kOutside) return kOutside;
  return (cr == kInside && w == kInside) ? kInside : 0;
}
__device__ __forceinline__ int f32_classify(const TrdRec &t, const ShapeLB &, F3 l)
{
  if (!in_range(l)) return 0;
  // perpendicular distances to the inclined faces, as TrdImplementation.h:288-300 forms them
  const float sx = ((float)t.halfx1plusx2 - (float)t.fx * l.z - fabsf(l.x)) * (float)t.calfx;
  const float sy = t.dy1 != t.dy2 ? ((float)t.halfy1plusy2 - (float)t.fy * l.z - fabsf(l.y)) * (float)t.calfy
                                  : (float)t.dy1 - fabsf(l.y);
  const float sz = (float)t.dz - fabsf(l.z);
  if (sx < -kBoxPad || sy < -kBoxPad || sz < -kBoxPad) return kOutside;
  if (sx > kBoxPad && sy > kBoxPad && sz > kBoxPad) return kInside;
  return 0;
}
// The FP64 DistanceToIn of a point certainly inside: -1 for Tube, Cone and Trd (their
// inside tests return before any distance); 0 (no shortcut) for the others.
template <class R>
__device__ __forceinline__ bool dist_in_inside_is_minus1() { return false; }
template <> __device__ __forceinline__ bool dist_in_inside_is_minus1<TubeRec>() { return true; }
template <> __device__ __forceinline__ bool dist_in_inside_is_minus1<ConeRec>() { return true; }
template <> __device__ __forceinline__ bool dist_in_inside_is_minus1<TrdRec>() { return true; }
// DistanceToOut of a point certainly outside is -1 for Box, Tube and Trd; for Cone only when
// it is outside in r or z (its scalar DistanceToOut does not reject by phi).
template <class R>
__device__ __forceinline__ bool dist_out_outside_is_minus1(const R &) { return false; }
__device__ __forceinline__ bool dist_out_outside_is_minus1(const BoxRec &) { return true; }
__device__ __forceinline__ bool dist_out_outside_is_minus1(const TubeRec &) { return true; }
__device__ __forceinline__ bool dist_out_outside_is_minus1(const TrdRec &) { return true; }
__device__ __forceinline__ bool dist_out_outside_is_minus1(const ConeRec &c) { return c.dphi >= kTwoPi; }

// True when the ray from l (outside the shape) certainly misses the padded descriptor.
__device__ __forceinline__ bool f32_certain_miss(const ShapeLB &s, F3 l, F3 d)
{
  if (!in_range(l)) return false;
  if (s.kind == 0.f) {
    const float lo[3] = {s.a0, s.a1, s.a2}, hi[3] = {s.a3, s.a4, s.a5};
    if (box_contains_f(lo, hi, l)) return false;
    const F3 inv{inv_dir(d.x), inv_dir(d.y), inv_dir(d.z)};
    float tmin, tmax;
    slab_f(lo, hi, l, inv, tmin, tmax);
    return !(tmin <= tmax) || tmax < 0.f;
  }
  const float rmin = fmaxf(s.a0 - kBoxPad, 0.f), rmax = s.a1 + kBoxPad;
  return shell_lb(rmin, rmax, s.a2 - kBoxPad, s.a3 + kBoxPad, l, d) == INFINITY;
}

// Full-phi Tube safeties in FP32 (the SafetyToInOld / SafetyToOutOld forms of
// TubeImplementation.h:758-802 that tube_safety_in / tube_safety_out follow: the z term
// |z| - dz, the radial terms r - rmax and rmin - r, combined by max, or their negatives by
// min), lowered by a proven bound so that they never exceed the FP64 value. With u = 2^-24,
// inputs rounded to nearest, sqrtf and every FP32 operation correctly rounded:
// r32 = sqrtf(fmaf(x, x, y * y)) lies within 3.1 u r of r (u r from the inputs, 2 u from the
// sum and the root); each FP32 term within 4.2 u (R + D) of the exact one, R = max(r, |z|),
// D = max(dz, rmax) (r32's error, the rounding of the constant and of the subtraction); the
// FP64 terms within 2^-50 (R + D) of the exact ones. max and min are 1-Lipschitz, so the FP32
// safety s is within (4.2 u + 2^-50)(R + D) < 2^-21 (R + D) of the FP64 one, and
// s - 2^-21 (R + D) (bound rounded up, subtraction rounded down) never exceeds it and lies at
// most 2^-20 (R + D) below it. Phi sections keep the FP64 kernel. (The Box's FP64 safety
// is three subtractions; an FP32 form of it measured slower than that, so the Box keeps it.)
__device__ __forceinline__ double tube_safety_mixed(const TubeRec &t, V3 p, bool out)
{
  const float x = (float)p.x, y = (float)p.y, z = fabsf((float)p.z);
  const float r  = sqrtf(fmaf(x, x, y * y));
  const float dz = (float)t.z, rmax = (float)t.rmax, rmin = (float)t.rmin;
  const bool hasmin = f64::tube_rmin(t);
  float s;
  if (out) {
    s = fminf(dz - z, rmax - r);
    if (hasmin) s = fminf(s, r - rmin);
  } else {
    s = fmaxf(z - dz, r - rmax);
    if (hasmin) s = fmaxf(s, rmin - r);
  }
  const float m = __fadd_ru(fmaxf(r, z), fmaxf(dz, rmax));
  return (double)__fsub_rd(s, __fmul_ru(4.76837158203125e-07f, m));
}

} // namespace mixed
} // namespace vg
