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
//     3 * 2^-23 (max|p| + max half-length) mm below it;
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

// Box safeties in FP32, lowered by 2^-22 (max_k |p_k| + max_k half-length_k): each FP32
// term |p_k| - h_k carries at most 2^-23 (|p_k| + h_k) of rounding (inputs and the
// subtraction), max/min are 1-Lipschitz, and the factor 2 covers the FP64 reference's own
// rounding. The subtraction of the bound is done in FP64.
__device__ __forceinline__ double box_safety_mixed(const BoxRec &b, V3 p, bool out)
{
  const float x = fabsf((float)p.x), y = fabsf((float)p.y), z = fabsf((float)p.z);
  const float dx = (float)b.dx, dy = (float)b.dy, dz = (float)b.dz;
  const float s  = out ? fminf(fminf(dx - x, dy - y), dz - z) : fmaxf(fmaxf(x - dx, y - dy), z - dz);
  const double bound = 2.384185791015625e-07 * ((double)fmaxf(fmaxf(x, y), z) + (double)fmaxf(fmaxf(dx, dy), dz));
  return (double)s - bound;
}

} // namespace mixed
} // namespace vg
