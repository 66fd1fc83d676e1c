// Mixed-precision Polyhedron and Polycone distances (VG_PREC_MIXED).
//
// Polyhedron: the FP64 kernels of
// shapes_polyhedron_fp64.cuh with one change. Before a quadrilateral is evaluated in FP64
// inside Quadrilaterals::DistanceToIn / DistanceToOut (VecGeom/volumes/Quadrilaterals.h:
// 326-376, 447-496), an FP32 test on the record's FP32 copy of its planes tries to prove
// that the FP64 code would reject it (point on the wrong side of its plane, ray moving the
// wrong way, crossing point outside a side plane or outside the segment's z range). A
// proven rejection skips the quadrilateral; anything else is evaluated exactly as the FP64
// kernel does, in the same order. A skipped quadrilateral would have been skipped by the
// FP64 loop too, so the winner, and the returned bits, are the FP64 kernel's.
//
// Error bounds (each at least twice the worst case, computed with rounding to nearest on
// values that are themselves bounds). Coordinates are local FP32 copies of the FP64 point
// (rounding 2^-24 relative), normals and plane distances the record's FP32 copies (2^-24
// relative), and every fmaf rounds once (2^-24 of its result). With P1 = |p|_1:
//   plane value p.n + d:        |fp32 - fp64| <= (P1 + |d|) 2^-21 + FP64 rounding -> 2^-20
//   projection d.n (|d|_1 <= 3^0.5): <= 2^-20 -> 2^-19
//   crossing distance t = v / -proj, for |proj| >= 2^-6 and |t| < 1e5:
//     |dt| <= (e_v + |t| e_proj) / (|proj| - e_proj) + |t| 2^-21
//   crossing point x = p + t d: per component <= |dt| + (|t| + max|p|) 2^-21
//   side or z value at x: <= 2 |dx| + (|x|_1 + |d_side|) 2^-20
// A rejection needs the FP32 value beyond the reference's kTolerance threshold by more
// than the bound; grazing rays (|proj| < 2^-6) and far crossings get no side/z screen.
#pragma once
#include "nav_mixed.cuh"
#include "shapes_more_fp64.cuh"
#include "shapes_polyhedron_fp64.cuh"

namespace vg {
namespace mixed {

constexpr float kTolF = 1e-9f; // kTolerance

struct PolyF32 {
  const double *q0; // first quadrilateral (FP64)
  const float *f0;  // its FP32 plane copy
  F3 p, d;          // local point and direction, FP32
  float P1, Pinf;   // |p|_1, max |p_k|
  __device__ const float *of(const double *q) const { return f0 + kPolyQuadFloats * (int)((q - q0) / kPolyQuadDoubles); }
};

__device__ __forceinline__ PolyF32 poly_f32(const f64::PolyhedronView &v, V3 p, V3 d)
{
  PolyF32 m;
  m.q0   = v.r + (int)v.h->offQuad0;
  m.f0   = reinterpret_cast<const float *>(v.r + (int)v.h->offQuadF);
  m.p    = f3(p);
  m.d    = f3(d);
  m.P1   = fabsf(m.p.x) + fabsf(m.p.y) + fabsf(m.p.z);
  m.Pinf = fmaxf(fmaxf(fabsf(m.p.x), fabsf(m.p.y)), fabsf(m.p.z));
  return m;
}

// FP32 plane value and projection of a quadrilateral, with their error bounds.
struct QuadEval {
  float pl, epl, pr;
};
__device__ __forceinline__ QuadEval quad_eval(const PolyF32 &m, const float *f)
{
  const float nx = __ldg(f), ny = __ldg(f + 1), nz = __ldg(f + 2), dq = __ldg(f + 3);
  QuadEval e;
  e.pl  = fmaf(m.p.x, nx, fmaf(m.p.y, ny, fmaf(m.p.z, nz, dq)));
  e.epl = (m.P1 + fabsf(dq)) * 0x1p-20f;
  e.pr  = fmaf(m.d.x, nx, fmaf(m.d.y, ny, m.d.z * nz));
  return e;
}
constexpr float kEpr = 0x1p-19f;

// Crossing point of the ray with the quadrilateral's plane at t = pl / -pr and its bound;
// false when the bound cannot be made small (grazing ray, far crossing).
__device__ __forceinline__ bool crossing(const PolyF32 &m, const QuadEval &e, F3 &x, float &ex)
{
  const float apr = fabsf(e.pr);
  if (!(apr >= 0x1p-6f)) return false;
  const float t  = e.pl / -e.pr;
  const float at = fabsf(t);
  if (!(at < 1e5f)) return false;
  const float et = (e.epl + at * kEpr) / (apr - kEpr) + at * 0x1p-21f;
  x  = F3{fmaf(m.d.x, t, m.p.x), fmaf(m.d.y, t, m.p.y), fmaf(m.d.z, t, m.p.z)};
  ex = et + (at + m.Pinf) * 0x1p-21f;
  return true;
}

// True when some side plane certainly puts x outside (Quadrilaterals.h:107-117 and the
// side loop of :359-366: a side value below -kTolerance rejects).
__device__ __forceinline__ bool sides_reject(const float *f, F3 x, float ex)
{
  const float X1 = fabsf(x.x) + fabsf(x.y) + fabsf(x.z);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float *s = f + 4 + 4 * j;
    const float sd = __ldg(s + 3);
    const float v  = fmaf(x.x, __ldg(s), fmaf(x.y, __ldg(s + 1), fmaf(x.z, __ldg(s + 2), sd)));
    const float es = 2.f * ex + (X1 + fabsf(sd)) * 0x1p-20f;
    if (v < -kTolF - es) return true;
  }
  return false;
}

// Quadrilaterals::DistanceToIn<behindPlanes> rejects quadrilateral f for this ray.
__device__ __forceinline__ bool rejects_in(const PolyF32 &m, const float *f, bool behind)
{
  const QuadEval e = quad_eval(m, f);
  if ((behind ? -e.pl : e.pl) < -kTolF - e.epl) return true; // (behind ? -dist : dist) > -kTolerance fails
  if ((behind ? e.pr : -e.pr) <= -kEpr) return true;          // (behind ? proj : -proj) > 0 fails
  F3 x;
  float ex;
  if (!crossing(m, e, x, ex)) return false;
  return sides_reject(f, x, ex);
}

// Quadrilaterals::DistanceToOut(point, direction, zMin, zMax) rejects quadrilateral f.
__device__ __forceinline__ bool rejects_out(const PolyF32 &m, const float *f, bool sameZ, float zMin, float zMax)
{
  const QuadEval e = quad_eval(m, f);
  if (e.pl >= kTolF + e.epl) return true; // t < kTolerance fails
  if (e.pr <= -kEpr) return true;         // proj > 0 fails
  F3 x;
  float ex;
  if (!crossing(m, e, x, ex)) return false;
  if (sameZ) return sides_reject(f, x, ex);
  const float ez = 2.f * ex + fmaxf(fabsf(zMin), fabsf(zMax)) * 0x1p-20f;
  return x.z < zMin - kTolF - ez || x.z >= zMax + kTolF + ez; // zMin - kTol <= zp < zMax + kTol fails
}

// qs_dist_in (shapes_polyhedron_fp64.cuh) with the FP32 screen in front of each
// quadrilateral, in rounds: every lane skips, in FP32, the quadrilaterals proven rejected,
// then the lanes that reached a candidate test it in FP64 together (same order and tests
// as the FP64 loop for each lane; the first valid quadrilateral wins).
static __device__ __noinline__ double qs_dist_in_m(const PolyF32 &m, f64::QuadSet s, V3 p, V3 d, bool behind)
{
  const unsigned mask = __activemask();
  double best = kInfLength;
  int i       = 0;
  bool active = true;
  while (true) {
    if (active) {
      while (i < s.n && rejects_in(m, m.of(s.at(i)), behind)) ++i;
      if (i >= s.n) active = false;
    }
    if (!__any_sync(mask, active)) break;
    if (!active) continue;
    const double *q = s.at(i++);
    const V3 n      = f64::qnormal(q);
    double distance = dot(p, n) + __ldg(q + 3);
    if (!((behind ? -distance : distance) > -kTolerance)) continue;
    const double proj = dot(d, n);
    if (!((behind ? proj : -proj) > 0)) continue;
    distance /= -(proj + copysign(1E-20, proj));
    const V3 x = V3{p.x + d.x * distance, p.y + d.y * distance, p.z + d.z * distance};
    bool valid = true;
    for (int j = 0; j < 4; ++j) {
      valid &= f64::qside(q, j, x) >= -kTolerance;
      if (!valid) break;
    }
    if (valid) best = distance;
    if (best < kInfLength) active = false;
  }
  return f64::dmax(0., best);
}

// qs_dist_out with the FP32 screen (zMin, zMax: the segment's z range), in rounds as above;
// every quadrilateral not proven rejected is tested in FP64 in order (minimum of the valid).
static __device__ __noinline__ double qs_dist_out_m(const PolyF32 &m, f64::QuadSet s, V3 p, V3 d, double zMin,
                                                    double zMax)
{
  const unsigned mask = __activemask();
  const bool sameZ    = zMin == zMax;
  const float zMinF = (float)zMin, zMaxF = (float)zMax;
  double best = kInfLength;
  int i       = 0;
  bool active = true;
  while (true) {
    if (active) {
      while (i < s.n && rejects_out(m, m.of(s.at(i)), sameZ, zMinF, zMaxF)) ++i;
      if (i >= s.n) active = false;
    }
    if (!__any_sync(mask, active)) break;
    if (!active) continue;
    const double *q = s.at(i++);
    const V3 n      = f64::qnormal(q);
    double t        = dot(p, n) + __ldg(q + 3);
    if (!(t < kTolerance)) continue;
    const double proj = dot(d, n);
    if (!(proj > 0)) continue;
    t /= -proj;
    if (!(t < best)) continue;
    bool valid;
    if (sameZ) {
      valid = f64::qs_rayhits(q, V3{p.x + t * d.x, p.y + t * d.y, p.z + t * d.z});
    } else {
      const double zp = p.z + t * d.z;
      valid           = (zp >= zMin - kTolerance) && (zp < zMax + kTolerance);
    }
    if (!valid) continue;
    best = t;
  }
  if (best > -kTolerance) best = f64::dmax(best, 0.);
  return best;
}

// ph_dist_in_seg / ph_dist_out_seg with the screened loops
__device__ __forceinline__ double ph_dist_in_seg_m(const PolyF32 &m, const f64::PolyhedronView &v, int s, V3 p, V3 d)
{
  double distance = qs_dist_in_m(m, v.outer(s), p, d, false);
  bool done       = distance < kInfLength;
  if (done) return distance;
  if (v.phi()) distance = qs_dist_in_m(m, v.phis(s), p, d, false);
  done |= distance < kInfLength;
  if (done) return distance;
  if (v.hasInnerRadius(s)) distance = qs_dist_in_m(m, v.inners(s), p, d, true);
  return distance;
}
__device__ __forceinline__ double ph_dist_out_seg_m(const PolyF32 &m, const f64::PolyhedronView &v, int s, double zMin,
                                                    double zMax, V3 p, V3 d)
{
  bool done       = false;
  double distance = kInfLength;
  if (v.hasInnerRadius(s)) {
    distance = qs_dist_in_m(m, v.inners(s), p, d, false);
    done     = distance < kInfLength;
    if (done) return distance;
  }
  if (v.phi()) {
    const double distphi = qs_dist_in_m(m, v.phis(s), p, d, true);
    if (!done && distance > -kTolerance) distance = distphi;
    done = distance > -kTolerance && distance < kInfLength;
    if (done) return distance;
  }
  const double distout = qs_dist_out_m(m, v.outer(s), p, d, zMin, zMax);
  if (!done) distance = distout;
  return distance;
}

// ph_dist_in (PolyhedronImplementation.h:872-945) with the screened segment loop; points
// beyond kMaxCoord (4 m, where the bounds above were not sized) take the FP64 kernel.
static __device__ __noinline__ double polyhedron_dist_in_mixed(const PolyhedronRec &rec, V3 p, V3 d)
{
  const f64::PolyhedronView v(rec);
  if ((p.z < v.z(0) + kTolerance) && d.z <= 0) return kInfLength;
  if ((p.z > v.z(v.nseg) - kTolerance) && d.z >= 0) return kInfLength;
  if (f64::ph_inside(v, p) == kInside) return -1.;
  double tubeDistance = 0.;
  {
    const V3 bp = V3{p.x, p.y, p.z - v.h->tubeOffset};
    if (!f64::tube_contains(v.h->bt, bp)) {
      tubeDistance = f64::tube_dist_in(v.h->bt, bp, d);
      if (tubeDistance == kInfLength) return kInfLength;
    }
  }
  const PolyF32 m = poly_f32(v, p, d);
  if (!(m.Pinf <= 4000.f)) return f64::ph_dist_in(v, p, d);
  int zi = v.findZ(p.z);
  zi     = zi < 0 ? 0 : (zi >= v.nseg ? v.nseg - 1 : zi);
  double distance = kInfLength;
  if (d.z >= 0) {
    for (; zi < v.nseg; ++zi) {
      distance = ph_dist_in_seg_m(m, v, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = ph_dist_in_seg_m(m, v, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  }
  f64::ph_endcaps(v, false, p, d, distance);
  return (distance >= tubeDistance - 1E-6) ? distance : kInfLength;
}

// ph_dist_out (PolyhedronImplementation.h:1045-1090) with the screened segment loop
static __device__ __noinline__ double polyhedron_dist_out_mixed(const PolyhedronRec &rec, V3 p, V3 d)
{
  const f64::PolyhedronView v(rec);
  const int zMax = v.nseg;
  if ((p.z < v.z(0) - kTolerance) || (p.z > v.z(zMax) + kTolerance)) return -1.;
  if (f64::ph_inside(v, p) == kOutside) return -1.;
  const PolyF32 m = poly_f32(v, p, d);
  if (!(m.Pinf <= 4000.f)) return f64::ph_dist_out(v, p, d);
  int zi = v.findZ(p.z);
  zi     = zi < 0 ? 0 : (zi >= zMax ? zMax - 1 : zi);
  double distance = kInfLength;
  if (d.z >= 0) {
    for (; zi < zMax; ++zi) {
      distance = ph_dist_out_seg_m(m, v, zi, v.z(zi), v.z(zi + 1), p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (v.z(zi) - p.z > distance) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = ph_dist_out_seg_m(m, v, zi, v.z(zi), v.z(zi + 1), p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (p.z - v.z(zi) > distance) break;
    }
  }
  f64::ph_endcaps(v, true, p, d, distance);
  if (distance >= kInfLength) distance = 0.;
  return distance;
}

// ---------------------------------------------------------------- Polycone
// PolyconeImplementation.h:148-180 DistanceToIn walks the sections from the point's one in
// the direction of the ray and stops at the first whose Cone DistanceToIn is below
// kInfLength. A section is not evaluated in FP64 when FP32 proves that the point lies
// outside its padded cylindrical shell (4e-3 mm beyond every radius and z face the cone
// has, rounded outward; the FP32 point is within 1e-3 mm of the FP64 one up to 4 m) and
// that the ray misses that shell: the cone's FP64 DistanceToIn is then kInfLength, its
// miss value, which is what the loop is given. Other sections run the FP64 Cone kernel,
// so the result is the FP64 kernel's.
__device__ __forceinline__ bool pc_section_certain_miss(const f64::PolyconeView &v, int i, F3 pf, F3 df)
{
  const float *sh = reinterpret_cast<const float *>(v.sec(i) + 1);
  const float rmin = __ldg(sh), rmax = __ldg(sh + 1), zlo = __ldg(sh + 2), zhi = __ldg(sh + 3);
  const float r2 = fmaf(pf.x, pf.x, pf.y * pf.y);
  const bool outside = pf.z < zlo || pf.z > zhi || r2 > rmax * rmax || (rmin > 0.f && r2 < rmin * rmin);
  return outside && shell_lb(rmin, rmax, zlo, zhi, pf, df) == INFINITY;
}

// The section loop in rounds: each lane first walks, in FP32, past the sections it can prove
// missed (their FP64 value would be kInfLength), then the lanes that reached a candidate
// evaluate it in FP64 together (one Cone kernel per round for the whole warp, instead of
// one per lane and iteration). Each lane sees the reference's sequence of values.
static __device__ __noinline__ double polycone_dist_in_mixed(const PolyconeRec &rec, V3 p, V3 d)
{
  const unsigned mask = __activemask();
  const f64::PolyconeView v(rec);
  const F3 pf = f3(p), df = f3(d);
  const bool screen = fabsf(pf.x) <= 4000.f && fabsf(pf.y) <= 4000.f && fabsf(pf.z) <= 4000.f;
  double distance = kInfLength;
  int increment   = f64::dgt(d.z, 0.) ? 1 : -1;
  if (f64::dabs_lt(d.z, kTolerance)) increment = 0;
  int index = v.index(p.z);
  if (index == -1) index = 0;
  if (index == -2) index = v.nsec - 1;
  bool active = true;
  while (true) {
    if (active && screen) { // FP32 walk: a proven miss is the FP64 loop's kInfLength iteration
      while (pc_section_certain_miss(v, index, pf, df)) {
        distance = kInfLength;
        if (!increment) {
          active = false;
          break;
        }
        index += increment;
        if (index < 0 || index >= v.nsec) {
          active = false;
          break;
        }
      }
    }
    if (!__any_sync(mask, active)) break;
    if (active) {
      distance = f64::cone_dist_in(v.cone(index), v.local(p, index), d);
      if (f64::dlt(distance, kInfLength) || !increment) {
        active = false;
      } else {
        index += increment;
        if (index < 0 || index >= v.nsec) active = false;
      }
    }
  }
  return distance;
}

} // namespace mixed
} // namespace vg
