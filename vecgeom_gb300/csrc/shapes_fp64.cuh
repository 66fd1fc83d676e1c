// FP64 device kernels of the primitive shapes: the plain-FP64 path whose results are
// compared bit-for-bit (Inside/Contains) and to 1e-9 mm (distances, safeties) with the
// reference's scalar FP64 path. Translation units that include this header are compiled
// with --fmad=false and IEEE division/sqrt, so each expression below rounds exactly like
// the reference's host build; the evaluation order of every expression follows the
// reference kernel cited above each function.
#pragma once
#include "fp64_int.cuh"
#include "vg_types.h"

namespace vg {
namespace f64 {

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 mk(double x, double y, double z) { return V3{x, y, z}; }
// x + copysign(1e-30, x). For |x| >= 2^-46 half an ulp of x exceeds 1e-30, so the sum
// rounds back to x and the FP64 addition is skipped.
__device__ __forceinline__ double nonzero(double x)
{
#if VG_FP64_SHORTCUTS
  if (dabs_lt(x, 1.4210854715202004e-14)) x = x + copysign(1.0e-30, x);
  return x;
#else
  return x + copysign(1.0e-30, x);
#endif
}
__device__ __forceinline__ double nonzeroabs(double x) { return fabs(x) + 1.0e-30; }
__device__ __forceinline__ double sgn(double x) { return copysign(1.0, x); }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double perp2(V3 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double max3(double a, double b, double c) { return dmax(a, dmax(b, c)); }
__device__ __forceinline__ double min3(double a, double b, double c) { return dmin(a, dmin(b, c)); }

// ---------------------------------------------------------------- transformations
// Generic Transform / TransformDirection / InverseTransform (Transformation3D.h:640-651,797-826).
//
// With VECGEOM_NO_SPECIALIZATION the reference applies the full 12-double transform to every
// point, also when the rotation is the identity. Its result is then known exactly without
// the multiplications: each component is  v + (u * 0) + (w * 0)  with v the component and u,
// w the other two; for finite inputs that is v itself when v != 0, and a zero that is -0
// only when v, u and w are all negative zeros. The identity case is recognised on the bit
// patterns (+1.0 on the diagonal, +0.0 elsewhere) and applied only to finite inputs, so the
// results are bit-identical to the multiplications they replace, which GB300 would issue on
// its narrow FP64 pipe.
__device__ __forceinline__ bool finite_bits(double x)
{
  return (__double_as_longlong(x) & 0x7FF0000000000000LL) != 0x7FF0000000000000LL;
}
// v + (u * +0.0) for finite u: v unless v is a zero, then -0 only when v and u are both -0
__device__ __forceinline__ double zadd(double v, double u)
{
  const long long vb = dbits(v);
  if ((vb & 0x7FFFFFFFFFFFFFFFLL) != 0) return v;
  return (vb < 0 && dbits(u) < 0) ? -0.0 : 0.0;
}
// Rotation about z: r[2] = r[5] = r[6] = r[7] = +0.0 and r[8] = +1.0 exactly. The terms with
// a zero factor are then known signed zeros, and the product with 1.0 is the operand.
__device__ __forceinline__ bool rot_is_z(const Xform &m)
{
  return VG_FP64_SHORTCUTS && __double_as_longlong(m.r[8]) == 0x3FF0000000000000LL && __double_as_longlong(m.r[2]) == 0 &&
         __double_as_longlong(m.r[5]) == 0 && __double_as_longlong(m.r[6]) == 0 &&
         __double_as_longlong(m.r[7]) == 0;
}
__device__ __forceinline__ bool rot_is_identity(const Xform &m)
{
  const long long one = 0x3FF0000000000000LL;
  return __double_as_longlong(m.r[0]) == one && __double_as_longlong(m.r[4]) == one &&
         __double_as_longlong(m.r[8]) == one && __double_as_longlong(m.r[1]) == 0 &&
         __double_as_longlong(m.r[2]) == 0 && __double_as_longlong(m.r[3]) == 0 &&
         __double_as_longlong(m.r[5]) == 0 && __double_as_longlong(m.r[6]) == 0 &&
         __double_as_longlong(m.r[7]) == 0;
}
// v + (u * 0) + (w * 0) for finite u, w
__device__ __forceinline__ double zsum3(double v, double u, double w)
{
  const long long vb = __double_as_longlong(v);
  if ((vb & 0x7FFFFFFFFFFFFFFFLL) != 0) return v;
  return (vb < 0 && __double_as_longlong(u) < 0 && __double_as_longlong(w) < 0) ? -0.0 : 0.0;
}
__device__ __forceinline__ V3 rotate(const Xform &m, V3 a)
{
  const bool fin = finite_bits(a.x) && finite_bits(a.y) && finite_bits(a.z);
  if (fin && rot_is_identity(m)) return V3{zsum3(a.x, a.y, a.z), zsum3(a.y, a.x, a.z), zsum3(a.z, a.x, a.y)};
  if (fin && rot_is_z(m)) {
    const double sx = a.x * m.r[0] + a.y * m.r[3], sy = a.x * m.r[1] + a.y * m.r[4];
    return V3{zadd(sx, a.z), zadd(sy, a.z), zsum3(a.z, a.x, a.y)};
  }
  double lx = a.x * m.r[0], ly = a.x * m.r[1], lz = a.x * m.r[2];
  lx += a.y * m.r[3];
  ly += a.y * m.r[4];
  lz += a.y * m.r[5];
  lx += a.z * m.r[6];
  ly += a.z * m.r[7];
  lz += a.z * m.r[8];
  return V3{lx, ly, lz};
}
__device__ __forceinline__ V3 to_local(const Xform &m, V3 p)
{
  // p - (+0.0) is p for every p, so a zero translation needs no subtraction
  const bool zt = __double_as_longlong(m.t[0]) == 0 && __double_as_longlong(m.t[1]) == 0 &&
                  __double_as_longlong(m.t[2]) == 0;
  return rotate(m, zt ? p : V3{p.x - m.t[0], p.y - m.t[1], p.z - m.t[2]});
}
__device__ __forceinline__ V3 to_master(const Xform &m, V3 l)
{
  const bool fin = finite_bits(l.x) && finite_bits(l.y) && finite_bits(l.z);
  if (fin && rot_is_identity(m))
    return V3{zsum3(m.t[0] + l.x, l.y, l.z), zsum3(m.t[1] + l.y, l.x, l.z), zsum3(m.t[2] + l.z, l.x, l.y)};
  if (fin && rot_is_z(m)) {
    double x = m.t[0];
    x += l.x * m.r[0];
    x += l.y * m.r[1];
    double y = m.t[1];
    y += l.x * m.r[3];
    y += l.y * m.r[4];
    return V3{zadd(x, l.z), zadd(y, l.z), zsum3(m.t[2], l.x, l.y) + l.z};
  }
  double x = m.t[0];
  x += l.x * m.r[0];
  x += l.y * m.r[1];
  x += l.z * m.r[2];
  double y = m.t[1];
  y += l.x * m.r[3];
  y += l.y * m.r[4];
  y += l.z * m.r[5];
  double z = m.t[2];
  z += l.x * m.r[6];
  z += l.y * m.r[7];
  z += l.z * m.r[8];
  return V3{x, y, z};
}

// ---------------------------------------------------------------- wedge
// Wedge_Evolution.h:335-347
__device__ __forceinline__ bool wedge_on_surface(double ax, double ay, double nx, double ny, V3 p)
{
  if (!dge(ax * p.x + ay * p.y, 0.)) return false;
  return dabs_lt(nx * p.x + ny * p.y, kTolerance);
}
// Wedge_Evolution.h:299-331 (forInside selects the surface-aware variant)
__device__ __forceinline__ void wedge_classify(const WedgeRec &w, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double startCheck = (-p.x * w.a1y + p.y * w.a1x);
  const double endCheck   = (-w.a2x * p.y + w.a2y * p.x);
  cout                    = dlt(startCheck, 0.);
  if (dlt(w.dphi, kPi))
    cout = cout || dlt(endCheck, 0.);
  else
    cout = cout && dlt(endCheck, 0.);
  if (forInside) {
    const bool onSurface = wedge_on_surface(w.a1x, w.a1y, w.n1x, w.n1y, p) || wedge_on_surface(w.a2x, w.a2y, w.n2x, w.n2y, p);
    cout                 = cout && !onSurface;
    cin                  = !onSurface && !cout;
  }
}
__device__ __forceinline__ double wedge_safety_out(const WedgeRec &w, V3 p)
{
  const double d1 = p.x * w.n1x + p.y * w.n1y;
  const double d2 = p.x * w.n2x + p.y * w.n2y;
  return dlt(w.dphi, kPi) ? dmin(d1, d2) : dmax(d1, d2);
}
__device__ __forceinline__ double wedge_safety_in(const WedgeRec &w, V3 p)
{
  const double d1 = p.x * w.n1x + p.y * w.n1y;
  const double d2 = p.x * w.n2x + p.y * w.n2y;
  return dlt(w.dphi, kPi) ? dmax(-d1, -d2) : dmin(-d1, -d2);
}

// ================================================================ Box
// BoxImplementation.h:84-167
__device__ __forceinline__ double box_safety_in(const BoxRec &b, V3 p)
{
  return max3(fabs(p.x) - b.dx, fabs(p.y) - b.dy, fabs(p.z) - b.dz);
}
__device__ __forceinline__ double box_safety_out(const BoxRec &b, V3 p)
{
  return min3(b.dx - fabs(p.x), b.dy - fabs(p.y), b.dz - fabs(p.z));
}
__device__ __forceinline__ int box_inside(const BoxRec &b, V3 p)
{
  const double dist = box_safety_in(b, p);
  return dabs_lt(dist, kHalfTolerance) ? kSurface : (dlt(dist, 0.) ? kInside : kOutside);
}
__device__ __forceinline__ bool box_contains(const BoxRec &b, V3 p) { return dlt(box_safety_in(b, p), 0.); }
// The products with sgn(d) = +-1 are sign flips (flipsign / negflipsign).
__device__ __forceinline__ double box_dist_in(const BoxRec &b, V3 p, V3 d)
{
  const double ix = 1.0 / nonzero(d.x), iy = 1.0 / nonzero(d.y), iz = 1.0 / nonzero(d.z);
  const double inx = negflipsign(b.dx, d.x) - p.x, iny = negflipsign(b.dy, d.y) - p.y,
               inz = negflipsign(b.dz, d.z) - p.z;
  const double ox = flipsign(b.dx, d.x) - p.x, oy = flipsign(b.dy, d.y) - p.y, oz = flipsign(b.dz, d.z) - p.z;
  const double absOrthogOut = fabs(min3(flipsign(ox, d.x), flipsign(oy, d.y), flipsign(oz, d.z)));
  const double distOut      = min3(ox * ix, oy * iy, oz * iz);
  const double distance     = max3(inx * ix, iny * iy, inz * iz);
  const bool miss = dge(distance, distOut) || dle(distOut, kHalfTolerance) || dle(absOrthogOut, kHalfTolerance);
  return miss ? kInfLength : distance;
}
__device__ __forceinline__ double box_dist_out(const BoxRec &b, V3 p, V3 d)
{
  const double ix = 1.0 / nonzero(d.x), iy = 1.0 / nonzero(d.y), iz = 1.0 / nonzero(d.z);
  const double safetyIn = box_safety_in(b, p);
  const double ox = flipsign(b.dx, d.x) - p.x, oy = flipsign(b.dy, d.y) - p.y, oz = flipsign(b.dz, d.z) - p.z;
  const double distance = min3(ox * ix, oy * iy, oz * iz);
  return dgt(safetyIn, kHalfTolerance) ? -1.0 : distance;
}

// ================================================================ Tube
// TubeImplementation.h:57-97 PointInCyclicalSector (includeSurface selects the -/+ band)
__device__ __forceinline__ bool tube_in_sector(const TubeRec &t, double x, double y, bool includeSurface)
{
  const double startCheck = (-x * t.a1y + y * t.a1x);
  const double endCheck   = (-t.a2x * y + t.a2y * x);
  const double tol        = includeSurface ? -kHalfTolerance : kHalfTolerance;
  if (dle(t.dphi, kPi)) return dge(startCheck, tol) && dge(endCheck, tol);
  return dge(startCheck, tol) || dge(endCheck, tol);
}
__device__ __forceinline__ bool tube_phi(const TubeRec &t) { return dlt(t.dphi, kTwoPi); }
__device__ __forceinline__ bool tube_rmin(const TubeRec &t) { return dgt(t.rmin, 0.); }

// TubeImplementation.h:103-162
__device__ __forceinline__ void tube_circle(const TubeRec &t, double b, double c, V3 pos, V3 dir, bool largest,
                                            bool insectorCheck, double &dist, bool &ok)
{
  double delta = b * b - c;
  ok           = dgt(delta, 0.) || (largest && deq(delta, 0.));
  if (!ok) delta = 0.;
  delta = sqrt(delta);
  if (!largest) delta = -delta;
  dist = -b + delta;
  ok   = ok && dge(dist, -2 * kTolerance);
  if (!ok || !insectorCheck) return;
  const double hitz = pos.z + dist * dir.z;
  ok                = dabs_le(hitz, t.z);
  if (!ok) return;
  if (tube_phi(t)) {
    const double hitx = pos.x + dist * dir.x;
    const double hity = pos.y + dist * dir.y;
    ok                = tube_in_sector(t, hitx, hity, true);
  }
}

// TubeImplementation.h:243-291
__device__ __forceinline__ void tube_phi_plane(const TubeRec &t, double ax, double ay, double nx, double ny, V3 pos,
                                               V3 dir, bool insectorCheck, double &dist, bool &ok)
{
  const double dirDotNorm = dir.x * nx + dir.y * ny;
  ok                      = insectorCheck ? dgt(dirDotNorm, 0.) : dlt(dirDotNorm, 0.);
  const double dirDotXY   = (dir.y * ax - dir.x * ay);
  dist                    = (ay * pos.x - ax * pos.y) / nonzero(dirDotXY);
  ok                      = ok && dgt(dist * fabs(dirDotNorm), -kHalfTolerance);
  const double hitx       = pos.x + dist * dir.x;
  const double hity       = pos.y + dist * dir.y;
  if (insectorCheck) {
    const double hitz = pos.z + dist * dir.z;
    const double r2   = hitx * hitx + hity * hity;
    ok                = ok && dabs_le(hitz, t.tolOz) && dge(r2, t.tolOrmin2) && dle(r2, t.tolOrmax2);
    ok                = ok && dgt(hitx * ax + hity * ay, 0.);
  } else {
    ok = ok && dge(hitx * ax + hity * ay, 0.);
  }
}

// TubeImplementation.h:293-322
__device__ __forceinline__ bool tube_moving_in_surface(const TubeRec &t, V3 p, V3 d, bool inner)
{
  const double rho = perp2(p);
  const bool zok   = dabs_lt(p.z, t.z + kTolerance);
  const bool on    = inner ? (dge(rho, t.tolOrmin2) && dle(rho, t.tolIrmin2) && zok)
                        : (dge(rho, t.tolIrmax2) && dle(rho, t.tolOrmax2) && zok);
  const V3 n = inner ? V3{-p.x, -p.y, 0.} : V3{p.x, p.y, 0.};
  return on && dle(dot(d, n), 0.);
}

// TubeImplementation.h:352-396
__device__ __forceinline__ void tube_classify(const TubeRec &t, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double absz = fabs(p.z);
  cout              = dgt(absz, forInside ? t.z + kHalfTolerance : t.z);
  if (forInside) cin = dlt(absz, t.z - kHalfTolerance);
  if (cout) return;
  const double r2 = p.x * p.x + p.y * p.y;
  if (forInside) {
    cout = dgt(r2, t.rmax * (t.rmax + 2.0 * kTolerance));
    cin  = cin && dlt(r2, fabs(t.rmax * (t.rmax - 2.0 * kTolerance)));
  } else {
    cout = dgt(r2, t.rmax * t.rmax);
  }
  if (cout) return;
  if (tube_rmin(t)) {
    if (forInside) {
      cout = dle(r2, fabs(t.rmin * (t.rmin - 2.0 * kTolerance)));
      cin  = cin && dgt(r2, t.rmin * (t.rmin + 2.0 * kTolerance));
    } else {
      cout = dle(r2, t.rmin * t.rmin);
    }
    if (cout) return;
  }
  if (tube_phi(t)) {
    bool ci = false, co = false;
    wedge_classify(t.w, p, forInside, ci, co);
    cout = co;
    if (forInside) cin = cin && ci;
  }
}
__device__ __forceinline__ int tube_inside(const TubeRec &t, V3 p)
{
  bool cin = false, cout = false;
  tube_classify(t, p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
__device__ __forceinline__ bool tube_contains(const TubeRec &t, V3 p)
{
  bool cin = false, cout = false;
  tube_classify(t, p, false, cin, cout);
  return !cout;
}

// TubeImplementation.h:456-596 DistanceToInKernel
static __device__ __noinline__ double tube_dist_in_kernel(const TubeRec &t, V3 point, V3 dir)
{
  double distz = fabs(point.z) - t.z;
  if (dgt(distz, kHalfTolerance) && dge(point.z * dir.z, 0.)) return kInfLength;
  const double rsq   = point.x * point.x + point.y * point.y;
  const double rdotn = point.x * dir.x + point.y * dir.y;
  if (dgt(rsq, t.tolIrmax2) && dge(rdotn, 0.)) return kInfLength;
  bool inside = dlt(distz, -kHalfTolerance) && dlt(rsq, t.tolIrmax2);
  if (tube_rmin(t)) inside = inside && dgt(rsq, t.tolIrmin2);
  if (tube_phi(t) && inside) inside = tube_in_sector(t, point.x, point.y, false);
  if (inside) return -1.0;

  double distance = kInfLength;
  distz /= nonzeroabs(dir.z);
  const double hitx = point.x + distz * dir.x;
  const double hity = point.y + distz * dir.y;
  const double r2   = hitx * hitx + hity * hity;
  bool okz          = dgt(distz, -kHalfTolerance) && dlt(point.z * dir.z, 0.) && dle(r2, t.rmax2);
  if (tube_rmin(t)) okz = okz && dle(t.rmin2, r2);
  if (tube_phi(t) && okz) okz = tube_in_sector(t, hitx, hity, true);
  if (okz) distance = distz;
  bool done = okz;

  bool onSurfIn = tube_moving_in_surface(t, point, dir, false);
  if (tube_rmin(t)) onSurfIn = onSurfIn || tube_moving_in_surface(t, point, dir, true);
  if (tube_phi(t)) onSurfIn = onSurfIn && tube_in_sector(t, point.x, point.y, true);
  if (!done && onSurfIn) distance = 0.;
  done = done || onSurfIn;
  if (done) return distance;

  const double invnsq = 1. / nonzero(1. - dir.z * dir.z);
  const double b      = invnsq * rdotn;
  const double crmax  = invnsq * (rsq - t.rmax2);
  double dist_rmax;
  bool ok_rmax;
  tube_circle(t, b, crmax, point, dir, false, true, dist_rmax, ok_rmax);
  if (ok_rmax && dlt(dist_rmax, distance)) return dist_rmax;

  if (tube_rmin(t)) {
    const double crmin = invnsq * (rsq - t.rmin2);
    double dist_rmin;
    bool ok_rmin;
    tube_circle(t, b, crmin, point, dir, true, true, dist_rmin, ok_rmin);
    if (ok_rmin && dlt(dist_rmin, distance)) distance = dist_rmin;
  }
  if (tube_phi(t)) {
    double dist_phi;
    bool ok_phi;
    tube_phi_plane(t, t.a1x, t.a1y, t.w.n1x, t.w.n1y, point, dir, true, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
    tube_phi_plane(t, t.a2x, t.a2y, t.w.n2x, t.w.n2y, point, dir, true, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
  }
  return distance;
}

// TubeImplementation.h:424-452 (far points are first moved to 100 x the shape size)
__device__ __forceinline__ double tube_dist_in(const TubeRec &t, V3 p, V3 d)
{
  const double ptDist = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double distToMove   = 0.;
  if (dgt(ptDist, 100. * t.maxVal)) {
    distToMove = ptDist - 100. * t.maxVal;
    p          = V3{p.x + distToMove * d.x, p.y + distToMove * d.y, p.z + distToMove * d.z};
  }
  return tube_dist_in_kernel(t, p, d) + distToMove;
}

// TubeImplementation.h:601-697 DistanceToOut
static __device__ __noinline__ double tube_dist_out(const TubeRec &t, V3 point, V3 dir)
{
  if (dlt(t.z - fabs(point.z), -kHalfTolerance)) return -1.;
  const double rsq   = point.x * point.x + point.y * point.y;
  const double rdotn = dir.x * point.x + dir.y * point.y;
  double crmax       = rsq - t.rmax2;
  double crmin       = rsq;
  if (dgt(crmax, 2.0 * kTolerance * t.rmax)) return -1.;
  if (tube_rmin(t)) {
    crmin -= t.rmin2;
    if (dlt(crmin, -2.0 * kTolerance * t.rmin)) return -1.;
  }
  if (tube_phi(t)) {
    bool ci = false, co = false;
    wedge_classify(t.w, point, true, ci, co);
    if (co) return -1.;
  }
  double distance      = kInfLength;
  const double invdirz = 1. / nonzero(dir.z);
  double distz         = (t.z - point.z) * invdirz;
  if (dlt(dir.z, 0.)) distz = (-t.z - point.z) * invdirz;
  if (dne(dir.z, 0.) && dlt(distz, distance)) distance = distz;
  const double invnsq = 1. / nonzero(1. - dir.z * dir.z);
  const double b      = invnsq * rdotn;
  if (tube_rmin(t)) {
    double dist_rmin;
    bool ok_rmin;
    crmin *= invnsq;
    tube_circle(t, b, crmin, point, dir, false, false, dist_rmin, ok_rmin);
    if (ok_rmin && dlt(dist_rmin, distance)) distance = dist_rmin;
  }
  double dist_rmax;
  bool ok_rmax;
  crmax *= invnsq;
  tube_circle(t, b, crmax, point, dir, true, false, dist_rmax, ok_rmax);
  if (ok_rmax && dlt(dist_rmax, distance)) distance = dist_rmax;
  if (tube_phi(t)) {
    double dist_phi;
    bool ok_phi;
    tube_phi_plane(t, t.a1x, t.a1y, t.w.n1x, t.w.n1y, point, dir, false, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
    tube_phi_plane(t, t.a2x, t.a2y, t.w.n2x, t.w.n2y, point, dir, false, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
  }
  return distance;
}

// TubeImplementation.h:758-781 SafetyToInOld (phi plane safety from :200-232)
__device__ __forceinline__ double tube_safety_in(const TubeRec &t, V3 p)
{
  double safety         = fabs(p.z) - t.z;
  const double r        = sqrt(p.x * p.x + p.y * p.y);
  const double safermax = r - t.rmax;
  if (dgt(safermax, safety)) safety = safermax;
  if (tube_rmin(t)) {
    const double safermin = t.rmin - r;
    if (dgt(safermin, safety)) safety = safermin;
  }
  if (tube_phi(t)) {
    if (tube_in_sector(t, p.x, p.y, false)) return safety;
    double safephi = dgt(t.dphi, kPi) ? sqrt(p.x * p.x + p.y * p.y) : kInfLength;
    const double phi1 = p.x * t.a1y - p.y * t.a1x;
    if (dgt(phi1, -kHalfTolerance) && dlt(phi1, safephi)) safephi = phi1;
    const double phi2 = -(p.x * t.a2y - p.y * t.a2x);
    if (dgt(phi2, -kHalfTolerance) && dlt(phi2, safephi)) safephi = phi2;
    if (dlt(safephi, kInfLength) && dgt(safephi, safety)) safety = safephi;
  }
  return safety;
}

// TubeImplementation.h:785-802 SafetyToOutOld
__device__ __forceinline__ double tube_safety_out(const TubeRec &t, V3 p)
{
  double safety         = t.z - fabs(p.z);
  const double r        = sqrt(p.x * p.x + p.y * p.y);
  const double safermax = t.rmax - r;
  if (dlt(safermax, safety)) safety = safermax;
  if (tube_rmin(t)) {
    const double safermin = r - t.rmin;
    if (dlt(safermin, safety)) safety = safermin;
  }
  if (tube_phi(t)) {
    const double safephi = wedge_safety_out(t.w, p);
    if (dlt(safephi, safety)) safety = safephi;
  }
  return safety;
}

// ================================================================ Cut tube
// CutPlanes.h / Plane.h on the record's two planes: DistPlane = p.n + d (Plane.h:98-107)
__device__ __forceinline__ double cut_dist0(const CutTubeRec &c, V3 p) { return p.x * c.n0x + p.y * c.n0y + p.z * c.n0z + c.d0; }
__device__ __forceinline__ double cut_dist1(const CutTubeRec &c, V3 p) { return p.x * c.n1x + p.y * c.n1y + p.z * c.n1z + c.d1; }
// CutPlanes::Inside (CutPlanes.h:130-142)
__device__ __forceinline__ int cut_inside(const CutTubeRec &c, V3 p)
{
  const double d0 = cut_dist0(c, p), d1 = cut_dist1(c, p);
  int inside      = (dlt(d0, 0.0) && dlt(d1, 0.0)) ? kInside : kOutside;
  if (dabs_lt(d0, kTolerance) || dabs_lt(d1, kTolerance)) inside = kSurface;
  return inside;
}
// Plane::DistanceToIn (Plane.h:128-147) masked to -kInfLength when moving along the normal
// (CutPlanes.h:144-156)
__device__ __forceinline__ double cut_plane_dist_in(double nx, double ny, double nz, double dd, V3 p, V3 dir)
{
  double distance  = -kInfLength;
  const double dt  = dir.x * nx + dir.y * ny + dir.z * nz;
  const double ndd = nonzero(dt);
  const double saf = p.x * nx + p.y * ny + p.z * nz + dd;
  if (dlt(ndd, 0.) && dgt(saf, -kTolerance)) distance = -saf / ndd;
  if (dgt(dt, 0.)) distance = -kInfLength;
  return distance;
}
// Plane::DistanceToOut (Plane.h:149-170)
__device__ __forceinline__ double cut_plane_dist_out(double nx, double ny, double nz, double dd, V3 p, V3 dir)
{
  double distance  = kInfLength;
  const double ndd = nonzero(dir.x * nx + dir.y * ny + dir.z * nz);
  const double saf = p.x * nx + p.y * ny + p.z * nz + dd;
  if (dgt(saf, kTolerance)) distance = -kInfLength;
  if (dgt(ndd, 0.) && dlt(saf, kTolerance)) distance = -saf / ndd;
  return distance;
}
__device__ __forceinline__ double cut_dist_in(const CutTubeRec &c, V3 p, V3 d)
{
  return dmax(cut_plane_dist_in(c.n0x, c.n0y, c.n0z, c.d0, p, d), cut_plane_dist_in(c.n1x, c.n1y, c.n1z, c.d1, p, d));
}
__device__ __forceinline__ double cut_dist_out(const CutTubeRec &c, V3 p, V3 d)
{
  return dmin(cut_plane_dist_out(c.n0x, c.n0y, c.n0z, c.d0, p, d), cut_plane_dist_out(c.n1x, c.n1y, c.n1z, c.d1, p, d));
}

// CutTubeImplementation.h:114-126 Contains
__device__ __forceinline__ bool cuttube_contains(const CutTubeRec &c, V3 p)
{
  const bool inCut = dlt(cut_dist0(c, p), 0.) && dlt(cut_dist1(c, p), 0.);
  if (!inCut) return false;
  return tube_contains(c.t, p);
}
// CutTubeImplementation.h:128-142 Inside
__device__ __forceinline__ int cuttube_inside(const CutTubeRec &c, V3 p)
{
  const int ic = cut_inside(c, p);
  if (ic == kOutside) return kOutside;
  const int it = tube_inside(c.t, p);
  return (ic == kSurface && it != kOutside) ? ic : it;
}
// CutTubeImplementation.h:171-258 DistanceToInKernel with stepMax = kInfLength: a value the
// reference gives below its stepMax does not depend on it (the cut-plane hit needs |d| <
// stepMax, the tube hit d < stepMax), so a navigator that accepts only distances below its
// current step makes the same choices as the reference's, which passes that step.
static __device__ __noinline__ double cuttube_dist_in_kernel(const CutTubeRec &c, V3 point, V3 dir)
{
  const double stepMax = kInfLength;
  double distance      = kInfLength;
  int insideCut        = cut_inside(c, point);
  int instart          = tube_inside(c.t, point);
  if (insideCut == kOutside || (insideCut == kSurface && instart != kOutside)) instart = insideCut;
  if (instart == kInside) distance = -1.;
  double dplanes         = cut_dist_in(c, point, dir);
  const double safplanes = dmax(cut_dist0(c, point), cut_dist1(c, point));
  const bool hitplanes   = dlt(fabs(dplanes), stepMax) && dgt(safplanes, -kTolerance);
  if (insideCut != kInside && !hitplanes) return distance;
  V3 propagated = point;
  if (!hitplanes) dplanes = 0.;
  if (hitplanes) {
    propagated = V3{propagated.x + dplanes * dir.x, propagated.y + dplanes * dir.y, propagated.z + dplanes * dir.z};
    insideCut  = cut_inside(c, propagated);
  }
  if (insideCut == kOutside || instart == kInside) return distance;
  const bool inside = hitplanes && (tube_inside(c.t, propagated) != kOutside);
  if (inside) {
    distance = dplanes;
    if (dabs_lt(distance, kTolerance)) distance = 0.;
    return distance;
  }
  const double dexit = cut_dist_out(c, propagated, dir);
  double dtube       = tube_dist_in_kernel(c.t, propagated, dir);
  if (dlt(dtube, 0.)) dtube = 0.;
  if (dlt(dexit, dtube)) dtube = kInfLength;
  if (dlt(dtube + dplanes, stepMax)) distance = dtube + dplanes;
  return distance;
}
// CutTubeImplementation.h:144-169 DistanceToIn (far points moved to 100 x max(rmax, dz))
__device__ __forceinline__ double cuttube_dist_in(const CutTubeRec &c, V3 p, V3 d)
{
  const double ptDist = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double distToMove   = 0.;
  if (dgt(ptDist, 100. * c.maxVal)) {
    distToMove = ptDist - 100. * c.maxVal;
    p          = V3{p.x + distToMove * d.x, p.y + distToMove * d.y, p.z + distToMove * d.z};
  }
  return cuttube_dist_in_kernel(c, p, d) + distToMove;
}
// CutTubeImplementation.h:262-280 DistanceToOut
__device__ __forceinline__ double cuttube_dist_out(const CutTubeRec &c, V3 p, V3 d)
{
  double distance    = cut_dist_out(c, p, d);
  const double dtube = tube_dist_out(c.t, p, d);
  if (dlt(dtube, distance)) distance = dtube;
  return distance;
}
// CutTubeImplementation.h:283-315 SafetyToIn / SafetyToOut
__device__ __forceinline__ double cuttube_safety_in(const CutTubeRec &c, V3 p)
{
  double safety        = dmax(cut_dist0(c, p), cut_dist1(c, p));
  const double saftube = tube_safety_in(c.t, p);
  if (dgt(saftube, safety)) safety = saftube;
  return safety;
}
__device__ __forceinline__ double cuttube_safety_out(const CutTubeRec &c, V3 p)
{
  double safety        = dmin(-cut_dist0(c, p), -cut_dist1(c, p));
  const double saftube = tube_safety_out(c.t, p);
  if (dlt(saftube, safety)) safety = saftube;
  return safety;
}

// ================================================================ Cone
__device__ __forceinline__ bool cone_phi(const ConeRec &c) { return dlt(c.dphi, kTwoPi); }
__device__ __forceinline__ bool cone_rmin(const ConeRec &c) { return dgt(c.rmin1, 0.) || dgt(c.rmin2, 0.); }
// ConeUtilities.h:113-131
__device__ __forceinline__ double cone_radius(const ConeRec &c, double z, bool inner)
{
  if (inner) return deq(c.rmin1, c.rmin2) ? c.rmin1 : c.innerSlope * z + c.innerOffset;
  return deq(c.origRmax1, c.origRmax2) ? c.origRmax1 : c.outerSlope * z + c.outerOffset;
}
// ConeUtilities.h:70-108 (kConeTolerance band)
__device__ __forceinline__ bool cone_in_sector(const ConeRec &c, double x, double y, bool includeSurface)
{
  const double startCheck = (-x * c.a1y) + (y * c.a1x);
  const double endCheck   = (-c.a2x * y) + (c.a2y * x);
  const double tol        = includeSurface ? -kConeTolerance : kConeTolerance;
  if (dle(c.dphi, kPi)) return dge(startCheck, tol) && dge(endCheck, tol);
  return dge(startCheck, tol) || dge(endCheck, tol);
}
// ConeUtilities.h:176-200
__device__ __forceinline__ V3 cone_normal(const ConeRec &c, V3 p, bool inner)
{
  const double rho = sqrt(perp2(p));
  if (inner) {
    if (deq(c.rmin1, c.rmin2) && dne(c.rmin1, 0.)) return V3{-p.x, -p.y, 0.};
    return V3{-p.x, -p.y, c.zNormInner * (rho * c.secRMin)};
  }
  if (deq(c.rmax1, c.rmax2) && dne(c.rmax1, 0.)) return V3{p.x, p.y, 0.};
  return V3{p.x, p.y, c.zNormOuter * (rho * c.secRMax)};
}
// ConeUtilities.h:204-216
__device__ __forceinline__ bool cone_on_surface(const ConeRec &c, V3 p, bool inner)
{
  const double rho      = perp2(p);
  const double coneRad  = cone_radius(c, p.z, inner);
  const double coneRad2 = coneRad * coneRad;
  const double tol      = inner ? c.innerTol : c.outerTol;
  return dge(rho, coneRad2 - tol * coneRad) && dle(rho, coneRad2 + tol * coneRad) &&
         dabs_lt(p.z, c.dz + kConeTolerance);
}
// ConeUtilities.h:146-174
__device__ __forceinline__ void cone_phi_plane(const ConeRec &c, double ax, double ay, double nx, double ny, V3 pos,
                                               V3 dir, bool insectorCheck, double &dist, bool &ok)
{
  dist = kInfLength;
  const double dn = (dir.x * nx) + (dir.y * ny);
  ok              = insectorCheck ? dgt(dn, 0.) : dlt(dn, 0.);
  const double dirDotXY = (dir.y * ax) - (dir.x * ay);
  if (dne(dirDotXY, 0.)) dist = ((ay * pos.x) - (ax * pos.y)) / nonzero(dirDotXY);
  ok                = ok && dgt(dist, -kConeTolerance);
  const double hitx = pos.x + dist * dir.x;
  const double hity = pos.y + dist * dir.y;
  if (insectorCheck) {
    const double hitz = pos.z + dist * dir.z;
    const double r2   = (hitx * hitx) + (hity * hity);
    const double inR  = cone_radius(c, hitz, true) + kTolerance;
    const double outR = cone_radius(c, hitz, false) - kTolerance;
    ok = ok && dabs_le(hitz, c.tolIz) && dge(r2, inR * inR) && dle(r2, outR * outR);
    ok = ok && dgt((hitx * ax) + (hity * ay), 0.);
  } else {
    ok = ok && dge((hitx * ax) + (hity * ay), 0.);
  }
}

// ConeUtilities.h:551-684 (scalar DetectIntersectionAndCalculateDistanceToConicalSurface)
static __device__ __noinline__ bool cone_conical(const ConeRec &c, V3 point, V3 dir, bool forDistToIn, bool inner,
                                          double &distance)
{
  distance           = kInfLength;
  const bool onCone  = cone_on_surface(c, point, inner);
  const double dn    = dot(dir, cone_normal(c, point, inner));
  if (onCone && deq(fabs(dn), 0.)) return false;
  if (onCone) {
    const bool moving = forDistToIn ? dle(dn, 0.) : dge(dn, 0.);
    const bool insec  = cone_phi(c) ? cone_in_sector(c, point.x, point.y, true) : true;
    if (insec && moving) {
      distance = 0.;
      return true;
    }
  }
  bool ok              = false;
  const double pDotV2D = point.x * dir.x + point.y * dir.y;
  double a, b, cc;
  if (inner) {
    if (deq(c.rmin1, c.rmin2)) {
      b  = pDotV2D;
      a  = perp2(dir);
      cc = perp2(point) - c.rmin2 * c.rmin2;
    } else {
      const double newPz = dgt(c.rmin2, c.rmin1) ? (point.z + c.dz + c.innerApex) * c.tanInnerApex
                                               : (point.z - c.dz - c.innerApex) * c.tanInnerApex;
      const double dirT  = dir.z * c.tanInnerApex;
      a                  = (dir.x * dir.x) + (dir.y * dir.y) - dirT * dirT;
      b                  = pDotV2D - (newPz * dirT);
      cc                 = perp2(point) - (newPz * newPz);
    }
    const double b2 = b * b;
    const double ac = a * cc;
    if (dlt(b2, ac)) return false;
    const double delta = sqrt(b2 - ac);
    if (forDistToIn) {
      distance = dge(b, 0.) ? (cc / nonzero(-b - delta)) : (-b + delta) / nonzero(a);
    } else {
      if (deq(b, 0.) && deq(delta, 0.)) return false;
      distance = dge(b, 0.) ? (-b - delta) / nonzero(a) : (cc / nonzero(-b + delta));
    }
    if (dlt(distance, 0.)) return false;
    ok = dabs_lt(point.z + (dir.z * distance), c.dz);
  } else {
    if (deq(c.origRmax1, c.origRmax2)) {
      a  = perp2(dir);
      b  = pDotV2D;
      cc = (perp2(point) - c.origRmax2 * c.origRmax2);
    } else {
      const double newPz = dgt(c.origRmax2, c.origRmax1) ? (point.z + c.dz + c.outerApex) * c.tanOuterApex
                                                       : (point.z - c.dz - c.outerApex) * c.tanOuterApex;
      const double dirT  = dir.z * c.tanOuterApex;
      a                  = dir.x * dir.x + dir.y * dir.y - dirT * dirT;
      b                  = (pDotV2D - (newPz * dirT));
      cc                 = (perp2(point) - (newPz * newPz));
    }
    const double d2 = b * b - a * cc;
    if (dlt(d2, 0.)) return false;
    const double delta = sqrt(d2);
    if (forDistToIn) {
      if (deq(b, 0.) && deq(delta, 0.)) return false;
      distance = dgt(b, 0.) ? (-b - delta) / nonzero(a) : (cc / nonzero(-b + delta));
      ok       = dabs_lt(point.z + (dir.z * distance), c.dz + kHalfTolerance);
    } else {
      distance = dlt(b, 0.) ? (-b + delta) / nonzero(a) : (cc / nonzero(-b - delta));
      ok       = dgt(distance, 0.);
    }
    if (dlt(distance, 0.)) return false;
  }
  if (cone_phi(c)) {
    double hitx = 0, hity = 0;
    if (dlt(distance, kInfLength)) {
      hitx = point.x + distance * dir.x;
      hity = point.y + distance * dir.y;
    }
    ok = ok && cone_in_sector(c, hitx, hity, true) && dlt(distance, kInfLength);
  }
  return ok;
}

// ConeUtilities.h:686-724
__device__ __forceinline__ void cone_classify(const ConeRec &c, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double absz = fabs(p.z);
  cout              = dgt(absz, forInside ? c.dz + kConeTolerance : c.dz);
  if (forInside) cin = dlt(absz, c.dz - kConeTolerance);
  if (cout) return;
  const double r2   = p.x * p.x + p.y * p.y;
  const double rmax = deq(c.origRmax1, c.origRmax2) ? c.origRmax1 : c.outerSlope * p.z + c.outerOffset;
  if (forInside) {
    cout = dgt(r2, rmax * (rmax + 2.0 * c.outerTol));
    cin  = cin && dlt(r2, fabs(rmax * (rmax - 2.0 * c.outerTol)));
  } else {
    cout = dgt(r2, rmax * rmax);
  }
  if (cout) return;
  if (cone_rmin(c)) {
    const double rmin = c.innerSlope * p.z + c.innerOffset;
    if (forInside) {
      cout = dle(r2, fabs(rmin * (rmin - 2.0 * c.innerTol)));
      cin  = cin && dgt(r2, rmin * (rmin + 2.0 * c.innerTol));
    } else {
      cout = dle(r2, rmin * rmin);
    }
    if (cout) return;
  }
  if (cone_phi(c)) {
    bool ci = false, co = false;
    wedge_classify(c.w, p, forInside, ci, co);
    cout = co;
    if (forInside) cin = cin && ci;
  }
}
__device__ __forceinline__ int cone_inside(const ConeRec &c, V3 p)
{
  bool cin = false, cout = false;
  cone_classify(c, p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
__device__ __forceinline__ bool cone_contains(const ConeRec &c, V3 p)
{
  bool cin = false, cout = false;
  cone_classify(c, p, false, cin, cout);
  return !cout;
}

// ConeImplementation.h:126-258
static __device__ __noinline__ double cone_dist_in(const ConeRec &c, V3 point, V3 dir)
{
  double distz = fabs(point.z) - c.dz;
  if ((dgt(distz, kConeTolerance) && dge(point.z * dir.z, 0.)) || (dabs_lt(distz, kConeTolerance) && dgt(point.z * dir.z, 0.)))
    return kInfLength;
  const double outerRad = cone_radius(c, point.z, false);
  const double rsq      = perp2(point);
  const double outerIn  = fabs(outerRad * (outerRad - 2.0 * c.outerTol));
  if (dgt(rsq, outerIn) && dge(dot(dir, cone_normal(c, point, false)), 0.)) return kInfLength;
  bool inside = dlt(distz, -kConeTolerance) && dlt(rsq, outerIn);
  if (cone_rmin(c)) {
    const double innerRad = cone_radius(c, point.z, true);
    inside                = inside && dgt(rsq, innerRad * (innerRad + 2.0 * c.innerTol));
  }
  if (cone_phi(c)) inside = inside && cone_in_sector(c, point.x, point.y, false);
  if (inside) return -1.0;

  double distance = kInfLength;
  distz /= nonzero(fabs(dir.z));
  const double hitx = point.x + distz * dir.x;
  const double hity = point.y + distz * dir.y;
  const double r2   = (hitx * hitx) + (hity * hity);
  bool top          = dge(point.z, c.tolIz) && dle(r2, c.sqRmax2 + kTolerance);
  bool bottom       = dle(point.z, -c.tolIz) && dle(r2, c.sqRmax1 + kTolerance);
  bool okz          = top || bottom;
  if (cone_rmin(c)) {
    top    = top && dge(r2, c.sqRmin2 - kTolerance);
    bottom = bottom && dge(r2, c.sqRmin1 - kTolerance);
    okz    = okz && (top || bottom);
  }
  if (cone_phi(c)) okz = okz && cone_in_sector(c, hitx, hity, true);
  if (okz) return distz;

  double dist_rOuter;
  if (cone_conical(c, point, dir, true, false, dist_rOuter) && dlt(dist_rOuter, distance)) return dist_rOuter;
  if (cone_rmin(c)) {
    double dist_rInner;
    if (cone_conical(c, point, dir, true, true, dist_rInner) && dlt(dist_rInner, distance)) distance = dist_rInner;
  }
  if (cone_phi(c)) {
    double dist_phi;
    bool ok_phi;
    cone_phi_plane(c, c.a1x, c.a1y, c.w.n1x, c.w.n1y, point, dir, true, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
    cone_phi_plane(c, c.a2x, c.a2y, c.w.n2x, c.w.n2y, point, dir, true, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
  }
  return distance;
}

// ConeImplementation.h:260-370
static __device__ __noinline__ double cone_dist_out(const ConeRec &c, V3 point, V3 dir)
{
  const double distz    = fabs(point.z) - c.dz;
  const double rsq      = perp2(point);
  const double outerRad = cone_radius(c, point.z, false);
  if (dgt(distz, kConeTolerance) || dgt(rsq, outerRad * (outerRad + 2.0 * c.outerTol))) return -1.0;
  if (cone_rmin(c)) {
    const double innerRad = cone_radius(c, point.z, true);
    if (dlt(rsq, fabs(innerRad * (innerRad - 2.0 * c.innerTol)))) return -1.0;
  }
  // (no phi-sector rejection on the scalar path, see ConeImplementation.h:292-296)
  const bool up   = dgt(dir.z, 0.);
  const bool down = dlt(dir.z, 0.);
  if ((up && dgt(point.z, 0.) && dabs_lt(distz, kConeTolerance)) || (down && dlt(point.z, 0.) && dabs_lt(distz, kConeTolerance)))
    return distz;
  double distance      = kInfLength;
  const double dirZInv = 1. / nonzero(dir.z);
  if (up) distance = (c.dz - point.z) * dirZInv;
  if (down) distance = (-c.dz - point.z) * dirZInv;
  double dist_rOuter;
  if (cone_conical(c, point, dir, false, false, dist_rOuter) && dlt(dist_rOuter, distance)) distance = dist_rOuter;
  if (cone_rmin(c)) {
    double dist_rInner;
    if (cone_conical(c, point, dir, false, true, dist_rInner) && dlt(dist_rInner, distance)) distance = dist_rInner;
  }
  if (cone_phi(c)) {
    const bool onStart = wedge_on_surface(c.w.a1x, c.w.a1y, c.w.n1x, c.w.n1y, point);
    const bool onEnd   = wedge_on_surface(c.w.a2x, c.w.a2y, c.w.n2x, c.w.n2y, point);
    const double dn1   = dir.x * (-c.w.n1x) + dir.y * (-c.w.n1y) + dir.z * (-0.0);
    const double dn2   = dir.x * (-c.w.n2x) + dir.y * (-c.w.n2y) + dir.z * (-0.0);
    if ((onStart && dgt(dn1, 0.)) || (onEnd && dgt(dn2, 0.))) return 0.;
    double dist_phi;
    bool ok_phi;
    cone_phi_plane(c, c.a1x, c.a1y, c.w.n1x, c.w.n1y, point, dir, false, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
    cone_phi_plane(c, c.a2x, c.a2y, c.w.n2x, c.w.n2y, point, dir, false, dist_phi, ok_phi);
    if (ok_phi && dlt(dist_phi, distance)) distance = dist_phi;
  }
  if (dlt(distance, 0.) && dabs_lt(distance, kTolerance)) distance = 0.;
  return distance;
}

// ConeImplementation.h:498-516
__device__ __forceinline__ double cone_safe_conical(const ConeRec &c, V3 p, bool inner)
{
  const double rho = sqrt(perp2(p));
  if (inner) return (rho - (c.tanRMin * p.z + (c.rmin1 + c.rmin2) * 0.5)) * c.invSecRMin;
  return ((c.tanRMax * p.z + (c.rmax1 + c.rmax2) * 0.5) - rho) * c.invSecRMax;
}

// ConeImplementation.h:372-436
__device__ __forceinline__ double cone_safety_in(const ConeRec &c, V3 p)
{
  const double distz    = fabs(p.z) - c.dz;
  const double outerRad = cone_radius(c, p.z, false);
  const double rsq      = perp2(p);
  bool inside           = dlt(distz, -kConeTolerance) && dlt(rsq, fabs(outerRad * (outerRad - 2.0 * c.outerTol)));
  if (cone_rmin(c)) {
    const double innerRad = cone_radius(c, p.z, true);
    inside                = inside && dgt(rsq, innerRad * (innerRad + 2.0 * c.innerTol));
  }
  if (cone_phi(c) && inside) inside = cone_in_sector(c, p.x, p.y, false);
  if (inside) return -1.0;
  const double safeOuter = -cone_safe_conical(c, p, false);
  const double safeInner = cone_rmin(c) ? -cone_safe_conical(c, p, true) : -kInfLength;
  double safety          = dmax(distz, dmax(safeOuter, safeInner));
  if (cone_phi(c)) safety = dmax(wedge_safety_in(c.w, p), safety);
  if (dabs_lt(safety, kTolerance)) safety = 0.;
  return safety;
}

// ConeImplementation.h:437-496
__device__ __forceinline__ double cone_safety_out(const ConeRec &c, V3 p)
{
  const double distz    = fabs(p.z) - c.dz;
  const double rsq      = perp2(p);
  const double outerRad = cone_radius(c, p.z, false);
  bool outside          = dgt(distz, kConeTolerance) || dgt(rsq, outerRad * (outerRad + 2.0 * c.outerTol));
  if (cone_rmin(c)) {
    const double innerRad = cone_radius(c, p.z, true);
    outside               = outside || dlt(rsq, fabs(innerRad * (innerRad - 2.0 * c.innerTol)));
  }
  if (outside) return -1.0;
  const double safeOuter = cone_safe_conical(c, p, false);
  const double safeInner = cone_rmin(c) ? cone_safe_conical(c, p, true) : kInfLength;
  double safety          = dmin(c.dz - fabs(p.z), dmin(safeOuter, safeInner));
  if (cone_phi(c)) safety = dmin(wedge_safety_out(c.w, p), safety);
  if (dabs_lt(safety, kTolerance)) safety = 0.;
  return safety;
}

} // namespace f64
} // namespace vg
