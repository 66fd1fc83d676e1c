// FP64 Sphere kernels on the flattened record (SphereRec, vg_types.h): the scalar path of
// VecGeom/volumes/kernel/SphereImplementation.h with SphereUtilities.h, the phi Wedge
// (Wedge_Evolution.h) and the ThetaCone (ThetaCone_Evolution.h), in the reference's
// operation order, so results are bit-identical in FP64.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {
namespace f64 {

constexpr double kSqrtTolerance = 3.1622777e-5; // VecGeom/base/Math.h:29
constexpr double kHalfPiS       = 0.5 * kPi;    // ThetaCone_Evolution.h:18

__device__ __forceinline__ double sph_mag2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V3 sph_add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 sph_scale(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 sph_neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
// GenericKernels.h:62-82
__device__ __forceinline__ double plus_tol_sq(double x) { return x * (x + 2.0 * kTolerance); }
__device__ __forceinline__ double minus_tol_sq(double x) { return fabs(x * (x - 2.0 * kTolerance)); }

// ---------------------------------------------------------------- ThetaCone
// IsOnSurfaceGeneric<ForStartTheta> (ThetaCone_Evolution.h:154-169)
__device__ __forceinline__ bool tc_on_surface(const SphereRec &s, V3 p, bool start)
{
  const double rhs  = start ? fabs(s.tanS * p.z) : fabs(s.tanE * p.z);
  const double rho2 = perp2(p);
  return rho2 >= minus_tol_sq(rhs) && rho2 <= plus_tol_sq(rhs);
}
// GetNormal<ForStartTheta> (:131-146)
__device__ __forceinline__ V3 tc_normal(const SphereRec &s, V3 p, bool start)
{
  if (start) {
    const V3 n{p.x, p.y, -s.tanS2 * p.z};
    return (s.tcS <= kHalfPiS) ? sph_neg(n) : n;
  }
  const V3 n{p.x, p.y, -s.tanE2 * p.z};
  return (s.tcE <= kHalfPiS) ? n : sph_neg(n);
}
__device__ __forceinline__ bool tc_moving(const SphereRec &s, V3 p, V3 d, bool start, bool movingOut)
{
  if (movingOut) return tc_on_surface(s, p, start) && (dot(d, tc_normal(s, p, start)) > 0.);
  return tc_on_surface(s, p, start) && (dot(d, tc_normal(s, p, start)) < 0.);
}
__device__ __forceinline__ double tc_line(double slope, double x, double y) // :323-330
{
  const double dist = (y - slope * x) / sqrt(1. + slope * slope);
  return fabs(dist);
}
// IsCompletelyInside (:622-690)
static __device__ __noinline__ bool tc_inside(const SphereRec &s, V3 p)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance, kAng = kTolerance;
  const double rho = sqrt(sph_mag2(p) - (p.z * p.z));
  const double c1  = fabs(p.z * s.tanS);
  const double c2  = fabs(p.z * s.tanE);
  const bool onZ   = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool onXY  = p.z == 0. && (p.x != 0. || p.y != 0.);
  bool ci = (onZ && ((fS == 0. && fE == kPi) || (p.z > 0. && fS == 0.) || (p.z < 0. && fE == kPi)));
  ci = ci || (!ci && (onXY && (fS < kHalfPiS && fE > kHalfPiS && (kHalfPiS - fS) > kAng && (fE - kHalfPiS) > kTolerance)));
  if (fS < kHalfPiS + hT) {
    if (fE < kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 + (2 * kAng * 10.), hi = c2 - (2 * kAng * 10.);
        ci = ci || (!ci && (((rho <= hi) && (rho >= lo) && (p.z > 0.) && (fS != 0.)) ||
                            ((rho <= hi) && (fS == 0.) && (p.z > 0.))));
      }
    }
    if (fE > kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 + (2 * kAng * 10.), hi = c2 + (2 * kAng * 10.);
        ci = ci || (!ci && (((rho >= lo) && (p.z > 0.)) || ((rho >= hi) && (p.z < 0.))));
      }
    }
    if (fE >= kHalfPiS - hT && fE <= kHalfPiS + hT) ci = ci && !(fabs(p.z) < hT);
  }
  if (fE > kHalfPiS + hT) {
    if (fS >= kHalfPiS - hT && fS <= kHalfPiS + hT) ci = ci && !(fabs(p.z) < hT);
    if (fS > kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 - (2 * kAng * 10.), hi = c2 + (2 * kAng * 10.);
        ci = ci || (!ci && (((rho <= lo) && (rho >= hi) && (p.z < 0.) && (fE != kPi)) ||
                            ((rho <= lo) && (p.z < 0.) && (fE == kPi))));
      }
    }
  }
  return ci;
}
// IsCompletelyOutside (:692-760)
static __device__ __noinline__ bool tc_outside(const SphereRec &s, V3 p)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance, kAng = kTolerance;
  const double rho = sqrt(perp2(p));
  const double c1  = fabs(p.z * s.tanS);
  const double c2  = fabs(p.z * s.tanE);
  const bool onZ   = p.z != 0. && p.x == 0. && p.y == 0.;
  const bool onXY  = p.z == 0. && (p.x != 0. || p.y != 0.);
  bool co = (onZ && (((fS != 0.) && (fE != kPi)) || (p.z > 0. && (fS != 0.)) || (p.z < 0. && (fE != kPi))));
  co = co || (!co && (onXY && (((fS < kHalfPiS) && (fE < kHalfPiS) && ((kHalfPiS - fS) > kAng) && ((kHalfPiS - fE) > kTolerance)) ||
                               ((fS > kHalfPiS && fE > kHalfPiS) && ((fS - kHalfPiS) > kAng) && ((fE - kHalfPiS) > kTolerance)))));
  if (fS < kHalfPiS + hT) {
    if (fE < kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 - (2 * kAng * 10.), hi = c2 + (2 * kAng * 10.);
        co = co || (!co && ((rho < lo) || (rho > hi) || (p.z < 0.)));
      }
    }
    if (fE > kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 - (2 * kAng * 10.), hi = c2 - (2 * kAng * 10.);
        co = co || (!co && (((rho < lo) && (p.z > 0.)) || ((rho < hi) && (p.z < 0.))));
      }
    }
    if (fE >= kHalfPiS - hT && fE <= kHalfPiS + hT) co = co && !(fabs(p.z) < hT);
  }
  if (fE > kHalfPiS + hT) {
    if (fS >= kHalfPiS - hT && fS <= kHalfPiS + hT) co = co && !(fabs(p.z) < hT);
    if (fS > kHalfPiS + hT) {
      if (fS < fE) {
        const double lo = c1 + (2 * kAng * 10.), hi = c2 - (2 * kAng * 10.);
        co = co || (!co && ((rho < hi) || (rho > lo) || (p.z > 0.)));
      }
    }
  }
  return co;
}
__device__ __forceinline__ bool tc_contains(const SphereRec &s, V3 p) { return !tc_outside(s, p); }
// SafetyToIn (:237-281)
static __device__ __noinline__ double tc_safety_in(const SphereRec &s, V3 p)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance;
  const double rad   = sqrt(p.x * p.x + p.y * p.y);
  const double sfTh1 = tc_line(s.slope1, rad, p.z);
  const double sfTh2 = tc_line(s.slope2, rad, p.z);
  double safeTheta   = dmin(sfTh1, sfTh2);
  if (tc_contains(s, p)) return 0.;
  if (fS < kPi / 2 + hT) {
    if (fE < kPi / 2 + hT) {
      if (fS < fE) {
        if (p.z < 0.) safeTheta = sfTh2;
      }
    }
    if (fE > kPi / 2 + hT) {
      if (fS < fE) {
        if (p.z > 0.) safeTheta = sfTh1;
        if (p.z < 0.) safeTheta = sfTh2;
      }
    }
  }
  if (fE > kPi / 2 + hT) {
    if (fS > kPi / 2 + hT) {
      if (fS < fE) {
        if (p.z > 0.) safeTheta = sfTh1;
      }
    }
  }
  return safeTheta;
}
// SafetyToOut (:283-321)
static __device__ __noinline__ double tc_safety_out(const SphereRec &s, V3 p)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance;
  const double rad         = sqrt(p.x * p.x + p.y * p.y);
  const double bisectorRad = fabs(p.z * s.tanBis);
  bool condition           = false;
  const double sfTh1       = tc_line(s.slope1, rad, p.z);
  const double sfTh2       = tc_line(s.slope2, rad, p.z);
  if (fS < kPi / 2 + hT) {
    if (fE < kPi / 2 + hT) {
      if (fS < fE) condition = (rad < bisectorRad) && (fS != 0.);
    }
    if (fE > kPi / 2 + hT) {
      if (fS < fE) condition = sfTh1 < sfTh2;
    }
  }
  if (fE > kPi / 2 + hT) {
    if (fS > kPi / 2 + hT) {
      if (fS < fE) condition = !((rad < bisectorRad) && (fE != kPi));
    }
  }
  return condition ? sfTh1 : sfTh2;
}
// DistanceToIn (:340-470)
static __device__ __noinline__ void tc_dist_in(const SphereRec &s, V3 point, V3 dir, double &dist1, double &dist2,
                                               bool &intsect1, bool &intsect2)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance;
  bool done            = false;
  double firstRoot     = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = point.x * dir.x + point.y * dir.y;
  const double rho2    = point.x * point.x + point.y * point.y;
  const double dirRho2 = perp2(dir);
  const double b       = pDotV2d - point.z * dir.z * s.tanS2;
  const double a       = dirRho2 - dir.z * dir.z * s.tanS2;
  const double c       = rho2 - point.z * point.z * s.tanS2;
  const double d2      = b * b - a * c;
  const double aInv    = 1. / nonzero(a);
  if (d2 > 0.) firstRoot = (-b + sqrt(fabs(d2))) * aInv;
  done = done || (fabs(firstRoot) < 3. * kTolerance);
  if (fabs(firstRoot) < 3. * kTolerance) firstRoot = 0.;
  if (!done && (firstRoot < 0.)) firstRoot = kInfLength;
  const double b2    = pDotV2d - point.z * dir.z * s.tanE2;
  const double a2    = dirRho2 - dir.z * dir.z * s.tanE2;
  const double c2    = rho2 - point.z * point.z * s.tanE2;
  const double d22   = b2 * b2 - a2 * c2;
  const double a2Inv = 1. / nonzero(a2);
  if (d22 > 0.) secondRoot = (-b2 - sqrt(fabs(d22))) * a2Inv;
  if (!done && (fabs(secondRoot) < 3. * kTolerance)) secondRoot = 0.;
  done = done || (fabs(secondRoot) < 3. * kTolerance);
  if (!done && (secondRoot < 0.)) secondRoot = kInfLength;
  if (fS < kHalfPiS + hT) {
    if (fE < kHalfPiS + hT) {
      if (fS < fE) {
        dist1           = firstRoot;
        dist2           = secondRoot;
        const double z1 = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
        intsect1        = ((d2 > 0.) && (z1 > 0.));
        intsect2        = ((d22 > 0.) && (z2 > 0.));
      }
    }
    if (fE >= kHalfPiS - hT && fE <= kHalfPiS + hT) {
      if (dir.z > 0.) dist2 = -point.z / dir.z;
      const double z2 = (point.z + dist2 * dir.z);
      intsect2        = ((dist2 != kInfLength) && (fabs(z2) < hT));
    }
    if (fE > kHalfPiS + hT) {
      if (fS < fE) {
        dist1 = firstRoot;
        if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
        done = false;
        done = done || (fabs(secondRoot) < 3. * kTolerance);
        if (fabs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
        if (!done && (secondRoot < 0.)) secondRoot = kInfLength;
        dist2           = secondRoot;
        const double z1 = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
        intsect1        = ((d2 > 0) && (dist1 != kInfLength) && (z1 > 0.));
        intsect2        = ((d22 > 0) && (dist2 != kInfLength) && (z2 < 0.));
      }
    }
  }
  if (fS >= kHalfPiS - hT) {
    if (fE > kHalfPiS + hT) {
      if (fS < fE) {
        if (d2 > 0.) firstRoot = (-b - sqrt(fabs(d2))) * aInv;
        done = false;
        done = done || (fabs(firstRoot) < 3. * kTolerance);
        if (fabs(firstRoot) < 3. * kTolerance) firstRoot = 0.;
        if (!done && (firstRoot < 0.)) firstRoot = kInfLength;
        dist1 = firstRoot;
        if (d22 > 0.) secondRoot = (-b2 + sqrt(fabs(d22))) * a2Inv;
        done = false;
        done = done || (fabs(secondRoot) < 3. * kTolerance);
        if (fabs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
        if (!done && (secondRoot < 0.)) secondRoot = kInfLength;
        dist2           = secondRoot;
        const double z1 = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
        intsect1        = ((d2 > 0) && (dist1 != kInfLength) && (z1 < 0.));
        intsect2        = ((d22 > 0) && (dist2 != kInfLength) && (z2 < 0.));
      }
    }
  }
  if (fS >= kHalfPiS - hT && fS <= kHalfPiS + hT) {
    if (dir.z < 0.) dist1 = -point.z / dir.z;
    const double z1 = (point.z + dist1 * dir.z);
    intsect1        = ((dist1 != kInfLength) && (fabs(z1) < hT));
  }
}
// DistanceToOut (:472-620)
static __device__ __noinline__ void tc_dist_out(const SphereRec &s, V3 point, V3 dir, double &dist1, double &dist2,
                                                bool &intsect1, bool &intsect2)
{
  const double fS = s.tcS, fE = s.tcE, hT = 0.5 * kTolerance;
  const double inf     = kInfLength;
  double firstRoot     = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = point.x * dir.x + point.y * dir.y;
  const double rho2    = point.x * point.x + point.y * point.y;
  const double b       = pDotV2d - point.z * dir.z * s.tanS2;
  const double a       = dir.x * dir.x + dir.y * dir.y - dir.z * dir.z * s.tanS2;
  const double c       = rho2 - point.z * point.z * s.tanS2;
  double d2            = b * b - a * c;
  if (d2 < 0. && fabs(d2) < kHalfTolerance) d2 = 0.;
  if ((d2 >= 0.) && b >= 0. && a != 0.) firstRoot = ((-b - sqrt(fabs(d2))) / nonzero(a));
  if ((d2 >= 0.) && b < 0.) firstRoot = ((c) / nonzero(-b + sqrt(fabs(d2))));
  if (firstRoot < 0.) firstRoot = kInfLength;
  const double b2 = point.x * dir.x + point.y * dir.y - point.z * dir.z * s.tanE2;
  const double a2 = dir.x * dir.x + dir.y * dir.y - dir.z * dir.z * s.tanE2;
  const double c2 = point.x * point.x + point.y * point.y - point.z * point.z * s.tanE2;
  double d22      = (b2 * b2) - (a2 * c2);
  if (d22 < 0. && fabs(d22) < kHalfTolerance) d22 = 0.;
  if ((d22 >= 0.) && b2 >= 0.) secondRoot = ((c2) / nonzero(-b2 - sqrt(fabs(d22))));
  if ((d22 >= 0.) && b2 < 0. && a2 != 0.) secondRoot = ((-b2 + sqrt(fabs(d22))) / nonzero(a2));
  if (secondRoot < 0. && fabs(secondRoot) > kTolerance) secondRoot = kInfLength;
  if (fabs(secondRoot) < kTolerance) secondRoot = 0.;
  if (fS < kPi / 2 + hT) {
    if (fE < kPi / 2 + hT) {
      if (fS < fE) {
        dist1                = firstRoot;
        dist2                = secondRoot;
        const double z1      = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
        intsect1             = ((d2 > 0) && (dist1 != kInfLength) && ((z1) > -kHalfTolerance));
        intsect2             = ((d22 > 0) && (dist2 != kInfLength) && ((z2) > -kHalfTolerance));
        const double dirRho2 = dir.x * dir.x + dir.y * dir.y;
        double zs            = kInfLength;
        if (fS) zs = dirRho2 / s.tanS;
        double ze = kInfLength;
        if (fE) ze = dirRho2 / s.tanE;
        const bool cond = (point.x == 0. && point.y == 0. && point.z == 0. && dir.z < zs && dir.z < ze);
        if (cond) dist1 = 0., dist2 = 0.;
        intsect1 = intsect1 || cond;
        intsect2 = intsect2 || cond;
      }
    }
    if (fE >= kPi / 2 - hT && fE <= kPi / 2 + hT) {
      dist1 = firstRoot;
      dist2 = inf;
      if (dir.z < 0.) dist2 = -1. * point.z / dir.z;
      const double z2 = (point.z + dist2 * dir.z), z1 = (point.z + dist1 * dir.z);
      intsect2 = ((dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && !(dir.z == 0.));
      intsect1 = ((d2 >= 0) && (dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && !(dir.z == 0.));
    }
    if (fE > kPi / 2 + hT) {
      if (fS < fE) {
        dist1 = firstRoot;
        if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / nonzero(a2));
        if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / nonzero(-b2 + sqrt(fabs(d22))));
        if (secondRoot < 0.) secondRoot = kInfLength;
        dist2           = secondRoot;
        const double z1 = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
        intsect1        = ((d2 >= 0) && (dist1 != kInfLength) && ((z1) > -kHalfTolerance));
        intsect2        = ((d22 >= 0) && (dist2 != kInfLength) && ((z2) < kHalfTolerance));
      }
    }
  }
  if (fE > kPi / 2 + hT) {
    if (fS < fE) {
      secondRoot = kInfLength;
      if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - sqrt(fabs(d22))) / nonzero(a2));
      if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / nonzero(-b2 + sqrt(fabs(d22))));
      dist2 = secondRoot;
      if (fS > kPi / 2 + hT) {
        if ((d2 >= 0.) && b > 0.) firstRoot = ((c) / nonzero(-b - sqrt(fabs(d2))));
        if ((d2 >= 0.) && b <= 0. && a != 0.) firstRoot = ((-b + sqrt(fabs(d2))) / nonzero(a));
        if (firstRoot < 0.) firstRoot = kInfLength;
        dist1                = firstRoot;
        const double z1      = (point.z + dist1 * dir.z);
        intsect1             = ((d2 > 0) && (dist1 != kInfLength) && ((z1) < kHalfTolerance));
        const double z2      = (point.z + dist2 * dir.z);
        intsect2             = ((d22 > 0) && (dist2 != kInfLength) && ((z2) < kHalfTolerance));
        const double dirRho2 = dir.x * dir.x + dir.y * dir.y;
        double zs            = -kInfLength;
        if (s.tanS) zs = -dirRho2 / s.tanS;
        double ze = -kInfLength;
        if (s.tanE) ze = -dirRho2 / s.tanE;
        const bool cond = (point.x == 0. && point.y == 0. && point.z == 0. && dir.z > zs && dir.z > ze);
        if (cond) dist1 = 0., dist2 = 0.;
        intsect1 = intsect1 || cond;
        intsect2 = intsect2 || cond;
      }
    }
  }
  if (fS >= kPi / 2 - hT && fS <= kPi / 2 + hT) {
    dist2 = secondRoot;
    dist1 = kInfLength;
    if (dir.z > 0.) dist1 = -1. * point.z / nonzero(dir.z);
    const double z1 = (point.z + dist1 * dir.z), z2 = (point.z + dist2 * dir.z);
    intsect1 = ((dist1 != kInfLength) && (fabs(z1) < kHalfTolerance) && (dir.z != 0.));
    intsect2 = ((d22 >= 0) && (dist2 != kInfLength) && (fabs(z2) < kHalfTolerance) && (dir.z != 0.));
  }
}

// ---------------------------------------------------------------- Sphere
__device__ __forceinline__ bool sph_full_phi(const SphereRec &s) { return s.fullPhi != 0.; }
__device__ __forceinline__ bool sph_full_theta(const SphereRec &s) { return s.fullTheta != 0.; }
__device__ __forceinline__ bool sph_wedge_contains(const SphereRec &s, V3 p)
{
  bool ci = false, co = false;
  wedge_classify(s.w, p, false, ci, co);
  return !co;
}
// SphereImplementation.h:87-131 GenericKernelForContainsAndInside
__device__ __forceinline__ void sphere_classify(const SphereRec &s, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double rad2 = sph_mag2(p);
  if (s.rmin)
    cin = rad2 <= minus_tol_sq(s.rmax) && rad2 >= plus_tol_sq(s.rmin);
  else
    cin = rad2 <= minus_tol_sq(s.rmax);
  if (s.rmin)
    cout = rad2 >= plus_tol_sq(s.rmax) || rad2 <= minus_tol_sq(s.rmin);
  else
    cout = rad2 >= plus_tol_sq(s.rmax);
  if (!sph_full_phi(s)) {
    bool ci = false, co = false;
    wedge_classify(s.w, p, forInside, ci, co);
    cout = cout || co;
    if (forInside) cin = cin && ci;
  }
  if (!sph_full_theta(s)) {
    const bool ci = forInside ? tc_inside(s, p) : false;
    const bool co = tc_outside(s, p);
    cout          = cout || co;
    if (forInside) cin = cin && ci;
  }
}
__device__ __forceinline__ int sphere_inside(const SphereRec &s, V3 p)
{
  bool ci = false, co = false;
  sphere_classify(s, p, true, ci, co);
  return ci ? kInside : (co ? kOutside : kSurface);
}
__device__ __forceinline__ bool sphere_contains(const SphereRec &s, V3 p)
{
  bool ci = false, co = false;
  sphere_classify(s, p, false, ci, co);
  return !co;
}
// SphereUtilities.h:148-164 / :128-146 (wedge and theta cone consulted in every case)
__device__ __forceinline__ bool sph_completely_inside(const SphereRec &s, V3 p)
{
  const double rad = sqrt(sph_mag2(p));
  const bool inRad = (rad < (s.rmax - kTolerance)) && (rad > (s.rmin + kTolerance));
  bool ci = false, co = false;
  wedge_classify(s.w, p, true, ci, co);
  return inRad && ci && tc_inside(s, p);
}
__device__ __forceinline__ bool sph_completely_outside(const SphereRec &s, V3 p)
{
  const double rad  = sqrt(sph_mag2(p));
  const bool outRad = (rad > (s.rmax + kTolerance)) || (rad < (s.rmin - kTolerance));
  bool ci = false, co = false;
  wedge_classify(s.w, p, true, ci, co);
  return outRad || co || tc_outside(s, p);
}
// Wedge_Evolution.h:236-245 IsPointOnSurfaceAndMovingOut (dot with the 3-vector -normal, z = 0)
__device__ __forceinline__ bool sph_wedge_moving(const SphereRec &s, V3 p, V3 d, bool start, bool movingOut)
{
  const double ax = start ? s.w.a1x : s.w.a2x, ay = start ? s.w.a1y : s.w.a2y;
  const double nx = start ? s.w.n1x : s.w.n2x, ny = start ? s.w.n1y : s.w.n2y;
  const bool on   = wedge_on_surface(ax, ay, nx, ny, p);
  const double dt = d.x * -nx + d.y * -ny + d.z * -0.;
  return movingOut ? (on && dt > 0.005 * kHalfTolerance) : (on && dt < 0.005 * kHalfTolerance);
}
// SphereUtilities.h:166-221 IsPointOnSurfaceAndMovingOut
static __device__ __noinline__ bool sph_on_surface_moving(const SphereRec &s, V3 p, V3 d, bool movingOut)
{
  auto onRadius = [&](double r) {
    const double m2 = sph_mag2(p);
    return m2 <= plus_tol_sq(r) && m2 >= minus_tol_sq(r);
  };
  auto radial = [&](bool inner) {
    if (movingOut) {
      if (inner) return onRadius(s.rmin) && (dot(d, sph_neg(p)) > kSqrtTolerance);
      return onRadius(s.rmax) && (dot(d, p) > kSqrtTolerance);
    }
    if (inner) return onRadius(s.rmin) && (dot(d, sph_neg(p)) < -kSqrtTolerance);
    return onRadius(s.rmax) && (dot(d, p) < -kSqrtTolerance);
  };
  const bool outerRad = radial(false);
  bool innerRad = false, sPhi = false, ePhi = false, sTh = false, eTh = false;
  if (s.rmin) innerRad = radial(true);
  if (s.dphi < (kTwoPi - kHalfTolerance)) {
    sPhi = sph_wedge_moving(s, p, d, true, movingOut);
    ePhi = sph_wedge_moving(s, p, d, false, movingOut);
  }
  if (s.dtheta < (kPi - kHalfTolerance)) {
    sTh = tc_moving(s, p, d, true, movingOut);
    eTh = tc_moving(s, p, d, false, movingOut);
  }
  return ((outerRad || innerRad) && sph_wedge_contains(s, p) && tc_contains(s, p)) ||
         ((sPhi || ePhi) && (sph_mag2(p) >= s.rmin * s.rmin) && (sph_mag2(p) <= s.rmax * s.rmax) && tc_contains(s, p)) ||
         ((sTh || eTh) && (sph_mag2(p) >= s.rmin * s.rmin) && (sph_mag2(p) <= s.rmax * s.rmax) &&
          sph_wedge_contains(s, p));
}
// Wedge_Evolution.h:391-432 DistanceToIn / DistanceToOut
__device__ __forceinline__ void sph_wedge_dist(const SphereRec &s, V3 p, V3 d, bool toIn, double &d1, double &d2)
{
  const WedgeRec &w  = s.w;
  d1                 = kInfLength;
  d2                 = kInfLength;
  const double comp1 = d.x * w.n1x + d.y * w.n1y;
  const double comp2 = d.x * w.n2x + d.y * w.n2y;
  if (toIn ? comp1 > 0. : comp1 < 0.) {
    const double tmp = -(p.x * w.n1x + p.y * w.n1y) / comp1;
    if (tmp > 0.) d1 = tmp;
  }
  if (toIn ? comp2 > 0. : comp2 < 0.) {
    const double tmp = -(p.x * w.n2x + p.y * w.n2y) / comp2;
    if (tmp > 0.) d2 = tmp;
  }
}
// SphereImplementation.h:326-366 GetMinDistFromPhi
static __device__ __noinline__ void sph_min_dist_phi(const SphereRec &s, V3 p, V3 d, bool toIn, double &distance)
{
  double distPhi1 = kInfLength, distPhi2 = kInfLength;
  sph_wedge_dist(s, p, d, toIn, distPhi1, distPhi2);
  const WedgeRec &w = s.w;
  double dist       = dmin(distPhi1, distPhi2);
  V3 tmp            = sph_add(p, sph_scale(dist, d));
  double rad2       = sph_mag2(tmp);
  bool tempCond     = ((dist == distPhi1) && wedge_on_surface(w.a1x, w.a1y, w.n1x, w.n1y, tmp)) ||
                  ((dist == distPhi2) && wedge_on_surface(w.a2x, w.a2y, w.n2x, w.n2y, tmp));
  const bool c1 = tempCond && (rad2 > s.rmin * s.rmin) && (rad2 < s.rmax * s.rmax) && tc_contains(s, tmp);
  if (c1) distance = dmin(dist, distance);
  dist     = dmax(distPhi1, distPhi2);
  tmp      = sph_add(p, sph_scale(dist, d));
  rad2     = sph_mag2(tmp);
  tempCond = ((dist == distPhi1) && wedge_on_surface(w.a1x, w.a1y, w.n1x, w.n1y, tmp)) ||
             ((dist == distPhi2) && wedge_on_surface(w.a2x, w.a2y, w.n2x, w.n2y, tmp));
  const bool c2 = tempCond && (rad2 > s.rmin * s.rmin) && (rad2 < s.rmax * s.rmax) && tc_contains(s, tmp);
  if ((!c1) && c2) distance = dmin(dist, distance);
}
// SphereImplementation.h:133-245 DistanceToIn
static __device__ __noinline__ double sphere_dist_in(const SphereRec &s, V3 point, V3 direction)
{
  double distance      = kInfLength;
  const double rad2    = sph_mag2(point);
  const double pDotV3d = dot(point, direction);
  double c             = rad2 - s.rmax * s.rmax;
  if (sph_completely_inside(s, point)) return -1.0;
  if (sph_on_surface_moving(s, point, direction, false)) return 0.0;
  double sd1 = kInfLength, sd2 = kInfLength;
  double d2  = (pDotV3d * pDotV3d - c);
  if (d2 < 0. || ((c > 0.) && (pDotV3d > 0.))) return distance;
  if (d2 >= 0.) sd1 = (-pDotV3d - sqrt(fabs(d2)));
  double outerDist = kInfLength, innerDist = kInfLength;
  const bool full  = s.fullSphere != 0.;
  if (full) {
    if (sd1 >= 0.) outerDist = sd1;
  } else {
    const V3 tmp = sph_add(point, sph_scale(sd1, direction));
    if (sph_wedge_contains(s, tmp) && tc_contains(s, tmp) && (sd1 >= 0.)) outerDist = sd1;
  }
  if (s.rmin) {
    c  = rad2 - s.rmin * s.rmin;
    d2 = pDotV3d * pDotV3d - c;
    if (d2 >= 0.) sd2 = (-pDotV3d + sqrt(fabs(d2)));
    if (full) {
      if (sd2 >= 0.) innerDist = sd2;
    } else {
      const V3 tmp = sph_add(point, sph_scale(sd2, direction));
      if ((sd2 >= 0.) && sph_wedge_contains(s, tmp) && tc_contains(s, tmp)) innerDist = sd2;
    }
  }
  distance = dmin(outerDist, innerDist);
  if (!sph_full_phi(s)) sph_min_dist_phi(s, point, direction, true, distance);
  double distThetaMin = kInfLength;
  if (!sph_full_theta(s)) {
    bool i1 = false, i2 = false;
    double t1 = kInfLength, t2 = kInfLength;
    tc_dist_in(s, point, direction, t1, t2, i1, i2);
    const V3 q1     = sph_add(point, sph_scale(t1, direction));
    const V3 q2     = sph_add(point, sph_scale(t2, direction));
    const double r1 = sph_mag2(q1), r2 = sph_mag2(q2);
    bool v1         = (r1 >= s.rmin * s.rmin && r1 <= s.rmax * s.rmax) && i1;
    bool v2         = (r2 >= s.rmin * s.rmin && r2 <= s.rmax * s.rmax) && i2;
    if (!sph_full_phi(s)) {
      v1 = v1 && sph_wedge_contains(s, q1);
      v2 = v2 && sph_wedge_contains(s, q2);
    }
    if (v2 && !v1) distThetaMin = t2;
    if (v1 && !v2) distThetaMin = t1;
    if (v1 && v2) distThetaMin = dmin(t1, t2);
  }
  distance             = dmin(distThetaMin, distance);
  const V3 directDir   = V3{0. - point.x, 0. - point.y, 0. - point.z};
  const double newDist = sqrt(sph_mag2(directDir));
  const double un      = sqrt(sph_mag2(directDir) + kMinimum); // Vector3D::Unit (Vector3D.h:284-290)
  const V3 u           = V3{directDir.x / un, directDir.y / un, directDir.z / un};
  if ((s.stheta > kHalfTolerance || s.eTheta < (kPi - kHalfTolerance)) && (fabs(u.x - direction.x) < kHalfTolerance) &&
      (fabs(u.y - direction.y) < kHalfTolerance) && (fabs(u.z - direction.z) < kHalfTolerance))
    distance = dmin(distance, newDist);
  return distance;
}
// SphereImplementation.h:247-324 DistanceToOut
static __device__ __noinline__ double sphere_dist_out(const SphereRec &s, V3 point, V3 direction)
{
  const double pDotV3d = dot(point, direction);
  const double rad2    = sph_mag2(point);
  double c             = rad2 - s.rmax * s.rmax;
  double sd1 = kInfLength, sd2 = kInfLength;
  if (sph_completely_outside(s, point)) return -1.0;
  if (sph_on_surface_moving(s, point, direction, true)) return 0.0;
  double d2 = (pDotV3d * pDotV3d - c);
  if (d2 >= 0.) sd1 = (-pDotV3d + sqrt(fabs(d2)));
  if (s.rmin) {
    c  = rad2 - s.rmin * s.rmin;
    d2 = (pDotV3d * pDotV3d - c);
    if ((d2 >= 0.) && (pDotV3d < 0.)) sd2 = (-pDotV3d - sqrt(fabs(d2)));
  }
  const double snxt   = dmin(sd1, sd2);
  const bool condSemi = ((s.stheta == 0. && s.eTheta == kPi / 2.) && direction.z >= 0.) ||
                        ((s.stheta == kPi / 2. && s.eTheta == kPi) && direction.z <= 0.);
  if (condSemi) return snxt;
  double distThetaMin = kInfLength;
  if (!sph_full_theta(s)) {
    bool i1 = false, i2 = false;
    double t1 = kInfLength, t2 = kInfLength;
    tc_dist_out(s, point, direction, t1, t2, i1, i2);
    if (i2 && !i1) distThetaMin = t2;
    if (!i2 && i1) distThetaMin = t1;
    if (i2 && i1) distThetaMin = dmin(t1, t2);
  }
  double distance = dmin(distThetaMin, snxt);
  if (!sph_full_phi(s)) {
    if (s.dphi <= kPi) {
      double dp1, dp2;
      sph_wedge_dist(s, point, direction, false, dp1, dp2);
      distance = dmin(dmin(dp1, dp2), distance);
    } else {
      sph_min_dist_phi(s, point, direction, false, distance);
    }
  }
  return distance;
}
// SphereImplementation.h:368-446 SafetyToIn / SafetyToOut
static __device__ __noinline__ double sphere_safety_in(const SphereRec &s, V3 point)
{
  const double rad = sqrt(sph_mag2(point));
  bool ci = false, co = false;
  sphere_classify(s, point, true, ci, co);
  if (ci) return -1.0;
  if (!ci && !co) return 0.0;
  double safety;
  if (s.rmin) {
    const double safeRMin = s.rmin - rad, safeRMax = rad - s.rmax;
    safety                = (safeRMin > safeRMax) ? safeRMin : safeRMax;
  } else {
    safety = (rad - s.rmax);
  }
  if (!sph_full_phi(s)) safety = dmax(wedge_safety_in(s.w, point), safety);
  if (!sph_full_theta(s)) safety = dmax(tc_safety_in(s, point), safety);
  return safety;
}
static __device__ __noinline__ double sphere_safety_out(const SphereRec &s, V3 point)
{
  const double rad = sqrt(sph_mag2(point));
  bool ci = false, co = false;
  sphere_classify(s, point, true, ci, co);
  if (co) return -1.0;
  if (!ci && !co) return 0.0;
  double safety;
  if (s.rmin) {
    const double safeRMin = (rad - s.rmin), safeRMax = (s.rmax - rad);
    safety                = (safeRMin < safeRMax) ? safeRMin : safeRMax;
  } else {
    safety = (s.rmax - rad);
  }
  if (!sph_full_phi(s)) safety = dmin(wedge_safety_out(s.w, point), safety);
  if (!sph_full_theta(s)) safety = dmin(tc_safety_out(s, point), safety);
  return safety;
}

} // namespace f64
} // namespace vg
