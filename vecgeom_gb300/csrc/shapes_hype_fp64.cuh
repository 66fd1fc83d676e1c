// FP64 hyperboloid (Hype) kernels on the flattened record (HypeRec, vg_types.h): the kernels
// of VecGeom/volumes/kernel/HypeImplementation.h with VecGeom/volumes/HypeUtilities.h and the
// scalar HypeHelpers specialisation (the one the reference's CUDA build runs), with the
// UniversalHype treatment of the inner surface, in the reference's operation order, so
// results are bit-identical in FP64. The near-tangent discriminant b*b - a*c is evaluated as
// the reference evaluates it (a plain product), which keeps the results bit-identical.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {
namespace f64 {

// HypeUtilities::ApproxDistOutside / ApproxDistInside
__device__ __forceinline__ double hy_dist_outside(double pr, double pz, double r0, double tanPhi)
{
  const double r1 = sqrt(r0 * r0 + tanPhi * tanPhi * pz * pz);
  const double z1 = pz;
  const double r2 = pr;
  const double z2 = sqrt((pr * pr - r0 * r0) / (tanPhi * tanPhi));
  const double dz = z2 - z1;
  const double dr = r2 - r1;
  const double r3 = sqrt(dr * dr + dz * dz);
  return r3 < 2.2250738585072014e-308 ? (r2 - r1) : (r2 - r1) * dz / r3; // DBL_MIN
}
__device__ __forceinline__ double hy_dist_inside(double pr, double pz, double r0, double tan2Phi)
{
  if (tan2Phi < 2.2250738585072014e-308) return r0 - pr;
  const double rh  = sqrt(r0 * r0 + pz * pz * tan2Phi);
  const double dr  = -rh;
  const double dz  = pz * tan2Phi;
  const double len = sqrt(dr * dr + dz * dz);
  return fabs((pr - rh) * dr) / len;
}

// GenericKernelForContainsAndInside
__device__ __forceinline__ void hy_classify(const HypeRec &h, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double r2    = perp2(p);
  const double oRad2 = (h.rmax2 + h.tOut2 * p.z * p.z);
  double iRad2       = 0.;
  cin                = false;
  cout               = fabs(p.z) > (h.dz + h.zTol);
  if (cout) return;
  cout = r2 > oRad2 + h.outerTol;
  if (cout) return;
  const bool inner = h.inner != 0.;
  if (inner) {
    iRad2 = (h.rmin2 + h.tIn2 * p.z * p.z);
    cout  = r2 < (iRad2 - h.innerTol);
  }
  if (cout) return;
  if (forInside) {
    cin = (fabs(p.z) < (h.dz - h.zTol)) && (r2 < oRad2 - h.outerTol);
    if (inner) cin = cin && (r2 > (iRad2 + h.innerTol));
  }
}
__device__ __forceinline__ int hype_inside(const HypeRec &h, V3 p)
{
  bool cin, cout;
  hy_classify(h, p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
__device__ __forceinline__ bool hype_contains(const HypeRec &h, V3 p)
{
  bool cin, cout;
  hy_classify(h, p, false, cin, cout);
  return !cout;
}

// HypeUtilities::IsCompletelyInside
__device__ __forceinline__ bool hy_completely_inside(const HypeRec &h, V3 p)
{
  const double r2    = perp2(p);
  const double oRad2 = (h.rmax2 + h.tOut2 * p.z * p.z);
  bool in            = (fabs(p.z) < (h.dz - h.zTol)) && (r2 < oRad2 - h.outerTol);
  if (h.inner != 0.) in = in && (r2 > ((h.rmin2 + h.tIn2 * p.z * p.z) + h.innerTol));
  return in;
}
// HypeUtilities::IsCompletelyOutside
__device__ __forceinline__ bool hy_completely_outside(const HypeRec &h, V3 p)
{
  const double r2 = perp2(p);
  if (fabs(p.z) > (h.dz + h.zTol)) return true;
  if (r2 > (h.rmax2 + h.tOut2 * p.z * p.z) + h.outerTol) return true;
  return h.inner != 0. && r2 < ((h.rmin2 + h.tIn2 * p.z * p.z) - h.innerTol);
}

// the z end caps' surface band (both IsPointOnSurfaceAndMoving* tests)
__device__ __forceinline__ bool hy_on_z_surface(const HypeRec &h, V3 p, double rho2)
{
  return ((rho2 - h.endOuterRadius2) < kTolerance) && ((h.endInnerRadius2 - rho2) < kTolerance) &&
         (fabs(fabs(p.z) - h.dz) < kTolerance);
}

// HypeUtilities::IsPointOnSurfaceAndMovingInside
__device__ __forceinline__ bool hy_on_surface_moving_in(const HypeRec &h, V3 p, V3 d)
{
  const double rho2 = perp2(p);
  if (hy_on_z_surface(h, p, rho2)) return p.z * d.z < 0.;
  double pz = p.z, vz = d.z;
  if (pz < 0.) vz = -vz;
  if (pz < 0.) pz = -pz;
  const bool outerSurf = fabs((h.rmax2 + h.tOut2 * p.z * p.z) - rho2) < h.outerTol;
  if (outerSurf) return (p.x * d.x + p.y * d.y - pz * h.tOut2 * vz) < 0.;
  if (h.inner == 0.) return false;
  const bool innerSurf = fabs((h.rmin2 + h.tIn2 * p.z * p.z) - rho2) < h.innerTol;
  return innerSurf && ((p.x * d.x + p.y * d.y - pz * h.tIn2 * vz) > 0.);
}

// IsPointMovingOutside{Outer,Inner}Surface
__device__ __forceinline__ bool hy_moving_out_outer(const HypeRec &h, V3 p, V3 d)
{
  return p.x * d.x + p.y * d.y + (-p.z * h.tOut2) * d.z > 0.;
}
__device__ __forceinline__ bool hy_moving_out_inner(const HypeRec &h, V3 p, V3 d)
{
  return -p.x * d.x + -p.y * d.y + (p.z * h.tIn2) * d.z > 0.;
}

// HypeUtilities::IsPointOnSurfaceAndMovingOutside
__device__ __forceinline__ bool hy_on_surface_moving_out(const HypeRec &h, V3 p, V3 d)
{
  const double rho2 = p.x * p.x + p.y * p.y;
  if (hy_on_z_surface(h, p, rho2) && p.z * d.z > 0.) return true;
  if (fabs((h.rmax2 + h.tOut2 * p.z * p.z) - rho2) < h.outerTol && hy_moving_out_outer(h, p, d)) return true;
  return h.inner != 0. && fabs((h.rmin2 + h.tIn2 * p.z * p.z) - rho2) < h.innerTol && hy_moving_out_inner(h, p, d);
}

// HypeUtilities::IsPointOn{Outer,Inner}SurfaceAndMovingOutside (|z| < dz)
__device__ __forceinline__ bool hy_on_outer_moving_out(const HypeRec &h, V3 p, V3 d)
{
  const double rho2 = p.x * p.x + p.y * p.y;
  const double absZ = fabs(p.z);
  return fabs((h.rmax2 + h.tOut2 * p.z * p.z) - rho2) < h.outerTol && absZ >= 0. && absZ < h.dz &&
         hy_moving_out_outer(h, p, d);
}
__device__ __forceinline__ bool hy_on_inner_moving_out(const HypeRec &h, V3 p, V3 d)
{
  if (h.inner == 0.) return false;
  const double rho2 = p.x * p.x + p.y * p.y;
  const double absZ = fabs(p.z);
  return fabs((h.rmin2 + h.tIn2 * p.z * p.z) - rho2) < h.innerTol && absZ >= 0. && absZ < h.dz &&
         hy_moving_out_inner(h, p, d);
}

// HypeUtilities::GetPointOfIntersectionWithZPlane<ForDistToIn>
__device__ __forceinline__ bool hy_z_plane(const HypeRec &h, V3 p, V3 d, bool forIn, double &zDist)
{
  zDist           = (sgn(forIn ? p.z : d.z) * h.dz - p.z) / nonzero(d.z);
  const double r2 = (p.x + zDist * d.x) * (p.x + zDist * d.x) + (p.y + zDist * d.y) * (p.y + zDist * d.y);
  if (h.inner == 0.) return r2 < h.endOuterRadius2;
  return (r2 < h.endOuterRadius2) && (r2 > h.endInnerRadius2);
}

// HypeHelpers<double, ForDistToIn, ForInnerSurface>::GetPointOfIntersectionWithHyperbolicSurface:
// dist is left unchanged when the quadratic has no real root
__device__ __forceinline__ bool hy_hyperbolic(const HypeRec &h, V3 p, V3 d, bool forIn, bool inner, double &dist)
{
  const double t2 = inner ? h.tIn2 : h.tOut2;
  const double r2 = inner ? h.rmin2 : h.rmax2;
  const double a  = perp2(d) - t2 * d.z * d.z;
  const double b  = (d.x * p.x + d.y * p.y - t2 * d.z * p.z);
  const double c  = perp2(p) - t2 * p.z * p.z - r2;
  const double disc = b * b - a * c;
  if (!(disc > 0.)) return false;
  // which root: inner surface for DistanceToIn / outer for DistanceToOut take the larger one
  const bool plusRoot = (inner == forIn);
  const bool direct   = inner ? (forIn ? b < 0. : b > 0.) : (forIn ? b >= 0. : b < 0.);
  const double sq     = sqrt(disc);
  if (direct)
    dist = plusRoot ? ((-b + sq) / a) : ((-b - sq) / a);
  else
    dist = plusRoot ? (c / (-b - sq)) : (c / (-b + sq));
  if (dist < 0.) dist = kInfLength;
  return fabs(p.z + dist * d.z) <= h.dz;
}

static __device__ __noinline__ double hype_dist_in(const HypeRec &h, V3 p, V3 d)
{
  const double absZ = fabs(p.z);
  double zDist = kInfLength, dist = kInfLength;
  const double r = perp2(p);
  if (hy_on_surface_moving_in(h, p, d)) return 0.0;
  if (hy_completely_inside(h, p)) return -1.0;
  const bool hittingZPlane = hy_z_plane(h, p, d, true, zDist);
  const bool above         = (absZ > h.dz) && (p.z * d.z < 0.);
  if (above && hittingZPlane) return zDist;
  const double nx = p.x + zDist * d.x, ny = p.y + zDist * d.y;
  const double rp2 = nx * nx + ny * ny;
  const bool outerFromOutsideZ = above && !hittingZPlane && (rp2 >= h.endOuterRadius2);
  const bool outerFromWithinZ  = (r > ((h.rmax2 + h.tOut2 * absZ * absZ) + kHalfTolerance)) && (absZ >= 0.) && (absZ <= h.dz);
  double distance = kInfLength;
  bool cond       = (outerFromOutsideZ || outerFromWithinZ || hy_on_outer_moving_out(h, p, d)) &&
              hy_hyperbolic(h, p, d, true, false, dist);
  if (cond) distance = dist;
  if (h.inner != 0.) {
    if (cond) return distance;
    const bool innerFromOutsideZ = above && !hittingZPlane && (rp2 <= h.endInnerRadius2);
    const bool innerFromWithinZ =
        (r < ((h.rmin2 + h.tIn2 * absZ * absZ) - kHalfTolerance)) && (absZ >= 0.) && (absZ <= h.dz);
    cond = (innerFromOutsideZ || innerFromWithinZ || hy_on_inner_moving_out(h, p, d)) &&
           hy_hyperbolic(h, p, d, true, true, dist);
    if (cond) distance = dist;
  }
  return distance;
}

static __device__ __noinline__ double hype_dist_out(const HypeRec &h, V3 p, V3 d)
{
  double zDist = kInfLength, dist = kInfLength;
  if (hy_on_surface_moving_out(h, p, d)) return 0.;
  if (hy_completely_outside(h, p)) return -1.;
  hy_z_plane(h, p, d, false, zDist);
  if (zDist < 0.) zDist = kInfLength;
  hy_hyperbolic(h, p, d, false, false, dist);
  if (dist < 0.) dist = kInfLength;
  double distance = zDist < dist ? zDist : dist;
  if (h.inner != 0.) {
    hy_hyperbolic(h, p, d, false, true, dist);
    if (dist < 0.) dist = kInfLength;
    distance = distance < dist ? distance : dist;
  }
  return distance;
}

static __device__ __noinline__ double hype_safety_in(const HypeRec &h, V3 p)
{
  const double absZ = fabs(p.z);
  const double r2   = perp2(p);
  const double r    = sqrt(r2);
  bool compIn, compOut;
  hy_classify(h, p, true, compIn, compOut);
  if (!compIn && !compOut) return 0.;
  if (compIn) return -1.0;
  const double sigz = absZ - h.dz;
  if ((sigz > kHalfTolerance) && (r < h.endOuterRadius) && (r > h.endInnerRadius)) return sigz;
  if ((sigz > kHalfTolerance) && (r > h.endOuterRadius))
    return sqrt((r - h.endOuterRadius) * (r - h.endOuterRadius) + (sigz) * (sigz));
  if ((sigz > kHalfTolerance) && (r < h.endInnerRadius))
    return sqrt((r - h.endInnerRadius) * (r - h.endInnerRadius) + (sigz) * (sigz));
  if ((r2 > ((h.rmax2 + h.tOut2 * absZ * absZ) + kHalfTolerance)) && (absZ > 0.) && (absZ < h.dz))
    return hy_dist_outside(r, absZ, h.rmax, h.tOut);
  if ((r2 < ((h.rmin2 + h.tIn2 * absZ * absZ) - kHalfTolerance)) && (absZ > 0.) && (absZ < h.dz))
    return hy_dist_inside(r, absZ, h.rmin, h.tIn2);
  return 0.;
}

static __device__ __noinline__ double hype_safety_out(const HypeRec &h, V3 p)
{
  const double r    = sqrt(p.x * p.x + p.y * p.y);
  const double absZ = fabs(p.z);
  bool inside, outside;
  hy_classify(h, p, true, inside, outside);
  if (!inside && !outside) return 0.;
  if (outside) return -1.0;
  const double distZ = fabs(fabs(p.z) - h.dz);
  const bool inner   = h.inner != 0.;
  double distInner   = 0.;
  if (inner && h.stIn != 0.) distInner = hy_dist_outside(r, absZ, h.rmin, h.tIn);
  if (inner && h.stIn == 0.) distInner = (r - h.rmin);
  if (!inner && h.stIn == 0.) distInner = kInfLength;
  const double distOuter = hy_dist_inside(r, absZ, h.rmax, h.tOut2);
  double safety          = distInner < distOuter ? distInner : distOuter;
  return safety < distZ ? safety : distZ;
}

} // namespace f64
} // namespace vg
