// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// The hyperboloid (Hype): VecGeom/volumes/HypeStruct.h, VecGeom/volumes/HypeUtilities.h and
// VecGeom/volumes/kernel/HypeImplementation.h, restated in scalar form (Real_v = double,
// with the scalar HypeHelpers specialisation of HypeUtilities.h).
#include "ref_shapes_more.h"

namespace oracle {

namespace {
// HypeUtilities::ApproxDistOutside: distance from (pr, pz) to the hyperbola r^2 = r0^2 +
// tanPhi^2 z^2 along the chord to its points at the same z and the same r
double ApproxDistOutside(double pr, double pz, double r0, double tanPhi)
{
  const double r1 = Sqrt(r0 * r0 + tanPhi * tanPhi * pz * pz);
  const double z1 = pz;
  const double r2 = pr;
  const double z2 = Sqrt((pr * pr - r0 * r0) / (tanPhi * tanPhi));
  const double dz = z2 - z1;
  const double dr = r2 - r1;
  const double r3 = Sqrt(dr * dr + dz * dz);
  return r3 < DBL_MIN ? (r2 - r1) : (r2 - r1) * dz / r3;
}
// HypeUtilities::ApproxDistInside: distance to the tangent of the hyperbola at z = pz
double ApproxDistInside(double pr, double pz, double r0, double tan2Phi)
{
  if (tan2Phi < DBL_MIN) return r0 - pr;
  const double rh  = Sqrt(r0 * r0 + pz * pz * tan2Phi);
  const double dr  = -rh;
  const double dz  = pz * tan2Phi;
  const double len = Sqrt(dr * dr + dz * dz);
  return Abs((pr - rh) * dr) / len;
}
} // namespace

// HypeStruct::CalculateCached
Hype::Hype(double rmin, double rmax, double stIn, double stOut, double dz)
    : fRmin(rmin), fRmax(rmax), fStIn(stIn), fStOut(stOut), fDz(dz)
{
  fTIn                   = std::tan(fStIn);
  fTOut                  = std::tan(fStOut);
  fTIn2                  = fTIn * fTIn;
  fTOut2                 = fTOut * fTOut;
  fRmin2                 = fRmin * fRmin;
  fRmax2                 = fRmax * fRmax;
  fDz2                   = fDz * fDz;
  fEndInnerRadius2       = fTIn2 * fDz2 + fRmin2;
  fEndOuterRadius2       = fTOut2 * fDz2 + fRmax2;
  fEndInnerRadius        = Sqrt(fEndInnerRadius2);
  fEndOuterRadius        = Sqrt(fEndOuterRadius2);
  zToleranceLevel        = kTolerance * fDz;
  innerRadToleranceLevel = kTolerance * fEndInnerRadius;
  outerRadToleranceLevel = kTolerance * fEndOuterRadius;
  fInner                 = (fRmin > 0.) || (fStIn != 0.); // HypeStruct::InnerSurfaceExists
}

// UnplacedHype::Extent (source/UnplacedHype.cpp:94-100)
void Hype::Extent(Vec3 &lo, Vec3 &hi) const
{
  const double r = fEndOuterRadius;
  lo             = Vec3(-r, -r, -fDz);
  hi             = Vec3(r, r, fDz);
}

// HypeImplementation::GenericKernelForContainsAndInside
void Hype::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double r2    = p.Perp2();
  const double oRad2 = (fRmax2 + fTOut2 * p.z() * p.z());
  double iRad2       = 0.;
  cin                = false;
  cout               = (Abs(p.z()) > (fDz + zToleranceLevel));
  if (cout) return;
  cout = cout || (r2 > oRad2 + outerRadToleranceLevel);
  if (cout) return;
  if (fInner) {
    iRad2 = (fRmin2 + fTIn2 * p.z() * p.z());
    cout  = cout || (r2 < (iRad2 - innerRadToleranceLevel));
  }
  if (cout) return;
  if (forInside) {
    cin = (Abs(p.z()) < (fDz - zToleranceLevel)) && (r2 < oRad2 - outerRadToleranceLevel);
    if (fInner) cin = cin && (r2 > (iRad2 + innerRadToleranceLevel));
  }
}

int Hype::Inside(Vec3 const &p) const
{
  bool cin, cout;
  ContainsAndInside(p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}

bool Hype::Contains(Vec3 const &p) const
{
  bool cin, cout;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}

// HypeUtilities::IsCompletelyInside / IsCompletelyOutside
bool Hype::IsCompletelyInside(Vec3 const &p) const
{
  const double r2    = p.Perp2();
  const double oRad2 = (fRmax2 + fTOut2 * p.z() * p.z());
  bool in            = (Abs(p.z()) < (fDz - zToleranceLevel)) && (r2 < oRad2 - outerRadToleranceLevel);
  if (fInner) {
    const double iRad2 = (fRmin2 + fTIn2 * p.z() * p.z());
    in                 = in && (r2 > (iRad2 + innerRadToleranceLevel));
  }
  return in;
}
bool Hype::IsCompletelyOutside(Vec3 const &p) const
{
  const double r2    = p.Perp2();
  const double oRad2 = (fRmax2 + fTOut2 * p.z() * p.z());
  bool out           = (Abs(p.z()) > (fDz + zToleranceLevel));
  if (out) return out;
  out = out || (r2 > oRad2 + outerRadToleranceLevel);
  if (out) return out;
  if (fInner) {
    const double iRad2 = (fRmin2 + fTIn2 * p.z() * p.z());
    out                = out || (r2 < (iRad2 - innerRadToleranceLevel));
  }
  return out;
}

// HypeUtilities::IsPointOnSurfaceAndMovingInside with IsPointMovingInside{Outer,Inner}Surface
bool Hype::OnSurfaceMovingInside(Vec3 const &p, Vec3 const &d) const
{
  const double rho2  = p.Perp2();
  const double radI2 = (fRmin2 + fTIn2 * p.z() * p.z());
  const double radO2 = (fRmax2 + fTOut2 * p.z() * p.z());
  const bool zSurf   = ((rho2 - fEndOuterRadius2) < kTolerance) && ((fEndInnerRadius2 - rho2) < kTolerance) &&
                     (Abs(Abs(p.z()) - fDz) < kTolerance);
  bool in = zSurf && (p.z() * d.z() < 0.);
  if (zSurf) return in;
  double pz = p.z(), vz = d.z();
  if (pz < 0.) vz = -vz;
  if (pz < 0.) pz = -pz;
  const bool outerSurf = Abs(radO2 - rho2) < outerRadToleranceLevel;
  in = in || (outerSurf && ((p.x() * d.x() + p.y() * d.y() - pz * fTOut2 * vz) < 0.));
  if (fInner) {
    if (outerSurf) return in;
    const bool innerSurf = Abs(radI2 - rho2) < innerRadToleranceLevel;
    in = in || (innerSurf && ((p.x() * d.x() + p.y() * d.y() - pz * fTIn2 * vz) > 0.));
  }
  return in;
}

// IsPointMovingOutside{Outer,Inner}Surface: the sign of the direction along the normal
namespace {
bool MovingOutsideOuter(Hype const &h, Vec3 const &p, Vec3 const &d)
{
  return Vec3(p.x(), p.y(), -p.z() * h.fTOut2).Dot(d) > 0.;
}
bool MovingOutsideInner(Hype const &h, Vec3 const &p, Vec3 const &d)
{
  return Vec3(-p.x(), -p.y(), p.z() * h.fTIn2).Dot(d) > 0.;
}
} // namespace

bool Hype::OnOuterSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const
{
  const double rho2  = p.x() * p.x() + p.y() * p.y();
  const double absZ  = Abs(p.z());
  const double radO2 = (fRmax2 + fTOut2 * p.z() * p.z());
  const bool surf    = (Abs(radO2 - rho2) < outerRadToleranceLevel) && (absZ >= 0.) && (absZ < fDz);
  return surf && MovingOutsideOuter(*this, p, d);
}
bool Hype::OnInnerSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const
{
  if (!fInner) return false;
  const double rho2  = p.x() * p.x() + p.y() * p.y();
  const double absZ  = Abs(p.z());
  const double radI2 = (fRmin2 + fTIn2 * p.z() * p.z());
  const bool surf    = (Abs(radI2 - rho2) < innerRadToleranceLevel) && (absZ >= 0.) && (absZ < fDz);
  return surf && MovingOutsideInner(*this, p, d);
}

// HypeUtilities::IsPointOnSurfaceAndMovingOutside
bool Hype::OnSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const
{
  const double rho2  = p.x() * p.x() + p.y() * p.y();
  const double radI2 = (fRmin2 + fTIn2 * p.z() * p.z());
  const double radO2 = (fRmax2 + fTOut2 * p.z() * p.z());
  const bool zSurf   = ((rho2 - fEndOuterRadius2) < kTolerance) && ((fEndInnerRadius2 - rho2) < kTolerance) &&
                     (Abs(Abs(p.z()) - fDz) < kTolerance);
  bool out = zSurf && (p.z() * d.z() > 0.);
  if (out) return out;
  const bool outerSurf = Abs(radO2 - rho2) < outerRadToleranceLevel;
  out                  = out || (outerSurf && MovingOutsideOuter(*this, p, d));
  if (out) return out;
  if (fInner) {
    const bool innerSurf = Abs(radI2 - rho2) < innerRadToleranceLevel;
    out                  = out || (innerSurf && MovingOutsideInner(*this, p, d));
  }
  return out;
}

// HypeUtilities::GetPointOfIntersectionWithZPlane<ForDistToIn>
bool Hype::ZPlaneIntersection(Vec3 const &p, Vec3 const &d, bool forDistToIn, double &zDist) const
{
  zDist           = (Sign(forDistToIn ? p.z() : d.z()) * fDz - p.z()) / NonZero(d.z());
  const double r2 = (p + zDist * d).Perp2();
  if (!fInner) return (r2 < fEndOuterRadius2);
  return ((r2 < fEndOuterRadius2) && (r2 > fEndInnerRadius2));
}

// HypeHelpers<double, ForDistToIn, ForInnerSurface>::GetPointOfIntersectionWithHyperbolicSurface
// (scalar specialisation: dist is left unchanged when the quadratic has no real root)
bool Hype::HyperbolicIntersection(Vec3 const &p, Vec3 const &d, bool forDistToIn, bool inner, double &dist) const
{
  const double t2 = inner ? fTIn2 : fTOut2;
  const double r2 = inner ? fRmin2 : fRmax2;
  const double a  = d.Perp2() - t2 * d.z() * d.z();
  const double b  = (d.x() * p.x() + d.y() * p.y() - t2 * d.z() * p.z());
  const double c  = p.Perp2() - t2 * p.z() * p.z() - r2;
  if (!(b * b - a * c > 0.)) return false;
  if (inner) {
    if (forDistToIn) {
      if (b < 0.)
        dist = ((-b + Sqrt(b * b - a * c)) / (a));
      else
        dist = ((c) / (-b - Sqrt(b * b - a * c)));
    } else {
      if (b > 0.)
        dist = ((-b - Sqrt(b * b - a * c)) / (a));
      else
        dist = ((c) / (-b + Sqrt(b * b - a * c)));
    }
  } else {
    if (forDistToIn) {
      if (b >= 0.)
        dist = ((-b - Sqrt(b * b - a * c)) / (a));
      else
        dist = ((c) / (-b + Sqrt(b * b - a * c)));
    } else {
      if (b < 0.)
        dist = ((-b + Sqrt(b * b - a * c)) / a);
      else
        dist = (c / (-b - Sqrt(b * b - a * c)));
    }
  }
  if (dist < 0.) dist = kInfLength;
  const double newPtZ = p.z() + dist * d.z();
  return (Abs(newPtZ) <= fDz);
}

double Hype::DistanceToIn(Vec3 const &p, Vec3 const &d, double) const
{
  const double absZ = Abs(p.z());
  double zDist = kInfLength, dist = kInfLength;
  const double r = p.Perp2();
  if (OnSurfaceMovingInside(p, d)) return 0.0;
  if (IsCompletelyInside(p)) return -1.0;
  const bool hittingZPlane = ZPlaneIntersection(p, d, true, zDist);
  const bool above         = (absZ > fDz) && (p.z() * d.z() < 0.);
  if (above && hittingZPlane) return zDist;
  const Vec3 newPt = p + zDist * d;
  const double rp2 = newPt.Perp2();
  const bool outerFromOutsideZ = above && !hittingZPlane && (rp2 >= fEndOuterRadius2);
  const bool outerFromWithinZ  = (r > ((fRmax2 + fTOut2 * absZ * absZ) + kHalfTolerance)) && (absZ >= 0.) && (absZ <= fDz);
  double distance = kInfLength;
  bool cond = (outerFromOutsideZ || outerFromWithinZ || OnOuterSurfaceMovingOutside(p, d)) &&
              HyperbolicIntersection(p, d, true, false, dist);
  if (cond) distance = dist;
  if (fInner) {
    if (cond) return distance;
    const bool innerFromOutsideZ = above && !hittingZPlane && (rp2 <= fEndInnerRadius2);
    const bool innerFromWithinZ =
        (r < ((fRmin2 + fTIn2 * absZ * absZ) - kHalfTolerance)) && (absZ >= 0.) && (absZ <= fDz);
    cond = (innerFromOutsideZ || innerFromWithinZ || OnInnerSurfaceMovingOutside(p, d)) &&
           HyperbolicIntersection(p, d, true, true, dist);
    if (cond) distance = dist;
  }
  return distance;
}

double Hype::DistanceToOut(Vec3 const &p, Vec3 const &d, double) const
{
  double zDist = kInfLength, dist = kInfLength;
  if (OnSurfaceMovingOutside(p, d)) return 0.;
  if (IsCompletelyOutside(p)) return -1.;
  ZPlaneIntersection(p, d, false, zDist);
  if (zDist < 0.) zDist = kInfLength;
  HyperbolicIntersection(p, d, false, false, dist);
  if (dist < 0.) dist = kInfLength;
  double distance = Min(zDist, dist);
  if (fInner) {
    HyperbolicIntersection(p, d, false, true, dist);
    if (dist < 0.) dist = kInfLength;
    distance = Min(distance, dist);
  }
  return distance;
}

double Hype::SafetyToIn(Vec3 const &p) const
{
  const double absZ = Abs(p.z());
  const double r2   = p.Perp2();
  const double r    = Sqrt(r2);
  bool compIn, compOut;
  ContainsAndInside(p, true, compIn, compOut);
  if (!compIn && !compOut) return 0.;
  if (compIn) return -1.0;
  const double sigz = absZ - fDz;
  if ((sigz > kHalfTolerance) && (r < fEndOuterRadius) && (r > fEndInnerRadius)) return sigz;
  if ((sigz > kHalfTolerance) && (r > fEndOuterRadius))
    return Sqrt((r - fEndOuterRadius) * (r - fEndOuterRadius) + (sigz) * (sigz));
  if ((sigz > kHalfTolerance) && (r < fEndInnerRadius))
    return Sqrt((r - fEndInnerRadius) * (r - fEndInnerRadius) + (sigz) * (sigz));
  if ((r2 > ((fRmax2 + fTOut2 * absZ * absZ) + kHalfTolerance)) && (absZ > 0.) && (absZ < fDz))
    return ApproxDistOutside(r, absZ, fRmax, fTOut);
  if ((r2 < ((fRmin2 + fTIn2 * absZ * absZ) - kHalfTolerance)) && (absZ > 0.) && (absZ < fDz))
    return ApproxDistInside(r, absZ, fRmin, fTIn2);
  return 0.;
}

double Hype::SafetyToOut(Vec3 const &p) const
{
  const double r    = Sqrt(p.x() * p.x() + p.y() * p.y());
  const double absZ = Abs(p.z());
  bool inside, outside;
  ContainsAndInside(p, true, inside, outside);
  if (!inside && !outside) return 0.;
  if (outside) return -1.0;
  const double distZ = Abs(Abs(p.z()) - fDz);
  double distInner   = 0.;
  if (fInner && fStIn != 0.) distInner = ApproxDistOutside(r, absZ, fRmin, fTIn);
  if (fInner && fStIn == 0.) distInner = (r - fRmin);
  if (!fInner && fStIn == 0.) distInner = kInfLength;
  const double distOuter = ApproxDistInside(r, absZ, fRmax, fTOut2);
  double safety          = Min(distInner, distOuter);
  safety                 = Min(safety, distZ);
  return safety;
}

} // namespace oracle
