// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// Scalar restatement of the Sphere: ThetaCone, the Wedge distances it uses, SphereUtilities
// and SphereImplementation. Citations are to the reference's files; every expression keeps
// the reference's operation order. ThetaCone_Evolution.h:18 defines kHalfPi as 0.5 * kPi,
// the value of ref_base.h's kHalfPi.
#include "ref_nav.h"
#include "ref_shapes_more.h"
#include <cmath>

namespace oracle {

// ====================================================================== ThetaCone
// ThetaCone_Evolution.h:44-69 constructor
ThetaCone::ThetaCone(double sTheta, double dTheta) : fSTheta(sTheta), fDTheta(dTheta), kAngTol(kTolerance)
{
  fETheta            = fSTheta + fDTheta;
  halfAngTol         = (0.5 * kAngTol);
  double tempfSTheta = fSTheta;
  double tempfETheta = fETheta;
  if (fSTheta > kPi / 2) tempfSTheta = kPi - fSTheta;
  if (fETheta > kPi / 2) tempfETheta = kPi - fETheta;
  tanSTheta   = std::tan(tempfSTheta);
  tanSTheta2  = tanSTheta * tanSTheta;
  tanETheta   = std::tan(tempfETheta);
  tanETheta2  = tanETheta * tanETheta;
  tanBisector = std::tan(tempfSTheta + (fDTheta / 2));
  if (fSTheta > kPi / 2 && fETheta > kPi / 2) tanBisector = std::tan(tempfSTheta - (fDTheta / 2));
  slope1 = std::tan(kPi / 2 - fSTheta);
  slope2 = std::tan(kPi / 2 - fETheta);
}

// ThetaCone_Evolution.h:131-146 GetNormal<ForStartTheta>
Vec3 ThetaCone::GetNormal(Vec3 const &p, bool start) const
{
  if (start) {
    const Vec3 n(p.x(), p.y(), -tanSTheta2 * p.z());
    return (fSTheta <= kHalfPi) ? -n : n;
  }
  const Vec3 n(p.x(), p.y(), -tanETheta2 * p.z());
  return (fETheta <= kHalfPi) ? n : -n;
}

// ThetaCone_Evolution.h:154-169 IsOnSurfaceGeneric<ForStartTheta>
bool ThetaCone::IsOnSurfaceGeneric(Vec3 const &p, bool start) const
{
  const double rhs  = start ? Abs(tanSTheta * p.z()) : Abs(tanETheta * p.z());
  const double rho2 = p.Perp2();
  return rho2 >= MakeMinusTolerantSquare<true>(rhs) && rho2 <= MakePlusTolerantSquare<true>(rhs);
}

// ThetaCone_Evolution.h:171-185 IsPointOnSurfaceAndMovingOut
bool ThetaCone::IsPointOnSurfaceAndMovingOut(Vec3 const &p, Vec3 const &d, bool start, bool movingOut) const
{
  if (movingOut) return IsOnSurfaceGeneric(p, start) && (d.Dot(GetNormal(p, start)) > 0.);
  return IsOnSurfaceGeneric(p, start) && (d.Dot(GetNormal(p, start)) < 0.);
}

// ThetaCone_Evolution.h:323-330 DistanceToLine
double ThetaCone::DistanceToLine(double slope, double x, double y) const
{
  const double dist = (y - slope * x) / Sqrt(1. + slope * slope);
  return Abs(dist);
}

// ThetaCone_Evolution.h:237-281 SafetyToIn
double ThetaCone::SafetyToIn(Vec3 const &p) const
{
  double safeTheta      = 0.;
  const double pointRad = Sqrt(p.x() * p.x() + p.y() * p.y());
  const double sfTh1    = DistanceToLine(slope1, pointRad, p.z());
  const double sfTh2    = DistanceToLine(slope2, pointRad, p.z());
  safeTheta             = Min(sfTh1, sfTh2);
  const bool done       = Contains(p);
  if (done) return 0.;
  if (fSTheta < kPi / 2 + halfAngTol) {
    if (fETheta < kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) {
        if (p.z() < 0.) safeTheta = sfTh2;
      }
    }
    if (fETheta > kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) {
        if (p.z() > 0.) safeTheta = sfTh1;
        if (p.z() < 0.) safeTheta = sfTh2;
      }
    }
  }
  if (fETheta > kPi / 2 + halfAngTol) {
    if (fSTheta > kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) {
        if (p.z() > 0.) safeTheta = sfTh1;
      }
    }
  }
  return safeTheta;
}

// ThetaCone_Evolution.h:283-321 SafetyToOut
double ThetaCone::SafetyToOut(Vec3 const &p) const
{
  const double pointRad    = Sqrt(p.x() * p.x() + p.y() * p.y());
  const double bisectorRad = Abs(p.z() * tanBisector);
  bool condition           = false;
  const double sfTh1       = DistanceToLine(slope1, pointRad, p.z());
  const double sfTh2       = DistanceToLine(slope2, pointRad, p.z());
  if (fSTheta < kPi / 2 + halfAngTol) {
    if (fETheta < kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) condition = (pointRad < bisectorRad) && (fSTheta != 0.);
    }
    if (fETheta > kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) condition = sfTh1 < sfTh2;
    }
  }
  if (fETheta > kPi / 2 + halfAngTol) {
    if (fSTheta > kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) condition = !((pointRad < bisectorRad) && (fETheta != kPi));
    }
  }
  return condition ? sfTh1 : sfTh2;
}

// ThetaCone_Evolution.h:340-470 DistanceToIn: the roots of both cones (a root within
// 3 kTolerance is 0; negative ones are discarded unless a root was within the tolerance)
void ThetaCone::DistanceToIn(Vec3 const &point, Vec3 const &dir, double &distThetaCone1, double &distThetaCone2,
                             bool &intsect1, bool &intsect2) const
{
  bool done            = false;
  double firstRoot     = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = point.x() * dir.x() + point.y() * dir.y();
  const double rho2    = point.x() * point.x() + point.y() * point.y();
  const double dirRho2 = dir.Perp2();
  const double b       = pDotV2d - point.z() * dir.z() * tanSTheta2;
  const double a       = dirRho2 - dir.z() * dir.z() * tanSTheta2;
  const double c       = rho2 - point.z() * point.z() * tanSTheta2;
  const double d2      = b * b - a * c;
  const double aInv    = 1. / NonZero(a);
  if (d2 > 0.) firstRoot = (-b + Sqrt(Abs(d2))) * aInv;
  done = done || (Abs(firstRoot) < 3. * kTolerance);
  if (Abs(firstRoot) < 3. * kTolerance) firstRoot = 0.;
  if (!done && (firstRoot < 0.)) firstRoot = kInfLength;
  const double b2    = pDotV2d - point.z() * dir.z() * tanETheta2;
  const double a2    = dirRho2 - dir.z() * dir.z() * tanETheta2;
  const double c2    = rho2 - point.z() * point.z() * tanETheta2;
  const double d22   = b2 * b2 - a2 * c2;
  const double a2Inv = 1. / NonZero(a2);
  if (d22 > 0.) secondRoot = (-b2 - Sqrt(Abs(d22))) * a2Inv;
  if (!done && (Abs(secondRoot) < 3. * kTolerance)) secondRoot = 0.;
  done = done || (Abs(secondRoot) < 3. * kTolerance);
  if (!done && (secondRoot < 0.)) secondRoot = kInfLength;

  if (fSTheta < kHalfPi + halfAngTol) {
    if (fETheta < kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        distThetaCone1        = firstRoot;
        distThetaCone2        = secondRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect1              = ((d2 > 0.) && (zOfCone1 > 0.));
        intsect2              = ((d22 > 0.) && (zOfCone2 > 0.));
      }
    }
    if (fETheta >= kHalfPi - halfAngTol && fETheta <= kHalfPi + halfAngTol) {
      if (dir.z() > 0.) distThetaCone2 = -point.z() / dir.z();
      const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
      intsect2              = ((distThetaCone2 != kInfLength) && (Abs(zOfCone2) < halfAngTol));
    }
    if (fETheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        distThetaCone1 = firstRoot;
        if (d22 > 0.) secondRoot = (-b2 + Sqrt(Abs(d22))) * a2Inv;
        done = false;
        done = done || (Abs(secondRoot) < 3. * kTolerance);
        if (Abs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
        if (!done && (secondRoot < 0.)) secondRoot = kInfLength;
        distThetaCone2        = secondRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect1 = ((d2 > 0) && (distThetaCone1 != kInfLength) && (zOfCone1 > 0.));
        intsect2 = ((d22 > 0) && (distThetaCone2 != kInfLength) && (zOfCone2 < 0.));
      }
    }
  }
  if (fSTheta >= kHalfPi - halfAngTol) {
    if (fETheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        if (d2 > 0.) firstRoot = (-b - Sqrt(Abs(d2))) * aInv;
        done = false;
        done = done || (Abs(firstRoot) < 3. * kTolerance);
        if (Abs(firstRoot) < 3. * kTolerance) firstRoot = 0.;
        if (!done && (firstRoot < 0.)) firstRoot = kInfLength;
        distThetaCone1 = firstRoot;
        if (d22 > 0.) secondRoot = (-b2 + Sqrt(Abs(d22))) * a2Inv;
        done = false;
        done = done || (Abs(secondRoot) < 3. * kTolerance);
        if (Abs(secondRoot) < 3. * kTolerance) secondRoot = 0.;
        if (!done && (secondRoot < 0.)) secondRoot = kInfLength;
        distThetaCone2        = secondRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect1 = ((d2 > 0) && (distThetaCone1 != kInfLength) && (zOfCone1 < 0.));
        intsect2 = ((d22 > 0) && (distThetaCone2 != kInfLength) && (zOfCone2 < 0.));
      }
    }
  }
  if (fSTheta >= kHalfPi - halfAngTol && fSTheta <= kHalfPi + halfAngTol) {
    if (dir.z() < 0.) distThetaCone1 = -point.z() / dir.z();
    const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
    intsect1              = ((distThetaCone1 != kInfLength) && (Abs(zOfCone1) < halfAngTol));
  }
}

// ThetaCone_Evolution.h:472-620 DistanceToOut
void ThetaCone::DistanceToOut(Vec3 const &point, Vec3 const &dir, double &distThetaCone1, double &distThetaCone2,
                              bool &intsect1, bool &intsect2) const
{
  const double inf     = kInfLength;
  double firstRoot     = kInfLength, secondRoot = kInfLength;
  const double pDotV2d = point.x() * dir.x() + point.y() * dir.y();
  const double rho2    = point.x() * point.x() + point.y() * point.y();
  const double b       = pDotV2d - point.z() * dir.z() * tanSTheta2;
  const double a       = dir.x() * dir.x() + dir.y() * dir.y() - dir.z() * dir.z() * tanSTheta2;
  const double c       = rho2 - point.z() * point.z() * tanSTheta2;
  double d2            = b * b - a * c;
  if (d2 < 0. && Abs(d2) < kHalfTolerance) d2 = 0.;
  if ((d2 >= 0.) && b >= 0. && a != 0.) firstRoot = ((-b - Sqrt(Abs(d2))) / NonZero(a));
  if ((d2 >= 0.) && b < 0.) firstRoot = ((c) / NonZero(-b + Sqrt(Abs(d2))));
  if (firstRoot < 0.) firstRoot = kInfLength;
  const double b2 = point.x() * dir.x() + point.y() * dir.y() - point.z() * dir.z() * tanETheta2;
  const double a2 = dir.x() * dir.x() + dir.y() * dir.y() - dir.z() * dir.z() * tanETheta2;
  const double c2 = point.x() * point.x() + point.y() * point.y() - point.z() * point.z() * tanETheta2;
  double d22      = (b2 * b2) - (a2 * c2);
  if (d22 < 0. && Abs(d22) < kHalfTolerance) d22 = 0.;
  if ((d22 >= 0.) && b2 >= 0.) secondRoot = ((c2) / NonZero(-b2 - Sqrt(Abs(d22))));
  if ((d22 >= 0.) && b2 < 0. && a2 != 0.) secondRoot = ((-b2 + Sqrt(Abs(d22))) / NonZero(a2));
  if (secondRoot < 0. && Abs(secondRoot) > kTolerance) secondRoot = kInfLength;
  if (Abs(secondRoot) < kTolerance) secondRoot = 0.;

  if (fSTheta < kPi / 2 + halfAngTol) {
    if (fETheta < kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) {
        distThetaCone1        = firstRoot;
        distThetaCone2        = secondRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect1 = ((d2 > 0) && (distThetaCone1 != kInfLength) && ((zOfCone1) > -kHalfTolerance));
        intsect2 = ((d22 > 0) && (distThetaCone2 != kInfLength) && ((zOfCone2) > -kHalfTolerance));
        const double dirRho2 = dir.x() * dir.x() + dir.y() * dir.y();
        double zs            = kInfLength;
        if (fSTheta) zs = dirRho2 / tanSTheta;
        double ze = kInfLength;
        if (fETheta) ze = dirRho2 / tanETheta;
        const bool cond = (point.x() == 0. && point.y() == 0. && point.z() == 0. && dir.z() < zs && dir.z() < ze);
        if (cond) distThetaCone1 = 0.;
        if (cond) distThetaCone2 = 0.;
        intsect1 = intsect1 || cond;
        intsect2 = intsect2 || cond;
      }
    }
    if (fETheta >= kPi / 2 - halfAngTol && fETheta <= kPi / 2 + halfAngTol) {
      distThetaCone1 = firstRoot;
      distThetaCone2 = inf;
      if (dir.z() < 0.) distThetaCone2 = -1. * point.z() / dir.z();
      const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
      const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
      intsect2 = ((distThetaCone2 != kInfLength) && (Abs(zOfCone2) < kHalfTolerance) && !(dir.z() == 0.));
      intsect1 = ((d2 >= 0) && (distThetaCone1 != kInfLength) && (Abs(zOfCone1) < kHalfTolerance) && !(dir.z() == 0.));
    }
    if (fETheta > kPi / 2 + halfAngTol) {
      if (fSTheta < fETheta) {
        distThetaCone1 = firstRoot;
        if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - Sqrt(Abs(d22))) / NonZero(a2));
        if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / NonZero(-b2 + Sqrt(Abs(d22))));
        if (secondRoot < 0.) secondRoot = kInfLength;
        distThetaCone2        = secondRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect1 = ((d2 >= 0) && (distThetaCone1 != kInfLength) && ((zOfCone1) > -kHalfTolerance));
        intsect2 = ((d22 >= 0) && (distThetaCone2 != kInfLength) && ((zOfCone2) < kHalfTolerance));
      }
    }
  }
  if (fETheta > kPi / 2 + halfAngTol) {
    if (fSTheta < fETheta) {
      secondRoot = kInfLength;
      if ((d22 >= 0.) && b2 > 0. && a2 != 0.) secondRoot = ((-b2 - Sqrt(Abs(d22))) / NonZero(a2));
      if ((d22 >= 0.) && b2 <= 0.) secondRoot = ((c2) / NonZero(-b2 + Sqrt(Abs(d22))));
      distThetaCone2 = secondRoot;
      if (fSTheta > kPi / 2 + halfAngTol) {
        if ((d2 >= 0.) && b > 0.) firstRoot = ((c) / NonZero(-b - Sqrt(Abs(d2))));
        if ((d2 >= 0.) && b <= 0. && a != 0.) firstRoot = ((-b + Sqrt(Abs(d2))) / NonZero(a));
        if (firstRoot < 0.) firstRoot = kInfLength;
        distThetaCone1        = firstRoot;
        const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
        intsect1              = ((d2 > 0) && (distThetaCone1 != kInfLength) && ((zOfCone1) < kHalfTolerance));
        const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
        intsect2              = ((d22 > 0) && (distThetaCone2 != kInfLength) && ((zOfCone2) < kHalfTolerance));
        const double dirRho2  = dir.x() * dir.x() + dir.y() * dir.y();
        double zs             = -kInfLength;
        if (tanSTheta) zs = -dirRho2 / tanSTheta;
        double ze = -kInfLength;
        if (tanETheta) ze = -dirRho2 / tanETheta;
        const bool cond = (point.x() == 0. && point.y() == 0. && point.z() == 0. && dir.z() > zs && dir.z() > ze);
        if (cond) distThetaCone1 = 0.;
        if (cond) distThetaCone2 = 0.;
        intsect1 = intsect1 || cond;
        intsect2 = intsect2 || cond;
      }
    }
  }
  if (fSTheta >= kPi / 2 - halfAngTol && fSTheta <= kPi / 2 + halfAngTol) {
    distThetaCone2 = secondRoot;
    distThetaCone1 = kInfLength;
    if (dir.z() > 0.) distThetaCone1 = -1. * point.z() / NonZero(dir.z());
    const double zOfCone1 = (point.z() + distThetaCone1 * dir.z());
    const double zOfCone2 = (point.z() + distThetaCone2 * dir.z());
    intsect1 = ((distThetaCone1 != kInfLength) && (Abs(zOfCone1) < kHalfTolerance) && (dir.z() != 0.));
    intsect2 = ((d22 >= 0) && (distThetaCone2 != kInfLength) && (Abs(zOfCone2) < kHalfTolerance) && (dir.z() != 0.));
  }
}

// ThetaCone_Evolution.h:622-690 IsCompletelyInside
bool ThetaCone::IsCompletelyInside(Vec3 const &p) const
{
  const double rho          = Sqrt(p.Mag2() - (p.z() * p.z()));
  const double cone1Radius  = Abs(p.z() * tanSTheta);
  const double cone2Radius  = Abs(p.z() * tanETheta);
  const bool isPointOnZAxis = p.z() != 0. && p.x() == 0. && p.y() == 0.;
  const bool isPointOnXY    = p.z() == 0. && (p.x() != 0. || p.y() != 0.);
  const double startTheta = fSTheta, endTheta = fETheta;
  bool ci = (isPointOnZAxis && ((startTheta == 0. && endTheta == kPi) || (p.z() > 0. && startTheta == 0.) ||
                                (p.z() < 0. && endTheta == kPi)));
  ci = ci || (!ci && (isPointOnXY && (startTheta < kHalfPi && endTheta > kHalfPi &&
                                      (kHalfPi - startTheta) > kAngTol && (endTheta - kHalfPi) > kTolerance)));
  if (fSTheta < kHalfPi + halfAngTol) {
    if (fETheta < kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin = cone1Radius + (2 * kAngTol * 10.);
        const double tolAngMax = cone2Radius - (2 * kAngTol * 10.);
        ci = ci || (!ci && (((rho <= tolAngMax) && (rho >= tolAngMin) && (p.z() > 0.) && (fSTheta != 0.)) ||
                            ((rho <= tolAngMax) && (fSTheta == 0.) && (p.z() > 0.))));
      }
    }
    if (fETheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin = cone1Radius + (2 * kAngTol * 10.);
        const double tolAngMax = cone2Radius + (2 * kAngTol * 10.);
        ci = ci || (!ci && (((rho >= tolAngMin) && (p.z() > 0.)) || ((rho >= tolAngMax) && (p.z() < 0.))));
      }
    }
    if (fETheta >= kHalfPi - halfAngTol && fETheta <= kHalfPi + halfAngTol) ci = ci && !(Abs(p.z()) < halfAngTol);
  }
  if (fETheta > kHalfPi + halfAngTol) {
    if (fSTheta >= kHalfPi - halfAngTol && fSTheta <= kHalfPi + halfAngTol) ci = ci && !(Abs(p.z()) < halfAngTol);
    if (fSTheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin = cone1Radius - (2 * kAngTol * 10.);
        const double tolAngMax = cone2Radius + (2 * kAngTol * 10.);
        ci = ci || (!ci && (((rho <= tolAngMin) && (rho >= tolAngMax) && (p.z() < 0.) && (fETheta != kPi)) ||
                            ((rho <= tolAngMin) && (p.z() < 0.) && (fETheta == kPi))));
      }
    }
  }
  return ci;
}

// ThetaCone_Evolution.h:692-760 IsCompletelyOutside
bool ThetaCone::IsCompletelyOutside(Vec3 const &p) const
{
  const double diff         = p.Perp2();
  const double rho          = Sqrt(diff);
  const double cone1Radius  = Abs(p.z() * tanSTheta);
  const double cone2Radius  = Abs(p.z() * tanETheta);
  const bool isPointOnZAxis = p.z() != 0. && p.x() == 0. && p.y() == 0.;
  const bool isPointOnXY    = p.z() == 0. && (p.x() != 0. || p.y() != 0.);
  bool co = (isPointOnZAxis && (((fSTheta != 0.) && (fETheta != kPi)) || (p.z() > 0. && (fSTheta != 0.)) ||
                                (p.z() < 0. && (fETheta != kPi))));
  co = co || (!co && (isPointOnXY && (((fSTheta < kHalfPi) && (fETheta < kHalfPi) && ((kHalfPi - fSTheta) > kAngTol) &&
                                       ((kHalfPi - fETheta) > kTolerance)) ||
                                      ((fSTheta > kHalfPi && fETheta > kHalfPi) && ((fSTheta - kHalfPi) > kAngTol) &&
                                       ((fETheta - kHalfPi) > kTolerance)))));
  if (fSTheta < kHalfPi + halfAngTol) {
    if (fETheta < kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin2 = cone1Radius - (2 * kAngTol * 10.);
        const double tolAngMax2 = cone2Radius + (2 * kAngTol * 10.);
        co = co || (!co && ((rho < tolAngMin2) || (rho > tolAngMax2) || (p.z() < 0.)));
      }
    }
    if (fETheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin2 = cone1Radius - (2 * kAngTol * 10.);
        const double tolAngMax2 = cone2Radius - (2 * kAngTol * 10.);
        co = co || (!co && (((rho < tolAngMin2) && (p.z() > 0.)) || ((rho < tolAngMax2) && (p.z() < 0.))));
      }
    }
    if (fETheta >= kHalfPi - halfAngTol && fETheta <= kHalfPi + halfAngTol) co = co && !(Abs(p.z()) < halfAngTol);
  }
  if (fETheta > kHalfPi + halfAngTol) {
    if (fSTheta >= kHalfPi - halfAngTol && fSTheta <= kHalfPi + halfAngTol) co = co && !(Abs(p.z()) < halfAngTol);
    if (fSTheta > kHalfPi + halfAngTol) {
      if (fSTheta < fETheta) {
        const double tolAngMin2 = cone1Radius + (2 * kAngTol * 10.);
        const double tolAngMax2 = cone2Radius - (2 * kAngTol * 10.);
        co = co || (!co && ((rho < tolAngMax2) || (rho > tolAngMin2) || (p.z() > 0.)));
      }
    }
  }
  return co;
}

// ====================================================================== Sphere
// SphereStruct.h:256-276 constructor with CheckPhiAngles (:160-170, :126-158) and
// CheckThetaAngles (:96-124); the wedge and the theta cone take the raw arguments
Sphere::Sphere(double pRmin, double pRmax, double pSPhi, double pDPhi, double pSTheta, double pDTheta)
    : fRmin(pRmin), fRmax(pRmax), fSPhi(pSPhi), fDPhi(pDPhi), fSTheta(pSTheta), fDTheta(pDTheta),
      fPhiWedge(pDPhi, pSPhi), fThetaCone(pSTheta, pDTheta)
{
  const double kAngTolerance = 1e-9;
  // CheckDPhiAngle
  if (pDPhi >= 2 * kPi - kAngTolerance * 0.5) {
    fDPhi          = 2 * kPi;
    fSPhi          = 0;
    fFullPhiSphere = true;
  } else {
    fFullPhiSphere = false;
    if (pDPhi > 0) fDPhi = pDPhi;
  }
  if (!fFullPhiSphere) { // CheckSPhiAngle
    if (pSPhi < 0)
      fSPhi = 2 * kPi - std::fmod(std::fabs(pSPhi), 2 * kPi);
    else
      fSPhi = std::fmod(pSPhi, 2 * kPi);
    if (fSPhi + fDPhi > 2 * kPi) fSPhi -= 2 * kPi;
  }
  fFullSphere = fFullPhiSphere && fFullThetaSphere;
  // CheckThetaAngles
  if ((pSTheta < 0) || (pSTheta > kPi)) {
  } else {
    fSTheta = pSTheta;
  }
  if (pDTheta + pSTheta >= kPi)
    fDTheta = kPi - pSTheta;
  else if (pDTheta > 0)
    fDTheta = pDTheta;
  fFullThetaSphere = !(fDTheta - fSTheta < kPi);
  fFullSphere      = fFullPhiSphere && fFullThetaSphere;
  eTheta           = fSTheta + fDTheta;
}

// Wedge_Evolution.h:236-245 (IsOnSurfaceGeneric<ForStartPhi> = IsOnSurfaceGeneric of that plane)
bool Sphere::WedgeOnSurfaceMoving(Vec3 const &p, Vec3 const &d, bool start, bool movingOut) const
{
  const Vec3 &n    = start ? fPhiWedge.normal1 : fPhiWedge.normal2;
  const Vec3 &al   = start ? fPhiWedge.along1 : fPhiWedge.along2;
  const bool onSf  = Wedge::IsOnSurfaceGeneric(al, n, p);
  const double dot = d.Dot(-n);
  return movingOut ? (onSf && dot > 0.005 * kHalfTolerance) : (onSf && dot < 0.005 * kHalfTolerance);
}

// Wedge_Evolution.h:391-410 DistanceToIn
void Sphere::WedgeDistanceToIn(Vec3 const &p, Vec3 const &d, double &d1, double &d2) const
{
  Wedge const &w     = fPhiWedge;
  d1                 = kInfLength;
  d2                 = kInfLength;
  const double comp1 = d.x() * w.normal1.x() + d.y() * w.normal1.y();
  const double comp2 = d.x() * w.normal2.x() + d.y() * w.normal2.y();
  if (comp1 > 0.) {
    const double tmp = -(p.x() * w.normal1.x() + p.y() * w.normal1.y()) / comp1;
    if (tmp > 0.) d1 = tmp;
  }
  if (comp2 > 0.) {
    const double tmp = -(p.x() * w.normal2.x() + p.y() * w.normal2.y()) / comp2;
    if (tmp > 0.) d2 = tmp;
  }
}

// Wedge_Evolution.h:412-432 DistanceToOut
void Sphere::WedgeDistanceToOut(Vec3 const &p, Vec3 const &d, double &d1, double &d2) const
{
  Wedge const &w     = fPhiWedge;
  const double comp1 = d.x() * w.normal1.x() + d.y() * w.normal1.y();
  const double comp2 = d.x() * w.normal2.x() + d.y() * w.normal2.y();
  d1                 = kInfLength;
  d2                 = kInfLength;
  if (comp1 < 0.) {
    const double tmp = -(p.x() * w.normal1.x() + p.y() * w.normal1.y()) / comp1;
    if (tmp > 0.) d1 = tmp;
  }
  if (comp2 < 0.) {
    const double tmp = -(p.x() * w.normal2.x() + p.y() * w.normal2.y()) / comp2;
    if (tmp > 0.) d2 = tmp;
  }
}

// SphereImplementation.h:87-131 GenericKernelForContainsAndInside
void Sphere::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double rad2 = p.Mag2();
  if (fRmin)
    cin = rad2 <= MakeMinusTolerantSquare<true>(fRmax) && rad2 >= MakePlusTolerantSquare<true>(fRmin);
  else
    cin = rad2 <= MakeMinusTolerantSquare<true>(fRmax);
  if (fRmin)
    cout = rad2 >= MakePlusTolerantSquare<true>(fRmax) || rad2 <= MakeMinusTolerantSquare<true>(fRmin);
  else
    cout = rad2 >= MakePlusTolerantSquare<true>(fRmax);
  if (!fFullPhiSphere) {
    bool ci = false, co = false;
    fPhiWedge.ContainsAndInside(p, forInside, ci, co);
    cout = cout || co;
    if (forInside) cin = cin && ci;
  }
  if (!fFullThetaSphere) {
    const bool ci = forInside ? fThetaCone.IsCompletelyInside(p) : false;
    const bool co = fThetaCone.IsCompletelyOutside(p);
    cout          = cout || co;
    if (forInside) cin = cin && ci;
  }
}

bool Sphere::Contains(Vec3 const &p) const
{
  bool ci = false, co = false;
  ContainsAndInside(p, false, ci, co);
  return !co;
}
int Sphere::Inside(Vec3 const &p) const
{
  bool ci = false, co = false;
  ContainsAndInside(p, true, ci, co);
  int inside = kSurface;
  if (co) inside = kOutside;
  if (ci) inside = kInside;
  return inside;
}

// SphereUtilities.h:148-164 IsCompletelyInside, :128-146 IsCompletelyOutside (the wedge and the
// theta cone are consulted whether or not the sphere is cut in phi or theta)
bool Sphere::IsCompletelyInside(Vec3 const &p) const
{
  const double rad = p.Mag();
  const bool inRad = (rad < (fRmax - kTolerance)) && (rad > (fRmin + kTolerance));
  bool ci = false, co = false;
  fPhiWedge.ContainsAndInside(p, true, ci, co);
  return inRad && ci && fThetaCone.IsCompletelyInside(p);
}
bool Sphere::IsCompletelyOutside(Vec3 const &p) const
{
  const double rad  = p.Mag();
  const bool outRad = (rad > (fRmax + kTolerance)) || (rad < (fRmin - kTolerance));
  bool ci = false, co = false;
  fPhiWedge.ContainsAndInside(p, true, ci, co);
  return outRad || co || fThetaCone.IsCompletelyOutside(p);
}

// SphereUtilities.h:40-52 IsPointOnInner/OuterRadius, :166-185 IsPointOnRadialSurfaceAndMovingOut,
// :187-221 IsPointOnSurfaceAndMovingOut
bool Sphere::IsPointOnSurfaceAndMovingOut(Vec3 const &p, Vec3 const &d, bool movingOut) const
{
  const double kSqrtTolerance = 3.1622777e-5; // VecGeom/base/Math.h:29 (double precision)
  auto onRadius = [&](double r) {
    const double mag2 = p.Mag2();
    return mag2 <= MakePlusTolerantSquare<true>(r) && mag2 >= MakeMinusTolerantSquare<true>(r);
  };
  auto radial = [&](bool inner) {
    if (movingOut) {
      if (inner) return onRadius(fRmin) && (d.Dot(-p) > kSqrtTolerance);
      return onRadius(fRmax) && (d.Dot(p) > kSqrtTolerance);
    }
    if (inner) return onRadius(fRmin) && (d.Dot(-p) < -kSqrtTolerance);
    return onRadius(fRmax) && (d.Dot(p) < -kSqrtTolerance);
  };
  const bool tempOuterRad = radial(false);
  bool tempInnerRad = false, tempStartPhi = false, tempEndPhi = false, tempStartTheta = false, tempEndTheta = false;
  if (fRmin) tempInnerRad = radial(true);
  if (fDPhi < (kTwoPi - kHalfTolerance)) {
    tempStartPhi = WedgeOnSurfaceMoving(p, d, true, movingOut);
    tempEndPhi   = WedgeOnSurfaceMoving(p, d, false, movingOut);
  }
  if (fDTheta < (kPi - kHalfTolerance)) {
    tempStartTheta = fThetaCone.IsPointOnSurfaceAndMovingOut(p, d, true, movingOut);
    tempEndTheta   = fThetaCone.IsPointOnSurfaceAndMovingOut(p, d, false, movingOut);
  }
  return ((tempOuterRad || tempInnerRad) && fPhiWedge.Contains(p) && fThetaCone.Contains(p)) ||
         ((tempStartPhi || tempEndPhi) && (p.Mag2() >= fRmin * fRmin) && (p.Mag2() <= fRmax * fRmax) &&
          fThetaCone.Contains(p)) ||
         ((tempStartTheta || tempEndTheta) && (p.Mag2() >= fRmin * fRmin) && (p.Mag2() <= fRmax * fRmax) &&
          fPhiWedge.Contains(p));
}

// SphereImplementation.h:326-366 GetMinDistFromPhi<DistToIn>
void Sphere::GetMinDistFromPhi(Vec3 const &localPoint, Vec3 const &localDir, bool toIn, bool done,
                               double &distance) const
{
  double distPhi1 = kInfLength, distPhi2 = kInfLength;
  if (toIn)
    WedgeDistanceToIn(localPoint, localDir, distPhi1, distPhi2);
  else
    WedgeDistanceToOut(localPoint, localDir, distPhi1, distPhi2);
  Wedge const &w = fPhiWedge;
  double dist    = Min(distPhi1, distPhi2);
  Vec3 tmpPt     = localPoint + dist * localDir;
  double rad2    = tmpPt.Mag2();
  bool tempCond  = ((dist == distPhi1) && Wedge::IsOnSurfaceGeneric(w.along1, w.normal1, tmpPt)) ||
                  ((dist == distPhi2) && Wedge::IsOnSurfaceGeneric(w.along2, w.normal2, tmpPt));
  const bool containsCond1 =
      tempCond && (rad2 > fRmin * fRmin) && (rad2 < fRmax * fRmax) && fThetaCone.Contains(tmpPt);
  if (!done && containsCond1) distance = Min(dist, distance);
  dist     = Max(distPhi1, distPhi2);
  tmpPt    = localPoint + dist * localDir;
  rad2     = tmpPt.Mag2();
  tempCond = ((dist == distPhi1) && Wedge::IsOnSurfaceGeneric(w.along1, w.normal1, tmpPt)) ||
             ((dist == distPhi2) && Wedge::IsOnSurfaceGeneric(w.along2, w.normal2, tmpPt));
  const bool containsCond2 =
      tempCond && (rad2 > fRmin * fRmin) && (rad2 < fRmax * fRmax) && fThetaCone.Contains(tmpPt);
  if ((!done) && (!containsCond1) && containsCond2) distance = Min(dist, distance);
}

// SphereImplementation.h:133-245 DistanceToIn
double Sphere::DistanceToIn(Vec3 const &point, Vec3 const &direction, double) const
{
  double distance      = kInfLength;
  const bool done      = false;
  const double rad2    = point.Mag2();
  const double pDotV3d = point.Dot(direction);
  double c             = rad2 - fRmax * fRmax;
  if (IsCompletelyInside(point)) return -1.0;
  if (IsPointOnSurfaceAndMovingOut(point, direction, false)) return 0.0;
  double sd1 = kInfLength, sd2 = kInfLength;
  double d2  = (pDotV3d * pDotV3d - c);
  if (d2 < 0. || ((c > 0.) && (pDotV3d > 0.))) return distance;
  if (d2 >= 0.) sd1 = (-pDotV3d - Sqrt(Abs(d2)));
  double outerDist = kInfLength, innerDist = kInfLength;
  if (fFullSphere) {
    if (sd1 >= 0.) outerDist = sd1;
  } else {
    const Vec3 tmpPt = point + sd1 * direction;
    if (fPhiWedge.Contains(tmpPt) && fThetaCone.Contains(tmpPt) && (sd1 >= 0.)) outerDist = sd1;
  }
  if (fRmin) {
    c  = rad2 - fRmin * fRmin;
    d2 = pDotV3d * pDotV3d - c;
    if (d2 >= 0.) sd2 = (-pDotV3d + Sqrt(Abs(d2)));
    if (fFullSphere) {
      if (sd2 >= 0.) innerDist = sd2;
    } else {
      const Vec3 tmpPt = point + sd2 * direction;
      if ((sd2 >= 0.) && fPhiWedge.Contains(tmpPt) && fThetaCone.Contains(tmpPt)) innerDist = sd2;
    }
  }
  distance = Min(outerDist, innerDist);
  if (!fFullPhiSphere) GetMinDistFromPhi(point, direction, true, done, distance);
  double distThetaMin = kInfLength;
  if (!fFullThetaSphere) {
    bool intsect1 = false, intsect2 = false;
    double distTheta1 = kInfLength, distTheta2 = kInfLength;
    fThetaCone.DistanceToIn(point, direction, distTheta1, distTheta2, intsect1, intsect2);
    const Vec3 coneIntSecPt1 = point + distTheta1 * direction;
    const double distCone1   = coneIntSecPt1.Mag2();
    const Vec3 coneIntSecPt2 = point + distTheta2 * direction;
    const double distCone2   = coneIntSecPt2.Mag2();
    bool isValidCone1 = (distCone1 >= fRmin * fRmin && distCone1 <= fRmax * fRmax) && intsect1;
    bool isValidCone2 = (distCone2 >= fRmin * fRmin && distCone2 <= fRmax * fRmax) && intsect2;
    if (!fFullPhiSphere) {
      isValidCone1 = isValidCone1 && fPhiWedge.Contains(coneIntSecPt1);
      isValidCone2 = isValidCone2 && fPhiWedge.Contains(coneIntSecPt2);
    }
    if (isValidCone2 && !isValidCone1) distThetaMin = distTheta2;
    if (isValidCone1 && !isValidCone2) distThetaMin = distTheta1;
    if (isValidCone1 && isValidCone2) distThetaMin = Min(distTheta1, distTheta2);
  }
  distance = Min(distThetaMin, distance);
  const Vec3 directDir = (Vec3(0., 0., 0.) - point);
  const double newDist = directDir.Mag();
  const Vec3 u         = directDir.Unit();
  if ((fSTheta > kHalfTolerance || eTheta < (kPi - kHalfTolerance)) && (Abs(u.x() - direction.x()) < kHalfTolerance) &&
      (Abs(u.y() - direction.y()) < kHalfTolerance) && (Abs(u.z() - direction.z()) < kHalfTolerance))
    distance = Min(distance, newDist);
  return distance;
}

// SphereImplementation.h:247-324 DistanceToOut
double Sphere::DistanceToOut(Vec3 const &point, Vec3 const &direction, double) const
{
  double distance      = kInfLength;
  const bool done      = false;
  const double pDotV3d = point.Dot(direction);
  const double rad2    = point.Mag2();
  double c             = rad2 - fRmax * fRmax;
  double sd1 = kInfLength, sd2 = kInfLength;
  if (IsCompletelyOutside(point)) return -1.0;
  if (IsPointOnSurfaceAndMovingOut(point, direction, true)) return 0.0;
  double d2 = (pDotV3d * pDotV3d - c);
  if (d2 >= 0.) sd1 = (-pDotV3d + Sqrt(Abs(d2)));
  if (fRmin) {
    c  = rad2 - fRmin * fRmin;
    d2 = (pDotV3d * pDotV3d - c);
    if ((d2 >= 0.) && (pDotV3d < 0.)) sd2 = (-pDotV3d - Sqrt(Abs(d2)));
  }
  const double snxt   = Min(sd1, sd2);
  const bool condSemi = ((fSTheta == 0. && eTheta == kPi / 2.) && direction.z() >= 0.) ||
                        ((fSTheta == kPi / 2. && eTheta == kPi) && direction.z() <= 0.);
  if (condSemi) return snxt;
  double distThetaMin = kInfLength;
  if (!fFullThetaSphere) {
    bool intsect1 = false, intsect2 = false;
    double distTheta1 = kInfLength, distTheta2 = kInfLength;
    fThetaCone.DistanceToOut(point, direction, distTheta1, distTheta2, intsect1, intsect2);
    if (intsect2 && !intsect1) distThetaMin = distTheta2;
    if (!intsect2 && intsect1) distThetaMin = distTheta1;
    if (intsect2 && intsect1) distThetaMin = Min(distTheta1, distTheta2);
  }
  distance = Min(distThetaMin, snxt);
  if (!fFullPhiSphere) {
    if (fDPhi <= kPi) {
      double distPhi1, distPhi2;
      WedgeDistanceToOut(point, direction, distPhi1, distPhi2);
      distance = Min(Min(distPhi1, distPhi2), distance);
    } else {
      GetMinDistFromPhi(point, direction, false, done, distance);
    }
  }
  return distance;
}

// SphereImplementation.h:368-406 SafetyToIn
double Sphere::SafetyToIn(Vec3 const &point) const
{
  const double rad = point.Mag();
  bool ci = false, co = false;
  ContainsAndInside(point, true, ci, co);
  if (ci) return -1.0;
  if (!ci && !co) return 0.0;
  double safety;
  if (fRmin) {
    const double safeRMin = fRmin - rad;
    const double safeRMax = rad - fRmax;
    safety                = (safeRMin > safeRMax) ? safeRMin : safeRMax;
  } else {
    safety = (rad - fRmax);
  }
  if (!fFullPhiSphere) safety = Max(fPhiWedge.SafetyToIn(point), safety);
  if (!fFullThetaSphere) safety = Max(fThetaCone.SafetyToIn(point), safety);
  return safety;
}

// SphereImplementation.h:408-446 SafetyToOut
double Sphere::SafetyToOut(Vec3 const &point) const
{
  const double rad = point.Mag();
  bool ci = false, co = false;
  ContainsAndInside(point, true, ci, co);
  if (co) return -1.0;
  if (!ci && !co) return 0.0;
  double safety;
  if (fRmin) {
    const double safeRMin = (rad - fRmin);
    const double safeRMax = (fRmax - rad);
    safety                = (safeRMin < safeRMax) ? safeRMin : safeRMax;
  } else {
    safety = (fRmax - rad);
  }
  if (!fFullPhiSphere) safety = Min(fPhiWedge.SafetyToOut(point), safety);
  if (!fFullThetaSphere) safety = Min(fThetaCone.SafetyToOut(point), safety);
  return safety;
}

// source/UnplacedSphere.cpp:74-160 Extent
void Sphere::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  aMin                 = Vec3(-fRmax, -fRmax, -fRmax);
  aMax                 = Vec3(fRmax, fRmax, fRmax);
  const double eTheta_ = fSTheta + fDTheta;
  if (fFullSphere) return;
  double st1 = 0., st2 = 0.;
  if (!fFullThetaSphere) {
    aMax[2] = ((fSTheta <= kPi / 2.) ? fRmax : fRmin) * std::cos(fSTheta);
    aMin[2] = ((eTheta_ <= kPi / 2.) ? fRmin : fRmax) * std::cos(eTheta_);
    st1     = std::sin(fSTheta);
    st2     = std::sin(eTheta);
    if (fSTheta <= kPi / 2.) {
      if ((eTheta_) < kPi / 2.) {
        aMax[0] = fRmax * st2;
        aMin[0] = -fRmax * st2;
        aMax[1] = fRmax * st2;
        aMin[1] = -fRmax * st2;
      }
    } else {
      aMax[0] = fRmax * st1;
      aMin[0] = -fRmax * st1;
      aMax[1] = fRmax * st1;
      aMin[1] = -fRmax * st1;
    }
  }
  if (!fFullPhiSphere) {
    double Rmax = fRmax;
    if (fSTheta > kPi / 2.) Rmax *= st1;
    if (eTheta_ < kPi / 2.) Rmax *= st2;
    const double Rmin    = fRmin * Min(st1, st2);
    const double Rin     = 0.5 * (Rmax + Rmin);
    const bool phi0out   = !fPhiWedge.Contains(Vec3(Rin, 0, 0));
    const bool phi90out  = !fPhiWedge.Contains(Vec3(0, Rin, 0));
    const bool phi180out = !fPhiWedge.Contains(Vec3(-Rin, 0, 0));
    const bool phi270out = !fPhiWedge.Contains(Vec3(0, -Rin, 0));
    if (!(phi0out || phi90out || phi180out || phi270out)) return;
    const double Cx = Rmax * std::cos(fSPhi);
    const double Dx = Rmax * std::cos(fSPhi + fDPhi);
    const double Cy = Rmax * std::sin(fSPhi);
    const double Dy = Rmax * std::sin(fSPhi + fDPhi);
    if (phi0out) aMax[0] = Max(Cx, Dx);
    if (phi90out) aMax[1] = Max(Cy, Dy);
    if (phi180out) aMin[0] = Min(Cx, Dx);
    if (phi270out) aMin[1] = Min(Cy, Dy);
    if (fDPhi >= kPi) return;
    const double Ax = Rmin * std::cos(fSPhi);
    const double Bx = Rmin * std::cos(fSPhi + fDPhi);
    const double Ay = Rmin * std::sin(fSPhi);
    const double By = Rmin * std::sin(fSPhi + fDPhi);
    double temp;
    temp    = Max(Ax, Bx);
    aMax[0] = temp > aMax[0] ? temp : aMax[0];
    temp    = Max(Ay, By);
    aMax[1] = temp > aMax[1] ? temp : aMax[1];
    temp    = Min(Ax, Bx);
    aMin[0] = temp < aMin[0] ? temp : aMin[0];
    temp    = Min(Ay, By);
    aMin[1] = temp < aMin[1] ? temp : aMin[1];
  }
}

} // namespace oracle
