// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// Scalar restatement of Wedge, Box, Tube and Cone. Citations are to the reference's files.
#include "ref_shapes.h"
#include <cstdio>
#include <cstdlib>
#include <cmath>

namespace oracle {

// ====================================================================== Wedge
// source/Wedge_Evolution.cpp (constructor)
Wedge::Wedge(double angle, double zero) : dphi(angle)
{
  along1  = Vec3(std::cos(zero), std::sin(zero), 0.);
  along2  = Vec3(std::cos(zero + angle), std::sin(zero + angle), 0.);
  normal1 = Vec3(-std::sin(zero), std::cos(zero), 0.);
  normal2 = Vec3(std::sin(zero + angle), -std::cos(zero + angle), 0.);
}

// VecGeom/volumes/Wedge_Evolution.h:335-347 IsOnSurfaceGeneric
bool Wedge::IsOnSurfaceGeneric(Vec3 const &along, Vec3 const &normal, Vec3 const &p)
{
  const bool c1 = along.x() * p.x() + along.y() * p.y() >= 0.;
  if (!c1) return false;
  return Abs(normal.x() * p.x() + normal.y() * p.y()) < kTolerance;
}

// VecGeom/volumes/Wedge_Evolution.h:299-331 GenericKernelForContainsAndInside
void Wedge::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double startCheck = (-p.x() * along1.y() + p.y() * along1.x());
  const double endCheck   = (-along2.x() * p.y() + along2.y() * p.x());
  cout                    = startCheck < 0.;
  if (dphi < kPi)
    cout = cout || (endCheck < 0.);
  else
    cout = cout && (endCheck < 0.);
  if (forInside) {
    const bool onSurface = IsOnSurfaceGeneric(along1, normal1, p) || IsOnSurfaceGeneric(along2, normal2, p);
    cout                 = cout && !onSurface;
    cin                  = !onSurface && !cout;
  }
}

// VecGeom/volumes/Wedge_Evolution.h:349-381 SafetyToOut / SafetyToIn
double Wedge::SafetyToOut(Vec3 const &p) const
{
  const double d1 = p.x() * normal1.x() + p.y() * normal1.y();
  const double d2 = p.x() * normal2.x() + p.y() * normal2.y();
  return dphi < kPi ? Min(d1, d2) : Max(d1, d2);
}
double Wedge::SafetyToIn(Vec3 const &p) const
{
  const double d1 = p.x() * normal1.x() + p.y() * normal1.y();
  const double d2 = p.x() * normal2.x() + p.y() * normal2.y();
  return dphi < kPi ? Max(-1 * d1, -1 * d2) : Min(-1 * d1, -1 * d2);
}

// ====================================================================== Box
// VecGeom/volumes/kernel/BoxImplementation.h:84-90 Inside, :76-80 Contains
int Box::Inside(Vec3 const &p) const
{
  const double dist = (p.Abs() - dim).Max();
  int in            = dist < 0. ? kInside : kOutside;
  if (Abs(dist) < kHalfTolerance) in = kSurface;
  return in;
}
bool Box::Contains(Vec3 const &p) const { return (p.Abs() - dim).Max() < 0.; }

Vec3 UnplacedShape::Normal(Vec3 const &, bool &) const
{
  std::fprintf(stderr, "oracle: Normal() is not restated for this shape\n");
  std::abort();
}

// BoxImplementation.h:172-192 NormalKernel: the faces within kHalfTolerance of the nearest
// one contribute their axis, averaged on edges and corners
Vec3 Box::Normal(Vec3 const &p, bool &valid) const
{
  const Vec3 safety = (p.Abs() - dim).Abs();
  const double safmin = safety.Min();
  valid               = safmin < kHalfTolerance;
  Vec3 normal(0., 0., 0.);
  for (int k = 0; k < 3; ++k)
    if (safety[k] - safmin < kHalfTolerance) normal[k] = Sign(p[k]);
  if (normal.Mag2() > 1.0) {
    const double m = normal.Mag();
    normal         = Vec3(normal[0] / m, normal[1] / m, normal[2] / m);
  }
  return normal;
}

// BoxImplementation.h:109-131
double Box::DistanceToIn(Vec3 const &p, Vec3 const &d, double) const
{
  const Vec3 invDir(1.0 / NonZero(d[0]), 1.0 / NonZero(d[1]), 1.0 / NonZero(d[2]));
  const Vec3 signDir(Sign(d[0]), Sign(d[1]), Sign(d[2]));
  const Vec3 tempIn        = -signDir * dim - p;
  const Vec3 tempOut       = signDir * dim - p;
  const double absOrthogOut = Abs((signDir * tempOut).Min());
  const double distOut      = (tempOut * invDir).Min();
  double distance           = (tempIn * invDir).Max();
  if (distance >= distOut || distOut <= kHalfTolerance || absOrthogOut <= kHalfTolerance) distance = kInfLength;
  return distance;
}

// BoxImplementation.h:136-151
double Box::DistanceToOut(Vec3 const &p, Vec3 const &d, double) const
{
  const Vec3 invDir(1.0 / NonZero(d[0]), 1.0 / NonZero(d[1]), 1.0 / NonZero(d[2]));
  const Vec3 signDir(Sign(d[0]), Sign(d[1]), Sign(d[2]));
  const double safetyIn = (p.Abs() - dim).Max();
  const Vec3 tempOut    = signDir * dim - p;
  double distance       = (tempOut * invDir).Min();
  if (safetyIn > kHalfTolerance) distance = -1.0;
  return distance;
}

// BoxImplementation.h:156-167
double Box::SafetyToIn(Vec3 const &p) const { return (p.Abs() - dim).Max(); }
double Box::SafetyToOut(Vec3 const &p) const { return (dim - p.Abs()).Min(); }

// ====================================================================== Tube
// VecGeom/volumes/TubeStruct.h:41-179 (constructor + CalculateCached)
Tube::Tube(double rmin, double rmax, double z, double sphi, double dphi)
    : fRmin(rmin < 0.0 ? 0.0 : rmin), fRmax(rmax), fZ(z), fSphi(sphi), fDphi(dphi), fPhiWedge(dphi, sphi)
{
  fTolIz     = fZ - kHalfTolerance;
  fTolOz     = fZ + kHalfTolerance;
  fRmin2     = fRmin * fRmin;
  fTolOrmin  = (fRmin - kHalfTolerance);
  fTolIrmin  = (fRmin + kHalfTolerance);
  fTolOrmin2 = fTolOrmin * fTolOrmin;
  fTolIrmin2 = fTolIrmin * fTolIrmin;
  fRmax2     = fRmax * fRmax;
  fTolOrmax  = (fRmax + kHalfTolerance);
  fTolIrmax  = (fRmax - kHalfTolerance);
  fTolOrmax2 = fTolOrmax * fTolOrmax;
  fTolIrmax2 = fTolIrmax * fTolIrmax;
  fAlongPhi1x = std::cos(fSphi);
  fAlongPhi1y = std::sin(fSphi);
  fAlongPhi2x = std::cos(fSphi + fDphi);
  fAlongPhi2y = std::sin(fSphi + fDphi);
  fMaxVal     = Max(fRmax, fZ);
}

// VecGeom/volumes/kernel/TubeImplementation.h:57-97 TubeUtilities::PointInCyclicalSector (onSurfaceT=false)
void Tube::PointInCyclicalSector(double x, double y, bool includeSurface, bool &ret) const
{
  const bool smallerthanpi = fDphi <= M_PI;
  const double startCheck  = (-x * fAlongPhi1y + y * fAlongPhi1x);
  const double endCheck    = (-fAlongPhi2x * y + fAlongPhi2y * x);
  const double t           = includeSurface ? -kHalfTolerance : kHalfTolerance;
  if (smallerthanpi)
    ret = (startCheck >= t) && (endCheck >= t);
  else
    ret = (startCheck >= t) || (endCheck >= t);
}

// TubeImplementation.h:103-162 CircleTrajectoryIntersection
void Tube::CircleTrajectoryIntersection(double b, double c, Vec3 const &pos, Vec3 const &dir, bool largest,
                                        bool insectorCheck, double &dist, bool &ok) const
{
  double delta = b * b - c;
  ok           = delta > 0.;
  if (largest) ok = ok || (delta == 0.);
  if (!ok) delta = 0.;
  delta = Sqrt(delta);
  if (!largest) delta = -delta;
  dist = -b + delta;
  ok   = ok && (dist >= -2 * kTolerance);
  if (!ok) return;
  if (insectorCheck) {
    const double hitz = pos.z() + dist * dir.z();
    ok                = ok && (Abs(hitz) <= fZ);
    if (!ok) return;
    if (PhiTreat()) {
      bool insector     = false;
      const double hitx = pos.x() + dist * dir.x();
      const double hity = pos.y() + dist * dir.y();
      PointInCyclicalSector(hitx, hity, true, insector);
      ok = ok && insector;
    }
  }
}

// TubeImplementation.h:243-291 PhiPlaneTrajectoryIntersection
void Tube::PhiPlaneTrajectoryIntersection(double alongX, double alongY, double normalX, double normalY,
                                          Vec3 const &pos, Vec3 const &dir, bool positiveDir, bool insectorCheck,
                                          double &dist, bool &ok) const
{
  dist                    = kInfLength;
  const double dirDotNorm = dir.x() * normalX + dir.y() * normalY;
  ok                      = insectorCheck ? (dirDotNorm > 0.) : (dirDotNorm < 0.);
  const double dirDotXY   = (dir.y() * alongX - dir.x() * alongY);
  dist                    = (alongY * pos.x() - alongX * pos.y()) / NonZero(dirDotXY);
  ok                      = ok && ((dist * Abs(dirDotNorm)) > -kHalfTolerance);
  if (insectorCheck) {
    const double hitx = pos.x() + dist * dir.x();
    const double hity = pos.y() + dist * dir.y();
    const double hitz = pos.z() + dist * dir.z();
    const double r2   = hitx * hitx + hity * hity;
    ok                = ok && Abs(hitz) <= fTolOz && (r2 >= fTolOrmin2) && (r2 <= fTolOrmax2);
    if (positiveDir) ok = ok && (hitx * alongX + hity * alongY) > 0.;
  } else {
    if (positiveDir) {
      const double hitx = pos.x() + dist * dir.x();
      const double hity = pos.y() + dist * dir.y();
      ok                = ok && (hitx * alongX + hity * alongY) >= 0.;
    }
  }
}

// TubeImplementation.h:200-232 PhiPlaneSafety (UniversalTube: sector type decided at run time)
void Tube::PhiPlaneSafety(Vec3 const &pos, bool inside, double &safety) const
{
  if (fDphi > M_PI)
    safety = Sqrt(pos.x() * pos.x() + pos.y() * pos.y());
  else
    safety = kInfLength;
  double phi1 = pos.x() * fAlongPhi1y - pos.y() * fAlongPhi1x;
  if (inside) phi1 *= -1;
  if (phi1 > -kHalfTolerance && phi1 < safety) safety = phi1;
  double phi2 = pos.x() * fAlongPhi2y - pos.y() * fAlongPhi2x;
  if (!inside) phi2 *= -1;
  if (phi2 > -kHalfTolerance && phi2 < safety) safety = phi2;
}

// TubeImplementation.h:293-322 IsOnTubeSurface / GetNormal / IsMovingInsideTubeSurface
bool Tube::IsMovingInsideTubeSurface(Vec3 const &p, Vec3 const &d, bool inner) const
{
  const double rho = p.Perp2();
  bool on;
  if (inner)
    on = (rho >= fTolOrmin2) && (rho <= fTolIrmin2) && (Abs(p.z()) < (fZ + kTolerance));
  else
    on = (rho >= fTolIrmax2) && (rho <= fTolOrmax2) && (Abs(p.z()) < (fZ + kTolerance));
  const Vec3 n = inner ? Vec3(-p.x(), -p.y(), 0.) : Vec3(p.x(), p.y(), 0.);
  return on && (d.Dot(n) <= 0.);
}

// TubeImplementation.h:352-396 GenericKernelForContainsAndInside
void Tube::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double absz = Abs(p[2]);
  if (forInside) {
    cout = absz > MakePlusTolerant<true>(fZ);
    cin  = absz < MakeMinusTolerant<true>(fZ);
  } else {
    cout = absz > fZ;
  }
  if (cout) return;
  const double r2 = p.x() * p.x() + p.y() * p.y();
  if (forInside) {
    cout = cout || (r2 > MakePlusTolerantSquare<true>(fRmax));
    cin  = cin && (r2 < MakeMinusTolerantSquare<true>(fRmax));
  } else {
    cout = cout || (r2 > fRmax * fRmax);
  }
  if (cout) return;
  if (RminTreat()) {
    if (forInside) {
      cout = cout || (r2 <= MakeMinusTolerantSquare<true>(fRmin));
      cin  = cin && (r2 > MakePlusTolerantSquare<true>(fRmin));
    } else {
      cout = cout || (r2 <= fRmin * fRmin);
    }
    if (cout) return;
  }
  if (PhiTreat()) {
    bool cinphi = false, coutphi = false;
    fPhiWedge.ContainsAndInside(p, forInside, cinphi, coutphi);
    cout = cout || coutphi;
    if (forInside) cin = cin && cinphi;
  }
}

int Tube::Inside(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, cin, cout);
  int in = kSurface;
  if (cout) in = kOutside;
  if (cin) in = kInside;
  return in;
}
bool Tube::Contains(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}

// TubeImplementation.h:424-452 DistanceToIn (far-point pre-step)
double Tube::DistanceToIn(Vec3 const &pointt, Vec3 const &dir, double) const
{
  Vec3 point          = pointt;
  const double ptDist = point.Mag();
  double distToMove   = 0.;
  const double order  = 100.;
  if (ptDist > order * fMaxVal) {
    distToMove = ptDist - order * fMaxVal;
    point      = point + distToMove * dir;
  }
  double distance = DistanceToInKernel(point, dir);
  distance += distToMove;
  return distance;
}

// TubeImplementation.h:456-596 DistanceToInKernel
double Tube::DistanceToInKernel(Vec3 const &point, Vec3 const &dir) const
{
  bool done       = false;
  double distance = kInfLength;
  double distz    = Abs(point.z()) - fZ;
  done            = done || (distz > kHalfTolerance && point.z() * dir.z() >= 0);
  const double rsq   = point.x() * point.x() + point.y() * point.y();
  const double rdotn = point.x() * dir.x() + point.y() * dir.y();
  done               = done || (rsq > fTolIrmax2 && rdotn >= 0);
  if (done) return distance;
  distance    = -1.0;
  bool inside = distz < -kHalfTolerance;
  inside      = inside && (rsq < fTolIrmax2);
  if (RminTreat()) inside = inside && (rsq > fTolIrmin2);
  if (PhiTreat() && inside) {
    bool insector;
    PointInCyclicalSector(point.x(), point.y(), false, insector);
    inside = inside && insector;
  }
  done = done || inside;
  if (done) return distance;
  distance = kInfLength;

  distz /= NonZeroAbs(dir.z());
  const double hitx = point.x() + distz * dir.x();
  const double hity = point.y() + distz * dir.y();
  const double r2   = hitx * hitx + hity * hity;
  bool okz          = distz > -kHalfTolerance && (point.z() * dir.z() < 0);
  okz               = okz && (r2 <= fRmax2);
  if (RminTreat()) okz = okz && (fRmin2 <= r2);
  if (PhiTreat() && okz) {
    bool insector;
    PointInCyclicalSector(hitx, hity, true, insector);
    okz = okz && insector;
  }
  if (!done && okz) distance = distz;
  done = done || okz;

  bool onSurfIn = IsMovingInsideTubeSurface(point, dir, false);
  if (RminTreat()) onSurfIn = onSurfIn || IsMovingInsideTubeSurface(point, dir, true);
  if (!PhiTreat()) {
    if (!done && onSurfIn) distance = 0.;
    done = done || onSurfIn;
    if (done) return distance;
  } else {
    bool insector = false;
    PointInCyclicalSector(point.x(), point.y(), true, insector);
    if (!done && insector && onSurfIn) distance = 0.;
    done = done || (insector && onSurfIn);
    if (done) return distance;
  }

  const double invnsq = 1. / NonZero(1. - dir.z() * dir.z());
  const double b      = invnsq * rdotn;
  const double crmax  = invnsq * (rsq - fRmax2);
  double dist_rmax;
  bool ok_rmax = false;
  CircleTrajectoryIntersection(b, crmax, point, dir, false, true, dist_rmax, ok_rmax);
  ok_rmax = ok_rmax && (dist_rmax < distance);
  if (!done && ok_rmax) distance = dist_rmax;
  done = done || ok_rmax;
  if (done) return distance;

  double dist_rmin = -kInfLength;
  bool ok_rmin     = false;
  if (RminTreat()) {
    const double crmin = invnsq * (rsq - fRmin2);
    CircleTrajectoryIntersection(b, crmin, point, dir, true, true, dist_rmin, ok_rmin);
    ok_rmin = ok_rmin && (dist_rmin < distance);
    if (!done && ok_rmin) distance = dist_rmin;
  }

  if (PhiTreat()) {
    double dist_phi;
    bool ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi1x, fAlongPhi1y, fPhiWedge.normal1.x(), fPhiWedge.normal1.y(), point,
                                   dir, true, true, dist_phi, ok_phi);
    ok_phi = ok_phi && (dist_phi < distance);
    if (!done && ok_phi) distance = dist_phi;
    done = done || ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi2x, fAlongPhi2y, fPhiWedge.normal2.x(), fPhiWedge.normal2.y(), point,
                                   dir, true, true, dist_phi, ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  return distance;
}

// TubeImplementation.h:601-697 DistanceToOut
double Tube::DistanceToOut(Vec3 const &point, Vec3 const &dir, double) const
{
  double distance = -1.;
  bool done       = false;
  double distz    = fZ - Abs(point.z());
  done            = done || (distz < -kHalfTolerance);
  if (done) return distance;
  const double rsq   = point.x() * point.x() + point.y() * point.y();
  const double rdotn = dir.x() * point.x() + dir.y() * point.y();
  double crmax       = rsq - fRmax2;
  double crmin       = rsq;
  done               = done || (crmax > 2.0 * kTolerance * fRmax);
  if (done) return distance;
  if (RminTreat()) {
    crmin -= fRmin2;
    done = done || (crmin < -2.0 * kTolerance * fRmin);
    if (done) return distance;
  }
  if (PhiTreat()) {
    bool cinphi = false, coutphi = false;
    fPhiWedge.ContainsAndInside(point, true, cinphi, coutphi);
    done = done || coutphi;
    if (done) return distance;
  }
  distance             = kInfLength;
  const double invdirz = 1. / NonZero(dir.z());
  distz                = (fZ - point.z()) * invdirz;
  if (dir.z() < 0) distz = (-fZ - point.z()) * invdirz;
  if (!done && dir.z() != 0. && distz < distance) distance = distz;

  const double invnsq = 1. / NonZero(1. - dir.z() * dir.z());
  const double b      = invnsq * rdotn;
  if (RminTreat()) {
    double dist_rmin = kInfLength;
    bool ok_rmin     = false;
    crmin *= invnsq;
    CircleTrajectoryIntersection(b, crmin, point, dir, false, false, dist_rmin, ok_rmin);
    if (ok_rmin && dist_rmin < distance) distance = dist_rmin;
  }
  double dist_rmax = kInfLength;
  bool ok_rmax     = false;
  crmax *= invnsq;
  CircleTrajectoryIntersection(b, crmax, point, dir, true, false, dist_rmax, ok_rmax);
  if (ok_rmax && dist_rmax < distance) distance = dist_rmax;

  if (PhiTreat()) {
    double dist_phi = kInfLength;
    bool ok_phi     = false;
    // UniversalTube: the sector type is not known at compile time, so both phi planes are
    // tested with the positive-direction check (TubeImplementation.h:678-688).
    PhiPlaneTrajectoryIntersection(fAlongPhi1x, fAlongPhi1y, fPhiWedge.normal1.x(), fPhiWedge.normal1.y(), point,
                                   dir, true, false, dist_phi, ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi2x, fAlongPhi2y, fPhiWedge.normal2.x(), fPhiWedge.normal2.y(), point,
                                   dir, true, false, dist_phi, ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  return distance;
}

// TubeImplementation.h:758-781 SafetyToInOld (TUBE_SAFETY_OLD is defined at :20)
double Tube::SafetyToIn(Vec3 const &point) const
{
  double safety         = Abs(point.z()) - fZ;
  const double r        = Sqrt(point.x() * point.x() + point.y() * point.y());
  const double safermax = r - fRmax;
  if (safermax > safety) safety = safermax;
  if (RminTreat()) {
    const double safermin = fRmin - r;
    if (safermin > safety) safety = safermin;
  }
  if (PhiTreat()) {
    bool insector;
    PointInCyclicalSector(point.x(), point.y(), false, insector);
    if (insector) return safety;
    double safephi;
    PhiPlaneSafety(point, false, safephi);
    if (!insector && safephi < kInfLength && safephi > safety) safety = safephi;
  }
  return safety;
}

// TubeImplementation.h:785-802 SafetyToOutOld
double Tube::SafetyToOut(Vec3 const &point) const
{
  double safety         = fZ - Abs(point.z());
  const double r        = Sqrt(point.x() * point.x() + point.y() * point.y());
  const double safermax = fRmax - r;
  if (safermax < safety) safety = safermax;
  if (RminTreat()) {
    const double safermin = r - fRmin;
    if (safermin < safety) safety = safermin;
  }
  if (PhiTreat()) {
    const double safephi = fPhiWedge.SafetyToOut(point);
    if (safephi < safety) safety = safephi;
  }
  return safety;
}

// source/UnplacedTube.cpp:214-266 Extent
void Tube::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  aMin = Vec3(-fRmax, -fRmax, -fZ);
  aMax = Vec3(fRmax, fRmax, fZ);
  if (fDphi == kTwoPi) return;
  const double Rin     = 0.5 * (fRmax + fRmin);
  const bool phi0out   = !fPhiWedge.Contains(Vec3(Rin, 0, 0));
  const bool phi90out  = !fPhiWedge.Contains(Vec3(0, Rin, 0));
  const bool phi180out = !fPhiWedge.Contains(Vec3(-Rin, 0, 0));
  const bool phi270out = !fPhiWedge.Contains(Vec3(0, -Rin, 0));
  if (!(phi0out || phi90out || phi180out || phi270out)) return;
  const double Cx = fRmax * std::cos(fSphi);
  const double Dx = fRmax * std::cos(fSphi + fDphi);
  const double Cy = fRmax * std::sin(fSphi);
  const double Dy = fRmax * std::sin(fSphi + fDphi);
  if (phi0out) aMax[0] = Max(Cx, Dx);
  if (phi90out) aMax[1] = Max(Cy, Dy);
  if (phi180out) aMin[0] = Min(Cx, Dx);
  if (phi270out) aMin[1] = Min(Cy, Dy);
  if (fDphi >= kPi) return;
  const double Ax = fRmin * std::cos(fSphi);
  const double Bx = fRmin * std::cos(fSphi + fDphi);
  const double Ay = fRmin * std::sin(fSphi);
  const double By = fRmin * std::sin(fSphi + fDphi);
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

// ====================================================================== Cone
// VecGeom/volumes/ConeStruct.h:327-336 constructor, :292-325 SetAndCheck{D,S}PhiAngle
Cone::Cone(double rmin1, double rmax1, double rmin2, double rmax2, double dz, double sphi, double dphi)
    : fRmin1(rmin1 < 0.0 ? 0.0 : rmin1), fRmax1(rmax1), fRmin2(rmin2 < 0.0 ? 0.0 : rmin2), fRmax2(rmax2), fDz(dz),
      fSPhi(sphi), fDPhi(dphi), _frmin1(rmin1), _frmin2(rmin2), _frmax1(rmax1), _frmax2(rmax2), fPhiWedge(dphi, sphi)
{
  // SetAndCheckDPhiAngle(dphi)
  if (dphi >= kTwoPi - 0.5 * kAngTolerance) {
    fDPhi = kTwoPi;
    fSPhi = 0;
  } else if (dphi > 0) {
    fDPhi = dphi;
  }
  fPhiWedge.dphi = fDPhi;
  // SetAndCheckSPhiAngle(sphi); the wedge keeps the vectors of its construction angles.
  if (sphi < 0)
    fSPhi = kTwoPi - std::fmod(std::fabs(sphi), kTwoPi);
  else
    fSPhi = std::fmod(sphi, kTwoPi);
  if (fSPhi + fDPhi > kTwoPi) fSPhi -= kTwoPi;
  fAlongPhi1x = std::cos(fSPhi);
  fAlongPhi1y = std::sin(fSPhi);
  fAlongPhi2x = std::cos(fSPhi + fDPhi);
  fAlongPhi2y = std::sin(fSPhi + fDPhi);
  CalculateCached();
}

// ConeStruct.h:85-150 CalculateCached
void Cone::CalculateCached()
{
  fOriginalRmax1 = fRmax1;
  fOriginalRmax2 = fRmax2;
  if (fRmin1 == fRmax1) fRmax1 += kConeTolerance;
  if (fRmin2 == fRmax2) fRmax2 += kConeTolerance;
  fSqRmin1       = fRmin1 * fRmin1;
  fSqRmax1       = fRmax1 * fRmax1;
  fSqRmin2       = fRmin2 * fRmin2;
  fSqRmax2       = fRmax2 * fRmax2;
  fConeTolerance = 1e-7;
  fTanRMin       = (fRmin2 - fRmin1) * 0.5 / fDz;
  fSecRMin       = std::sqrt(1.0 + fTanRMin * fTanRMin);
  fInvSecRMin    = 1. / NonZero(fSecRMin);
  fTanRMax       = (fRmax2 - fRmax1) * 0.5 / fDz;
  fSecRMax       = std::sqrt(1.0 + fTanRMax * fTanRMax);
  fInvSecRMax    = 1. / NonZero(fSecRMax);
  fInnerSlope     = -(fRmin1 - fRmin2) / (2. * fDz);
  fOuterSlope     = -(fRmax1 - fRmax2) / (2. * fDz);
  fInnerOffset    = fRmin2 - fInnerSlope * fDz;
  fOuterOffset    = fRmax2 - fOuterSlope * fDz;
  fInnerTolerance = kConeTolerance * fSecRMin;
  fOuterTolerance = kConeTolerance * fSecRMax;
  if (fRmin2 > fRmin1) {
    fInnerConeApex     = 2 * fDz * fRmin1 / (fRmin2 - fRmin1);
    fTanInnerApexAngle = fRmin2 / (2 * fDz + fInnerConeApex);
  } else {
    fInnerConeApex     = 2 * fDz * fRmin2 / NonZero(fRmin1 - fRmin2);
    fTanInnerApexAngle = fRmin1 / (2 * fDz + fInnerConeApex);
  }
  if (fRmin1 == 0. || fRmin2 == 0.) fInnerConeApex = 0.;
  if (fRmin1 == 0.) fTanInnerApexAngle = fRmin2 / (2 * fDz);
  if (fRmin2 == 0.) fTanInnerApexAngle = fRmin1 / (2 * fDz);
  if (fRmax2 > fRmax1) {
    fOuterConeApex     = 2 * fDz * fRmax1 / (fRmax2 - fRmax1);
    fTanOuterApexAngle = fRmax2 / (2 * fDz + fOuterConeApex);
  } else {
    fOuterConeApex     = 2 * fDz * fRmax2 / NonZero(fRmax1 - fRmax2);
    fTanOuterApexAngle = fRmax1 / (2 * fDz + fOuterConeApex);
  }
  if (fRmax1 == 0. || fRmax2 == 0.) fOuterConeApex = 0.;
  if (fRmax1 == 0.) fTanOuterApexAngle = fRmax2 / (2 * fDz);
  if (fRmax2 == 0.) fTanOuterApexAngle = fRmax1 / (2 * fDz);
  fZNormInner = fTanRMin / NonZero(fSecRMin);
  fZNormOuter = -fTanRMax / NonZero(fSecRMax);
  fTolIz      = fDz - kHalfTolerance;
  fTolOz      = fDz + kHalfTolerance;
}

// VecGeom/volumes/ConeUtilities.h:113-131 GetRadiusOfConeAtPoint
double Cone::RadiusAt(double z, bool inner) const
{
  if (inner) return (fRmin1 == fRmin2) ? fRmin1 : fInnerSlope * z + fInnerOffset;
  return (fOriginalRmax1 == fOriginalRmax2) ? fOriginalRmax1 : fOuterSlope * z + fOuterOffset;
}

// ConeUtilities.h:70-108 PointInCyclicalSector (kConeTolerance band)
void Cone::PointInCyclicalSector(double x, double y, bool includeSurface, bool &ret) const
{
  const bool smallerthanpi = fDPhi <= M_PI;
  const double startCheck  = (-x * fAlongPhi1y) + (y * fAlongPhi1x);
  const double endCheck    = (-fAlongPhi2x * y) + (fAlongPhi2y * x);
  const double t           = includeSurface ? -kConeTolerance : kConeTolerance;
  if (smallerthanpi)
    ret = (startCheck >= t) && (endCheck >= t);
  else
    ret = (startCheck >= t) || (endCheck >= t);
}

// ConeUtilities.h:176-200 GetNormal
Vec3 Cone::GetNormal(Vec3 const &p, bool inner) const
{
  const double rho = p.Perp();
  if (inner) {
    if ((fRmin1 == fRmin2) && (fRmin1 != 0.)) return Vec3(-p.x(), -p.y(), 0.);
    return Vec3(-p.x(), -p.y(), fZNormInner * (rho * fSecRMin));
  }
  if ((fRmax1 == fRmax2) && (fRmax1 != 0.)) return Vec3(p.x(), p.y(), 0.);
  return Vec3(p.x(), p.y(), fZNormOuter * (rho * fSecRMax));
}

// ConeUtilities.h:204-216 IsOnConicalSurface
bool Cone::IsOnConicalSurface(Vec3 const &p, bool inner) const
{
  const double rho      = p.Perp2();
  const double coneRad  = RadiusAt(p.z(), inner);
  const double coneRad2 = coneRad * coneRad;
  const double tol      = inner ? fInnerTolerance : fOuterTolerance;
  return (rho >= (coneRad2 - tol * coneRad)) && (rho <= (coneRad2 + tol * coneRad)) &&
         (Abs(p.z()) < (fDz + kConeTolerance));
}

// ConeUtilities.h:146-174 PhiPlaneTrajectoryIntersection
void Cone::PhiPlaneTrajectoryIntersection(double alongX, double alongY, double normalX, double normalY,
                                          Vec3 const &pos, Vec3 const &dir, bool positiveDir, bool insectorCheck,
                                          double &dist, bool &ok) const
{
  dist = kInfLength;
  if (insectorCheck)
    ok = ((dir.x() * normalX) + (dir.y() * normalY) > 0.);
  else
    ok = ((dir.x() * normalX) + (dir.y() * normalY) < 0.);
  const double dirDotXY = (dir.y() * alongX) - (dir.x() * alongY);
  if (dirDotXY != 0) dist = ((alongY * pos.x()) - (alongX * pos.y())) / NonZero(dirDotXY);
  ok = ok && (dist > -kConeTolerance);
  if (insectorCheck) {
    const double hitx          = pos.x() + dist * dir.x();
    const double hity          = pos.y() + dist * dir.y();
    const double hitz          = pos.z() + dist * dir.z();
    const double r2            = (hitx * hitx) + (hity * hity);
    const double innerRadIrTol = RadiusAt(hitz, true) + kTolerance;
    const double outerRadIrTol = RadiusAt(hitz, false) - kTolerance;
    ok = ok && Abs(hitz) <= fTolIz && (r2 >= innerRadIrTol * innerRadIrTol) && (r2 <= outerRadIrTol * outerRadIrTol);
    if (positiveDir) ok = ok && ((hitx * alongX) + (hity * alongY)) > 0.;
  } else {
    if (positiveDir) {
      const double hitx = pos.x() + dist * dir.x();
      const double hity = pos.y() + dist * dir.y();
      ok                = ok && ((hitx * alongX) + (hity * alongY)) >= 0.;
    }
  }
}

// ConeUtilities.h, scalar ConeHelpers<Precision>::DetectIntersectionAndCalculateDistanceToConicalSurface
// (:551-684)
bool Cone::ConicalIntersection(Vec3 const &point, Vec3 const &direction, bool forDistToIn, bool inner,
                               double &distance) const
{
  distance                  = kInfLength;
  const bool onConical      = IsOnConicalSurface(point, inner);
  const Vec3 normal         = GetNormal(point, inner);
  const bool tangentToSurface = Abs(direction.Dot(normal)) == 0.;
  if (onConical && tangentToSurface) return false;
  if (onConical) {
    const double dn   = direction.Dot(GetNormal(point, inner));
    const bool moving = forDistToIn ? (dn <= 0.) : (dn >= 0.);
    if (!PhiTreat()) {
      if (moving) {
        distance = 0.;
        return true;
      }
    } else {
      bool insector = false;
      PointInCyclicalSector(point.x(), point.y(), true, insector);
      if (insector && moving) {
        distance = 0.;
        return true;
      }
    }
  }
  bool ok             = false;
  const double pDotV2D = point.x() * direction.x() + point.y() * direction.y();
  double a = kInfLength, b = kInfLength, c = kInfLength;
  if (inner) {
    if (fRmin1 == fRmin2) {
      b = pDotV2D;
      a = direction.Perp2();
      c = point.Perp2() - fRmin2 * fRmin2;
    } else {
      double newPz;
      if (fRmin2 > fRmin1)
        newPz = (point.z() + fDz + fInnerConeApex) * fTanInnerApexAngle;
      else
        newPz = (point.z() - fDz - fInnerConeApex) * fTanInnerApexAngle;
      const double dirT = direction.z() * fTanInnerApexAngle;
      a                 = (direction.x() * direction.x()) + (direction.y() * direction.y()) - dirT * dirT;
      b                 = pDotV2D - (newPz * dirT);
      c                 = point.Perp2() - (newPz * newPz);
    }
    const double b2 = b * b;
    const double ac = a * c;
    if (b2 < ac) return false;
    const double d2    = b2 - ac;
    const double delta = Sqrt(d2);
    if (forDistToIn) {
      if (b >= 0.)
        distance = (c / NonZero(-b - delta));
      else
        distance = (-b + delta) / NonZero(a);
    } else {
      if (b == 0. && delta == 0.) return false;
      if (b >= 0.)
        distance = (-b - delta) / NonZero(a);
      else
        distance = (c / NonZero(-b + delta));
    }
    if (distance < 0.) return false;
    const double newZ = point.z() + (direction.z() * distance);
    ok                = (Abs(newZ) < fDz);
  } else {
    if (fOriginalRmax1 == fOriginalRmax2) {
      a = direction.Perp2();
      b = pDotV2D;
      c = (point.Perp2() - fOriginalRmax2 * fOriginalRmax2);
    } else {
      double newPz;
      if (fOriginalRmax2 > fOriginalRmax1)
        newPz = (point.z() + fDz + fOuterConeApex) * fTanOuterApexAngle;
      else
        newPz = (point.z() - fDz - fOuterConeApex) * fTanOuterApexAngle;
      const double dirT = direction.z() * fTanOuterApexAngle;
      a                 = direction.x() * direction.x() + direction.y() * direction.y() - dirT * dirT;
      b                 = (pDotV2D - (newPz * dirT));
      c                 = (point.Perp2() - (newPz * newPz));
    }
    const double b2 = b * b;
    const double ac = a * c;
    const double d2 = b2 - ac;
    if (d2 < 0) return false;
    const double delta = Sqrt(d2);
    if (forDistToIn) {
      if (b == 0. && delta == 0.) return false;
      if (b > 0.)
        distance = (-b - delta) / NonZero(a);
      else
        distance = (c / NonZero(-b + delta));
      const double newZ = point.z() + (direction.z() * distance);
      ok                = (Abs(newZ) < fDz + kHalfTolerance);
    } else {
      if (b < 0.)
        distance = (-b + delta) / NonZero(a);
      else
        distance = (c / NonZero(-b - delta));
      ok = distance > 0.;
    }
    if (distance < 0.) return false;
  }
  if (PhiTreat()) {
    double hitx = 0, hity = 0;
    bool insector = false;
    if (distance < kInfLength) {
      hitx = point.x() + distance * direction.x();
      hity = point.y() + distance * direction.y();
    }
    PointInCyclicalSector(hitx, hity, true, insector);
    ok = ok && (insector && (distance < kInfLength));
  }
  return ok;
}

// ConeUtilities.h:686-724 scalar GenericKernelForContainsAndInside
void Cone::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double absz = Abs(p[2]);
  if (forInside) {
    cout = absz > fDz + kConeTolerance;
    cin  = absz < fDz - kConeTolerance;
  } else {
    cout = absz > fDz;
  }
  if (cout) return;
  const double r2 = p.x() * p.x() + p.y() * p.y();
  double rmax     = 0.;
  if (fOriginalRmax1 == fOriginalRmax2)
    rmax = fOriginalRmax1;
  else
    rmax = fOuterSlope * p.z() + fOuterOffset;
  if (forInside) {
    cout = cout || (r2 > MakePlusTolerantSquare<true>(rmax, fOuterTolerance));
    cin  = cin && (r2 < MakeMinusTolerantSquare<true>(rmax, fOuterTolerance));
  } else {
    cout = cout || (r2 > rmax * rmax);
  }
  if (cout) return;
  if (RminTreat()) {
    const double rmin = fInnerSlope * p.z() + fInnerOffset;
    if (forInside) {
      cout = cout || (r2 <= MakeMinusTolerantSquare<true>(rmin, fInnerTolerance));
      cin  = cin && (r2 > MakePlusTolerantSquare<true>(rmin, fInnerTolerance));
    } else {
      cout = cout || (r2 <= rmin * rmin);
    }
    if (cout) return;
  }
  if (PhiTreat()) {
    bool cinphi = false, coutphi = false;
    fPhiWedge.ContainsAndInside(p, forInside, cinphi, coutphi);
    cout = cout || coutphi;
    if (forInside) cin = cin && cinphi;
  }
}

int Cone::Inside(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, cin, cout);
  int in = kSurface;
  if (cout) in = kOutside;
  if (cin) in = kInside;
  return in;
}
bool Cone::Contains(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}

// VecGeom/volumes/kernel/ConeImplementation.h:126-258 DistanceToIn
double Cone::DistanceToIn(Vec3 const &point, Vec3 const &dir, double) const
{
  bool done       = false;
  double distance = kInfLength;
  double distz    = Abs(point.z()) - fDz;
  const bool outZAndGoingOut = (distz > kConeTolerance && (point.z() * dir.z()) >= 0.) ||
                               (Abs(distz) < kConeTolerance && (point.z() * dir.z()) > 0.);
  done = done || outZAndGoingOut;
  if (done) return distance;
  const double outerRad = RadiusAt(point.z(), false);
  const double rsq      = point.Perp2();
  done = done || ((rsq > MakeMinusTolerantSquare<true>(outerRad, fOuterTolerance)) &&
                  (dir.Dot(GetNormal(point, false)) >= 0.));
  if (done) return distance;
  distance    = -1.0;
  bool inside = distz < -kConeTolerance;
  inside      = inside && (rsq < MakeMinusTolerantSquare<true>(outerRad, fOuterTolerance));
  if (RminTreat()) {
    const double innerRad = RadiusAt(point.z(), true);
    inside                = inside && (rsq > MakePlusTolerantSquare<true>(innerRad, fInnerTolerance));
  }
  if (PhiTreat()) {
    bool insector;
    PointInCyclicalSector(point.x(), point.y(), false, insector);
    inside = inside && insector;
  }
  done = done || inside;
  if (done) return distance;
  distance = kInfLength;
  distz /= NonZero(Abs(dir.z()));
  const double hitx      = point.x() + distz * dir.x();
  const double hity      = point.y() + distz * dir.y();
  const double r2        = (hitx * hitx) + (hity * hity);
  const double innerZTol = fTolIz;
  bool isHittingTopPlane    = (point.z() >= innerZTol) && (r2 <= fSqRmax2 + kTolerance);
  bool isHittingBottomPlane = (point.z() <= -innerZTol) && (r2 <= fSqRmax1 + kTolerance);
  bool okz                  = (isHittingTopPlane || isHittingBottomPlane);
  if (RminTreat()) {
    isHittingTopPlane    = isHittingTopPlane && (r2 >= fSqRmin2 - kTolerance);
    isHittingBottomPlane = isHittingBottomPlane && (r2 >= fSqRmin1 - kTolerance);
    okz                  = okz && (isHittingTopPlane || isHittingBottomPlane);
  }
  if (PhiTreat()) {
    bool insector;
    PointInCyclicalSector(hitx, hity, true, insector);
    okz = okz && insector;
  }
  if (!done && okz) distance = distz;
  done = done || okz;
  if (done) return distance;

  double dist_rOuter = kInfLength;
  bool ok_outer      = ConicalIntersection(point, dir, true, false, dist_rOuter);
  ok_outer           = ok_outer && (dist_rOuter < distance);
  if (!done && ok_outer) distance = dist_rOuter;
  done = done || ok_outer;
  if (done) return distance;

  double dist_rInner = kInfLength;
  if (RminTreat()) {
    bool ok_inner = ConicalIntersection(point, dir, true, true, dist_rInner);
    ok_inner      = ok_inner && (dist_rInner < distance);
    if (!done && ok_inner) distance = dist_rInner;
  }
  if (PhiTreat()) {
    double dist_phi;
    bool ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi1x, fAlongPhi1y, fPhiWedge.normal1.x(), fPhiWedge.normal1.y(), point,
                                   dir, true, true, dist_phi, ok_phi);
    ok_phi = ok_phi && (dist_phi < distance);
    if (!done && ok_phi) distance = dist_phi;
    done = done || ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi2x, fAlongPhi2y, fPhiWedge.normal2.x(), fPhiWedge.normal2.y(), point,
                                   dir, true, true, dist_phi, ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  return distance;
}

// ConeImplementation.h:260-370 DistanceToOut
double Cone::DistanceToOut(Vec3 const &point, Vec3 const &direction, double) const
{
  double distance = kInfLength;
  bool done       = false;
  const double distz = Abs(point.z()) - fDz;
  distance           = -1.0;
  bool outside       = distz > kConeTolerance;
  const double rsq      = point.Perp2();
  const double outerRad = RadiusAt(point.z(), false);
  outside               = outside || (rsq > MakePlusTolerantSquare<true>(outerRad, fOuterTolerance));
  done                  = done || outside;
  if (done) return distance;
  if (RminTreat() && !outside) {
    const double innerRad = RadiusAt(point.z(), true);
    outside               = outside || (rsq < MakeMinusTolerantSquare<true>(innerRad, fInnerTolerance));
    done                  = done || outside;
    if (done) return distance;
  }
  // The reference guards the phi test with !MaskEmpty(outside); on the scalar path
  // `outside` is false here, so the phi sector is not tested (ConeImplementation.h:292-296).
  done = done || outside;
  if (done) return distance;
  const bool isGoingUp   = direction.z() > 0.;
  const bool isGoingDown = direction.z() < 0.;
  const bool isOnZPlaneAndMovingOutside =
      !outside && ((isGoingUp && point.z() > 0. && Abs(distz) < kConeTolerance) ||
                   (isGoingDown && point.z() < 0. && Abs(distz) < kConeTolerance));
  if (!done && isOnZPlaneAndMovingOutside) distance = distz;
  done = done || isOnZPlaneAndMovingOutside;
  if (done) return distance;
  distance             = kInfLength;
  const double dirZInv = 1. / NonZero(direction.z());
  if (isGoingUp) distance = (fDz - point.z()) * dirZInv;
  if (isGoingDown) distance = (-fDz - point.z()) * dirZInv;

  double dist_rOuter = kInfLength;
  const bool ok_outer = ConicalIntersection(point, direction, false, false, dist_rOuter);
  if (!done && ok_outer && dist_rOuter < distance) distance = dist_rOuter;
  double dist_rInner = kInfLength;
  if (RminTreat()) {
    const bool ok_inner = ConicalIntersection(point, direction, false, true, dist_rInner);
    if (!done && ok_inner && dist_rInner < distance) distance = dist_rInner;
  }
  if (PhiTreat()) {
    const bool isOnStartPhi = Wedge::IsOnSurfaceGeneric(fPhiWedge.along1, fPhiWedge.normal1, point);
    const bool isOnEndPhi   = Wedge::IsOnSurfaceGeneric(fPhiWedge.along2, fPhiWedge.normal2, point);
    const bool cond         = (isOnStartPhi && direction.Dot(-fPhiWedge.normal1) > 0.) ||
                      (isOnEndPhi && direction.Dot(-fPhiWedge.normal2) > 0.);
    if (!done && cond) distance = 0.;
    done = done || cond;
    if (done) return distance;
    double dist_phi;
    bool ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi1x, fAlongPhi1y, fPhiWedge.normal1.x(), fPhiWedge.normal1.y(), point,
                                   direction, true, false, dist_phi, ok_phi);
    ok_phi = ok_phi && (dist_phi < distance);
    if (!done && ok_phi) distance = dist_phi;
    done = done || ok_phi;
    PhiPlaneTrajectoryIntersection(fAlongPhi2x, fAlongPhi2y, fPhiWedge.normal2.x(), fPhiWedge.normal2.y(), point,
                                   direction, true, false, dist_phi, ok_phi);
    if (ok_phi && dist_phi < distance) distance = dist_phi;
  }
  if (distance < 0. && Abs(distance) < kTolerance) distance = 0.;
  return distance;
}

// ConeImplementation.h:372-436 SafetyToIn
double Cone::SafetyToIn(Vec3 const &point) const
{
  double safety = -kInfLength;
  const double distz = Abs(point.z()) - fDz;
  safety             = -1.0;
  bool inside        = distz < -kConeTolerance;
  const double outerRad = RadiusAt(point.z(), false);
  const double rsq      = point.Perp2();
  inside                = inside && (rsq < MakeMinusTolerantSquare<true>(outerRad, fOuterTolerance));
  if (RminTreat()) {
    const double innerRad = RadiusAt(point.z(), true);
    inside                = inside && (rsq > MakePlusTolerantSquare<true>(innerRad, fInnerTolerance));
  }
  if (PhiTreat() && inside) {
    bool insector;
    PointInCyclicalSector(point.x(), point.y(), false, insector);
    inside = inside && insector;
  }
  if (inside) return safety;
  safety                     = 0.;
  const double safeZ         = Abs(point.z()) - fDz;
  const double safeDistOuter = -SafeDistanceToConicalSurface(point, false);
  double safeDistInner       = -kInfLength;
  if (RminTreat()) safeDistInner = -SafeDistanceToConicalSurface(point, true);
  safety = Max(safeZ, Max(safeDistOuter, safeDistInner));
  if (PhiTreat()) {
    const double safetyPhi = fPhiWedge.SafetyToIn(point);
    safety                 = Max(safetyPhi, safety);
  }
  if (Abs(safety) < kTolerance) safety = 0.;
  return safety;
}

// ConeImplementation.h:437-496 SafetyToOut
double Cone::SafetyToOut(Vec3 const &point) const
{
  double safety         = kInfLength;
  const double distz    = Abs(point.z()) - fDz;
  const double rsq      = point.Perp2();
  safety                = -1.0;
  bool outside          = distz > kConeTolerance;
  const double outerRad = RadiusAt(point.z(), false);
  outside               = outside || (rsq > MakePlusTolerantSquare<true>(outerRad, fOuterTolerance));
  if (RminTreat()) {
    const double innerRad = RadiusAt(point.z(), true);
    outside               = outside || (rsq < MakeMinusTolerantSquare<true>(innerRad, fInnerTolerance));
  }
  if (outside) return safety;
  safety                     = 0.;
  const double safeZ         = fDz - Abs(point.z());
  const double safeDistOuter = SafeDistanceToConicalSurface(point, false);
  double safeDistInner       = kInfLength;
  if (RminTreat()) safeDistInner = SafeDistanceToConicalSurface(point, true);
  safety = Min(safeZ, Min(safeDistOuter, safeDistInner));
  if (PhiTreat()) {
    const double safetyPhi = fPhiWedge.SafetyToOut(point);
    safety                 = Min(safetyPhi, safety);
  }
  if (Abs(safety) < kTolerance) safety = 0.;
  return safety;
}

// ConeImplementation.h:498-516 SafeDistanceToConicalSurface
double Cone::SafeDistanceToConicalSurface(Vec3 const &point, bool inner) const
{
  const double rho = point.Perp();
  if (inner) {
    const double pRMin = fTanRMin * point.z() + (fRmin1 + fRmin2) * 0.5;
    return (rho - pRMin) * fInvSecRMin;
  }
  const double pRMax = fTanRMax * point.z() + (fRmax1 + fRmax2) * 0.5;
  return (pRMax - rho) * fInvSecRMax;
}

// source/UnplacedCone.cpp:149-211 Extent
void Cone::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  const double max = _frmax1 > _frmax2 ? _frmax1 : _frmax2;
  const double min = _frmin1 > _frmin2 ? _frmin2 : _frmin1;
  aMin             = Vec3(-max, -max, -fDz);
  aMax             = Vec3(max, max, fDz);
  if (fDPhi == kTwoPi) return;
  const double Rin     = 0.5 * (max + min);
  const bool phi0out   = !fPhiWedge.Contains(Vec3(Rin, 0, 0));
  const bool phi90out  = !fPhiWedge.Contains(Vec3(0, Rin, 0));
  const bool phi180out = !fPhiWedge.Contains(Vec3(-Rin, 0, 0));
  const bool phi270out = !fPhiWedge.Contains(Vec3(0, -Rin, 0));
  if (!(phi0out || phi90out || phi180out || phi270out)) return;
  const double Cx = max * std::cos(fSPhi);
  const double Dx = max * std::cos(fSPhi + fDPhi);
  const double Cy = max * std::sin(fSPhi);
  const double Dy = max * std::sin(fSPhi + fDPhi);
  if (phi0out) aMax[0] = Max(Cx, Dx);
  if (phi90out) aMax[1] = Max(Cy, Dy);
  if (phi180out) aMin[0] = Min(Cx, Dx);
  if (phi270out) aMin[1] = Min(Cy, Dy);
  if (fDPhi >= kPi) return;
  const double Ax = min * std::cos(fSPhi);
  const double Bx = min * std::cos(fSPhi + fDPhi);
  const double Ay = min * std::sin(fSPhi);
  const double By = min * std::sin(fSPhi + fDPhi);
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

} // namespace oracle
