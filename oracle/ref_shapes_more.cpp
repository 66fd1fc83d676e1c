// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
#include "ref_shapes_more.h"
#include "ref_nav.h"
#include <cmath>

namespace oracle {

constexpr double kTiny = 1e-30;

// ====================================================================== Trd
// TrdStruct.h:68-86 CalculateCached
Trd::Trd(double x1, double x2, double y1, double y2, double z) : fDX1(x1), fDX2(x2), fDY1(y1), fDY2(y2), fDZ(z)
{
  fX2minusX1    = fDX2 - fDX1;
  fY2minusY1    = fDY2 - fDY1;
  fHalfX1plusX2 = 0.5 * (fDX1 + fDX2);
  fHalfY1plusY2 = 0.5 * (fDY1 + fDY2);
  fFx           = 0.5 * (fDX1 - fDX2) / fDZ;
  fFy           = 0.5 * (fDY1 - fDY2) / fDZ;
  fSecxz        = std::sqrt(1 + fFx * fFx);
  fSecyz        = std::sqrt(1 + fFy * fFy);
  fCalfX        = 1. / Sqrt(1.0 + fFx * fFx);
  fCalfY        = 1. / Sqrt(1.0 + fFy * fFy);
  fToleranceX   = kTolerance * Sqrt(fX2minusX1 * fX2minusX1 + 4 * fDZ * fDZ);
  // the reference uses the x extent for the y tolerance as well (TrdStruct.h:85)
  fToleranceY = kTolerance * Sqrt(fX2minusX1 * fX2minusX1 + 4 * fDZ * fDZ);
}

// TrdImplementation.h:138-173 UnplacedInside (UniversalTrd: the y faces always take the
// cross-product test, HasVaryingY<UniversalTrd> is kUnknown)
void Trd::UnplacedInside(Vec3 const &point, bool surfaceT, bool &cin, bool &cout) const
{
  const double pzPlusDz = point.z() + fDZ;
  cout                  = Abs(point.z()) > (surfaceT ? fDZ + kHalfTolerance : fDZ);
  if (surfaceT) cin = Abs(point.z()) < fDZ - kHalfTolerance;
  double cross = fX2minusX1 * pzPlusDz - (2.0 * fDZ) * (Abs(point.x()) - fDX1);
  if (surfaceT) {
    cout = cout || (cross < -fToleranceX);
    cin  = cin && (cross > fToleranceX);
  } else {
    cout = cout || (cross < 0);
  }
  cross = fY2minusY1 * pzPlusDz - (2.0 * fDZ) * (Abs(point.y()) - fDY1);
  if (surfaceT) {
    cout = cout || (cross < -fToleranceY);
    cin  = cin && (cross > fToleranceY);
  } else {
    cout = cout || (cross < 0);
  }
}

// TrdImplementation.h:243-287 Inside (outside overrides inside), Contains
int Trd::Inside(Vec3 const &p) const
{
  bool in = false, out = false;
  UnplacedInside(p, true, in, out);
  int r = kSurface;
  if (in) r = kInside;
  if (out) r = kOutside;
  return r;
}
bool Trd::Contains(Vec3 const &p) const
{
  bool in = false, out = false;
  UnplacedInside(p, false, in, out);
  return !out;
}

// TrdImplementation.h:69-117 FaceTrajectoryIntersection
void Trd::Face(Vec3 const &pos, Vec3 const &dir, bool forY, bool mirrored, bool toInside, double &dist, bool &ok) const
{
  double alongV, posV, dirV, posK, dirK, fV, fK, halfKplus, v1, ndotv;
  if (forY) {
    alongV = fY2minusY1, v1 = fDY1, posV = pos.y(), posK = pos.x(), dirV = dir.y(), dirK = dir.x();
    fK = fFx, fV = fFy, halfKplus = fHalfX1plusX2;
  } else {
    alongV = fX2minusX1, v1 = fDX1, posV = pos.x(), posK = pos.y(), dirV = dir.x(), dirK = dir.y();
    fK = fFy, fV = fFx, halfKplus = fHalfY1plusY2;
  }
  if (mirrored) {
    posV *= -1.;
    dirV *= -1.;
  }
  ndotv = dirV + fV * dir.z();
  ok    = toInside ? (ndotv < 0.) : (ndotv > 0.);
  if (!ok) return;
  const double alongZ = 2.0 * fDZ;
  dist = (alongZ * (posV - v1) - alongV * (pos.z() + fDZ)) / (dir.z() * alongV - dirV * alongZ + kTiny);
  ok   = ok && (dist > -kHalfTolerance);
  if (ok) {
    const double hitz = pos.z() + dist * dir.z();
    ok                = ok && (Abs(hitz) <= fDZ);
    const double hitk = posK + dist * dirK;
    const double dK   = halfKplus - fK * hitz;
    ok                = ok && (Abs(hitk) <= dK);
    if (ok && Abs(dist) < kHalfTolerance) dist = 0.0;
  }
}

// TrdImplementation.h:118-137 Safety
double Trd::Safety(Vec3 const &pos, bool inside) const
{
  double dist        = fDZ - Abs(pos.z());
  const double distx = fHalfX1plusX2 - fFx * pos.z();
  const double safx  = (distx - Abs(pos.x())) * fCalfX;
  if (distx >= 0 && safx < dist) dist = safx;
  if (VaryingY()) {
    const double disty = fHalfY1plusY2 - fFy * pos.z();
    const double safy  = (disty - Abs(pos.y())) * fCalfY;
    if (disty >= 0 && safy < dist) dist = safy;
  } else {
    const double safy = fDY1 - Abs(pos.y());
    if (safy < dist) dist = safy;
  }
  return inside ? dist : -dist;
}

// TrdImplementation.h:288-370 DistanceToIn
double Trd::DistanceToIn(Vec3 const &point, Vec3 const &direction, double) const
{
  double distance = kInfLength;
  const bool inz  = Abs(point.z()) < fDZ - kHalfTolerance;
  double distx    = fHalfX1plusX2 - fFx * point.z();
  const bool inx  = (distx - Abs(point.x())) * fCalfX > kHalfTolerance;
  double disty;
  bool iny;
  if (VaryingY()) {
    disty = fHalfY1plusY2 - fFy * point.z();
    iny   = (disty - Abs(point.y())) * fCalfY > kHalfTolerance;
  } else {
    disty = Abs(point.y()) - fDY1;
    iny   = disty < -kHalfTolerance;
  }
  const bool inside = inx && iny && inz;
  if (inside) distance = -1.;
  bool done = inside;
  bool okz  = point.z() * direction.z() < 0.;
  okz       = okz && !inz;
  if (okz) {
    const double distz = (Abs(point.z()) - fDZ) / Abs(direction.z());
    const double hitx  = Abs(point.x() + distz * direction.x());
    const double hity  = Abs(point.y() + distz * direction.y());
    const bool okzt    = point.z() > (fDZ - kHalfTolerance) && hitx <= fDX2 && hity <= fDY2;
    const bool okzb    = point.z() < (-fDZ + kHalfTolerance) && hitx <= fDX1 && hity <= fDY1;
    okz                = okz && (okzt || okzb);
    if (okz) distance = distz;
  }
  done = done || okz;
  if (done) {
    if (Abs(distance) < kHalfTolerance) distance = 0.0;
    return distance;
  }
  bool okx = false;
  if (!inx) {
    Face(point, direction, false, false, true, distx, okx);
    if (okx) distance = distx;
    Face(point, direction, false, true, true, distx, okx);
    if (okx) distance = distx;
  }
  done = done || okx;
  if (done) {
    if (Abs(distance) < kHalfTolerance) distance = 0.0;
    return distance;
  }
  bool oky = false;
  if (VaryingY()) {
    if (!iny) {
      Face(point, direction, true, false, true, disty, oky);
      if (oky) distance = disty;
      Face(point, direction, true, true, true, disty, oky);
      if (oky) distance = disty;
    }
  } else {
    if (!iny) {
      disty /= Abs(direction.y());
      const double zhit = point.z() + disty * direction.z();
      const double xhit = point.x() + disty * direction.x();
      const double dx   = fHalfX1plusX2 - fFx * zhit;
      oky = point.y() * direction.y() < 0 && disty > -kHalfTolerance && Abs(xhit) < dx && Abs(zhit) < fDZ;
      if (oky) distance = disty;
    }
  }
  if (Abs(distance) < kHalfTolerance) distance = 0.0;
  return distance;
}

// TrdImplementation.h:371-470 DistanceToOut
double Trd::DistanceToOut(Vec3 const &point, Vec3 const &dir, double) const
{
  double distance     = 0.0;
  const double invdir = 1. / Abs(dir.z() + kTiny);
  const double safz   = fDZ - Abs(point.z());
  bool out            = safz < -kHalfTolerance;
  double distx        = fHalfX1plusX2 - fFx * point.z();
  out                 = out || ((distx - Abs(point.x())) * fCalfX < -kHalfTolerance);
  double disty;
  if (VaryingY()) {
    disty = fHalfY1plusY2 - fFy * point.z();
    out   = out || ((disty - Abs(point.y())) * fCalfY < -kHalfTolerance);
  } else {
    disty = fDY1 - Abs(point.y());
    out   = out || (disty < -kHalfTolerance);
  }
  if (out) return -1.;
  auto clamp = [](double d) { return Abs(d) < kHalfTolerance ? 0.0 : d; };
  if (dir.z() > 0.) {
    const double distz = (fDZ - point.z()) * invdir;
    const double hitx  = Abs(point.x() + distz * dir.x());
    const double hity  = Abs(point.y() + distz * dir.y());
    if (hitx <= fDX2 && hity <= fDY2) return clamp(distz);
  }
  if (dir.z() < 0.) {
    const double distz = (point.z() + fDZ) * invdir;
    const double hitx  = Abs(point.x() + distz * dir.x());
    const double hity  = Abs(point.y() + distz * dir.y());
    if (hitx <= fDX1 && hity <= fDY1) return clamp(distz);
  }
  bool okx;
  Face(point, dir, false, false, false, distx, okx);
  if (okx) return clamp(distx);
  Face(point, dir, false, true, false, distx, okx);
  if (okx) return clamp(distx);
  bool oky;
  if (VaryingY()) {
    Face(point, dir, true, false, false, disty, oky);
    if (oky) return clamp(disty);
    Face(point, dir, true, true, false, disty, oky);
    if (oky) distance = disty;
  } else {
    double plane = fDY1;
    if (dir.y() < 0.) plane = -fDY1;
    disty             = (plane - point.y()) / dir.y();
    const double zhit = point.z() + disty * dir.z();
    const double xhit = point.x() + disty * dir.x();
    const double dx   = fHalfX1plusX2 - fFx * zhit;
    oky               = Abs(xhit) < dx && Abs(zhit) < fDZ;
    if (oky) distance = disty;
  }
  return clamp(distance);
}

// source/UnplacedTrd / UnplacedTrd.h:218-222 Extent
void Trd::Extent(Vec3 &lo, Vec3 &hi) const
{
  lo = Vec3(-Max(fDX1, fDX2), -Max(fDY1, fDY2), -fDZ);
  hi = Vec3(Max(fDX1, fDX2), Max(fDY1, fDY2), fDZ);
}

// ====================================================================== Trap
// UnplacedTrapezoid.h:56-64 (tan of the alphas), TrapezoidStruct.h CalculateCached
// (tan(theta) cos(phi), tan(theta) sin(phi)), UnplacedTrapezoid.cpp:447-466
// FromParametersToCorners, then MakePlanes on those corners.
Trap::Trap(const double *par)
{
  const double dz = par[0], theta = par[1], phi = par[2], dy1 = par[3], dx1 = par[4], dx2 = par[5];
  const double ta1 = std::tan(par[6]), dy2 = par[7], dx3 = par[8], dx4 = par[9], ta2 = std::tan(par[10]);
  const double tcp = std::tan(theta) * std::cos(phi), tsp = std::tan(theta) * std::sin(phi);
  fDz                = dz;
  const double a1    = ta1 * dy1, a2 = ta2 * dy2;
  const double xz    = tcp * dz, yz = tsp * dz;
  Vec3 pt[8];
  pt[0] = Vec3(-xz - a1 - dx1, -yz - dy1, -dz);
  pt[1] = Vec3(-xz - a1 + dx1, -yz - dy1, -dz);
  pt[2] = Vec3(-xz + a1 - dx2, -yz + dy1, -dz);
  pt[3] = Vec3(-xz + a1 + dx2, -yz + dy1, -dz);
  pt[4] = Vec3(+xz - a2 - dx3, +yz - dy2, +dz);
  pt[5] = Vec3(+xz - a2 + dx3, +yz - dy2, +dz);
  pt[6] = Vec3(+xz + a2 - dx4, +yz + dy2, +dz);
  pt[7] = Vec3(+xz + a2 + dx4, +yz + dy2, +dz);
  MakePlanes(pt);
}
// UnplacedTrapezoid.cpp:496-524 fromCornersToParameters: dz from the last corner, planes
// straight from the corners (the derived parameters are not used by the queries).
Trap::Trap(const Vec3 *corners)
{
  fDz = corners[7].z();
  MakePlanes(corners);
}
Trap::Trap(double dz, const double *planes) : fDz(dz)
{
  for (int i = 0; i < 4; ++i)
    fA[i] = planes[4 * i], fB[i] = planes[4 * i + 1], fC[i] = planes[4 * i + 2], fD[i] = planes[4 * i + 3];
}
// UnplacedTrapezoid.cpp:630-679 MakePlanes: faces (0,1,5,4) -Y, (2,6,7,3) +Y, (0,4,6,2) -X,
// (1,3,7,5) +X.
void Trap::MakePlanes(const Vec3 *pt)
{
  MakeAPlane(pt[0], pt[1], pt[5], pt[4], 0);
  MakeAPlane(pt[2], pt[6], pt[7], pt[3], 1);
  MakeAPlane(pt[0], pt[4], pt[6], pt[2], 2);
  MakeAPlane(pt[1], pt[3], pt[7], pt[5], 3);
}
// UnplacedTrapezoid.cpp:569-620 MakeAPlane: normal (p3 - p1) x (p4 - p2) scaled by 1/|n|
// (Vector3D::Normalize), d = -n . (p1 + p2 + p3 + p4) / 4 (summed left to right, times 0.25).
void Trap::MakeAPlane(Vec3 const &p1, Vec3 const &p2, Vec3 const &p3, Vec3 const &p4, int i)
{
  const Vec3 u = p3 - p1, v = p4 - p2;
  Vec3 n(u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]);
  const double inv = 1. / n.Mag();
  n                = n * inv;
  const Vec3 c     = 0.25 * (((p1 + p2) + p3) + p4);
  fA[i] = n[0], fB[i] = n[1], fC[i] = n[2], fD[i] = -n.Dot(c);
}
// TrapezoidImplementation.h:82-106 + PlaneShell.h GenericKernelForContainsAndInside
void Trap::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double h = forInside ? kHalfTolerance : 0.;
  cout           = Abs(p.z()) > fDz + (forInside ? kHalfTolerance : 0.);
  if (forInside) cin = Abs(p.z()) < fDz - kHalfTolerance;
  double dist[4];
  for (int i = 0; i < 4; ++i) dist[i] = PlaneDist(i, p);
  for (int i = 0; i < 4; ++i) {
    cout = cout || dist[i] > 0. + h;
    if (forInside) cin = cin && dist[i] < 0. - h;
  }
}
// TrapezoidImplementation.h:65-78 Inside (outside assigned first, then inside), :56-64 Contains
int Trap::Inside(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, cin, cout);
  int r = kSurface;
  if (cout) r = kOutside;
  if (cin) r = kInside;
  return r;
}
bool Trap::Contains(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}
// TrapezoidImplementation.h:107-126 (z slab) + PlaneShell.h DistanceToIn (side planes clip
// [smin, smax]; early returns with kInfLength)
double Trap::DistanceToIn(Vec3 const &p, Vec3 const &d, double) const
{
  const double sz  = Sign(d.z());
  const double max = sz * fDz - p.z();
  if (sz * max < 0.0 + kHalfTolerance) return kInfLength;
  const double invdir = 1.0 / NonZero(d.z());
  double smax         = max * invdir;
  double smin         = -(sz * fDz + p.z()) * invdir;
  double pdist[4], proj[4], vdist[4];
  for (int i = 0; i < 4; ++i) {
    pdist[i] = PlaneDist(i, p);
    proj[i]  = PlaneProj(i, d);
    vdist[i] = -pdist[i] / NonZero(proj[i]);
  }
  for (int i = 0; i < 4; ++i) {
    if (pdist[i] > 0. + kHalfTolerance && proj[i] >= 0.) return kInfLength;
    if (pdist[i] > 0. - kHalfTolerance && proj[i] > 0.) return kInfLength;
  }
  for (int i = 0; i < 4; ++i) {
    const bool posPoint = pdist[i] > 0. - kHalfTolerance;
    const bool posDir   = proj[i] > 0;
    const bool fromIn   = !posPoint && posDir;
    const bool fromOut  = posPoint && !posDir;
    if ((fromIn && vdist[i] < smin) || (fromOut && vdist[i] > smax)) return kInfLength;
    if (fromOut && vdist[i] > smin) smin = vdist[i];
    if (fromIn && vdist[i] < smax) smax = vdist[i];
  }
  return smin <= smax ? smin : kInfLength;
}
// TrapezoidImplementation.h:151-167 + PlaneShell.h DistanceToOut (planes taken in order:
// -1 when outside a plane, then any smaller exit distance of a plane the ray leaves by)
double Trap::DistanceToOut(Vec3 const &p, Vec3 const &d, double) const
{
  if (Abs(p.z()) > fDz + kHalfTolerance) return -1.;
  double distance    = kInfLength;
  const double distz = (Sign(d.z()) * fDz - p.z()) / NonZero(d.z());
  if (d.z() != 0.) distance = distz;
  double out = kInfLength;
  double pdist[4], proj[4], vdist[4];
  for (int i = 0; i < 4; ++i) {
    pdist[i] = PlaneDist(i, p);
    proj[i]  = PlaneProj(i, d);
    vdist[i] = -pdist[i] / NonZero(proj[i]);
  }
  for (int i = 0; i < 4; ++i) {
    if (pdist[i] > kHalfTolerance) out = -1.;
    if (proj[i] > 0. && vdist[i] < out) out = vdist[i];
  }
  if (out < distance) distance = out;
  return distance;
}
// TrapezoidImplementation.h:183-200 + PlaneShell.h SafetyToIn (N = 4: sequential maximum)
double Trap::SafetyToIn(Vec3 const &p) const
{
  double safety = Abs(p.z()) - fDz;
  double dist[4];
  for (int i = 0; i < 4; ++i) dist[i] = PlaneDist(i, p);
  for (int i = 0; i < 4; ++i)
    if (dist[i] > safety) safety = dist[i];
  return safety;
}
// TrapezoidImplementation.h:201-218 + PlaneShell.h SafetyToOut (N = 4: sequential minimum)
double Trap::SafetyToOut(Vec3 const &p) const
{
  double safety = fDz - Abs(p.z());
  double dist[4];
  for (int i = 0; i < 4; ++i) dist[i] = -PlaneDist(i, p);
  for (int i = 0; i < 4; ++i)
    if (dist[i] < safety) safety = dist[i];
  return safety;
}
// UnplacedTrapezoid.cpp:298-337 Extent on the corners of UnplacedTrapezoid.cpp:468-494
// fromPlanesToCorners (each corner re-derived from the planes).
void Trap::Extent(Vec3 &lo, Vec3 &hi) const
{
  const double z = fDz;
  double y[8], x[8];
  y[0] = y[1] = -(fD[0] - z * fC[0]) / fB[0];
  y[2] = y[3] = -(fD[1] - z * fC[1]) / fB[1];
  y[4] = y[5] = -(fD[0] + z * fC[0]) / fB[0];
  y[6] = y[7] = -(fD[1] + z * fC[1]) / fB[1];
  // corner k lies on the y plane yp (0 or 1) and the x plane xp (2 or 3), at z = -+fDz
  for (int k = 0; k < 8; ++k) {
    const int yp = (k >> 1) & 1, xp = 2 + (k & 1);
    const double s = (k < 4) ? -z : z;
    x[k] = ((fB[xp] / fB[yp]) * (fD[yp] + s * fC[yp]) - (fD[xp] + s * fC[xp])) / fA[xp];
  }
  auto mx = [](const double *v) { return Max(Max(Max(v[0], v[1]), Max(v[2], v[3])), Max(Max(v[4], v[5]), Max(v[6], v[7]))); };
  auto mn = [](const double *v) { return Min(Min(Min(v[0], v[1]), Min(v[2], v[3])), Min(Min(v[4], v[5]), Min(v[6], v[7]))); };
  lo = Vec3(mn(x), mn(y), -fDz);
  hi = Vec3(mx(x), mx(y), fDz);
}

// ====================================================================== Polycone
// PolyconeStruct.h:124-239 Init (sections are ConeStruct(prevRmin, prevRmax, rMin, rMax,
// dz, phiStart, phiTotal) shifted to the middle of their z range)
Polycone::Polycone(double phiStart, double phiTotal, int nz, const double *zPlane, const double *rInner,
                   const double *rOuter)
{
  // SetAndCheckDPhiAngle / SetAndCheckSPhiAngle
  if (phiTotal >= kTwoPi - 0.5 * kAngTolerance) {
    fDeltaPhi = kTwoPi;
    fStartPhi = 0;
  } else if (phiTotal > 0) {
    fDeltaPhi = phiTotal;
  }
  fStartPhi = phiStart < 0 ? kTwoPi - std::fmod(std::fabs(phiStart), kTwoPi) : std::fmod(phiStart, kTwoPi);
  if (fStartPhi + fDeltaPhi > kTwoPi) fStartPhi -= kTwoPi;
  std::vector<double> z(zPlane, zPlane + nz), rin(rInner, rInner + nz), rout(rOuter, rOuter + nz);
  if (zPlane[0] > zPlane[nz - 1])
    for (int i = 0; i < nz; ++i) z[i] = zPlane[nz - 1 - i], rin[i] = rInner[nz - 1 - i], rout[i] = rOuter[nz - 1 - i];
  if (phiTotal <= 0. || phiTotal > kTwoPi - kTolerance) {
    fStartPhi = 0;
    fDeltaPhi = kTwoPi;
  } else {
    fStartPhi = phiStart;
    while (fStartPhi < 0) fStartPhi += kTwoPi;
  }
  double prevZ = z[0], prevRmax = 0, prevRmin = 0;
  int dirZ = 1;
  if (z[1] < z[0]) dirZ = -1;
  for (int i = 0; i < nz; ++i) {
    const double rMin = rin[i], rMax = rout[i], zz = z[i];
    if (i > 0) {
      if (((zz > prevZ + kTolerance) && (dirZ > 0)) || ((zz < prevZ - kTolerance) && (dirZ < 0))) {
        const double dz = (zz - prevZ) / 2;
        fSolids.emplace_back(new Cone(prevRmin, prevRmax, rMin, rMax, dz, phiStart, phiTotal));
        fZs.push_back(zz);
        const int zi = (int)fZs.size() - 1;
        fShift.push_back(fZs[zi - 1] + 0.5 * (fZs[zi] - fZs[zi - 1]));
      }
    } else {
      fZs.push_back(zz);
    }
    prevZ    = zz;
    prevRmin = rMin;
    prevRmax = rMax;
  }
}

// PolyconeStruct.h:246-253 GetSectionIndex
int Polycone::GetSectionIndex(double zposition) const
{
  if (zposition < fZs[0]) return -1;
  for (int i = 0; i < NSections(); ++i)
    if (zposition >= fZs[i] && zposition <= fZs[i + 1]) return i;
  return -2;
}

// PolyconeImplementation.h:58-79 GenericKernelForASection
void Polycone::SectionKernel(int isect, Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  if (isect < 0) {
    cin  = false;
    cout = true;
    return;
  }
  fSolids[isect]->ContainsAndInside(Local(p, isect), forInside, cin, cout);
}

// PolyconeImplementation.h:103-147 GenericKernelForContainsAndInside
void Polycone::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const int indexLow  = GetSectionIndex(p.z() - kTolerance);
  const int indexHigh = GetSectionIndex(p.z() + kTolerance);
  if (indexLow < 0 && indexHigh < 0) {
    cout = true;
    return;
  }
  if (indexLow < 0 && indexHigh == 0) {
    SectionKernel(0, p, forInside, cin, cout);
    return;
  }
  if (indexHigh < 0 && indexLow == (NSections() - 1)) {
    SectionKernel(NSections() - 1, p, forInside, cin, cout);
    return;
  }
  if (indexLow >= 0 && indexHigh >= 0) {
    if (indexLow == indexHigh) {
      SectionKernel(indexLow, p, forInside, cin, cout);
      return;
    }
    bool inLow = false, outLow = false, inHigh = false, outHigh = false;
    SectionKernel(indexLow, p, forInside, inLow, outLow);
    SectionKernel(indexHigh, p, forInside, inHigh, outHigh);
    const bool surfLow  = !inLow && !outLow;
    const bool surfHigh = !inHigh && !outHigh;
    if (surfLow && surfHigh) {
      cin = true;
      return;
    }
    if (outLow && outHigh) {
      cout = true;
      return;
    }
  }
}

int Polycone::Inside(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, cin, cout);
  int r = kSurface;
  if (cout) r = kOutside;
  if (cin) r = kInside;
  return r;
}
bool Polycone::Contains(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}

// PolyconeImplementation.h:148-180 DistanceToIn
double Polycone::DistanceToIn(Vec3 const &p, Vec3 const &v, double smax) const
{
  double distance = kInfLength;
  int increment   = (v.z() > 0) ? 1 : -1;
  if (std::fabs(v.z()) < kTolerance) increment = 0;
  int index = GetSectionIndex(p.z());
  if (index == -1) index = 0;
  if (index == -2) index = NSections() - 1;
  do {
    distance = fSolids[index]->DistanceToIn(Local(p, index), v, smax);
    if (distance < kInfLength || !increment) break;
    index += increment;
  } while (index >= 0 && index < NSections());
  return distance;
}

// PolyconeImplementation.h:181-300 DistanceToOut
double Polycone::DistanceToOut(Vec3 const &point, Vec3 const &dir, double smax) const
{
  double distance = kInfLength;
  Vec3 pn         = point;
  if (NSections() == 1) return fSolids[0]->DistanceToOut(Local(point, 0), dir, smax);
  const int indexLow  = GetSectionIndex(point.z() - kTolerance);
  const int indexHigh = GetSectionIndex(point.z() + kTolerance);
  int index           = 0;
  if (indexLow < 0 && indexHigh < 0) {
    return -1;
  } else if (indexLow < 0 && indexHigh >= 0) {
    index = indexHigh;
    if (fSolids[index]->Inside(Local(point, index)) == kOutside) return -1;
  } else if (indexLow != indexHigh && (indexLow >= 0)) {
    if (fSolids[indexLow]->Inside(Local(point, indexLow)) == kOutside)
      index = indexHigh;
    else
      index = indexLow;
  } else {
    index = indexLow;
    if (index < 0) index = GetSectionIndex(point.z());
  }
  if (index < 0) return 0.;
  if (fSolids[index]->Inside(Local(point, index)) == kOutside) return -1;
  double totalDistance = 0.;
  double dist;
  int increment = (dir.z() > 0) ? 1 : -1;
  if (std::fabs(dir.z()) < kTolerance) increment = 0;
  int istep = 0;
  do {
    if ((totalDistance != 0) || (istep < 2)) {
      pn = point + totalDistance * dir;
      pn[2] -= fShift[index];
      if (fSolids[index]->Inside(pn) == kOutside) break;
    } else {
      pn[2] -= fShift[index];
    }
    istep++;
    dist = fSolids[index]->DistanceToOut(pn, dir, smax);
    if (dist == -1) return distance;
    if (std::fabs(dist) < 0.5 * kTolerance) {
      int index1 = index;
      if ((index > 0) && (index < NSections() - 1)) {
        index1 += increment;
      } else {
        if ((index == 0) && (increment > 0)) index1 += increment;
        if ((index == NSections() - 1) && (increment < 0)) index1 += increment;
      }
      Vec3 pte = point + (totalDistance + dist) * dir;
      pte[2] -= fShift[index1];
      const int inside22 = fSolids[index1]->Inside(pte);
      if (inside22 == 3 || (increment == 0)) break;
    }
    totalDistance += dist;
    index += increment;
  } while (increment != 0 && index >= 0 && index < NSections());
  return totalDistance;
}

// PolyconeImplementation.h:301-354 SafetyToIn
double Polycone::SafetyToIn(Vec3 const &p) const
{
  int index  = GetSectionIndex(p.z());
  bool needZ = false;
  if (index < 0) {
    needZ = true;
    if (index == -1) index = 0;
    if (index == -2) index = NSections() - 1;
  }
  double safety = fSolids[index]->SafetyToIn(Local(p, index));
  if (needZ) return safety;
  if (safety < kTolerance) return safety;
  double minSafety = safety;
  double zbase     = fZs[index + 1];
  for (int i = index + 1; i < NSections(); ++i) {
    const double dz = fZs[i] - zbase;
    if (dz >= minSafety) break;
    safety = fSolids[i]->SafetyToIn(Local(p, i));
    if (safety < minSafety) minSafety = safety;
  }
  if (index > 0) {
    zbase = fZs[index - 1];
    for (int i = index - 1; i >= 0; --i) {
      const double dz = zbase - fZs[i];
      if (dz >= minSafety) break;
      safety = fSolids[i]->SafetyToIn(Local(p, i));
      if (safety < minSafety) minSafety = safety;
    }
  }
  return minSafety;
}

// PolyconeImplementation.h:355-410 SafetyToOut
double Polycone::SafetyToOut(Vec3 const &point) const
{
  bool compIn = false, compOut = false;
  ContainsAndInside(point, true, compIn, compOut);
  if (compOut) return -1;
  const int index = GetSectionIndex(point.z());
  if (index < 0) return -1;
  double safety    = fSolids[index]->SafetyToOut(Local(point, index));
  double minSafety = safety;
  if (minSafety == kInfLength) return 0.;
  if (minSafety < kTolerance) return 0.;
  double zbase = fZs[index + 1];
  for (int i = index + 1; i < NSections(); ++i) {
    const double dz = fZs[i] - zbase;
    if (dz >= minSafety) break;
    safety = fSolids[i]->SafetyToIn(Local(point, i));
    if (safety < minSafety) minSafety = safety;
  }
  if (index > 0) {
    zbase = fZs[index - 1];
    for (int i = index - 1; i >= 0; --i) {
      const double dz = zbase - fZs[i];
      if (dz >= minSafety) break;
      safety = fSolids[i]->SafetyToIn(Local(point, i));
      if (safety < minSafety) minSafety = safety;
    }
  }
  return minSafety;
}

// source/UnplacedPolycone.cpp:865-902 Extent (the xy part is a cone's extent over the radius range)
void Polycone::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  double maxR = 0, minR = kInfLength;
  for (auto const &s : fSolids) {
    maxR = Max(maxR, Max(s->_frmax1, s->_frmax2));
    minR = Min(minR, Min(s->_frmin1, s->_frmin2));
  }
  double zlo, zhi;
  if (fZs[0] > fZs[NSections()]) {
    zhi = fZs[0];
    zlo = fZs[NSections()];
  } else {
    zlo = fZs[0];
    zhi = fZs[NSections()];
  }
  Cone tempCone(minR, maxR, minR, maxR, 1, fStartPhi, fDeltaPhi);
  tempCone.Extent(aMin, aMax);
  aMin[2] = zlo;
  aMax[2] = zhi;
}

// ====================================================================== Boolean subtraction
// BooleanImplementation.h:64-72 Contains
bool BooleanMinus::Contains(Vec3 const &p) const
{
  if (!fLeft->Contains(p)) return false;
  return !fRight->Contains(p);
}

// BooleanImplementation.h:73-107 Inside
int BooleanMinus::Inside(Vec3 const &p) const
{
  const int a = fLeft->Inside(p);
  if (a == kOutside) return kOutside;
  const int b = fRight->Inside(p);
  if (a == kInside && b == kOutside) return kInside;
  if ((a == kInside && b == kSurface) || (b == kOutside && a == kSurface)) return kSurface;
  return kOutside;
}

// BooleanImplementation.h:108-147 DistanceToIn (push loop with kPushTolerance)
double BooleanMinus::DistanceToIn(Vec3 const &p, Vec3 const &dir, double stepMax) const
{
  double d1, d2, snxt = 0.;
  Vec3 hitpoint      = p;
  bool insideRight   = fRight->Contains(p);
  const double epsil = kPushTolerance;
  while (true) {
    if (insideRight) {
      d1 = fRight->PlacedDistanceToOut(hitpoint, dir, stepMax);
      snxt += (d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) : 0.;
      hitpoint = hitpoint + ((d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) * dir : 0. * dir);
      if (fLeft->Contains(hitpoint)) {
        const double check = fLeft->PlacedDistanceToOut(hitpoint, dir, kInfLength);
        if (check > epsil) return snxt;
      }
    }
    d2 = fLeft->DistanceToIn(hitpoint, dir, stepMax);
    d2 = Max(d2, 0.);
    if (d2 == kInfLength) return kInfLength;
    d1 = fRight->DistanceToIn(hitpoint, dir, stepMax);
    if (d2 < d1 - kTolerance) {
      snxt += d2 + epsil;
      return snxt;
    }
    snxt += (d1 >= 0. && d1 < kInfLength) ? d1 + epsil : 0.;
    hitpoint    = hitpoint + ((d1 >= 0. && d1 < kInfLength) ? (d1 + epsil) * dir : epsil * dir);
    insideRight = true;
  }
}

// BooleanImplementation.h:148-157 DistanceToOut
double BooleanMinus::DistanceToOut(Vec3 const &p, Vec3 const &d, double stepMax) const
{
  const double distancel = fLeft->PlacedDistanceToOut(p, d, stepMax);
  const double dinright  = fRight->DistanceToIn(p, d, stepMax);
  return Min(distancel, dinright);
}

// BooleanImplementation.h:158-170 SafetyToIn
double BooleanMinus::SafetyToIn(Vec3 const &p) const
{
  if (fLeft->Contains(p) && fRight->Contains(p)) return fRight->SafetyToOut(fRight->T.Transform(p));
  return fLeft->SafetyToIn(p);
}

// BooleanImplementation.h:171-178 SafetyToOut (the left operand is queried in the
// boolean's own frame, as the reference does)
double BooleanMinus::SafetyToOut(Vec3 const &p) const
{
  const double sl = fLeft->SafetyToOut(p);
  const double sr = fRight->SafetyToIn(p);
  return Min(sl, sr);
}

// source/UnplacedBooleanVolume.cpp:403-441 TransformedExtent: the operand's extent box
// corners brought into the boolean's frame
static void TransformedExtent(PlacedVolume const *pv, Vec3 &aMin, Vec3 &aMax)
{
  Vec3 lower, upper;
  pv->Shape()->Extent(lower, upper);
  const Vec3 delta = upper - lower;
  double mn[3] = {kInfLength, kInfLength, kInfLength}, mx[3] = {-kInfLength, -kInfLength, -kInfLength};
  for (int x = 0; x <= 1; ++x)
    for (int y = 0; y <= 1; ++y)
      for (int z = 0; z <= 1; ++z) {
        Vec3 c(lower.x() + x * delta.x(), lower.y() + y * delta.y(), lower.z() + z * delta.z());
        const Vec3 t = pv->T.InverseTransform(c);
        for (int k = 0; k < 3; ++k) {
          mn[k] = std::min(mn[k], t[k]);
          mx[k] = std::max(mx[k], t[k]);
        }
      }
  aMin = Vec3(mn[0], mn[1], mn[2]);
  aMax = Vec3(mx[0], mx[1], mx[2]);
}

// ====================================================================== Boolean union
// BooleanUnionImplementation.h:62-69 Contains
bool BooleanUnion::Contains(Vec3 const &p) const
{
  if (fLeft->Contains(p)) return true;
  return fRight->Contains(p);
}

// BooleanUnionImplementation.h:71-118 Inside (touching solids on both surfaces count as
// inside when their outward normals oppose)
int BooleanUnion::Inside(Vec3 const &p) const
{
  const int a = fLeft->Inside(p);
  if (a == kInside) return kInside;
  const int b = fRight->Inside(p);
  if (b == kInside) return kInside;
  if (a == kSurface && b == kSurface) {
    bool va = false, vb = false;
    const Vec3 na = fLeft->T.InverseTransformDirection(fLeft->Shape()->Normal(fLeft->T.Transform(p), va));
    const Vec3 nb = fRight->T.InverseTransformDirection(fRight->Shape()->Normal(fRight->T.Transform(p), vb));
    return na.Dot(nb) < 0 ? kInside : kSurface;
  }
  return (a == kSurface || b == kSurface) ? kSurface : kOutside;
}

// BooleanUnionImplementation.h:120-128 DistanceToIn
double BooleanUnion::DistanceToIn(Vec3 const &p, Vec3 const &d, double stepMax) const
{
  const double d1 = fLeft->DistanceToIn(p, d, stepMax);
  const double d2 = fRight->DistanceToIn(p, d, stepMax);
  return Min(d1, d2);
}

// BooleanUnionImplementation.h:130-178 DistanceToOut: leave the operand the point is in,
// push by kPushTolerance, continue through the other operand while it connects
double BooleanUnion::DistanceToOut(Vec3 const &point, Vec3 const &dir, double) const
{
  double dist           = 0.;
  const double pushdist = kPushTolerance;
  const int positionA   = fLeft->Inside(point);
  Vec3 nextp            = point;
  bool connecting       = false;
  auto kernel = [&](PlacedVolume const *A, PlacedVolume const *B) {
    do {
      connecting       = false;
      const double d1  = A->PlacedDistanceToOut(nextp, dir, kInfLength);
      dist += (d1 >= 0. && d1 < kInfLength) ? d1 : 0;
      dist += pushdist;
      nextp = point + dist * dir;
      if (B->Inside(nextp) != kOutside) {
        const double d2 = B->PlacedDistanceToOut(nextp, dir, kInfLength);
        dist += (d2 >= 0. && d2 < kInfLength) ? d2 : 0;
        dist += pushdist;
        nextp      = point + dist * dir;
        connecting = true;
      }
    } while (connecting && (A->Inside(nextp) != kOutside));
  };
  if (positionA != kOutside)
    kernel(fLeft, fRight);
  else
    kernel(fRight, fLeft);
  double distance = dist - pushdist;
  if (distance < kTolerance && positionA == kOutside && fRight->Inside(point) == kOutside) distance = -kTolerance;
  return distance;
}

// BooleanUnionImplementation.h:180-191 SafetyToIn
double BooleanUnion::SafetyToIn(Vec3 const &p) const
{
  const double a = fLeft->SafetyToIn(p);
  const double b = fRight->SafetyToIn(p);
  return Min(a, b);
}

// BooleanUnionImplementation.h:193-218 SafetyToOut
double BooleanUnion::SafetyToOut(Vec3 const &p) const
{
  const int ia = fLeft->Inside(p);
  const int ib = fRight->Inside(p);
  if (ia == kOutside && ib == kOutside) return -kTolerance;
  if (ia != kOutside && ib != kOutside)
    return Max(fLeft->SafetyToOut(p), fRight->SafetyToOut(fRight->T.Transform(p)));
  if (ia == kSurface || ib == kSurface) return -kTolerance;
  if (ia == kOutside) return fRight->SafetyToOut(fRight->T.Transform(p));
  return fLeft->SafetyToOut(p);
}

// source/UnplacedBooleanVolume.cpp:461-476 Extent of the union: both operands' boxes
void BooleanUnion::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  Vec3 l0, l1, r0, r1;
  TransformedExtent(fLeft, l0, l1);
  TransformedExtent(fRight, r0, r1);
  aMin = Vec3(Min(l0.x(), r0.x()), Min(l0.y(), r0.y()), Min(l0.z(), r0.z()));
  aMax = Vec3(Max(l1.x(), r1.x()), Max(l1.y(), r1.y()), Max(l1.z(), r1.z()));
}

// source/UnplacedBooleanVolume.cpp:443-458 TransformedExtent of the left operand
void BooleanMinus::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  Vec3 lower, upper;
  fLeft->Shape()->Extent(lower, upper);
  const Vec3 delta = upper - lower;
  double mn[3] = {kInfLength, kInfLength, kInfLength}, mx[3] = {-kInfLength, -kInfLength, -kInfLength};
  for (int x = 0; x <= 1; ++x)
    for (int y = 0; y <= 1; ++y)
      for (int z = 0; z <= 1; ++z) {
        Vec3 c(lower.x() + x * delta.x(), lower.y() + y * delta.y(), lower.z() + z * delta.z());
        const Vec3 t = fLeft->T.InverseTransform(c);
        for (int k = 0; k < 3; ++k) {
          mn[k] = std::min(mn[k], t[k]);
          mx[k] = std::max(mx[k], t[k]);
        }
      }
  aMin = Vec3(mn[0], mn[1], mn[2]);
  aMax = Vec3(mx[0], mx[1], mx[2]);
}

// ====================================================================== Cut tube
// Plane.h:40-49 Set(normal, origin): zero components below kTolerance, then normalise
void CutPlane::Set(Vec3 normal, Vec3 const &origin)
{
  for (int i = 0; i < 3; ++i)
    if (Abs(normal[i]) < kTolerance) normal[i] = 0.0;
  const double inv = 1. / normal.Mag();
  n                = inv * normal;
  d                = inv * -normal.Dot(origin);
}

// CutTubeStruct.h:38-49
CutTube::CutTube(double rmin, double rmax, double z, double sphi, double dphi, Vec3 bottom, Vec3 top)
    : fDz(z), fTube(rmin, rmax, kInfLength, sphi, dphi)
{
  fCut[0].Set(bottom.Unit(), Vec3(0., 0., -z));
  fCut[1].Set(top.Unit(), Vec3(0., 0., z));
  fCosPhi1 = std::cos(sphi);
  fSinPhi1 = std::sin(sphi);
  fCosPhi2 = std::cos(sphi + dphi);
  fSinPhi2 = std::sin(sphi + dphi);
  fMaxVal  = Max(rmax, z);
}

// CutPlanes.h Inside (:130-142): inside both, surface within kTolerance of either
int CutTube::CutInside(Vec3 const &p) const
{
  const double d0 = fCut[0].Dist(p), d1 = fCut[1].Dist(p);
  int inside      = (d0 < 0.0 && d1 < 0.0) ? kInside : kOutside;
  if (Abs(d0) < kTolerance || Abs(d1) < kTolerance) inside = kSurface;
  return inside;
}

// CutPlanes.h DistanceToIn (:144-156) with Plane::DistanceToIn (Plane.h:128-147): per plane
// -saf/ndd when approaching from outside the tolerance band, -kInfLength when the
// direction is along the normal; the larger of the two
double CutTube::CutDistanceToIn(Vec3 const &p, Vec3 const &dir) const
{
  double dd[2];
  for (int i = 0; i < 2; ++i) {
    double distance  = -kInfLength;
    const double ndd = NonZero(dir.Dot(fCut[i].n));
    const double saf = fCut[i].Dist(p);
    const bool valid = ndd < 0. && saf > -kTolerance;
    if (valid) distance = -saf / ndd;
    if (dir.Dot(fCut[i].n) > 0.) distance = -kInfLength;
    dd[i] = distance;
  }
  return Max(dd[0], dd[1]);
}

// CutPlanes.h DistanceToOut (:158-166) with Plane::DistanceToOut (Plane.h:149-170)
double CutTube::CutDistanceToOut(Vec3 const &p, Vec3 const &dir) const
{
  double dd[2];
  for (int i = 0; i < 2; ++i) {
    double distance  = kInfLength;
    const double ndd = NonZero(dir.Dot(fCut[i].n));
    const double saf = fCut[i].Dist(p);
    const bool valid = ndd > 0. && saf < kTolerance;
    if (saf > kTolerance) distance = -kInfLength;
    if (valid) distance = -saf / ndd;
    dd[i] = distance;
  }
  return Min(dd[0], dd[1]);
}

double CutTube::CutSafetyToIn(Vec3 const &p) const { return Max(fCut[0].Dist(p), fCut[1].Dist(p)); }
double CutTube::CutSafetyToOut(Vec3 const &p) const { return Min(-fCut[0].Dist(p), -fCut[1].Dist(p)); }

// CutTubeImplementation.h:114-126 Contains
bool CutTube::Contains(Vec3 const &p) const
{
  const bool inCut = fCut[0].Dist(p) < 0. && fCut[1].Dist(p) < 0.;
  if (!inCut) return false;
  return fTube.Contains(p) && inCut;
}

// CutTubeImplementation.h:128-142 Inside
int CutTube::Inside(Vec3 const &p) const
{
  const int ic = CutInside(p);
  if (ic == kOutside) return kOutside;
  int inside = fTube.Inside(p);
  if (ic == kOutside || (ic == kSurface && inside != kOutside)) inside = ic;
  return inside;
}

// CutTubeImplementation.h:144-169 DistanceToIn: far points are first moved to 100 x the
// largest dimension from the origin along the ray
double CutTube::DistanceToIn(Vec3 const &pointT, Vec3 const &dir, double stepMax) const
{
  Vec3 point          = pointT;
  const double ptDist = point.Mag();
  double distToMove   = 0.;
  const double order  = 100.;
  if (ptDist > order * fMaxVal) {
    distToMove = ptDist - order * fMaxVal;
    point      = point + distToMove * dir;
  }
  double distance = DistanceToInKernel(point, dir, stepMax);
  distance += distToMove;
  return distance;
}

// CutTubeImplementation.h:171-258 DistanceToInKernel (USE_CONV_WRONG_SIDE): points inside
// give -1; the ray is first moved to the cut planes when it hits them within stepMax, then
// the tube distance from there, limited by the exit from the cut planes
double CutTube::DistanceToInKernel(Vec3 const &point, Vec3 const &direction, double stepMax) const
{
  double distance = kInfLength;
  int insideCut   = CutInside(point);
  int instart     = fTube.Inside(point);
  if (insideCut == kOutside || (insideCut == kSurface && instart != kOutside)) instart = insideCut;
  if (instart == kInside) distance = -1.;
  double dplanes         = CutDistanceToIn(point, direction);
  const double safplanes = CutSafetyToIn(point);
  const bool hitplanes   = Abs(dplanes) < stepMax && safplanes > -kTolerance;
  if (insideCut != kInside && !hitplanes) return distance;
  Vec3 propagated = point;
  if (!hitplanes) dplanes = 0.;
  if (hitplanes) {
    propagated = propagated + dplanes * direction;
    insideCut  = CutInside(propagated);
  }
  bool done = insideCut == kOutside;
  done      = done || instart == kInside;
  if (done) return distance;
  instart           = fTube.Inside(propagated);
  const bool inside = hitplanes && (instart != kOutside);
  if (inside && !done) distance = dplanes;
  done = done || inside;
  if (done) {
    if (Abs(distance) < kTolerance) distance = 0.;
    return distance;
  }
  const double dexit = CutDistanceToOut(propagated, direction);
  double dtube       = fTube.DistanceToInKernel(propagated, direction);
  if (dtube < 0.) dtube = 0.;
  if (dexit < dtube) dtube = kInfLength;
  if (!done && (dtube + dplanes) < stepMax) distance = dtube + dplanes;
  return distance;
}

// CutTubeImplementation.h:262-280 DistanceToOut
double CutTube::DistanceToOut(Vec3 const &point, Vec3 const &direction, double stepMax) const
{
  double distance    = CutDistanceToOut(point, direction);
  const double dtube = fTube.DistanceToOut(point, direction, stepMax);
  if (dtube < distance) distance = dtube;
  return distance;
}

// CutTubeImplementation.h:283-298 SafetyToIn
double CutTube::SafetyToIn(Vec3 const &point) const
{
  double safety        = CutSafetyToIn(point);
  const double saftube = fTube.SafetyToIn(point);
  if (saftube > safety) safety = saftube;
  return safety;
}

// CutTubeImplementation.h:301-315 SafetyToOut
double CutTube::SafetyToOut(Vec3 const &point) const
{
  double safety        = CutSafetyToOut(point);
  const double saftube = fTube.SafetyToOut(point);
  if (saftube < safety) safety = saftube;
  return safety;
}

// source/UnplacedCutTube.cpp:128-172 Extent (ZlimitTop / ZlimitBottom, UnplacedCutTube.h:135-147)
void CutTube::Extent(Vec3 &aMin, Vec3 &aMax) const
{
  const Vec3 tn = fCut[1].n, bn = fCut[0].n;
  const double rmax = fTube.fRmax, rmin = fTube.fRmin, sphi = fTube.fSphi, dphi = fTube.fDphi, z = fDz;
  auto zTop = [&](double r, double ph) { return z - (r / tn.z()) * (tn.x() * std::cos(ph) + tn.y() * std::sin(ph)); };
  auto zBot = [&](double r, double ph) { return -z - (r / bn.z()) * (bn.x() * std::cos(ph) + bn.y() * std::sin(ph)); };
  const double dztop    = rmax * Sqrt(1. - tn.z() * tn.z()) / tn.z();
  const double dzbottom = -rmax * Sqrt(1. - bn.z() * bn.z()) / bn.z();
  aMin = Vec3(-rmax, -rmax, -z - dzbottom);
  aMax = Vec3(rmax, rmax, z + dztop);
  if (dphi == kTwoPi) return;
  Wedge const &w = fTube.fPhiWedge;
  if (!w.Contains(Vec3(-tn.x(), -tn.y(), 0.))) {
    aMax[2] = Max(zTop(rmax, sphi), zTop(rmax, sphi + dphi));
    aMax[2] = Max(aMax[2], Max(zTop(rmin, sphi), zTop(rmin, sphi + dphi)));
  }
  if (!w.Contains(Vec3(-bn.x(), -bn.y(), 0.))) {
    aMin[2] = Min(zBot(rmax, sphi), zBot(rmax, sphi + dphi));
    aMin[2] = Min(aMin[2], Min(zBot(rmin, sphi), zBot(rmin, sphi + dphi)));
  }
  if (!w.Contains(Vec3(1., 0., 0.))) {
    aMax[0] = Max(rmax * fCosPhi1, rmax * fCosPhi2);
    aMax[0] = Max(aMax[0], Max(rmin * fCosPhi1, rmin * fCosPhi2));
  }
  if (!w.Contains(Vec3(-1., 0., 0.))) {
    aMin[0] = Min(rmax * fCosPhi1, rmax * fCosPhi2);
    aMin[0] = Min(aMin[0], Min(rmin * fCosPhi1, rmin * fCosPhi2));
  }
  if (!w.Contains(Vec3(0., 1., 0.))) {
    aMax[1] = Max(rmax * fSinPhi1, rmax * fSinPhi2);
    aMax[1] = Max(aMax[1], Max(rmin * fSinPhi1, rmin * fSinPhi2));
  }
  if (!w.Contains(Vec3(0., -1., 0.))) {
    aMin[1] = Min(rmax * fSinPhi1, rmax * fSinPhi2);
    aMin[1] = Min(aMin[1], Min(rmin * fSinPhi1, rmin * fSinPhi2));
  }
}

} // namespace oracle
