// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// Torus2: cubic/quartic solvers and the kernels of VecGeom/volumes/kernel/TorusImplementation2.h.
#include "ref_shapes_more.h"
#include <cmath>

namespace oracle {
namespace {
// TorusImplementation2.h:25-61 SolveCubic
unsigned SolveCubic(double a, double b, double c, double *x)
{
  const double ott     = 1. / 3.;
  const double sq3     = Sqrt(3.);
  const double inv6sq3 = 1. / (6. * sq3);
  unsigned ireal       = 1;
  const double p       = b - a * a * ott;
  const double q       = c - a * b * ott + 2. * a * a * a * ott * ott * ott;
  double delta         = 4 * p * p * p + 27. * q * q;
  double t, u;
  if (delta >= 0) {
    delta = Sqrt(delta);
    t     = (-3 * q * sq3 + delta) * inv6sq3;
    u     = (3 * q * sq3 + delta) * inv6sq3;
    x[0]  = CopySign(1., t) * std::cbrt(Abs(t)) - CopySign(1., u) * std::cbrt(Abs(u)) - a * ott;
  } else {
    delta = Sqrt(-delta);
    t     = -0.5 * q;
    u     = delta * inv6sq3;
    x[0]  = 2. * std::pow(t * t + u * u, 0.5 * ott) * std::cos(ott * std::atan2(u, t));
    x[0] -= a * ott;
  }
  t     = x[0] * x[0] + a * x[0] + b;
  u     = a + x[0];
  delta = u * u - 4. * t;
  if (delta >= 0) {
    ireal = 3;
    delta = Sqrt(delta);
    x[1]  = 0.5 * (-u - delta);
    x[2]  = 0.5 * (-u + delta);
  }
  return ireal;
}
void CmpSwap(double *a, int i, int j)
{
  if (a[i] > a[j]) {
    const double c = a[j];
    a[j]           = a[i];
    a[i]           = c;
  }
}
// TorusImplementation2.h:73-81 Sort4
void Sort4(double *a)
{
  CmpSwap(a, 0, 2);
  CmpSwap(a, 1, 3);
  CmpSwap(a, 0, 1);
  CmpSwap(a, 2, 3);
  CmpSwap(a, 1, 2);
}
// TorusImplementation2.h:84-150 SolveQuartic
int SolveQuartic(double a, double b, double c, double d, double *x)
{
  const double e = b - 3. * a * a / 8.;
  const double f = c + a * a * a / 8. - 0.5 * a * b;
  const double g = d - 3. * a * a * a * a / 256. + a * a * b / 16. - a * c / 4.;
  double xx[4]   = {kInfLength, kInfLength, kInfLength, kInfLength};
  double delta;
  double h       = 0.;
  unsigned ireal = 0;
  if (Abs(f) < 1E-6) {
    delta = e * e - 4. * g;
    if (delta < 0.) return 0;
    delta = Sqrt(delta);
    h     = 0.5 * (-e - delta);
    if (h >= 0) {
      h          = Sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    h = 0.5 * (-e + delta);
    if (h >= 0) {
      h          = Sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    Sort4(x);
    return ireal;
  }
  if (Abs(g) < 1E-6) {
    x[ireal++]        = -0.25 * a;
    const unsigned nc = SolveCubic(0, e, f, xx);
    for (unsigned i = 0; i < nc; i++) x[ireal++] = xx[i] - 0.25 * a;
    Sort4(x);
    return ireal;
  }
  ireal = SolveCubic(2. * e, e * e - 4. * g, -f * f, xx);
  if (ireal == 1) {
    if (xx[0] <= 0) return 0;
    h = Sqrt(xx[0]);
  } else {
    for (unsigned i = 0; i < 3; i++) {
      h = xx[i];
      if (h >= 0) break;
    }
    if (h <= 0) return 0;
    h = Sqrt(h);
  }
  const double j = 0.5 * (e + h * h - f / h);
  ireal          = 0;
  delta          = h * h - 4. * j;
  if (delta >= 0) {
    delta      = Sqrt(delta);
    x[ireal++] = 0.5 * (-h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (-h + delta) - 0.25 * a;
  }
  delta = h * h - 4. * g / j;
  if (delta >= 0) {
    delta      = Sqrt(delta);
    x[ireal++] = 0.5 * (h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (h + delta) - 0.25 * a;
  }
  Sort4(x);
  return ireal;
}
} // namespace

// TorusStruct2.h:36-43 and UnplacedTorus2.h:64-74 (bounding tube)
Torus2::Torus2(double rmin, double rmax, double rtor, double sphi, double dphi)
    : fRmin(rmin), fRmax(rmax), fRtor(rtor), fSphi(sphi), fDphi(dphi), fRmin2(rmin * rmin), fRmax2(rmax * rmax),
      fRtor2(rtor * rtor), fPhiWedge(dphi, sphi),
      fBoundingTube(rtor - rmax - kTolerance, rtor + rmax + kTolerance, rmax, sphi, dphi)
{
}

// TorusImplementation2.h:252-290 GenericKernelForContainsAndInside
void Torus2::ContainsAndInside(Vec3 const &p, bool forInside, bool notForDisk, bool &cin, bool &cout) const
{
  const double tol   = 100. * kTolerance;
  const double rxy   = Sqrt(p[0] * p[0] + p[1] * p[1]);
  const double radsq = (rxy - fRtor) * (rxy - fRtor) + p[2] * p[2];
  if (forInside) {
    cout = radsq > (tol * fRmax + fRmax2);
    cin  = radsq < (-tol * fRmax + fRmax2);
  } else {
    cout = radsq > fRmax2;
  }
  if (cout) return;
  if (forInside) {
    cout = cout || (radsq < (-tol * fRmin + fRmin2));
    cin  = cin && (radsq > (tol * fRmin + fRmin2));
  } else {
    cout = cout || (radsq < fRmin2);
  }
  if (cout) return;
  if ((fDphi < kTwoPi) && notForDisk) {
    bool ci = false, co = false;
    fPhiWedge.ContainsAndInside(p, forInside, ci, co);
    cout = cout || co;
    if (forInside) cin = cin && ci;
  }
}

int Torus2::Inside(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, true, cin, cout);
  int r = kSurface;
  if (cout) r = kOutside;
  if (cin) r = kInside;
  return r;
}
// TorusImplementation2.h:411-420: Contains takes the tolerant kernel without the phi test.
bool Torus2::Contains(Vec3 const &p) const
{
  bool cin = false, cout = false;
  ContainsAndInside(p, true, false, cin, cout);
  return !cout;
}

double Torus2::DistSqrToTorusR(Vec3 const &point, Vec3 const &dir, double dist) const
{
  const Vec3 p      = point + dir * dist;
  const double rxy  = p.Perp();
  return (rxy - fRtor) * (rxy - fRtor) + p.z() * p.z();
}

// TorusImplementation2.h:292-389 ToBoundary (quartic, root filter, Newton polish <= 100 iterations)
double Torus2::ToBoundary(Vec3 const &pt, Vec3 const &dir, double radius, bool out) const
{
  double s            = kInfLength;
  const double tol    = 100. * kTolerance;
  const double r0sq   = pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2];
  const double rdotn  = pt[0] * dir[0] + pt[1] * dir[1] + pt[2] * dir[2];
  const double rsumsq = fRtor2 + radius * radius;
  const double a      = 4. * rdotn;
  const double b      = 2. * (r0sq + 2. * rdotn * rdotn - rsumsq + 2. * fRtor2 * dir[2] * dir[2]);
  const double c      = 4. * (r0sq * rdotn - rsumsq * rdotn + 2. * fRtor2 * pt[2] * dir[2]);
  const double d      = r0sq * r0sq - 2. * r0sq * rsumsq + 4. * fRtor2 * pt[2] * pt[2] +
                   (fRtor2 - radius * radius) * (fRtor2 - radius * radius);
  double x[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  int nsol    = 0;
  if (Abs(dir[2]) < 1E-3 && Abs(pt[2]) < 0.1 * radius) {
    double r0              = fRtor - Sqrt((radius - pt[2]) * (radius + pt[2]));
    const double invdirxy2 = 1. / (1 - dir.z() * dir.z());
    const double b0        = (pt[0] * dir[0] + pt[1] * dir[1]) * invdirxy2;
    double c0              = (pt[0] * pt[0] + (pt[1] - r0) * (pt[1] + r0)) * invdirxy2;
    double delta           = b0 * b0 - c0;
    if (delta > 0) {
      x[nsol] = -b0 - Sqrt(delta);
      if (x[nsol] > -tol) nsol++;
      x[nsol] = -b0 + Sqrt(delta);
      if (x[nsol] > -tol) nsol++;
    }
    r0    = fRtor + Sqrt((radius - pt[2]) * (radius + pt[2]));
    c0    = (pt[0] * pt[0] + (pt[1] - r0) * (pt[1] + r0)) * invdirxy2;
    delta = b0 * b0 - c0;
    if (delta > 0) {
      x[nsol] = -b0 - Sqrt(delta);
      if (x[nsol] > -tol) nsol++;
      x[nsol] = -b0 + Sqrt(delta);
      if (x[nsol] > -tol) nsol++;
    }
    if (nsol) Sort4(x);
  } else {
    nsol = SolveQuartic(a, b, c, d, x);
  }
  if (!nsol) return kInfLength;
  const bool inner = Abs(radius - fRmin) < kTolerance;
  for (int i = 0; i < nsol; i++) {
    if (x[i] < -10) continue;
    Vec3 r0   = pt + x[i] * dir;
    Vec3 norm = r0;
    r0[2]     = 0.;
    const double inv = 1. / r0.Mag();
    r0               = r0 * inv;
    r0               = r0 * fRtor;
    norm             = norm - r0;
    const double ndotd = norm.Dot(dir);
    if (inner ^ out) {
      if (ndotd < 0) continue;
    } else {
      if (ndotd > 0) continue;
    }
    if (fDphi < kTwoPi) {
      bool ci = false, co = false;
      fPhiWedge.ContainsAndInside(r0, true, ci, co);
      if (co) continue;
    }
    s            = x[i];
    double eps   = kInfLength;
    double delta = s * s * s * s + a * s * s * s + b * s * s + c * s + d;
    double eps0  = -delta / (4. * s * s * s + 3. * a * s * s + 2. * b * s + c);
    int ntry     = 0;
    while (Abs(eps) > kTolerance) {
      if (Abs(eps0) > 100) break;
      s += eps0;
      if (Abs(s + eps0) < kTolerance) break;
      delta = s * s * s * s + a * s * s * s + b * s * s + c * s + d;
      eps   = -delta / (4. * s * s * s + 3. * a * s * s + 2. * b * s + c);
      if (Abs(eps) >= Abs(eps0)) break;
      ntry++;
      if (ntry > 100) break;
      eps0 = eps;
    }
    if (s < -tol) continue;
    return Max(0., s);
  }
  return kInfLength;
}

// TorusImplementation2.h:140-222 DistanceToOut
double Torus2::DistanceToOut(Vec3 const &point, Vec3 const &dir, double) const
{
  const bool hasphi  = fDphi < kTwoPi;
  const bool hasrmin = fRmin > 0;
  bool done          = false;
  double distance    = kInfLength;
  const double distz = Abs(point.z()) - fRmax;
  done               = done || (distz > kHalfTolerance);
  const double rsq   = point.x() * point.x() + point.y() * point.y();
  const double outerExcl = fRtor + fRmax + kHalfTolerance;
  done                   = done || (rsq > outerExcl * outerExcl);
  const double innerExcl = fRtor - fRmax - kHalfTolerance;
  done                   = done || (rsq < innerExcl * innerExcl);
  if (done) return -1.;
  if (Inside(point) == kOutside) return -1.;
  const double dout = ToBoundary(point, dir, fRmax, true);
  double din        = kInfLength;
  if (hasrmin) din = ToBoundary(point, dir, fRmin, true);
  distance = Min(dout, din);
  if (hasphi) {
    // Wedge::DistanceToOut (Wedge_Evolution.h:399-428)
    const double comp1 = dir.x() * fPhiWedge.normal1.x() + dir.y() * fPhiWedge.normal1.y();
    const double comp2 = dir.x() * fPhiWedge.normal2.x() + dir.y() * fPhiWedge.normal2.y();
    double distPhi1 = kInfLength, distPhi2 = kInfLength;
    if (comp1 < 0.) {
      const double t = -(point.x() * fPhiWedge.normal1.x() + point.y() * fPhiWedge.normal1.y()) / comp1;
      if (t > 0.) distPhi1 = t;
    }
    if (comp2 < 0.) {
      const double t = -(point.x() * fPhiWedge.normal2.x() + point.y() * fPhiWedge.normal2.y()) / comp2;
      if (t > 0.) distPhi2 = t;
    }
    if (distPhi1 < distance) {
      const Vec3 ip = point + dir * distPhi1;
      bool ci = false, co = false;
      ContainsAndInside(ip, false, false, ci, co);
      if (!co) {
        const double diri = ip.x() * fPhiWedge.along1.x() + ip.y() * fPhiWedge.along1.y();
        if (diri >= 0) distance = distPhi1;
      }
    }
    if (distPhi2 < distance) {
      const Vec3 ip = point + dir * distPhi2;
      bool ci = false, co = false;
      ContainsAndInside(ip, false, false, ci, co);
      if (!co) {
        const double diri2 = ip.x() * fPhiWedge.along2.x() + ip.y() * fPhiWedge.along2.y();
        if (diri2 >= 0 && distPhi2 < distance) distance = distPhi2;
      }
    }
  }
  if (done || distance >= kInfLength) distance = -1.;
  return distance;
}

// TorusImplementation2.h:421-488 DistanceToIn (VECGEOM_NO_SPECIALIZATION branch)
double Torus2::DistanceToIn(Vec3 const &point, Vec3 const &dir, double smax) const
{
  Vec3 localPoint     = point;
  double distance     = kInfLength;
  bool done           = false;
  double tubeDistance = kInfLength;
  const bool inBounds = fBoundingTube.Contains(localPoint);
  if (!inBounds)
    tubeDistance = fBoundingTube.DistanceToIn(localPoint, dir, smax);
  else
    tubeDistance = 0.;
  if (inBounds) {
    if (Inside(point) == kInside) {
      done     = true;
      distance = -1.;
    }
  } else {
    done = tubeDistance == kInfLength;
  }
  if (done) return distance;
  localPoint = localPoint + tubeDistance * dir;
  if (fDphi < kTwoPi) {
    // Wedge::DistanceToIn (Wedge_Evolution.h:383-397)
    double d1 = kInfLength, d2 = kInfLength;
    const double comp1 = dir.x() * fPhiWedge.normal1.x() + dir.y() * fPhiWedge.normal1.y();
    const double comp2 = dir.x() * fPhiWedge.normal2.x() + dir.y() * fPhiWedge.normal2.y();
    if (comp1 > 0.) {
      const double t = -(localPoint.x() * fPhiWedge.normal1.x() + localPoint.y() * fPhiWedge.normal1.y()) / comp1;
      if (t > 0.) d1 = t;
    }
    if (comp2 > 0.) {
      const double t = -(localPoint.x() * fPhiWedge.normal2.x() + localPoint.y() * fPhiWedge.normal2.y()) / comp2;
      if (t > 0.) d2 = t;
    }
    if (d1 != kInfLength) {
      const double daxis = DistSqrToTorusR(localPoint, dir, d1);
      if (daxis >= fRmin2 && daxis < fRmax2) {
        distance = d1;
        if (Abs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    if (d2 != kInfLength) {
      const double daxis = DistSqrToTorusR(localPoint, dir, d2);
      if (daxis >= fRmin2 && daxis < fRmax2) {
        distance = Min(d2, distance);
        if (Abs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    distance = kInfLength;
  }
  double dd = ToBoundary(localPoint, dir, fRmax, false);
  if (fRmin > 0.) dd = Min(dd, ToBoundary(localPoint, dir, fRmin, false));
  distance = Min(distance, dd);
  distance += tubeDistance;
  if (Abs(distance) > kInfLength) distance = kInfLength;
  return distance;
}

// TorusImplementation2.h:391-409 SafetyToOut, :489-510 SafetyToIn
double Torus2::SafetyToOut(Vec3 const &p) const
{
  const double rxy = Sqrt(p[0] * p[0] + p[1] * p[1]);
  const double rad = Sqrt((rxy - fRtor) * (rxy - fRtor) + p[2] * p[2]);
  double safety    = fRmax - rad;
  if (fRmin) safety = Min(rad - fRmin, fRmax - rad);
  if (fDphi < kTwoPi) safety = Min(fPhiWedge.SafetyToOut(p), safety);
  return safety;
}
double Torus2::SafetyToIn(Vec3 const &p) const
{
  const double rxy = Sqrt(p[0] * p[0] + p[1] * p[1]);
  const double rad = Sqrt((rxy - fRtor) * (rxy - fRtor) + p[2] * p[2]);
  double safety    = rad - fRmax;
  if (fRmin) safety = Max(fRmin - rad, rad - fRmax);
  if (fDphi < kTwoPi && rxy != 0.) safety = Max(fPhiWedge.SafetyToIn(p), safety);
  return safety;
}

} // namespace oracle
