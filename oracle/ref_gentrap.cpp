// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// The generic trapezoid (GenTrap): VecGeom/volumes/GenTrapStruct.h,
// VecGeom/volumes/SecondOrderSurfaceShell.h and the generic kernels of
// VecGeom/volumes/kernel/GenTrapImplementation.h, restated in scalar form.
#include "ref_shapes_more.h"

namespace oracle {

namespace {
Vec3 Cross(Vec3 const &l, Vec3 const &r) // Vector3D.h:230-234
{
  return Vec3(l[1] * r[2] - l[2] * r[1], l[2] * r[0] - l[0] * r[2], l[0] * r[1] - l[1] * r[0]);
}
void Normalize(Vec3 &v) // Vector3D.h:198
{
  const double s = 1. / v.Mag();
  v              = Vec3(v[0] * s, v[1] * s, v[2] * s);
}
// GenTrapStruct.h SegmentsCrossing
bool SegmentsCrossing(Vec3 p, Vec3 p1, Vec3 q, Vec3 q1)
{
  const Vec3 r = p1 - p, s = q1 - q;
  const Vec3 rxs = Cross(r, s);
  if (rxs.Mag2() < kTolerance) return false;
  const double t = Cross(q - p, s).z() / rxs.z();
  if (t < kTolerance || t > 1. - kTolerance) return false;
  const double u = Cross(q - p, r).z() / rxs.z();
  if (u < kTolerance || u > 1. - kTolerance) return false;
  return true;
}
} // namespace

// GenTrapStruct::Initialize: orientation (the signed areas of both quadrilaterals), the
// switch to clockwise order, crossing opposite segments and convexity.
bool GenTrap::Initialize(double *vx, double *vy, double dz, const char **err)
{
  if (!(dz > 0.)) { // SecondOrderSurfaceShell::Initialize throws
    *err = "Half-length of generic trapezoid must be positive";
    return false;
  }
  Vec3 v[8];
  for (int i = 0; i < 8; ++i) v[i] = Vec3(vx[i], vy[i], i < 4 ? -dz : dz);
  double sum1 = 0., sum2 = 0.;
  for (int i = 0; i < 4; ++i) {
    const int j = (i + 1) % 4;
    sum1 += v[i].x() * v[j].y() - v[j].x() * v[i].y();
    sum2 += v[i + 4].x() * v[j + 4].y() - v[j + 4].x() * v[i + 4].y();
  }
  if (sum1 * sum2 < -kTolerance) {
    *err = "generic trap defined with opposite clockwise";
    return false;
  }
  if (sum1 > kTolerance) {
    Vec3 t = v[1];
    v[1]   = v[3];
    v[3]   = t;
    t      = v[5];
    v[5]   = v[7];
    v[7]   = t;
  }
  double dX[8], dY[8];
  for (int i = 0; i < 4; ++i) {
    const int j = (i + 1) % 4;
    dX[i]       = v[j].x() - v[i].x();
    dX[i + 4]   = v[j + 4].x() - v[i + 4].x();
    dY[i]       = v[j].y() - v[i].y();
    dY[i + 4]   = v[j + 4].y() - v[i + 4].y();
  }
  if (SegmentsCrossing(v[0], v[1], v[3], v[2]) || SegmentsCrossing(v[1], v[2], v[0], v[3]) ||
      SegmentsCrossing(v[4], v[5], v[7], v[6]) || SegmentsCrossing(v[5], v[6], v[4], v[7])) {
    *err = "generic trap defined with crossing opposite segments";
    return false;
  }
  for (int i = 0; i < 4; ++i) { // ComputeIsConvexQuadrilaterals
    const int j = (i + 1) % 4;
    if (dX[i] * dY[j] - dY[i] * dX[j] > kTolerance || dX[i + 4] * dY[j + 4] - dY[i + 4] * dX[j + 4] > kTolerance) {
      *err = "generic trap defined with top/bottom quadrilaterals not convex";
      return false;
    }
  }
  for (int i = 0; i < 8; ++i) vx[i] = v[i].x(), vy[i] = v[i].y();
  return true;
}

GenTrap::GenTrap(const double *vxin, const double *vyin, double dz)
{
  double vx[8], vy[8];
  for (int i = 0; i < 8; ++i) vx[i] = vxin[i], vy[i] = vyin[i];
  const char *err = nullptr;
  valid           = Initialize(vx, vy, dz, &err);
  // the device object: Initialize again on the (clockwise) host vertices
  fDz            = dz;
  fInverseDz     = 1. / dz;
  fHalfInverseDz = 0.5 / dz;
  for (int i = 0; i < 8; ++i) fVerticesX[i] = vx[i], fVerticesY[i] = vy[i];
  InitShell();
  for (int i = 0; i < 4; ++i) {
    const int j     = (i + 1) % 4;
    fDegenerated[i] = (Abs(vx[i] - vx[j]) < kTolerance) && (Abs(vy[i] - vy[j]) < kTolerance) &&
                      (Abs(vx[i + 4] - vx[j + 4]) < kTolerance) && (Abs(vy[i + 4] - vy[j + 4]) < kTolerance);
    fConnX[i]       = vx[i] - vx[i + 4];
    fConnY[i]       = vy[i] - vy[i + 4];
    fDeltaX[i]      = vx[j] - vx[i];
    fDeltaX[i + 4]  = vx[j + 4] - vx[i + 4];
    fDeltaY[i]      = vy[j] - vy[i];
    fDeltaY[i + 4]  = vy[j + 4] - vy[i + 4];
  }
  // ComputeIsTwisted
  fIsTwisted = false;
  for (int i = 0; i < 4; ++i) {
    const double dx1 = vx[(i + 1) % 4] - vx[i], dy1 = vy[(i + 1) % 4] - vy[i];
    if (dx1 == 0 && dy1 == 0) continue;
    const double dx2 = vx[4 + (i + 1) % 4] - vx[4 + i], dy2 = vy[4 + (i + 1) % 4] - vy[4 + i];
    if (dx2 == 0 && dy2 == 0) continue;
    if (std::fabs(dy1 * dx2 - dx1 * dy2) < kTolerance) continue;
    fIsTwisted = true;
  }
  // ComputeBoundingBox
  Vec3 lo, hi;
  Extent(lo, hi);
  for (int k = 0; k < 3; ++k) {
    fBBorig[k] = 0.5 * (lo[k] + hi[k]);
    fBBdim[k]  = 0.5 * (hi[k] - lo[k]);
  }
}

// SecondOrderSurfaceShell::Initialize
void GenTrap::InitShell()
{
  const double dz = fDz;
  fDz2            = 0.5 / dz;
  const double *vx = fVerticesX, *vy = fVerticesY;
  for (int i = 0; i < 4; ++i) {
    const int j = (i + 1) % 4;
    const Vec3 va(vx[i], vy[i], -dz), vb(vx[i + 4], vy[i + 4], dz), vc(vx[j], vy[j], -dz), vd(vx[j + 4], vy[j + 4], dz);
    fxa[i] = vx[i], fya[i] = vy[i], fxb[i] = vx[i + 4], fyb[i] = vy[i + 4];
    fxc[i] = vx[j], fyc[i] = vy[j], fxd[i] = vx[4 + j], fyd[i] = vy[4 + j];
    fdegen[i] = (Abs(fxa[i] - fxc[i]) < kTolerance) && (Abs(fya[i] - fyc[i]) < kTolerance) &&
                (Abs(fxb[i] - fxd[i]) < kTolerance) && (Abs(fyb[i] - fyd[i]) < kTolerance);
    ftx1[i]       = fDz2 * (fxb[i] - fxa[i]);
    fty1[i]       = fDz2 * (fyb[i] - fya[i]);
    ftx2[i]       = fDz2 * (fxd[i] - fxc[i]);
    fty2[i]       = fDz2 * (fyd[i] - fyc[i]);
    ft1crosst2[i] = ftx1[i] * fty2[i] - ftx2[i] * fty1[i];
    fDeltatx[i]   = ftx2[i] - ftx1[i];
    fDeltaty[i]   = fty2[i] - fty1[i];
    fNormals[i]   = Cross(vb - va, vc - va);
    if (fNormals[i].Mag2() < kTolerance) {
      fNormals[i] = Cross(vb - va, vd - vb);
      if (fNormals[i].Mag2() < kTolerance) fNormals[i] = Vec3(0., 0., 1.);
    }
    Normalize(fNormals[i]);
    fViCrossHi0[i]  = Cross(vb - va, vc - va);
    fViCrossVj[i]   = Cross(vb - va, vd - vc);
    fHi1CrossHi0[i] = Cross(vd - vb, vc - va);
  }
  fisplanar = true;
  for (int i = 0; i < 4; ++i) {
    fiscurved[i] = !(((Abs(fxc[i] - fxa[i]) < kTolerance) && (Abs(fyc[i] - fya[i]) < kTolerance)) ||
                     ((Abs(fxd[i] - fxb[i]) < kTolerance) && (Abs(fyd[i] - fyb[i]) < kTolerance)) ||
                     (Abs((fxc[i] - fxa[i]) * (fyd[i] - fyb[i]) - (fxd[i] - fxb[i]) * (fyc[i] - fya[i])) < kTolerance));
    if (fiscurved[i]) fisplanar = false;
  }
}

// GenTrapStruct::Extent
void GenTrap::Extent(Vec3 &lo, Vec3 &hi) const
{
  lo = hi = Vec3(fVerticesX[0], fVerticesY[0], 0.);
  lo[2]   = -fDz;
  hi[2]   = fDz;
  for (int i = 0; i < 4; ++i) {
    for (int k : {i, i + 4}) {
      if (lo[0] > fVerticesX[k]) lo[0] = fVerticesX[k];
      if (hi[0] < fVerticesX[k]) hi[0] = fVerticesX[k];
      if (lo[1] > fVerticesY[k]) lo[1] = fVerticesY[k];
      if (hi[1] < fVerticesY[k]) hi[1] = fVerticesY[k];
    }
  }
}

// ------------------------------------------------------------ SecondOrderSurfaceShell
// CheckInside: the point against the section of the lateral surfaces at its z
void GenTrap::CheckInside(Vec3 const &p, bool &cin, bool &cout, bool &onsurf) const
{
  const double tolerancesq = 10000. * kTolerance * kTolerance;
  onsurf                   = false;
  cin                      = Abs(p.z()) < MakeMinusTolerant<true>(fDz);
  cout                     = Abs(p.z()) > MakePlusTolerant<true>(fDz);
  if (cout) return;
  double vX[4], vY[4];
  const double dzp = fDz + p[2];
  for (int i = 0; i < 4; ++i) {
    vX[i] = fxa[i] + ftx1[i] * dzp;
    vY[i] = fya[i] + fty1[i] * dzp;
  }
  bool degenerated = true;
  for (int i = 0; i < 4; ++i) {
    const int j            = (i + 1) % 4;
    const double DeltaX    = vX[j] - vX[i];
    const double DeltaY    = vY[j] - vY[i];
    const double deltasq   = DeltaX * DeltaX + DeltaY * DeltaY;
    const bool samevertex  = deltasq < MakePlusTolerant<true>(0.);
    degenerated            = degenerated && samevertex;
    const double cross     = (p.x() - vX[i]) * DeltaY - (p.y() - vY[i]) * DeltaX;
    const bool onsurfi     = (cross * cross < tolerancesq * deltasq) && (!samevertex);
    cout                   = cout || ((cross < MakeMinusTolerant<true>(0.)) && (!onsurfi));
    cin                    = cin && (samevertex || ((cross > MakePlusTolerant<true>(0.)) && (!onsurfi)));
  }
  onsurf = (!cout) && (!cin);
  cout   = cout || degenerated;
}

// InSurfLimits: the point's vertical and horizontal ratios on surface i lie in [0, 1]
bool GenTrap::InSurfLimits(Vec3 const &p, int i) const
{
  const double rz = fDz2 * (p.z() + fDz);
  bool insurf     = (rz > MakeMinusTolerant<true>(0.)) && (rz < MakePlusTolerant<true>(1.));
  if (!insurf) return false;
  double r     = kInfLength;
  double num   = (p.x() - fxa[i]) - rz * (fxb[i] - fxa[i]);
  double denom = (fxc[i] - fxa[i]) + rz * (fxd[i] - fxc[i] - fxb[i] + fxa[i]);
  if (Abs(denom) > 1.e-6) r = num / NonZero(denom);
  num   = (p.y() - fya[i]) - rz * (fyb[i] - fya[i]);
  denom = (fyc[i] - fya[i]) + rz * (fyd[i] - fyc[i] - fyb[i] + fya[i]);
  if (Abs(denom) > 1.e-6) r = num / NonZero(denom);
  return insurf && (r > MakeMinusTolerant<true>(0.)) && (r < MakePlusTolerant<true>(1.));
}

// UNormal: un-normalised outward normal of surface i at the point, with the ratios rz, r
// (r keeps its previous value when both denominators are small)
void GenTrap::UNormal(Vec3 const &p, int i, Vec3 &unorm, double &rz, double &r) const
{
  rz           = fDz2 * (p.z() + fDz);
  double num   = (p.x() - fxa[i]) - rz * (fxb[i] - fxa[i]);
  double denom = (fxc[i] - fxa[i]) + rz * (fxd[i] - fxc[i] - fxb[i] + fxa[i]);
  if (Abs(denom) > 1.e-6) r = num / NonZero(denom);
  num   = (p.y() - fya[i]) - rz * (fyb[i] - fya[i]);
  denom = (fyc[i] - fya[i]) + rz * (fyd[i] - fyc[i] - fyb[i] + fya[i]);
  if (Abs(denom) > 1.e-6) r = num / NonZero(denom);
  unorm = fViCrossHi0[i] + rz * fViCrossVj[i] + r * fHi1CrossHi0[i];
}

// ComputeSminSmax: the two roots of the second-order crossing equation per surface; planar
// surfaces take the plane crossing
void GenTrap::ComputeSminSmax(Vec3 const &p, Vec3 const &d, double smin[4], double smax[4]) const
{
  const double big = kInfLength;
  const double dzp = fDz + p[2];
  double a[4], b[4], c[4], dd[4], signa[4], inva[4];
  for (int i = 0; i < 4; ++i) {
    const double xs1 = fxa[i] + ftx1[i] * dzp;
    const double ys1 = fya[i] + fty1[i] * dzp;
    const double xs2 = fxc[i] + ftx2[i] * dzp;
    const double ys2 = fyc[i] + fty2[i] * dzp;
    const double dxs = xs2 - xs1;
    const double dys = ys2 - ys1;
    a[i]             = (fDeltatx[i] * d[1] - fDeltaty[i] * d[0] + ft1crosst2[i] * d[2]) * d[2];
    b[i]             = dxs * d[1] - dys * d[0] +
           (fDeltatx[i] * p[1] - fDeltaty[i] * p[0] + fty2[i] * xs1 - fty1[i] * xs2 + ftx1[i] * ys2 - ftx2[i] * ys1) *
               d[2];
    c[i]  = dxs * p[1] - dys * p[0] + xs1 * ys2 - xs2 * ys1;
    dd[i] = b[i] * b[i] - 4 * a[i] * c[i];
  }
  for (int i = 0; i < 4; ++i) {
    signa[i] = 0.;
    if (a[i] < -kTolerance) signa[i] = -1.;
    if (a[i] > kTolerance) signa[i] = 1.;
    inva[i] = c[i] / NonZero(b[i] * b[i]);
    if (Abs(a[i]) > kTolerance) inva[i] = 1. / NonZero(2. * a[i]);
  }
  for (int i = 0; i < 4; ++i) {
    double sqrtd = signa[i] * Sqrt(Abs(dd[i]));
    if (dd[i] < 0.) sqrtd = big;
    smin[i] = (-b[i] - sqrtd) * inva[i];
    smax[i] = (-b[i] + sqrtd) * inva[i];
  }
  for (int i = 0; i < 4; ++i) {
    if (fiscurved[i]) continue;
    const Vec3 pa(fxa[i], fya[i], -fDz);
    const Vec3 vecAP        = p - pa;
    const double dotAPNorm  = vecAP.Dot(fNormals[i]);
    const double dotDirNorm = d.Dot(fNormals[i]);
    smin[i]                 = -dotAPNorm / NonZero(dotDirNorm);
    smax[i]                 = kInfLength;
  }
}

double GenTrap::ShellDistanceToOut(Vec3 const &p, Vec3 const &d) const
{
  if (fisplanar) return ShellDistanceToOutPlanar(p, d);
  const double tolerance = 100. * kTolerance;
  double dist            = kInfLength;
  double smin[4], smax[4];
  Vec3 unorm;
  double r = -1.0, rz;
  bool cin, cout, onsurf;
  CheckInside(p, cin, cout, onsurf);
  if (cout) return -1.0;
  ComputeSminSmax(p, d, smin, smax);
  for (int i = 0; i < 4; ++i) {
    const bool crtbound = (Abs(smin[i]) < tolerance || Abs(smax[i]) < tolerance);
    if (crtbound) {
      if (fiscurved[i])
        UNormal(p, i, unorm, rz, r);
      else
        unorm = fNormals[i];
    }
    if (Abs(smin[i]) < tolerance && d.Dot(unorm) < 0) smin[i] = kInfLength;
    if (Abs(smax[i]) < tolerance && d.Dot(unorm) < 0) smax[i] = kInfLength;
    if ((smin[i] > -tolerance) && (smin[i] < dist)) dist = Max(smin[i], 0.);
    if ((smax[i] > -tolerance) && (smax[i] < dist)) dist = Max(smax[i], 0.);
  }
  if (dist < tolerance && onsurf) dist = 0.;
  return dist;
}

double GenTrap::ShellDistanceToOutPlanar(Vec3 const &p, Vec3 const &d) const
{
  double distance = kInfLength;
  bool outside    = Abs(p.z()) > MakePlusTolerant<true>(fDz);
  for (int i = 0; i < 4 && !outside; ++i) {
    if (fdegen[i]) continue;
    const Vec3 pa(fxa[i], fya[i], -fDz);
    const Vec3 vecAP        = p - pa;
    const double dotAPNorm  = vecAP.Dot(fNormals[i]);
    const bool otherside    = dotAPNorm > 10. * kTolerance;
    const double dotDirNorm = d.Dot(fNormals[i]);
    const bool outgoing     = dotDirNorm > 0.;
    outside                 = outside || otherside;
    const bool valid        = outgoing && !otherside;
    if (!valid) continue;
    const double snext = -dotAPNorm / NonZero(dotDirNorm);
    if (snext < distance) distance = Max(snext, 0.);
  }
  if (distance < kTolerance) distance = 0.;
  if (outside) distance = -1.;
  return distance;
}

double GenTrap::ShellDistanceToInPlanar(Vec3 const &p, Vec3 const &d, bool done) const
{
  double distance = kInfLength;
  bool inside     = Abs(p.z()) < MakeMinusTolerant<true>(fDz);
  for (int i = 0; i < 4; ++i) {
    if (fdegen[i]) continue;
    const Vec3 pa(fxa[i], fya[i], -fDz);
    const Vec3 vecAP        = p - pa;
    const double dotAPNorm  = vecAP.Dot(fNormals[i]);
    const bool otherside    = dotAPNorm < -10. * kTolerance;
    const double dotDirNorm = d.Dot(fNormals[i]);
    const bool ingoing      = dotDirNorm < 0.;
    inside                  = inside && otherside;
    bool valid              = ingoing && !otherside;
    if (!valid) continue;
    const double snext = -dotAPNorm / NonZero(dotDirNorm);
    const Vec3 psurf   = p + snext * d;
    valid              = valid && InSurfLimits(psurf, i);
    if (!done && valid && snext < distance) distance = Max(snext, 0.);
  }
  if (!done && distance < kTolerance) distance = 0.;
  if (!done && inside) distance = -1.;
  return distance;
}

double GenTrap::ShellDistanceToIn(Vec3 const &p, Vec3 const &d, bool done) const
{
  if (fisplanar) return ShellDistanceToInPlanar(p, d, done);
  double distance        = kInfLength;
  const double tolerance = 100. * kTolerance;
  Vec3 unorm;
  double r = -1.0, rz;
  bool cin, cout, onsurf;
  CheckInside(p, cin, cout, onsurf);
  if (cin && !done) distance = -1.0;
  const bool checked = cin || done;
  if (checked) return distance;
  double smin[4], smax[4];
  ComputeSminSmax(p, d, smin, smax);
  for (int i = 0; i < 4; ++i) {
    double crtdist = smin[i];
    Vec3 hit       = p + crtdist * d;
    bool crossing  = (crtdist > -tolerance) && (Abs(hit.z()) < fDz + kTolerance);
    if (crossing) {
      UNormal(hit, i, unorm, rz, r);
      crossing = crossing && d.Dot(unorm) < 0.;
      crossing = crossing && (r >= 0.) && (r <= 1.);
      if (crossing && crtdist < distance) distance = Max(crtdist, 0.);
    }
    if (!crossing) {
      crtdist  = smax[i];
      hit      = p + crtdist * d;
      crossing = (crtdist > -tolerance) && (Abs(hit.z()) < fDz + kTolerance);
      if (!crossing) continue;
      if (fiscurved[i])
        UNormal(hit, i, unorm, rz, r);
      else
        unorm = fNormals[i];
      crossing = crossing && (d.Dot(unorm) < 0.);
      crossing = crossing && (r >= 0.) && (r <= 1.);
      if (crossing && crtdist < distance) distance = Max(crtdist, 0.);
    }
  }
  if (distance < tolerance && onsurf) distance = 0.;
  return distance;
}

double GenTrap::SafetyCurved(Vec3 const &p, bool in) const
{
  double safety = kInfLength, safplanar = kInfLength;
  double dx, dy, dpx, dpy, lsq, u;
  double dx1 = 0., dx2 = 0., dy1 = 0., dy2 = 0.;
  bool cin, cout, onsurf;
  CheckInside(p, cin, cout, onsurf);
  if (onsurf) return 0.;
  bool wrong = in && cout;
  wrong      = wrong || (!in && cin);
  if (wrong) return -1.;
  double vX[4], vY[4];
  const double dzp = fDz + p[2];
  for (int i = 0; i < 4; ++i) {
    vX[i] = fxa[i] + ftx1[i] * dzp;
    vY[i] = fya[i] + fty1[i] * dzp;
  }
  double umin = 0.;
  for (int i = 0; i < 4; ++i) {
    if (!fiscurved[i]) {
      const Vec3 pa(fxa[i], fya[i], -fDz);
      const double sface = Abs((p - pa).Dot(fNormals[i]));
      if (sface < safplanar) safplanar = sface;
      continue;
    }
    const int j = (i + 1) % 4;
    dx          = vX[j] - vX[i];
    dy          = vY[j] - vY[i];
    dpx         = p[0] - vX[i];
    dpy         = p[1] - vY[i];
    lsq         = dx * dx + dy * dy;
    u           = (dpx * dx + dpy * dy) / NonZero(lsq);
    if (u > 1) {
      dpx = p[0] - vX[j];
      dpy = p[1] - vY[j];
    }
    if (u >= 0 && u <= 1) {
      dpx = dpx - u * dx;
      dpy = dpy - u * dy;
    }
    const double ssq = dpx * dpx + dpy * dpy;
    if (ssq < safety) {
      dx1    = fxc[i] - fxa[i];
      dx2    = fxd[i] - fxb[i];
      dy1    = fyc[i] - fya[i];
      dy2    = fyd[i] - fyb[i];
      umin   = u;
      safety = ssq;
    }
  }
  if (umin < 0 || umin > 1) umin = 0.;
  dx = dx1 + umin * (dx2 - dx1);
  dy = dy1 + umin * (dy2 - dy1);
  safety *= 1. - 4. * fDz * fDz / (dx * dx + dy * dy + 4. * fDz * fDz);
  safety = Sqrt(safety);
  if (safplanar < safety) safety = safplanar;
  return safety;
}

double GenTrap::ShellSafetyToOut(Vec3 const &p, double safmax) const
{
  const double eps = 100. * kTolerance;
  double safety    = safmax;
  if (Abs(safety) < eps) return safety;
  double safetyface;
  if (fisplanar) {
    for (int i = 0; i < 4; ++i) {
      if (fdegen[i]) continue;
      const Vec3 pa(fxa[i], fya[i], -fDz);
      safetyface = (pa - p).Dot(fNormals[i]);
      if (safetyface < safety) safety = safetyface;
    }
    if (Abs(safety) < eps) safety = 0.;
    return safety;
  }
  safetyface = SafetyCurved(p, true);
  if (safetyface < safety) safety = safetyface;
  if (safety > 0. && safety < eps) safety = 0.;
  return safety;
}

double GenTrap::ShellSafetyToIn(Vec3 const &p, double safmax) const
{
  const double eps = 100. * kTolerance;
  double safety    = safmax;
  if (Abs(safety) < eps) return safety;
  double safetyface;
  if (fisplanar) {
    for (int i = 0; i < 4; ++i) {
      if (fdegen[i]) continue;
      const Vec3 pa(fxa[i], fya[i], -fDz);
      safetyface = (p - pa).Dot(fNormals[i]);
      if (safetyface > safety) safety = safetyface;
    }
    if (Abs(safety) < eps) safety = 0.;
    return safety;
  }
  safetyface = SafetyCurved(p, false);
  if (safetyface > safety) safety = safetyface;
  if (safety > 0. && safety < eps) safety = 0.;
  return safety;
}

// ------------------------------------------------------------ GenTrapImplementation
// IsInTopOrBottomPolygon: the crossing point of a ray with the top (or bottom) face
bool GenTrap::IsInTopOrBottomPolygon(double x, double y, bool top) const
{
  bool cout = false, degenerate = true;
  for (int i = 0; i < 4; ++i) {
    const int k          = i + (top ? 4 : 0);
    const double deltaX  = fDeltaX[k], deltaY = fDeltaY[k];
    const double cornerX = fVerticesX[k], cornerY = fVerticesY[k];
    double cross         = (x - cornerX) * deltaY;
    cross -= (y - cornerY) * deltaX;
    degenerate = degenerate && (deltaX < MakePlusTolerant<true>(0.)) && (deltaY < MakePlusTolerant<true>(0.));
    cout       = cout || (cross < 0. - (Abs(deltaX) + Abs(deltaY)) * kHalfTolerance);
    if (cout) return false;
  }
  return !(cout || degenerate);
}

// GenericKernelForContainsAndInside: the bounding box, then the side of each lateral edge
// of the section at the point's z
void GenTrap::ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const
{
  const double tolerancesq = 10000. * kTolerance * kTolerance;
  const Vec3 q             = p - Vec3(fBBorig[0], fBBorig[1], fBBorig[2]);
  const double dist        = (q.Abs() - Vec3(fBBdim[0], fBBdim[1], fBBdim[2])).Max();
  cin                      = forInside ? dist < -kHalfTolerance : false;
  cout                     = dist > kHalfTolerance;
  if (cout) return;
  const double cf = fHalfInverseDz * (fDz - p.z());
  double vX[4], vY[4];
  for (int i = 0; i < 4; ++i) {
    vX[i] = fVerticesX[i + 4] + cf * fConnX[i];
    vY[i] = fVerticesY[i + 4] + cf * fConnY[i];
  }
  for (int i = 0; i < 4; ++i) {
    if (fDegenerated[i]) continue;
    const int j         = (i + 1) % 4;
    const double DeltaX = vX[j] - vX[i];
    const double DeltaY = vY[j] - vY[i];
    const double cross  = (p.x() - vX[i]) * DeltaY - (p.y() - vY[i]) * DeltaX;
    if (forInside) {
      const bool onsurf = (cross * cross < tolerancesq * (DeltaX * DeltaX + DeltaY * DeltaY));
      cout              = cout || ((cross < -kHalfTolerance) && !onsurf);
      cin               = cin && (cross > kHalfTolerance) && !onsurf;
    } else {
      cout = cout || (cross < 0.);
    }
    if (cout) return;
  }
}

int GenTrap::Inside(Vec3 const &p) const
{
  bool cin, cout;
  ContainsAndInside(p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}

bool GenTrap::Contains(Vec3 const &p) const
{
  bool cin, cout;
  ContainsAndInside(p, false, cin, cout);
  return !cout;
}

double GenTrap::DistanceToIn(Vec3 const &p, Vec3 const &d, double) const
{
  const Box bb(fBBdim[0], fBBdim[1], fBBdim[2]);
  const double bbdistance = bb.DistanceToIn(p - Vec3(fBBorig[0], fBBorig[1], fBBorig[2]), d, kInfLength);
  double distance         = kInfLength;
  bool done               = bbdistance >= kInfLength;
  if (done) return distance;
  const double zsafety = Abs(p.z()) - fDz;
  bool canhitz         = zsafety > MakeMinusTolerant<true>(0.);
  canhitz              = canhitz && (p.z() * d.z() < 0);
  if (canhitz) {
    const double next   = zsafety / NonZeroAbs(d.z());
    const double coord1 = p.x() + next * d.x();
    const double coord2 = p.y() + next * d.y();
    const bool top      = d.z() < 0;
    const bool hits     = IsInTopOrBottomPolygon(coord1, coord2, top);
    if (hits) return bbdistance;
  }
  const double disttoplanes = ShellDistanceToIn(p, d, done);
  return Min(disttoplanes, distance);
}

double GenTrap::DistanceToOut(Vec3 const &p, Vec3 const &d, double) const
{
  const double sign      = d.z() < 0 ? -1.0 : 1.0;
  const double distmin   = (sign * fDz - p.z()) / NonZero(d.z());
  const double distplane = ShellDistanceToOut(p, d);
  return Min(distmin, distplane);
}

double GenTrap::SafetyToIn(Vec3 const &p) const
{
  const Box bb(fBBdim[0], fBBdim[1], fBBdim[2]);
  const Vec3 q = p - Vec3(fBBorig[0], fBBorig[1], fBBorig[2]);
  if (!bb.Contains(q)) return bb.SafetyToIn(q);
  const double safety = Abs(p[2]) - fDz;
  return ShellSafetyToIn(p, safety);
}

double GenTrap::SafetyToOut(Vec3 const &p) const
{
  const double safety = fDz - Abs(p[2]);
  return ShellSafetyToOut(p, safety);
}

// NormalKernel with GetClosestEdge (used by the known-answer tests, which build points
// along the shape's own normals)
Vec3 GenTrap::Normal(Vec3 const &p, bool &validNormal) const
{
  validNormal = true;
  Vec3 normal(0., 0., 0.);
  const double safz = Abs(fDz - Abs(p.z()));
  const bool onZ    = safz < 10. * kTolerance;
  if (onZ && p.z() > 0.) normal[2] = 1.;
  if (onZ && p.z() < 0.) normal[2] = -1.;
  if (onZ) return normal;
  const double cf = fHalfInverseDz * (fDz - p.z());
  double vX[4], vY[4];
  for (int i = 0; i < 4; ++i) {
    vX[i] = fVerticesX[i + 4] + cf * fConnX[i];
    vY[i] = fVerticesY[i + 4] + cf * fConnY[i];
  }
  // GetClosestEdge
  int iseg = 0;
  double frac = -1., safe = kInfLength, ssq = kInfLength;
  for (int i = 0; i < 4; ++i) {
    const int j     = (i + 1) % 4;
    const double dx = vX[j] - vX[i], dy = vY[j] - vY[i];
    double dpx = p.x() - vX[i], dpy = p.y() - vY[i];
    const double lsq = dx * dx + dy * dy;
    if (lsq < kTolerance) {
      ssq = dpx * dpx + dpy * dpy;
      if (ssq < safe) iseg = i, frac = -1., safe = ssq;
      continue;
    }
    double u = (dpx * dx + dpy * dy) / NonZero(lsq);
    if (u > 1) dpx = p.x() - vX[j], dpy = p.y() - vY[j];
    if (u >= 0 && u <= 1) dpx = dpx - u * dx, dpy = dpy - u * dy;
    if (u > 1 || u < 0) u = -1.;
    ssq = dpx * dpx + dpy * dpy;
    if (ssq < safe) iseg = i, frac = u, safe = ssq;
  }
  if (frac < 0.) frac = 0.;
  if (!fIsTwisted) return fNormals[iseg];
  const int jseg = (iseg + 1) % 4;
  double x0 = vX[iseg], y0 = vY[iseg];
  const double x2 = vX[jseg], y2 = vY[jseg];
  x0 += frac * (x2 - x0);
  y0 += frac * (y2 - y0);
  double x1 = fVerticesX[iseg + 4], y1 = fVerticesY[iseg + 4];
  x1 += frac * (fVerticesX[jseg + 4] - x1);
  y1 += frac * (fVerticesY[jseg + 4] - y1);
  const double ax = x1 - x0, ay = y1 - y0, az = fDz - p.z();
  const double bx = x2 - x0, by = y2 - y0, bz = 0.;
  normal = Vec3(ay * bz - az * by, az * bx - ax * bz, ax * by - ay * bx);
  Normalize(normal);
  return normal;
}

} // namespace oracle
