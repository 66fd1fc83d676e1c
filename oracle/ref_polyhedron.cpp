// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
//
// Polyhedron: construction as in VecGeom/volumes/PolyhedronStruct.h:112-430 (constructor +
// Initialize), quadrilateral sets as in VecGeom/volumes/Quadrilaterals.h +
// source/Quadrilaterals.cpp, plane sets as in VecGeom/volumes/Planes.h + source/Planes.cpp,
// and the scalar kernels of VecGeom/volumes/kernel/PolyhedronImplementation.h with
// EInnerRadii::kGeneric / EPhiCutout::kGeneric (the type UnplacedPolyhedron uses).
#include "ref_shapes_more.h"

namespace oracle {
namespace {

Vec3 Normalized(Vec3 const &v) // Vector3D::Normalized (Vector3D.h:202)
{
  const double inv = 1. / v.Mag();
  return Vec3(v[0] * inv, v[1] * inv, v[2] * inv);
}
Vec3 FixZeroes(Vec3 v) // Vector3D::FixZeroes (Vector3D.h:298-305)
{
  for (int i = 0; i < 3; ++i)
    if (Abs(v[i]) < kTolerance) v[i] = 0.;
  return v;
}
Vec3 Cross(Vec3 const &l, Vec3 const &r) // Vector3D::Cross (Vector3D.h:230-234)
{
  return Vec3(l[1] * r[2] - l[2] * r[1], l[2] * r[0] - l[0] * r[2], l[0] * r[1] - l[1] * r[0]);
}
Vec3 FromCylindrical(double r, double phi, double z) { return Vec3(r * std::cos(phi), r * std::sin(phi), z); }
bool Same(Vec3 const &a, Vec3 const &b) // operator== with tolerance (Vector3D.h:387-390)
{
  return Abs(a[0] - b[0]) < kTolerance && Abs(a[1] - b[1]) < kTolerance && Abs(a[2] - b[2]) < kTolerance;
}
double NormalizeAngle(double a) // GenericKernels.h:143-146
{
  return a + kTwoPi * (double)((a < 0 ? 1 : 0) - (int)(a / kTwoPi));
}
// DistanceToLineSegmentSquared1 (GenericKernels.h:190-215), scalar path
double DistanceToLineSegmentSquared(Vec3 const &c0, Vec3 const &c1, Vec3 const &p)
{
  const Vec3 line = c1 - c0;
  const Vec3 proj = p - c0;
  const double dot0 = proj.Dot(line);
  if (dot0 <= 0) return (p - c0).Mag2();
  const double dot1 = line.Mag2();
  if (dot1 <= dot0) return (p - c1).Mag2();
  return ((c0 + (dot0 / dot1) * line) - p).Mag2();
}

} // namespace

// ---------------------------------------------------------------- Quads
void Quads::Resize(int n)
{
  normal.assign(n, Vec3());
  dist.assign(n, 0.);
  for (int j = 0; j < 4; ++j) {
    sideN[j].assign(n, Vec3());
    sideD[j].assign(n, 0.);
    corner[j].assign(n, Vec3());
  }
}

// Quadrilaterals::Set (source/Quadrilaterals.cpp:44-123) with Planes::Set (source/Planes.cpp:31-45)
void Quads::Set(int i, Vec3 const &c0, Vec3 const &c1, Vec3 const &c2, Vec3 const &c3)
{
  corner[0][i] = c0, corner[1][i] = c1, corner[2][i] = c2, corner[3][i] = c3;
  Vec3 ch[4];
  ch[0]        = corner[0][i];
  int assigned = 1, tested = 1;
  while (tested < 4) {
    bool chosen = true;
    for (int j = 0; j < assigned; ++j)
      if (Same(ch[j], corner[tested][i])) {
        chosen = false;
        break;
      }
    if (chosen) ch[assigned++] = corner[tested][i];
    ++tested;
  }
  const double a = ch[0][1] * (ch[1][2] - ch[2][2]) + ch[1][1] * (ch[2][2] - ch[0][2]) + ch[2][1] * (ch[0][2] - ch[1][2]);
  const double b = ch[0][2] * (ch[1][0] - ch[2][0]) + ch[1][2] * (ch[2][0] - ch[0][0]) + ch[2][2] * (ch[0][0] - ch[1][0]);
  const double c = ch[0][0] * (ch[1][1] - ch[2][1]) + ch[1][0] * (ch[2][1] - ch[0][1]) + ch[2][0] * (ch[0][1] - ch[1][1]);
  double d       = -ch[0][0] * (ch[1][1] * ch[2][2] - ch[2][1] * ch[1][2]) -
             ch[1][0] * (ch[2][1] * ch[0][2] - ch[0][1] * ch[2][2]) - ch[2][0] * (ch[0][1] * ch[1][2] - ch[1][1] * ch[0][2]);
  Vec3 n(a, b, c);
  const double inv = 1. / n.Mag();
  n                = Vec3(n[0] * inv, n[1] * inv, n[2] * inv);
  d *= inv;
  n         = FixZeroes(n);
  normal[i] = n;
  dist[i]   = d;
  const Vec3 cs[4] = {c0, c1, c2, c3};
  for (int j = 0; j < 4; ++j) {
    const Vec3 &a0 = cs[j], &a1 = cs[(j + 1) % 4];
    if (!Same(a1, a0)) {
      const Vec3 sv    = FixZeroes(Normalized(Cross(n, a1 - a0)));
      const double il  = 1. / sv.Mag();
      sideN[j][i]      = il * sv;
      sideD[j][i]      = il * -sv.Dot(a0);
    } else {
      sideN[j][i] = Vec3(0, 0, 0);
      sideD[j][i] = 0.;
    }
  }
}

// Planes::Contains (VecGeom/volumes/Planes.h:192-206)
bool Quads::Contains(Vec3 const &p) const
{
  for (int i = 0; i < size(); ++i)
    if (!(p.Dot(normal[i]) + dist[i] < 0)) return false;
  return true;
}

// Planes::Inside (VecGeom/volumes/Planes.h:246-266)
int Quads::Inside(Vec3 const &p) const
{
  int result = kInside;
  for (int i = 0; i < size(); ++i) {
    const double r = normal[i][0] * p[0] + normal[i][1] * p[1] + normal[i][2] * p[2] + dist[i];
    if (r > kHalfTolerance) result = kOutside;
    if (result == kInside && r > -kHalfTolerance) result = kSurface;
    if (result == kOutside) break;
  }
  return result;
}

int Quads::Inside(Vec3 const &p, int i) const // Planes.h:268-281
{
  int result     = kInside;
  const double r = normal[i][0] * p[0] + normal[i][1] * p[1] + normal[i][2] * p[2] + dist[i];
  if (r > kHalfTolerance) result = kOutside;
  if (result == kInside && r > -kHalfTolerance) result = kSurface;
  return result;
}

bool Quads::RayHits(int i, Vec3 const &x) const // Quadrilaterals.h:107-117
{
  for (int j = 0; j < 4; ++j)
    if (!(x.Dot(sideN[j][i]) + sideD[j][i] >= -kTolerance)) return false;
  return true;
}

// Quadrilaterals::DistanceToIn<Real_v, behindPlanesT> (Quadrilaterals.h:326-376), scalar loop
double Quads::DistanceToIn(Vec3 const &p, Vec3 const &d, bool behind) const
{
  double best = kInfLength;
  for (int i = 0; i < size(); ++i) {
    const Vec3 &n   = normal[i];
    double distance = p.Dot(n) + dist[i];
    if (!((behind ? -distance : distance) > -kTolerance)) continue;
    const double proj = d.Dot(n);
    if (!((behind ? proj : -proj) > 0)) continue;
    distance /= -(proj + CopySign(1E-20, proj));
    const Vec3 x = p + d * distance;
    bool valid   = true;
    for (int j = 0; j < 4; ++j) {
      valid &= x.Dot(sideN[j][i]) + sideD[j][i] >= -kTolerance;
      if (!valid) break;
    }
    if (valid) best = distance;
    if (best < kInfLength) break;
  }
  return Max(0., best);
}

// Quadrilaterals::DistanceToOut(point, direction, zMin, zMax) (Quadrilaterals.h:447-496)
double Quads::DistanceToOut(Vec3 const &p, Vec3 const &d, double zMin, double zMax) const
{
  double best = kInfLength;
  for (int i = 0; i < size(); ++i) {
    const Vec3 &n = normal[i];
    double t      = p.Dot(n) + dist[i];
    if (!(t < kTolerance)) continue;
    const double proj = d.Dot(n);
    if (!(proj > 0)) continue;
    t /= -proj;
    if (!(t < best)) continue;
    bool valid;
    if (zMin == zMax) {
      valid = RayHits(i, p + t * d);
    } else {
      const double zp = p[2] + t * d[2];
      valid           = (zp >= zMin - kTolerance) && (zp < zMax + kTolerance);
    }
    if (!valid) continue;
    best = t;
  }
  if (best > -kTolerance) best = Max(best, 0.);
  return best;
}

// Quadrilaterals::ScalarDistanceSquared (Quadrilaterals.h:507-578)
double Quads::ScalarDistanceSquared(int i, Vec3 const &p) const
{
  const Vec3 &n     = normal[i];
  double distance   = p.Dot(n) + dist[i];
  const Vec3 x      = p - distance * n;
  bool within[4];
  for (int j = 0; j < 4; ++j)
    within[j] = x[0] * sideN[j][i][0] + x[1] * sideN[j][i][1] + x[2] * sideN[j][i][2] + sideD[j][i] >= 0;
  if (within[0] && within[1] && within[2] && within[3]) return distance * distance;
  double dsq = kInfLength;
  for (int j = 0; j < 4; ++j) {
    if (!within[j]) {
      distance = DistanceToLineSegmentSquared(corner[j][i], corner[(j + 1) % 4][i], p);
      if (distance < dsq) dsq = distance;
    }
  }
  return dsq;
}

// ---------------------------------------------------------------- Polyhedron
// PolyhedronStruct(phiStart, phiDelta, sideCount, zPlaneCount, zPlanes, rMin, rMax) and
// Initialize (PolyhedronStruct.h:112-125, 262-430).
Polyhedron::Polyhedron(double phiStart, double phiDelta, int sideCount, int nz, const double *zPlanes,
                       const double *rMin, const double *rMax)
    : fSideCount(sideCount), fHasPhiCutout(phiDelta < kTwoPi), fHasLargePhiCutout(phiDelta < kPi),
      fPhiStart(NormalizeAngle(phiStart)), fPhiDelta(phiDelta > kTwoPi ? kTwoPi : phiDelta),
      fPhiWedge(fPhiDelta, fPhiStart), fBoundingTube(0, 1, 1, fPhiStart, fPhiDelta)
{
  fZPlanes.assign(zPlanes, zPlanes + nz);
  fRMin.assign(rMin, rMin + nz);
  fRMax.assign(rMax, rMax + nz);
  fSameZ.assign(nz, false);
  for (int i = 0; i < nz; i++)
    if (i > 0 && i < nz - 1 && fZPlanes[i] == fZPlanes[i + 1]) fSameZ[i] = true;
  fZSegments.resize(nz - 1);
  for (int i = 0; i < nz - 1; ++i) {
    const bool hasInner = rMin[i] > 0 || rMin[i + 1] > 0;
    int mult            = (zPlanes[i] == zPlanes[i + 1] && rMax[i] == rMax[i + 1]) ? 0 : 1;
    fZSegments[i].outer.Resize(sideCount * mult);
    if (fHasPhiCutout) {
      mult = (zPlanes[i] == zPlanes[i + 1]) ? 0 : 1;
      fZSegments[i].phi.Resize(2 * mult);
    }
    mult = (zPlanes[i] == zPlanes[i + 1] && rMin[i] == rMin[i + 1]) ? 0 : 1;
    if (hasInner && mult > 0) {
      fZSegments[i].inner.Resize(sideCount * mult);
      fHasInnerRadii = true;
    } else {
      fZSegments[i].inner.Resize(0);
    }
  }
  phiStart = NormalizeAngle(phiStart);
  if (phiDelta > kTwoPi) phiDelta = kTwoPi;
  const double sidePhi = phiDelta / sideCount;
  std::vector<double> vphi(sideCount + 1);
  fPhiSections.assign(sideCount + 1, Vec3());
  for (int i = 0; i < sideCount + 1; ++i) {
    vphi[i]               = NormalizeAngle(phiStart + i * sidePhi);
    const Vec3 cornerVec  = FixZeroes(Normalized(FromCylindrical(1., vphi[i], 0)));
    fPhiSections[i]       = Cross(Normalized(cornerVec), Vec3(0, 0, -1));
  }
  if (!fHasPhiCutout) vphi[sideCount] = vphi[0];
  const double cosHalf = std::cos(0.5 * sidePhi);
  double innerRadius = kInfLength, outerRadius = -kInfLength;
  for (int i = 0; i < nz; ++i) {
    if (rMin[i] < innerRadius) innerRadius = rMin[i];
    if (rMax[i] > outerRadius) outerRadius = rMax[i];
  }
  outerRadius /= cosHalf;
  const double boundingTubeZ  = 0.5 * (zPlanes[nz - 1] - zPlanes[0]) + kTolerance;
  const double kPhiTolerance  = 100 * kTolerance;
  const double boundsPhiStart = !fHasPhiCutout ? 0 : phiStart - kPhiTolerance;
  const double boundsPhiDelta = !fHasPhiCutout ? kTwoPi : phiDelta + 2 * kPhiTolerance;
  fBoundingTube = Tube(innerRadius - kHalfTolerance, outerRadius + kHalfTolerance, boundingTubeZ, boundsPhiStart,
                       boundsPhiDelta);
  fBoundingTubeOffset = 0.5 * (zPlanes[0] + zPlanes[nz - 1]);

  auto VI = [sideCount](int plane, int corner) { return plane * (sideCount + 1) + corner; };
  std::vector<Vec3> ov(nz * (sideCount + 1)), iv(nz * (sideCount + 1));
  for (int i = 0; i < nz; ++i) {
    for (int j = 0, jMax = sideCount + (fHasPhiCutout ? 1 : 0); j < jMax; ++j) {
      ov[VI(i, j)] = FixZeroes(FromCylindrical(rMax[i] / cosHalf, vphi[j], zPlanes[i]));
      iv[VI(i, j)] = FixZeroes(FromCylindrical(rMin[i] / cosHalf, vphi[j], zPlanes[i]));
    }
    if (!fHasPhiCutout) {
      ov[VI(i, sideCount)] = ov[VI(i, 0)];
      iv[VI(i, sideCount)] = iv[VI(i, 0)];
    }
  }
  auto WrongNormal = [](Vec3 const &n, Vec3 const &c) { return n[0] * c[0] + n[1] * c[1] < 0; };
  for (int ip = 0; ip < nz - 1; ++ip) {
    ZSegment &s = fZSegments[ip];
    for (int k = 0; k < s.outer.size(); ++k) {
      s.outer.Set(k, ov[VI(ip, k)], ov[VI(ip, k + 1)], ov[VI(ip + 1, k + 1)], ov[VI(ip + 1, k)]);
      if (WrongNormal(s.outer.normal[k], ov[VI(ip, k)])) s.outer.FlipSign(k);
    }
    for (int k = 0; k < s.inner.size(); ++k) {
      s.inner.Set(k, iv[VI(ip, k)], iv[VI(ip, k + 1)], iv[VI(ip + 1, k + 1)], iv[VI(ip + 1, k)]);
      if (WrongNormal(s.inner.normal[k], iv[VI(ip, k)])) s.inner.FlipSign(k);
    }
    if (fHasPhiCutout && s.phi.size() == 2) {
      s.phi.Set(0, iv[VI(ip, 0)], iv[VI(ip + 1, 0)], ov[VI(ip + 1, 0)], ov[VI(ip, 0)]);
      if (s.phi.normal[0].Dot(fPhiSections[0]) > 0) s.phi.FlipSign(0);
      s.phi.Set(1, ov[VI(ip, sideCount)], ov[VI(ip + 1, sideCount)], iv[VI(ip + 1, sideCount)],
                iv[VI(ip, sideCount)]);
      if (s.phi.normal[1].Dot(fPhiSections[fSideCount]) < 0) s.phi.FlipSign(1);
    }
  }
}

// FindZSegmentKernel (PolyhedronImplementation.h:288-305)
int Polyhedron::FindZSegment(double z) const
{
  int index = -1, b = 0;
  const int n = (int)fZPlanes.size();
  while (b < n - 1 && z - kTolerance > fZPlanes[b]) {
    ++index;
    ++b;
  }
  if (z + kTolerance > fZPlanes[b]) return index + 1;
  return index;
}

// FindPhiSegment (PolyhedronImplementation.h:318-343)
int Polyhedron::FindPhiSegment(Vec3 const &p) const
{
  int index    = -1;
  double first = p[0] * fPhiSections[0][0] + p[1] * fPhiSections[0][1] + p[2] * fPhiSections[0][2];
  for (int i = 1; i < fSideCount + 1; ++i) {
    const double second = p[0] * fPhiSections[i][0] + p[1] * fPhiSections[i][1] + p[2] * fPhiSections[i][2];
    if (first > -kTolerance && second < kTolerance) index = i - 1;
    if (index >= 0) break;
    first = second;
  }
  return index;
}

// DistanceToInZSegment (PolyhedronImplementation.h:345-380)
double Polyhedron::DistanceToInZSegment(int si, Vec3 const &p, Vec3 const &d) const
{
  ZSegment const &s = fZSegments[si];
  double distance   = s.outer.DistanceToIn(p, d, false);
  bool done         = distance < kInfLength;
  if (done) return distance;
  if (fHasPhiCutout) distance = s.phi.DistanceToIn(p, d, false);
  done |= distance < kInfLength;
  if (done) return distance;
  if (s.hasInnerRadius()) distance = s.inner.DistanceToIn(p, d, true);
  return distance;
}

// DistanceToOutZSegment (PolyhedronImplementation.h:382-420)
double Polyhedron::DistanceToOutZSegment(int si, double zMin, double zMax, Vec3 const &p, Vec3 const &d) const
{
  ZSegment const &s = fZSegments[si];
  bool done         = false;
  double distance   = kInfLength;
  if (s.hasInnerRadius()) {
    distance = s.inner.DistanceToIn(p, d, false);
    done     = distance < kInfLength;
    if (done) return distance;
  }
  if (fHasPhiCutout) {
    const double distphi = s.phi.DistanceToIn(p, d, true);
    if (!done && distance > -kTolerance) distance = distphi;
    done = distance > -kTolerance && distance < kInfLength;
    if (done) return distance;
  }
  const double distout = s.outer.DistanceToOut(p, d, zMin, zMax);
  if (!done) distance = distout;
  return distance;
}

// ScalarSafetyToZSegmentSquared (PolyhedronImplementation.h:422-556)
double Polyhedron::SafetyToZSegmentSquared(int si, int &phiIndex, Vec3 const &p, bool ptInside, int &iSurf) const
{
  ZSegment const &s   = fZSegments[si];
  const bool cutout   = phiIndex < 0;
  double safetySq     = kInfLength;
  if (fHasPhiCutout && s.phi.size() == 2) {
    if (ptInside || cutout) {
      iSurf        = 0;
      safetySq     = s.phi.ScalarDistanceSquared(0, p);
      const double saf = s.phi.ScalarDistanceSquared(1, p);
      if (saf < safetySq) {
        safetySq = saf;
        iSurf    = 1;
      }
      if (cutout) {
        if (fHasLargePhiCutout && s.hasInnerRadius()) {
          if (s.inner.size() > 0) {
            double si2 = s.inner.ScalarDistanceSquared(0, p);
            if (si2 < safetySq) {
              iSurf    = 2;
              phiIndex = 0;
              safetySq = si2;
            }
            if (s.inner.size() > 1) {
              si2 = s.inner.ScalarDistanceSquared(s.inner.size() - 1, p);
              if (si2 < safetySq) {
                iSurf    = 2;
                phiIndex = s.inner.size() - 1;
                safetySq = si2;
              }
            }
          }
        }
        return safetySq;
      }
    }
  }
  const int nseg = (int)fZSegments.size();
  if (cutout && si > 0 && si < nseg - 1 && fZPlanes[si] == fZPlanes[si + 1]) {
    double so = kInfLength;
    if (s.outer.size() > 0) {
      so = s.outer.ScalarDistanceSquared(0, p);
      if (so < safetySq) {
        iSurf    = 3;
        phiIndex = 0;
        safetySq = so;
      }
      if (s.outer.size() > 1) {
        so = s.outer.ScalarDistanceSquared(s.outer.size() - 1, p);
        if (so < safetySq) {
          iSurf    = 3;
          phiIndex = s.outer.size() - 1;
          safetySq = so;
        }
      }
    }
    double sin2 = kInfLength;
    if (s.hasInnerRadius()) {
      if (s.inner.size() > 0) {
        sin2 = s.inner.ScalarDistanceSquared(0, p);
        if (sin2 < safetySq) {
          iSurf    = 2;
          phiIndex = 0;
          safetySq = sin2;
        }
        if (s.inner.size() > 1) {
          sin2 = s.inner.ScalarDistanceSquared(s.inner.size() - 1, p);
          if (sin2 < safetySq) {
            iSurf    = 2;
            phiIndex = s.inner.size() - 1;
            safetySq = sin2;
          }
        }
      }
    }
    return safetySq;
  }
  double so = kInfLength;
  if (s.outer.size() > 0) so = s.outer.ScalarDistanceSquared(phiIndex, p);
  double sin2 = kInfLength;
  if (s.hasInnerRadius()) {
    if (s.inner.size() > 0) sin2 = s.inner.ScalarDistanceSquared(phiIndex, p);
  }
  if (sin2 < safetySq) {
    iSurf    = 2;
    safetySq = sin2;
  }
  if (so < safetySq) {
    iSurf    = 3;
    safetySq = so;
  }
  return safetySq;
}

// ScalarDistanceToEndcaps<pointInsideT> (PolyhedronImplementation.h:558-610)
void Polyhedron::DistanceToEndcaps(bool pointInside, Vec3 const &p, Vec3 const &d, double &distance) const
{
  const int nseg = (int)fZSegments.size();
  ZSegment const *s;
  double zPlane;
  const bool first = pointInside ? (d[2] < 0) : !(d[2] < 0);
  if (first) {
    s      = &fZSegments[0];
    zPlane = fZPlanes[0];
  } else {
    s      = &fZSegments[nseg - 1];
    zPlane = fZPlanes[nseg];
  }
  const double t = (zPlane - p[2]) / NonZero(d[2]);
  if (t < -kTolerance || t >= distance) return;
  const Vec3 x = p + t * d;
  if (!s->outer.Contains(x)) return;
  if (s->hasInnerRadius()) {
    if (s->inner.Contains(x)) return;
  }
  if (fHasPhiCutout) {
    if (InPhiCutoutWedge(*s, x)) return;
  }
  distance = t;
}

// ScalarSafetyToEndcapsSquared (PolyhedronImplementation.h:612-650)
void Polyhedron::SafetyToEndcapsSquared(Vec3 const &p, double &distanceSq, int &iz) const
{
  const int nseg        = (int)fZSegments.size();
  const double firstD   = fZPlanes[0] - p[2];
  const double lastD    = fZPlanes[nseg] - p[2];
  const bool isFirst    = Abs(firstD) < Abs(lastD);
  iz                    = 0;
  ZSegment const &s     = isFirst ? fZSegments[0] : fZSegments[nseg - 1];
  const double t        = isFirst ? firstD : lastD;
  const double tsq      = t * t;
  if (tsq >= distanceSq) return;
  const Vec3 x(p[0], p[1], p[2] + t);
  if (!s.outer.Contains(x)) return;
  if (s.hasInnerRadius()) {
    if (s.inner.Contains(x)) return;
  }
  if (fHasPhiCutout) {
    if (InPhiCutoutWedge(s, x)) return;
  }
  iz         = isFirst ? -1 : 1;
  distanceSq = tsq;
}

// InPhiCutoutWedge (PolyhedronImplementation.h:652-672); the reference reads two phi
// planes that exist for every non-degenerate segment of a phi-cut polyhedron.
bool Polyhedron::InPhiCutoutWedge(ZSegment const &s, Vec3 const &p) const
{
  if (s.phi.size() < 2) return false;
  const bool s0 = p.Dot(s.phi.normal[0]) + s.phi.dist[0] >= 0;
  const bool s1 = p.Dot(s.phi.normal[1]) + s.phi.dist[1] >= 0;
  if (fHasLargePhiCutout) return s0 || s1;
  return s0 && s1;
}

// ScalarContainsKernel (PolyhedronImplementation.h:674-730)
bool Polyhedron::Contains(Vec3 const &p) const
{
  if (!fBoundingTube.Contains(Vec3(p[0], p[1], p[2] - fBoundingTubeOffset))) return false;
  const int zIndex = FindZSegment(p[2]);
  if (!((zIndex >= 0) && (zIndex < (int)fZSegments.size()))) return false;
  ZSegment const &s = fZSegments[zIndex];
  if (fSameZ[zIndex]) {
    const int phiIndex = FindPhiSegment(p);
    if (phiIndex < 0) return false;
    const Vec3 &vout   = s.outer.size() ? s.outer.sideN[0][phiIndex] : s.inner.sideN[0][phiIndex];
    const double r     = Abs(p.Dot(vout));
    const bool in1     = (r >= fRMin[zIndex]) && (r <= fRMax[zIndex]);
    const bool in2     = (r >= fRMin[zIndex + 1]) && (r <= fRMax[zIndex + 1]);
    return in1 | in2;
  }
  if (!s.outer.Contains(p)) return false;
  if (s.hasInnerRadius()) {
    if (s.inner.Contains(p)) return false;
  }
  if (fHasPhiCutout) {
    if (!s.phi.Contains(p)) return false;
  }
  return true;
}

// ScalarInsideKernel (PolyhedronImplementation.h:732-790)
int Polyhedron::Inside(Vec3 const &p) const
{
  if (!fBoundingTube.Contains(Vec3(p[0], p[1], p[2] - fBoundingTubeOffset))) return kOutside;
  const int nseg = (int)fZSegments.size();
  int zIndex     = FindZSegment(p[2]);
  if (zIndex > (nseg - 1)) zIndex = nseg - 1;
  if (zIndex < 0) zIndex = 0;
  ZSegment const &s = fZSegments[zIndex];
  if (fSameZ[zIndex]) return InsideSegBorder(p, zIndex);
  {
    const int io = s.outer.Inside(p);
    if (io != kInside) return io;
  }
  if (s.hasInnerRadius()) {
    const int ii = s.inner.Inside(p);
    if (ii == kInside) return kOutside;
    if (ii == kSurface) return kSurface;
  }
  if (fHasPhiCutout) {
    const int ip = s.phi.Inside(p);
    if (ip != kInside) return ip;
  }
  const double dz = Abs(Abs(p[2] - fBoundingTubeOffset) - 0.5 * (fZPlanes[nseg] - fZPlanes[0]));
  if (dz < kTolerance) return kSurface;
  return kInside;
}

// Wedge::Inside (VecGeom/volumes/Wedge_Evolution.h, Inside via GenericKernelForContainsAndInside)
static int WedgeInside(Wedge const &w, Vec3 const &p)
{
  bool ci = false, co = false;
  w.ContainsAndInside(p, true, ci, co);
  return co ? kOutside : (ci ? kInside : kSurface);
}

// ScalarInsideSegBorder (PolyhedronImplementation.h:792-830)
int Polyhedron::InsideSegBorder(Vec3 const &p, int zIndex) const
{
  ZSegment const &s  = fZSegments[zIndex];
  const int phiIndex = FindPhiSegment(p);
  if (phiIndex < 0) return kOutside;
  const Vec3 &vout = s.outer.size() ? s.outer.sideN[0][phiIndex] : s.inner.sideN[0][phiIndex];
  const double r   = Abs(p.Dot(vout));
  const bool in1   = (r > fRMin[zIndex] - kTolerance) && (r < fRMax[zIndex] + kTolerance);
  const bool in2   = (r > fRMin[zIndex + 1] - kTolerance) && (r < fRMax[zIndex + 1] + kTolerance);
  if (in1 && in2) {
    if ((r < fRMin[zIndex] + kTolerance) || (r > fRMax[zIndex] - kTolerance) || (r < fRMin[zIndex + 1] + kTolerance) ||
        (r > fRMax[zIndex + 1] - kTolerance))
      return kSurface;
    if (fHasPhiCutout) return WedgeInside(fPhiWedge, p);
    return kInside;
  }
  if (!in1 && !in2) return kOutside;
  return kSurface;
}

// ScalarInsideSegPhi (PolyhedronImplementation.h:832-870)
int Polyhedron::InsideSegPhi(Vec3 const &p, int zIndex, int phiIndex) const
{
  if (phiIndex < 0) return kOutside;
  const int nseg  = (int)fZSegments.size();
  const double dz = Abs(p[2] - fBoundingTubeOffset) - 0.5 * (fZPlanes[nseg] - fZPlanes[0]);
  if (dz > kHalfTolerance) return kOutside;
  if (fSameZ[zIndex]) return InsideSegBorder(p, zIndex);
  ZSegment const &s = fZSegments[zIndex];
  {
    const int io = s.outer.Inside(p, phiIndex);
    if (io != kInside) return io;
  }
  if (s.hasInnerRadius()) {
    const int ii = s.inner.Inside(p, phiIndex);
    if (ii == kInside) return kOutside;
    if (ii == kSurface) return kSurface;
  }
  if (fHasPhiCutout) {
    const int ip = WedgeInside(fPhiWedge, p);
    if (ip != kInside) return ip;
  }
  if (Abs(dz) < kHalfTolerance) return kSurface;
  return kInside;
}

// ScalarDistanceToInKernel (PolyhedronImplementation.h:872-945)
double Polyhedron::DistanceToIn(Vec3 const &p, Vec3 const &d, double stepMax) const
{
  const int nseg = (int)fZSegments.size();
  if ((p[2] < fZPlanes[0] + kTolerance) && d[2] <= 0) return kInfLength;
  if ((p[2] > fZPlanes[nseg] - kTolerance) && d[2] >= 0) return kInfLength;
  if (Inside(p) == kInside) return -1.;
  double tubeDistance = 0.;
  {
    const Vec3 bp(p[0], p[1], p[2] - fBoundingTubeOffset);
    if (!fBoundingTube.Contains(bp)) {
      tubeDistance = fBoundingTube.DistanceToIn(bp, d, stepMax);
      if (tubeDistance == kInfLength) return kInfLength;
    }
  }
  int zIndex = FindZSegment(p[2]);
  zIndex     = zIndex < 0 ? 0 : (zIndex >= nseg ? nseg - 1 : zIndex);
  const bool goingRight = d[2] >= 0;
  double distance       = kInfLength;
  if (goingRight) {
    for (; zIndex < nseg; ++zIndex) {
      distance = DistanceToInZSegment(zIndex, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  } else {
    for (; zIndex >= 0; --zIndex) {
      distance = DistanceToInZSegment(zIndex, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  }
  DistanceToEndcaps(false, p, d, distance);
  return (distance >= tubeDistance - 1E-6) ? distance : kInfLength;
}

// ScalarSafetyKernel (PolyhedronImplementation.h:947-990)
double Polyhedron::SafetyKernel(Vec3 const &p, bool ptInside) const
{
  double safety = kInfLength;
  double dz;
  int iSurf = 0, iz = 0;
  const int zMax = (int)fZSegments.size();
  int zIndex     = FindZSegment(p[2]);
  zIndex         = zIndex < 0 ? 0 : (zIndex >= zMax ? zMax - 1 : zIndex);
  int phiIndex   = FindPhiSegment(p);
  const int inside = InsideSegPhi(p, zIndex, phiIndex);
  if (inside == kSurface) return 0.;
  const bool contains = (inside == kInside);
  if (contains ^ ptInside) return -1.;
  for (int z = zIndex; z < zMax;) {
    safety = Min(safety, SafetyToZSegmentSquared(z, phiIndex, p, ptInside, iSurf));
    ++z;
    dz = fZPlanes[z] - p[2];
    if (dz * dz > safety) break;
  }
  for (int z = zIndex - 1; z >= 0; --z) {
    safety = Min(safety, SafetyToZSegmentSquared(z, phiIndex, p, ptInside, iSurf));
    dz     = p[2] - fZPlanes[z];
    if (dz * dz > safety) break;
  }
  SafetyToEndcapsSquared(p, safety, iz);
  return Sqrt(safety);
}

// ScalarDistanceToOutKernel (PolyhedronImplementation.h:1045-1090)
double Polyhedron::DistanceToOut(Vec3 const &p, Vec3 const &d, double) const
{
  const int zMax = (int)fZSegments.size();
  if ((p[2] < fZPlanes[0] - kTolerance) || (p[2] > fZPlanes[zMax] + kTolerance)) return -1.;
  if (Inside(p) == kOutside) return -1.;
  int zIndex = FindZSegment(p[2]);
  zIndex     = zIndex < 0 ? 0 : (zIndex >= zMax ? zMax - 1 : zIndex);
  const bool goingRight = d[2] >= 0;
  double distance       = kInfLength;
  if (goingRight) {
    for (; zIndex < zMax; ++zIndex) {
      distance = DistanceToOutZSegment(zIndex, fZPlanes[zIndex], fZPlanes[zIndex + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (fZPlanes[zIndex] - p[2] > distance) break;
    }
  } else {
    for (; zIndex >= 0; --zIndex) {
      distance = DistanceToOutZSegment(zIndex, fZPlanes[zIndex], fZPlanes[zIndex + 1], p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (p[2] - fZPlanes[zIndex] > distance) break;
    }
  }
  DistanceToEndcaps(true, p, d, distance);
  if (distance >= kInfLength) distance = 0.;
  return distance;
}

// UnplacedPolyhedron::Extent (source/UnplacedPolyhedron.cpp:273-303)
void Polyhedron::Extent(Vec3 &lo, Vec3 &hi) const
{
  lo                   = Vec3(kInfLength, kInfLength, kInfLength);
  hi                   = Vec3(-kInfLength, -kInfLength, -kInfLength);
  const double sidePhi = fPhiDelta / fSideCount;
  const double conv    = 1. / std::cos(0.5 * sidePhi);
  for (int iphi = 0; iphi <= fSideCount; ++iphi) {
    const double phi  = fPhiStart + iphi * sidePhi;
    const double corx = conv * std::cos(phi), cory = conv * std::sin(phi);
    for (size_t k = 0; k < fZPlanes.size(); ++k) {
      const Vec3 a(fRMin[k] * corx, fRMin[k] * cory, fZPlanes[k]);
      const Vec3 b(fRMax[k] * corx, fRMax[k] * cory, fZPlanes[k]);
      for (int i = 0; i < 3; ++i) {
        lo[i] = Min(lo[i], a[i]);
        hi[i] = Max(hi[i], a[i]);
      }
      for (int i = 0; i < 3; ++i) {
        lo[i] = Min(lo[i], b[i]);
        hi[i] = Max(hi[i], b[i]);
      }
    }
  }
}

} // namespace oracle
