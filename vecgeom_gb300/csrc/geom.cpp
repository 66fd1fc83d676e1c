// Host geometry builder (see geom.h). Compiled with -ffp-contract=off so that the
// precomputed records, daughter boxes and cached global matrices round exactly as the
// reference's host code does.
#include "geom.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cuda_runtime.h>
#include <numeric>
#include <utility>

namespace vg {

// ---------------------------------------------------------------- transformations
HostXform HostXform::Identity()
{
  HostXform x;
  for (int i = 0; i < 3; ++i) x.m.t[i] = 0.;
  for (int i = 0; i < 9; ++i) x.m.r[i] = (i % 4 == 0) ? 1. : 0.;
  return x;
}

// Transformation3D(tx,ty,tz,r0..r8) + SetProperties (source/Transformation3D.cpp:54-62,118-126,174-185)
HostXform HostXform::FromArrays(const double *t, const double *r)
{
  HostXform x;
  std::memcpy(x.m.t, t, sizeof(x.m.t));
  std::memcpy(x.m.r, r, sizeof(x.m.r));
  x.has_trans = std::fabs(t[0]) > kTolerance || std::fabs(t[1]) > kTolerance || std::fabs(t[2]) > kTolerance;
  int code    = 0;
  for (int i = 0; i < 9; ++i) code |= (std::fabs(r[i]) > kTolerance) << i;
  x.has_rot  = !(code == 0x111 && r[0] == 1. && r[4] == 1. && r[8] == 1.);
  x.identity = !x.has_trans && !x.has_rot;
  return x;
}

// Transformation3D::MultiplyFromRight (Transformation3D.h:878-942): this <- this * rhs
void HostXform::MultiplyFromRight(HostXform const &rhs)
{
  if (rhs.identity) return;
  identity = false;
  double *t = m.t, *r = m.r;
  const double *rt = rhs.m.t, *rr = rhs.m.r;
  if (rhs.has_trans) {
    has_trans = true;
    for (int row = 0; row < 3; ++row) {
      t[row] += r[3 * row] * rt[0];
      t[row] += r[3 * row + 1] * rt[1];
      t[row] += r[3 * row + 2] * rt[2];
    }
  }
  if (rhs.has_rot) {
    has_rot = true;
    for (int row = 0; row < 3; ++row) {
      const double a = r[3 * row], b = r[3 * row + 1], c = r[3 * row + 2];
      for (int col = 0; col < 3; ++col) r[3 * row + col] = a * rr[col];
      for (int col = 0; col < 3; ++col) r[3 * row + col] += b * rr[3 + col];
      for (int col = 0; col < 3; ++col) r[3 * row + col] += c * rr[6 + col];
    }
  }
}

// InverseTransform (Transformation3D.h:797-826): master = t + R local
void HostXform::InverseTransform(const double *l, double *out) const
{
  for (int row = 0; row < 3; ++row) {
    double v = m.t[row];
    v += l[0] * m.r[3 * row];
    v += l[1] * m.r[3 * row + 1];
    v += l[2] * m.r[3 * row + 2];
    out[row] = v;
  }
}

// ---------------------------------------------------------------- shape records
namespace {
template <class T>
void pack(HostShape &s, T const &rec)
{
  static_assert(sizeof(T) % sizeof(double) == 0, "records are double-sized");
  s.rec.resize(sizeof(T) / sizeof(double));
  std::memcpy(s.rec.data(), &rec, sizeof(T));
}

// Wedge constructor (source/Wedge_Evolution.cpp)
WedgeRec make_wedge(double dphi, double sphi)
{
  WedgeRec w;
  w.dphi = dphi;
  w.a1x  = std::cos(sphi);
  w.a1y  = std::sin(sphi);
  w.a2x  = std::cos(sphi + dphi);
  w.a2y  = std::sin(sphi + dphi);
  w.n1x  = -std::sin(sphi);
  w.n1y  = std::cos(sphi);
  w.n2x  = std::sin(sphi + dphi);
  w.n2y  = -std::cos(sphi + dphi);
  return w;
}
bool wedge_contains(WedgeRec const &w, double x, double y)
{
  const double startCheck = (-x * w.a1y + y * w.a1x);
  const double endCheck   = (-w.a2x * y + w.a2y * x);
  bool out                = startCheck < 0.;
  out                     = (w.dphi < kPi) ? (out || endCheck < 0.) : (out && endCheck < 0.);
  return !out;
}

// Extent of a phi section of radii [rin, rout] (UnplacedTube.cpp:214-266, UnplacedCone.cpp:149-211)
void phi_section_extent(WedgeRec const &w, double sphi, double dphi, double rin, double rout, double halfz, double *lo,
                        double *hi)
{
  lo[0] = -rout, lo[1] = -rout, lo[2] = -halfz;
  hi[0] = rout, hi[1] = rout, hi[2] = halfz;
  if (dphi == kTwoPi) return;
  const double Rin     = 0.5 * (rout + rin);
  const bool phi0out   = !wedge_contains(w, Rin, 0);
  const bool phi90out  = !wedge_contains(w, 0, Rin);
  const bool phi180out = !wedge_contains(w, -Rin, 0);
  const bool phi270out = !wedge_contains(w, 0, -Rin);
  if (!(phi0out || phi90out || phi180out || phi270out)) return;
  const double Cx = rout * std::cos(sphi), Dx = rout * std::cos(sphi + dphi);
  const double Cy = rout * std::sin(sphi), Dy = rout * std::sin(sphi + dphi);
  auto mx = [](double a, double b) { return a > b ? a : b; };
  auto mn = [](double a, double b) { return a < b ? a : b; };
  if (phi0out) hi[0] = mx(Cx, Dx);
  if (phi90out) hi[1] = mx(Cy, Dy);
  if (phi180out) lo[0] = mn(Cx, Dx);
  if (phi270out) lo[1] = mn(Cy, Dy);
  if (dphi >= kPi) return;
  const double Ax = rin * std::cos(sphi), Bx = rin * std::cos(sphi + dphi);
  const double Ay = rin * std::sin(sphi), By = rin * std::sin(sphi + dphi);
  double t;
  t     = mx(Ax, Bx);
  hi[0] = t > hi[0] ? t : hi[0];
  t     = mx(Ay, By);
  hi[1] = t > hi[1] ? t : hi[1];
  t     = mn(Ax, Bx);
  lo[0] = t < lo[0] ? t : lo[0];
  t     = mn(Ay, By);
  lo[1] = t < lo[1] ? t : lo[1];
}
double nonzero(double x) { return x + std::copysign(1.0e-30, x); }
} // namespace

void make_box(const double *p, HostShape &s)
{
  BoxRec b{p[0], p[1], p[2]};
  s.type = kShapeBox;
  pack(s, b);
  for (int i = 0; i < 3; ++i) s.lo[i] = -p[i], s.hi[i] = p[i];
}

// TubeStruct constructor + CalculateCached (VecGeom/volumes/TubeStruct.h:41-179)
void make_tube(const double *p, HostShape &s)
{
  TubeRec t;
  t.rmin      = p[0] < 0.0 ? 0.0 : p[0];
  t.rmax      = p[1];
  t.z         = p[2];
  t.sphi      = p[3];
  t.dphi      = p[4];
  t.tolIz     = t.z - kHalfTolerance;
  t.tolOz     = t.z + kHalfTolerance;
  t.rmin2     = t.rmin * t.rmin;
  t.tolOrmin  = t.rmin - kHalfTolerance;
  t.tolIrmin  = t.rmin + kHalfTolerance;
  t.tolOrmin2 = t.tolOrmin * t.tolOrmin;
  t.tolIrmin2 = t.tolIrmin * t.tolIrmin;
  t.rmax2     = t.rmax * t.rmax;
  t.tolOrmax  = t.rmax + kHalfTolerance;
  t.tolIrmax  = t.rmax - kHalfTolerance;
  t.tolOrmax2 = t.tolOrmax * t.tolOrmax;
  t.tolIrmax2 = t.tolIrmax * t.tolIrmax;
  t.a1x       = std::cos(t.sphi);
  t.a1y       = std::sin(t.sphi);
  t.a2x       = std::cos(t.sphi + t.dphi);
  t.a2y       = std::sin(t.sphi + t.dphi);
  t.maxVal    = t.rmax > t.z ? t.rmax : t.z;
  t.w         = make_wedge(p[4], p[3]);
  s.type      = kShapeTube;
  pack(s, t);
  phi_section_extent(t.w, t.sphi, t.dphi, t.rmin, t.rmax, t.z, s.lo, s.hi);
}

// CutTubeStruct constructor (CutTubeStruct.h:38-49) with CutPlanes::Set / Plane::Set
// (Plane.h:40-49), UnplacedCutTube's normal check (UnplacedCutTube.h:36-50) and Extent
// (source/UnplacedCutTube.cpp:128-172).
bool make_cut_tube(const double *p, HostShape &s, std::string &err)
{
  const double rmin = p[0], rmax = p[1], z = p[2], sphi = p[3], dphi = p[4];
  if (!(p[7] < 0) || !(p[10] > 0)) {
    err = "illegal normal direction for cut planes (bottom z must be < 0, top z > 0)";
    return false;
  }
  CutTubeRec c{};
  const double tp[5] = {rmin, rmax, kInfLength, sphi, dphi};
  HostShape ts;
  make_tube(tp, ts);
  std::memcpy(&c.t, ts.rec.data(), sizeof(TubeRec));
  auto set_plane = [](const double *nin, double oz, double *n, double &d) {
    // Vector3D::Unit (Vector3D.h:284-290), then Plane::Set: zero components below
    // kTolerance and normalise again
    const double m2 = nin[0] * nin[0] + nin[1] * nin[1] + nin[2] * nin[2];
    const double s  = std::sqrt(m2 + kMinimum);
    double v[3]     = {nin[0] / s, nin[1] / s, nin[2] / s};
    for (double &x : v)
      if (std::fabs(x) < kTolerance) x = 0.0;
    const double inv = 1. / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) n[k] = inv * v[k];
    d = inv * -(v[0] * 0. + v[1] * 0. + v[2] * oz);
  };
  double n0[3], n1[3];
  set_plane(p + 5, -z, n0, c.d0);
  set_plane(p + 8, z, n1, c.d1);
  c.n0x = n0[0], c.n0y = n0[1], c.n0z = n0[2], c.n1x = n1[0], c.n1y = n1[1], c.n1z = n1[2];
  c.dz     = z;
  c.maxVal = rmax > z ? rmax : z;
  s.type   = kShapeCutTube;
  pack(s, c);
  // Extent
  const double cp1 = std::cos(sphi), sp1 = std::sin(sphi), cp2 = std::cos(sphi + dphi), sp2 = std::sin(sphi + dphi);
  auto zTop = [&](double r, double ph) { return z - (r / n1[2]) * (n1[0] * std::cos(ph) + n1[1] * std::sin(ph)); };
  auto zBot = [&](double r, double ph) { return -z - (r / n0[2]) * (n0[0] * std::cos(ph) + n0[1] * std::sin(ph)); };
  const double dztop    = rmax * std::sqrt(1. - n1[2] * n1[2]) / n1[2];
  const double dzbottom = -rmax * std::sqrt(1. - n0[2] * n0[2]) / n0[2];
  s.lo[0] = -rmax, s.lo[1] = -rmax, s.lo[2] = -z - dzbottom;
  s.hi[0] = rmax, s.hi[1] = rmax, s.hi[2] = z + dztop;
  if (dphi == kTwoPi) return true;
  auto mx = [](double a, double b) { return a > b ? a : b; };
  auto mn = [](double a, double b) { return a < b ? a : b; };
  auto contains = [&](double x, double y) { return wedge_contains(c.t.w, x, y); };
  if (!contains(-n1[0], -n1[1]))
    s.hi[2] = mx(mx(zTop(rmax, sphi), zTop(rmax, sphi + dphi)), mx(zTop(rmin, sphi), zTop(rmin, sphi + dphi)));
  if (!contains(-n0[0], -n0[1]))
    s.lo[2] = mn(mn(zBot(rmax, sphi), zBot(rmax, sphi + dphi)), mn(zBot(rmin, sphi), zBot(rmin, sphi + dphi)));
  if (!contains(1., 0.)) s.hi[0] = mx(mx(rmax * cp1, rmax * cp2), mx(rmin * cp1, rmin * cp2));
  if (!contains(-1., 0.)) s.lo[0] = mn(mn(rmax * cp1, rmax * cp2), mn(rmin * cp1, rmin * cp2));
  if (!contains(0., 1.)) s.hi[1] = mx(mx(rmax * sp1, rmax * sp2), mx(rmin * sp1, rmin * sp2));
  if (!contains(0., -1.)) s.lo[1] = mn(mn(rmax * sp1, rmax * sp2), mn(rmin * sp1, rmin * sp2));
  return true;
}

// GenTrapStruct::Initialize (GenTrapStruct.h) and SecondOrderSurfaceShell<4>::Initialize
// (SecondOrderSurfaceShell.h). The record is the object the reference's device holds:
// UnplacedGenTrap::CopyToGpu (source/UnplacedGenTrap.cpp:343-357) builds it again from the
// host's vertices, which Initialize has already put in clockwise order. The shapes the
// reference's Initialize reports as errors (and keeps half-built) are rejected here.
bool make_gentrap(const double *p, HostShape &s, std::string &err)
{
  double vx[8], vy[8];
  for (int i = 0; i < 8; ++i) vx[i] = p[i], vy[i] = p[8 + i];
  const double dz = p[16];
  if (!(dz > 0.)) {
    err = "Half-length of generic trapezoid must be positive";
    return false;
  }
  // orientation: signed doubled areas of both bases, accumulated edge by edge
  double sum1 = 0., sum2 = 0.;
  for (int i = 0; i < 4; ++i) {
    const int j = (i + 1) % 4;
    sum1 += vx[i] * vy[j] - vx[j] * vy[i];
    sum2 += vx[i + 4] * vy[j + 4] - vx[j + 4] * vy[i + 4];
  }
  if (sum1 * sum2 < -kTolerance) {
    err = "generic trap defined with opposite clockwise";
    return false;
  }
  if (sum1 > kTolerance) { // anticlockwise: swap vertices 1 <-> 3 and 5 <-> 7
    std::swap(vx[1], vx[3]), std::swap(vy[1], vy[3]);
    std::swap(vx[5], vx[7]), std::swap(vy[5], vy[7]);
  }
  GenTrapRec r{};
  for (int i = 0; i < 8; ++i) r.vx[i] = vx[i], r.vy[i] = vy[i];
  for (int i = 0; i < 4; ++i) {
    const int j     = (i + 1) % 4;
    r.deltax[i]     = vx[j] - vx[i];
    r.deltax[i + 4] = vx[j + 4] - vx[i + 4];
    r.deltay[i]     = vy[j] - vy[i];
    r.deltay[i + 4] = vy[j + 4] - vy[i + 4];
  }
  // SegmentsCrossing on the z = -dz / +dz vertices: both parameters strictly inside (0, 1)
  auto crossing = [&](int a, int a1, int b, int b1) {
    const double za = a < 4 ? -dz : dz, zb = b < 4 ? -dz : dz;
    const double r0 = vx[a1] - vx[a], r1 = vy[a1] - vy[a], r2 = (a1 < 4 ? -dz : dz) - za;
    const double s0 = vx[b1] - vx[b], s1 = vy[b1] - vy[b], s2 = (b1 < 4 ? -dz : dz) - zb;
    const double c0 = r1 * s2 - r2 * s1, c1 = r2 * s0 - r0 * s2, c2 = r0 * s1 - r1 * s0;
    if (c0 * c0 + c1 * c1 + c2 * c2 < kTolerance) return false;
    const double q0 = vx[b] - vx[a], q1 = vy[b] - vy[a];
    const double t  = (q0 * s1 - q1 * s0) / c2;
    if (t < kTolerance || t > 1. - kTolerance) return false;
    const double u = (q0 * r1 - q1 * r0) / c2;
    if (u < kTolerance || u > 1. - kTolerance) return false;
    return true;
  };
  if (crossing(0, 1, 3, 2) || crossing(1, 2, 0, 3) || crossing(4, 5, 7, 6) || crossing(5, 6, 4, 7)) {
    err = "generic trap defined with crossing opposite segments";
    return false;
  }
  for (int i = 0; i < 4; ++i) { // ComputeIsConvexQuadrilaterals
    const int j = (i + 1) % 4;
    if (r.deltax[i] * r.deltay[j] - r.deltay[i] * r.deltax[j] > kTolerance ||
        r.deltax[i + 4] * r.deltay[j + 4] - r.deltay[i + 4] * r.deltax[j + 4] > kTolerance) {
      err = "generic trap defined with top/bottom quadrilaterals not convex";
      return false;
    }
  }
  r.dz = dz, r.invDz = 1. / dz, r.halfInvDz = 0.5 / dz, r.dz2 = 0.5 / dz;
  auto cross3 = [](const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  for (int i = 0; i < 4; ++i) {
    const int j   = (i + 1) % 4;
    r.connx[i]    = vx[i] - vx[i + 4];
    r.conny[i]    = vy[i] - vy[i + 4];
    const bool dg = std::fabs(vx[i] - vx[j]) < kTolerance && std::fabs(vy[i] - vy[j]) < kTolerance &&
                    std::fabs(vx[i + 4] - vx[j + 4]) < kTolerance && std::fabs(vy[i + 4] - vy[j + 4]) < kTolerance;
    if (dg) r.degenerated |= 1LL << i;
    const double xa = vx[i], ya = vy[i], xb = vx[i + 4], yb = vy[i + 4];
    const double xc = vx[j], yc = vy[j], xd = vx[j + 4], yd = vy[j + 4];
    r.tx1[i]       = r.dz2 * (xb - xa);
    r.ty1[i]       = r.dz2 * (yb - ya);
    r.tx2[i]       = r.dz2 * (xd - xc);
    r.ty2[i]       = r.dz2 * (yd - yc);
    r.t1crosst2[i] = r.tx1[i] * r.ty2[i] - r.tx2[i] * r.ty1[i];
    r.deltatx[i]   = r.tx2[i] - r.tx1[i];
    r.deltaty[i]   = r.ty2[i] - r.ty1[i];
    // vi = b - a, hi0 = c - a, vj = d - c, hi1 = d - b (z components from +-dz)
    const double vi[3] = {xb - xa, yb - ya, dz - (-dz)}, hi0[3] = {xc - xa, yc - ya, -dz - (-dz)};
    const double vj[3] = {xd - xc, yd - yc, dz - (-dz)}, hi1[3] = {xd - xb, yd - yb, dz - dz};
    double n[3];
    cross3(vi, hi0, n);
    if (n[0] * n[0] + n[1] * n[1] + n[2] * n[2] < kTolerance) {
      cross3(vi, hi1, n);
      if (n[0] * n[0] + n[1] * n[1] + n[2] * n[2] < kTolerance) n[0] = 0., n[1] = 0., n[2] = 1.;
    }
    const double inv = 1. / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) r.normal[i][k] = n[k] * inv;
    cross3(vi, hi0, r.viCrossHi0[i]);
    cross3(vi, vj, r.viCrossVj[i]);
    cross3(hi1, hi0, r.hi1CrossHi0[i]);
    const bool flat = (std::fabs(xc - xa) < kTolerance && std::fabs(yc - ya) < kTolerance) ||
                      (std::fabs(xd - xb) < kTolerance && std::fabs(yd - yb) < kTolerance) ||
                      std::fabs((xc - xa) * (yd - yb) - (xd - xb) * (yc - ya)) < kTolerance;
    if (!flat) r.curved |= 1LL << i;
  }
  r.planar = r.curved == 0;
  // GenTrapStruct::Extent over the eight vertices, then ComputeBoundingBox
  double lo[3] = {vx[0], vy[0], -dz}, hi[3] = {vx[0], vy[0], dz};
  for (int i = 0; i < 8; ++i) {
    if (lo[0] > vx[i]) lo[0] = vx[i];
    if (hi[0] < vx[i]) hi[0] = vx[i];
    if (lo[1] > vy[i]) lo[1] = vy[i];
    if (hi[1] < vy[i]) hi[1] = vy[i];
  }
  for (int k = 0; k < 3; ++k) {
    r.bborig[k] = 0.5 * (lo[k] + hi[k]);
    r.bbdim[k]  = 0.5 * (hi[k] - lo[k]);
    s.lo[k] = lo[k], s.hi[k] = hi[k];
  }
  s.type = kShapeGenTrap;
  pack(s, r);
  return true;
}

// HypeStruct::CalculateCached (VecGeom/volumes/HypeStruct.h:49-75) and UnplacedHype::Extent
// (source/UnplacedHype.cpp:94-100).
void make_hype(const double *p, HostShape &s)
{
  HypeRec h{};
  h.rmin = p[0], h.rmax = p[1], h.stIn = p[2], h.stOut = p[3], h.dz = p[4];
  h.tIn             = std::tan(h.stIn);
  h.tOut            = std::tan(h.stOut);
  h.tIn2            = h.tIn * h.tIn;
  h.tOut2           = h.tOut * h.tOut;
  h.rmin2           = h.rmin * h.rmin;
  h.rmax2           = h.rmax * h.rmax;
  h.dz2             = h.dz * h.dz;
  h.endInnerRadius2 = h.tIn2 * h.dz2 + h.rmin2;
  h.endOuterRadius2 = h.tOut2 * h.dz2 + h.rmax2;
  h.endInnerRadius  = std::sqrt(h.endInnerRadius2);
  h.endOuterRadius  = std::sqrt(h.endOuterRadius2);
  h.zTol            = kTolerance * h.dz;
  h.innerTol        = kTolerance * h.endInnerRadius;
  h.outerTol        = kTolerance * h.endOuterRadius;
  h.inner           = (h.rmin > 0. || h.stIn != 0.) ? 1. : 0.;
  s.type            = kShapeHype;
  pack(s, h);
  const double r = h.endOuterRadius;
  s.lo[0] = -r, s.lo[1] = -r, s.lo[2] = -h.dz;
  s.hi[0] = r, s.hi[1] = r, s.hi[2] = h.dz;
}

// SphereStruct constructor (SphereStruct.h:256-276: CheckPhiAngles :160-170 / :126-158,
// CheckThetaAngles :96-124), ThetaCone constructor (ThetaCone_Evolution.h:44-69) and
// UnplacedSphere::Extent (source/UnplacedSphere.cpp:74-160).
void make_sphere(const double *p, HostShape &s)
{
  const double pRmin = p[0], pRmax = p[1], pSPhi = p[2], pDPhi = p[3], pSTheta = p[4], pDTheta = p[5];
  SphereRec r{};
  r.rmin = pRmin, r.rmax = pRmax, r.sphi = pSPhi, r.dphi = pDPhi, r.stheta = pSTheta, r.dtheta = pDTheta;
  bool fullPhi               = true;
  const double kAngTolerance = 1e-9;
  if (pDPhi >= 2 * kPi - kAngTolerance * 0.5) {
    r.dphi = 2 * kPi, r.sphi = 0, fullPhi = true;
  } else {
    fullPhi = false;
    if (pDPhi > 0) r.dphi = pDPhi;
  }
  if (!fullPhi) {
    r.sphi = (pSPhi < 0) ? 2 * kPi - std::fmod(std::fabs(pSPhi), 2 * kPi) : std::fmod(pSPhi, 2 * kPi);
    if (r.sphi + r.dphi > 2 * kPi) r.sphi -= 2 * kPi;
  }
  if (!((pSTheta < 0) || (pSTheta > kPi))) r.stheta = pSTheta;
  if (pDTheta + pSTheta >= kPi)
    r.dtheta = kPi - pSTheta;
  else if (pDTheta > 0)
    r.dtheta = pDTheta;
  const bool fullTheta = !(r.dtheta - r.stheta < kPi);
  r.fullPhi = fullPhi ? 1. : 0., r.fullTheta = fullTheta ? 1. : 0., r.fullSphere = (fullPhi && fullTheta) ? 1. : 0.;
  r.eTheta = r.stheta + r.dtheta;
  r.w      = make_wedge(pDPhi, pSPhi);
  // the theta cone from the raw angles
  r.tcS = pSTheta, r.tcE = pSTheta + pDTheta;
  double ts = r.tcS, te = r.tcE;
  if (r.tcS > kPi / 2) ts = kPi - r.tcS;
  if (r.tcE > kPi / 2) te = kPi - r.tcE;
  r.tanS   = std::tan(ts);
  r.tanS2  = r.tanS * r.tanS;
  r.tanE   = std::tan(te);
  r.tanE2  = r.tanE * r.tanE;
  r.tanBis = std::tan(ts + (pDTheta / 2));
  if (r.tcS > kPi / 2 && r.tcE > kPi / 2) r.tanBis = std::tan(ts - (pDTheta / 2));
  r.slope1 = std::tan(kPi / 2 - r.tcS);
  r.slope2 = std::tan(kPi / 2 - r.tcE);
  s.type   = kShapeSphere;
  pack(s, r);
  // Extent
  const double rmax = r.rmax, rmin = r.rmin;
  for (int k = 0; k < 3; ++k) s.lo[k] = -rmax, s.hi[k] = rmax;
  const double eTheta = r.stheta + r.dtheta;
  if (fullPhi && fullTheta) return;
  double st1 = 0., st2 = 0.;
  auto mx = [](double a, double b) { return a > b ? a : b; };
  auto mn = [](double a, double b) { return a < b ? a : b; };
  if (!fullTheta) {
    s.hi[2] = ((r.stheta <= kPi / 2.) ? rmax : rmin) * std::cos(r.stheta);
    s.lo[2] = ((eTheta <= kPi / 2.) ? rmin : rmax) * std::cos(eTheta);
    st1     = std::sin(r.stheta);
    st2     = std::sin(r.eTheta);
    if (r.stheta <= kPi / 2.) {
      if (eTheta < kPi / 2.) s.hi[0] = rmax * st2, s.lo[0] = -rmax * st2, s.hi[1] = rmax * st2, s.lo[1] = -rmax * st2;
    } else {
      s.hi[0] = rmax * st1, s.lo[0] = -rmax * st1, s.hi[1] = rmax * st1, s.lo[1] = -rmax * st1;
    }
  }
  if (!fullPhi) {
    double Rmax = rmax;
    if (r.stheta > kPi / 2.) Rmax *= st1;
    if (eTheta < kPi / 2.) Rmax *= st2;
    const double Rmin    = rmin * mn(st1, st2);
    const double Rin     = 0.5 * (Rmax + Rmin);
    const bool phi0out   = !wedge_contains(r.w, Rin, 0), phi90out = !wedge_contains(r.w, 0, Rin);
    const bool phi180out = !wedge_contains(r.w, -Rin, 0), phi270out = !wedge_contains(r.w, 0, -Rin);
    if (!(phi0out || phi90out || phi180out || phi270out)) return;
    const double Cx = Rmax * std::cos(r.sphi), Dx = Rmax * std::cos(r.sphi + r.dphi);
    const double Cy = Rmax * std::sin(r.sphi), Dy = Rmax * std::sin(r.sphi + r.dphi);
    if (phi0out) s.hi[0] = mx(Cx, Dx);
    if (phi90out) s.hi[1] = mx(Cy, Dy);
    if (phi180out) s.lo[0] = mn(Cx, Dx);
    if (phi270out) s.lo[1] = mn(Cy, Dy);
    if (r.dphi >= kPi) return;
    const double Ax = Rmin * std::cos(r.sphi), Bx = Rmin * std::cos(r.sphi + r.dphi);
    const double Ay = Rmin * std::sin(r.sphi), By = Rmin * std::sin(r.sphi + r.dphi);
    double t;
    t = mx(Ax, Bx), s.hi[0] = t > s.hi[0] ? t : s.hi[0];
    t = mx(Ay, By), s.hi[1] = t > s.hi[1] ? t : s.hi[1];
    t = mn(Ax, Bx), s.lo[0] = t < s.lo[0] ? t : s.lo[0];
    t = mn(Ay, By), s.lo[1] = t < s.lo[1] ? t : s.lo[1];
  }
}

// ConeStruct constructor, SetAndCheck{D,S}PhiAngle and CalculateCached (ConeStruct.h:85-336)
void make_cone(const double *p, HostShape &s)
{
  ConeRec c;
  c.rmin1  = p[0] < 0.0 ? 0.0 : p[0];
  c.rmax1  = p[1];
  c.rmin2  = p[2] < 0.0 ? 0.0 : p[2];
  c.rmax2  = p[3];
  c.dz     = p[4];
  c.sphi   = p[5];
  c.dphi   = p[6];
  c.frmin1 = p[0], c.frmax1 = p[1], c.frmin2 = p[2], c.frmax2 = p[3];
  c.w      = make_wedge(p[6], p[5]); // the wedge keeps its construction angles
  const double dPhi = p[6], sPhi = p[5];
  if (dPhi >= kTwoPi - 0.5 * kAngTolerance) {
    c.dphi = kTwoPi;
    c.sphi = 0;
  } else if (dPhi > 0) {
    c.dphi = dPhi;
  }
  c.w.dphi = c.dphi;
  c.sphi   = sPhi < 0 ? kTwoPi - std::fmod(std::fabs(sPhi), kTwoPi) : std::fmod(sPhi, kTwoPi);
  if (c.sphi + c.dphi > kTwoPi) c.sphi -= kTwoPi;
  c.a1x = std::cos(c.sphi);
  c.a1y = std::sin(c.sphi);
  c.a2x = std::cos(c.sphi + c.dphi);
  c.a2y = std::sin(c.sphi + c.dphi);

  c.origRmax1 = c.rmax1;
  c.origRmax2 = c.rmax2;
  if (c.rmin1 == c.rmax1) c.rmax1 += kConeTolerance;
  if (c.rmin2 == c.rmax2) c.rmax2 += kConeTolerance;
  c.sqRmin1    = c.rmin1 * c.rmin1;
  c.sqRmax1    = c.rmax1 * c.rmax1;
  c.sqRmin2    = c.rmin2 * c.rmin2;
  c.sqRmax2    = c.rmax2 * c.rmax2;
  c.tanRMin    = (c.rmin2 - c.rmin1) * 0.5 / c.dz;
  c.secRMin    = std::sqrt(1.0 + c.tanRMin * c.tanRMin);
  c.invSecRMin = 1. / nonzero(c.secRMin);
  c.tanRMax    = (c.rmax2 - c.rmax1) * 0.5 / c.dz;
  c.secRMax    = std::sqrt(1.0 + c.tanRMax * c.tanRMax);
  c.invSecRMax = 1. / nonzero(c.secRMax);
  c.innerSlope  = -(c.rmin1 - c.rmin2) / (2. * c.dz);
  c.outerSlope  = -(c.rmax1 - c.rmax2) / (2. * c.dz);
  c.innerOffset = c.rmin2 - c.innerSlope * c.dz;
  c.outerOffset = c.rmax2 - c.outerSlope * c.dz;
  c.innerTol    = kConeTolerance * c.secRMin;
  c.outerTol    = kConeTolerance * c.secRMax;
  if (c.rmin2 > c.rmin1) {
    c.innerApex    = 2 * c.dz * c.rmin1 / (c.rmin2 - c.rmin1);
    c.tanInnerApex = c.rmin2 / (2 * c.dz + c.innerApex);
  } else {
    c.innerApex    = 2 * c.dz * c.rmin2 / nonzero(c.rmin1 - c.rmin2);
    c.tanInnerApex = c.rmin1 / (2 * c.dz + c.innerApex);
  }
  if (c.rmin1 == 0. || c.rmin2 == 0.) c.innerApex = 0.;
  if (c.rmin1 == 0.) c.tanInnerApex = c.rmin2 / (2 * c.dz);
  if (c.rmin2 == 0.) c.tanInnerApex = c.rmin1 / (2 * c.dz);
  if (c.rmax2 > c.rmax1) {
    c.outerApex    = 2 * c.dz * c.rmax1 / (c.rmax2 - c.rmax1);
    c.tanOuterApex = c.rmax2 / (2 * c.dz + c.outerApex);
  } else {
    c.outerApex    = 2 * c.dz * c.rmax2 / nonzero(c.rmax1 - c.rmax2);
    c.tanOuterApex = c.rmax1 / (2 * c.dz + c.outerApex);
  }
  if (c.rmax1 == 0. || c.rmax2 == 0.) c.outerApex = 0.;
  if (c.rmax1 == 0.) c.tanOuterApex = c.rmax2 / (2 * c.dz);
  if (c.rmax2 == 0.) c.tanOuterApex = c.rmax1 / (2 * c.dz);
  c.zNormInner = c.tanRMin / nonzero(c.secRMin);
  c.zNormOuter = -c.tanRMax / nonzero(c.secRMax);
  c.tolIz      = c.dz - kHalfTolerance;
  c.tolOz      = c.dz + kHalfTolerance;
  s.type       = kShapeCone;
  pack(s, c);
  const double rout = c.frmax1 > c.frmax2 ? c.frmax1 : c.frmax2;
  const double rin  = c.frmin1 > c.frmin2 ? c.frmin2 : c.frmin1;
  phi_section_extent(c.w, c.sphi, c.dphi, rin, rout, c.dz, s.lo, s.hi);
}

// TrdStruct.h:68-86 CalculateCached (the y tolerance uses the x extent, as the reference does)
void make_trd(const double *p, HostShape &s)
{
  TrdRec t{};
  t.dx1 = p[0], t.dx2 = p[1], t.dy1 = p[2], t.dy2 = p[3], t.dz = p[4];
  t.x2minusx1    = t.dx2 - t.dx1;
  t.y2minusy1    = t.dy2 - t.dy1;
  t.halfx1plusx2 = 0.5 * (t.dx1 + t.dx2);
  t.halfy1plusy2 = 0.5 * (t.dy1 + t.dy2);
  t.fx           = 0.5 * (t.dx1 - t.dx2) / t.dz;
  t.fy           = 0.5 * (t.dy1 - t.dy2) / t.dz;
  t.calfx        = 1. / std::sqrt(1.0 + t.fx * t.fx);
  t.calfy        = 1. / std::sqrt(1.0 + t.fy * t.fy);
  t.tolx         = kTolerance * std::sqrt(t.x2minusx1 * t.x2minusx1 + 4 * t.dz * t.dz);
  t.toly         = kTolerance * std::sqrt(t.x2minusx1 * t.x2minusx1 + 4 * t.dz * t.dz);
  s.type         = kShapeTrd;
  pack(s, t);
  const double mx = t.dx1 > t.dx2 ? t.dx1 : t.dx2, my = t.dy1 > t.dy2 ? t.dy1 : t.dy2;
  s.lo[0] = -mx, s.lo[1] = -my, s.lo[2] = -t.dz;
  s.hi[0] = mx, s.hi[1] = my, s.hi[2] = t.dz;
}

// Trapezoid: the side planes as given (dz + TrapezoidStruct::GetPlane(0..3)), or from the eight
// corners, either given (UnplacedTrapezoid.cpp:496-524,
// dz from the last corner) or made from the 11 parameters (UnplacedTrapezoid.h:56-64: tan of
// alpha1/alpha2; TrapezoidStruct.h CalculateCached: tan(theta) cos(phi), tan(theta) sin(phi);
// UnplacedTrapezoid.cpp:447-466 FromParametersToCorners). Planes: UnplacedTrapezoid.cpp:630-679
// (faces 0154 -Y, 2673 +Y, 0462 -X, 1375 +X), each by MakeAPlane (:569-620): n = (p3 - p1) x
// (p4 - p2) times 1/|n|, d = -n . ((p1 + p2 + p3 + p4) 0.25). Extent: UnplacedTrapezoid.cpp:
// 298-337 on the corners re-derived from the planes (:468-494 fromPlanesToCorners).
bool make_trap(const double *p, int np, HostShape &s, std::string &err)
{
  double pt[8][3];
  TrapRec t{};
  if (np == 17) { // dz, then (a, b, c, d) of the planes -Y, +Y, -X, +X as the reference holds them
    t.dz = p[0];
    for (int i = 0; i < 4; ++i) t.a[i] = p[1 + 4 * i], t.b[i] = p[2 + 4 * i], t.c[i] = p[3 + 4 * i], t.d[i] = p[4 + 4 * i];
  } else if (np == 24) {
    for (int k = 0; k < 8; ++k)
      for (int j = 0; j < 3; ++j) pt[k][j] = p[3 * k + j];
    t.dz = pt[7][2];
  } else if (np == 11) {
    const double dz = p[0], dy1 = p[3], dx1 = p[4], dx2 = p[5], dy2 = p[7], dx3 = p[8], dx4 = p[9];
    const double ta1 = std::tan(p[6]), ta2 = std::tan(p[10]);
    const double tcp = std::tan(p[1]) * std::cos(p[2]), tsp = std::tan(p[1]) * std::sin(p[2]);
    const double a1 = ta1 * dy1, a2 = ta2 * dy2, xz = tcp * dz, yz = tsp * dz;
    const double c[8][3] = {{-xz - a1 - dx1, -yz - dy1, -dz}, {-xz - a1 + dx1, -yz - dy1, -dz},
                            {-xz + a1 - dx2, -yz + dy1, -dz}, {-xz + a1 + dx2, -yz + dy1, -dz},
                            {+xz - a2 - dx3, +yz - dy2, +dz}, {+xz - a2 + dx3, +yz - dy2, +dz},
                            {+xz + a2 - dx4, +yz + dy2, +dz}, {+xz + a2 + dx4, +yz + dy2, +dz}};
    std::memcpy(pt, c, sizeof(pt));
    t.dz = dz;
  } else {
    err = "a trapezoid takes 11 parameters, 8 corners (24 values) or dz and 4 planes (17 values)";
    return false;
  }
  static const int face[4][4] = {{0, 1, 5, 4}, {2, 6, 7, 3}, {0, 4, 6, 2}, {1, 3, 7, 5}};
  for (int i = 0; i < 4 && np != 17; ++i) {
    const double *p1 = pt[face[i][0]], *p2 = pt[face[i][1]], *p3 = pt[face[i][2]], *p4 = pt[face[i][3]];
    const double u[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
    const double v[3] = {p4[0] - p2[0], p4[1] - p2[1], p4[2] - p2[2]};
    double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    const double inv = 1. / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (double &x : n) x = x * inv;
    double c[3];
    for (int j = 0; j < 3; ++j) c[j] = 0.25 * (((p1[j] + p2[j]) + p3[j]) + p4[j]);
    t.a[i] = n[0], t.b[i] = n[1], t.c[i] = n[2];
    t.d[i] = -(n[0] * c[0] + n[1] * c[1] + n[2] * c[2]);
  }
  if (!(t.dz > 0.) || !std::isfinite(t.dz)) {
    err = "trapezoid half length must be positive";
    return false;
  }
  t.dz_plus  = t.dz + kHalfTolerance;
  t.dz_minus = t.dz - kHalfTolerance;
  s.type     = kShapeTrap;
  pack(s, t);
  const double z = t.dz;
  double x[8], y[8];
  for (int k = 0; k < 8; ++k) {
    const int yp = (k >> 1) & 1, xp = 2 + (k & 1);
    const double sz = (k < 4) ? -z : z;
    y[k] = -(t.d[yp] + sz * t.c[yp]) / t.b[yp];
    x[k] = ((t.b[xp] / t.b[yp]) * (t.d[yp] + sz * t.c[yp]) - (t.d[xp] + sz * t.c[xp])) / t.a[xp];
  }
  auto mx = [](const double *v) {
    auto M = [](double a, double b) { return a > b ? a : b; };
    return M(M(M(v[0], v[1]), M(v[2], v[3])), M(M(v[4], v[5]), M(v[6], v[7])));
  };
  auto mn = [](const double *v) {
    auto M = [](double a, double b) { return a < b ? a : b; };
    return M(M(M(v[0], v[1]), M(v[2], v[3])), M(M(v[4], v[5]), M(v[6], v[7])));
  };
  s.lo[0] = mn(x), s.lo[1] = mn(y), s.lo[2] = -z;
  s.hi[0] = mx(x), s.hi[1] = mx(y), s.hi[2] = z;
  return true;
}

// PolyconeStruct.h:124-239 Init: one ConeStruct(prevRmin, prevRmax, rMin, rMax, dz, phiStart,
// phiTotal) per z interval longer than kTolerance, shifted to the interval's middle.
bool make_polycone(const double *p, int np, HostShape &s, std::string &err)
{
  const double phiStart = p[0], phiTotal = p[1];
  const int nz = (int)p[2];
  if (nz < 2 || np < 3 + 3 * nz) {
    err = "polycone needs at least 2 z planes";
    return false;
  }
  const double *zPlane = p + 3, *rInner = p + 3 + nz, *rOuter = p + 3 + 2 * nz;
  std::vector<double> z(zPlane, zPlane + nz), rin(rInner, rInner + nz), rout(rOuter, rOuter + nz);
  if (zPlane[0] > zPlane[nz - 1])
    for (int i = 0; i < nz; ++i) z[i] = zPlane[nz - 1 - i], rin[i] = rInner[nz - 1 - i], rout[i] = rOuter[nz - 1 - i];
  double deltaPhi = 0, startPhi = 0;
  if (phiTotal <= 0. || phiTotal > kTwoPi - kTolerance) {
    startPhi = 0;
    deltaPhi = kTwoPi;
  } else {
    deltaPhi = phiTotal;
    startPhi = phiStart;
    while (startPhi < 0) startPhi += kTwoPi;
  }
  std::vector<double> zs, shifts;
  std::vector<HostShape> cones;
  double prevZ = z[0], prevRmax = 0, prevRmin = 0;
  const int dirZ = z[1] < z[0] ? -1 : 1;
  double maxR = 0, minR = kInfLength;
  for (int i = 0; i < nz; ++i) {
    if (i > 0) {
      if (((z[i] > prevZ + kTolerance) && dirZ > 0) || ((z[i] < prevZ - kTolerance) && dirZ < 0)) {
        const double cp[7] = {prevRmin, prevRmax, rin[i], rout[i], (z[i] - prevZ) / 2, phiStart, phiTotal};
        HostShape c;
        make_cone(cp, c);
        cones.push_back(std::move(c));
        zs.push_back(z[i]);
        const size_t zi = zs.size() - 1;
        shifts.push_back(zs[zi - 1] + 0.5 * (zs[zi] - zs[zi - 1]));
        const ConeRec &cr = *reinterpret_cast<const ConeRec *>(cones.back().rec.data());
        maxR = std::max(maxR, std::max(cr.frmax1, cr.frmax2));
        minR = std::min(minR, std::min(cr.frmin1, cr.frmin2));
      }
    } else {
      zs.push_back(z[i]);
    }
    prevZ = z[i], prevRmin = rin[i], prevRmax = rout[i];
  }
  const int nsec = (int)cones.size();
  if (nsec < 1) {
    err = "polycone has no section longer than the tolerance";
    return false;
  }
  const int base = polycone_section_base(nsec);
  std::vector<double> r(base + nsec * kPolyconeSectionDoubles, 0.);
  r[0] = nsec, r[1] = startPhi, r[2] = deltaPhi;
  for (int i = 0; i <= nsec; ++i) r[4 + i] = zs[i];
  for (int i = 0; i < nsec; ++i) {
    double *sec = r.data() + base + i * kPolyconeSectionDoubles;
    sec[0]      = shifts[i];
    std::memcpy(sec + 4, cones[i].rec.data(), sizeof(ConeRec));
    // the section's cylindrical shell (every radius the cone record holds), padded by
    // 4e-3 mm and rounded outward to FP32, for the mixed-precision screen
    const ConeRec &c  = *reinterpret_cast<const ConeRec *>(cones[i].rec.data());
    const double rlo  = std::min(std::min(c.rmin1, c.rmin2), std::min(c.frmin1, c.frmin2));
    const double rhi  = std::max(std::max(std::max(c.rmax1, c.rmax2), std::max(c.frmax1, c.frmax2)),
                                 std::max(c.origRmax1, c.origRmax2));
    const double pad  = 4e-3;
    auto down = [](double v) { const float f = (float)v; return (double)f > v ? std::nextafter(f, -INFINITY) : f; };
    auto up   = [](double v) { const float f = (float)v; return (double)f < v ? std::nextafter(f, INFINITY) : f; };
    const float shell[4] = {std::max(0.f, down(rlo - pad)), up(rhi + pad), down(shifts[i] - c.dz - pad),
                            up(shifts[i] + c.dz + pad)};
    std::memcpy(sec + 1, shell, sizeof(shell));
  }
  s.type = kShapePolycone;
  s.rec  = std::move(r);
  // source/UnplacedPolycone.cpp:865-902: xy extent of a Cone(minR, maxR, minR, maxR, 1, sphi, dphi)
  const double tp[7] = {minR, maxR, minR, maxR, 1, startPhi, deltaPhi};
  HostShape tmp;
  make_cone(tp, tmp);
  for (int k = 0; k < 2; ++k) s.lo[k] = tmp.lo[k], s.hi[k] = tmp.hi[k];
  s.lo[2] = zs[0] > zs[nsec] ? zs[nsec] : zs[0];
  s.hi[2] = zs[0] > zs[nsec] ? zs[0] : zs[nsec];
  return true;
}

// TorusStruct2.h:36-43; bounding tube from UnplacedTorus2.h:64-74
void make_torus2(const double *p, HostShape &s)
{
  TorusRec t{};
  t.rmin = p[0], t.rmax = p[1], t.rtor = p[2], t.sphi = p[3], t.dphi = p[4];
  t.rmin2 = t.rmin * t.rmin, t.rmax2 = t.rmax * t.rmax, t.rtor2 = t.rtor * t.rtor;
  t.w                = make_wedge(t.dphi, t.sphi);
  const double bp[5] = {t.rtor - t.rmax - kTolerance, t.rtor + t.rmax + kTolerance, t.rmax, t.sphi, t.dphi};
  HostShape bt;
  make_tube(bp, bt);
  std::memcpy(&t.bt, bt.rec.data(), sizeof(TubeRec));
  s.type = kShapeTorus2;
  pack(s, t);
  for (int k = 0; k < 3; ++k) s.lo[k] = bt.lo[k], s.hi[k] = bt.hi[k];
}

// ---------------------------------------------------------------- polyhedron
// Construction of PolyhedronStruct(phiStart, phiDelta, sideCount, zPlaneCount, zPlanes,
// rMin, rMax) + Initialize (VecGeom/volumes/PolyhedronStruct.h:112-125, 262-430), with
// the quadrilateral and plane setters of source/Quadrilaterals.cpp:44-123 and
// source/Planes.cpp:31-52, evaluated in the same order so the record is bit-identical.
namespace {
struct HV {
  double v[3];
  double operator[](int i) const { return v[i]; }
};
HV hv(double x, double y, double z) { return HV{{x, y, z}}; }
HV hsub(HV a, HV b) { return hv(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
double hdot(HV a, HV b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double hmag(HV a) { return std::sqrt(hdot(a, a)); }
HV hscale(HV a, double s) { return hv(a[0] * s, a[1] * s, a[2] * s); }
HV hcross(HV l, HV r) { return hv(l[1] * r[2] - l[2] * r[1], l[2] * r[0] - l[0] * r[2], l[0] * r[1] - l[1] * r[0]); }
HV hfix(HV a)
{
  for (int i = 0; i < 3; ++i)
    if (std::fabs(a.v[i]) < kTolerance) a.v[i] = 0.;
  return a;
}
HV hnormalized(HV a) { return hscale(a, 1. / hmag(a)); }
bool hsame(HV a, HV b)
{
  return std::fabs(a[0] - b[0]) < kTolerance && std::fabs(a[1] - b[1]) < kTolerance &&
         std::fabs(a[2] - b[2]) < kTolerance;
}
HV hcyl(double r, double phi, double z) { return hv(r * std::cos(phi), r * std::sin(phi), z); }
double normalize_angle(double a) { return a + kTwoPi * (double)((a < 0 ? 1 : 0) - (int)(a / kTwoPi)); }

// One quadrilateral (kPolyQuadDoubles doubles) from its four corners.
void set_quad(double *q, HV c0, HV c1, HV c2, HV c3)
{
  const HV cs[4] = {c0, c1, c2, c3};
  HV ch[4]       = {hv(0, 0, 0), hv(0, 0, 0), hv(0, 0, 0), hv(0, 0, 0)};
  ch[0]          = c0;
  int assigned = 1, tested = 1;
  while (tested < 4) {
    bool chosen = true;
    for (int j = 0; j < assigned; ++j)
      if (hsame(ch[j], cs[tested])) {
        chosen = false;
        break;
      }
    if (chosen) ch[assigned++] = cs[tested];
    ++tested;
  }
  const double a = ch[0][1] * (ch[1][2] - ch[2][2]) + ch[1][1] * (ch[2][2] - ch[0][2]) + ch[2][1] * (ch[0][2] - ch[1][2]);
  const double b = ch[0][2] * (ch[1][0] - ch[2][0]) + ch[1][2] * (ch[2][0] - ch[0][0]) + ch[2][2] * (ch[0][0] - ch[1][0]);
  const double c = ch[0][0] * (ch[1][1] - ch[2][1]) + ch[1][0] * (ch[2][1] - ch[0][1]) + ch[2][0] * (ch[0][1] - ch[1][1]);
  double d = -ch[0][0] * (ch[1][1] * ch[2][2] - ch[2][1] * ch[1][2]) - ch[1][0] * (ch[2][1] * ch[0][2] - ch[0][1] * ch[2][2]) -
             ch[2][0] * (ch[0][1] * ch[1][2] - ch[1][1] * ch[0][2]);
  HV n             = hv(a, b, c);
  const double inv = 1. / hmag(n);
  n                = hscale(n, inv);
  d *= inv;
  n = hfix(n);
  q[0] = n[0], q[1] = n[1], q[2] = n[2], q[3] = d;
  for (int j = 0; j < 4; ++j) {
    const HV a0 = cs[j], a1 = cs[(j + 1) % 4];
    double *sp  = q + 4 + 4 * j;
    if (!hsame(a1, a0)) {
      const HV sv     = hfix(hnormalized(hcross(n, hsub(a1, a0))));
      const double il = 1. / hmag(sv);
      sp[0] = il * sv[0], sp[1] = il * sv[1], sp[2] = il * sv[2];
      sp[3] = il * -hdot(sv, a0);
    } else {
      sp[0] = sp[1] = sp[2] = sp[3] = 0.;
    }
  }
  for (int k = 0; k < 4; ++k)
    for (int i = 0; i < 3; ++i) q[20 + 3 * k + i] = cs[k][i];
}
void flip_quad(double *q)
{
  for (int i = 0; i < 4; ++i) q[i] = -q[i];
}
} // namespace

bool make_polyhedron(const double *p, int np, HostShape &s, std::string &err)
{
  const double phiStartIn = p[0], phiDeltaIn = p[1];
  const int S = (int)p[2], nz = (int)p[3];
  if (S < 1 || nz < 2 || np < 4 + 3 * nz || !(phiDeltaIn > 0)) {
    err = "polyhedron needs >= 1 side, >= 2 z planes and phiDelta > 0";
    return false;
  }
  const double *zp = p + 4, *rmin = p + 4 + nz, *rmax = p + 4 + 2 * nz;
  for (int i = 0; i < nz; ++i) {
    if (i + 1 < nz && !(zp[i] <= zp[i + 1])) {
      err = "polyhedron z planes must be non-decreasing";
      return false;
    }
    if (!(rmin[i] >= 0) || !(rmax[i] >= rmin[i])) {
      err = "polyhedron radii must satisfy 0 <= rmin <= rmax";
      return false;
    }
  }
  const int nseg          = nz - 1;
  const bool hasPhiCutout = phiDeltaIn < kTwoPi, largePhiCutout = phiDeltaIn < kPi;
  const double fPhiStart  = normalize_angle(phiStartIn);
  const double fPhiDelta  = phiDeltaIn > kTwoPi ? kTwoPi : phiDeltaIn;
  // quadrilateral counts per segment
  std::vector<int> nout(nseg), nphi(nseg), nin(nseg);
  bool hasInnerRadii = false;
  for (int i = 0; i < nseg; ++i) {
    const bool hasInner = rmin[i] > 0 || rmin[i + 1] > 0;
    nout[i]             = S * ((zp[i] == zp[i + 1] && rmax[i] == rmax[i + 1]) ? 0 : 1);
    nphi[i]             = hasPhiCutout ? 2 * ((zp[i] == zp[i + 1]) ? 0 : 1) : 0;
    const int mult      = (zp[i] == zp[i + 1] && rmin[i] == rmin[i + 1]) ? 0 : 1;
    nin[i]              = (hasInner && mult > 0) ? S * mult : 0;
    if (nin[i] > 0) hasInnerRadii = true;
  }
  // layout
  const int hdr = ((int)(sizeof(PolyhedronRec) / sizeof(double)) + 3) / 4 * 4;
  int off       = hdr;
  auto take     = [&](int n) {
    const int o = off;
    off += (n + 3) / 4 * 4;
    return o;
  };
  const int oZ = take(nz), oRmin = take(nz), oRmax = take(nz), oSameZ = take(nz), oPhiSec = take(3 * (S + 1));
  const int oSeg = take(4 * nseg);
  std::vector<int> qbase(nseg);
  int nquads = 0;
  for (int i = 0; i < nseg; ++i) {
    qbase[i] = take(kPolyQuadDoubles * (nout[i] + nphi[i] + nin[i]));
    nquads += nout[i] + nphi[i] + nin[i];
  }
  const int oQ0 = nseg > 0 ? qbase[0] : off; // quadrilaterals are contiguous (a multiple of 4 doubles each)
  const int oQF = take((nquads * kPolyQuadFloats + 1) / 2);
  std::vector<double> rec(off, 0.);
  PolyhedronRec h{};
  h.nsides = S, h.nseg = nseg, h.nz = nz;
  h.flags  = (hasInnerRadii ? kPolyFlagInner : 0) | (hasPhiCutout ? kPolyFlagPhi : 0) |
            (largePhiCutout ? kPolyFlagLargePhi : 0);
  h.phiStart = fPhiStart, h.phiDelta = fPhiDelta;
  h.offZ = oZ, h.offRMin = oRmin, h.offRMax = oRmax, h.offSameZ = oSameZ, h.offPhiSec = oPhiSec, h.offSeg = oSeg;
  h.offQuad0 = oQ0, h.offQuadF = oQF;
  h.w = make_wedge(fPhiDelta, fPhiStart);
  for (int i = 0; i < nz; ++i) {
    rec[oZ + i] = zp[i], rec[oRmin + i] = rmin[i], rec[oRmax + i] = rmax[i];
    rec[oSameZ + i] = (i > 0 && i < nz - 1 && zp[i] == zp[i + 1]) ? 1. : 0.;
  }
  for (int i = 0; i < nseg; ++i) {
    rec[oSeg + 4 * i] = nout[i], rec[oSeg + 4 * i + 1] = nphi[i], rec[oSeg + 4 * i + 2] = nin[i];
    rec[oSeg + 4 * i + 3] = qbase[i];
  }
  // phi of the corners and the phi-section planes
  const double phiStart = normalize_angle(phiStartIn);
  const double phiDelta = phiDeltaIn > kTwoPi ? kTwoPi : phiDeltaIn;
  const double sidePhi  = phiDelta / S;
  std::vector<double> vphi(S + 1);
  std::vector<HV> phiSec(S + 1);
  for (int i = 0; i < S + 1; ++i) {
    vphi[i]         = normalize_angle(phiStart + i * sidePhi);
    const HV corner = hfix(hnormalized(hcyl(1., vphi[i], 0)));
    phiSec[i]       = hcross(hnormalized(corner), hv(0, 0, -1));
    for (int k = 0; k < 3; ++k) rec[oPhiSec + 3 * i + k] = phiSec[i][k];
  }
  if (!hasPhiCutout) vphi[S] = vphi[0];
  const double cosHalf = std::cos(0.5 * sidePhi);
  double innerRadius = kInfLength, outerRadius = -kInfLength;
  for (int i = 0; i < nz; ++i) {
    if (rmin[i] < innerRadius) innerRadius = rmin[i];
    if (rmax[i] > outerRadius) outerRadius = rmax[i];
  }
  outerRadius /= cosHalf;
  const double kPhiTolerance = 100 * kTolerance;
  const double bp[5] = {innerRadius - kHalfTolerance, outerRadius + kHalfTolerance,
                        0.5 * (zp[nz - 1] - zp[0]) + kTolerance, !hasPhiCutout ? 0 : phiStart - kPhiTolerance,
                        !hasPhiCutout ? kTwoPi : phiDelta + 2 * kPhiTolerance};
  HostShape bt;
  make_tube(bp, bt);
  std::memcpy(&h.bt, bt.rec.data(), sizeof(TubeRec));
  h.tubeOffset = 0.5 * (zp[0] + zp[nz - 1]);
  // vertices and quadrilaterals
  auto VI = [S](int plane, int corner) { return plane * (S + 1) + corner; };
  std::vector<HV> ov(nz * (S + 1), hv(0, 0, 0)), iv(nz * (S + 1), hv(0, 0, 0));
  for (int i = 0; i < nz; ++i) {
    for (int j = 0, jMax = S + (hasPhiCutout ? 1 : 0); j < jMax; ++j) {
      ov[VI(i, j)] = hfix(hcyl(rmax[i] / cosHalf, vphi[j], zp[i]));
      iv[VI(i, j)] = hfix(hcyl(rmin[i] / cosHalf, vphi[j], zp[i]));
    }
    if (!hasPhiCutout) {
      ov[VI(i, S)] = ov[VI(i, 0)];
      iv[VI(i, S)] = iv[VI(i, 0)];
    }
  }
  auto wrong = [](const double *q, HV c) { return q[0] * c[0] + q[1] * c[1] < 0; };
  for (int ip = 0; ip < nseg; ++ip) {
    double *qo = rec.data() + qbase[ip];
    double *qp = qo + kPolyQuadDoubles * nout[ip];
    double *qi = qp + kPolyQuadDoubles * nphi[ip];
    for (int k = 0; k < nout[ip]; ++k) {
      double *q = qo + kPolyQuadDoubles * k;
      set_quad(q, ov[VI(ip, k)], ov[VI(ip, k + 1)], ov[VI(ip + 1, k + 1)], ov[VI(ip + 1, k)]);
      if (wrong(q, ov[VI(ip, k)])) flip_quad(q);
    }
    for (int k = 0; k < nin[ip]; ++k) {
      double *q = qi + kPolyQuadDoubles * k;
      set_quad(q, iv[VI(ip, k)], iv[VI(ip, k + 1)], iv[VI(ip + 1, k + 1)], iv[VI(ip + 1, k)]);
      if (wrong(q, iv[VI(ip, k)])) flip_quad(q);
    }
    if (hasPhiCutout && nphi[ip] == 2) {
      set_quad(qp, iv[VI(ip, 0)], iv[VI(ip + 1, 0)], ov[VI(ip + 1, 0)], ov[VI(ip, 0)]);
      if (hdot(hv(qp[0], qp[1], qp[2]), phiSec[0]) > 0) flip_quad(qp);
      double *q1 = qp + kPolyQuadDoubles;
      set_quad(q1, ov[VI(ip, S)], ov[VI(ip + 1, S)], iv[VI(ip + 1, S)], iv[VI(ip, S)]);
      if (hdot(hv(q1[0], q1[1], q1[2]), phiSec[S]) < 0) flip_quad(q1);
    }
  }
  // FP32 copies of the planes of every quadrilateral, in record order
  float *qf = reinterpret_cast<float *>(rec.data() + oQF);
  for (int k = 0; k < nquads; ++k)
    for (int i = 0; i < kPolyQuadFloats; ++i) qf[kPolyQuadFloats * k + i] = (float)rec[oQ0 + kPolyQuadDoubles * k + i];
  std::memcpy(rec.data(), &h, sizeof(h));
  s.type = kShapePolyhedron;
  s.rec  = std::move(rec);
  // UnplacedPolyhedron::Extent (source/UnplacedPolyhedron.cpp:273-303)
  for (int k = 0; k < 3; ++k) s.lo[k] = kInfLength, s.hi[k] = -kInfLength;
  const double sp   = fPhiDelta / S;
  const double conv = 1. / std::cos(0.5 * sp);
  for (int iphi = 0; iphi <= S; ++iphi) {
    const double phi = fPhiStart + iphi * sp;
    const double cx = conv * std::cos(phi), cy = conv * std::sin(phi);
    for (int k = 0; k < nz; ++k) {
      const double a[3] = {rmin[k] * cx, rmin[k] * cy, zp[k]}, b[3] = {rmax[k] * cx, rmax[k] * cy, zp[k]};
      for (int i = 0; i < 3; ++i) { // Min(a, b) = a < b ? a : b, Max(a, b) = a > b ? a : b
        s.lo[i] = s.lo[i] < a[i] ? s.lo[i] : a[i];
        s.hi[i] = s.hi[i] > a[i] ? s.hi[i] : a[i];
      }
      for (int i = 0; i < 3; ++i) {
        s.lo[i] = s.lo[i] < b[i] ? s.lo[i] : b[i];
        s.hi[i] = s.hi[i] > b[i] ? s.hi[i] : b[i];
      }
    }
  }
  return true;
}

// ---------------------------------------------------------------- registry
Geometry::~Geometry()
{
  if (arena) cudaFree(arena);
}

int32_t Geometry::add_shape(int32_t type, const double *p, int np, std::string &err)
{
  if (closed) {
    err = "geometry is closed";
    return -1;
  }
  HostShape s;
  auto need = [&](int k) {
    if (np < k) {
      err = "too few shape parameters";
      return false;
    }
    return true;
  };
  switch (type) {
  case kShapeBox:
    if (!need(3)) return -1;
    make_box(p, s);
    break;
  case kShapeTube:
    if (!need(5)) return -1;
    make_tube(p, s);
    break;
  case kShapeCone:
    if (!need(7)) return -1;
    make_cone(p, s);
    break;
  case kShapeTrd:
    if (!need(5)) return -1;
    make_trd(p, s);
    break;
  case kShapeTrap:
    if (!make_trap(p, np, s, err)) return -1;
    break;
  case kShapePolyhedron:
    if (!need(4) || !make_polyhedron(p, np, s, err)) {
      if (err.empty()) err = "too few polyhedron parameters";
      return -1;
    }
    break;
  case kShapeTorus2:
    if (!need(5)) return -1;
    make_torus2(p, s);
    break;
  case kShapeCutTube:
    if (!need(11) || !make_cut_tube(p, s, err)) return -1;
    break;
  case kShapeSphere:
    if (!need(6)) return -1;
    make_sphere(p, s);
    break;
  case kShapeGenTrap:
    if (!need(17) || !make_gentrap(p, s, err)) return -1;
    break;
  case kShapeHype:
    if (!need(5)) return -1;
    make_hype(p, s);
    break;
  case kShapePolycone:
    if (!need(3) || !make_polycone(p, np, s, err)) return -1;
    break;
  case kShapeBoolMinus: {
    if (!need(2)) return -1;
    const int32_t l = (int32_t)p[0], r = (int32_t)p[1];
    if (l < 0 || r < 0 || l >= (int32_t)pvs.size() || r >= (int32_t)pvs.size()) {
      err = "invalid boolean operand placed-volume id";
      return -1;
    }
    for (int32_t op : {l, r})
      if (shapes[lvs[pvs[op].lv].shape].type == kShapeBoolMinus) {
        err = "boolean operands must be primitive shapes";
        return -1;
      }
    BoolRec b{(double)l, (double)r, 0., 0.};
    s.type     = kShapeBoolMinus;
    s.left_pv  = l;
    s.right_pv = r;
    pack(s, b);
    // source/UnplacedBooleanVolume.cpp:403-458: extent of the left operand in this frame
    HostShape const &ls = shapes[lvs[pvs[l].lv].shape];
    const double delta[3] = {ls.hi[0] - ls.lo[0], ls.hi[1] - ls.lo[1], ls.hi[2] - ls.lo[2]};
    double mn[3] = {kInfLength, kInfLength, kInfLength}, mx[3] = {-kInfLength, -kInfLength, -kInfLength};
    for (int x = 0; x <= 1; ++x)
      for (int y = 0; y <= 1; ++y)
        for (int z = 0; z <= 1; ++z) {
          const double c[3] = {ls.lo[0] + x * delta[0], ls.lo[1] + y * delta[1], ls.lo[2] + z * delta[2]};
          double t[3];
          pvs[l].xf.InverseTransform(c, t);
          for (int k = 0; k < 3; ++k) mn[k] = std::min(mn[k], t[k]), mx[k] = std::max(mx[k], t[k]);
        }
    for (int k = 0; k < 3; ++k) s.lo[k] = mn[k], s.hi[k] = mx[k];
    break;
  }
  default:
    err = "unknown shape type " + std::to_string(type);
    return -1;
  }
  shapes.push_back(std::move(s));
  return (int32_t)shapes.size() - 1;
}

int32_t Geometry::add_lv(int32_t shape, std::string &err)
{
  if (closed || shape < 0 || shape >= (int32_t)shapes.size()) {
    err = closed ? "geometry is closed" : "invalid shape id";
    return -1;
  }
  lvs.push_back(HostLV{shape, {}});
  return (int32_t)lvs.size() - 1;
}

// LogicalVolume::Place / PlaceDaughter (source/LogicalVolume.cpp:125-155): ids in creation order.
int32_t Geometry::place(int32_t lv, const double *t, const double *r, int32_t mother_lv, std::string &err)
{
  if (closed || lv < 0 || lv >= (int32_t)lvs.size() || mother_lv >= (int32_t)lvs.size()) {
    err = closed ? "geometry is closed" : "invalid logical volume id";
    return -1;
  }
  if (lvs[lv].daughters.size() >= 65535 || (mother_lv >= 0 && lvs[mother_lv].daughters.size() >= 65534)) {
    err = "more than 65535 daughters in one logical volume";
    return -1;
  }
  HostPV pv{lv, HostXform::FromArrays(t, r), -1};
  pvs.push_back(pv);
  const int32_t id = (int32_t)pvs.size() - 1;
  if (mother_lv >= 0) {
    pvs[id].child = (int32_t)lvs[mother_lv].daughters.size();
    lvs[mother_lv].daughters.push_back(id);
  }
  return id;
}

// ABBoxManager::ComputeABBox (source/ABBoxManager.cpp:109-140): the 8 corners of the
// shape's extent mapped to the mother frame, widened by 1e-3 mm.
void Geometry::daughter_box(int32_t pvid, double *box) const
{
  HostPV const &pv    = pvs[pvid];
  HostShape const &sh = shapes[lvs[pv.lv].shape];
  const double delta[3] = {sh.hi[0] - sh.lo[0], sh.hi[1] - sh.lo[1], sh.hi[2] - sh.lo[2]};
  double mn[3] = {kInfLength, kInfLength, kInfLength}, mx[3] = {-kInfLength, -kInfLength, -kInfLength};
  for (int x = 0; x <= 1; ++x)
    for (int y = 0; y <= 1; ++y)
      for (int z = 0; z <= 1; ++z) {
        const double corner[3] = {sh.lo[0] + x * delta[0], sh.lo[1] + y * delta[1], sh.lo[2] + z * delta[2]};
        double tc[3];
        pv.xf.InverseTransform(corner, tc);
        for (int k = 0; k < 3; ++k) {
          mn[k] = std::min(mn[k], tc[k]);
          mx[k] = std::max(mx[k], tc[k]);
        }
      }
  for (int k = 0; k < 3; ++k) box[k] = mn[k] - 1E-3, box[3 + k] = mx[k] + 1E-3;
}

// ---------------------------------------------------------------- BVH (source/BVH.cpp:48-385)
namespace {
struct Box6 {
  double lo[3], hi[3];
};
inline double surface_area(Box6 const &b)
{
  const double e0 = b.hi[0] - b.lo[0], e1 = b.hi[1] - b.lo[1], e2 = b.hi[2] - b.lo[2];
  return 2. * (e0 * e1 + e1 * e2 + e2 * e0);
}
inline Box6 merge(Box6 const &a, Box6 const &b)
{
  Box6 r;
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = a.lo[k] < b.lo[k] ? a.lo[k] : b.lo[k];
    r.hi[k] = a.hi[k] > b.hi[k] ? a.hi[k] : b.hi[k];
  }
  return r;
}
// Sort key of a primitive: its centroid pushed 1% further from its lower corner; keys are
// compared lexicographically starting at the sort axis (BVH.cpp:194-202, 261-268).
struct SahKey {
  double k[3];
};
inline bool key_less(SahKey const &a, SahKey const &b, int ax)
{
  const int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  return a.k[ax] < b.k[ax] ||
         (a.k[ax] == b.k[ax] && (a.k[a1] < b.k[a1] || (a.k[a1] == b.k[a1] && a.k[a2] < b.k[a2])));
}

// Surface-area-heuristic split of prims[b, e); returns the pivot (BVH.cpp:254-306).
int *sah_split(std::vector<Box6> const &boxes, std::vector<SahKey> const &keys, int *b, int *e)
{
  const long n  = e - b;
  double best   = (double)n;
  int bestAxis  = -1;
  int bestObj   = -1;
  std::vector<double> leftArea(n), rightArea(n);
  for (int axis = 0; axis < 3; ++axis) {
    std::sort(b, e, [&](int x, int y) { return key_less(keys[x], keys[y], axis); });
    Box6 acc     = boxes[b[0]];
    leftArea[0]  = 0.;
    for (long i = 1; i < n; ++i) {
      leftArea[i] = surface_area(acc);
      acc         = merge(acc, boxes[b[i]]);
    }
    Box6 racc = boxes[b[n - 1]];
    for (long i = n - 1; i >= 0; --i) {
      racc         = merge(racc, boxes[b[i]]);
      rightArea[i] = surface_area(racc);
    }
    const double total = rightArea[0];
    for (long i = 0; i < n; ++i) {
      const double metric = (leftArea[i] / total) * i + (rightArea[i] / total) * (n - i) + 0.1 * std::labs(n / 2 - i / n);
      if (metric < best) {
        best     = metric;
        bestAxis = axis;
        bestObj  = b[i];
      }
    }
  }
  if (bestAxis < 0) return e;
  SahKey const pivotKey = keys[bestObj];
  return std::partition(b, e, [&](size_t x) { return key_less(keys[(int)x], pivotKey, bestAxis); });
}
} // namespace

void Geometry::build_bvh(int32_t lvid, HostBVH &out) const
{
  HostLV const &lv = lvs[lvid];
  const int n      = (int)lv.daughters.size();
  std::vector<Box6> boxes(n);
  std::vector<SahKey> keys(n);
  out.prim_box.resize(6 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    daughter_box(lv.daughters[i], &out.prim_box[6 * (size_t)i]);
    std::memcpy(boxes[i].lo, &out.prim_box[6 * (size_t)i], 3 * sizeof(double));
    std::memcpy(boxes[i].hi, &out.prim_box[6 * (size_t)i + 3], 3 * sizeof(double));
    for (int k = 0; k < 3; ++k) {
      const double c = 0.5 * (boxes[i].hi[k] + boxes[i].lo[k]);
      keys[i].k[k]   = c + 0.01 * (c - boxes[i].lo[k]);
    }
  }
  const int half = n / 2;
  out.depth      = std::min(half > 0 ? std::max(0, (int)std::log2(half)) : 0, 32);
  const int nn   = (2 << out.depth) - 1;
  out.prim.resize(n);
  std::iota(out.prim.begin(), out.prim.end(), 0);
  out.nchild.assign(nn, 0);
  out.offset.assign(nn, -1);
  out.node_box.assign(6 * (size_t)nn, 0.);
  // Work list of (node, first, last) ranges; the two halves of a split are disjoint, so the
  // processing order does not change the result.
  struct Item {
    int node, first, last;
  };
  std::vector<Item> work{{0, 0, n}};
  while (!work.empty()) {
    const Item it = work.back();
    work.pop_back();
    if (it.node >= nn) continue;
    out.nchild[it.node] = it.last - it.first;
    out.offset[it.node] = it.first;
    if (it.first == it.last) continue;
    Box6 nb = boxes[out.prim[it.first]];
    for (int i = it.first + 1; i < it.last; ++i) nb = merge(nb, boxes[out.prim[i]]);
    std::memcpy(&out.node_box[6 * (size_t)it.node], nb.lo, 3 * sizeof(double));
    std::memcpy(&out.node_box[6 * (size_t)it.node + 3], nb.hi, 3 * sizeof(double));
    if (it.last - it.first == 1) continue;
    int *base  = out.prim.data();
    int *pivot = sah_split(boxes, keys, base + it.first, base + it.last);
    const int p = (int)(pivot - base);
    work.push_back({2 * it.node + 2, p, it.last});
    work.push_back({2 * it.node + 1, it.first, p});
  }
  for (int id = 0; id < nn / 2; ++id)
    if (out.nchild[id] > 8 && out.nchild[id] == out.nchild[2 * id + 1] + out.nchild[2 * id + 2]) out.nchild[id] = -1;
}

// ---------------------------------------------------------------- NavIndex table
// Layout per touchable (source/NavIndexTable.cpp:9-84): [mother, placed-volume id,
// (level u8, has-matrix u8, ndaughters u16), daughter indices..., pad to even], then the
// node's global matrix (3 translation + 9 rotation doubles) 8-byte aligned. Nodes are in
// depth-first pre-order; index 0 is the "outside" state.
void Geometry::build_nav_table()
{
  struct Frame {
    int32_t pv;
    int level;
    uint32_t mother;
    int dind;
    HostXform mat;
  };
  // Pass 1: size (matches the reference's two-pass allocation: 4 bytes + nodes, +1 word).
  size_t bytes = sizeof(uint32_t);
  {
    std::vector<std::pair<int32_t, int>> st{{world, 0}};
    int maxlev = 0;
    while (!st.empty()) {
      auto [pv, lev] = st.back();
      st.pop_back();
      maxlev             = std::max(maxlev, lev);
      const size_t nd    = lvs[pvs[pv].lv].daughters.size();
      bytes += (3 + nd + ((nd + 1) & 1)) * sizeof(uint32_t) + 12 * sizeof(double);
      for (int32_t d : lvs[pvs[pv].lv].daughters) st.push_back({d, lev + 1});
    }
    max_depth = maxlev + 1;
  }
  nav_words = bytes / sizeof(uint32_t) + 1;
  nav.assign(nav_words + 1, 0u);
  uint32_t cur = 1;
  std::vector<Frame> st;
  st.push_back({world, 0, 0u, 0, HostXform::Identity()});
  while (!st.empty()) {
    Frame f = st.back();
    st.pop_back();
    const std::vector<int32_t> &ds = lvs[pvs[f.pv].lv].daughters;
    const uint16_t nd              = (uint16_t)ds.size();
    const uint32_t self            = cur;
    nav[cur]                       = f.mother;
    if (f.mother > 0) nav[f.mother + 3 + f.dind] = cur;
    nav[cur + 1]          = (uint32_t)f.pv;
    HostXform mat         = f.mat;
    if (f.level > 0) mat.MultiplyFromRight(pvs[f.pv].xf); // the world's own placement is not applied
    unsigned char *meta   = reinterpret_cast<unsigned char *>(&nav[cur + 2]);
    meta[0]               = (unsigned char)f.level;
    meta[1]               = (unsigned char)(0x04 + 0x02 * (int)mat.has_trans + (int)mat.has_rot);
    std::memcpy(meta + 2, &nd, 2);
    cur += 3 + nd + ((nd + 1) & 1);
    if (cur & 1u) ++cur;
    std::memcpy(&nav[cur], mat.m.t, 3 * sizeof(double));
    std::memcpy(&nav[cur + 6], mat.m.r, 9 * sizeof(double));
    cur += 24;
    // push daughters in reverse so that they are visited in order
    for (int i = (int)ds.size() - 1; i >= 0; --i) st.push_back({ds[i], f.level + 1, self, i, mat});
  }
  nav.resize(nav_words);
}

// ---------------------------------------------------------------- close + upload
int Geometry::build_host(std::string &err)
{
  if (closed) {
    err = "geometry already closed";
    return -1;
  }
  if (built) return 0;
  lv_bvh.assign(lvs.size(), -1);
  bvhs.clear();
  if (world >= 0) {
    for (size_t l = 0; l < lvs.size(); ++l) {
      if (lvs[l].daughters.empty()) continue;
      HostBVH b;
      build_bvh((int32_t)l, b);
      lv_bvh[l] = (int32_t)bvhs.size();
      bvhs.push_back(std::move(b));
    }
    build_nav_table();
    if (max_depth > 255) {
      err = "geometry deeper than 255 levels";
      return -1;
    }
  }
  built = true;
  return 0;
}

int Geometry::close(std::string &err)
{
  if (build_host(err) != 0) return -1;
  if (upload(err) != 0) return -1;
  closed = true;
  return 0;
}

namespace {
float round_down(double x)
{
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -INFINITY);
  return f;
}
float round_up(double x)
{
  float f = (float)x;
  if ((double)f < x) f = std::nextafter(f, INFINITY);
  return f;
}
struct Arena {
  std::vector<unsigned char> host;
  size_t add(const void *p, size_t bytes)
  {
    const size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + bytes);
    if (bytes) std::memcpy(host.data() + off, p, bytes);
    return off;
  }
  template <class T>
  size_t add(std::vector<T> const &v)
  {
    return add(v.data(), v.size() * sizeof(T));
  }
};
} // namespace

int Geometry::upload(std::string &err)
{
  Arena a;
  // shapes
  std::vector<double> sdata;
  std::vector<int32_t> stype, soff;
  for (auto const &s : shapes) {
    while (sdata.size() % 4) sdata.push_back(0.); // 32-byte aligned records
    stype.push_back(s.type);
    soff.push_back((int32_t)sdata.size());
    sdata.insert(sdata.end(), s.rec.begin(), s.rec.end());
  }
  std::vector<int32_t> lv_shape, lv_dstart, lv_nd, daughters;
  for (auto const &lv : lvs) {
    lv_shape.push_back(lv.shape);
    lv_dstart.push_back((int32_t)daughters.size());
    lv_nd.push_back((int32_t)lv.daughters.size());
    daughters.insert(daughters.end(), lv.daughters.begin(), lv.daughters.end());
  }
  std::vector<int32_t> pv_lv, pv_child;
  std::vector<Xform> pv_xf;
  for (auto const &pv : pvs) {
    pv_lv.push_back(pv.lv);
    pv_child.push_back(pv.child);
    pv_xf.push_back(pv.xf.m);
  }
  // BVH arrays: node arrays concatenated; prim slots follow the LV daughter layout.
  std::vector<int32_t> bvh_node0, bvh_prim0, node_nchild, node_offset, prim_id(daughters.size(), 0);
  std::vector<double> node_box, prim_box(6 * daughters.size(), 0.);
  std::vector<NodeF> node_f;
  std::vector<float> prim_box_f(6 * daughters.size(), 0.f);
  // Learned proposal: BVH depth per LV, and per daughter slot the depth-3 subtree (0..7,
  // node 7 + k in breadth-first numbering) of the leaf that holds it; -1 where the leaf
  // sits above depth 3 or the BVH is shallower.
  std::vector<int32_t> lv_depth(lvs.size(), -1), dau_slot3(daughters.size(), -1);
  for (size_t l = 0; l < lvs.size(); ++l) {
    if (lv_bvh[l] < 0) continue;
    HostBVH const &b   = bvhs[lv_bvh[l]];
    const int32_t base = lv_dstart[l];
    lv_depth[l]        = b.depth;
    for (size_t i = 0; i < b.nchild.size(); ++i) {
      if (b.nchild[i] <= 0) continue;
      int depth = 0;
      while ((size_t(2) << depth) - 1 <= i) ++depth; // nodes of depth d: [2^d - 1, 2^(d+1) - 1)
      if (depth < 3) continue;
      size_t a = i;
      for (int d = depth; d > 3; --d) a = (a - 1) / 2;
      for (int j = 0; j < b.nchild[i]; ++j) dau_slot3[base + b.prim[b.offset[i] + j]] = (int32_t)a - 7;
    }
    bvh_node0.push_back((int32_t)node_nchild.size());
    bvh_prim0.push_back(base);
    for (size_t i = 0; i < b.nchild.size(); ++i) {
      node_nchild.push_back(b.nchild[i]);
      node_offset.push_back(b.offset[i] < 0 ? -1 : base + b.offset[i]);
      NodeF nf;
      for (int k = 0; k < 3; ++k) {
        node_box.push_back(b.node_box[6 * i + k]);
        nf.lo[k] = round_down(b.node_box[6 * i + k]);
        nf.hi[k] = round_up(b.node_box[6 * i + 3 + k]);
      }
      for (int k = 0; k < 3; ++k) node_box.push_back(b.node_box[6 * i + 3 + k]);
      nf.nchild = b.nchild[i];
      nf.offset = b.offset[i] < 0 ? -1 : base + b.offset[i];
      node_f.push_back(nf);
    }
    for (size_t i = 0; i < b.prim.size(); ++i) prim_id[base + i] = b.prim[i];
    for (size_t i = 0; i < 6 * b.prim.size(); ++i) {
      prim_box[6 * (size_t)base + i]   = b.prim_box[i];
      prim_box_f[6 * (size_t)base + i] = (i % 6 < 3) ? round_down(b.prim_box[i]) : round_up(b.prim_box[i]);
    }
  }
  const size_t o_sdata = a.add(sdata), o_stype = a.add(stype), o_soff = a.add(soff);
  const size_t o_lvs = a.add(lv_shape), o_lvd = a.add(lv_dstart), o_lvn = a.add(lv_nd), o_lvb = a.add(lv_bvh);
  const size_t o_dau = a.add(daughters), o_pvl = a.add(pv_lv), o_pvc = a.add(pv_child), o_pvx = a.add(pv_xf);
  const size_t o_bn0 = a.add(bvh_node0), o_bp0 = a.add(bvh_prim0), o_nnc = a.add(node_nchild);
  const size_t o_nof = a.add(node_offset), o_nbx = a.add(node_box), o_pid = a.add(prim_id);
  const size_t o_lvdp = a.add(lv_depth), o_ds3 = a.add(dau_slot3);
  // VUnplacedVolume::fBBox (UnplacedVolume.h:45, ComputeBBox = Extent) of every shape
  std::vector<double> shape_bbox(6 * shapes.size());
  for (size_t i = 0; i < shapes.size(); ++i)
    for (int k = 0; k < 3; ++k) shape_bbox[6 * i + k] = shapes[i].lo[k], shape_bbox[6 * i + 3 + k] = shapes[i].hi[k];
  const size_t o_sbb = a.add(shape_bbox);
  // FP32 bounding descriptors of the shapes (mixed-precision navigator): kind 0 = box
  // (lo, hi; flag 1 when the box is the shape itself), kind 1 = cylindrical shell (rmin,
  // rmax, zlo, zhi; flag 1 when the shell is the shape itself). Radii and z are rounded
  // outward to FP32.
  std::vector<float> lbd(8 * shapes.size(), 0.f);
  for (size_t i = 0; i < shapes.size(); ++i) {
    HostShape const &s = shapes[i];
    float *d           = &lbd[8 * i];
    auto shell = [&](double rmin, double rmax, double zlo, double zhi, bool exact) {
      d[0] = 1.f, d[1] = exact ? 1.f : 0.f;
      d[2] = round_down(rmin < 0 ? 0 : rmin), d[3] = round_up(rmax), d[4] = round_down(zlo), d[5] = round_up(zhi);
    };
    if (s.type == kShapeTube) {
      const TubeRec &t = *reinterpret_cast<const TubeRec *>(s.rec.data());
      shell(t.rmin, t.rmax, -t.z, t.z, t.dphi >= kTwoPi);
    } else if (s.type == kShapeCone) {
      const ConeRec &c = *reinterpret_cast<const ConeRec *>(s.rec.data());
      shell(std::min(c.rmin1, c.rmin2), std::max(std::max(c.rmax1, c.rmax2), std::max(c.origRmax1, c.origRmax2)),
            -c.dz, c.dz, false);
    } else if (s.type == kShapePolycone) {
      const int nsec = (int)s.rec[0];
      double rmin = kInfLength, rmax = 0.;
      for (int k = 0; k < nsec; ++k) {
        const ConeRec &c =
            *reinterpret_cast<const ConeRec *>(s.rec.data() + polycone_section_base(nsec) + k * kPolyconeSectionDoubles + 4);
        rmin = std::min(rmin, std::min(c.rmin1, c.rmin2));
        rmax = std::max(rmax, std::max(std::max(c.rmax1, c.rmax2), std::max(c.origRmax1, c.origRmax2)));
      }
      shell(rmin, rmax, s.rec[4], s.rec[4 + nsec], false);
    } else if (s.type == kShapeTorus2) {
      const TorusRec &t = *reinterpret_cast<const TorusRec *>(s.rec.data());
      shell(t.rtor - t.rmax, t.rtor + t.rmax, -t.rmax, t.rmax, false);
    } else {
      d[0] = 0.f, d[1] = (s.type == kShapeBox) ? 1.f : 0.f;
      for (int k = 0; k < 3; ++k) d[2 + k] = round_down(s.lo[k]), d[5 + k] = round_up(s.hi[k]);
    }
  }
  // per prim slot: box, placed volume, descriptor and FP32 placement in one record
  std::vector<LeafRec> leaf_rec(daughters.size());
  for (size_t l = 0; l < lvs.size(); ++l) {
    if (lv_bvh[l] < 0) continue;
    const int32_t base = lv_dstart[l];
    for (int32_t k = 0; k < lv_nd[l]; ++k) {
      const size_t slot  = (size_t)base + k;
      const int32_t prim = prim_id[slot];
      const int32_t pv   = daughters[(size_t)base + prim];
      LeafRec &r         = leaf_rec[slot];
      std::memset(&r, 0, sizeof(r));
      for (int c = 0; c < 3; ++c) {
        r.lo[c] = prim_box_f[6 * ((size_t)base + prim) + c];
        r.hi[c] = prim_box_f[6 * ((size_t)base + prim) + 3 + c];
      }
      r.pv              = pv;
      const int32_t shp = lvs[pvs[pv].lv].shape;
      r.type            = stype[shp];
      r.off             = soff[shp];
      std::memcpy(r.lb, &lbd[8 * (size_t)shp], sizeof(r.lb));
      const Xform &m = pvs[pv].xf.m;
      for (int c = 0; c < 3; ++c) {
        r.t[c] = (float)m.t[c];
        if (!(std::fabs(m.t[c]) <= 4000.)) r.exact_only = 1; // the FP32 pad covers |t| <= 4 m
      }
      for (int c = 0; c < 9; ++c) r.r[c] = (float)m.r[c];
    }
  }
  const size_t o_pbx = a.add(prim_box), o_nf = a.add(node_f), o_pbf = a.add(prim_box_f), o_nav = a.add(nav);
  std::vector<PvRec> pv_rec(pvs.size());
  for (size_t i = 0; i < pvs.size(); ++i) {
    PvRec &r   = pv_rec[i];
    r.lv       = pvs[i].lv;
    r.shape    = lvs[r.lv].shape;
    r.type     = stype[r.shape];
    r.off      = soff[r.shape];
    r.nd       = lv_nd[r.lv];
    const int b = lv_bvh[r.lv];
    r.node0    = b >= 0 ? bvh_node0[b] : -1;
    r.depth    = lv_depth[r.lv];
    r.child    = pvs[i].child;
  }
  const size_t o_lbd = a.add(lbd), o_lrec = a.add(leaf_rec), o_pvr = a.add(pv_rec);
  shape_lbd_host     = lbd;

  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaMalloc(&arena, a.host.size() ? a.host.size() : 256);
  if (e == cudaSuccess) e = cudaMemcpy(arena, a.host.data(), a.host.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    err = std::string("CUDA error during geometry upload: ") + cudaGetErrorString(e);
    return -1;
  }
  arena_bytes      = a.host.size();
  unsigned char *d = static_cast<unsigned char *>(arena);
  auto P = [d](size_t off) { return d + off; };
  dev.shape_data  = reinterpret_cast<const double *>(P(o_sdata));
  dev.shape_type  = reinterpret_cast<const int32_t *>(P(o_stype));
  dev.shape_off   = reinterpret_cast<const int32_t *>(P(o_soff));
  dev.lv_shape    = reinterpret_cast<const int32_t *>(P(o_lvs));
  dev.lv_dstart   = reinterpret_cast<const int32_t *>(P(o_lvd));
  dev.lv_nd       = reinterpret_cast<const int32_t *>(P(o_lvn));
  dev.lv_bvh      = reinterpret_cast<const int32_t *>(P(o_lvb));
  dev.daughters   = reinterpret_cast<const int32_t *>(P(o_dau));
  dev.pv_lv       = reinterpret_cast<const int32_t *>(P(o_pvl));
  dev.pv_child    = reinterpret_cast<const int32_t *>(P(o_pvc));
  dev.pv_xf       = reinterpret_cast<const Xform *>(P(o_pvx));
  dev.bvh_node0   = reinterpret_cast<const int32_t *>(P(o_bn0));
  dev.bvh_prim0   = reinterpret_cast<const int32_t *>(P(o_bp0));
  dev.node_nchild = reinterpret_cast<const int32_t *>(P(o_nnc));
  dev.node_offset = reinterpret_cast<const int32_t *>(P(o_nof));
  dev.node_box    = reinterpret_cast<const double *>(P(o_nbx));
  dev.prim_id     = reinterpret_cast<const int32_t *>(P(o_pid));
  dev.prim_box    = reinterpret_cast<const double *>(P(o_pbx));
  dev.node_f      = reinterpret_cast<const NodeF *>(P(o_nf));
  dev.prim_box_f  = reinterpret_cast<const float *>(P(o_pbf));
  dev.nav         = reinterpret_cast<const uint32_t *>(P(o_nav));
  dev.nav_words   = (uint32_t)nav_words;
  dev.lv_depth    = reinterpret_cast<const int32_t *>(P(o_lvdp));
  dev.dau_slot3   = reinterpret_cast<const int32_t *>(P(o_ds3));
  dev.shape_bbox  = reinterpret_cast<const double *>(P(o_sbb));
  dev.shape_lbd   = reinterpret_cast<const float *>(P(o_lbd));
  dev.leaf_rec    = reinterpret_cast<const LeafRec *>(P(o_lrec));
  dev.pv_rec      = reinterpret_cast<const PvRec *>(P(o_pvr));
  dev.type_mask   = 0;
  for (const int32_t t : stype) dev.type_mask |= 1u << t;
  dev.world_pv    = world;
  dev.max_depth   = max_depth;
  dev.n_pv        = (int32_t)pvs.size();
  dev.n_lv        = (int32_t)lvs.size();
  return 0;
}

} // namespace vg
