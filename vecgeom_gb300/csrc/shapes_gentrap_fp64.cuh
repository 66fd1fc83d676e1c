// FP64 generic-trapezoid (GenTrap) kernels on the flattened record (GenTrapRec, vg_types.h):
// the generic kernels of VecGeom/volumes/kernel/GenTrapImplementation.h with the four
// lateral surfaces of VecGeom/volumes/SecondOrderSurfaceShell.h (planar, or twisted:
// hyperbolic paraboloids crossed by solving a second-order equation), in the reference's
// operation order, so results are bit-identical in FP64. These are the kernels the
// reference's CUDA build runs for every GenTrap.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {
namespace f64 {

__device__ __forceinline__ bool gt_bit(long long m, int i) { return (m >> i) & 1; }
__device__ __forceinline__ double gt_min(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double gt_max(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ V3 gt_v3(const double *a) { return V3{a[0], a[1], a[2]}; }
// surface i: a = vertex i (-dz), b = vertex i+4 (+dz), c = vertex j (-dz), d = vertex j+4
__device__ __forceinline__ double gt_xa(const GenTrapRec &g, int i) { return g.vx[i]; }
__device__ __forceinline__ double gt_ya(const GenTrapRec &g, int i) { return g.vy[i]; }
__device__ __forceinline__ double gt_xb(const GenTrapRec &g, int i) { return g.vx[i + 4]; }
__device__ __forceinline__ double gt_yb(const GenTrapRec &g, int i) { return g.vy[i + 4]; }
__device__ __forceinline__ double gt_xc(const GenTrapRec &g, int i) { return g.vx[(i + 1) & 3]; }
__device__ __forceinline__ double gt_yc(const GenTrapRec &g, int i) { return g.vy[(i + 1) & 3]; }
__device__ __forceinline__ double gt_xd(const GenTrapRec &g, int i) { return g.vx[4 + ((i + 1) & 3)]; }
__device__ __forceinline__ double gt_yd(const GenTrapRec &g, int i) { return g.vy[4 + ((i + 1) & 3)]; }

// (p - a_i) . n_i with a_i = (xa, ya, -dz)
__device__ __forceinline__ double gt_dot_ap(const GenTrapRec &g, int i, V3 p)
{
  return (p.x - gt_xa(g, i)) * g.normal[i][0] + (p.y - gt_ya(g, i)) * g.normal[i][1] +
         (p.z - (-g.dz)) * g.normal[i][2];
}
__device__ __forceinline__ double gt_dot_n(const GenTrapRec &g, int i, V3 d)
{
  return d.x * g.normal[i][0] + d.y * g.normal[i][1] + d.z * g.normal[i][2];
}

// SecondOrderSurfaceShell::CheckInside
__device__ __forceinline__ void gt_check_inside(const GenTrapRec &g, V3 p, bool &cin, bool &cout, bool &onsurf)
{
  const double tolerancesq = 10000. * kTolerance * kTolerance;
  onsurf                   = false;
  cin                      = fabs(p.z) < g.dz - kHalfTolerance;
  cout                     = fabs(p.z) > g.dz + kHalfTolerance;
  if (cout) return;
  double vX[4], vY[4];
  const double dzp = g.dz + p.z;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    vX[i] = gt_xa(g, i) + g.tx1[i] * dzp;
    vY[i] = gt_ya(g, i) + g.ty1[i] * dzp;
  }
  bool degenerated = true;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int j           = (i + 1) & 3;
    const double DeltaX   = vX[j] - vX[i];
    const double DeltaY   = vY[j] - vY[i];
    const double deltasq  = DeltaX * DeltaX + DeltaY * DeltaY;
    const bool samevertex = deltasq < kHalfTolerance;
    degenerated           = degenerated && samevertex;
    const double cross    = (p.x - vX[i]) * DeltaY - (p.y - vY[i]) * DeltaX;
    const bool onsurfi    = (cross * cross < tolerancesq * deltasq) && !samevertex;
    cout                  = cout || ((cross < -kHalfTolerance) && !onsurfi);
    cin                   = cin && (samevertex || ((cross > kHalfTolerance) && !onsurfi));
  }
  onsurf = !cout && !cin;
  cout   = cout || degenerated;
}

// SecondOrderSurfaceShell::InSurfLimits
__device__ __forceinline__ bool gt_in_surf_limits(const GenTrapRec &g, V3 p, int i)
{
  const double rz = g.dz2 * (p.z + g.dz);
  if (!((rz > -kHalfTolerance) && (rz < 1. + kHalfTolerance))) return false;
  double r     = kInfLength;
  double num   = (p.x - gt_xa(g, i)) - rz * (gt_xb(g, i) - gt_xa(g, i));
  double denom = (gt_xc(g, i) - gt_xa(g, i)) + rz * (gt_xd(g, i) - gt_xc(g, i) - gt_xb(g, i) + gt_xa(g, i));
  if (fabs(denom) > 1.e-6) r = num / nonzero(denom);
  num   = (p.y - gt_ya(g, i)) - rz * (gt_yb(g, i) - gt_ya(g, i));
  denom = (gt_yc(g, i) - gt_ya(g, i)) + rz * (gt_yd(g, i) - gt_yc(g, i) - gt_yb(g, i) + gt_ya(g, i));
  if (fabs(denom) > 1.e-6) r = num / nonzero(denom);
  return (r > -kHalfTolerance) && (r < 1. + kHalfTolerance);
}

// SecondOrderSurfaceShell::UNormal (r keeps its value when both denominators are small)
__device__ __forceinline__ V3 gt_unormal(const GenTrapRec &g, V3 p, int i, double &r)
{
  const double rz = g.dz2 * (p.z + g.dz);
  double num      = (p.x - gt_xa(g, i)) - rz * (gt_xb(g, i) - gt_xa(g, i));
  double denom    = (gt_xc(g, i) - gt_xa(g, i)) + rz * (gt_xd(g, i) - gt_xc(g, i) - gt_xb(g, i) + gt_xa(g, i));
  if (fabs(denom) > 1.e-6) r = num / nonzero(denom);
  num   = (p.y - gt_ya(g, i)) - rz * (gt_yb(g, i) - gt_ya(g, i));
  denom = (gt_yc(g, i) - gt_ya(g, i)) + rz * (gt_yd(g, i) - gt_yc(g, i) - gt_yb(g, i) + gt_ya(g, i));
  if (fabs(denom) > 1.e-6) r = num / nonzero(denom);
  V3 u;
  u.x = g.viCrossHi0[i][0] + rz * g.viCrossVj[i][0] + r * g.hi1CrossHi0[i][0];
  u.y = g.viCrossHi0[i][1] + rz * g.viCrossVj[i][1] + r * g.hi1CrossHi0[i][1];
  u.z = g.viCrossHi0[i][2] + rz * g.viCrossVj[i][2] + r * g.hi1CrossHi0[i][2];
  return u;
}

// SecondOrderSurfaceShell::ComputeSminSmax for surface i
__device__ __forceinline__ void gt_smin_smax(const GenTrapRec &g, V3 p, V3 d, int i, double &smin, double &smax)
{
  if (!gt_bit(g.curved, i)) { // planar surface: the plane crossing, smax not checked
    smin = -gt_dot_ap(g, i, p) / nonzero(gt_dot_n(g, i, d));
    smax = kInfLength;
    return;
  }
  const double dzp = g.dz + p.z;
  const double xs1 = gt_xa(g, i) + g.tx1[i] * dzp;
  const double ys1 = gt_ya(g, i) + g.ty1[i] * dzp;
  const double xs2 = gt_xc(g, i) + g.tx2[i] * dzp;
  const double ys2 = gt_yc(g, i) + g.ty2[i] * dzp;
  const double dxs = xs2 - xs1;
  const double dys = ys2 - ys1;
  const double a   = (g.deltatx[i] * d.y - g.deltaty[i] * d.x + g.t1crosst2[i] * d.z) * d.z;
  const double b   = dxs * d.y - dys * d.x +
                   (g.deltatx[i] * p.y - g.deltaty[i] * p.x + g.ty2[i] * xs1 - g.ty1[i] * xs2 + g.tx1[i] * ys2 -
                    g.tx2[i] * ys1) *
                       d.z;
  const double c  = dxs * p.y - dys * p.x + xs1 * ys2 - xs2 * ys1;
  const double dd = b * b - 4 * a * c;
  double signa    = 0.;
  if (a < -kTolerance) signa = -1.;
  if (a > kTolerance) signa = 1.;
  double inva = c / nonzero(b * b);
  if (fabs(a) > kTolerance) inva = 1. / nonzero(2. * a);
  double sqrtd = signa * sqrt(fabs(dd));
  if (dd < 0.) sqrtd = kInfLength;
  smin = (-b - sqrtd) * inva;
  smax = (-b + sqrtd) * inva;
}

// ---------------------------------------------------------------- Inside / Contains
// GenericKernelForContainsAndInside: bounding box (tolerant), then the side of each lateral
// edge of the section at the point's z
__device__ __forceinline__ void gt_classify(const GenTrapRec &g, V3 p, bool forInside, bool &cin, bool &cout)
{
  const double tolerancesq = 10000. * kTolerance * kTolerance;
  const double dist        = max3(fabs(p.x - g.bborig[0]) - g.bbdim[0], fabs(p.y - g.bborig[1]) - g.bbdim[1],
                                  fabs(p.z - g.bborig[2]) - g.bbdim[2]);
  cin                      = forInside && dist < -kHalfTolerance;
  cout                     = dist > kHalfTolerance;
  if (cout) return;
  const double cf = g.halfInvDz * (g.dz - p.z);
  double vX[4], vY[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    vX[i] = g.vx[i + 4] + cf * g.connx[i];
    vY[i] = g.vy[i + 4] + cf * g.conny[i];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (gt_bit(g.degenerated, i)) continue;
    const int j         = (i + 1) & 3;
    const double DeltaX = vX[j] - vX[i];
    const double DeltaY = vY[j] - vY[i];
    const double cross  = (p.x - vX[i]) * DeltaY - (p.y - vY[i]) * DeltaX;
    if (forInside) {
      const bool onsurf = cross * cross < tolerancesq * (DeltaX * DeltaX + DeltaY * DeltaY);
      cout              = cout || ((cross < -kHalfTolerance) && !onsurf);
      cin               = cin && (cross > kHalfTolerance) && !onsurf;
    } else {
      cout = cout || (cross < 0.);
    }
    if (cout) return;
  }
}
__device__ __forceinline__ int gentrap_inside(const GenTrapRec &g, V3 p)
{
  bool cin, cout;
  gt_classify(g, p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
__device__ __forceinline__ bool gentrap_contains(const GenTrapRec &g, V3 p)
{
  bool cin, cout;
  gt_classify(g, p, false, cin, cout);
  return !cout;
}

// ---------------------------------------------------------------- DistanceToIn
// IsInTopOrBottomPolygon: the crossing with the top (or bottom) face lies in its polygon
__device__ __forceinline__ bool gt_in_top_or_bottom(const GenTrapRec &g, double x, double y, bool top)
{
  bool degenerate = true;
  const int o     = top ? 4 : 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double deltaX = g.deltax[o + i], deltaY = g.deltay[o + i];
    double cross        = (x - g.vx[o + i]) * deltaY;
    cross -= (y - g.vy[o + i]) * deltaX;
    degenerate = degenerate && (deltaX < kHalfTolerance) && (deltaY < kHalfTolerance);
    if (cross < 0. - (fabs(deltaX) + fabs(deltaY)) * kHalfTolerance) return false;
  }
  return !degenerate;
}

// SecondOrderSurfaceShell::DistanceToInPlanar (done is false on this path)
__device__ __forceinline__ double gt_shell_dist_in_planar(const GenTrapRec &g, V3 p, V3 d)
{
  double distance = kInfLength;
  bool inside     = fabs(p.z) < g.dz - kHalfTolerance;
  for (int i = 0; i < 4; ++i) {
    if (gt_bit(g.degenerated, i)) continue;
    const double dotAPNorm  = gt_dot_ap(g, i, p);
    const bool otherside    = dotAPNorm < -10. * kTolerance;
    const double dotDirNorm = gt_dot_n(g, i, d);
    inside                  = inside && otherside;
    if (!(dotDirNorm < 0.) || otherside) continue;
    const double snext = -dotAPNorm / nonzero(dotDirNorm);
    const V3 psurf{p.x + snext * d.x, p.y + snext * d.y, p.z + snext * d.z};
    if (gt_in_surf_limits(g, psurf, i) && snext < distance) distance = gt_max(snext, 0.);
  }
  if (distance < kTolerance) distance = 0.;
  if (inside) distance = -1.;
  return distance;
}

// SecondOrderSurfaceShell::DistanceToIn (twisted surfaces; done is false on this path)
static __device__ __noinline__ double gt_shell_dist_in(const GenTrapRec &g, V3 p, V3 d)
{
  const double tolerance = 100. * kTolerance;
  double distance        = kInfLength;
  double r               = -1.0;
  bool cin, cout, onsurf;
  gt_check_inside(g, p, cin, cout, onsurf);
  if (cin) return -1.0;
  for (int i = 0; i < 4; ++i) {
    double smin, smax;
    gt_smin_smax(g, p, d, i, smin, smax);
    double crtdist = smin;
    V3 hit{p.x + crtdist * d.x, p.y + crtdist * d.y, p.z + crtdist * d.z};
    bool crossing = (crtdist > -tolerance) && (fabs(hit.z) < g.dz + kTolerance);
    if (crossing) {
      const V3 unorm = gt_unormal(g, hit, i, r);
      crossing       = dot(d, unorm) < 0. && (r >= 0.) && (r <= 1.);
      if (crossing && crtdist < distance) distance = gt_max(crtdist, 0.);
    }
    if (!crossing) {
      crtdist  = smax;
      hit      = V3{p.x + crtdist * d.x, p.y + crtdist * d.y, p.z + crtdist * d.z};
      crossing = (crtdist > -tolerance) && (fabs(hit.z) < g.dz + kTolerance);
      if (!crossing) continue;
      const V3 unorm = gt_bit(g.curved, i) ? gt_unormal(g, hit, i, r) : gt_v3(g.normal[i]);
      crossing       = (dot(d, unorm) < 0.) && (r >= 0.) && (r <= 1.);
      if (crossing && crtdist < distance) distance = gt_max(crtdist, 0.);
    }
  }
  if (distance < tolerance && onsurf) distance = 0.;
  return distance;
}

static __device__ __noinline__ double gentrap_dist_in(const GenTrapRec &g, V3 p, V3 d)
{
  const BoxRec bb{g.bbdim[0], g.bbdim[1], g.bbdim[2]};
  const double bbdistance = box_dist_in(bb, V3{p.x - g.bborig[0], p.y - g.bborig[1], p.z - g.bborig[2]}, d);
  if (bbdistance >= kInfLength) return kInfLength;
  const double zsafety = fabs(p.z) - g.dz;
  if (zsafety > -kHalfTolerance && p.z * d.z < 0) {
    const double next = zsafety / nonzeroabs(d.z);
    if (gt_in_top_or_bottom(g, p.x + next * d.x, p.y + next * d.y, d.z < 0)) return bbdistance;
  }
  const double disttoplanes = g.planar ? gt_shell_dist_in_planar(g, p, d) : gt_shell_dist_in(g, p, d);
  return gt_min(disttoplanes, kInfLength);
}

// ---------------------------------------------------------------- DistanceToOut
__device__ __forceinline__ double gt_shell_dist_out_planar(const GenTrapRec &g, V3 p, V3 d)
{
  double distance = kInfLength;
  bool outside    = fabs(p.z) > g.dz + kHalfTolerance;
  for (int i = 0; i < 4 && !outside; ++i) {
    if (gt_bit(g.degenerated, i)) continue;
    const double dotAPNorm  = gt_dot_ap(g, i, p);
    const bool otherside    = dotAPNorm > 10. * kTolerance;
    const double dotDirNorm = gt_dot_n(g, i, d);
    outside                 = outside || otherside;
    if (!(dotDirNorm > 0.) || otherside) continue;
    const double snext = -dotAPNorm / nonzero(dotDirNorm);
    if (snext < distance) distance = gt_max(snext, 0.);
  }
  if (distance < kTolerance) distance = 0.;
  if (outside) distance = -1.;
  return distance;
}

static __device__ __noinline__ double gt_shell_dist_out(const GenTrapRec &g, V3 p, V3 d)
{
  const double tolerance = 100. * kTolerance;
  double dist            = kInfLength;
  double r               = -1.0;
  V3 unorm{0., 0., 0.};
  bool cin, cout, onsurf;
  gt_check_inside(g, p, cin, cout, onsurf);
  if (cout) return -1.0;
  for (int i = 0; i < 4; ++i) {
    double smin, smax;
    gt_smin_smax(g, p, d, i, smin, smax);
    if (fabs(smin) < tolerance || fabs(smax) < tolerance)
      unorm = gt_bit(g.curved, i) ? gt_unormal(g, p, i, r) : gt_v3(g.normal[i]);
    if (fabs(smin) < tolerance && dot(d, unorm) < 0) smin = kInfLength;
    if (fabs(smax) < tolerance && dot(d, unorm) < 0) smax = kInfLength;
    if (smin > -tolerance && smin < dist) dist = gt_max(smin, 0.);
    if (smax > -tolerance && smax < dist) dist = gt_max(smax, 0.);
  }
  if (dist < tolerance && onsurf) dist = 0.;
  return dist;
}

static __device__ __noinline__ double gentrap_dist_out(const GenTrapRec &g, V3 p, V3 d)
{
  const double sign      = d.z < 0 ? -1.0 : 1.0;
  const double distmin   = (sign * g.dz - p.z) / nonzero(d.z);
  const double distplane = g.planar ? gt_shell_dist_out_planar(g, p, d) : gt_shell_dist_out(g, p, d);
  return gt_min(distmin, distplane);
}

// ---------------------------------------------------------------- safeties
// SecondOrderSurfaceShell::SafetyCurved
static __device__ __noinline__ double gt_safety_curved(const GenTrapRec &g, V3 p, bool in)
{
  double safety = kInfLength, safplanar = kInfLength;
  double dx1 = 0., dx2 = 0., dy1 = 0., dy2 = 0.;
  bool cin, cout, onsurf;
  gt_check_inside(g, p, cin, cout, onsurf);
  if (onsurf) return 0.;
  if ((in && cout) || (!in && cin)) return -1.;
  double vX[4], vY[4];
  const double dzp = g.dz + p.z;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    vX[i] = gt_xa(g, i) + g.tx1[i] * dzp;
    vY[i] = gt_ya(g, i) + g.ty1[i] * dzp;
  }
  double umin = 0.;
  for (int i = 0; i < 4; ++i) {
    if (!gt_bit(g.curved, i)) {
      const double sface = fabs(gt_dot_ap(g, i, p));
      if (sface < safplanar) safplanar = sface;
      continue;
    }
    const int j      = (i + 1) & 3;
    const double dx  = vX[j] - vX[i];
    const double dy  = vY[j] - vY[i];
    double dpx       = p.x - vX[i];
    double dpy       = p.y - vY[i];
    const double lsq = dx * dx + dy * dy;
    const double u   = (dpx * dx + dpy * dy) / nonzero(lsq);
    if (u > 1) {
      dpx = p.x - vX[j];
      dpy = p.y - vY[j];
    }
    if (u >= 0 && u <= 1) {
      dpx = dpx - u * dx;
      dpy = dpy - u * dy;
    }
    const double ssq = dpx * dpx + dpy * dpy;
    if (ssq < safety) {
      dx1    = gt_xc(g, i) - gt_xa(g, i);
      dx2    = gt_xd(g, i) - gt_xb(g, i);
      dy1    = gt_yc(g, i) - gt_ya(g, i);
      dy2    = gt_yd(g, i) - gt_yb(g, i);
      umin   = u;
      safety = ssq;
    }
  }
  if (umin < 0 || umin > 1) umin = 0.;
  const double dx = dx1 + umin * (dx2 - dx1);
  const double dy = dy1 + umin * (dy2 - dy1);
  safety *= 1. - 4. * g.dz * g.dz / (dx * dx + dy * dy + 4. * g.dz * g.dz);
  safety = sqrt(safety);
  if (safplanar < safety) safety = safplanar;
  return safety;
}

static __device__ __noinline__ double gentrap_safety_in(const GenTrapRec &g, V3 p)
{
  const V3 q{p.x - g.bborig[0], p.y - g.bborig[1], p.z - g.bborig[2]};
  const double bbsafety = max3(fabs(q.x) - g.bbdim[0], fabs(q.y) - g.bbdim[1], fabs(q.z) - g.bbdim[2]);
  if (!(bbsafety < 0.)) return bbsafety; // outside the bounding box: its safety
  const double eps = 100. * kTolerance;
  double safety    = fabs(p.z) - g.dz;
  if (fabs(safety) < eps) return safety;
  if (g.planar) {
    for (int i = 0; i < 4; ++i) {
      if (gt_bit(g.degenerated, i)) continue;
      const double sf = gt_dot_ap(g, i, p);
      if (sf > safety) safety = sf;
    }
    if (fabs(safety) < eps) safety = 0.;
    return safety;
  }
  const double sf = gt_safety_curved(g, p, false);
  if (sf > safety) safety = sf;
  if (safety > 0. && safety < eps) safety = 0.;
  return safety;
}

static __device__ __noinline__ double gentrap_safety_out(const GenTrapRec &g, V3 p)
{
  const double eps = 100. * kTolerance;
  double safety    = g.dz - fabs(p.z);
  if (fabs(safety) < eps) return safety;
  if (g.planar) {
    for (int i = 0; i < 4; ++i) {
      if (gt_bit(g.degenerated, i)) continue;
      // (a - p) . n
      const double sf = (gt_xa(g, i) - p.x) * g.normal[i][0] + (gt_ya(g, i) - p.y) * g.normal[i][1] +
                        (-g.dz - p.z) * g.normal[i][2];
      if (sf < safety) safety = sf;
    }
    if (fabs(safety) < eps) safety = 0.;
    return safety;
  }
  const double sf = gt_safety_curved(g, p, true);
  if (sf < safety) safety = sf;
  if (safety > 0. && safety < eps) safety = 0.;
  return safety;
}

} // namespace f64
} // namespace vg
