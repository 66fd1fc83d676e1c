// FP64 device kernels of Torus2 (VecGeom/volumes/kernel/TorusImplementation2.h). The cubic
// resolvent uses CUDA's cbrt/pow/cos/atan2, so roots can differ from the host's by a few
// ulps before the Newton polish; results are compared with a stated tolerance.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {


namespace f64 {

// TorusImplementation2.h:25-61
__device__ __forceinline__ unsigned solve_cubic(double a, double b, double c, double *x)
{
  const double ott     = 1. / 3.;
  const double sq3     = sqrt(3.);
  const double inv6sq3 = 1. / (6. * sq3);
  unsigned ireal       = 1;
  const double p       = b - a * a * ott;
  const double q       = c - a * b * ott + 2. * a * a * a * ott * ott * ott;
  double delta         = 4 * p * p * p + 27. * q * q;
  double t, u;
  if (delta >= 0) {
    delta = sqrt(delta);
    t     = (-3 * q * sq3 + delta) * inv6sq3;
    u     = (3 * q * sq3 + delta) * inv6sq3;
    x[0]  = copysign(1., t) * cbrt(fabs(t)) - copysign(1., u) * cbrt(fabs(u)) - a * ott;
  } else {
    delta = sqrt(-delta);
    t     = -0.5 * q;
    u     = delta * inv6sq3;
    x[0]  = 2. * pow(t * t + u * u, 0.5 * ott) * cos(ott * atan2(u, t));
    x[0] -= a * ott;
  }
  t     = x[0] * x[0] + a * x[0] + b;
  u     = a + x[0];
  delta = u * u - 4. * t;
  if (delta >= 0) {
    ireal = 3;
    delta = sqrt(delta);
    x[1]  = 0.5 * (-u - delta);
    x[2]  = 0.5 * (-u + delta);
  }
  return ireal;
}
__device__ __forceinline__ void cswap(double &a, double &b)
{
  if (a > b) {
    const double c = b;
    b              = a;
    a              = c;
  }
}
__device__ __forceinline__ void sort4(double *x)
{
  cswap(x[0], x[2]);
  cswap(x[1], x[3]);
  cswap(x[0], x[1]);
  cswap(x[2], x[3]);
  cswap(x[1], x[2]);
}
// TorusImplementation2.h:84-150
static __device__ __noinline__ int solve_quartic(double a, double b, double c, double d, double *x)
{
  const double e = b - 3. * a * a / 8.;
  const double f = c + a * a * a / 8. - 0.5 * a * b;
  const double g = d - 3. * a * a * a * a / 256. + a * a * b / 16. - a * c / 4.;
  double xx[4]   = {kInfLength, kInfLength, kInfLength, kInfLength};
  double delta, h = 0.;
  unsigned ireal  = 0;
  if (fabs(f) < 1E-6) {
    delta = e * e - 4. * g;
    if (delta < 0.) return 0;
    delta = sqrt(delta);
    h     = 0.5 * (-e - delta);
    if (h >= 0) {
      h          = sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    h = 0.5 * (-e + delta);
    if (h >= 0) {
      h          = sqrt(h);
      x[ireal++] = -h - 0.25 * a;
      x[ireal++] = h - 0.25 * a;
    }
    sort4(x);
    return ireal;
  }
  if (fabs(g) < 1E-6) {
    x[ireal++]        = -0.25 * a;
    const unsigned nc = solve_cubic(0, e, f, xx);
    for (unsigned i = 0; i < nc; i++) x[ireal++] = xx[i] - 0.25 * a;
    sort4(x);
    return ireal;
  }
  ireal = solve_cubic(2. * e, e * e - 4. * g, -f * f, xx);
  if (ireal == 1) {
    if (xx[0] <= 0) return 0;
    h = sqrt(xx[0]);
  } else {
    for (unsigned i = 0; i < 3; i++) {
      h = xx[i];
      if (h >= 0) break;
    }
    if (h <= 0) return 0;
    h = sqrt(h);
  }
  const double j = 0.5 * (e + h * h - f / h);
  ireal          = 0;
  delta          = h * h - 4. * j;
  if (delta >= 0) {
    delta      = sqrt(delta);
    x[ireal++] = 0.5 * (-h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (-h + delta) - 0.25 * a;
  }
  delta = h * h - 4. * g / j;
  if (delta >= 0) {
    delta      = sqrt(delta);
    x[ireal++] = 0.5 * (h - delta) - 0.25 * a;
    x[ireal++] = 0.5 * (h + delta) - 0.25 * a;
  }
  sort4(x);
  return ireal;
}

// TorusImplementation2.h:252-290
__device__ __forceinline__ void torus_classify(const TorusRec &t, V3 p, bool forInside, bool notForDisk, bool &cin,
                                               bool &cout)
{
  const double tol   = 100. * kTolerance;
  const double rxy   = sqrt(p.x * p.x + p.y * p.y);
  const double radsq = (rxy - t.rtor) * (rxy - t.rtor) + p.z * p.z;
  if (forInside) {
    cout = radsq > (tol * t.rmax + t.rmax2);
    cin  = radsq < (-tol * t.rmax + t.rmax2);
  } else {
    cout = radsq > t.rmax2;
  }
  if (cout) return;
  if (forInside) {
    cout = radsq < (-tol * t.rmin + t.rmin2);
    cin  = cin && (radsq > (tol * t.rmin + t.rmin2));
  } else {
    cout = radsq < t.rmin2;
  }
  if (cout) return;
  if (t.dphi < kTwoPi && notForDisk) {
    bool ci = false, co = false;
    wedge_classify(t.w, p, forInside, ci, co);
    cout = co;
    if (forInside) cin = cin && ci;
  }
}
__device__ __forceinline__ int torus_inside(const TorusRec &t, V3 p)
{
  bool cin = false, cout = false;
  torus_classify(t, p, true, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
// Contains takes the tolerant kernel without the phi test (TorusImplementation2.h:411-420)
__device__ __forceinline__ bool torus_contains(const TorusRec &t, V3 p)
{
  bool cin = false, cout = false;
  torus_classify(t, p, true, false, cin, cout);
  return !cout;
}

__device__ __forceinline__ double quartic(double s, double a, double b, double c, double d)
{
  return s * s * s * s + a * s * s * s + b * s * s + c * s + d;
}
__device__ __forceinline__ double quartic_d(double s, double a, double b, double c)
{
  return 4. * s * s * s + 3. * a * s * s + 2. * b * s + c;
}

// TorusImplementation2.h:292-389 ToBoundary
static __device__ __noinline__ double torus_to_boundary(const TorusRec &t, V3 pt, V3 dir, double radius, bool out)
{
  const double tol    = 100. * kTolerance;
  const double r0sq   = pt.x * pt.x + pt.y * pt.y + pt.z * pt.z;
  const double rdotn  = pt.x * dir.x + pt.y * dir.y + pt.z * dir.z;
  const double rsumsq = t.rtor2 + radius * radius;
  const double a      = 4. * rdotn;
  const double b      = 2. * (r0sq + 2. * rdotn * rdotn - rsumsq + 2. * t.rtor2 * dir.z * dir.z);
  const double c      = 4. * (r0sq * rdotn - rsumsq * rdotn + 2. * t.rtor2 * pt.z * dir.z);
  const double d      = r0sq * r0sq - 2. * r0sq * rsumsq + 4. * t.rtor2 * pt.z * pt.z +
                   (t.rtor2 - radius * radius) * (t.rtor2 - radius * radius);
  double x[4] = {kInfLength, kInfLength, kInfLength, kInfLength};
  int nsol    = 0;
  if (fabs(dir.z) < 1E-3 && fabs(pt.z) < 0.1 * radius) {
    const double invdirxy2 = 1. / (1 - dir.z * dir.z);
    const double b0        = (pt.x * dir.x + pt.y * dir.y) * invdirxy2;
    for (int side = 0; side < 2; ++side) {
      const double root = sqrt((radius - pt.z) * (radius + pt.z));
      const double r0   = side == 0 ? t.rtor - root : t.rtor + root;
      const double c0   = (pt.x * pt.x + (pt.y - r0) * (pt.y + r0)) * invdirxy2;
      const double del  = b0 * b0 - c0;
      if (del > 0) {
        x[nsol] = -b0 - sqrt(del);
        if (x[nsol] > -tol) nsol++;
        x[nsol] = -b0 + sqrt(del);
        if (x[nsol] > -tol) nsol++;
      }
    }
    if (nsol) sort4(x);
  } else {
    nsol = solve_quartic(a, b, c, d, x);
  }
  if (!nsol) return kInfLength;
  const bool inner = fabs(radius - t.rmin) < kTolerance;
  for (int i = 0; i < nsol; i++) {
    if (x[i] < -10) continue;
    V3 r0{pt.x + x[i] * dir.x, pt.y + x[i] * dir.y, pt.z + x[i] * dir.z};
    V3 norm           = r0;
    r0.z              = 0.;
    const double inv  = 1. / sqrt(r0.x * r0.x + r0.y * r0.y + r0.z * r0.z);
    r0                = V3{r0.x * inv, r0.y * inv, r0.z * inv};
    r0                = V3{r0.x * t.rtor, r0.y * t.rtor, r0.z * t.rtor};
    norm              = V3{norm.x - r0.x, norm.y - r0.y, norm.z - r0.z};
    const double ndotd = dot(norm, dir);
    if (inner ^ out) {
      if (ndotd < 0) continue;
    } else {
      if (ndotd > 0) continue;
    }
    if (t.dphi < kTwoPi) {
      bool ci = false, co = false;
      wedge_classify(t.w, r0, true, ci, co);
      if (co) continue;
    }
    double s    = x[i];
    double eps  = kInfLength;
    double eps0 = -quartic(s, a, b, c, d) / quartic_d(s, a, b, c);
    for (int ntry = 0; fabs(eps) > kTolerance;) {
      if (fabs(eps0) > 100) break;
      s += eps0;
      if (fabs(s + eps0) < kTolerance) break;
      eps = -quartic(s, a, b, c, d) / quartic_d(s, a, b, c);
      if (fabs(eps) >= fabs(eps0)) break;
      ntry++;
      if (ntry > 100) break;
      eps0 = eps;
    }
    if (s < -tol) continue;
    return dmax(0., s);
  }
  return kInfLength;
}

// TorusImplementation2.h:140-222
static __device__ __noinline__ double torus_dist_out(const TorusRec &t, V3 p, V3 dir)
{
  const double rsq       = p.x * p.x + p.y * p.y;
  const double outerExcl = t.rtor + t.rmax + kHalfTolerance;
  const double innerExcl = t.rtor - t.rmax - kHalfTolerance;
  if (fabs(p.z) - t.rmax > kHalfTolerance || rsq > outerExcl * outerExcl || rsq < innerExcl * innerExcl) return -1.;
  if (torus_inside(t, p) == kOutside) return -1.;
  double distance = torus_to_boundary(t, p, dir, t.rmax, true);
  if (t.rmin > 0) distance = dmin(distance, torus_to_boundary(t, p, dir, t.rmin, true));
  if (t.dphi < kTwoPi) {
    const double comp1 = dir.x * t.w.n1x + dir.y * t.w.n1y;
    const double comp2 = dir.x * t.w.n2x + dir.y * t.w.n2y;
    double dp1 = kInfLength, dp2 = kInfLength;
    if (comp1 < 0.) {
      const double s = -(p.x * t.w.n1x + p.y * t.w.n1y) / comp1;
      if (s > 0.) dp1 = s;
    }
    if (comp2 < 0.) {
      const double s = -(p.x * t.w.n2x + p.y * t.w.n2y) / comp2;
      if (s > 0.) dp2 = s;
    }
    bool ci, co;
    if (dp1 < distance) {
      const V3 ip{p.x + dir.x * dp1, p.y + dir.y * dp1, p.z + dir.z * dp1};
      co = false;
      torus_classify(t, ip, false, false, ci, co);
      if (!co && ip.x * t.w.a1x + ip.y * t.w.a1y >= 0) distance = dp1;
    }
    if (dp2 < distance) {
      const V3 ip{p.x + dir.x * dp2, p.y + dir.y * dp2, p.z + dir.z * dp2};
      co = false;
      torus_classify(t, ip, false, false, ci, co);
      if (!co && ip.x * t.w.a2x + ip.y * t.w.a2y >= 0) distance = dp2;
    }
  }
  return distance >= kInfLength ? -1. : distance;
}

// TorusImplementation2.h:421-488 (VECGEOM_NO_SPECIALIZATION branch)
static __device__ __noinline__ double torus_dist_in(const TorusRec &t, V3 p, V3 dir)
{
  const bool inBounds = tube_contains(t.bt, p);
  const double tubeDistance = inBounds ? 0. : tube_dist_in(t.bt, p, dir);
  if (inBounds) {
    if (torus_inside(t, p) == kInside) return -1.;
  } else if (tubeDistance == kInfLength) {
    return kInfLength;
  }
  const V3 lp{p.x + tubeDistance * dir.x, p.y + tubeDistance * dir.y, p.z + tubeDistance * dir.z};
  double distance = kInfLength;
  if (t.dphi < kTwoPi) {
    double d1 = kInfLength, d2 = kInfLength;
    const double comp1 = dir.x * t.w.n1x + dir.y * t.w.n1y;
    const double comp2 = dir.x * t.w.n2x + dir.y * t.w.n2y;
    if (comp1 > 0.) {
      const double s = -(lp.x * t.w.n1x + lp.y * t.w.n1y) / comp1;
      if (s > 0.) d1 = s;
    }
    if (comp2 > 0.) {
      const double s = -(lp.x * t.w.n2x + lp.y * t.w.n2y) / comp2;
      if (s > 0.) d2 = s;
    }
    for (int k = 0; k < 2; ++k) {
      const double dk = k == 0 ? d1 : d2;
      if (dk == kInfLength) continue;
      const V3 q{lp.x + dir.x * dk, lp.y + dir.y * dk, lp.z + dir.z * dk};
      const double rxy   = sqrt(q.x * q.x + q.y * q.y);
      const double daxis = (rxy - t.rtor) * (rxy - t.rtor) + q.z * q.z;
      if (daxis >= t.rmin2 && daxis < t.rmax2) {
        distance = k == 0 ? dk : dmin(dk, distance);
        if (fabs(distance) < kTolerance) return distance + tubeDistance;
      }
    }
    distance = kInfLength;
  }
  double dd = torus_to_boundary(t, lp, dir, t.rmax, false);
  if (t.rmin > 0.) dd = dmin(dd, torus_to_boundary(t, lp, dir, t.rmin, false));
  distance = dmin(distance, dd);
  distance += tubeDistance;
  if (fabs(distance) > kInfLength) distance = kInfLength;
  return distance;
}

// TorusImplementation2.h:391-409, 489-510
__device__ __forceinline__ double torus_safety_out(const TorusRec &t, V3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t.rtor) * (rxy - t.rtor) + p.z * p.z);
  double safety    = t.rmax - rad;
  if (t.rmin != 0.) safety = dmin(rad - t.rmin, t.rmax - rad);
  if (t.dphi < kTwoPi) safety = dmin(wedge_safety_out(t.w, p), safety);
  return safety;
}
__device__ __forceinline__ double torus_safety_in(const TorusRec &t, V3 p)
{
  const double rxy = sqrt(p.x * p.x + p.y * p.y);
  const double rad = sqrt((rxy - t.rtor) * (rxy - t.rtor) + p.z * p.z);
  double safety    = rad - t.rmax;
  if (t.rmin != 0.) safety = dmax(t.rmin - rad, rad - t.rmax);
  if (t.dphi < kTwoPi && rxy != 0.) safety = dmax(wedge_safety_in(t.w, p), safety);
  return safety;
}

} // namespace f64
} // namespace vg
