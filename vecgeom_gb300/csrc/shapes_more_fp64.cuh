// FP64 device kernels of Trd and Polycone (same compilation rules as shapes_fp64.cuh).
#pragma once
#include "shapes_fp64.cuh"

namespace vg {



namespace f64 {

constexpr double kTiny = 1e-30;

// ================================================================ Trd
// TrdImplementation.h:138-173 (y faces always take the cross-product test)
__device__ __forceinline__ void trd_classify(const TrdRec &t, V3 p, bool surfaceT, bool &cin, bool &cout)
{
  const double pzPlusDz = p.z + t.dz;
  cout                  = dgt(fabs(p.z), surfaceT ? t.dz + kHalfTolerance : t.dz);
  if (surfaceT) cin = dabs_lt(p.z, t.dz - kHalfTolerance);
  const double cx = t.x2minusx1 * pzPlusDz - (2.0 * t.dz) * (fabs(p.x) - t.dx1);
  const double cy = t.y2minusy1 * pzPlusDz - (2.0 * t.dz) * (fabs(p.y) - t.dy1);
  if (surfaceT) {
    cout = cout || dlt(cx, -t.tolx) || dlt(cy, -t.toly);
    cin  = cin && dgt(cx, t.tolx) && dgt(cy, t.toly);
  } else {
    cout = cout || dlt(cx, 0.) || dlt(cy, 0.);
  }
}
__device__ __forceinline__ int trd_inside(const TrdRec &t, V3 p)
{
  bool in = false, out = false;
  trd_classify(t, p, true, in, out);
  return out ? kOutside : (in ? kInside : kSurface);
}
__device__ __forceinline__ bool trd_contains(const TrdRec &t, V3 p)
{
  bool in = false, out = false;
  trd_classify(t, p, false, in, out);
  return !out;
}
// TrdImplementation.h:69-117 FaceTrajectoryIntersection
__device__ __forceinline__ bool trd_face(const TrdRec &t, V3 pos, V3 dir, bool forY, bool mirrored, bool toInside,
                                         double &dist)
{
  const double alongV = forY ? t.y2minusy1 : t.x2minusx1;
  const double v1     = forY ? t.dy1 : t.dx1;
  double posV         = forY ? pos.y : pos.x;
  double dirV         = forY ? dir.y : dir.x;
  const double posK   = forY ? pos.x : pos.y;
  const double dirK   = forY ? dir.x : dir.y;
  const double fK     = forY ? t.fx : t.fy;
  const double fV     = forY ? t.fy : t.fx;
  const double halfK  = forY ? t.halfx1plusx2 : t.halfy1plusy2;
  if (mirrored) {
    posV = -posV;
    dirV = -dirV;
  }
  const double ndotv = dirV + fV * dir.z;
  if (toInside ? !dlt(ndotv, 0.) : !dgt(ndotv, 0.)) return false;
  const double alongZ = 2.0 * t.dz;
  dist = (alongZ * (posV - v1) - alongV * (pos.z + t.dz)) / (dir.z * alongV - dirV * alongZ + kTiny);
  if (!dgt(dist, -kHalfTolerance)) return false;
  const double hitz = pos.z + dist * dir.z;
  const double hitk = posK + dist * dirK;
  const bool ok     = dabs_le(hitz, t.dz) && dabs_le(hitk, halfK - fK * hitz);
  if (ok && dabs_lt(dist, kHalfTolerance)) dist = 0.0;
  return ok;
}
__device__ __forceinline__ double trd_clamp(double d) { return dabs_lt(d, kHalfTolerance) ? 0.0 : d; }
// TrdImplementation.h:288-370
static __device__ __noinline__ double trd_dist_in(const TrdRec &t, V3 p, V3 d)
{
  double distance  = kInfLength;
  const bool inz   = dabs_lt(p.z, t.dz - kHalfTolerance);
  double distx     = t.halfx1plusx2 - t.fx * p.z;
  const bool inx   = dgt((distx - fabs(p.x)) * t.calfx, kHalfTolerance);
  const bool vary  = dne(t.dy1, t.dy2);
  double disty     = vary ? t.halfy1plusy2 - t.fy * p.z : fabs(p.y) - t.dy1;
  const bool iny   = vary ? dgt((disty - fabs(p.y)) * t.calfy, kHalfTolerance) : dlt(disty, -kHalfTolerance);
  if (inx && iny && inz) return -1.;
  if (dlt(p.z * d.z, 0.) && !inz) {
    const double distz = (fabs(p.z) - t.dz) / fabs(d.z);
    const double hitx  = fabs(p.x + distz * d.x);
    const double hity  = fabs(p.y + distz * d.y);
    const bool okzt    = dgt(p.z, t.dz - kHalfTolerance) && dle(hitx, t.dx2) && dle(hity, t.dy2);
    const bool okzb    = dlt(p.z, -t.dz + kHalfTolerance) && dle(hitx, t.dx1) && dle(hity, t.dy1);
    if (okzt || okzb) return trd_clamp(distz);
  }
  bool okx = false;
  if (!inx) {
    if (trd_face(t, p, d, false, false, true, distx)) distance = distx;
    okx = trd_face(t, p, d, false, true, true, distx);
    if (okx) distance = distx;
  }
  if (okx) return trd_clamp(distance);
  if (!iny) {
    if (vary) {
      if (trd_face(t, p, d, true, false, true, disty)) distance = disty;
      if (trd_face(t, p, d, true, true, true, disty)) distance = disty;
    } else {
      disty /= fabs(d.y);
      const double zhit = p.z + disty * d.z;
      const double xhit = p.x + disty * d.x;
      const double dx   = t.halfx1plusx2 - t.fx * zhit;
      if (dlt(p.y * d.y, 0.) && dgt(disty, -kHalfTolerance) && dabs_lt(xhit, dx) && dabs_lt(zhit, t.dz)) distance = disty;
    }
  }
  return trd_clamp(distance);
}
// TrdImplementation.h:371-470
static __device__ __noinline__ double trd_dist_out(const TrdRec &t, V3 p, V3 d)
{
  const double invdir = 1. / fabs(d.z + kTiny);
  const bool vary     = dne(t.dy1, t.dy2);
  double distx        = t.halfx1plusx2 - t.fx * p.z;
  double disty        = vary ? t.halfy1plusy2 - t.fy * p.z : t.dy1 - fabs(p.y);
  const bool out      = dlt(t.dz - fabs(p.z), -kHalfTolerance) || dlt((distx - fabs(p.x)) * t.calfx, -kHalfTolerance) ||
                   (vary ? dlt((disty - fabs(p.y)) * t.calfy, -kHalfTolerance) : dlt(disty, -kHalfTolerance));
  if (out) return -1.;
  if (dgt(d.z, 0.)) {
    const double distz = (t.dz - p.z) * invdir;
    if (dabs_le(p.x + distz * d.x, t.dx2) && dabs_le(p.y + distz * d.y, t.dy2)) return trd_clamp(distz);
  }
  if (dlt(d.z, 0.)) {
    const double distz = (p.z + t.dz) * invdir;
    if (dabs_le(p.x + distz * d.x, t.dx1) && dabs_le(p.y + distz * d.y, t.dy1)) return trd_clamp(distz);
  }
  if (trd_face(t, p, d, false, false, false, distx)) return trd_clamp(distx);
  if (trd_face(t, p, d, false, true, false, distx)) return trd_clamp(distx);
  double distance = 0.0;
  if (vary) {
    if (trd_face(t, p, d, true, false, false, disty)) return trd_clamp(disty);
    if (trd_face(t, p, d, true, true, false, disty)) distance = disty;
  } else {
    const double plane = dlt(d.y, 0.) ? -t.dy1 : t.dy1;
    disty              = (plane - p.y) / d.y;
    const double zhit  = p.z + disty * d.z;
    const double xhit  = p.x + disty * d.x;
    const double dx    = t.halfx1plusx2 - t.fx * zhit;
    if (dabs_lt(xhit, dx) && dabs_lt(zhit, t.dz)) distance = disty;
  }
  return trd_clamp(distance);
}
// TrdImplementation.h:118-137
__device__ __forceinline__ double trd_safety(const TrdRec &t, V3 p, bool inside)
{
  double dist        = t.dz - fabs(p.z);
  const double distx = t.halfx1plusx2 - t.fx * p.z;
  const double safx  = (distx - fabs(p.x)) * t.calfx;
  if (dge(distx, 0.) && dlt(safx, dist)) dist = safx;
  if (dne(t.dy1, t.dy2)) {
    const double disty = t.halfy1plusy2 - t.fy * p.z;
    const double safy  = (disty - fabs(p.y)) * t.calfy;
    if (dge(disty, 0.) && dlt(safy, dist)) dist = safy;
  } else {
    const double safy = t.dy1 - fabs(p.y);
    if (dlt(safy, dist)) dist = safy;
  }
  return inside ? dist : -dist;
}
__device__ __forceinline__ double trd_safety_in(const TrdRec &t, V3 p) { return trd_safety(t, p, false); }
__device__ __forceinline__ double trd_safety_out(const TrdRec &t, V3 p) { return trd_safety(t, p, true); }

// ================================================================ Trap
// Two z planes at +-dz and four side planes (PlaneShell<4>, VecGeom/base/PlaneShell.h),
// evaluated in the reference's order: plane value a x + b y + c z + d summed left to right.
__device__ __forceinline__ double trap_plane(const TrapRec &t, int i, V3 p)
{
  return t.a[i] * p.x + t.b[i] * p.y + t.c[i] * p.z + t.d[i];
}
__device__ __forceinline__ double trap_proj(const TrapRec &t, int i, V3 v)
{
  return t.a[i] * v.x + t.b[i] * v.y + t.c[i] * v.z;
}
// TrapezoidImplementation.h:65-106 + PlaneShell.h GenericKernelForContainsAndInside: outside
// beyond dz + tol or a plane value above tol; inside within dz - tol and every plane value
// below -tol (inside is assigned last)
__device__ __forceinline__ int trap_inside(const TrapRec &t, V3 p)
{
  bool out = dlt(t.dz_plus, fabs(p.z));
  bool in  = dabs_lt(p.z, t.dz_minus);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double s = trap_plane(t, i, p);
    out            = out || dgt(s, kHalfTolerance);
    in             = in && dlt(s, -kHalfTolerance);
  }
  return in ? kInside : (out ? kOutside : kSurface);
}
__device__ __forceinline__ bool trap_contains(const TrapRec &t, V3 p)
{
  bool out = dlt(t.dz, fabs(p.z));
#pragma unroll
  for (int i = 0; i < 4; ++i) out = out || dgt(trap_plane(t, i, p), 0.);
  return !out;
}
// TrapezoidImplementation.h:107-126 + PlaneShell.h DistanceToIn. The z slab gives [smin, smax];
// each side plane the ray crosses inward raises smin, outward lowers smax; kInfLength as soon
// as the ray provably misses. The reference tests every plane for the first kind of miss
// before clipping; any miss returns kInfLength, so one pass in plane order gives the same
// value. Exit distances -pdist / proj are divided only for the planes that use them.
static __device__ __noinline__ double trap_dist_in(const TrapRec &t, V3 p, V3 d)
{
  const double sdz = flipsign(t.dz, d.z); // Sign(d.z) * dz
  const double max = sdz - p.z;
  if (dlt(flipsign(max, d.z), kHalfTolerance)) return kInfLength;
  const double invdir = 1.0 / nonzero(d.z);
  double smax         = max * invdir;
  double smin         = -(sdz + p.z) * invdir;
  bool pos[4], dirp[4];
  double pd[4], pj[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pd[i]   = trap_plane(t, i, p);
    pj[i]   = trap_proj(t, i, d);
    pos[i]  = dgt(pd[i], -kHalfTolerance);
    dirp[i] = dgt(pj[i], 0.);
    if ((dgt(pd[i], kHalfTolerance) && dge(pj[i], 0.)) || (pos[i] && dirp[i])) return kInfLength;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const bool fromIn = !pos[i] && dirp[i], fromOut = pos[i] && !dirp[i];
    if (fromIn || fromOut) {
      const double v = -pd[i] / nonzero(pj[i]);
      if (fromIn) {
        if (dlt(v, smin)) return kInfLength;
        if (dlt(v, smax)) smax = v;
      } else {
        if (dgt(v, smax)) return kInfLength;
        if (dgt(v, smin)) smin = v;
      }
    }
  }
  return dle(smin, smax) ? smin : kInfLength;
}
// TrapezoidImplementation.h:151-167 + PlaneShell.h DistanceToOut: -1 beyond dz + tol;
// otherwise the z exit, lowered by the plane pass (-1 when outside a plane, then any smaller
// exit distance, planes in order).
static __device__ __noinline__ double trap_dist_out(const TrapRec &t, V3 p, V3 d)
{
  if (dlt(t.dz_plus, fabs(p.z))) return -1.;
  double distance = kInfLength;
  if (dne(d.z, 0.)) distance = (flipsign(t.dz, d.z) - p.z) / nonzero(d.z);
  double out = kInfLength;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const double pd = trap_plane(t, i, p);
    const double pj = trap_proj(t, i, d);
    if (dgt(pd, kHalfTolerance)) out = -1.;
    if (dgt(pj, 0.)) {
      const double v = -pd / nonzero(pj);
      if (dlt(v, out)) out = v;
    }
  }
  return dlt(out, distance) ? out : distance;
}
// TrapezoidImplementation.h:183-218 + PlaneShell.h SafetyToIn / SafetyToOut (N = 4): the
// z-plane value, then the largest (smallest, negated) plane value taken in plane order
__device__ __forceinline__ double trap_safety_in(const TrapRec &t, V3 p)
{
  double safety = fabs(p.z) - t.dz;
#pragma unroll
  for (int i = 0; i < 4; ++i) safety = dmax(trap_plane(t, i, p), safety);
  return safety;
}
__device__ __forceinline__ double trap_safety_out(const TrapRec &t, V3 p)
{
  double safety = t.dz - fabs(p.z);
#pragma unroll
  for (int i = 0; i < 4; ++i) safety = dmin(-trap_plane(t, i, p), safety);
  return safety;
}

// ================================================================ Polycone
struct PolyconeView {
  const double *r;
  int nsec;
  __device__ PolyconeView(const PolyconeRec &rec) : r(&rec.nsec), nsec((int)rec.nsec) {}
  __device__ double z(int i) const { return r[4 + i]; }
  __device__ const double *sec(int i) const { return r + polycone_section_base(nsec) + i * kPolyconeSectionDoubles; }
  __device__ double shift(int i) const { return sec(i)[0]; }
  __device__ const ConeRec &cone(int i) const { return *reinterpret_cast<const ConeRec *>(sec(i) + 4); }
  __device__ V3 local(V3 p, int i) const { return V3{p.x, p.y, p.z - shift(i)}; }
  // PolyconeStruct.h:246-253 GetSectionIndex
  __device__ int index(double zp) const
  {
    if (dlt(zp, z(0))) return -1;
    for (int i = 0; i < nsec; ++i)
      if (dge(zp, z(i)) && dle(zp, z(i + 1))) return i;
    return -2;
  }
};

// PolyconeImplementation.h:58-147
__device__ __forceinline__ void pc_section(const PolyconeView &v, int i, V3 p, bool forInside, bool &cin, bool &cout)
{
  if (i < 0) {
    cin  = false;
    cout = true;
    return;
  }
  cone_classify(v.cone(i), v.local(p, i), forInside, cin, cout);
}
static __device__ __noinline__ void polycone_classify(const PolyconeRec &rec, V3 p, bool forInside, bool &cin, bool &cout)
{
  const PolyconeView v(rec);
  const int lo = v.index(p.z - kTolerance);
  const int hi = v.index(p.z + kTolerance);
  if (lo < 0 && hi < 0) {
    cout = true;
    return;
  }
  if (lo < 0 && hi == 0) return pc_section(v, 0, p, forInside, cin, cout);
  if (hi < 0 && lo == v.nsec - 1) return pc_section(v, v.nsec - 1, p, forInside, cin, cout);
  if (lo >= 0 && hi >= 0) {
    if (lo == hi) return pc_section(v, lo, p, forInside, cin, cout);
    bool inL = false, outL = false, inH = false, outH = false;
    pc_section(v, lo, p, forInside, inL, outL);
    pc_section(v, hi, p, forInside, inH, outH);
    if (!inL && !outL && !inH && !outH) {
      cin = true;
      return;
    }
    if (outL && outH) cout = true;
  }
}
__device__ __forceinline__ int polycone_inside(const PolyconeRec &r, V3 p)
{
  bool cin = false, cout = false;
  polycone_classify(r, p, true, cin, cout);
  return cin ? kInside : (cout ? kOutside : kSurface);
}
__device__ __forceinline__ bool polycone_contains(const PolyconeRec &r, V3 p)
{
  bool cin = false, cout = false;
  polycone_classify(r, p, false, cin, cout);
  return !cout;
}
// PolyconeImplementation.h:148-180
static __device__ __noinline__ double polycone_dist_in(const PolyconeRec &rec, V3 p, V3 d)
{
  const PolyconeView v(rec);
  double distance = kInfLength;
  int increment   = dgt(d.z, 0.) ? 1 : -1;
  if (dabs_lt(d.z, kTolerance)) increment = 0;
  int index = v.index(p.z);
  if (index == -1) index = 0;
  if (index == -2) index = v.nsec - 1;
  do {
    distance = cone_dist_in(v.cone(index), v.local(p, index), d);
    if (dlt(distance, kInfLength) || !increment) break;
    index += increment;
  } while (index >= 0 && index < v.nsec);
  return distance;
}
// PolyconeImplementation.h:181-300, in two parts so that a kernel can interleave the
// section loops of different queries on one lane (k_polycone_dist_out_refill): the setup
// before the loop, and one pass of the loop. polycone_dist_out runs them back to back.
struct PolyconeOutLoop {
  V3 point, dir, pn;
  double total;
  int index, increment, istep;
};
// Setup: true with the result in r when the query ends before the section loop.
__device__ __forceinline__ bool polycone_out_setup(const PolyconeView &v, V3 point, V3 dir, double &r,
                                                   PolyconeOutLoop &L)
{
  if (v.nsec == 1) {
    r = cone_dist_out(v.cone(0), v.local(point, 0), dir);
    return true;
  }
  const int lo = v.index(point.z - kTolerance);
  const int hi = v.index(point.z + kTolerance);
  int index    = 0;
  r            = -1.;
  if (lo < 0 && hi < 0) return true;
  if (lo < 0 && hi >= 0) {
    index = hi;
    if (cone_inside(v.cone(index), v.local(point, index)) == kOutside) return true;
  } else if (lo != hi && lo >= 0) {
    index = (cone_inside(v.cone(lo), v.local(point, lo)) == kOutside) ? hi : lo;
  } else {
    index = lo;
    if (index < 0) index = v.index(point.z);
  }
  if (index < 0) {
    r = 0.;
    return true;
  }
  if (cone_inside(v.cone(index), v.local(point, index)) == kOutside) return true;
  L.point     = point;
  L.dir       = dir;
  L.pn        = point;
  L.total     = 0.;
  L.index     = index;
  L.increment = dgt(dir.z, 0.) ? 1 : -1;
  if (dabs_lt(dir.z, kTolerance)) L.increment = 0;
  L.istep = 0;
  return false;
}
// One pass of the section loop: true with the result in r when the query ends.
__device__ __forceinline__ bool polycone_out_pass(const PolyconeView &v, PolyconeOutLoop &L, double &r)
{
  const V3 point = L.point, dir = L.dir;
  if (dne(L.total, 0.) || (L.istep < 2)) {
    L.pn = V3{point.x + L.total * dir.x, point.y + L.total * dir.y, point.z + L.total * dir.z};
    L.pn.z -= v.shift(L.index);
    if (cone_inside(v.cone(L.index), L.pn) == kOutside) {
      r = L.total;
      return true;
    }
  } else {
    L.pn.z -= v.shift(L.index);
  }
  L.istep++;
  const double dist = cone_dist_out(v.cone(L.index), L.pn, dir);
  if (deq(dist, -1.)) {
    r = kInfLength;
    return true;
  }
  if (dabs_lt(dist, 0.5 * kTolerance)) {
    int index1 = L.index;
    if ((L.index > 0) && (L.index < v.nsec - 1)) {
      index1 += L.increment;
    } else {
      if ((L.index == 0) && (L.increment > 0)) index1 += L.increment;
      if ((L.index == v.nsec - 1) && (L.increment < 0)) index1 += L.increment;
    }
    const double s = L.total + dist;
    V3 pte{point.x + s * dir.x, point.y + s * dir.y, point.z + s * dir.z};
    pte.z -= v.shift(index1);
    if (cone_inside(v.cone(index1), pte) == 3 || L.increment == 0) {
      r = L.total;
      return true;
    }
  }
  L.total += dist;
  L.index += L.increment;
  if (L.increment != 0 && L.index >= 0 && L.index < v.nsec) return false;
  r = L.total;
  return true;
}
static __device__ __noinline__ double polycone_dist_out(const PolyconeRec &rec, V3 point, V3 dir)
{
  const PolyconeView v(rec);
  double r;
  PolyconeOutLoop L;
  if (polycone_out_setup(v, point, dir, r, L)) return r;
  while (!polycone_out_pass(v, L, r)) {
  }
  return r;
}
// PolyconeImplementation.h:301-354
static __device__ __noinline__ double polycone_safety_in(const PolyconeRec &rec, V3 p)
{
  const PolyconeView v(rec);
  int index  = v.index(p.z);
  bool needZ = false;
  if (index < 0) {
    needZ = true;
    index = (index == -1) ? 0 : v.nsec - 1;
  }
  double safety = cone_safety_in(v.cone(index), v.local(p, index));
  if (needZ || dlt(safety, kTolerance)) return safety;
  double minSafety = safety;
  double zbase     = v.z(index + 1);
  for (int i = index + 1; i < v.nsec; ++i) {
    if (dge(v.z(i) - zbase, minSafety)) break;
    safety = cone_safety_in(v.cone(i), v.local(p, i));
    if (dlt(safety, minSafety)) minSafety = safety;
  }
  if (index > 0) {
    zbase = v.z(index - 1);
    for (int i = index - 1; i >= 0; --i) {
      if (dge(zbase - v.z(i), minSafety)) break;
      safety = cone_safety_in(v.cone(i), v.local(p, i));
      if (dlt(safety, minSafety)) minSafety = safety;
    }
  }
  return minSafety;
}
// PolyconeImplementation.h:355-410
static __device__ __noinline__ double polycone_safety_out(const PolyconeRec &rec, V3 p)
{
  const PolyconeView v(rec);
  bool cin = false, cout = false;
  polycone_classify(rec, p, true, cin, cout);
  if (cout) return -1;
  const int index = v.index(p.z);
  if (index < 0) return -1;
  double minSafety = cone_safety_out(v.cone(index), v.local(p, index));
  if (deq(minSafety, kInfLength) || dlt(minSafety, kTolerance)) return 0.;
  double zbase = v.z(index + 1);
  for (int i = index + 1; i < v.nsec; ++i) {
    if (dge(v.z(i) - zbase, minSafety)) break;
    const double s = cone_safety_in(v.cone(i), v.local(p, i));
    if (dlt(s, minSafety)) minSafety = s;
  }
  if (index > 0) {
    zbase = v.z(index - 1);
    for (int i = index - 1; i >= 0; --i) {
      if (dge(zbase - v.z(i), minSafety)) break;
      const double s = cone_safety_in(v.cone(i), v.local(p, i));
      if (dlt(s, minSafety)) minSafety = s;
    }
  }
  return minSafety;
}

} // namespace f64
} // namespace vg
