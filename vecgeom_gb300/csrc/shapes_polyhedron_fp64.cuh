// FP64 Polyhedron kernels on the flattened record (PolyhedronRec, vg_types.h): the scalar
// path of VecGeom/volumes/kernel/PolyhedronImplementation.h with EInnerRadii::kGeneric and
// EPhiCutout::kGeneric (the specialisation UnplacedPolyhedron uses), over quadrilateral
// sets as in VecGeom/volumes/Quadrilaterals.h and plane sets as in VecGeom/volumes/Planes.h.
// Same operation order as the reference, so results are bit-identical in FP64.
#pragma once
#include "shapes_fp64.cuh"

namespace vg {
namespace f64 {

// A set of quadrilaterals: n records of kPolyQuadDoubles doubles.
struct QuadSet {
  const double *q;
  int n;
  __device__ const double *at(int i) const { return q + kPolyQuadDoubles * i; }
};

__device__ __forceinline__ V3 qnormal(const double *q) { return V3{__ldg(q), __ldg(q + 1), __ldg(q + 2)}; }
__device__ __forceinline__ double qplane(const double *q, V3 p) // point.Dot(normal) + distance
{
  return p.x * __ldg(q) + p.y * __ldg(q + 1) + p.z * __ldg(q + 2) + __ldg(q + 3);
}
__device__ __forceinline__ double qside(const double *q, int j, V3 x) // side plane j
{
  const double *s = q + 4 + 4 * j;
  return x.x * __ldg(s) + x.y * __ldg(s + 1) + x.z * __ldg(s + 2) + __ldg(s + 3);
}
__device__ __forceinline__ V3 qcorner(const double *q, int k)
{
  return V3{__ldg(q + 20 + 3 * k), __ldg(q + 21 + 3 * k), __ldg(q + 22 + 3 * k)};
}

// Planes::Contains (Planes.h:192-206)
__device__ __forceinline__ bool qs_contains(QuadSet s, V3 p)
{
  for (int i = 0; i < s.n; ++i)
    if (!(qplane(s.at(i), p) < 0)) return false;
  return true;
}
// Planes::Inside (Planes.h:246-266)
__device__ __forceinline__ int qs_inside(QuadSet s, V3 p)
{
  int result = kInside;
  for (int i = 0; i < s.n; ++i) {
    const double r = qplane(s.at(i), p);
    if (r > kHalfTolerance) result = kOutside;
    if (result == kInside && r > -kHalfTolerance) result = kSurface;
    if (result == kOutside) break;
  }
  return result;
}
__device__ __forceinline__ int qs_inside1(QuadSet s, V3 p, int i) // Planes.h:268-281
{
  int result     = kInside;
  const double r = qplane(s.at(i), p);
  if (r > kHalfTolerance) result = kOutside;
  if (result == kInside && r > -kHalfTolerance) result = kSurface;
  return result;
}
__device__ __forceinline__ bool qs_rayhits(const double *q, V3 x) // Quadrilaterals.h:107-117
{
  for (int j = 0; j < 4; ++j)
    if (!(qside(q, j, x) >= -kTolerance)) return false;
  return true;
}

// Quadrilaterals::DistanceToIn<double, behindPlanesT> (Quadrilaterals.h:326-376)
static __device__ __noinline__ double qs_dist_in(QuadSet s, V3 p, V3 d, bool behind)
{
  double best = kInfLength;
  for (int i = 0; i < s.n; ++i) {
    const double *q  = s.at(i);
    const V3 n       = qnormal(q);
    double distance  = dot(p, n) + __ldg(q + 3);
    if (!((behind ? -distance : distance) > -kTolerance)) continue;
    const double proj = dot(d, n);
    if (!((behind ? proj : -proj) > 0)) continue;
    distance /= -(proj + copysign(1E-20, proj));
    const V3 x = V3{p.x + d.x * distance, p.y + d.y * distance, p.z + d.z * distance};
    bool valid = true;
    for (int j = 0; j < 4; ++j) {
      valid &= qside(q, j, x) >= -kTolerance;
      if (!valid) break;
    }
    if (valid) best = distance;
    if (best < kInfLength) break;
  }
  return dmax(0., best);
}

// Quadrilaterals::DistanceToOut(point, direction, zMin, zMax) (Quadrilaterals.h:447-496)
static __device__ __noinline__ double qs_dist_out(QuadSet s, V3 p, V3 d, double zMin, double zMax)
{
  double best = kInfLength;
  for (int i = 0; i < s.n; ++i) {
    const double *q = s.at(i);
    const V3 n      = qnormal(q);
    double t        = dot(p, n) + __ldg(q + 3);
    if (!(t < kTolerance)) continue;
    const double proj = dot(d, n);
    if (!(proj > 0)) continue;
    t /= -proj;
    if (!(t < best)) continue;
    bool valid;
    if (zMin == zMax) {
      valid = qs_rayhits(q, V3{p.x + t * d.x, p.y + t * d.y, p.z + t * d.z});
    } else {
      const double zp = p.z + t * d.z;
      valid           = (zp >= zMin - kTolerance) && (zp < zMax + kTolerance);
    }
    if (!valid) continue;
    best = t;
  }
  if (best > -kTolerance) best = dmax(best, 0.);
  return best;
}

// DistanceToLineSegmentSquared1 (GenericKernels.h:190-215)
__device__ __forceinline__ double line_segment_sq(V3 c0, V3 c1, V3 p)
{
  const V3 line     = V3{c1.x - c0.x, c1.y - c0.y, c1.z - c0.z};
  const V3 proj     = V3{p.x - c0.x, p.y - c0.y, p.z - c0.z};
  const double dot0 = dot(proj, line);
  if (dot0 <= 0) return dot(proj, proj);
  const double dot1 = dot(line, line);
  if (dot1 <= dot0) {
    const V3 e = V3{p.x - c1.x, p.y - c1.y, p.z - c1.z};
    return dot(e, e);
  }
  const double t = dot0 / dot1;
  const V3 e     = V3{(c0.x + t * line.x) - p.x, (c0.y + t * line.y) - p.y, (c0.z + t * line.z) - p.z};
  return dot(e, e);
}

// Quadrilaterals::ScalarDistanceSquared (Quadrilaterals.h:507-578)
__device__ __forceinline__ double qs_dist_sq(const double *q, V3 p)
{
  const V3 n            = qnormal(q);
  const double distance = dot(p, n) + __ldg(q + 3);
  const V3 x            = V3{p.x - distance * n.x, p.y - distance * n.y, p.z - distance * n.z};
  bool within[4];
  for (int j = 0; j < 4; ++j) within[j] = qside(q, j, x) >= 0;
  if (within[0] && within[1] && within[2] && within[3]) return distance * distance;
  double dsq = kInfLength;
  for (int j = 0; j < 4; ++j)
    if (!within[j]) {
      const double dl = line_segment_sq(qcorner(q, j), qcorner(q, (j + 1) % 4), p);
      if (dl < dsq) dsq = dl;
    }
  return dsq;
}

struct PolyhedronView {
  const double *r;
  int S, nseg, nz, flags, oZ, oRmin, oRmax, oSameZ, oPhiSec, oSeg;
  const PolyhedronRec *h;
  __device__ explicit PolyhedronView(const PolyhedronRec &rec)
      : r(&rec.nsides), S((int)rec.nsides), nseg((int)rec.nseg), nz((int)rec.nz), flags((int)rec.flags),
        oZ((int)rec.offZ), oRmin((int)rec.offRMin), oRmax((int)rec.offRMax), oSameZ((int)rec.offSameZ),
        oPhiSec((int)rec.offPhiSec), oSeg((int)rec.offSeg), h(&rec)
  {
  }
  __device__ bool inner() const { return flags & kPolyFlagInner; }
  __device__ bool phi() const { return flags & kPolyFlagPhi; }
  __device__ bool largePhi() const { return flags & kPolyFlagLargePhi; }
  __device__ double z(int i) const { return __ldg(r + oZ + i); }
  __device__ double rmin(int i) const { return __ldg(r + oRmin + i); }
  __device__ double rmax(int i) const { return __ldg(r + oRmax + i); }
  __device__ bool sameZ(int i) const { return __ldg(r + oSameZ + i) != 0.; }
  __device__ V3 phisec(int i) const
  {
    const double *v = r + oPhiSec + 3 * i;
    return V3{__ldg(v), __ldg(v + 1), __ldg(v + 2)};
  }
  __device__ QuadSet outer(int s) const
  {
    const double *e = r + oSeg + 4 * s;
    return QuadSet{r + (int)__ldg(e + 3), (int)__ldg(e)};
  }
  __device__ QuadSet phis(int s) const
  {
    const double *e = r + oSeg + 4 * s;
    return QuadSet{r + (int)__ldg(e + 3) + kPolyQuadDoubles * (int)__ldg(e), (int)__ldg(e + 1)};
  }
  __device__ QuadSet inners(int s) const
  {
    const double *e = r + oSeg + 4 * s;
    return QuadSet{r + (int)__ldg(e + 3) + kPolyQuadDoubles * ((int)__ldg(e) + (int)__ldg(e + 1)), (int)__ldg(e + 2)};
  }
  __device__ bool hasInnerRadius(int s) const { return __ldg(r + oSeg + 4 * s + 2) > 0.; }
  // FindZSegmentKernel (PolyhedronImplementation.h:288-305)
  __device__ int findZ(double pz) const
  {
    int index = -1, b = 0;
    while (b < nz - 1 && pz - kTolerance > z(b)) {
      ++index;
      ++b;
    }
    if (pz + kTolerance > z(b)) return index + 1;
    return index;
  }
  // FindPhiSegment (PolyhedronImplementation.h:318-343)
  __device__ int findPhi(V3 p) const
  {
    int index = -1;
    V3 ps     = phisec(0);
    double f  = p.x * ps.x + p.y * ps.y + p.z * ps.z;
    for (int i = 1; i < S + 1; ++i) {
      ps               = phisec(i);
      const double sec = p.x * ps.x + p.y * ps.y + p.z * ps.z;
      if (f > -kTolerance && sec < kTolerance) index = i - 1;
      if (index >= 0) break;
      f = sec;
    }
    return index;
  }
};

// DistanceToInZSegment (PolyhedronImplementation.h:345-380)
__device__ __forceinline__ double ph_dist_in_seg(const PolyhedronView &v, int s, V3 p, V3 d)
{
  double distance = qs_dist_in(v.outer(s), p, d, false);
  bool done       = distance < kInfLength;
  if (done) return distance;
  if (v.phi()) distance = qs_dist_in(v.phis(s), p, d, false);
  done |= distance < kInfLength;
  if (done) return distance;
  if (v.hasInnerRadius(s)) distance = qs_dist_in(v.inners(s), p, d, true);
  return distance;
}

// DistanceToOutZSegment (PolyhedronImplementation.h:382-420)
__device__ __forceinline__ double ph_dist_out_seg(const PolyhedronView &v, int s, double zMin, double zMax, V3 p, V3 d)
{
  bool done       = false;
  double distance = kInfLength;
  if (v.hasInnerRadius(s)) {
    distance = qs_dist_in(v.inners(s), p, d, false);
    done     = distance < kInfLength;
    if (done) return distance;
  }
  if (v.phi()) {
    const double distphi = qs_dist_in(v.phis(s), p, d, true);
    if (!done && distance > -kTolerance) distance = distphi;
    done = distance > -kTolerance && distance < kInfLength;
    if (done) return distance;
  }
  const double distout = qs_dist_out(v.outer(s), p, d, zMin, zMax);
  if (!done) distance = distout;
  return distance;
}

// InPhiCutoutWedge (PolyhedronImplementation.h:652-672)
__device__ __forceinline__ bool ph_in_cutout(const PolyhedronView &v, int s, V3 p)
{
  const QuadSet ph = v.phis(s);
  if (ph.n < 2) return false;
  const bool s0 = qplane(ph.at(0), p) >= 0;
  const bool s1 = qplane(ph.at(1), p) >= 0;
  return v.largePhi() ? (s0 || s1) : (s0 && s1);
}

// ScalarDistanceToEndcaps<pointInsideT> (PolyhedronImplementation.h:558-610)
__device__ __forceinline__ void ph_endcaps(const PolyhedronView &v, bool pointInside, V3 p, V3 d, double &distance)
{
  const bool first = pointInside ? (d.z < 0) : !(d.z < 0);
  const int s      = first ? 0 : v.nseg - 1;
  const double zpl = first ? v.z(0) : v.z(v.nseg);
  const double t   = (zpl - p.z) / nonzero(d.z);
  if (t < -kTolerance || t >= distance) return;
  const V3 x = V3{p.x + t * d.x, p.y + t * d.y, p.z + t * d.z};
  if (!qs_contains(v.outer(s), x)) return;
  if (v.hasInnerRadius(s) && qs_contains(v.inners(s), x)) return;
  if (v.phi() && ph_in_cutout(v, s, x)) return;
  distance = t;
}

// ScalarSafetyToEndcapsSquared (PolyhedronImplementation.h:612-650)
__device__ __forceinline__ void ph_safety_endcaps_sq(const PolyhedronView &v, V3 p, double &distSq)
{
  const double firstD = v.z(0) - p.z;
  const double lastD  = v.z(v.nseg) - p.z;
  const bool isFirst  = fabs(firstD) < fabs(lastD);
  const int s         = isFirst ? 0 : v.nseg - 1;
  const double t      = isFirst ? firstD : lastD;
  const double tsq    = t * t;
  if (tsq >= distSq) return;
  const V3 x = V3{p.x, p.y, p.z + t};
  if (!qs_contains(v.outer(s), x)) return;
  if (v.hasInnerRadius(s) && qs_contains(v.inners(s), x)) return;
  if (v.phi() && ph_in_cutout(v, s, x)) return;
  distSq = tsq;
}

__device__ __forceinline__ int ph_wedge_inside(const WedgeRec &w, V3 p)
{
  bool ci = false, co = false;
  wedge_classify(w, p, true, ci, co);
  return co ? kOutside : (ci ? kInside : kSurface);
}

// The reference reads the rmax-edge side vector of the outer set, or of the inner set when
// the outer one is empty (PolyhedronImplementation.h:700-704, 806-809).
__device__ __forceinline__ V3 ph_vout(const PolyhedronView &v, int s, int phiIndex)
{
  const QuadSet o = v.outer(s);
  const double *q = o.n ? o.at(phiIndex) : v.inners(s).at(phiIndex);
  return V3{__ldg(q + 4), __ldg(q + 5), __ldg(q + 6)};
}

// ScalarInsideSegBorder (PolyhedronImplementation.h:792-830)
__device__ __forceinline__ int ph_seg_border(const PolyhedronView &v, V3 p, int zi)
{
  const int phiIndex = v.findPhi(p);
  if (phiIndex < 0) return kOutside;
  const double r = fabs(dot(p, ph_vout(v, zi, phiIndex)));
  const bool in1 = (r > v.rmin(zi) - kTolerance) && (r < v.rmax(zi) + kTolerance);
  const bool in2 = (r > v.rmin(zi + 1) - kTolerance) && (r < v.rmax(zi + 1) + kTolerance);
  if (in1 && in2) {
    if ((r < v.rmin(zi) + kTolerance) || (r > v.rmax(zi) - kTolerance) || (r < v.rmin(zi + 1) + kTolerance) ||
        (r > v.rmax(zi + 1) - kTolerance))
      return kSurface;
    if (v.phi()) return ph_wedge_inside(v.h->w, p);
    return kInside;
  }
  if (!in1 && !in2) return kOutside;
  return kSurface;
}

__device__ __forceinline__ bool ph_in_bounding_tube(const PolyhedronView &v, V3 p)
{
  return tube_contains(v.h->bt, V3{p.x, p.y, p.z - v.h->tubeOffset});
}

// ScalarInsideKernel (PolyhedronImplementation.h:732-790)
static __device__ __noinline__ int ph_inside(const PolyhedronView &v, V3 p)
{
  if (!ph_in_bounding_tube(v, p)) return kOutside;
  int zi = v.findZ(p.z);
  if (zi > v.nseg - 1) zi = v.nseg - 1;
  if (zi < 0) zi = 0;
  if (v.sameZ(zi)) return ph_seg_border(v, p, zi);
  {
    const int io = qs_inside(v.outer(zi), p);
    if (io != kInside) return io;
  }
  if (v.hasInnerRadius(zi)) {
    const int ii = qs_inside(v.inners(zi), p);
    if (ii == kInside) return kOutside;
    if (ii == kSurface) return kSurface;
  }
  if (v.phi()) {
    const int ip = qs_inside(v.phis(zi), p);
    if (ip != kInside) return ip;
  }
  const double dz = fabs(fabs(p.z - v.h->tubeOffset) - 0.5 * (v.z(v.nseg) - v.z(0)));
  if (dz < kTolerance) return kSurface;
  return kInside;
}

// ScalarContainsKernel (PolyhedronImplementation.h:674-730)
static __device__ __noinline__ bool ph_contains(const PolyhedronView &v, V3 p)
{
  if (!ph_in_bounding_tube(v, p)) return false;
  const int zi = v.findZ(p.z);
  if (!((zi >= 0) && (zi < v.nseg))) return false;
  if (v.sameZ(zi)) {
    const int phiIndex = v.findPhi(p);
    if (phiIndex < 0) return false;
    const double r = fabs(dot(p, ph_vout(v, zi, phiIndex)));
    const bool in1 = (r >= v.rmin(zi)) && (r <= v.rmax(zi));
    const bool in2 = (r >= v.rmin(zi + 1)) && (r <= v.rmax(zi + 1));
    return in1 | in2;
  }
  if (!qs_contains(v.outer(zi), p)) return false;
  if (v.hasInnerRadius(zi) && qs_contains(v.inners(zi), p)) return false;
  if (v.phi() && !qs_contains(v.phis(zi), p)) return false;
  return true;
}

// ScalarInsideSegPhi (PolyhedronImplementation.h:832-870)
__device__ __forceinline__ int ph_seg_phi(const PolyhedronView &v, V3 p, int zi, int phiIndex)
{
  if (phiIndex < 0) return kOutside;
  const double dz = fabs(p.z - v.h->tubeOffset) - 0.5 * (v.z(v.nseg) - v.z(0));
  if (dz > kHalfTolerance) return kOutside;
  if (v.sameZ(zi)) return ph_seg_border(v, p, zi);
  {
    const int io = qs_inside1(v.outer(zi), p, phiIndex);
    if (io != kInside) return io;
  }
  if (v.hasInnerRadius(zi)) {
    const int ii = qs_inside1(v.inners(zi), p, phiIndex);
    if (ii == kInside) return kOutside;
    if (ii == kSurface) return kSurface;
  }
  if (v.phi()) {
    const int ip = ph_wedge_inside(v.h->w, p);
    if (ip != kInside) return ip;
  }
  if (fabs(dz) < kHalfTolerance) return kSurface;
  return kInside;
}

// ScalarSafetyToZSegmentSquared (PolyhedronImplementation.h:422-556)
__device__ __forceinline__ double ph_safety_seg_sq(const PolyhedronView &v, int si, int &phiIndex, V3 p, bool ptInside)
{
  const bool cutout = phiIndex < 0;
  double safetySq   = kInfLength;
  const QuadSet ph = v.phis(si), in = v.inners(si), out = v.outer(si);
  const bool hasInner = v.hasInnerRadius(si);
  if (v.phi() && ph.n == 2) {
    if (ptInside || cutout) {
      safetySq         = qs_dist_sq(ph.at(0), p);
      const double saf = qs_dist_sq(ph.at(1), p);
      if (saf < safetySq) safetySq = saf;
      if (cutout) {
        if (v.largePhi() && hasInner) {
          if (in.n > 0) {
            double s2 = qs_dist_sq(in.at(0), p);
            if (s2 < safetySq) {
              phiIndex = 0;
              safetySq = s2;
            }
            if (in.n > 1) {
              s2 = qs_dist_sq(in.at(in.n - 1), p);
              if (s2 < safetySq) {
                phiIndex = in.n - 1;
                safetySq = s2;
              }
            }
          }
        }
        return safetySq;
      }
    }
  }
  if (cutout && si > 0 && si < v.nseg - 1 && v.z(si) == v.z(si + 1)) {
    if (out.n > 0) {
      double so = qs_dist_sq(out.at(0), p);
      if (so < safetySq) {
        phiIndex = 0;
        safetySq = so;
      }
      if (out.n > 1) {
        so = qs_dist_sq(out.at(out.n - 1), p);
        if (so < safetySq) {
          phiIndex = out.n - 1;
          safetySq = so;
        }
      }
    }
    if (hasInner && in.n > 0) {
      double s2 = qs_dist_sq(in.at(0), p);
      if (s2 < safetySq) {
        phiIndex = 0;
        safetySq = s2;
      }
      if (in.n > 1) {
        s2 = qs_dist_sq(in.at(in.n - 1), p);
        if (s2 < safetySq) {
          phiIndex = in.n - 1;
          safetySq = s2;
        }
      }
    }
    return safetySq;
  }
  double so = kInfLength;
  if (out.n > 0) so = qs_dist_sq(out.at(phiIndex), p);
  double s2 = kInfLength;
  if (hasInner && in.n > 0) s2 = qs_dist_sq(in.at(phiIndex), p);
  if (s2 < safetySq) safetySq = s2;
  if (so < safetySq) safetySq = so;
  return safetySq;
}

// ScalarSafetyKernel (PolyhedronImplementation.h:947-990)
static __device__ __noinline__ double ph_safety(const PolyhedronView &v, V3 p, bool ptInside)
{
  double safety = kInfLength;
  const int zMax = v.nseg;
  int zi         = v.findZ(p.z);
  zi             = zi < 0 ? 0 : (zi >= zMax ? zMax - 1 : zi);
  int phiIndex   = v.findPhi(p);
  const int ins  = ph_seg_phi(v, p, zi, phiIndex);
  if (ins == kSurface) return 0.;
  const bool contains = (ins == kInside);
  if (contains ^ ptInside) return -1.;
  for (int z = zi; z < zMax;) {
    safety = dmin(safety, ph_safety_seg_sq(v, z, phiIndex, p, ptInside));
    ++z;
    const double dz = v.z(z) - p.z;
    if (dz * dz > safety) break;
  }
  for (int z = zi - 1; z >= 0; --z) {
    safety          = dmin(safety, ph_safety_seg_sq(v, z, phiIndex, p, ptInside));
    const double dz = p.z - v.z(z);
    if (dz * dz > safety) break;
  }
  ph_safety_endcaps_sq(v, p, safety);
  return sqrt(safety);
}

// ScalarDistanceToInKernel (PolyhedronImplementation.h:872-945)
static __device__ __noinline__ double ph_dist_in(const PolyhedronView &v, V3 p, V3 d)
{
  if ((p.z < v.z(0) + kTolerance) && d.z <= 0) return kInfLength;
  if ((p.z > v.z(v.nseg) - kTolerance) && d.z >= 0) return kInfLength;
  if (ph_inside(v, p) == kInside) return -1.;
  double tubeDistance = 0.;
  {
    const V3 bp = V3{p.x, p.y, p.z - v.h->tubeOffset};
    if (!tube_contains(v.h->bt, bp)) {
      tubeDistance = tube_dist_in(v.h->bt, bp, d);
      if (tubeDistance == kInfLength) return kInfLength;
    }
  }
  int zi = v.findZ(p.z);
  zi     = zi < 0 ? 0 : (zi >= v.nseg ? v.nseg - 1 : zi);
  double distance = kInfLength;
  if (d.z >= 0) {
    for (; zi < v.nseg; ++zi) {
      distance = ph_dist_in_seg(v, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = ph_dist_in_seg(v, zi, p, d);
      if (distance >= 0 && distance < kInfLength) break;
    }
  }
  ph_endcaps(v, false, p, d, distance);
  return (distance >= tubeDistance - 1E-6) ? distance : kInfLength;
}

// ScalarDistanceToOutKernel (PolyhedronImplementation.h:1045-1090)
static __device__ __noinline__ double ph_dist_out(const PolyhedronView &v, V3 p, V3 d)
{
  const int zMax = v.nseg;
  if ((p.z < v.z(0) - kTolerance) || (p.z > v.z(zMax) + kTolerance)) return -1.;
  if (ph_inside(v, p) == kOutside) return -1.;
  int zi = v.findZ(p.z);
  zi     = zi < 0 ? 0 : (zi >= zMax ? zMax - 1 : zi);
  double distance = kInfLength;
  if (d.z >= 0) {
    for (; zi < zMax; ++zi) {
      distance = ph_dist_out_seg(v, zi, v.z(zi), v.z(zi + 1), p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (v.z(zi) - p.z > distance) break;
    }
  } else {
    for (; zi >= 0; --zi) {
      distance = ph_dist_out_seg(v, zi, v.z(zi), v.z(zi + 1), p, d);
      if (distance >= 0 && distance < kInfLength) break;
      if (p.z - v.z(zi) > distance) break;
    }
  }
  ph_endcaps(v, true, p, d, distance);
  if (distance >= kInfLength) distance = 0.;
  return distance;
}

__device__ __forceinline__ int polyhedron_inside(const PolyhedronRec &r, V3 p) { return ph_inside(PolyhedronView(r), p); }
__device__ __forceinline__ bool polyhedron_contains(const PolyhedronRec &r, V3 p)
{
  return ph_contains(PolyhedronView(r), p);
}
__device__ __forceinline__ double polyhedron_dist_in(const PolyhedronRec &r, V3 p, V3 d)
{
  return ph_dist_in(PolyhedronView(r), p, d);
}
__device__ __forceinline__ double polyhedron_dist_out(const PolyhedronRec &r, V3 p, V3 d)
{
  return ph_dist_out(PolyhedronView(r), p, d);
}
__device__ __forceinline__ double polyhedron_safety_in(const PolyhedronRec &r, V3 p)
{
  return ph_safety(PolyhedronView(r), p, false);
}
__device__ __forceinline__ double polyhedron_safety_out(const PolyhedronRec &r, V3 p)
{
  return ph_safety(PolyhedronView(r), p, true);
}

} // namespace f64
} // namespace vg
