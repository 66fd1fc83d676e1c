// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
// Trd, Polycone, Polyhedron, Torus2 and the boolean subtraction.
#pragma once
#include "ref_shapes.h"
#include <memory>
#include <vector>

namespace oracle {

struct PlacedVolume;

// VecGeom/volumes/TrdStruct.h, VecGeom/volumes/kernel/TrdImplementation.h (UniversalTrd)
struct Trd : UnplacedShape {
  double fDX1, fDX2, fDY1, fDY2, fDZ;
  double fX2minusX1, fY2minusY1, fHalfX1plusX2, fHalfY1plusY2, fCalfX, fCalfY, fSecxz, fSecyz;
  double fToleranceX, fToleranceY, fFx, fFy;
  Trd(double x1, double x2, double y1, double y2, double z);
  bool VaryingY() const { return fDY1 != fDY2; }
  void UnplacedInside(Vec3 const &p, bool surfaceT, bool &cin, bool &cout) const;
  void Face(Vec3 const &pos, Vec3 const &dir, bool forY, bool mirrored, bool toInside, double &dist, bool &ok) const;
  double Safety(Vec3 const &p, bool inside) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override { return Safety(p, false); }
  double SafetyToOut(Vec3 const &p) const override { return Safety(p, true); }
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/TrapezoidStruct.h, source/UnplacedTrapezoid.cpp (construction),
// VecGeom/volumes/kernel/TrapezoidImplementation.h with VecGeom/base/PlaneShell.h (the
// VECGEOM_PLANESHELL build, CMakeLists.txt:156 default ON): two z planes at +-fDz and four
// side planes a x + b y + c z + d = 0 with outward unit normals, in the order -Y, +Y, -X, +X.
struct Trap : UnplacedShape {
  double fDz = 0.;
  double fA[4] = {}, fB[4] = {}, fC[4] = {}, fD[4] = {};
  // UnplacedTrapezoid(dz, theta, phi, dy1, dx1, dx2, alpha1, dy2, dx3, dx4, alpha2), angles in radians
  explicit Trap(const double *par);
  // UnplacedTrapezoid(TrapCorners): corners p0(---) p1(+--) p2(-+-) p3(++-) p4(--+) p5(+-+) p6(-++) p7(+++)
  explicit Trap(const Vec3 *corners);
  // dz and the planes as an UnplacedTrapezoid holds them (TrapezoidStruct GetPlane(0..3))
  Trap(double dz, const double *planes);
  void MakePlanes(const Vec3 *pt);
  void MakeAPlane(Vec3 const &p1, Vec3 const &p2, Vec3 const &p3, Vec3 const &p4, int i);
  double PlaneDist(int i, Vec3 const &p) const { return fA[i] * p.x() + fB[i] * p.y() + fC[i] * p.z() + fD[i]; }
  double PlaneProj(int i, Vec3 const &d) const { return fA[i] * d.x() + fB[i] * d.y() + fC[i] * d.z(); }
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/PolyconeStruct.h (Init), VecGeom/volumes/kernel/PolyconeImplementation.h
struct Polycone : UnplacedShape {
  double fStartPhi = 0, fDeltaPhi = 0;
  std::vector<std::unique_ptr<Cone>> fSolids;
  std::vector<double> fShift;
  std::vector<double> fZs;
  Polycone(double phiStart, double phiTotal, int nz, const double *z, const double *rmin, const double *rmax);
  int NSections() const { return (int)fSolids.size(); }
  int GetSectionIndex(double z) const;
  Vec3 Local(Vec3 const &p, int i) const { return Vec3(p.x(), p.y(), p.z() - fShift[i]); }
  void SectionKernel(int isect, Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/kernel/BooleanImplementation.h (kSubtraction); operands are placed volumes.
struct BooleanMinus : UnplacedShape {
  PlacedVolume const *fLeft, *fRight;
  BooleanMinus(PlacedVolume const *l, PlacedVolume const *r) : fLeft(l), fRight(r) {}
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/ThetaCone_Evolution.h: the theta range [sTheta, sTheta + dTheta] of a
// sphere as two cones about the z axis.
struct ThetaCone {
  double fSTheta, fDTheta, kAngTol, halfAngTol, fETheta, tanSTheta, tanETheta, tanBisector, slope1, slope2,
      tanSTheta2, tanETheta2;
  ThetaCone() {}
  ThetaCone(double sTheta, double dTheta);
  bool IsOnSurfaceGeneric(Vec3 const &p, bool start) const;
  Vec3 GetNormal(Vec3 const &p, bool start) const;
  bool IsPointOnSurfaceAndMovingOut(Vec3 const &p, Vec3 const &d, bool start, bool movingOut) const;
  bool IsCompletelyInside(Vec3 const &p) const;
  bool IsCompletelyOutside(Vec3 const &p) const;
  bool Contains(Vec3 const &p) const { return !IsCompletelyOutside(p); }
  double DistanceToLine(double slope, double x, double y) const;
  double SafetyToIn(Vec3 const &p) const;
  double SafetyToOut(Vec3 const &p) const;
  void DistanceToIn(Vec3 const &p, Vec3 const &d, double &d1, double &d2, bool &i1, bool &i2) const;
  void DistanceToOut(Vec3 const &p, Vec3 const &d, double &d1, double &d2, bool &i1, bool &i2) const;
};

// VecGeom/volumes/SphereStruct.h, VecGeom/volumes/SphereUtilities.h,
// VecGeom/volumes/kernel/SphereImplementation.h, source/UnplacedSphere.cpp.
struct Sphere : UnplacedShape {
  double fRmin, fRmax, fSPhi, fDPhi, fSTheta, fDTheta, eTheta;
  bool fFullPhiSphere = true, fFullThetaSphere = true, fFullSphere = true;
  Wedge fPhiWedge;
  ThetaCone fThetaCone;
  Sphere(double rmin, double rmax, double sphi, double dphi, double stheta, double dtheta);
  // Wedge_Evolution.h:236-245 IsPointOnSurfaceAndMovingOut, :391-432 DistanceToIn / DistanceToOut
  bool WedgeOnSurfaceMoving(Vec3 const &p, Vec3 const &d, bool start, bool movingOut) const;
  void WedgeDistanceToIn(Vec3 const &p, Vec3 const &d, double &d1, double &d2) const;
  void WedgeDistanceToOut(Vec3 const &p, Vec3 const &d, double &d1, double &d2) const;
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  bool IsCompletelyInside(Vec3 const &p) const;
  bool IsCompletelyOutside(Vec3 const &p) const;
  bool IsPointOnSurfaceAndMovingOut(Vec3 const &p, Vec3 const &d, bool movingOut) const;
  void GetMinDistFromPhi(Vec3 const &p, Vec3 const &d, bool toIn, bool done, double &distance) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/GenTrapStruct.h (Initialize, Extent, SegmentsCrossing, convexity, twist),
// VecGeom/volumes/SecondOrderSurfaceShell.h (the four lateral surfaces, planar or twisted)
// and the generic kernels of VecGeom/volumes/kernel/GenTrapImplementation.h, which are the
// kernels the reference's CUDA build and its SIMD backends run. (The scalar CPU build
// routes planar GenTraps through a TessellatedSection instead; that helper is not built
// for CUDA.) The object is the one the reference's device holds: UnplacedGenTrap::CopyToGpu
// (source/UnplacedGenTrap.cpp:343-357) re-initialises the device copy from the host's
// fVerticesX/Y, which Initialize has already reordered clockwise, so the surface shell is
// always built from the clockwise vertices.
struct GenTrap : UnplacedShape {
  // GenTrapStruct
  double fBBdim[3] = {}, fBBorig[3] = {};
  double fVerticesX[8] = {}, fVerticesY[8] = {};
  double fDz = 0., fInverseDz = 0., fHalfInverseDz = 0.;
  bool fIsTwisted = false;
  double fConnX[4] = {}, fConnY[4] = {};
  double fDeltaX[8] = {}, fDeltaY[8] = {};
  bool fDegenerated[4] = {};
  // SecondOrderSurfaceShell<4>
  double fxa[4], fya[4], fxb[4], fyb[4], fxc[4], fyc[4], fxd[4], fyd[4];
  double ftx1[4], fty1[4], ftx2[4], fty2[4], ft1crosst2[4], fDeltatx[4], fDeltaty[4];
  double fDz2 = 0.;
  bool fiscurved[4] = {}, fisplanar = true, fdegen[4] = {};
  Vec3 fNormals[4], fViCrossHi0[4], fViCrossVj[4], fHi1CrossHi0[4];
  bool valid = true; // what the reference's Initialize returns for the caller's vertices

  GenTrap(const double *vx, const double *vy, double dz);
  // Initialize (GenTrapStruct.h) on the given vertices: false with a message for the
  // shapes it reports as errors; on success vx/vy hold the clockwise order it keeps
  static bool Initialize(double *vx, double *vy, double dz, const char **err);
  void InitShell();
  // SecondOrderSurfaceShell
  void CheckInside(Vec3 const &p, bool &cin, bool &cout, bool &onsurf) const;
  bool InSurfLimits(Vec3 const &p, int i) const;
  void UNormal(Vec3 const &p, int i, Vec3 &unorm, double &rz, double &r) const;
  void ComputeSminSmax(Vec3 const &p, Vec3 const &d, double smin[4], double smax[4]) const;
  double ShellDistanceToOut(Vec3 const &p, Vec3 const &d) const;
  double ShellDistanceToOutPlanar(Vec3 const &p, Vec3 const &d) const;
  double ShellDistanceToIn(Vec3 const &p, Vec3 const &d, bool done) const;
  double ShellDistanceToInPlanar(Vec3 const &p, Vec3 const &d, bool done) const;
  double ShellSafetyToOut(Vec3 const &p, double safmax) const;
  double ShellSafetyToIn(Vec3 const &p, double safmax) const;
  double SafetyCurved(Vec3 const &p, bool in) const;
  // GenTrapImplementation
  bool IsInTopOrBottomPolygon(double x, double y, bool top) const;
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  Vec3 Normal(Vec3 const &p, bool &valid) const override;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/HypeStruct.h (CalculateCached), VecGeom/volumes/HypeUtilities.h,
// VecGeom/volumes/kernel/HypeImplementation.h with the UniversalHype treatment
// (shapetypes/HypeTypes.h: the inner surface is treated when rmin > 0 or the inner stereo
// angle is not 0) and the scalar HypeHelpers specialisation (the one the CUDA build runs).
struct Hype : UnplacedShape {
  double fRmin, fRmax, fStIn, fStOut, fDz;
  double fTIn, fTOut, fTIn2, fTOut2, fRmin2, fRmax2, fDz2;
  double fEndInnerRadius2, fEndOuterRadius2, fEndInnerRadius, fEndOuterRadius;
  double zToleranceLevel, innerRadToleranceLevel, outerRadToleranceLevel;
  bool fInner;
  Hype(double rmin, double rmax, double stIn, double stOut, double dz);
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  bool IsCompletelyInside(Vec3 const &p) const;
  bool IsCompletelyOutside(Vec3 const &p) const;
  bool OnSurfaceMovingInside(Vec3 const &p, Vec3 const &d) const;
  bool OnSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const;
  bool OnOuterSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const;
  bool OnInnerSurfaceMovingOutside(Vec3 const &p, Vec3 const &d) const;
  bool ZPlaneIntersection(Vec3 const &p, Vec3 const &d, bool forDistToIn, double &zDist) const;
  bool HyperbolicIntersection(Vec3 const &p, Vec3 const &d, bool forDistToIn, bool inner, double &dist) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/Plane.h: a plane n.p + d (n unit), positive on the outside.
struct CutPlane {
  Vec3 n;
  double d = 0.;
  void Set(Vec3 normal, Vec3 const &origin); // Plane.h:40-49
  double Dist(Vec3 const &p) const { return p.Dot(n) + d; } // Plane.h:98-107 DistPlane
};

// VecGeom/volumes/CutTubeStruct.h, VecGeom/volumes/CutPlanes.h,
// VecGeom/volumes/kernel/CutTubeImplementation.h: a tube (UniversalTube of infinite
// half-length) between two cut planes through (0, 0, -dz) and (0, 0, +dz).
struct CutTube : UnplacedShape {
  double fDz;
  Tube fTube;
  CutPlane fCut[2];
  double fCosPhi1, fSinPhi1, fCosPhi2, fSinPhi2, fMaxVal;
  CutTube(double rmin, double rmax, double z, double sphi, double dphi, Vec3 bottom, Vec3 top);
  int CutInside(Vec3 const &p) const;             // CutPlanes.h Inside
  double CutDistanceToIn(Vec3 const &p, Vec3 const &d) const;
  double CutDistanceToOut(Vec3 const &p, Vec3 const &d) const;
  double CutSafetyToIn(Vec3 const &p) const;
  double CutSafetyToOut(Vec3 const &p) const;
  double DistanceToInKernel(Vec3 const &p, Vec3 const &d, double stepMax) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// VecGeom/volumes/kernel/BooleanUnionImplementation.h (kUnion); operands are placed volumes.
// Test infrastructure beyond the product's shapes: the reference's boolean unit test
// subtracts a union, so the oracle restates the union to check its subtraction there.
struct BooleanUnion : UnplacedShape {
  PlacedVolume const *fLeft, *fRight;
  BooleanUnion(PlacedVolume const *l, PlacedVolume const *r) : fLeft(l), fRight(r) {}
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

} // namespace oracle

namespace oracle {
// VecGeom/volumes/TorusStruct2.h, VecGeom/volumes/kernel/TorusImplementation2.h
struct Torus2 : UnplacedShape {
  double fRmin, fRmax, fRtor, fSphi, fDphi, fRmin2, fRmax2, fRtor2;
  Wedge fPhiWedge;
  Tube fBoundingTube;
  Torus2(double rmin, double rmax, double rtor, double sphi, double dphi);
  void ContainsAndInside(Vec3 const &p, bool forInside, bool notForDisk, bool &cin, bool &cout) const;
  double ToBoundary(Vec3 const &pt, Vec3 const &dir, double radius, bool out) const;
  double DistSqrToTorusR(Vec3 const &p, Vec3 const &d, double dist) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override { fBoundingTube.Extent(lo, hi); }
};
} // namespace oracle

namespace oracle {
// Set of quadrilaterals (VecGeom/volumes/Quadrilaterals.h, source/Quadrilaterals.cpp):
// plane (normal, distance), four side planes for the bounds check, four corners.
struct Quads {
  std::vector<Vec3> normal;
  std::vector<double> dist;
  std::vector<Vec3> sideN[4];
  std::vector<double> sideD[4];
  std::vector<Vec3> corner[4];
  explicit Quads(int n = 0) { Resize(n); }
  void Resize(int n);
  int size() const { return (int)dist.size(); }
  void Set(int i, Vec3 const &c0, Vec3 const &c1, Vec3 const &c2, Vec3 const &c3);
  void FlipSign(int i)
  {
    normal[i] = -normal[i];
    dist[i]   = -dist[i];
  }
  bool Contains(Vec3 const &p) const;
  int Inside(Vec3 const &p) const;
  int Inside(Vec3 const &p, int i) const;
  bool RayHits(int i, Vec3 const &x) const;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, bool behind) const;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double zMin, double zMax) const;
  double ScalarDistanceSquared(int i, Vec3 const &p) const;
};

struct ZSegment {
  Quads outer, phi, inner;
  bool hasInnerRadius() const { return inner.size() > 0; }
};

// VecGeom/volumes/PolyhedronStruct.h (construction), VecGeom/volumes/kernel/
// PolyhedronImplementation.h (scalar kernels), EInnerRadii/EPhiCutout = kGeneric as used by
// UnplacedPolyhedron (VecGeom/volumes/UnplacedPolyhedron.h:82-84).
struct Polyhedron : UnplacedShape {
  int fSideCount;
  bool fHasInnerRadii = false, fHasPhiCutout, fHasLargePhiCutout;
  double fPhiStart, fPhiDelta;
  Wedge fPhiWedge;
  std::vector<ZSegment> fZSegments;
  std::vector<double> fZPlanes, fRMin, fRMax;
  std::vector<bool> fSameZ;
  std::vector<Vec3> fPhiSections;
  Tube fBoundingTube;
  double fBoundingTubeOffset = 0.;
  Polyhedron(double phiStart, double phiDelta, int sideCount, int nz, const double *z, const double *rmin,
             const double *rmax);
  int FindZSegment(double z) const;
  int FindPhiSegment(Vec3 const &p) const;
  double DistanceToInZSegment(int s, Vec3 const &p, Vec3 const &d) const;
  double DistanceToOutZSegment(int s, double zMin, double zMax, Vec3 const &p, Vec3 const &d) const;
  double SafetyToZSegmentSquared(int s, int &phiIndex, Vec3 const &p, bool ptInside, int &iSurf) const;
  void DistanceToEndcaps(bool pointInside, Vec3 const &p, Vec3 const &d, double &distance) const;
  void SafetyToEndcapsSquared(Vec3 const &p, double &distance, int &iz) const;
  bool InPhiCutoutWedge(ZSegment const &s, Vec3 const &p) const;
  int InsideSegBorder(Vec3 const &p, int zIndex) const;
  int InsideSegPhi(Vec3 const &p, int zIndex, int phiIndex) const;
  double SafetyKernel(Vec3 const &p, bool ptInside) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const override;
  double SafetyToIn(Vec3 const &p) const override { return SafetyKernel(p, false); }
  double SafetyToOut(Vec3 const &p) const override { return SafetyKernel(p, true); }
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};
} // namespace oracle
