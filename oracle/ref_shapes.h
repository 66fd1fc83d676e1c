// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h for the rules that govern this folder).
//
// Scalar restatement of the reference's per-shape kernels. Each shape keeps the
// reference's precomputed members (names follow the reference *Struct) and restates the
// scalar (Real_v = double, bool masks, early returns allowed) path of its *Implementation.
#pragma once
#include "ref_base.h"
#include <vector>

namespace oracle {

// Shared query interface, mirroring VUnplacedVolume (VecGeom/volumes/UnplacedVolume.h:89-230).
struct UnplacedShape {
  virtual ~UnplacedShape() {}
  virtual int Inside(Vec3 const &p) const                                     = 0;
  virtual bool Contains(Vec3 const &p) const                                  = 0;
  virtual double DistanceToIn(Vec3 const &p, Vec3 const &d, double smax) const  = 0;
  virtual double DistanceToOut(Vec3 const &p, Vec3 const &d, double smax) const = 0;
  virtual double SafetyToIn(Vec3 const &p) const                              = 0;
  virtual double SafetyToOut(Vec3 const &p) const                             = 0;
  virtual void Extent(Vec3 &lo, Vec3 &hi) const                               = 0;
  virtual bool IsAssembly() const { return false; }
  // Surface normal (VUnplacedVolume::Normal). Restated only where an oracle query needs it
  // (the Box, for the boolean union's Inside); reaching the default is a test-setup error.
  virtual Vec3 Normal(Vec3 const &p, bool &valid) const;
};

// ---------------------------------------------------------------- Wedge
// VecGeom/volumes/Wedge_Evolution.h:43-200, source/Wedge_Evolution.cpp (constructor).
struct Wedge {
  double dphi = 0.;
  Vec3 along1, along2, normal1, normal2;
  Wedge() {}
  Wedge(double angle, double zero);
  // GenericKernelForContainsAndInside (Wedge_Evolution.h:299-331)
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  static bool IsOnSurfaceGeneric(Vec3 const &along, Vec3 const &normal, Vec3 const &p);
  bool Contains(Vec3 const &p) const
  {
    bool ci = false, co = false;
    ContainsAndInside(p, false, ci, co);
    return !co;
  }
  double SafetyToOut(Vec3 const &p) const;
  double SafetyToIn(Vec3 const &p) const;
};

// ---------------------------------------------------------------- Box
// VecGeom/volumes/kernel/BoxImplementation.h:84-167, VecGeom/volumes/BoxStruct.h:19-27
struct Box : UnplacedShape {
  Vec3 dim;
  Box(double dx, double dy, double dz) : dim(dx, dy, dz) {}
  Vec3 Normal(Vec3 const &p, bool &valid) const override;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override
  {
    lo = -dim;
    hi = dim;
  }
};

// ---------------------------------------------------------------- Tube
// VecGeom/volumes/TubeStruct.h:15-180 (members + CalculateCached),
// VecGeom/volumes/kernel/TubeImplementation.h (UniversalTube kernels).
struct Tube : UnplacedShape {
  double fRmin, fRmax, fZ, fSphi, fDphi;
  double fRmin2, fRmax2, fAlongPhi1x, fAlongPhi1y, fAlongPhi2x, fAlongPhi2y;
  double fTolIrmin2, fTolOrmin2, fTolIrmax2, fTolOrmax2, fTolIz, fTolOz;
  double fTolIrmin, fTolOrmin, fTolIrmax, fTolOrmax, fMaxVal;
  Wedge fPhiWedge;
  Tube(double rmin, double rmax, double z, double sphi, double dphi);
  bool PhiTreat() const { return fDphi < kTwoPi; }
  bool RminTreat() const { return fRmin > 0; }
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  void PointInCyclicalSector(double x, double y, bool includeSurface, bool &ret) const;
  void CircleTrajectoryIntersection(double b, double c, Vec3 const &pos, Vec3 const &dir, bool largest,
                                    bool insectorCheck, double &dist, bool &ok) const;
  void PhiPlaneTrajectoryIntersection(double alongX, double alongY, double normalX, double normalY, Vec3 const &pos,
                                      Vec3 const &dir, bool positiveDir, bool insectorCheck, double &dist,
                                      bool &ok) const;
  void PhiPlaneSafety(Vec3 const &pos, bool inside, double &safety) const;
  bool IsMovingInsideTubeSurface(Vec3 const &p, Vec3 const &d, bool inner) const;
  double DistanceToInKernel(Vec3 const &p, Vec3 const &d) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

// ---------------------------------------------------------------- Cone
// VecGeom/volumes/ConeStruct.h:23-336, VecGeom/volumes/ConeUtilities.h (scalar ConeHelpers),
// VecGeom/volumes/kernel/ConeImplementation.h (UniversalCone kernels).
struct Cone : UnplacedShape {
  double fRmin1, fRmax1, fRmin2, fRmax2, fDz, fSPhi, fDPhi;
  double _frmin1, _frmin2, _frmax1, _frmax2;
  Wedge fPhiWedge;
  double fAlongPhi1x, fAlongPhi1y, fAlongPhi2x, fAlongPhi2y;
  double fInnerSlope, fOuterSlope, fInnerOffset, fOuterOffset, fInnerTolerance, fOuterTolerance;
  double fSqRmin1, fSqRmin2, fSqRmax1, fSqRmax2, fTolIz, fTolOz;
  double fInnerConeApex, fTanInnerApexAngle, fOuterConeApex, fTanOuterApexAngle;
  double fSecRMin, fSecRMax, fInvSecRMin, fInvSecRMax, fTanRMin, fTanRMax, fZNormInner, fZNormOuter;
  double fConeTolerance, fOriginalRmax1, fOriginalRmax2;
  Cone(double rmin1, double rmax1, double rmin2, double rmax2, double dz, double sphi, double dphi);
  void CalculateCached();
  bool PhiTreat() const { return fDPhi < kTwoPi; }
  bool RminTreat() const { return fRmin1 > 0 || fRmin2 > 0; }
  double RadiusAt(double z, bool inner) const;
  void PointInCyclicalSector(double x, double y, bool includeSurface, bool &ret) const;
  Vec3 GetNormal(Vec3 const &p, bool inner) const;
  bool IsOnConicalSurface(Vec3 const &p, bool inner) const;
  void PhiPlaneTrajectoryIntersection(double alongX, double alongY, double normalX, double normalY, Vec3 const &pos,
                                      Vec3 const &dir, bool positiveDir, bool insectorCheck, double &dist,
                                      bool &ok) const;
  bool ConicalIntersection(Vec3 const &p, Vec3 const &d, bool forDistToIn, bool inner, double &distance) const;
  void ContainsAndInside(Vec3 const &p, bool forInside, bool &cin, bool &cout) const;
  double SafeDistanceToConicalSurface(Vec3 const &p, bool inner) const;
  int Inside(Vec3 const &p) const override;
  bool Contains(Vec3 const &p) const override;
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double) const override;
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double) const override;
  double SafetyToIn(Vec3 const &p) const override;
  double SafetyToOut(Vec3 const &p) const override;
  void Extent(Vec3 &lo, Vec3 &hi) const override;
};

} // namespace oracle
