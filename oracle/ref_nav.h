// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
//
// Geometry model (logical/placed volumes), daughter bounding boxes, the per-volume BVH,
// the NavIndex table, NavStateIndex operations, GlobalLocator and the BVH navigator step,
// restated from the reference in its own object style (pointers between volumes, a
// recursive visitor for the table, std::sort/std::partition for the SAH build).
#pragma once
#include "ref_shapes.h"
#include <cstdint>
#include <memory>
#include <vector>

namespace oracle {

struct LogicalVolume;
struct BVH;

// VecGeom/volumes/PlacedVolume.h + SpecializedPlacedVolImplHelper.h:98-170: Inside, Contains,
// DistanceToIn and SafetyToIn transform into the local frame first; DistanceToOut,
// SafetyToOut and UnplacedContains take local coordinates (PlacedVolImplHelper.h:70-123).
struct PlacedVolume {
  int id;
  LogicalVolume *lv;
  Transformation3D T;
  int childId = -1;
  const UnplacedShape *Shape() const;
  bool IsAssembly() const { return Shape()->IsAssembly(); }
  bool UnplacedContains(Vec3 const &p) const { return Shape()->Contains(p); }
  bool Contains(Vec3 const &p, Vec3 &lp) const
  {
    lp = T.Transform(p);
    return Shape()->Contains(lp);
  }
  bool Contains(Vec3 const &p) const { return Shape()->Contains(T.Transform(p)); }
  int Inside(Vec3 const &p) const { return Shape()->Inside(T.Transform(p)); }
  double DistanceToIn(Vec3 const &p, Vec3 const &d, double s) const
  {
    return Shape()->DistanceToIn(T.Transform(p), T.TransformDirection(d), s);
  }
  double DistanceToOut(Vec3 const &p, Vec3 const &d, double s) const { return Shape()->DistanceToOut(p, d, s); }
  // PlacedDistanceToOut (SpecializedPlacedVolImplHelper.h:148-163): mother-frame input
  double PlacedDistanceToOut(Vec3 const &p, Vec3 const &d, double s) const
  {
    return Shape()->DistanceToOut(T.Transform(p), T.TransformDirection(d), s);
  }
  double SafetyToIn(Vec3 const &p) const { return Shape()->SafetyToIn(T.Transform(p)); }
  double SafetyToOut(Vec3 const &p) const { return Shape()->SafetyToOut(p); }
};

struct LogicalVolume {
  int id;
  UnplacedShape *shape;
  std::vector<PlacedVolume *> daughters;
  BVH *bvh = nullptr;
};

// VecGeom/base/AABB.h
struct AABB {
  Vec3 mn, mx;
  AABB() {}
  AABB(Vec3 a, Vec3 b) : mn(a), mx(b) {}
  Vec3 Center() const { return 0.5 * (mx + mn); }
  Vec3 Size() const { return mx - mn; }
  double SurfaceArea() const
  {
    const Vec3 e = Size();
    return 2. * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
  }
  bool Contains(Vec3 const &p) const
  {
    return p[0] >= mn[0] && p[0] <= mx[0] && p[1] >= mn[1] && p[1] <= mx[1] && p[2] >= mn[2] && p[2] <= mx[2];
  }
  double Safety(Vec3 const &p) const { return ((p - Center()).Abs() - 0.5 * Size()).Max(); }
  void ComputeIntersectionInvDir(Vec3 const &p, Vec3 const &invdir, double &tmin, double &tmax) const;
  bool IntersectInvDir(Vec3 const &p, Vec3 const &invdir, double step) const
  {
    double tmin, tmax;
    ComputeIntersectionInvDir(p, invdir, tmin, tmax);
    return tmin <= tmax && tmax >= 0.0 && tmin < step;
  }
  static AABB Union(AABB const &A, AABB const &B);
};

// VecGeom/base/BVH.h, source/BVH.cpp
struct BVH {
  static constexpr int kMaxDepth = 32;
  LogicalVolume const &lv;
  std::vector<int> primId, offset, nchild;
  std::vector<AABB> nodes, aabbs;
  int depth = 0;
  int maxStackSeen = 0;
  BVH(LogicalVolume const &v, std::vector<AABB> const &daughterBoxes);
  void ComputeNodes(unsigned id, int *first, int *last, unsigned nnodes);
  void CheckDaughterIntersections(Vec3 const &lp, Vec3 const &ld, double &step, PlacedVolume const *last,
                                  PlacedVolume const *&hit, int *nvisited = nullptr) const;
  bool LevelLocate(PlacedVolume const *excl, Vec3 const &lp, PlacedVolume const *&pvol, Vec3 &dlp) const;
  double ComputeSafety(Vec3 const &lp, double safety) const;
  void ApproachNextDaughter(Vec3 const &lp, Vec3 const &ld, double &step, PlacedVolume const *last) const;
};

// NavStateIndex (VecGeom/navigation/NavStateIndex.h:39-41)
struct NavState {
  uint32_t navInd     = 0;
  uint32_t lastExited = 0;
  uint8_t onBoundary  = 0;
  uint8_t pad[3]      = {0, 0, 0};
};
static_assert(sizeof(NavState) == 12, "NavState is 12 bytes");

struct Geometry {
  std::vector<std::unique_ptr<UnplacedShape>> shapes;
  std::vector<std::unique_ptr<LogicalVolume>> lvs;
  std::vector<std::unique_ptr<PlacedVolume>> pvs;
  std::vector<std::unique_ptr<BVH>> bvhs;
  PlacedVolume *world = nullptr;
  int maxDepth        = 0;
  std::vector<uint64_t> tableStorage; // 8-byte aligned backing store of the NavIndex table
  uint32_t *table    = nullptr;
  size_t tableWords  = 0;
  bool closed        = false;

  int AddShape(UnplacedShape *s);
  int AddLogicalVolume(int shape);
  int Place(int lv, const double *tr, const double *rot);
  int PlaceDaughter(int motherLv, int lv, const double *tr, const double *rot);
  void Close();
  void ComputeABBox(PlacedVolume const *pv, Vec3 &lo, Vec3 &hi) const;
  void BuildNavIndexTable();

  // NavStateIndex static helpers (NavStateIndex.h:172-265)
  uint32_t NavInd(uint32_t i) const { return table[i]; }
  uint32_t Pop(uint32_t n) const { return n > 0 ? table[n] : 0; }
  uint32_t Push(uint32_t n, PlacedVolume const *v) const { return n > 0 ? table[n + 3 + v->childId] : 1; }
  PlacedVolume const *Top(uint32_t n) const { return n > 0 ? pvs[table[n + 1]].get() : nullptr; }
  unsigned char Level(uint32_t n) const { return reinterpret_cast<const unsigned char *>(&table[n + 2])[0]; }
  unsigned short NDaughters(uint32_t n) const;
  void TopMatrix(uint32_t n, Transformation3D &trans) const;

  // Level locators. BVHLevelLocator (VecGeom/navigation/BVHLevelLocator.h:44-96 ->
  // BVH::LevelLocate) normally; with `simple`, SimpleLevelLocator
  // (VecGeom/navigation/SimpleLevelLocator.h:122-140): every daughter in order, the first
  // one that contains the point. The simple forms are the brute-force second navigator the
  // reference validates its BVH navigator against.
  bool LevelLocate(LogicalVolume const *lv, PlacedVolume const *excl, Vec3 const &lp, PlacedVolume const *&pvol,
                   Vec3 &dlp, bool simple) const;

  // GlobalLocator (VecGeom/navigation/GlobalLocator.h:35-200) with BVHLevelLocator (or, with
  // `simple`, SimpleLevelLocator) on every logical volume that has daughters.
  PlacedVolume const *LocateGlobalPoint(PlacedVolume const *vol, Vec3 const &p, NavState &s, bool top,
                                        bool simple = false) const;
  PlacedVolume const *LocateGlobalPointExclVolume(PlacedVolume const *vol, PlacedVolume const *excl, Vec3 const &p,
                                                  NavState &s, bool simple = false) const;
  PlacedVolume const *RelocatePointFromPathForceDifferent(Vec3 const &lp, NavState &s, bool simple = false) const;

  // VNavigatorHelper<BVHNavigator<false>>::ComputeStepAndPropagatedState (VNavigator.h:436-492);
  // with `simple`, VNavigatorHelper<NewSimpleNavigator<false>> (NewSimpleNavigator.h:33-63:
  // DistanceToIn of every daughter in order) relocating with SimpleLevelLocator.
  double ComputeStepAndPropagatedState(Vec3 const &gp, Vec3 const &gd, double stepLimit, NavState const &in,
                                       NavState &out, int *nvisited = nullptr, bool simple = false) const;

  // test/benchmark/TestNavIndex.cpp:30-96 GlobalToLocalVisitor over every placed-volume path
  // (visitAllPlacedVolumesPassNavIndex, :101-127), applied to `tab` (this geometry's own
  // NavIndex table, or a table built elsewhere for the same geometry). Returns the
  // reference's error code: 0 pass, 1 bad child id, 2 index mismatch, 3 top volume, 4 level,
  // 5 push/pop, 6 daughter count, 7 cached global matrix; *paths receives the paths visited.
  int CheckNavIndexTable(const uint32_t *tab, size_t words, long *paths) const;
  // BVH::ApproachNextDaughter (source/BVH.cpp:394-449) in the frame of the state's volume,
  // `last` = the state's last-exited volume, as CheckDaughterIntersections gets it
  double ApproachNextDaughter(Vec3 const &gp, Vec3 const &gd, double step, NavState const &in) const;
  // VNavigatorHelper::ComputeStepAndSafetyAndPropagatedState (VNavigator.h:1014-1064)
  double ComputeStepAndSafetyAndPropagatedState(Vec3 const &gp, Vec3 const &gd, double stepLimit,
                                                NavState const &in, NavState &out, double &safety) const;
};

} // namespace oracle
