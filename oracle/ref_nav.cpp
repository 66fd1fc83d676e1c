// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
#include "ref_nav.h"
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <stdexcept>
#include <utility>

namespace oracle {

const UnplacedShape *PlacedVolume::Shape() const { return lv->shape; }

// VecGeom/base/AABB.h:136-154 ComputeIntersectionInvDir
void AABB::ComputeIntersectionInvDir(Vec3 const &p, Vec3 const &invdir, double &tmin, double &tmax) const
{
  Vec3 t0 = (mn - p) * invdir;
  Vec3 t1 = (mx - p) * invdir;
  for (int i = 0; i < 3; ++i)
    if (t0[i] > t1[i]) std::swap(t0[i], t1[i]);
  tmin = t0.Max();
  tmax = t1.Min() * (1. + 2 * kEpsilon);
}

// AABB.h:209-217 Union
AABB AABB::Union(AABB const &A, AABB const &B)
{
  return AABB(Vec3(Min(A.mn[0], B.mn[0]), Min(A.mn[1], B.mn[1]), Min(A.mn[2], B.mn[2])),
              Vec3(Max(A.mx[0], B.mx[0]), Max(A.mx[1], B.mx[1]), Max(A.mx[2], B.mx[2])));
}

// ---------------------------------------------------------------- BVH construction
namespace {
// source/BVH.cpp:194-202 less3D
bool less3D(Vec3 const &l, Vec3 const &r, int ax)
{
  return l[ax] < r[ax] ||
         (l[ax] == r[ax] && (l[(ax + 1) % 3] < r[(ax + 1) % 3] ||
                             (l[(ax + 1) % 3] == r[(ax + 1) % 3] && l[(ax + 2) % 3] < r[(ax + 2) % 3])));
}

// source/BVH.cpp:217-236 sweepSurfaceArea
std::vector<std::pair<double, double>> sweepSurfaceArea(const AABB *boxes, int const *begin, int const *end)
{
  if (begin >= end) return {};
  std::vector<std::pair<double, double>> areas(end - begin, {0., 0.});
  AABB box{boxes[*begin]};
  for (auto it = begin + 1; it < end; ++it) {
    areas[it - begin].first = box.SurfaceArea();
    box                     = AABB::Union(box, boxes[*it]);
  }
  AABB box2{boxes[*(end - 1)]};
  for (long k = (end - begin) - 1; k >= 0; --k) {
    box2                 = AABB::Union(box2, boxes[begin[k]]);
    areas[k].second      = box2.SurfaceArea();
  }
  return areas;
}

// source/BVH.cpp:254-306 surfaceAreaHeuristic (including its integer "balance" term)
int *surfaceAreaHeuristic(const AABB *boxes, int *begin, int *end)
{
  int bestSplitAxis          = -1;
  double bestTraversalMetric = std::distance(begin, end);
  int bestSplitObject        = -1;
  const long nObj            = std::distance(begin, end);
  int currentSortAxis        = 0;
  auto sorter = [boxes, &currentSortAxis](int a, int b) {
    const Vec3 cA          = boxes[a].Center();
    const Vec3 cB          = boxes[b].Center();
    constexpr double shift = 0.01;
    return less3D(cA + shift * (cA - boxes[a].mn), cB + shift * (cB - boxes[b].mn), currentSortAxis);
  };
  for (int axis = 0; axis <= 2; ++axis) {
    currentSortAxis = axis;
    std::sort(begin, end, sorter);
    const auto sweep        = sweepSurfaceArea(boxes, begin, end);
    const double totSurfArea = sweep.front().second;
    for (int *split = begin; split < end; ++split) {
      const double left  = sweep[split - begin].first / totSurfArea;
      const double right = sweep[split - begin].second / totSurfArea;
      const long k       = std::distance(begin, split);
      const double splitMetric =
          left * k + right * std::distance(split, end) + 0.1 * std::labs(nObj / 2 - k / nObj);
      if (splitMetric < bestTraversalMetric) {
        bestTraversalMetric = splitMetric;
        bestSplitAxis       = axis;
        bestSplitObject     = *split;
      }
    }
  }
  if (bestSplitAxis == -1) return end;
  currentSortAxis = bestSplitAxis;
  return std::partition(begin, end, [sorter, bestSplitObject](size_t i) { return sorter(i, bestSplitObject); });
}
} // namespace

// source/BVH.cpp:48-87 constructor
BVH::BVH(LogicalVolume const &v, std::vector<AABB> const &daughterBoxes) : lv(v), aabbs(daughterBoxes)
{
  const int n = (int)aabbs.size();
  if (n <= 0) throw std::logic_error("Cannot construct BVH for volume with no children!");
  primId.resize(n);
  std::iota(primId.begin(), primId.end(), 0);
  const int half = n / 2;
  depth          = std::min(half > 0 ? std::max(0, (int)std::log2(half)) : 0, kMaxDepth);
  const unsigned nn = (2u << depth) - 1;
  nchild.assign(nn, 0);
  offset.assign(nn, -1);
  nodes.assign(nn, AABB());
  ComputeNodes(0, primId.data(), primId.data() + n, nn);
  for (unsigned id = 0; id < nn / 2; ++id)
    if (nchild[id] > 8 && (nchild[id] == nchild[2 * id + 1] + nchild[2 * id + 2])) nchild[id] = -1;
}

// source/BVH.cpp:359-385 ComputeNodes
void BVH::ComputeNodes(unsigned id, int *first, int *last, unsigned nnodes)
{
  if (id >= nnodes) return;
  nchild[id] = (int)std::distance(first, last);
  offset[id] = (int)std::distance(primId.data(), first);
  if (first == last) return;
  nodes[id] = aabbs[*first];
  for (auto it = std::next(first); it != last; ++it) nodes[id] = AABB::Union(nodes[id], aabbs[*it]);
  if (std::next(first) == last) return;
  int *pivot = surfaceAreaHeuristic(aabbs.data(), first, last);
  ComputeNodes(2 * id + 1, first, pivot, nnodes);
  ComputeNodes(2 * id + 2, pivot, last, nnodes);
}

// ---------------------------------------------------------------- BVH traversals
// VecGeom/base/BVH.h:96-146 CheckDaughterIntersections
void BVH::CheckDaughterIntersections(Vec3 const &lp, Vec3 const &ld, double &step, PlacedVolume const *last,
                                     PlacedVolume const *&hit, int *nvisited) const
{
  unsigned stack[kMaxDepth], *ptr = &stack[1];
  stack[0] = 0;
  const Vec3 invdir(1.0 / NonZero(ld[0]), 1.0 / NonZero(ld[1]), 1.0 / NonZero(ld[2]));
  do {
    const unsigned id = *--ptr;
    if (nvisited) ++*nvisited;
    if (nchild[id] >= 0) {
      for (int i = 0; i < nchild[id]; ++i) {
        const int prim = primId[offset[id] + i];
        if (aabbs[prim].IntersectInvDir(lp, invdir, step)) {
          PlacedVolume const *vol = lv.daughters[prim];
          const double dist       = vol->DistanceToIn(lp, ld, step);
          if (dist < step && !(dist <= 0.0 && vol == last)) step = dist, hit = vol;
        }
      }
    } else {
      const unsigned childL = 2 * id + 1;
      const unsigned childR = 2 * id + 2;
      double tminL = kInfLength, tmaxL = -kInfLength, tminR = kInfLength, tmaxR = -kInfLength;
      nodes[childL].ComputeIntersectionInvDir(lp, invdir, tminL, tmaxL);
      nodes[childR].ComputeIntersectionInvDir(lp, invdir, tminR, tmaxR);
      const bool traverseL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < step;
      const bool traverseR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < step;
      if (tminR < tminL) {
        if (traverseR) *ptr++ = childR;
        if (traverseL) *ptr++ = childL;
      } else {
        if (traverseL) *ptr++ = childL;
        if (traverseR) *ptr++ = childR;
      }
    }
  } while (ptr > stack);
}

// VUnplacedVolume::ApproachSolid (VecGeom/volumes/UnplacedVolume.h:272-280): the slab
// distance of BoxImplementation::IntersectCachedKernel2 (BoxImplementation.h:324-368) to the
// shape's bounding box (its Extent) within [0, kInfLength], kInfLength on a miss.
static double ApproachSolid(UnplacedShape const &s, Vec3 const &p, Vec3 const &inv)
{
  Vec3 c[2];
  s.Extent(c[0], c[1]);
  const int sx = inv.x() < 0, sy = inv.y() < 0, sz = inv.z() < 0;
  double tmin        = (c[sx].x() - p.x()) * inv.x();
  const double tymax = (c[1 - sy].y() - p.y()) * inv.y();
  if (tmin > tymax) return kInfLength;
  double tmax        = (c[1 - sx].x() - p.x()) * inv.x();
  const double tymin = (c[sy].y() - p.y()) * inv.y();
  if (tymin > tmax) return kInfLength;
  tmin               = Max(tmin, tymin);
  tmax               = Min(tmax, tymax);
  const double tzmin = (c[sz].z() - p.z()) * inv.z();
  const double tzmax = (c[1 - sz].z() - p.z()) * inv.z();
  if (tmin > tzmax || tzmin > tmax) return kInfLength;
  tmin = Max(tmin, tzmin);
  tmax = Min(tmax, tzmax);
  if (!(tmin <= kInfLength + kTolerance && tmax > 0. - kTolerance)) return kInfLength;
  return tmin;
}

// source/BVH.cpp:394-449 ApproachNextDaughter: CheckDaughterIntersections' traversal with the
// daughters' bounding-box approach distance in place of their DistanceToIn
void BVH::ApproachNextDaughter(Vec3 const &lp, Vec3 const &ld, double &step, PlacedVolume const *last) const
{
  unsigned stack[kMaxDepth] = {0}, *ptr = &stack[1];
  const Vec3 invdir(1.0 / NonZero(ld[0]), 1.0 / NonZero(ld[1]), 1.0 / NonZero(ld[2]));
  do {
    const unsigned id = *--ptr;
    if (nchild[id] >= 0) {
      for (int i = 0; i < nchild[id]; ++i) {
        const int prim = primId[offset[id] + i];
        if (aabbs[prim].IntersectInvDir(lp, invdir, step)) {
          PlacedVolume const *vol = lv.daughters[prim];
          const Vec3 p            = vol->T.Transform(lp);
          const Vec3 d            = vol->T.TransformDirection(ld);
          const Vec3 inv(1.0 / NonZero(d[0]), 1.0 / NonZero(d[1]), 1.0 / NonZero(d[2]));
          const double dist = ApproachSolid(*vol->Shape(), p, inv);
          if (dist < step && !(dist <= 0.0 && vol == last)) step = dist;
        }
      }
    } else {
      const unsigned childL = 2 * id + 1;
      const unsigned childR = 2 * id + 2;
      double tminL = kInfLength, tmaxL = -kInfLength, tminR = kInfLength, tmaxR = -kInfLength;
      nodes[childL].ComputeIntersectionInvDir(lp, invdir, tminL, tmaxL);
      nodes[childR].ComputeIntersectionInvDir(lp, invdir, tminR, tmaxR);
      const bool traverseL = tminL <= tmaxL && tmaxL >= 0.0 && tminL < step;
      const bool traverseR = tminR <= tmaxR && tmaxR >= 0.0 && tminR < step;
      if (tminR < tminL) {
        if (traverseR) *ptr++ = childR;
        if (traverseL) *ptr++ = childL;
      } else {
        if (traverseL) *ptr++ = childL;
        if (traverseR) *ptr++ = childR;
      }
    }
  } while (ptr > stack);
}

double Geometry::ApproachNextDaughter(Vec3 const &gp, Vec3 const &gd, double step, NavState const &in) const
{
  Transformation3D m;
  TopMatrix(in.navInd, m);
  LogicalVolume const *lv = Top(in.navInd)->lv;
  if (!lv->daughters.empty()) lv->bvh->ApproachNextDaughter(m.Transform(gp), m.TransformDirection(gd), step, Top(in.lastExited));
  return step;
}

// BVH.h:236-285 LevelLocate (excluded-volume variant)
bool BVH::LevelLocate(PlacedVolume const *excl, Vec3 const &lp, PlacedVolume const *&pvol, Vec3 &dlp) const
{
  unsigned stack[kMaxDepth], *ptr = &stack[1];
  stack[0] = 0;
  do {
    const unsigned id = *--ptr;
    if (nchild[id] >= 0) {
      for (int i = 0; i < nchild[id]; ++i) {
        const int prim = primId[offset[id] + i];
        if (aabbs[prim].Contains(lp)) {
          PlacedVolume const *vol = lv.daughters[prim];
          if (vol != excl && vol->Contains(lp, dlp)) {
            pvol = vol;
            return true;
          }
        }
      }
    } else {
      const unsigned childL = 2 * id + 1;
      if (nodes[childL].Contains(lp)) *ptr++ = childL;
      const unsigned childR = 2 * id + 2;
      if (nodes[childR].Contains(lp)) *ptr++ = childR;
    }
  } while (ptr > stack);
  return false;
}

// BVH.h:172-209 ComputeSafety
double BVH::ComputeSafety(Vec3 const &lp, double safety) const
{
  unsigned stack[kMaxDepth], *ptr = &stack[1];
  stack[0] = 0;
  do {
    const unsigned id = *--ptr;
    if (nchild[id] >= 0) {
      for (int i = 0; i < nchild[id]; ++i) {
        const int prim = primId[offset[id] + i];
        if (aabbs[prim].Safety(lp) < safety) {
          const double dist = lv.daughters[prim]->SafetyToIn(lp);
          if (dist < safety) safety = dist;
        }
      }
    } else {
      const unsigned childL = 2 * id + 1;
      const unsigned childR = 2 * id + 2;
      const double safetyL  = nodes[childL].Safety(lp);
      const double safetyR  = nodes[childR].Safety(lp);
      const bool traverseL  = safetyL < safety;
      const bool traverseR  = safetyR < safety;
      if (safetyR < safetyL) {
        if (traverseR) *ptr++ = childR;
        if (traverseL) *ptr++ = childL;
      } else {
        if (traverseL) *ptr++ = childL;
        if (traverseR) *ptr++ = childR;
      }
    }
  } while (ptr > stack);
  return safety;
}

// ---------------------------------------------------------------- Geometry construction
int Geometry::AddShape(UnplacedShape *s)
{
  shapes.emplace_back(s);
  return (int)shapes.size() - 1;
}
int Geometry::AddLogicalVolume(int shape)
{
  auto lv   = std::make_unique<LogicalVolume>();
  lv->id    = (int)lvs.size();
  lv->shape = shapes.at(shape).get();
  lvs.push_back(std::move(lv));
  return (int)lvs.size() - 1;
}
// LogicalVolume::Place: a new placed volume takes the next id (source/PlacedVolume.cpp:32).
int Geometry::Place(int lv, const double *tr, const double *rot)
{
  auto pv = std::make_unique<PlacedVolume>();
  pv->id  = (int)pvs.size();
  pv->lv  = lvs.at(lv).get();
  pv->T   = Transformation3D::FromArrays(tr, rot);
  pvs.push_back(std::move(pv));
  return (int)pvs.size() - 1;
}
// source/LogicalVolume.cpp:125-155 PlaceDaughter: child id = position in the daughter list.
int Geometry::PlaceDaughter(int motherLv, int lv, const double *tr, const double *rot)
{
  const int id          = Place(lv, tr, rot);
  LogicalVolume *mother = lvs.at(motherLv).get();
  pvs[id]->childId      = (int)mother->daughters.size();
  mother->daughters.push_back(pvs[id].get());
  return id;
}

// source/ABBoxManager.cpp:109-140 ComputeABBox
void Geometry::ComputeABBox(PlacedVolume const *pv, Vec3 &lowerc, Vec3 &upperc) const
{
  Vec3 lower, upper;
  pv->Shape()->Extent(lower, upper);
  const Vec3 delta = upper - lower;
  double minx = kInfLength, miny = kInfLength, minz = kInfLength;
  double maxx = -kInfLength, maxy = -kInfLength, maxz = -kInfLength;
  for (int x = 0; x <= 1; ++x)
    for (int y = 0; y <= 1; ++y)
      for (int z = 0; z <= 1; ++z) {
        Vec3 corner;
        corner[0]     = lower.x() + x * delta.x();
        corner[1]     = lower.y() + y * delta.y();
        corner[2]     = lower.z() + z * delta.z();
        const Vec3 tc = pv->T.InverseTransform(corner);
        minx          = std::min(minx, tc.x());
        miny          = std::min(miny, tc.y());
        minz          = std::min(minz, tc.z());
        maxx          = std::max(maxx, tc.x());
        maxy          = std::max(maxy, tc.y());
        maxz          = std::max(maxz, tc.z());
      }
  lowerc = Vec3(minx - 1E-3, miny - 1E-3, minz - 1E-3);
  upperc = Vec3(maxx + 1E-3, maxy + 1E-3, maxz + 1E-3);
}

unsigned short Geometry::NDaughters(uint32_t n) const
{
  unsigned short nd;
  std::memcpy(&nd, reinterpret_cast<const unsigned char *>(&table[n + 2]) + 2, 2);
  return nd;
}

// NavStateIndex.h:232-265 TopMatrixImpl
void Geometry::TopMatrix(uint32_t n, Transformation3D &trans) const
{
  unsigned char hasm;
  while (true) {
    if (n == 0) return;
    hasm = reinterpret_cast<const unsigned char *>(&table[n + 2])[1];
    if (hasm & 0x04) break;
    Transformation3D t = Top(n)->T;
    t.MultiplyFromRight(trans);
    trans = t;
    n     = NavInd(n);
  }
  if ((hasm & 0x03) == 0) return;
  const bool hasTrans = (hasm & 0x02) > 0;
  const bool hasRot   = (hasm & 0x01) > 0;
  const unsigned nd   = NDaughters(n);
  size_t w            = n + 3 + nd + ((nd + 1) & 1);
  if (w & 1) ++w; // round the byte address up to 8 (the table base is 8-byte aligned)
  double m[12];
  std::memcpy(m, &table[w], sizeof(m));
  Transformation3D t;
  if (hasTrans)
    for (int i = 0; i < 3; ++i) t.t[i] = m[i];
  if (hasRot)
    for (int i = 0; i < 9; ++i) t.r[i] = m[3 + i];
  t.hasTrans = hasTrans;
  t.hasRot   = hasRot;
  t.identity = !hasTrans && !hasRot;
  t.MultiplyFromRight(trans);
  trans = t;
}

// source/NavIndexTable.cpp:9-84 BuildNavIndexVisitor::apply, management/NavIndexTable.h:96-157
// (two passes: count, then fill; every level caches its global matrix).
void Geometry::BuildNavIndexTable()
{
  std::vector<PlacedVolume const *> path;
  size_t tableSize = sizeof(uint32_t);
  uint32_t current = 1;
  bool doCount     = true;
  std::function<uint32_t(PlacedVolume const *, int, uint32_t, int)> visit;
  auto apply = [&](int level, uint32_t mother, int dind) -> uint32_t {
    const uint32_t newMother = current;
    const LogicalVolume *lv  = path.back()->lv;
    const unsigned short nd  = (unsigned short)lv->daughters.size();
    if (lv->daughters.size() >= 65535) throw std::runtime_error("more than 65535 daughters");
    const size_t currentSize = (3 + nd + ((nd + 1) & 1)) * sizeof(uint32_t) + 12 * sizeof(double);
    if (doCount) {
      tableSize += currentSize;
      return 0;
    }
    table[current] = mother;
    if (mother > 0) table[mother + 3 + dind] = current;
    table[current + 1] = (level >= 0) ? (uint32_t)path[level]->id : 0;
    unsigned char *ddt = reinterpret_cast<unsigned char *>(&table[current + 2]);
    ddt[0]             = (unsigned char)level;
    ddt[1]             = 0;
    std::memcpy(ddt + 2, &nd, 2);
    for (size_t i = 0; i < nd; ++i) table[current + 3 + i] = 0;
    current += 3 + nd + ((nd + 1) & 1);
    Transformation3D mat;
    for (size_t i = 1; i < path.size(); ++i) mat.MultiplyFromRight(path[i]->T);
    ddt[1] = (unsigned char)(0x04 + 0x02 * (unsigned short)mat.hasTrans + (unsigned short)mat.hasRot);
    if ((current * sizeof(uint32_t)) % sizeof(double) != 0) current++;
    double m[12];
    for (int i = 0; i < 3; ++i) m[i] = mat.t[i];
    for (int i = 0; i < 9; ++i) m[i + 3] = mat.r[i];
    std::memcpy(&table[current], m, sizeof(m));
    current += 12 * sizeof(double) / sizeof(uint32_t);
    return newMother;
  };
  visit = [&](PlacedVolume const *pv, int level, uint32_t mother, int dind) -> uint32_t {
    path.push_back(pv);
    const uint32_t nm = apply(level, mother, dind);
    for (size_t i = 0; i < pv->lv->daughters.size(); ++i) visit(pv->lv->daughters[i], level + 1, nm, (int)i);
    path.pop_back();
    return nm;
  };
  visit(world, 0, 0, 0);
  const size_t nelem = tableSize / sizeof(uint32_t) + 1;
  tableStorage.assign((nelem + 1) / 2 + 1, 0);
  table      = reinterpret_cast<uint32_t *>(tableStorage.data());
  tableWords = nelem;
  table[0]   = 0;
  doCount    = false;
  current    = 1;
  visit(world, 0, 0, 0);
}

// GeoManager::CloseGeometry (source/GeoManager.cpp:192-220) + BVHManager::Init
// (source/BVHManager.cpp:24-30).
void Geometry::Close()
{
  if (world) {
    std::function<int(PlacedVolume const *)> depthOf = [&](PlacedVolume const *pv) {
      int d = 0;
      for (auto *c : pv->lv->daughters) d = std::max(d, depthOf(c));
      return d + 1;
    };
    maxDepth = depthOf(world);
    for (auto &lv : lvs) {
      if (lv->daughters.empty()) continue;
      std::vector<AABB> boxes(lv->daughters.size());
      for (size_t d = 0; d < lv->daughters.size(); ++d) ComputeABBox(lv->daughters[d], boxes[d].mn, boxes[d].mx);
      bvhs.emplace_back(new BVH(*lv, boxes));
      lv->bvh = bvhs.back().get();
    }
    BuildNavIndexTable();
  }
  closed = true;
}

// ---------------------------------------------------------------- GlobalLocator
bool Geometry::LevelLocate(LogicalVolume const *lv, PlacedVolume const *excl, Vec3 const &lp,
                           PlacedVolume const *&pvol, Vec3 &dlp, bool simple) const
{
  if (!simple) return lv->bvh->LevelLocate(excl, lp, pvol, dlp);
  // SimpleLevelLocator.h:122-140 LevelLocateKernel<ExclV, false> with CheckCandidateVol (:20-45)
  for (PlacedVolume const *d : lv->daughters) {
    if (d == excl) continue;
    if (d->Contains(lp, dlp)) {
      pvol = d;
      return true;
    }
  }
  return false;
}

// GlobalLocator.h:35-82 LocateGlobalPoint (BVHLevelLocator::LevelLocate -> BVH::LevelLocate)
PlacedVolume const *Geometry::LocateGlobalPoint(PlacedVolume const *vol, Vec3 const &point, NavState &s, bool top,
                                                bool simple) const
{
  PlacedVolume const *cand = vol;
  Vec3 cur                 = point;
  if (top) cand = vol->UnplacedContains(point) ? vol : nullptr;
  if (cand) {
    s.navInd                = Push(s.navInd, cand);
    LogicalVolume const *lv = cand->lv;
    bool godeeper           = true;
    while (!lv->daughters.empty() && godeeper) {
      Vec3 tp;
      PlacedVolume const *pv = nullptr;
      godeeper               = LevelLocate(lv, nullptr, cur, pv, tp, simple);
      if (godeeper) {
        s.navInd = Push(s.navInd, pv);
        cand     = Top(s.navInd);
        lv       = cand->lv;
        cur      = tp;
      }
    }
  }
  return cand ? Top(s.navInd) : nullptr;
}

// GlobalLocator.h:88-135 LocateGlobalPointExclVolume (top = false)
PlacedVolume const *Geometry::LocateGlobalPointExclVolume(PlacedVolume const *vol, PlacedVolume const *excl,
                                                          Vec3 const &point, NavState &s, bool simple) const
{
  PlacedVolume const *cand = vol;
  Vec3 cur                 = point;
  if (cand) {
    s.navInd                = Push(s.navInd, cand);
    LogicalVolume const *lv = cand->lv;
    bool godeeper           = true;
    while (!lv->daughters.empty() && godeeper) {
      godeeper = false;
      Vec3 tp;
      godeeper = LevelLocate(lv, excl, cur, cand, tp, simple);
      if (godeeper) {
        lv       = cand->lv;
        cur      = tp;
        s.navInd = Push(s.navInd, cand);
      }
    }
  }
  return cand;
}

// GlobalLocator.h:171-200 RelocatePointFromPathForceDifferent
PlacedVolume const *Geometry::RelocatePointFromPathForceDifferent(Vec3 const &lp, NavState &s, bool simple) const
{
  PlacedVolume const *currentmother = Top(s.navInd);
  PlacedVolume const *entryvol      = currentmother;
  if (currentmother) {
    Vec3 tmp = lp;
    while (currentmother) {
      if (currentmother == entryvol || currentmother->IsAssembly() || !currentmother->UnplacedContains(tmp)) {
        s.navInd      = Pop(s.navInd);
        tmp           = currentmother->T.InverseTransform(tmp);
        currentmother = Top(s.navInd);
      } else {
        break;
      }
    }
    if (currentmother) {
      s.navInd = Pop(s.navInd);
      return LocateGlobalPointExclVolume(currentmother, entryvol, tmp, s, simple);
    }
  }
  return currentmother;
}

// ---------------------------------------------------------------- navigation step
double Geometry::ComputeStepAndPropagatedState(Vec3 const &gp, Vec3 const &gd, double stepLimit, NavState const &in,
                                               NavState &out, int *nvisited, bool simple) const
{
  // DoGlobalToLocalTransformation (VNavigator.h:258-270)
  Transformation3D m;
  TopMatrix(in.navInd, m);
  const Vec3 lp = m.Transform(gp);
  const Vec3 ld = m.TransformDirection(gd);

  PlacedVolume const *pvol = Top(in.navInd);
  LogicalVolume const *lv  = pvol->lv;
  PlacedVolume const *hit  = nullptr;
  // TreatDistanceToMother (VNavigator.h:238-249)
  double step = pvol->DistanceToOut(lp, ld, stepLimit);
  if (step < 0.) step = 0.;
  // BVHNavigator::CheckDaughterIntersections (BVHNavigator.h:53-61); volumes without
  // daughters have no BVH and no daughter to hit.
  if (!lv->daughters.empty()) {
    PlacedVolume const *last = Top(in.lastExited);
    if (!simple) {
      lv->bvh->CheckDaughterIntersections(lp, ld, step, last, hit, nvisited);
    } else {
      // NewSimpleNavigator::CheckDaughterIntersections (NewSimpleNavigator.h:33-63, without
      // CHECKCONTAINS): DistanceToIn of every daughter in order with the running step
      for (PlacedVolume const *d : lv->daughters) {
        const double dd  = d->DistanceToIn(lp, ld, step);
        const bool valid = (dd < step && !std::isinf(dd)) && !((dd <= 0.) && last == d);
        hit              = valid ? d : hit;
        step             = valid ? dd : step;
      }
    }
  }
  // PrepareOutState (VNavigator.h:192-235)
  out = in;
  if (step == kInfLength && stepLimit > 0.) {
    step           = kTolerance;
    out.onBoundary = 1;
    do {
      out.navInd = Pop(out.navInd);
    } while (Top(out.navInd) != nullptr && Top(out.navInd)->IsAssembly());
    return step;
  }
  if (step > stepLimit) {
    out.onBoundary = 0;
    return stepLimit;
  }
  out.onBoundary = 1;
  out.lastExited = out.navInd;
  if (hit) out.navInd = Push(out.navInd, hit);
  if (step < 0.) step = 0.;
  // Relocate(MovePointAfterBoundary(...)) (VNavigator.h:168-173, 1070-1091)
  const double extra = 1E-6;
  const Vec3 after   = lp + (step + extra) * ld;
  if (Top(out.navInd) == Top(in.navInd)) {
    RelocatePointFromPathForceDifferent(after, out, simple);
  } else {
    PlacedVolume const *next = Top(out.navInd);
    out.navInd               = Pop(out.navInd);
    LocateGlobalPoint(next, next->T.Transform(after), out, false, simple);
  }
  while (Top(out.navInd) != nullptr && Top(out.navInd)->IsAssembly()) out.navInd = Pop(out.navInd);
  return step;
}

// VNavigator.h:1014-1064 with BVHSafetyEstimator::ComputeSafetyForLocalPoint (BVHSafetyEstimator.h:38-46)
double Geometry::ComputeStepAndSafetyAndPropagatedState(Vec3 const &gp, Vec3 const &gd, double stepLimit,
                                                        NavState const &in, NavState &out, double &safety) const
{
  Transformation3D m;
  TopMatrix(in.navInd, m);
  const Vec3 lp            = m.Transform(gp);
  PlacedVolume const *pvol = Top(in.navInd);
  safety                   = pvol->SafetyToOut(lp);
  if (safety > 0.0 && !pvol->lv->daughters.empty()) safety = pvol->lv->bvh->ComputeSafety(lp, safety);
  return ComputeStepAndPropagatedState(gp, gd, stepLimit, in, out);
}

// test/benchmark/TestNavIndex.cpp:30-127: walk every placed-volume path from the world,
// passing the index made by PushImpl from the mother's index, and check at each node the
// index recomputed from the path, the top volume, the level, Pop/Push consistency, the
// daughter count and the cached global matrix (NavStateIndex::TopMatrixImpl) against the
// product of the path's transformations (NavStatePath::TopMatrix, NavStatePath.h:616-628).
// The accessors read `tab` through this geometry's own helpers, so the table pointer is
// swapped in for the duration of the walk (single-threaded test use only).
int Geometry::CheckNavIndexTable(const uint32_t *tab, size_t words, long *paths) const
{
  Geometry *self       = const_cast<Geometry *>(this);
  uint32_t *saved      = self->table;
  const size_t savedWr = self->tableWords;
  self->table          = const_cast<uint32_t *>(tab);
  self->tableWords     = words;
  std::vector<PlacedVolume const *> path;
  long visited = 0;
  std::function<int(PlacedVolume const *, uint32_t)> visit = [&](PlacedVolume const *pv, uint32_t nav) -> int {
    if (nav == 0 || nav >= words) return 2;
    path.push_back(pv);
    ++visited;
    // GlobalToLocalVisitor::apply (TestNavIndex.cpp:36-96)
    const int level  = (int)path.size() - 1;
    uint32_t ind     = 1;
    PlacedVolume const *pd = nullptr;
    for (int i = 1; i < level + 1; ++i) {
      pd = path[i];
      if (pd->childId < 0) return 1;
      ind = Push(ind, pd);
    }
    if (ind != nav) return 2;
    if (Top(ind) != pv) return 3;
    if (level != (int)Level(ind)) return 4;
    if (level > 0 && ind != Push(Pop(ind), pd)) return 5;
    if (NDaughters(ind) != pv->lv->daughters.size()) return 6;
    Transformation3D byPath, byIndex;
    for (int i = 1; i < level + 1; ++i) byPath.MultiplyFromRight(path[i]->T);
    TopMatrix(ind, byIndex);
    for (int k = 0; k < 3; ++k)
      if (!(byPath.t[k] == byIndex.t[k])) return 7;
    for (int k = 0; k < 9; ++k)
      if (!(byPath.r[k] == byIndex.r[k])) return 7;
    for (PlacedVolume const *d : pv->lv->daughters) {
      const int e = visit(d, Push(nav, d));
      if (e) return e;
    }
    path.pop_back();
    return 0;
  };
  const int err    = world ? visit(world, 1) : 0;
  self->table      = saved;
  self->tableWords = savedWr;
  if (paths) *paths = visited;
  return err;
}

} // namespace oracle
