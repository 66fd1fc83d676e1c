// ORACLE — TEST INFRASTRUCTURE ONLY. The compiled-reference oracle: the reference's own
// C++ sources (VecGeom/ and source/, compiled in place by oracle/build_ref.py against the
// scalar VecCore stand-in in oracle/compiled_ref/shim/) behind the same extern "C" surface as the
// hand-written oracle (ref_api.cpp), so that the Python wrapper drives either one with the
// same builder calls and compares them. The product never links it; tests use it to pin the
// hand-written oracle to the reference's own code.
//
// The reference keeps its geometry in process-wide singletons (GeoManager, NavIndexTable,
// BVHManager), so one process holds one geometry: a second oracle_geom_create fails.
// Placed volumes are looked up by id after closing (GeoManager::CloseGeometry moves them
// into a compact buffer, GeoManager.cpp:70-150).
#include "VecGeom/base/Transformation3D.h"
#include "VecGeom/management/BVHManager.h"
#include "VecGeom/management/GeoManager.h"
#include "VecGeom/management/NavIndexTable.h"
#include "VecGeom/navigation/BVHLevelLocator.h"
#include "VecGeom/navigation/BVHNavigator.h"
#include "VecGeom/navigation/GlobalLocator.h"
#include "VecGeom/navigation/NavigationState.h"
#include "VecGeom/volumes/LogicalVolume.h"
#include "VecGeom/volumes/PlacedVolume.h"
#include "VecGeom/volumes/UnplacedBooleanVolume.h"
#include "VecGeom/volumes/UnplacedBox.h"
#include "VecGeom/volumes/UnplacedCone.h"
#include "VecGeom/volumes/UnplacedCutTube.h"
#include "VecGeom/volumes/UnplacedGenTrap.h"
#include "VecGeom/volumes/UnplacedHype.h"
#include "VecGeom/volumes/UnplacedOrb.h"
#include "VecGeom/volumes/UnplacedPolycone.h"
#include "VecGeom/volumes/UnplacedPolyhedron.h"
#include "VecGeom/volumes/UnplacedSphere.h"
#include "VecGeom/volumes/UnplacedTorus2.h"
#include "VecGeom/volumes/UnplacedTrapezoid.h"
#include "VecGeom/volumes/UnplacedTrd.h"
#include "VecGeom/volumes/UnplacedTube.h"
#include "vecgeom_gb300_mirror.hpp"
#include "vecgeom_gb300_navigator.hpp"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

using namespace vecgeom;

namespace {

static_assert(sizeof(NavigationState) == 12 && std::is_trivially_copyable<NavigationState>::value,
              "NavStateIndex is the 12-byte {nav index, last exited, on boundary} state");

struct RefGeometry {
  std::vector<VUnplacedVolume const *> shapes;
  std::vector<LogicalVolume *> lvs;
  int npv       = 0;
  int world     = -1;
  bool closed   = false;
};

RefGeometry *g_geom = nullptr;

VPlacedVolume const *pv_at(int id) { return GeoManager::Instance().FindPlacedVolume(id); }

NavigationState to_state(const void *s)
{
  NavigationState st;
  std::memcpy(static_cast<void *>(&st), s, sizeof(st));
  return st;
}
// The three fields; the three bytes of padding after fOnBoundary are written as zeros.
void from_state(NavigationState const &st, void *s)
{
  std::memcpy(s, static_cast<const void *>(&st), sizeof(st));
  std::memset(static_cast<char *>(s) + 9, 0, 3);
}

template <class F>
double ParallelFor(size_t n, int nthreads, F &&f)
{
  const auto t0 = std::chrono::steady_clock::now();
  if (nthreads <= 1 || n < 1024) {
    f(size_t(0), n);
  } else {
    std::vector<std::thread> th;
    const size_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
      const size_t b = t * chunk, e = std::min(n, b + chunk);
      if (b < e) th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto &t : th)
      t.join();
  }
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

Transformation3D *make_transform(const double *tr, const double *rot)
{
  return new Transformation3D(tr[0], tr[1], tr[2], rot[0], rot[1], rot[2], rot[3], rot[4], rot[5], rot[6], rot[7],
                              rot[8]);
}

} // namespace

extern "C" {

void *oracle_geom_create()
{
  if (g_geom) return nullptr;
  g_geom = new RefGeometry();
  return g_geom;
}
void oracle_geom_destroy(void *) {}

// Shape codes and parameter layouts as in ref_api.cpp (plus 15, an Orb of radius p[0], which
// only this harness makes: a shape outside the product's set); every shape is made the way the
// reference's own factories make it (GeoManager::MakeInstance where a Maker exists, which
// with volume specialisation off gives the universal kernels).
int oracle_add_shape(void *, int type, const double *p, int np)
{
  RefGeometry *g          = g_geom;
  VUnplacedVolume const *s = nullptr;
  switch (type) {
  case 1: s = new UnplacedBox(p[0], p[1], p[2]); break;
  case 2: s = GeoManager::MakeInstance<UnplacedTube>(p[0], p[1], p[2], p[3], p[4]); break;
  case 3: s = GeoManager::MakeInstance<UnplacedCone>(p[0], p[1], p[2], p[3], p[4], p[5], p[6]); break;
  case 4: {
    const int nz = (int)p[2];
    s            = GeoManager::MakeInstance<UnplacedPolycone>(p[0], p[1], nz, p + 3, p + 3 + nz, p + 3 + 2 * nz);
    break;
  }
  case 5: {
    const int nz = (int)p[3];
    s            = new UnplacedPolyhedron(p[0], p[1], (int)p[2], nz, p + 4, p + 4 + nz, p + 4 + 2 * nz);
    break;
  }
  case 6: s = new UnplacedTorus2(p[0], p[1], p[2], p[3], p[4]); break;
  case 7: s = GeoManager::MakeInstance<UnplacedTrd>(p[0], p[1], p[2], p[3], p[4]); break;
  case 8:
    s = new UnplacedBooleanVolume<kSubtraction>(kSubtraction, pv_at((int)p[0]), pv_at((int)p[1]));
    break;
  case 10: s = new UnplacedBooleanVolume<kUnion>(kUnion, pv_at((int)p[0]), pv_at((int)p[1])); break;
  case 11:
    s = new UnplacedCutTube(p[0], p[1], p[2], p[3], p[4], Vector3D<Precision>(p[5], p[6], p[7]),
                            Vector3D<Precision>(p[8], p[9], p[10]));
    break;
  case 12: s = GeoManager::MakeInstance<UnplacedSphere>(p[0], p[1], p[2], p[3], p[4], p[5]); break;
  case 13:
    if (np != 17) return -1;
    s = new UnplacedGenTrap(p, p + 8, p[16]);
    break;
  case 14: s = GeoManager::MakeInstance<UnplacedHype>(p[0], p[1], p[2], p[3], p[4]); break;
  case 9:
    if (np == 11) {
      s = GeoManager::MakeInstance<UnplacedTrapezoid>(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], p[9],
                                                      p[10]);
    } else if (np == 24) {
      TrapCorners c;
      for (int k = 0; k < 8; ++k)
        c[k] = Vector3D<Precision>(p[3 * k], p[3 * k + 1], p[3 * k + 2]);
      s = GeoManager::MakeInstance<UnplacedTrapezoid>(c);
    } else {
      return -1; // the 17-value (dz, four planes) form is the product's own mirror constructor
    }
    break;
  case 15: s = new UnplacedOrb(p[0]); break; // reference only: a shape the product does not build
  default: return -1;
  }
  g->shapes.push_back(s);
  return (int)g->shapes.size() - 1;
}

int oracle_add_lv(void *, int shape)
{
  RefGeometry *g = g_geom;
  g->lvs.push_back(new LogicalVolume(g->shapes.at(shape)));
  return (int)g->lvs.size() - 1;
}

int oracle_place(void *, int lv, const double *tr, const double *rot)
{
  RefGeometry *g = g_geom;
  g->lvs.at(lv)->Place(make_transform(tr, rot));
  return g->npv++;
}

int oracle_place_daughter(void *, int mother, int lv, const double *tr, const double *rot)
{
  RefGeometry *g = g_geom;
  g->lvs.at(mother)->PlaceDaughter(g->lvs.at(lv), make_transform(tr, rot));
  return g->npv++;
}

void oracle_set_world(void *, int pv) { g_geom->world = pv; }

// GeoManager::SetWorldAndClose (placed-volume compaction, bounding boxes, the navigation
// index table), then the BVHs (BVHManager::Init) and, for every logical volume with
// daughters, the BVH navigator and level locator, the combination the device path
// reproduces. A volume without daughters has no BVH (BVHManager.cpp:24-30) and keeps the
// default NewSimpleNavigator (LogicalVolume.cpp:61-62), as the reference's own set-up does
// (test/globalbenchmarks/XRayBenchmarkFromROOTFile.cpp:203-214): both step with the
// mother's DistanceToOut alone there.
int oracle_close(void *)
{
  RefGeometry *g = g_geom;
  if (g->closed || g->world < 0) return -1;
  GeoManager::Instance().SetWorldAndClose(pv_at(g->world));
  BVHManager::Init();
  for (auto &lvol : GeoManager::Instance().GetLogicalVolumesMap()) {
    if (lvol.second->GetDaughters().size() == 0) continue;
    lvol.second->SetNavigator(BVHNavigator<>::Instance());
    lvol.second->SetLevelLocator(BVHLevelLocator::GetInstance());
  }
  g->closed = true;
  return 0;
}

int oracle_shape_extent(void *, int shape, double *lo, double *hi)
{
  Vector3D<Precision> a, b;
  g_geom->shapes.at(shape)->Extent(a, b);
  for (int k = 0; k < 3; ++k)
    lo[k] = a[k], hi[k] = b[k];
  return 0;
}

// q: 0 Inside, 1 Contains, 2 DistanceToIn, 3 DistanceToOut, 4 SafetyToIn, 5 SafetyToOut,
// 6 PlacedDistanceToOut (VPlacedVolume's virtual interface).
double oracle_placed_query(void *, int pv, int q, size_t n, const double *x, const double *y, const double *z,
                           const double *dx, const double *dy, const double *dz, double step_max, double *outd,
                           int *outi, int nthreads)
{
  VPlacedVolume const *v = pv_at(pv);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const Vector3D<Precision> p(x[i], y[i], z[i]);
      switch (q) {
      case 0: outi[i] = v->Inside(p); break;
      case 1: outi[i] = v->Contains(p) ? 1 : 0; break;
      case 2: outd[i] = v->DistanceToIn(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), step_max); break;
      case 3: outd[i] = v->DistanceToOut(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), step_max); break;
      case 4: outd[i] = v->SafetyToIn(p); break;
      case 5: outd[i] = v->SafetyToOut(p); break;
      case 6: outd[i] = v->PlacedDistanceToOut(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), step_max); break;
      }
    }
  });
}

// The same queries on an unplaced shape (VUnplacedVolume), points in its own frame.
double oracle_shape_query(void *, int shape, int q, size_t n, const double *x, const double *y, const double *z,
                          const double *dx, const double *dy, const double *dz, double step_max, double *outd,
                          int *outi, int nthreads)
{
  VUnplacedVolume const *s = g_geom->shapes.at(shape);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const Vector3D<Precision> p(x[i], y[i], z[i]);
      switch (q) {
      case 0: outi[i] = s->Inside(p); break;
      case 1: outi[i] = s->Contains(p) ? 1 : 0; break;
      case 2: outd[i] = s->DistanceToIn(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), step_max); break;
      case 3: outd[i] = s->DistanceToOut(p, Vector3D<Precision>(dx[i], dy[i], dz[i]), step_max); break;
      case 4: outd[i] = s->SafetyToIn(p); break;
      case 5: outd[i] = s->SafetyToOut(p); break;
      }
    }
  });
}

// The table as allocated (NavIndexTable.h AllocateTable: GetTableSize() / 4 + 1 words).
// GetTableSize() counts each node without the one word of padding that aligns the world's
// matrix (source/NavIndexTable.cpp:24 against :71), so the last word of the last matrix
// lies in the extra word the allocation adds; every word of the allocation is written.
size_t oracle_nav_table_words(void *) { return NavIndexTable::Instance()->GetTableSize() / sizeof(NavIndex_t) + 1; }
void oracle_nav_table(void *, uint32_t *out)
{
  std::memcpy(out, NavIndexTable::Instance()->GetTable(), oracle_nav_table_words(nullptr) * sizeof(NavIndex_t));
}
int oracle_max_depth(void *) { return GeoManager::Instance().getMaxDepth(); }

// GlobalLocator::LocateGlobalPoint(world, p, state, true) per track.
double oracle_nav_locate(void *, size_t n, const double *x, const double *y, const double *z, void *out,
                         int nthreads)
{
  VPlacedVolume const *world = GeoManager::Instance().GetWorld();
  char *o                    = static_cast<char *>(out);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      NavigationState s;
      GlobalLocator::LocateGlobalPoint(world, Vector3D<Precision>(x[i], y[i], z[i]), s, true);
      from_state(s, o + 12 * i);
    }
  });
}

// One ComputeStepAndPropagatedState per track with the navigator of the state's volume.
// States outside the world are passed through with step 0, as the hand-written oracle does
// (the reference would dereference a null volume). No node count (nvisited must be null).
double oracle_nav_step(void *, size_t n, const double *x, const double *y, const double *z, const double *dx,
                       const double *dy, const double *dz, const double *step_limit, const void *in, void *out,
                       double *step, int *nvisited, int nthreads)
{
  if (nvisited) return -1.0;
  const char *ip = static_cast<const char *>(in);
  char *op       = static_cast<char *>(out);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      NavigationState si = to_state(ip + 12 * i), so;
      if (si.IsOutside()) {
        from_state(si, op + 12 * i);
        step[i] = 0.;
        continue;
      }
      VNavigator const *nav = si.Top()->GetLogicalVolume()->GetNavigator();
      step[i] = nav->ComputeStepAndPropagatedState(Vector3D<Precision>(x[i], y[i], z[i]),
                                                   Vector3D<Precision>(dx[i], dy[i], dz[i]), step_limit[i], si, so);
      from_state(so, op + 12 * i);
    }
  });
}

// ComputeStepAndSafetyAndPropagatedState (calcsafety = true) per track.
double oracle_nav_step_safety(void *, size_t n, const double *x, const double *y, const double *z, const double *dx,
                              const double *dy, const double *dz, const double *step_limit, const void *in, void *out,
                              double *step, double *safety, int nthreads)
{
  const char *ip = static_cast<const char *>(in);
  char *op       = static_cast<char *>(out);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      NavigationState si = to_state(ip + 12 * i), so;
      VNavigator const *nav = si.Top()->GetLogicalVolume()->GetNavigator();
      step[i] = nav->ComputeStepAndSafetyAndPropagatedState(Vector3D<Precision>(x[i], y[i], z[i]),
                                                            Vector3D<Precision>(dx[i], dy[i], dz[i]), step_limit[i],
                                                            si, so, true, safety[i]);
      from_state(so, op + 12 * i);
    }
  });
}

// Straight tracks transported to the world's edge: ComputeStepAndPropagatedState with the
// step limit kInfLength, the point moved by step * direction, until the state leaves the
// world or max_steps is reached. Per track the number of steps and the final state; `trace`
// and `trace_step` (nullable, n * max_steps) receive each step's nav index and length.
double oracle_nav_transport(void *, size_t n, const double *x, const double *y, const double *z, const double *dx,
                            const double *dy, const double *dz, const void *in, int max_steps, int *nsteps,
                            void *final_state, uint32_t *trace, double *trace_step, int nthreads)
{
  const char *ip = static_cast<const char *>(in);
  char *fp       = static_cast<char *>(final_state);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      Vector3D<Precision> p(x[i], y[i], z[i]);
      const Vector3D<Precision> d(dx[i], dy[i], dz[i]);
      NavigationState s = to_state(ip + 12 * i), o;
      int k             = 0;
      while (!s.IsOutside() && k < max_steps) {
        VNavigator const *nav = s.Top()->GetLogicalVolume()->GetNavigator();
        const Precision st    = nav->ComputeStepAndPropagatedState(p, d, kInfLength, s, o);
        if (trace) trace[i * (size_t)max_steps + k] = o.GetNavIndex();
        if (trace_step) trace_step[i * (size_t)max_steps + k] = st;
        p = p + st * d;
        s = o;
        ++k;
      }
      nsteps[i] = k;
      from_state(s, fp + 12 * i);
    }
  });
}

// The reference-side bridge (include/vecgeom_gb300_mirror.hpp) on the closed geometry:
// mirror it into the product geometry `g` (a vg_geom handle created by the caller).
int oracle_mirror_to_product(void *g, int32_t *failed_pv)
{
  return vecgeom_gb300::MirrorGeometry(static_cast<vg_geom *>(g), failed_pv);
}

// The reference-side navigator adapter (include/vecgeom_gb300_navigator.hpp) installed on
// every volume with daughters, in place of BVHNavigator, with no product geometry: its
// per-track methods (the ones that stay on the host) step the tracks, one
// ComputeStepAndPropagatedState each, as oracle_nav_step does with the reference navigator.
double oracle_adapter_step(size_t n, const double *x, const double *y, const double *z, const double *dx,
                           const double *dy, const double *dz, const double *step_limit, const void *in, void *out,
                           double *step)
{
  static vecgeom_gb300::GPUNavigator adapter(nullptr, 0);
  for (auto &lvol : GeoManager::Instance().GetLogicalVolumesMap())
    if (lvol.second->GetDaughters().size() > 0) lvol.second->SetNavigator(&adapter);
  const char *ip = static_cast<const char *>(in);
  char *op       = static_cast<char *>(out);
  for (size_t i = 0; i < n; ++i) {
    NavigationState si = to_state(ip + 12 * i), so;
    if (si.IsOutside()) {
      from_state(si, op + 12 * i);
      step[i] = 0.;
      continue;
    }
    VNavigator const *nav = si.Top()->GetLogicalVolume()->GetNavigator();
    step[i] = nav->ComputeStepAndPropagatedState(Vector3D<Precision>(x[i], y[i], z[i]),
                                                 Vector3D<Precision>(dx[i], dy[i], dz[i]), step_limit[i], si, so);
    from_state(so, op + 12 * i);
  }
  for (auto &lvol : GeoManager::Instance().GetLogicalVolumesMap())
    if (lvol.second->GetDaughters().size() > 0) lvol.second->SetNavigator(BVHNavigator<>::Instance());
  return 0.0;
}

} // extern "C"
