// ORACLE — TEST INFRASTRUCTURE ONLY (see ref_base.h).
//
// extern "C" surface of the oracle for ctypes (tests, smoke check, bench cpu_baseline).
// Geometry is described with the same call sequence as the product's C-ABI, so both
// sides assign identical placed-volume ids and child ids. Batched queries split the
// track range into contiguous chunks over std::thread workers.
#include "ref_nav.h"
#include "ref_shapes_more.h"
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

using namespace oracle;

namespace {
template <class F>
double ParallelFor(size_t n, int nthreads, F &&f)
{
  auto t0 = std::chrono::steady_clock::now();
  if (nthreads <= 1 || n < 1024) {
    f(0, n);
  } else {
    std::vector<std::thread> th;
    const size_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
      const size_t b = t * chunk, e = std::min(n, b + chunk);
      if (b >= e) break;
      th.emplace_back([&f, b, e]() { f(b, e); });
    }
    for (auto &t : th) t.join();
  }
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
} // namespace

extern "C" {

void *oracle_geom_create() { return new Geometry(); }
void oracle_geom_destroy(void *g) { delete static_cast<Geometry *>(g); }

// type: 1 Box, 2 Tube, 3 Cone, 4 Polycone, 5 Polyhedron, 6 Torus2, 7 Trd, 8 BooleanSubtraction,
// 10 BooleanUnion (oracle only), 11 CutTube (rmin, rmax, dz, sphi, dphi, bottom normal, top
// normal), 12 Sphere (rmin, rmax, sphi, dphi, stheta, dtheta), 13 GenTrap (x of the eight
// vertices, their y, dz), 14 Hype (rmin, rmax, inner stereo angle, outer stereo angle, dz),
// 9 Trapezoid (11 parameters, 24 = eight corners x, y, z, or 17 = dz and four planes a, b, c, d)
int oracle_add_shape(void *gp, int type, const double *p, int np)
{
  Geometry *g = static_cast<Geometry *>(gp);
  UnplacedShape *s = nullptr;
  switch (type) {
  case 1: s = new Box(p[0], p[1], p[2]); break;
  case 2: s = new Tube(p[0], p[1], p[2], p[3], p[4]); break;
  case 3: s = new Cone(p[0], p[1], p[2], p[3], p[4], p[5], p[6]); break;
  case 4: {
    const int nz = (int)p[2];
    s            = new Polycone(p[0], p[1], nz, p + 3, p + 3 + nz, p + 3 + 2 * nz);
    break;
  }
  case 5: {
    const int nz = (int)p[3];
    s            = new Polyhedron(p[0], p[1], (int)p[2], nz, p + 4, p + 4 + nz, p + 4 + 2 * nz);
    break;
  }
  case 6: s = new Torus2(p[0], p[1], p[2], p[3], p[4]); break;
  case 7: s = new Trd(p[0], p[1], p[2], p[3], p[4]); break;
  case 8: s = new BooleanMinus(g->pvs.at((int)p[0]).get(), g->pvs.at((int)p[1]).get()); break;
  case 10: s = new BooleanUnion(g->pvs.at((int)p[0]).get(), g->pvs.at((int)p[1]).get()); break;
  case 12: s = new Sphere(p[0], p[1], p[2], p[3], p[4], p[5]); break;
  case 13:
    if (np != 17) return -1;
    s = new GenTrap(p, p + 8, p[16]);
    break;
  case 14: s = new Hype(p[0], p[1], p[2], p[3], p[4]); break;
  case 11: s = new CutTube(p[0], p[1], p[2], p[3], p[4], Vec3(p[5], p[6], p[7]), Vec3(p[8], p[9], p[10])); break;
  case 9:
    if (np == 24) {
      Vec3 c[8];
      for (int k = 0; k < 8; ++k) c[k] = Vec3(p[3 * k], p[3 * k + 1], p[3 * k + 2]);
      s = new Trap(c);
    } else if (np == 11) {
      s = new Trap(p);
    } else if (np == 17) {
      s = new Trap(p[0], p + 1);
    } else {
      return -1;
    }
    break;
  default: return -1;
  }
  (void)np;
  return g->AddShape(s);
}
int oracle_add_lv(void *g, int shape) { return static_cast<Geometry *>(g)->AddLogicalVolume(shape); }
int oracle_place(void *g, int lv, const double *tr, const double *rot)
{
  return static_cast<Geometry *>(g)->Place(lv, tr, rot);
}
int oracle_place_daughter(void *g, int mother, int lv, const double *tr, const double *rot)
{
  return static_cast<Geometry *>(g)->PlaceDaughter(mother, lv, tr, rot);
}
void oracle_set_world(void *g, int pv) { static_cast<Geometry *>(g)->world = static_cast<Geometry *>(g)->pvs.at(pv).get(); }
int oracle_close(void *g)
{
  try {
    static_cast<Geometry *>(g)->Close();
  } catch (...) {
    return -1;
  }
  return 0;
}
int oracle_shape_extent(void *gp, int shape, double *lo, double *hi)
{
  Vec3 a, b;
  static_cast<Geometry *>(gp)->shapes.at(shape)->Extent(a, b);
  for (int i = 0; i < 3; ++i) lo[i] = a[i], hi[i] = b[i];
  return 0;
}

// GenTrapStruct::Initialize on the given vertices: 1 when the reference accepts them, 0 when
// it reports an error (and keeps a half-built shape).
int oracle_gentrap_valid(const double *vx, const double *vy, double dz)
{
  double x[8], y[8];
  for (int i = 0; i < 8; ++i) x[i] = vx[i], y[i] = vy[i];
  const char *err = nullptr;
  return GenTrap::Initialize(x, y, dz, &err) ? 1 : 0;
}

// VUnplacedVolume::Normal of a shape at a point in its frame (restated for the shapes whose
// known-answer tests need it); returns the valid flag.
int oracle_shape_normal(void *gp, int shape, const double *p, double *n)
{
  bool valid  = false;
  const Vec3 v = static_cast<Geometry *>(gp)->shapes.at(shape)->Normal(Vec3(p[0], p[1], p[2]), valid);
  for (int k = 0; k < 3; ++k) n[k] = v[k];
  return valid ? 1 : 0;
}

// q: 0 Inside, 1 Contains, 2 DistanceToIn, 3 DistanceToOut, 4 SafetyToIn, 5 SafetyToOut.
// Returns the wall time of the batched loop (seconds).
double oracle_placed_query(void *gp, int pv, int q, size_t n, const double *x, const double *y, const double *z,
                           const double *dx, const double *dy, const double *dz, double step_max, double *outd,
                           int *outi, int nthreads)
{
  Geometry *g           = static_cast<Geometry *>(gp);
  PlacedVolume const *v = g->pvs.at(pv).get();
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const Vec3 p(x[i], y[i], z[i]);
      switch (q) {
      case 0: outi[i] = v->Inside(p); break;
      case 1: outi[i] = v->Contains(p) ? 1 : 0; break;
      case 2: outd[i] = v->DistanceToIn(p, Vec3(dx[i], dy[i], dz[i]), step_max); break;
      case 3: outd[i] = v->DistanceToOut(p, Vec3(dx[i], dy[i], dz[i]), step_max); break;
      case 4: outd[i] = v->SafetyToIn(p); break;
      case 5: outd[i] = v->SafetyToOut(p); break;
      case 6: outd[i] = v->PlacedDistanceToOut(p, Vec3(dx[i], dy[i], dz[i]), step_max); break;
      }
    }
  });
}

// The same queries on an unplaced shape, points in its own frame (VUnplacedVolume).
double oracle_shape_query(void *gp, int shape, int q, size_t n, const double *x, const double *y, const double *z,
                          const double *dx, const double *dy, const double *dz, double step_max, double *outd,
                          int *outi, int nthreads)
{
  Geometry *g            = static_cast<Geometry *>(gp);
  UnplacedShape const *s = g->shapes.at(shape).get();
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const Vec3 p(x[i], y[i], z[i]);
      switch (q) {
      case 0: outi[i] = s->Inside(p); break;
      case 1: outi[i] = s->Contains(p) ? 1 : 0; break;
      case 2: outd[i] = s->DistanceToIn(p, Vec3(dx[i], dy[i], dz[i]), step_max); break;
      case 3: outd[i] = s->DistanceToOut(p, Vec3(dx[i], dy[i], dz[i]), step_max); break;
      case 4: outd[i] = s->SafetyToIn(p); break;
      case 5: outd[i] = s->SafetyToOut(p); break;
      }
    }
  });
}

size_t oracle_nav_table_words(void *g) { return static_cast<Geometry *>(g)->tableWords; }
void oracle_nav_table(void *gp, uint32_t *out)
{
  Geometry *g = static_cast<Geometry *>(gp);
  std::memcpy(out, g->table, g->tableWords * sizeof(uint32_t));
}
int oracle_max_depth(void *g) { return static_cast<Geometry *>(g)->maxDepth; }

// BVH arrays of logical volume `lv` (daughters > 0): sizes first, then the arrays.
int oracle_bvh_sizes(void *gp, int lv, int *nnodes, int *nprims, int *depth)
{
  Geometry *g = static_cast<Geometry *>(gp);
  BVH *b      = g->lvs.at(lv)->bvh;
  if (!b) return -1;
  *nnodes = (int)b->nodes.size();
  *nprims = (int)b->primId.size();
  *depth  = b->depth;
  return 0;
}
int oracle_bvh_arrays(void *gp, int lv, int *primId, int *offset, int *nchild, double *nodes6, double *aabbs6)
{
  Geometry *g = static_cast<Geometry *>(gp);
  BVH *b      = g->lvs.at(lv)->bvh;
  if (!b) return -1;
  for (size_t i = 0; i < b->primId.size(); ++i) primId[i] = b->primId[i];
  for (size_t i = 0; i < b->nodes.size(); ++i) {
    offset[i] = b->offset[i];
    nchild[i] = b->nchild[i];
    for (int k = 0; k < 3; ++k) nodes6[6 * i + k] = b->nodes[i].mn[k], nodes6[6 * i + 3 + k] = b->nodes[i].mx[k];
  }
  for (size_t i = 0; i < b->aabbs.size(); ++i)
    for (int k = 0; k < 3; ++k) aabbs6[6 * i + k] = b->aabbs[i].mn[k], aabbs6[6 * i + 3 + k] = b->aabbs[i].mx[k];
  return 0;
}

// GlobalLocator::LocateGlobalPoint(world, p, state, true) per track.
double oracle_nav_locate(void *gp, size_t n, const double *x, const double *y, const double *z, NavState *out,
                         int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      NavState s;
      g->LocateGlobalPoint(g->world, Vec3(x[i], y[i], z[i]), s, true);
      out[i] = s;
    }
  });
}

// One ComputeStepAndPropagatedState per track. nvisited (nullable) receives the BVH nodes popped.
double oracle_nav_step(void *gp, size_t n, const double *x, const double *y, const double *z, const double *dx,
                       const double *dy, const double *dz, const double *step_limit, const NavState *in,
                       NavState *out, double *step, int *nvisited, int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      int nv = 0;
      if (in[i].navInd == 0) { // outside the world: the reference would dereference a null volume
        out[i]  = in[i];
        step[i] = 0.;
        if (nvisited) nvisited[i] = 0;
        continue;
      }
      step[i] = g->ComputeStepAndPropagatedState(Vec3(x[i], y[i], z[i]), Vec3(dx[i], dy[i], dz[i]), step_limit[i],
                                                 in[i], out[i], nvisited ? &nv : nullptr);
      if (nvisited) nvisited[i] = nv;
    }
  });
}

// BVH::ApproachNextDaughter per track in the state's volume; step[] in/out (states outside
// the world keep their step).
double oracle_nav_approach(void *gp, size_t n, const double *x, const double *y, const double *z, const double *dx,
                           const double *dy, const double *dz, const NavState *in, double *step, int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i)
      if (in[i].navInd != 0)
        step[i] = g->ApproachNextDaughter(Vec3(x[i], y[i], z[i]), Vec3(dx[i], dy[i], dz[i]), step[i], in[i]);
  });
}

// Step + safety (VNavigator.h:1014-1064).
double oracle_nav_step_safety(void *gp, size_t n, const double *x, const double *y, const double *z,
                              const double *dx, const double *dy, const double *dz, const double *step_limit,
                              const NavState *in, NavState *out, double *step, double *safety, int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i)
      step[i] = g->ComputeStepAndSafetyAndPropagatedState(Vec3(x[i], y[i], z[i]), Vec3(dx[i], dy[i], dz[i]),
                                                          step_limit[i], in[i], out[i], safety[i]);
  });
}

// Full transport of straight tracks: step (with the step limit kInfLength) and move the
// point by the step, until the state leaves the world or max_steps is reached.
// Records per track the number of steps and the final state; `trace` (nullable, size
// n*max_steps) receives the nav index after each step, `trace_step` the step lengths.
double oracle_nav_transport(void *gp, size_t n, const double *x, const double *y, const double *z, const double *dx,
                            const double *dy, const double *dz, const NavState *in, int max_steps, int *nsteps,
                            NavState *final_state, uint32_t *trace, double *trace_step, int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      Vec3 p(x[i], y[i], z[i]);
      const Vec3 d(dx[i], dy[i], dz[i]);
      NavState s = in[i], o;
      int k      = 0;
      while (s.navInd != 0 && k < max_steps) {
        const double st = g->ComputeStepAndPropagatedState(p, d, kInfLength, s, o);
        if (trace) trace[i * (size_t)max_steps + k] = o.navInd;
        if (trace_step) trace_step[i * (size_t)max_steps + k] = st;
        p = p + st * d;
        s = o;
        ++k;
      }
      nsteps[i]      = k;
      final_state[i] = s;
    }
  });
}

// The brute-force second navigator (NewSimpleNavigator + SimpleLevelLocator): one step per
// track, as oracle_nav_step, and LocateGlobalPoint from the world.
double oracle_nav_step_simple(void *gp, size_t n, const double *x, const double *y, const double *z,
                              const double *dx, const double *dy, const double *dz, const double *step_limit,
                              const NavState *in, NavState *out, double *step, int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      if (in[i].navInd == 0) {
        out[i]  = in[i];
        step[i] = 0.;
        continue;
      }
      step[i] = g->ComputeStepAndPropagatedState(Vec3(x[i], y[i], z[i]), Vec3(dx[i], dy[i], dz[i]), step_limit[i],
                                                 in[i], out[i], nullptr, true);
    }
  });
}

double oracle_nav_locate_simple(void *gp, size_t n, const double *x, const double *y, const double *z, NavState *out,
                                int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  return ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      NavState s;
      g->LocateGlobalPoint(g->world, Vec3(x[i], y[i], z[i]), s, true, true);
      out[i] = s;
    }
  });
}

// persistency/gdml/test/TestVGDMLNavigation/TestVGDMLNavigation.cpp:38-49 nearly_equal
static bool NearlyEqual(double x, double y)
{
  if (x == y) return true;
  if (x * y == 0.0) return std::abs(x - y) < DBL_EPSILON * DBL_EPSILON;
  return std::abs(x - y) < (std::abs(x) + std::abs(y)) * DBL_EPSILON;
}

// TestVGDMLNavigation.cpp:54-91 navigate(): each track is located from its start point, then
// stepped until it leaves the world (or max_steps) with the BVH navigator, and at every step
// the brute-force navigator (NewSimpleNavigator, the reference's own reference) steps the
// same state; the point moves by max(step, kTolerance) along the direction. counts[0] steps
// compared, [1] steps not nearly equal (the reference test's criterion), [2] steps that
// differ in any bit, [3] out-states that differ in any field, [4] start states that the
// two locators place differently.
double oracle_nav_crosscheck(void *gp, size_t n, const double *x, const double *y, const double *z,
                             const double *dx, const double *dy, const double *dz, int max_steps, long *counts,
                             int nthreads)
{
  Geometry *g = static_cast<Geometry *>(gp);
  std::vector<long> part((size_t)std::max(1, nthreads) * 5, 0);
  std::atomic<int> slot{0};
  const double t = ParallelFor(n, nthreads, [&](size_t b, size_t e) {
    long *c = &part[(size_t)(slot++) * 5];
    for (size_t i = b; i < e; ++i) {
      Vec3 p(x[i], y[i], z[i]);
      const Vec3 d(dx[i], dy[i], dz[i]);
      NavState cur, cs;
      g->LocateGlobalPoint(g->world, p, cur, true);
      g->LocateGlobalPoint(g->world, p, cs, true, true);
      if (cur.navInd != cs.navInd) ++c[4];
      for (int k = 0; k < max_steps && cur.navInd != 0; ++k) {
        NavState nb, ns;
        const double ref  = g->ComputeStepAndPropagatedState(p, d, kInfLength, cur, ns, nullptr, true);
        const double step = g->ComputeStepAndPropagatedState(p, d, kInfLength, cur, nb);
        ++c[0];
        if (!NearlyEqual(step, ref)) ++c[1];
        if (std::memcmp(&step, &ref, sizeof(double)) != 0) ++c[2];
        if (nb.navInd != ns.navInd || nb.lastExited != ns.lastExited || nb.onBoundary != ns.onBoundary) ++c[3];
        p   = p + std::max(step, kTolerance) * d;
        cur = nb;
      }
    }
  });
  for (int k = 0; k < 5; ++k) {
    counts[k] = 0;
    for (size_t s2 = 0; s2 < part.size() / 5; ++s2) counts[k] += part[s2 * 5 + k];
  }
  return t;
}

// test/benchmark/TestNavIndex.cpp on a NavIndex table (this geometry's own when tab is null)
int oracle_check_nav_index(void *gp, const uint32_t *tab, size_t words, long *paths)
{
  Geometry *g = static_cast<Geometry *>(gp);
  if (!tab) return g->CheckNavIndexTable(g->table, g->tableWords, paths);
  return g->CheckNavIndexTable(tab, words, paths);
}

} // extern "C"
