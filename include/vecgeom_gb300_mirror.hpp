/* vecgeom_gb300_mirror.hpp — the reference-side bridge: mirror a closed VecGeom geometry
 * into a vg_geom through the C-ABI (header-only; compile it in a translation unit that
 * has VecGeom's headers on its include path and links libvecgeom_gb300).
 *
 *   vg_geom *g = nullptr;
 *   vg_geom_create(&g);
 *   if (vecgeom_gb300::MirrorGeometry(g) == VG_OK) vg_geom_close(g);
 *
 * Replays the geometry held by vecgeom::GeoManager (after CloseGeometry or SetWorldAndClose)
 * with the builder calls of vecgeom_gb300.h, so that placed-volume ids, daughter orders,
 * transformations and shape parameters are the reference's, and with them the NavIndex
 * table, the BVHs and every query result: placed volumes in id order (VPlacedVolume ids,
 * source/PlacedVolume.cpp:32), logical volumes and their shapes in id order, each
 * placement with the 12 numbers of its Transformation3D (Transformation3D.h:116-118), every
 * daughter with vg_geom_place_daughter in its mother's GetDaughters() order, boolean
 * operands (already placed, smaller ids) by id.
 *
 * Shapes: Box, Tube, Cone, Polycone (its historical z/rmin/rmax planes), Polyhedron, Torus2,
 * Trd, Trapezoid (the side planes it holds, bit-exact), Sphere, Hype, GenTrap, CutTube and
 * the boolean subtraction. Any other shape (a scaled shape, an assembly, a union ...) makes
 * MirrorGeometry return VG_EINVAL with the placed volume in *failed_pv: keep that geometry
 * on the reference's own path.
 */
#ifndef VECGEOM_GB300_MIRROR_HPP
#define VECGEOM_GB300_MIRROR_HPP

#include "vecgeom_gb300.h"

#include "VecGeom/management/GeoManager.h"
#include "VecGeom/volumes/LogicalVolume.h"
#include "VecGeom/volumes/PlacedVolume.h"
#include "VecGeom/volumes/UnplacedBooleanVolume.h"
#include "VecGeom/volumes/UnplacedBox.h"
#include "VecGeom/volumes/UnplacedCone.h"
#include "VecGeom/volumes/UnplacedCutTube.h"
#include "VecGeom/volumes/UnplacedGenTrap.h"
#include "VecGeom/volumes/UnplacedHype.h"
#include "VecGeom/volumes/UnplacedPolycone.h"
#include "VecGeom/volumes/UnplacedPolyhedron.h"
#include "VecGeom/volumes/UnplacedSphere.h"
#include "VecGeom/volumes/UnplacedTorus2.h"
#include "VecGeom/volumes/UnplacedTrapezoid.h"
#include "VecGeom/volumes/UnplacedTrd.h"
#include "VecGeom/volumes/UnplacedTube.h"

#include <map>
#include <vector>

namespace vecgeom_gb300 {

namespace mirror_detail {

using namespace vecgeom;

struct Mirror {
  vg_geom *g;
  std::map<LogicalVolume const *, int32_t> lv_id;       // reference logical volume -> vg id
  std::map<VPlacedVolume const *, int32_t> pv_id;       // reference placed volume -> vg id
  std::map<VPlacedVolume const *, LogicalVolume const *> mother;

  // VG_OK-style codes: >= 0 an id, < 0 an error; -2 an operand that is not placed yet
  int32_t Shape(VUnplacedVolume const *u)
  {
    if (auto b = dynamic_cast<UnplacedBox const *>(u)) return vg_geom_add_box(g, b->x(), b->y(), b->z());
    if (auto t = dynamic_cast<UnplacedCutTube const *>(u)) {
      // the stored unit normals; the product normalises again, which keeps a unit vector
      auto bn = t->BottomNormal(), tn = t->TopNormal();
      return vg_geom_add_cut_tube(g, t->rmin(), t->rmax(), t->z(), t->sphi(), t->dphi(), bn.x(), bn.y(), bn.z(),
                                  tn.x(), tn.y(), tn.z());
    }
    if (auto t = dynamic_cast<UnplacedTube const *>(u))
      return vg_geom_add_tube(g, t->rmin(), t->rmax(), t->z(), t->sphi(), t->dphi());
    if (auto c = dynamic_cast<UnplacedCone const *>(u)) {
      auto const &s = c->GetStruct();
      return vg_geom_add_cone(g, s.fRmin1, s.fRmax1, s.fRmin2, s.fRmax2, s.fDz, s.fSPhi, s.fDPhi);
    }
    if (auto p = dynamic_cast<UnplacedPolycone const *>(u)) {
      PolyconeHistorical const *h = p->GetStruct().GetOriginalParameters();
      const int nz                = h->fHNum_z_planes;
      return vg_geom_add_polycone(g, h->fHStart_angle, h->fHOpening_angle, nz, h->fHZ_values, h->fHRmin, h->fHRmax);
    }
    if (auto p = dynamic_cast<UnplacedPolyhedron const *>(u)) {
      const int nz = (int)p->GetZPlanes().size();
      return vg_geom_add_polyhedron(g, p->GetPhiStart(), p->GetPhiDelta(), p->GetSideCount(), nz, &p->GetZPlanes()[0],
                                    &p->GetRMin()[0], &p->GetRMax()[0]);
    }
    if (auto t = dynamic_cast<UnplacedTorus2 const *>(u))
      return vg_geom_add_torus2(g, t->rmin(), t->rmax(), t->rtor(), t->sphi(), t->dphi());
    if (auto t = dynamic_cast<UnplacedTrd const *>(u))
      return vg_geom_add_trd(g, t->dx1(), t->dx2(), t->dy1(), t->dy2(), t->dz());
    if (auto t = dynamic_cast<UnplacedTrapezoid const *>(u)) {
      auto const &s = t->GetStruct();
      double pl[16];
      for (unsigned i = 0; i < 4; ++i) {
        auto const q = s.GetPlane(i);
        pl[4 * i] = q.fA, pl[4 * i + 1] = q.fB, pl[4 * i + 2] = q.fC, pl[4 * i + 3] = q.fD;
      }
      return vg_geom_add_trap_planes(g, s.fDz, pl);
    }
    if (auto s = dynamic_cast<UnplacedSphere const *>(u))
      return vg_geom_add_sphere(g, s->GetInnerRadius(), s->GetOuterRadius(), s->GetStartPhiAngle(),
                                s->GetDeltaPhiAngle(), s->GetStartThetaAngle(), s->GetDeltaThetaAngle());
    if (auto h = dynamic_cast<UnplacedHype const *>(u))
      return vg_geom_add_hype(g, h->GetRmin(), h->GetRmax(), h->GetStIn(), h->GetStOut(), h->GetDz());
    if (auto t = dynamic_cast<UnplacedGenTrap const *>(u))
      return vg_geom_add_gentrap(g, t->GetVerticesX(), t->GetVerticesY(), t->GetDZ());
    if (auto b = dynamic_cast<UnplacedBooleanVolume<kSubtraction> const *>(u)) {
      auto l = pv_id.find(b->GetLeft()), r = pv_id.find(b->GetRight());
      if (l == pv_id.end() || r == pv_id.end()) return -2;
      return vg_geom_add_boolean_subtraction(g, l->second, r->second);
    }
    return VG_EINVAL;
  }

  // Logical volumes are created in the reference's id order (LogicalVolume::id()): a volume
  // that is needed first creates every lower-id one not created yet, each with its shape.
  std::vector<LogicalVolume const *> lv_order;
  size_t lv_next = 0;

  int32_t Logical(LogicalVolume const *lv)
  {
    auto it = lv_id.find(lv);
    if (it != lv_id.end()) return it->second;
    while (lv_next < lv_order.size()) {
      LogicalVolume const *l = lv_order[lv_next++];
      const int32_t s        = Shape(l->GetUnplacedVolume());
      if (s < 0) return s;
      const int32_t id = vg_geom_add_logical_volume(g, s);
      if (id < 0) return id;
      lv_id[l] = id;
      if (l == lv) return id;
    }
    return VG_EINVAL;
  }

  int32_t Place(VPlacedVolume const *pv)
  {
    const int32_t lv = Logical(pv->GetLogicalVolume());
    if (lv < 0) return lv;
    Transformation3D const *t = pv->GetTransformation();
    double tr[3], rot[9];
    for (int k = 0; k < 3; ++k)
      tr[k] = t->Translation(k);
    for (int k = 0; k < 9; ++k)
      rot[k] = t->Rotation(k);
    auto m       = mother.find(pv);
    int32_t id   = -1;
    if (m == mother.end()) {
      id = vg_geom_place(g, lv, tr, rot);
    } else {
      const int32_t mlv = Logical(m->second);
      if (mlv < 0) return mlv;
      id = vg_geom_place_daughter(g, mlv, lv, tr, rot);
    }
    if (id >= 0) pv_id[pv] = id;
    return id;
  }
};

} // namespace mirror_detail

/** Mirror the geometry of vecgeom::GeoManager::Instance() into `g` (freshly created, nothing
 *  added) and set its world; the caller then calls vg_geom_close (or vg_geom_build). On
 *  VG_EINVAL, *failed_pv (nullable) receives the id of the placed volume that could not be
 *  mirrored. */
inline int MirrorGeometry(vg_geom *g, int32_t *failed_pv = nullptr)
{
  using namespace vecgeom;
  GeoManager &gm = GeoManager::Instance();
  if (!g || !gm.GetWorld()) return VG_EINVAL;
  mirror_detail::Mirror m{g, {}, {}, {}, {}, 0};
  for (auto const &e : gm.GetLogicalVolumesMap()) { // keyed by id, so in id order
    m.lv_order.push_back(e.second);
    for (VPlacedVolume const *d : e.second->GetDaughters())
      m.mother[d] = e.second;
  }
  const int n = (int)gm.GetPlacedVolumesCount();
  for (int k = 0; k < n; ++k) {
    VPlacedVolume const *pv = gm.FindPlacedVolume(k);
    const int32_t id        = pv ? m.Place(pv) : VG_EINVAL;
    if (id != k) { // ids must come out as the reference's
      if (failed_pv) *failed_pv = k;
      return id < 0 ? id : VG_EINVAL;
    }
  }
  auto w = m.pv_id.find(gm.GetWorld());
  if (w == m.pv_id.end()) return VG_EINVAL;
  return vg_geom_set_world(g, w->second);
}

} // namespace vecgeom_gb300

#endif
