/* vecgeom_gb300_navigator.hpp — the reference-side navigator adapter: a vecgeom::VNavigator
 * whose vector-navigation entry point runs on the GPU (header-only; compile it where
 * VecGeom's headers are on the include path, built with VECGEOM_USE_NAVINDEX so that a
 * NavigationState is the 12-byte NavStateIndex, and link libvecgeom_gb300).
 *
 *   vg_geom *g = ...;  // vecgeom_gb300::MirrorGeometry + vg_geom_close (vecgeom_gb300_mirror.hpp)
 *   vecgeom_gb300::GPUNavigator nav(g, VG_PREC_MIXED | VG_NAV_SORT | VG_NAV_QUEUE);
 *   for (auto &lv : vecgeom::GeoManager::Instance().GetLogicalVolumesMap())
 *     if (lv.second->GetDaughters().size()) lv.second->SetNavigator(&nav);
 *   nav.ComputeStepsAndPropagatedStates(points, dirs, limits, in_states, out_states, steps);
 *
 * ComputeStepsAndPropagatedStates (VecGeom/navigation/VNavigator.h:127-132) gathers the
 * batch's states into one array, makes one call of the host-array entry point
 * vg_nav_compute_step_and_next_volume_host (copies, sort, persistent step kernel) and
 * scatters the out-states back: one GPU call per basket instead of one CPU step per track,
 * with results identical to the reference's BVHNavigator. Every per-track method (and the
 * other vector methods) is served by the reference navigator the adapter wraps
 * (BVHNavigator<> by default), so the adapter can replace it on any logical volume.
 */
#ifndef VECGEOM_GB300_NAVIGATOR_HPP
#define VECGEOM_GB300_NAVIGATOR_HPP

#include "vecgeom_gb300.h"

#include "VecGeom/base/SOA3D.h"
#include "VecGeom/navigation/BVHNavigator.h"
#include "VecGeom/navigation/NavigationState.h"
#include "VecGeom/navigation/VNavigator.h"

#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace vecgeom_gb300 {

class GPUNavigator : public vecgeom::VNavigator {
  using Precision         = vecgeom::Precision;
  using NavigationState   = vecgeom::NavigationState;
  using Vec3              = vecgeom::Vector3D<Precision>;
  using SOA3D             = vecgeom::SOA3D<Precision>;
  using LogicalVolume     = vecgeom::LogicalVolume;
  using VPlacedVolume     = vecgeom::VPlacedVolume;

  static_assert(sizeof(NavigationState) == sizeof(vg_navstate) && std::is_trivially_copyable<NavigationState>::value,
                "the adapter needs the NavIndex build: NavStateIndex = {nav index, last exited, on boundary}");

  vg_geom *g_;
  uint32_t flags_;
  void *stream_;
  vecgeom::VNavigator const *cpu_;

public:
  GPUNavigator(vg_geom *g, uint32_t flags, void *stream = nullptr,
               vecgeom::VNavigator const *cpu = vecgeom::BVHNavigator<>::Instance())
      : vecgeom::VNavigator(const_cast<vecgeom::VSafetyEstimator *>(cpu->GetSafetyEstimator())), g_(g),
        flags_(flags), stream_(stream), cpu_(cpu)
  {
  }

  const char *GetName() const override { return "GPUNavigator"; }

  // ------------------------------------------------ the vector entry point, on the GPU
  void ComputeStepsAndPropagatedStates(SOA3D const &p, SOA3D const &d, Precision const *limits,
                                       NavigationState const *const *in, NavigationState **out,
                                       Precision *steps) const override
  {
    const size_t n = p.size();
    std::vector<vg_navstate> sin(n), sout(n);
    for (size_t i = 0; i < n; ++i)
      std::memcpy(&sin[i], static_cast<void const *>(in[i]), sizeof(vg_navstate));
    const int rc = vg_nav_compute_step_and_next_volume_host(g_, p.x(), p.y(), p.z(), d.x(), d.y(), d.z(), limits,
                                                            sin.data(), sout.data(), steps, nullptr, n, flags_,
                                                            stream_);
    if (rc != VG_OK) throw std::runtime_error(vg_last_error());
    for (size_t i = 0; i < n; ++i)
      std::memcpy(static_cast<void *>(out[i]), &sout[i], sizeof(vg_navstate));
  }

  // ------------------------------------------------ everything else: the wrapped navigator
  Precision ComputeStepAndPropagatedState(Vec3 const &gp, Vec3 const &gd, Precision limit, NavigationState const &in,
                                          NavigationState &out) const override
  {
    return cpu_->ComputeStepAndPropagatedState(gp, gd, limit, in, out);
  }
  Precision ComputeStep(Vec3 const &gp, Vec3 const &gd, Precision limit, NavigationState const &in,
                        NavigationState &out) const override
  {
    return cpu_->ComputeStep(gp, gd, limit, in, out);
  }
  Precision ComputeStepAndSafety(Vec3 const &gp, Vec3 const &gd, Precision limit, NavigationState &in, bool calcsafety,
                                 Precision &safety, bool indicateDaughterHit = false) const override
  {
    return cpu_->ComputeStepAndSafety(gp, gd, limit, in, calcsafety, safety, indicateDaughterHit);
  }
  Precision ComputeStepAndSafetyAndPropagatedState(Vec3 const &gp, Vec3 const &gd, Precision limit,
                                                   NavigationState const &in, NavigationState &out, bool calcsafety,
                                                   Precision &safety) const override
  {
    return cpu_->ComputeStepAndSafetyAndPropagatedState(gp, gd, limit, in, out, calcsafety, safety);
  }
  bool CheckDaughterIntersections(LogicalVolume const *lv, Vec3 const &lp, Vec3 const &ld, NavigationState const *in,
                                  NavigationState *out, Precision &step, VPlacedVolume const *&hit) const override
  {
    return cpu_->CheckDaughterIntersections(lv, lp, ld, in, out, step, hit);
  }
  bool CheckDaughterIntersections(LogicalVolume const *lv, Vec3 const &lp, Vec3 const &ld, VPlacedVolume const *blocked,
                                  Precision &step, VPlacedVolume const *&hit) const override
  {
    return cpu_->CheckDaughterIntersections(lv, lp, ld, blocked, step, hit);
  }
  void ComputeStepsAndSafetiesAndPropagatedStates(SOA3D const &p, SOA3D const &d, Precision const *limits,
                                                  vecgeom::NavStatePool const &in, vecgeom::NavStatePool &out,
                                                  Precision *steps, bool const *calcsafety,
                                                  Precision *safeties) const override
  {
    cpu_->ComputeStepsAndSafetiesAndPropagatedStates(p, d, limits, in, out, steps, calcsafety, safeties);
  }
  void ComputeStepsAndSafetiesAndPropagatedStates(SOA3D const &p, SOA3D const &d, Precision const *limits,
                                                  NavigationState const *const *in, NavigationState **out,
                                                  Precision *steps, bool const *calcsafety,
                                                  Precision *safeties) const override
  {
    cpu_->ComputeStepsAndSafetiesAndPropagatedStates(p, d, limits, in, out, steps, calcsafety, safeties);
  }
  void ComputeStepsAndSafeties(SOA3D const &p, SOA3D const &d, Precision const *limits,
                               NavigationState const *const *in, Precision *steps, bool const *calcsafety,
                               Precision *safeties) const override
  {
    cpu_->ComputeStepsAndSafeties(p, d, limits, in, steps, calcsafety, safeties);
  }

protected:
  // VNavigator's shared relocation hook; the reference's helpers call it only from inside
  // their own step methods, which this adapter forwards whole to the wrapped navigator.
  void Relocate(Vec3 const &, NavigationState const &__restrict__, NavigationState &__restrict__) const override
  {
    throw std::logic_error("GPUNavigator::Relocate is not used: steps are forwarded whole");
  }
};

} // namespace vecgeom_gb300

#endif
