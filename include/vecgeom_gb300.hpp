/* vecgeom_gb300.hpp — C++ host layer over the C-ABI (vecgeom_gb300.h) in the shape of
 * VecGeom's SoA interfaces, for C++ callers that hold their tracks in device memory.
 *
 * Reference interfaces mirrored (file:line within the VecGeom project):
 *   SOA3D<Precision> (x(), y(), z(), size())        VecGeom/base/SOA3D.h:47-64
 *   NavStatePool (a fixed pool of states)            VecGeom/navigation/NavStatePool.h
 *   VPlacedVolume SoA virtuals                       VecGeom/volumes/PlacedVolume.h:271-425
 *   VUnplacedVolume SoA virtuals                     VecGeom/volumes/UnplacedVolume.h:89-223
 *   VNavigator::ComputeStepsAndPropagatedStates      VecGeom/navigation/VNavigator.h:128-132
 *   VNavigator::ComputeStepsAndSafetiesAndPropagatedStates (NavStatePool form)
 *                                                    VecGeom/navigation/VNavigator.h:913-940
 *   GlobalLocator::LocateGlobalPoint                 VecGeom/navigation/GlobalLocator.h:35-82
 *   Inside_t / EnumInside values                     VecGeom/base/Global.h:67-80
 *
 * Differences a caller sees: the arrays are device memory (the SOA3D and NavStatePool
 * here own or view device arrays); the navigator's in/out states are NavStatePools (the
 * reference's NavigationState** form is the same data, one pointer per track); every call
 * is asynchronous on the object's stream; errors throw vecgeom_gb300::Error with the
 * library's message. Results are those of the C-ABI entry points named beside each method.
 * Header only: include it and link libvecgeom_gb300.so and the CUDA runtime. */
#pragma once

#include "vecgeom_gb300.h"

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <utility>
#include <vector>

namespace vecgeom_gb300 {

using Precision = double;
using Inside_t  = int; // VecGeom/base/Global.h:80
enum EnumInside { kInside = 1, kSurface = 2, kOutside = 3 };
static_assert(sizeof(bool) == 1, "Contains writes one byte per point");
static_assert(sizeof(Inside_t) == sizeof(int32_t), "Inside writes 32-bit codes");

class Error : public std::runtime_error {
public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

private:
  int code_;
};

inline void Check(int rc, const char *what)
{
  if (rc < 0) throw Error(rc, std::string(what) + ": " + vg_last_error());
}
inline void CheckCuda(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) throw Error(VG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Device array owned by the adapter (cudaMalloc / cudaFree).
template <typename T>
class DeviceArray {
public:
  DeviceArray() = default;
  explicit DeviceArray(size_t n) { Resize(n); }
  ~DeviceArray() { Release(); }
  DeviceArray(const DeviceArray &)            = delete;
  DeviceArray &operator=(const DeviceArray &) = delete;
  DeviceArray(DeviceArray &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
  DeviceArray &operator=(DeviceArray &&o) noexcept
  {
    if (this != &o) {
      Release();
      p_ = o.p_, n_ = o.n_;
      o.p_ = nullptr, o.n_ = 0;
    }
    return *this;
  }
  void Resize(size_t n)
  {
    if (n == n_) return;
    Release();
    if (n) CheckCuda(cudaMalloc(reinterpret_cast<void **>(&p_), n * sizeof(T)), "cudaMalloc");
    n_ = n;
  }
  T *data() { return p_; }
  const T *data() const { return p_; }
  size_t size() const { return n_; }
  void CopyFromHost(const T *h, size_t n, cudaStream_t s = nullptr)
  {
    Resize(n);
    if (n) CheckCuda(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s), "copy to device");
  }
  void CopyToHost(T *h, cudaStream_t s = nullptr) const
  {
    if (n_) CheckCuda(cudaMemcpyAsync(h, p_, n_ * sizeof(T), cudaMemcpyDeviceToHost, s), "copy to host");
    CheckCuda(cudaStreamSynchronize(s), "stream synchronize");
  }

private:
  void Release()
  {
    if (p_) cudaFree(p_);
    p_ = nullptr, n_ = 0;
  }
  T *p_     = nullptr;
  size_t n_ = 0;
};

// SOA3D<Precision> in device memory: three coordinate arrays of size() entries, either owned
// (SOA3D(n), FromHost) or viewed (SOA3D(x, y, z, n), the reference's view constructor).
template <typename T>
class SOA3D {
  static_assert(std::is_same<T, double>::value, "the kernels take FP64 SoA streams");

public:
  SOA3D() = default;
  explicit SOA3D(size_t n) : size_(n), own_x_(n), own_y_(n), own_z_(n)
  {
    x_ = own_x_.data(), y_ = own_y_.data(), z_ = own_z_.data();
  }
  SOA3D(T *x, T *y, T *z, size_t n) : x_(x), y_(y), z_(z), size_(n) {}
  static SOA3D FromHost(const T *x, const T *y, const T *z, size_t n, cudaStream_t s = nullptr)
  {
    SOA3D r(n);
    r.own_x_.CopyFromHost(x, n, s), r.own_y_.CopyFromHost(y, n, s), r.own_z_.CopyFromHost(z, n, s);
    return r;
  }
  SOA3D(SOA3D &&) noexcept            = default;
  SOA3D &operator=(SOA3D &&) noexcept = default;
  size_t size() const { return size_; }
  T *x() { return x_; }
  T *y() { return y_; }
  T *z() { return z_; }
  const T *x() const { return x_; }
  const T *y() const { return y_; }
  const T *z() const { return z_; }

private:
  T *x_ = nullptr, *y_ = nullptr, *z_ = nullptr;
  size_t size_ = 0;
  DeviceArray<T> own_x_, own_y_, own_z_;
};

// NavStatePool in device memory: one vg_navstate (bit-identical to NavStateIndex) per track.
class NavStatePool {
public:
  NavStatePool() = default;
  explicit NavStatePool(size_t n) : states_(n) {}
  size_t size() const { return states_.size(); }
  vg_navstate *data() { return states_.data(); }
  const vg_navstate *data() const { return states_.data(); }
  void CopyFromHost(const vg_navstate *h, size_t n, cudaStream_t s = nullptr) { states_.CopyFromHost(h, n, s); }
  std::vector<vg_navstate> ToHost(cudaStream_t s = nullptr) const
  {
    std::vector<vg_navstate> h(size());
    states_.CopyToHost(h.data(), s);
    return h;
  }

private:
  DeviceArray<vg_navstate> states_;
};

// A geometry: builder calls (the reference's Unplaced* constructors, LogicalVolume,
// PlaceDaughter, SetWorld, CloseGeometry) and the closed, device-resident result.
class Geometry {
public:
  Geometry() { Check(vg_geom_create(&g_), "vg_geom_create"); }
  ~Geometry() { vg_geom_destroy(g_); }
  Geometry(const Geometry &)            = delete;
  Geometry &operator=(const Geometry &) = delete;
  // A geometry saved with Save (its builder calls replayed) and closed.
  static Geometry Load(const std::string &path)
  {
    Geometry g;
    Check(vg_geom_load(g.g_, path.c_str()), "vg_geom_load");
    Check(vg_geom_close(g.g_), "vg_geom_close");
    return g;
  }
  Geometry(Geometry &&o) noexcept : g_(o.g_) { o.g_ = nullptr; }
  void Save(const std::string &path) const { Check(vg_geom_save(g_, path.c_str()), "vg_geom_save"); }
  int32_t AddBox(double dx, double dy, double dz) { return Id(vg_geom_add_box(g_, dx, dy, dz), "box"); }
  int32_t AddTube(double rmin, double rmax, double dz, double sphi, double dphi)
  {
    return Id(vg_geom_add_tube(g_, rmin, rmax, dz, sphi, dphi), "tube");
  }
  int32_t AddCone(double rmin1, double rmax1, double rmin2, double rmax2, double dz, double sphi, double dphi)
  {
    return Id(vg_geom_add_cone(g_, rmin1, rmax1, rmin2, rmax2, dz, sphi, dphi), "cone");
  }
  int32_t AddTrd(double dx1, double dx2, double dy1, double dy2, double dz)
  {
    return Id(vg_geom_add_trd(g_, dx1, dx2, dy1, dy2, dz), "trd");
  }
  int32_t AddLogicalVolume(int32_t shape) { return Id(vg_geom_add_logical_volume(g_, shape), "logical volume"); }
  int32_t Place(int32_t lv, const double trans[3], const double rot[9])
  {
    return Id(vg_geom_place(g_, lv, trans, rot), "placement");
  }
  int32_t PlaceDaughter(int32_t mother_lv, int32_t lv, const double trans[3], const double rot[9])
  {
    return Id(vg_geom_place_daughter(g_, mother_lv, lv, trans, rot), "daughter placement");
  }
  void SetWorld(int32_t pv) { Check(vg_geom_set_world(g_, pv), "vg_geom_set_world"); }
  void CloseGeometry() { Check(vg_geom_close(g_), "vg_geom_close"); }
  vg_geom *handle() { return g_; }
  const vg_geom *handle() const { return g_; }

private:
  static int32_t Id(int32_t id, const char *what)
  {
    if (id < 0) throw Error(id, std::string("adding a ") + what + ": " + vg_last_error());
    return id;
  }
  vg_geom *g_ = nullptr;
};

// Options shared by the query and navigation objects: precision flags and the stream.
struct Launch {
  uint32_t flags      = VG_PREC_FP64;
  cudaStream_t stream = nullptr;
};

// VUnplacedVolume's SoA queries on a shape by id, points in the shape's own frame
// (vg_shape_* entry points).
class UnplacedVolume {
public:
  UnplacedVolume(const Geometry &g, int32_t shape, Launch l = {}) : g_(g.handle()), id_(shape), l_(l) {}
  void Contains(SOA3D<Precision> const &p, bool *const output) const
  {
    Check(vg_shape_contains(g_, id_, p.x(), p.y(), p.z(), p.size(), reinterpret_cast<uint8_t *>(output), l_.flags,
                            l_.stream),
          "vg_shape_contains");
  }
  void Inside(SOA3D<Precision> const &p, Inside_t *const output) const
  {
    Check(vg_shape_inside(g_, id_, p.x(), p.y(), p.z(), p.size(), reinterpret_cast<int32_t *>(output), l_.flags,
                          l_.stream),
          "vg_shape_inside");
  }
  void DistanceToIn(SOA3D<Precision> const &p, SOA3D<Precision> const &d, Precision const *const step_max,
                    Precision *const output) const
  {
    Check(vg_shape_distance_to_in(g_, id_, p.x(), p.y(), p.z(), d.x(), d.y(), d.z(), step_max, p.size(), output,
                                  l_.flags, l_.stream),
          "vg_shape_distance_to_in");
  }
  void DistanceToOut(SOA3D<Precision> const &p, SOA3D<Precision> const &d, Precision const *const step_max,
                     Precision *const output) const
  {
    Check(vg_shape_distance_to_out(g_, id_, p.x(), p.y(), p.z(), d.x(), d.y(), d.z(), step_max, p.size(), output,
                                   l_.flags, l_.stream),
          "vg_shape_distance_to_out");
  }
  void SafetyToIn(SOA3D<Precision> const &p, Precision *const output) const
  {
    Check(vg_shape_safety_to_in(g_, id_, p.x(), p.y(), p.z(), p.size(), output, l_.flags, l_.stream),
          "vg_shape_safety_to_in");
  }
  void SafetyToOut(SOA3D<Precision> const &p, Precision *const output) const
  {
    Check(vg_shape_safety_to_out(g_, id_, p.x(), p.y(), p.z(), p.size(), output, l_.flags, l_.stream),
          "vg_shape_safety_to_out");
  }
  int32_t id() const { return id_; }

private:
  const vg_geom *g_;
  int32_t id_;
  Launch l_;
};

// VPlacedVolume's SoA queries on a placed volume by id (vg_placed_* entry points): Inside,
// Contains, DistanceToIn and SafetyToIn take mother-frame points, DistanceToOut and
// SafetyToOut local points, as the reference's do.
class PlacedVolume {
public:
  PlacedVolume(const Geometry &g, int32_t pv, Launch l = {}) : g_(g.handle()), id_(pv), l_(l) {}
  void Contains(SOA3D<Precision> const &p, bool *const output) const
  {
    Check(vg_placed_contains(g_, id_, p.x(), p.y(), p.z(), p.size(), reinterpret_cast<uint8_t *>(output), l_.flags,
                             l_.stream),
          "vg_placed_contains");
  }
  void Inside(SOA3D<Precision> const &p, Inside_t *const output) const
  {
    Check(vg_placed_inside(g_, id_, p.x(), p.y(), p.z(), p.size(), reinterpret_cast<int32_t *>(output), l_.flags,
                           l_.stream),
          "vg_placed_inside");
  }
  void DistanceToIn(SOA3D<Precision> const &p, SOA3D<Precision> const &d, Precision const *const step_max,
                    Precision *const output) const
  {
    Check(vg_placed_distance_to_in(g_, id_, p.x(), p.y(), p.z(), d.x(), d.y(), d.z(), step_max, p.size(), output,
                                   l_.flags, l_.stream),
          "vg_placed_distance_to_in");
  }
  void DistanceToOut(SOA3D<Precision> const &p, SOA3D<Precision> const &d, Precision const *const step_max,
                     Precision *const output) const
  {
    Check(vg_placed_distance_to_out(g_, id_, p.x(), p.y(), p.z(), d.x(), d.y(), d.z(), step_max, p.size(), output,
                                    l_.flags, l_.stream),
          "vg_placed_distance_to_out");
  }
  void SafetyToIn(SOA3D<Precision> const &p, Precision *const output) const
  {
    Check(vg_placed_safety_to_in(g_, id_, p.x(), p.y(), p.z(), p.size(), output, l_.flags, l_.stream),
          "vg_placed_safety_to_in");
  }
  void SafetyToOut(SOA3D<Precision> const &p, Precision *const output) const
  {
    Check(vg_placed_safety_to_out(g_, id_, p.x(), p.y(), p.z(), p.size(), output, l_.flags, l_.stream),
          "vg_placed_safety_to_out");
  }
  int32_t id() const { return id_; }

private:
  const vg_geom *g_;
  int32_t id_;
  Launch l_;
};

// GlobalLocator::LocateGlobalPoint(world, p, state, true) for every point (vg_nav_locate_point).
struct GlobalLocator {
  static void LocateGlobalPoints(const Geometry &g, SOA3D<Precision> const &p, NavStatePool &out,
                                 cudaStream_t s = nullptr)
  {
    if (out.size() < p.size()) throw Error(VG_EINVAL, "LocateGlobalPoints: state pool smaller than the points");
    Check(vg_nav_locate_point(g.handle(), p.x(), p.y(), p.z(), p.size(), out.data(), s), "vg_nav_locate_point");
  }
};

// BVHNavigator<false>'s SoA step. Launch::flags may add the scheduling flags VG_NAV_SORT,
// VG_NAV_QUEUE and VG_NAV_LEARNED to VG_PREC_MIXED; their workspace is kept by the navigator
// (grown on demand), so one navigator serves one stream at a time.
class BVHNavigator {
public:
  explicit BVHNavigator(const Geometry &g, Launch l = {}) : g_(g.handle()), l_(l) {}
  // VNavigator::ComputeStepsAndPropagatedStates: step_limits may be null (no physics limit);
  // status (nullable, device, one int32 per track) receives VG_TRACK_* give-up codes.
  void ComputeStepsAndPropagatedStates(SOA3D<Precision> const &points, SOA3D<Precision> const &dirs,
                                       Precision const *step_limits, NavStatePool const &in_states,
                                       NavStatePool &out_states, Precision *out_steps,
                                       int32_t *status = nullptr)
  {
    const size_t n = Sized(points, dirs, in_states, out_states);
    if (l_.flags & (VG_NAV_SORT | VG_NAV_QUEUE | VG_NAV_LEARNED)) {
      ws_.Resize(vg_nav_step_workspace_bytes(n, l_.flags));
      Check(vg_nav_compute_step_and_next_volume_ws(g_, points.x(), points.y(), points.z(), dirs.x(), dirs.y(),
                                                   dirs.z(), step_limits, in_states.data(), out_states.data(),
                                                   out_steps, status, nullptr, n, l_.flags, ws_.data(), ws_.size(),
                                                   l_.stream),
            "vg_nav_compute_step_and_next_volume_ws");
      return;
    }
    Check(vg_nav_compute_step_and_next_volume(g_, points.x(), points.y(), points.z(), dirs.x(), dirs.y(), dirs.z(),
                                              step_limits, in_states.data(), out_states.data(), out_steps, status,
                                              n, l_.flags, l_.stream),
          "vg_nav_compute_step_and_next_volume");
  }
  // VNavigator::ComputeStepsAndSafetiesAndPropagatedStates (NavStatePool form). The safety of
  // every track is computed (BVHSafetyEstimator); `calc_safeties` is accepted for the
  // reference's signature and may be null.
  void ComputeStepsAndSafetiesAndPropagatedStates(SOA3D<Precision> const &points, SOA3D<Precision> const &dirs,
                                                  Precision const *step_limits, NavStatePool const &in_states,
                                                  NavStatePool &out_states, Precision *out_steps,
                                                  bool const *calc_safeties, Precision *out_safeties,
                                                  int32_t *status = nullptr)
  {
    (void)calc_safeties;
    const size_t n = Sized(points, dirs, in_states, out_states);
    Check(vg_nav_compute_step_and_safety(g_, points.x(), points.y(), points.z(), dirs.x(), dirs.y(), dirs.z(),
                                         step_limits, in_states.data(), out_states.data(), out_steps, out_safeties,
                                         status, n, l_.flags & VG_PREC_MIXED, l_.stream),
          "vg_nav_compute_step_and_safety");
  }

private:
  static size_t Sized(SOA3D<Precision> const &p, SOA3D<Precision> const &d, NavStatePool const &in,
                      NavStatePool const &out)
  {
    const size_t n = p.size();
    if (d.size() != n || in.size() < n || out.size() < n)
      throw Error(VG_EINVAL, "navigator: points, directions and state pools differ in size");
    return n;
  }
  const vg_geom *g_;
  Launch l_;
  DeviceArray<unsigned char> ws_;
};

} // namespace vecgeom_gb300
