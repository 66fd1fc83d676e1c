// Drives the C++ layer (include/vecgeom_gb300.hpp) the way a VecGeom caller would: loads a
// saved geometry, uploads SoA points and directions, runs the placed and unplaced SoA queries,
// the global locator and the BVH navigator (plain FP64, scheduled mixed precision, step +
// safety), and writes every output to a file that tests/test_cpp_adapter.py compares with the
// same calls made through the C-ABI from Python.
//
// usage: adapter_check <geometry file> <input file> <output file> <placed volume> <shape>
// input: uint64 n, then x, y, z, dx, dy, dz (n doubles each)
// output, in order: Inside (int32), Contains (uint8), DistanceToIn, DistanceToOut, SafetyToIn,
// SafetyToOut (doubles) of the placed volume, the same six of the shape, located states,
// FP64 out-states and steps, mixed sorted work-queue out-states and steps, step + safety
// out-states, steps and safeties.
#include "vecgeom_gb300.hpp"

#include <cstdio>
#include <cstdlib>
#include <vector>

namespace vg = vecgeom_gb300;

template <class T>
static void put(std::FILE *f, const std::vector<T> &v)
{
  if (std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) throw vg::Error(VG_EINVAL, "short write");
}

template <class T>
static std::vector<T> fetch(const T *dev, size_t n)
{
  std::vector<T> h(n);
  vg::CheckCuda(cudaMemcpy(h.data(), dev, n * sizeof(T), cudaMemcpyDeviceToHost), "fetch");
  return h;
}

int main(int argc, char **argv)
{
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s geom input output pv shape\n", argv[0]);
    return 2;
  }
  try {
    vg::Geometry geo = vg::Geometry::Load(argv[1]);
    std::FILE *in    = std::fopen(argv[2], "rb");
    if (!in) throw vg::Error(VG_EINVAL, "cannot open the input file");
    uint64_t n = 0;
    if (std::fread(&n, sizeof(n), 1, in) != 1) throw vg::Error(VG_EINVAL, "short input");
    std::vector<double> c[6];
    for (auto &v : c) {
      v.resize(n);
      if (std::fread(v.data(), sizeof(double), n, in) != n) throw vg::Error(VG_EINVAL, "short input");
    }
    std::fclose(in);
    const int32_t pv = std::atoi(argv[4]), shape = std::atoi(argv[5]);

    auto pts  = vg::SOA3D<double>::FromHost(c[0].data(), c[1].data(), c[2].data(), n);
    auto dirs = vg::SOA3D<double>::FromHost(c[3].data(), c[4].data(), c[5].data(), n);
    vg::DeviceArray<vg::Inside_t> ins(n);
    vg::DeviceArray<bool> con(n);
    vg::DeviceArray<double> d[4];
    for (auto &a : d) a.Resize(n);

    std::FILE *out = std::fopen(argv[3], "wb");
    if (!out) throw vg::Error(VG_EINVAL, "cannot open the output file");
    auto queries = [&](auto const &vol) {
      vol.Inside(pts, ins.data());
      vol.Contains(pts, con.data());
      vol.DistanceToIn(pts, dirs, nullptr, d[0].data());
      vol.DistanceToOut(pts, dirs, nullptr, d[1].data());
      vol.SafetyToIn(pts, d[2].data());
      vol.SafetyToOut(pts, d[3].data());
      put(out, fetch(ins.data(), n));
      put(out, fetch(reinterpret_cast<const uint8_t *>(con.data()), n));
      for (auto &a : d) put(out, fetch(a.data(), n));
    };
    queries(vg::PlacedVolume(geo, pv));
    queries(vg::UnplacedVolume(geo, shape));

    vg::NavStatePool located(n), next(n);
    vg::GlobalLocator::LocateGlobalPoints(geo, pts, located);
    put(out, located.ToHost());
    vg::DeviceArray<double> steps(n), safeties(n);
    vg::BVHNavigator plain(geo);
    plain.ComputeStepsAndPropagatedStates(pts, dirs, nullptr, located, next, steps.data());
    put(out, next.ToHost());
    put(out, fetch(steps.data(), n));
    vg::BVHNavigator scheduled(geo, vg::Launch{VG_PREC_MIXED | VG_NAV_SORT | VG_NAV_QUEUE, nullptr});
    scheduled.ComputeStepsAndPropagatedStates(pts, dirs, nullptr, located, next, steps.data());
    put(out, next.ToHost());
    put(out, fetch(steps.data(), n));
    plain.ComputeStepsAndSafetiesAndPropagatedStates(pts, dirs, nullptr, located, next, steps.data(), nullptr,
                                                     safeties.data());
    put(out, next.ToHost());
    put(out, fetch(steps.data(), n));
    put(out, fetch(safeties.data(), n));
    std::fclose(out);
  } catch (const vg::Error &e) {
    std::fprintf(stderr, "adapter_check: %s (code %d)\n", e.what(), e.code());
    return 1;
  }
  return 0;
}
