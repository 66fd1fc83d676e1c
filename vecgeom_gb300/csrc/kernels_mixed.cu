// Mixed-precision navigation kernels (VG_PREC_MIXED): same inputs and outputs as the FP64
// kernels; FP32 is used only for conservative pruning (see nav_mixed.cuh). Compiled with
// --fmad=false like every translation unit; the FP32 code requests fused multiply-adds
// explicitly.
#include "launch.h"
#include "nav_mixed.cuh"

namespace vg {
namespace {

inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

__global__ void __launch_bounds__(256) k_step_mixed(const DevGeom g, const double *__restrict__ x,
                                                    const double *__restrict__ y, const double *__restrict__ z,
                                                    const double *__restrict__ dx, const double *__restrict__ dy,
                                                    const double *__restrict__ dz, const double *__restrict__ limit,
                                                    const NavState *__restrict__ in, NavState *__restrict__ out,
                                                    double *__restrict__ step, int32_t *__restrict__ status,
                                                    int32_t *__restrict__ nvisited, size_t n)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const size_t stride       = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const NavState s = in[i];
    NavState o;
    int st = 0, nv = 0;
    const double lim = limit ? __ldg(limit + i) : kInfLength;
    step[i] = mixed::compute_step_mixed(g, lbs, f64::V3{__ldg(x + i), __ldg(y + i), __ldg(z + i)},
                                        f64::V3{__ldg(dx + i), __ldg(dy + i), __ldg(dz + i)}, lim, s, o, st,
                                        nvisited ? &nv : nullptr);
    out[i] = o;
    if (status) status[i] = st;
    if (nvisited) nvisited[i] = nv;
  }
}

__global__ void __launch_bounds__(256) k_locate_mixed(const DevGeom g, const double *__restrict__ x,
                                                      const double *__restrict__ y, const double *__restrict__ z,
                                                      size_t n, NavState *__restrict__ out)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const size_t stride       = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    NavState s{0u, 0u, 0, {0, 0, 0}};
    int st = 0;
    mixed::locate_global_point_mixed(g, lbs, g.world_pv, f64::V3{__ldg(x + i), __ldg(y + i), __ldg(z + i)}, s.navInd,
                                     true, st);
    out[i] = s;
  }
}

} // namespace

cudaError_t launch_step_mixed(const DevGeom &g, const StepArgs &a, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  k_step_mixed<<<grid_for(a.n, 256), 256, 0, s>>>(g, a.x, a.y, a.z, a.dx, a.dy, a.dz, a.limit, a.in, a.out, a.step,
                                                  a.status, a.nvisited, a.n);
  return cudaGetLastError();
}

cudaError_t launch_locate_mixed(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                                NavState *out, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  k_locate_mixed<<<grid_for(n, 256), 256, 0, s>>>(g, x, y, z, n, out);
  return cudaGetLastError();
}

} // namespace vg
