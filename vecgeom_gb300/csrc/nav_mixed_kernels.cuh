// Mixed-precision navigation kernels (VG_PREC_MIXED) and the templates that launch them,
// compiled once per shape set: every translation unit that includes this header defines
// VG_NAV_SET (the namespace of its launchers) and may define VG_SHAPE_MASK (the shape types
// its dispatch holds, dispatch_fp64.cuh) first. Same inputs and outputs as the FP64
// kernels; FP32 is used only for conservative pruning (see nav_mixed.cuh). Compiled with
// --fmad=false like every translation unit; the FP32 code requests fused multiply-adds
// explicitly.
#pragma once
#ifndef VG_NAV_SET
#error "define VG_NAV_SET before including nav_mixed_kernels.cuh"
#endif
#define VG_FP64_INT_COMPARE 0 // latency-bound navigation code (fp64_int.cuh)
#include "launch.h"
#include "nav_mixed.cuh"

namespace vg {
namespace VG_NAV_SET {
namespace {

inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

__device__ __forceinline__ void step_one_mixed(const DevGeom &g, const mixed::ShapeLB *lbs, const StepArgs &a,
                                               size_t t)
{
  const NavState s = a.in[t];
  NavState o;
  int st = 0, nv = 0;
  const double lim = a.limit ? __ldg(a.limit + t) : kInfLength;
  a.step[t] = mixed::compute_step_mixed(g, lbs, f64::V3{__ldg(a.x + t), __ldg(a.y + t), __ldg(a.z + t)},
                                        f64::V3{__ldg(a.dx + t), __ldg(a.dy + t), __ldg(a.dz + t)}, lim, s, o, st,
                                        a.nvisited ? &nv : nullptr, a.proposal ? (int)__ldg(a.proposal + t) : -1);
  a.out[t] = o;
  if (a.status) a.status[t] = st;
  if (a.nvisited) a.nvisited[t] = nv;
}

#ifdef VG_NAV_UNSCHEDULED_KERNELS // unsorted step and locate: compiled in one unit only
__global__ void __launch_bounds__(256) k_step_mixed(const DevGeom g, const StepArgs a)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const size_t stride       = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride)
    step_one_mixed(g, lbs, a, a.order ? (size_t)__ldg(a.order + i) : i);
}
#endif

// Persistent variant: one grid of resident blocks; each warp takes the next 32 entries of
// the visiting order from a global counter (zeroed before the launch), so warps that drew
// cheap tracks take more of them. Threads x MinBlocks sets the register budget per thread:
// 256 x 1 (no spills, 8 warps per SM), 256 x 2 (128 registers, 16 warps), 128 x 3 (168
// registers, 12 warps) or 128 x 5 (102 registers, 20 warps).
template <int Threads, int MinBlocks>
__global__ void __launch_bounds__(Threads, MinBlocks) k_step_mixed_queue(const DevGeom g, const StepArgs a,
                                                                         unsigned long long *__restrict__ counter)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const int lane            = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.n) break;
    const size_t i = (size_t)base + lane;
    if (i < a.n) step_one_mixed(g, lbs, a, a.order ? (size_t)__ldg(a.order + i) : i);
  }
}

// Split step (queue configurations 5-8): the first kernel computes each step up to its
// relocation, leaves the relocation code in the out-state's first pad byte and the
// relocation point (FP64) in a.reloc at the track's visiting position; the second kernel
// relocates those tracks over the same visiting order, reading that point back with
// coalesced loads, and clears the byte. Each kernel's body is about half of the fused one
// (fewer instruction-cache misses, its own register budget). Results are those of the fused
// kernel: the same operations on the same values.
__device__ __forceinline__ void step_one_mixed_split(const DevGeom &g, const StepArgs &a, size_t t, size_t i)
{
  const NavState s = a.in[t];
  NavState o       = s;
  int st = kTrackOk, nv = 0, reloc = mixed::kRelocNone;
  double step = 0.;
  if (s.navInd == 0) {
    st = kTrackErrState;
  } else {
    const double lim = a.limit ? __ldg(a.limit + t) : kInfLength;
    const Xform m    = f64::nav_top_matrix(g, s.navInd);
    const f64::V3 lp = f64::to_local(m, f64::V3{__ldg(a.x + t), __ldg(a.y + t), __ldg(a.z + t)});
    const f64::V3 ld = f64::rotate(m, f64::V3{__ldg(a.dx + t), __ldg(a.dy + t), __ldg(a.dz + t)});
    step = mixed::step_before_relocation_mixed(g, lp, ld, lim, s, o, st, a.nvisited ? &nv : nullptr,
                                               a.proposal ? (int)__ldg(a.proposal + t) : -1, reloc);
    if (reloc != mixed::kRelocNone) {
      const f64::V3 q = mixed::relocation_point(lp, ld, step);
      a.reloc[i]           = q.x;
      a.reloc[a.n + i]     = q.y;
      a.reloc[2 * a.n + i] = q.z;
    }
  }
  o.pad[0]  = (uint8_t)reloc;
  a.step[t] = step;
  a.out[t]  = o;
  if (a.status) a.status[t] = st;
  if (a.nvisited) a.nvisited[t] = nv;
}

__device__ __forceinline__ void relocate_one_mixed(const DevGeom &g, const mixed::ShapeLB *lbs, const StepArgs &a,
                                                   size_t t, size_t i)
{
  NavState o = a.out[t];
  if (o.pad[0] == mixed::kRelocNone) return;
  const int reloc = o.pad[0];
  o.pad[0]        = 0;
  const f64::V3 q{a.reloc[i], a.reloc[a.n + i], a.reloc[2 * a.n + i]};
  int st = kTrackOk;
  mixed::relocate_from_point_mixed(g, lbs, q, reloc, o, st);
  a.out[t] = o;
  if (a.status) a.status[t] = st;
}

// The relocation kernel (72 registers unbounded) waits on memory: it gets a 64-register
// budget, for 32 resident warps per SM.
template <int Threads, int MinBlocks, bool Relocate>
__global__ void __launch_bounds__(Threads, Relocate ? 1024 / Threads : MinBlocks)
    k_step_mixed_split(const DevGeom g, const StepArgs a, unsigned long long *__restrict__ counter)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const int lane            = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= a.n) break;
    const size_t i = (size_t)base + lane;
    if (i >= a.n) continue;
    const size_t t = a.order ? (size_t)__ldg(a.order + i) : i;
    if (Relocate)
      relocate_one_mixed(g, lbs, a, t, i);
    else
      step_one_mixed_split(g, a, t, i);
  }
}

#ifdef VG_NAV_UNSCHEDULED_KERNELS
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
#endif

// ComputeStepAndSafetyAndPropagatedState: the safety of the input state (FP64), then the step
// (FP64 or mixed). A give-up in either part sets the track's status.
template <bool Mixed>
__global__ void __launch_bounds__(256) k_step_safety(const DevGeom g, const StepArgs a, double *__restrict__ safety)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const size_t stride       = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const NavState s = a.in[i];
    const f64::V3 p{__ldg(a.x + i), __ldg(a.y + i), __ldg(a.z + i)}, d{__ldg(a.dx + i), __ldg(a.dy + i),
                                                                       __ldg(a.dz + i)};
    int st_saf = kTrackOk, st = kTrackOk;
    safety[i] = f64::safety_of_state(g, p, s.navInd, st_saf);
    NavState o;
    const double lim = a.limit ? __ldg(a.limit + i) : kInfLength;
    a.step[i] = Mixed ? mixed::compute_step_mixed(g, lbs, p, d, lim, s, o, st, nullptr)
                      : f64::compute_step(g, p, d, lim, s, o, st, nullptr);
    a.out[i] = o;
    if (a.status) a.status[i] = st != kTrackOk ? st : st_saf;
  }
}

// Transport stream iteration (see TransportArgs): persistent warps take 32-entry chunks of
// the visiting order from a global counter.
template <bool Mixed, int Threads, int MinBlocks>
__global__ void __launch_bounds__(Threads, MinBlocks) k_transport_iter(const DevGeom g, const TransportArgs a,
                                                                       unsigned long long *__restrict__ counter)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  const int lane            = threadIdx.x & 31;
  const size_t n            = a.n_dev && *a.n_dev < a.n ? (size_t)*a.n_dev : a.n;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const size_t i = (size_t)base + lane;
    if (i >= n) continue;
    const size_t t = __ldg(a.list + i);
    const NavState s = a.st[t];
    NavState o;
    int st = 0;
    const f64::V3 p{a.x[t], a.y[t], a.z[t]}, d{__ldg(a.dx + t), __ldg(a.dy + t), __ldg(a.dz + t)};
    const double step =
        Mixed ? mixed::compute_step_mixed(g, lbs, p, d, kInfLength, s, o, st, nullptr,
                                          a.proposal ? (int)__ldg(a.proposal + t) : -1)
              : f64::compute_step(g, p, d, kInfLength, s, o, st, nullptr);
    const int k = a.nsteps[t];
    if (t < a.trace_n) {
      a.trace_st[t * (size_t)a.max_steps + k]   = o;
      a.trace_step[t * (size_t)a.max_steps + k] = step;
    }
    a.x[t]      = p.x + step * d.x; // OracleTransport: p = p + step * d
    a.y[t]      = p.y + step * d.y;
    a.z[t]      = p.z + step * d.z;
    a.st[t]     = o;
    a.nsteps[t] = k + 1;
    if (st != kTrackOk) {
      a.status[t] = st; // a track that gave up leaves the stream with its status
      continue;
    }
    if (o.navInd != 0 && k + 1 < a.max_steps) a.next[atomicAdd(a.next_count, 1u)] = (uint32_t)t;
  }
}

// Transport stream tail: each thread takes the next live track from a global counter and
// steps it until it leaves the world, gives up or reaches max_steps, then takes another
// (refill per lane). Each step is the iteration kernel's step on the same state, so the
// results are those of running the remaining iterations one by one; what it saves is the
// per-iteration sort, proposal and host round trip once too few tracks are left to fill
// the GPU. No proposals (they only reorder the traversal).
template <bool Mixed>
__global__ void __launch_bounds__(256, 2) k_transport_drain(const DevGeom g, const TransportArgs a,
                                                            unsigned long long *__restrict__ counter)
{
  const mixed::ShapeLB *lbs = reinterpret_cast<const mixed::ShapeLB *>(g.shape_lbd);
  for (;;) {
    const unsigned long long i = atomicAdd(counter, 1ull);
    if (i >= a.n) break;
    const size_t t = __ldg(a.list + i);
    NavState s     = a.st[t];
    f64::V3 p{a.x[t], a.y[t], a.z[t]};
    const f64::V3 d{__ldg(a.dx + t), __ldg(a.dy + t), __ldg(a.dz + t)};
    int k = a.nsteps[t];
    for (;;) {
      NavState o;
      int st = 0;
      const double step = Mixed ? mixed::compute_step_mixed(g, lbs, p, d, kInfLength, s, o, st, nullptr, -1)
                                : f64::compute_step(g, p, d, kInfLength, s, o, st, nullptr);
      if (t < a.trace_n) {
        a.trace_st[t * (size_t)a.max_steps + k]   = o;
        a.trace_step[t * (size_t)a.max_steps + k] = step;
      }
      p = f64::V3{p.x + step * d.x, p.y + step * d.y, p.z + step * d.z}; // OracleTransport: p += step d
      s = o;
      ++k;
      if (st != kTrackOk) {
        a.status[t] = st;
        break;
      }
      if (o.navInd == 0 || k >= a.max_steps) break;
    }
    a.x[t]      = p.x;
    a.y[t]      = p.y;
    a.z[t]      = p.z;
    a.st[t]     = s;
    a.nsteps[t] = k;
  }
}

#ifdef VG_NAV_UNSCHEDULED_KERNELS
__global__ void k_transport_init(const NavState *__restrict__ st, size_t n, int32_t *__restrict__ nsteps,
                                 int32_t *__restrict__ status, uint32_t *__restrict__ list,
                                 unsigned int *__restrict__ count)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    nsteps[t] = 0;
    status[t] = 0;
    if (st[t].navInd != 0) list[atomicAdd(count, 1u)] = (uint32_t)t;
  }
}
#endif

template <bool Mixed, int Threads, int MinBlocks>
cudaError_t launch_transport(const DevGeom &g, const TransportArgs &a, unsigned long long *counter, cudaStream_t s)
{
  static int resident = 0;
  if (resident == 0) {
    int r = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_transport_iter<Mixed, Threads, MinBlocks>, Threads, 0);
    if (e != cudaSuccess) return e;
    resident = r > 0 ? r : 1;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  size_t blocks = (size_t)sms * resident, need = (a.n + Threads - 1) / Threads;
  if (blocks > need) blocks = need;
  k_transport_iter<Mixed, Threads, MinBlocks><<<(unsigned)blocks, Threads, 0, s>>>(g, a, counter);
  return cudaGetLastError();
}


template <int Threads, int MinBlocks>
cudaError_t launch_queue(const DevGeom &g, const StepArgs &a, unsigned long long *counter, cudaStream_t s)
{
  static int resident = 0; // blocks per SM (the same on every device the library targets)
  if (resident == 0) {
    int r = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_step_mixed_queue<Threads, MinBlocks>, Threads, 0);
    if (e != cudaSuccess) return e;
    resident = r > 0 ? r : 1;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  size_t blocks = (size_t)sms * resident, need = (a.n + Threads - 1) / Threads;
  if (blocks > need) blocks = need;
  k_step_mixed_queue<Threads, MinBlocks><<<(unsigned)blocks, Threads, 0, s>>>(g, a, counter);
  return cudaGetLastError();
}


template <int Threads, int MinBlocks, bool Relocate>
cudaError_t launch_split(const DevGeom &g, const StepArgs &a, unsigned long long *counter, cudaStream_t s)
{
  static int resident = 0;
  if (resident == 0) {
    int r = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &r, k_step_mixed_split<Threads, MinBlocks, Relocate>, Threads, 0);
    if (e != cudaSuccess) return e;
    resident = r > 0 ? r : 1;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  size_t blocks = (size_t)sms * resident, need = (a.n + Threads - 1) / Threads;
  if (blocks > need) blocks = need;
  k_step_mixed_split<Threads, MinBlocks, Relocate><<<(unsigned)blocks, Threads, 0, s>>>(g, a, counter);
  return cudaGetLastError();
}

template <int Threads, int MinBlocks>
cudaError_t launch_queue_split(const DevGeom &g, const StepArgs &a, unsigned long long *counter, cudaStream_t s)
{
  cudaError_t e = launch_split<Threads, MinBlocks, false>(g, a, counter, s);
  if (e == cudaSuccess && a.steps_done) e = cudaEventRecord(a.steps_done, s); // step[] is final
  if (e == cudaSuccess) e = launch_split<Threads, MinBlocks, true>(g, a, counter, s);
  return e;
}

} // namespace
} // namespace VG_NAV_SET
} // namespace vg
