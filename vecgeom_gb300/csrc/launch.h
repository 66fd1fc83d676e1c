// Kernel launchers shared between the C-ABI (capi.cpp) and the CUDA translation units.
#pragma once
#include "vg_types.h"
#include <cstddef>
#include <cuda_runtime.h>

namespace vg {

struct QueryArgs {
  const double *x, *y, *z, *dx, *dy, *dz;
  size_t n;
  void *out;
};

struct StepArgs {
  const double *x, *y, *z, *dx, *dy, *dz, *limit;
  const NavState *in;
  NavState *out;
  double *step;
  int32_t *status;
  int32_t *nvisited;
  size_t n;
  const uint32_t *order = nullptr; // optional visiting order (track indices); null: 0..n-1
  const int8_t *proposal = nullptr; // optional learned first subtree per track (-1: none)
  const unsigned int *n_dev = nullptr; // optional device count: only the first min(n, *n_dev) entries
  double *reloc = nullptr; // split step (work-queue configurations 5-8): 3 n doubles, the
                           // relocation point of the i-th visited track at i, n + i, 2n + i
  cudaEvent_t steps_done = nullptr; // optional: recorded once step[] is final (the work-queue
                                    // launcher records it before a split step's relocation)
};

// Sort key of a track: logical volume of its state above 3*cell_bits Morton bits of its
// position cell in the world box.
struct SortKeyParams {
  float lo[3];    // world box low corner (mm)
  float scale[3]; // cells per mm along each axis
  int cell_bits;  // bits per axis (<= 10)
  int lv_bits;    // bits of the logical-volume id
};

// Shape queries; `lbd` (8 floats, the shape's FP32 descriptor) / `mixed` select the
// mixed-precision variant (VG_PREC_MIXED).
cudaError_t launch_shape_query_fp64(int type, const double *rec, const Xform &xf, int apply_xf, int q,
                                    const QueryArgs &a, cudaStream_t s, const float *lbd = nullptr);
// `type`: the shape's type tag (host copy), which selects Polycone DistanceToOut's refill kernel.
cudaError_t launch_shape_query_dyn_fp64(const DevGeom &g, int shape, int type, const Xform &xf, int apply_xf, int q,
                                        const QueryArgs &a, cudaStream_t s, bool mixed = false);
cudaError_t launch_locate_fp64(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                               NavState *out, cudaStream_t s);
cudaError_t launch_step_fp64(const DevGeom &g, const StepArgs &a, cudaStream_t s);
// BVH::ApproachNextDaughter per track in its state's volume; step in/out, status nullable
cudaError_t launch_approach_fp64(const DevGeom &g, const double *x, const double *y, const double *z,
                                 const double *dx, const double *dy, const double *dz, const NavState *in,
                                 double *step, int32_t *status, size_t n, cudaStream_t s);
cudaError_t launch_step_mixed(const DevGeom &g, const StepArgs &a, cudaStream_t s);
cudaError_t launch_step_mixed_queue(const DevGeom &g, const StepArgs &a, unsigned long long *counter,
                                    int blocks_per_sm, cudaStream_t s);
cudaError_t launch_locate_mixed(const DevGeom &g, const double *x, const double *y, const double *z, size_t n,
                                NavState *out, cudaStream_t s);
size_t nav_sort_workspace_bytes(size_t n);
int sort_key_bits(const SortKeyParams &p);
const uint32_t *nav_sort_keys_of(const uint32_t *order, const void *ws, size_t n); // keys paired with `order`
// Keys + stable radix sort of the n tracks (or of the n track ids in `list`); *order
// receives the sorted track indices (inside the workspace). keys_done: the keys of all n
// tracks were already written by launch_nav_sort_keys (ranges of tracks, e.g. as their
// inputs arrive), only the radix passes run. n_dev (optional, device memory): sort only the
// first min(n, *n_dev) entries; n then only sizes the grids (a count the host does not know).
cudaError_t launch_nav_sort(const DevGeom &g, const SortKeyParams &p, const double *x, const double *y,
                            const double *z, const NavState *in, size_t n, void *ws, const uint32_t **order,
                            cudaStream_t s, const uint32_t *list = nullptr, bool keys_done = false,
                            const unsigned int *n_dev = nullptr);
cudaError_t launch_nav_sort_keys(const DevGeom &g, const SortKeyParams &p, const double *x, const double *y,
                                 const double *z, const NavState *in, size_t begin, size_t end, void *ws,
                                 cudaStream_t s);

// One iteration of the transport stream over the n track ids in `list` (visiting order):
// step each track, move it (p += step d), store its new state in place, count the step,
// record the trace of tracks < trace_n, and append the tracks still alive to `next`.
struct TransportArgs {
  double *x, *y, *z;
  const double *dx, *dy, *dz;
  NavState *st;
  int32_t *nsteps;
  int32_t *status;
  int max_steps;
  NavState *trace_st;
  double *trace_step;
  size_t trace_n;
  const uint32_t *list;
  size_t n;
  uint32_t *next;
  unsigned int *next_count;
  const int8_t *proposal;
  const unsigned int *n_dev = nullptr; // optional device count: only the first min(n, *n_dev) entries
};
cudaError_t launch_transport_iter(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                  int blocks_per_sm, cudaStream_t s);
// Device-side loop of the transport stream (transport_loop.cu): control block in device
// memory; n[c] is the count the iteration from list c runs on (0 once stopped), `it` the
// iterations made, `live` and `cur` the survivors and their list when the loop stopped.
struct TransportCtl {
  unsigned int n[2];
  int it;
  int stop;
  unsigned int live;
  int cur;
  int pad[2];
};
// What the loop needs; the lists, counts, counter, slots and sort workspace are device
// memory of n entries each (slots, sort_ws: null when VG_NAV_LEARNED / VG_NAV_SORT are off).
struct TransportLoop {
  const DevGeom *g;
  TransportArgs ta; // the track arrays, max_steps and traces; list/n/next fields are set per iteration
  size_t n;
  uint32_t *list[2];
  unsigned int *cnt[2];
  unsigned long long *counter;
  TransportCtl *ctl;
  bool mixed;
  int queue_blocks;
  bool sort_on;
  SortKeyParams sort;
  void *sort_ws;
  int8_t *slots;
  int propose_tensor;
  const uint16_t *wbf;
  int *mlp_err;
  int max_steps;
  unsigned int drain_below;
};
// Runs the iterations until the loop's rule stops them, synchronises `s` and copies the
// control block to *out.
cudaError_t run_transport_loop(const TransportLoop &loop, cudaStream_t s, TransportCtl *out);
cudaError_t launch_mlp_propose_tc(const DevGeom &g, const StepArgs &a, const uint16_t *wbf, int8_t *slot, int *err,
                                  cudaStream_t s);
// Transport tail: steps every track of `list` to its end in one launch (refill per lane).
cudaError_t launch_transport_drain(const DevGeom &g, const TransportArgs &a, bool mixed, unsigned long long *counter,
                                   cudaStream_t s);
cudaError_t launch_transport_init(const NavState *st, size_t n, int32_t *nsteps, int32_t *status, uint32_t *list,
                                  unsigned int *count, cudaStream_t s);
// Builds of the navigation kernels per shape set: set_all dispatches every shape type,
// set_core only kCoreShapeMask (smaller step kernels). The launchers above pick the build
// for the geometry's shape set.
inline bool core_shapes_only(const DevGeom &g) { return (g.type_mask & ~kCoreShapeMask) == 0u; }
#define VG_NAV_SET_DECLS                                                                                           \
  cudaError_t launch_step_fp64(const DevGeom &g, const StepArgs &a, cudaStream_t s);                               \
  cudaError_t launch_step_mixed_queue(const DevGeom &g, const StepArgs &a, unsigned long long *counter,             \
                                      int blocks_per_sm, cudaStream_t s);                                          \
  cudaError_t launch_transport_iter(const DevGeom &g, const TransportArgs &a, bool mixed,                          \
                                    unsigned long long *counter, int blocks_per_sm, cudaStream_t s);               \
  cudaError_t launch_transport_drain(const DevGeom &g, const TransportArgs &a, bool mixed,                         \
                                     unsigned long long *counter, cudaStream_t s);
namespace set_all {
VG_NAV_SET_DECLS
}
namespace set_core {
VG_NAV_SET_DECLS
}
#undef VG_NAV_SET_DECLS
// Fixed scratch of the no-allocation step entry point (noalloc.cu).
size_t noalloc_max_tracks();
cudaError_t noalloc_scratch(void **ptr, size_t *bytes);
// Step + safety of the input state (ComputeStepAndSafetyAndPropagatedState).
cudaError_t launch_step_safety(const DevGeom &g, const StepArgs &a, double *safety, bool mixed, cudaStream_t s);
// Learned proposal per track (features + BF16 MLP, SIMT) into `slot` (n bytes).
cudaError_t launch_mlp_propose(const DevGeom &g, const StepArgs &a, const uint16_t *wbf, int8_t *slot, cudaStream_t s);
// flags: VG_PREC_FP64 (0) or VG_PREC_MIXED (1)
inline cudaError_t launch_step(const DevGeom &g, const StepArgs &a, uint32_t flags, cudaStream_t s)
{
  return (flags & 1u) ? launch_step_mixed(g, a, s) : launch_step_fp64(g, a, s);
}

} // namespace vg
