// Device-side loop of the transport stream: the iterations (sort of the live tracks,
// proposals, one persistent step-and-move kernel, compaction of the survivors) run inside a
// CUDA graph whose while-node repeats them on the GPU until the stream ends, with no host
// round trip per iteration. The body holds two iterations (list 0 -> list 1, then list 1 ->
// list 0) so that every pointer in it is fixed; before each iteration a one-thread kernel
// reads the live count the previous one left, decides whether to go on (the host loop's
// rule: stop after max_steps iterations, when no track is alive, or when few enough are
// alive for the tail pass) and hands the count to the iteration's kernels through device
// memory. Every kernel of an iteration reads its track count there (StepArgs::n_dev,
// TransportArgs::n_dev), so an iteration after the decision to stop does nothing. The loop
// ends because the iteration count is checked against max_steps on every decision.
#include "launch.h"

namespace vg {
namespace {

__global__ void k_transport_decide(TransportCtl *__restrict__ ctl, const unsigned int *__restrict__ cnt, int c,
                                   int max_steps, unsigned int drain_below, cudaGraphConditionalHandle loop)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (ctl->stop) {
    ctl->n[c] = 0;
    cudaGraphSetConditional(loop, 0);
    return;
  }
  const unsigned int live = *cnt;
  if (ctl->it >= max_steps || live == 0u || live < drain_below) {
    ctl->stop = 1;
    ctl->n[c] = 0;
    ctl->live = live;
    ctl->cur  = c;
    cudaGraphSetConditional(loop, 0);
  } else {
    ctl->n[c] = live;
    ctl->it += 1;
  }
}

// One iteration from list c to list c ^ 1, with its count at ctl->n[c].
cudaError_t enqueue_iteration(const TransportLoop &L, int c, cudaStream_t s)
{
  const unsigned int *n_dev = &L.ctl->n[c];
  const uint32_t *order     = L.list[c];
  cudaError_t e             = cudaSuccess;
  if (L.sort_on) {
    const uint32_t *sorted = nullptr;
    e = launch_nav_sort(*L.g, L.sort, L.ta.x, L.ta.y, L.ta.z, L.ta.st, L.n, L.sort_ws, &sorted, s, L.list[c], false,
                        n_dev);
    if (e != cudaSuccess) return e;
    if (sorted) order = sorted;
  }
  if (L.slots) {
    StepArgs pa{L.ta.x, L.ta.y, L.ta.z, L.ta.dx, L.ta.dy, L.ta.dz, nullptr, L.ta.st, nullptr, nullptr,
                nullptr, nullptr, L.n};
    pa.order = L.list[c]; // live tracks in (near) track order, as the step's proposals
    pa.n_dev = n_dev;
    e = L.propose_tensor ? launch_mlp_propose_tc(*L.g, pa, L.wbf, L.slots, L.mlp_err, s)
                         : launch_mlp_propose(*L.g, pa, L.wbf, L.slots, s);
    if (e != cudaSuccess) return e;
  }
  e = cudaMemsetAsync(L.cnt[c ^ 1], 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  TransportArgs ta = L.ta;
  ta.list          = order;
  ta.n             = L.n;
  ta.next          = L.list[c ^ 1];
  ta.next_count    = L.cnt[c ^ 1];
  ta.proposal      = L.slots;
  ta.n_dev         = n_dev;
  return launch_transport_iter(*L.g, ta, L.mixed, L.counter, L.queue_blocks, s);
}

} // namespace

cudaError_t run_transport_loop(const TransportLoop &L, cudaStream_t s, TransportCtl *out)
{
  cudaGraph_t graph      = nullptr;
  cudaGraphExec_t exec   = nullptr;
  cudaStream_t cs        = nullptr;
  cudaGraphNode_t wnode  = nullptr;
  cudaGraphConditionalHandle loop{};
  cudaError_t e = cudaGraphCreate(&graph, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&loop, graph, 1u, cudaGraphCondAssignDefault);
  cudaGraphNodeParams cp{};
  cp.type               = cudaGraphNodeTypeConditional;
  cp.conditional.handle = loop;
  cp.conditional.type   = cudaGraphCondTypeWhile;
  cp.conditional.size   = 1;
  if (e == cudaSuccess) e = cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &cp);
  // the body is recorded from a private stream (the caller's may be the legacy default
  // stream, which cannot be captured); nothing runs on it
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(cs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaError_t ce = cudaSuccess;
    for (int c = 0; c < 2 && ce == cudaSuccess; ++c) {
      k_transport_decide<<<1, 32, 0, cs>>>(L.ctl, L.cnt[c], c, L.max_steps, L.drain_below, loop);
      ce = cudaGetLastError();
      if (ce == cudaSuccess) ce = enqueue_iteration(L, c, cs);
    }
    cudaGraph_t body = nullptr;
    e                = cudaStreamEndCapture(cs, &body);
    if (e == cudaSuccess) e = ce;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaMemsetAsync(L.ctl, 0, sizeof(TransportCtl), s);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, L.ctl, sizeof(TransportCtl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return e;
}

} // namespace vg
