// Learned first-hit proposal for the BVH traversal: a small MLP that, for a track in a
// logical volume whose BVH has depth >= 3, predicts which of the 8 depth-3 subtrees
// (breadth-first nodes 7..14) holds the first daughter the ray hits, or "none" (class 8).
// The mixed-precision step explores the proposed subtree first, so the exact FP64
// traversal starts from a tight step bound; the full traversal still runs, so the result
// does not depend on the proposal.
//
// Network: 80 inputs -> 64 (ReLU) -> 64 (ReLU) -> 16 logits (9 used). Inputs (FP32):
//   [0,3)   local point, (p - c) / h with c, h the centre and half-size of the BVH root box
//   [3,6)   local direction
//   [6,22)  embedding of the logical volume (16, learned)
//   [22,70) bounds of the 8 depth-3 nodes relative to the point, (lo - p) / h, (hi - p) / h
//   [70,78) FP32 slab entry distance of each depth-3 node / max(h), clamped to [-4, 4]
//           (4 when the ray misses the node)
//   [78,80) zero
// Parameters live in one flat FP32 vector (layout below); inference uses a BF16 copy of
// the weights with FP32 accumulation.
#pragma once
#include "launch.h"
#include <cstddef>
#include <cstdint>

namespace vg {

constexpr int kMlpIn = 80, kMlpHid = 64, kMlpOut = 16, kMlpCls = 9, kMlpEmb = 16, kMlpEmbOff = 6;
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpHid * kMlpIn;
constexpr int kMlpW2 = kMlpB1 + kMlpHid;
constexpr int kMlpB2 = kMlpW2 + kMlpHid * kMlpHid;
constexpr int kMlpW3 = kMlpB2 + kMlpHid;
constexpr int kMlpB3 = kMlpW3 + kMlpOut * kMlpHid;
constexpr int kMlpE  = kMlpB3 + kMlpOut; // embedding table [n_lv][16]
inline size_t mlp_param_count(int n_lv) { return (size_t)kMlpE + (size_t)n_lv * kMlpEmb; }

// Features (and optionally labels) for n tracks. lv[i] = -1 where no proposal applies
// (state outside the world or BVH shallower than 3); label[i] = 0..7 subtree, 8 none,
// -1 not applicable. Labels come from the plain FP64 traversal.
cudaError_t launch_learn_features(const DevGeom &g, const StepArgs &a, float *feat, int32_t *lv, int8_t *label,
                                  cudaStream_t s);

// One forward + backward pass over a batch given by `idx` (nb samples of the feature
// set): gradients (flat, same layout as the parameters, overwritten) and the summed loss.
// ws: scratch of mlp_train_ws_floats(nb) floats.
size_t mlp_train_ws_floats(int nb);
cudaError_t launch_mlp_grad(const float *params, int n_lv, const float *feat, const int32_t *lv, const int8_t *label,
                            const uint32_t *idx, int nb, float *grads, float *loss, float *ws, cudaStream_t s);
cudaError_t launch_mlp_adam(float *params, const float *grads, float *m, float *v, size_t n, float lr, float b1,
                            float b2, float eps, int t, cudaStream_t s);
// BF16 copy of the parameters for inference (same layout, rounded to nearest even).
cudaError_t launch_mlp_to_bf16(const float *params, uint16_t *wbf, size_t n, cudaStream_t s);
// Proposals for n tracks from precomputed features (SIMT, BF16 weights, FP32 sums):
// slot[i] = 0..7, or -1 for "none" and for tracks without a proposal.
cudaError_t launch_mlp_infer_feat(const uint16_t *wbf, int n_lv, const float *feat, const int32_t *lv, size_t n,
                                  int8_t *slot, float *logits, cudaStream_t s);

// Tensor-core (tcgen05) versions: same semantics, `err` (device int) is set to 1 if a
// bounded wait for an MMA gave up.
cudaError_t launch_mlp_propose_tc(const DevGeom &g, const StepArgs &a, const uint16_t *wbf, int8_t *slot, int *err,
                                  cudaStream_t s);
cudaError_t launch_mlp_infer_feat_tc(const uint16_t *wbf, const float *feat, const int32_t *lv, size_t n, int8_t *slot,
                                     float *logits, int *err, cudaStream_t s);

} // namespace vg
