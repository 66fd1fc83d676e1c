// Device side of the learned proposal shared by the feature, inference and step kernels:
// the input features of one track (layout in learn.h) and its training label.
#pragma once
#include "learn.h"
#include "nav_fp64.cuh"

namespace vg {
namespace learn {

using f64::V3;

// Depth-3 node `7 + s` is reachable when its three ancestors are internal nodes.
__device__ __forceinline__ bool slot_reachable(const DevGeom &g, int node0, int s)
{
  int n = 7 + s;
  for (int d = 0; d < 3; ++d) {
    n = (n - 1) >> 1;
    if (__ldg(&g.node_nchild[node0 + n]) >= 0) return false;
  }
  return true;
}

__device__ __forceinline__ float safe_inv(float d) { return d != 0.f ? 1.f / d : copysignf(INFINITY, d); }

// Features of a track in state `navInd` at global point/direction (gp, gd). Returns false
// (and lv = -1) when no proposal applies. lp/ld receive the FP64 local point/direction
// (for the training label); the features themselves use an FP32 transform (p - t formed in
// FP64, the rotation in FP32), the same in training and inference, so that inference,
// which discards lp/ld, issues almost no FP64 work.
__device__ __forceinline__ bool features(const DevGeom &g, uint32_t navInd, V3 gp, V3 gd, float *f, int &lv, V3 &lp,
                                         V3 &ld)
{
  lv = -1;
  if (navInd == 0) return false;
  const Xform m = f64::nav_top_matrix(g, navInd);
  lp            = f64::to_local(m, gp);
  ld            = f64::rotate(m, gd);
  float rf[9];
  for (int k = 0; k < 9; ++k) rf[k] = (float)m.r[k];
  const float q[3]  = {(float)(gp.x - m.t[0]), (float)(gp.y - m.t[1]), (float)(gp.z - m.t[2])};
  const float gf[3] = {(float)gd.x, (float)gd.y, (float)gd.z};
  const int l   = g.pv_lv[f64::nav_top(g, navInd)];
  if (g.lv_depth[l] < 3) return false;
  lv              = l;
  const int node0 = g.bvh_node0[g.lv_bvh[l]];
  const NodeF root = g.node_f[node0];
  float c[3], h[3], hs = 0.f;
  for (int k = 0; k < 3; ++k) {
    c[k] = 0.5f * (root.lo[k] + root.hi[k]);
    h[k] = fmaxf(0.5f * (root.hi[k] - root.lo[k]), 1e-3f);
    hs   = fmaxf(hs, h[k]);
  }
  float p[3], d[3];
  for (int k = 0; k < 3; ++k) {
    p[k] = fmaf(q[0], rf[k], fmaf(q[1], rf[3 + k], q[2] * rf[6 + k]));
    d[k] = fmaf(gf[0], rf[k], fmaf(gf[1], rf[3 + k], gf[2] * rf[6 + k]));
  }
  const float inv[3] = {safe_inv(d[0]), safe_inv(d[1]), safe_inv(d[2])};
  for (int k = 0; k < 3; ++k) {
    f[k]     = (p[k] - c[k]) / h[k];
    f[3 + k] = d[k];
  }
  for (int k = 0; k < kMlpEmb; ++k) f[kMlpEmbOff + k] = 0.f;
  for (int s = 0; s < 8; ++s) {
    float *b = f + 22 + 6 * s;
    if (!slot_reachable(g, node0, s)) {
      for (int k = 0; k < 6; ++k) b[k] = 0.f;
      f[70 + s] = 4.f;
      continue;
    }
    const NodeF nd = g.node_f[node0 + 7 + s];
    float tmin = -INFINITY, tmax = INFINITY;
    for (int k = 0; k < 3; ++k) {
      b[k]     = (nd.lo[k] - p[k]) / h[k];
      b[3 + k] = (nd.hi[k] - p[k]) / h[k];
      float t0 = (nd.lo[k] - p[k]) * inv[k], t1 = (nd.hi[k] - p[k]) * inv[k];
      if (t0 > t1) {
        const float t = t0;
        t0            = t1;
        t1            = t;
      }
      if (!(t0 != t0)) tmin = fmaxf(tmin, t0);
      if (!(t1 != t1)) tmax = fminf(tmax, t1);
    }
    const bool hit = tmin <= tmax && tmax >= 0.f;
    f[70 + s]      = hit ? fminf(fmaxf(tmin / hs, -4.f), 4.f) : 4.f;
  }
  f[78] = f[79] = 0.f;
  return true;
}

// Training label from the plain FP64 traversal: 0..7 depth-3 subtree of the first daughter
// hit, 8 when no daughter is hit, -1 when the hit daughter's leaf lies above depth 3 or
// the traversal gave up.
__device__ __forceinline__ int label_fp64(const DevGeom &g, NavState const &s, int lv, V3 lp, V3 ld)
{
  double step = f64::shape_dist_out(g, g.lv_shape[lv], lp, ld);
  if (step < 0.) step = 0.;
  int hit        = -1;
  const int last = f64::nav_top(g, s.lastExited);
  if (f64::bvh_check_daughters(g, lv, lp, ld, step, last, hit, nullptr) != kTrackOk) return -1;
  if (hit < 0) return 8;
  return g.dau_slot3[g.lv_dstart[lv] + g.pv_child[hit]];
}

} // namespace learn
} // namespace vg
