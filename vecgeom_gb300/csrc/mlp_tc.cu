// Tensor-core inference of the learned proposal on sm_103a: one CTA of 128 threads handles
// tiles of 128 tracks. Each thread builds its track's feature row (BF16) in shared memory;
// one thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128) for the three
// layers with the accumulator in tensor memory; each warp reads its 32 rows back with
// tcgen05.ld, applies bias + ReLU, rounds to BF16 and writes the next layer's operand.
// Inference semantics equal the SIMT kernel's (learn.cu): BF16 inputs, weights, biases
// and hidden activations, FP32 sums.
//
// Shared-memory operands use the canonical K-major layout without swizzle: 8 x 16-byte
// core matrices, rows of a core matrix 16 bytes apart, core matrices 128 bytes apart
// along K (leading byte offset) and K/8 x 128 bytes apart along M/N (stride byte offset).
// Every wait on the MMA completion barrier is bounded; on time-out the kernel records an
// error, drains its outstanding MMA (bounded), frees its tensor memory and returns.
#define VG_FP64_INT_COMPARE 0 // latency-bound navigation code (fp64_int.cuh)
#include "learn_features.cuh"
#include <cuda_bf16.h>

namespace vg {
namespace {

constexpr int kTile    = 128;
constexpr int kTmemCols = 64;
constexpr uint32_t kWaitLimit = 1u << 20; // try_wait polls; each may suspend briefly

// shared-memory plan (bytes, 1024-aligned blocks)
constexpr int kOffW1   = 0;                        // 64 x 80 bf16
constexpr int kOffW2   = kOffW1 + 64 * 80 * 2;     // 64 x 64
constexpr int kOffW3   = kOffW2 + 64 * 64 * 2;     // 16 x 64
// One operand buffer serves the three layers: each layer's input is written only after the
// MMA that read the previous contents has completed (its barrier wait).
constexpr int kOffA    = 22528;                    // 128 x 80 (layer 1), then 128 x 64 (layers 2, 3)
constexpr int kOffBias = kOffA + kTile * 80 * 2;   // b1[64], b2[64], b3[16] as float
constexpr int kOffBar  = kOffBias + 144 * 4;       // mbarrier (8 B) + tmem address (4 B)
constexpr int kSmemBytes = kOffBar + 64;
static_assert(kOffW3 + 16 * 64 * 2 <= kOffA, "weights overlap the operand tiles");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) of a K-major BF16 operand with K columns
__device__ __forceinline__ int kmajor_off(int r, int k, int K)
{
  return (r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int K)
{
  const uint64_t lbo = 128, sbo = (uint64_t)(K >> 3) * 128;
  uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (lbo >> 4) << 16;
  d |= (sbo >> 4) << 32;
  d |= (uint64_t)1 << 46; // descriptor version of sm_100-family tensor cores
  return d;                // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: F32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
               "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity)
{
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's row (warp w reads lanes 32w..32w+31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t tobf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }

// 16-byte store of columns [8 kb, 8 kb + 8) of row r of a K-major operand with K columns:
// one row segment of a core matrix, so a quarter warp (8 rows of one row group) writes
// 128 contiguous bytes and the store is free of bank conflicts.
__device__ __forceinline__ void store_chunk(unsigned char *base, int r, int kb, int K, uint4 v)
{
  *reinterpret_cast<uint4 *>(base + (r >> 3) * (K >> 3) * 128 + kb * 128 + (r & 7) * 16) = v;
}
__device__ __forceinline__ float frombf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }

// Feature source: computed from step inputs (Step = true) or read from a feature array.
// At most 102 registers, so that five CTAs fit per SM (shared memory allows five; the
// feature gather is latency-bound and gains from the fifth: 0.70 ms instead of 0.74 ms per
// 2^22 tracks).
template <bool Step>
__global__ void __launch_bounds__(kTile, 5) k_mlp_propose_tc(const DevGeom g, const StepArgs a, const float *__restrict__ feat,
                                                          const int32_t *__restrict__ lvin, size_t n,
                                                          const uint16_t *__restrict__ wbf, int8_t *__restrict__ slot,
                                                          float *__restrict__ logits, int *__restrict__ err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  const int t = threadIdx.x, warp = t >> 5;
  uint64_t *bar    = reinterpret_cast<uint64_t *>(sm + kOffBar);
  uint32_t *tslot  = reinterpret_cast<uint32_t *>(sm + kOffBar + 8);
  float *bias      = reinterpret_cast<float *>(sm + kOffBias);
  const uint32_t barA = smem_u32(bar);

  // weights -> canonical K-major tiles; biases -> FP32
  for (int e = t; e < 64 * 80; e += kTile)
    *reinterpret_cast<uint16_t *>(sm + kOffW1 + kmajor_off(e / 80, e % 80, 80)) = wbf[kMlpW1 + e];
  for (int e = t; e < 64 * 64; e += kTile)
    *reinterpret_cast<uint16_t *>(sm + kOffW2 + kmajor_off(e / 64, e % 64, 64)) = wbf[kMlpW2 + e];
  for (int e = t; e < 16 * 64; e += kTile)
    *reinterpret_cast<uint16_t *>(sm + kOffW3 + kmajor_off(e / 64, e % 64, 64)) = wbf[kMlpW3 + e];
  for (int e = t; e < 64; e += kTile) bias[e] = frombf(wbf[kMlpB1 + e]), bias[64 + e] = frombf(wbf[kMlpB2 + e]);
  for (int e = t; e < 16; e += kTile) bias[128 + e] = frombf(wbf[kMlpB3 + e]);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(barA) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem  = *tslot;
  const uint32_t lane0 = (uint32_t)(warp * 32) << 16;
  uint32_t parity      = 0;
  bool ok              = true;

  const uint32_t aW1 = smem_u32(sm + kOffW1), aW2 = smem_u32(sm + kOffW2), aW3 = smem_u32(sm + kOffW3);
  const uint32_t aA = smem_u32(sm + kOffA);
  if (Step && a.n_dev && *a.n_dev < n) n = *a.n_dev; // a count known on the device only
  const size_t ntiles = (n + kTile - 1) / kTile;
  for (size_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const size_t i = tile * kTile + t;
    size_t trk     = i;
    bool valid     = false;
    float f[kMlpIn];
    int lv = -1;
    if (i < n) {
      if (Step) {
        trk = a.order ? (size_t)__ldg(a.order + i) : i;
        learn::V3 lp, ld;
        valid = learn::features(g, a.in[trk].navInd, learn::V3{a.x[trk], a.y[trk], a.z[trk]},
                                learn::V3{a.dx[trk], a.dy[trk], a.dz[trk]}, f, lv, lp, ld);
      } else {
        lv    = lvin[i];
        valid = lv >= 0;
        if (valid)
          for (int k = 0; k < kMlpIn; ++k) f[k] = feat[i * kMlpIn + k];
      }
    }
    // layer-1 operand row: features rounded to BF16, embedding row of the volume
    uint16_t x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = valid ? tobf(f[k]) : (uint16_t)0;
    if (valid) {
      const uint4 *er = reinterpret_cast<const uint4 *>(wbf + kMlpE + (size_t)lv * kMlpEmb);
      const uint4 e0 = __ldg(er), e1 = __ldg(er + 1);
      const uint32_t ew[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
#pragma unroll
      for (int j = 0; j < kMlpEmb; ++j) x[kMlpEmbOff + j] = (uint16_t)(ew[j >> 1] >> (16 * (j & 1)));
    }
#pragma unroll
    for (int kb = 0; kb < kMlpIn / 8; ++kb)
      store_chunk(sm + kOffA, t, kb, 80,
                  make_uint4(pack2(x[8 * kb], x[8 * kb + 1]), pack2(x[8 * kb + 2], x[8 * kb + 3]),
                             pack2(x[8 * kb + 4], x[8 * kb + 5]), pack2(x[8 * kb + 6], x[8 * kb + 7])));
    fence_async_smem();
    __syncthreads();
    if (t == 0) {
      tc_fence_after();
      for (int ks = 0; ks < 5; ++ks)
        mma_bf16(tmem, smem_desc(aA + ks * 256, 80), smem_desc(aW1 + ks * 256, 80), idesc_bf16(128, 64), ks > 0);
      mma_commit(barA);
    }
    ok = __all_sync(0xffffffffu, bar_wait(barA, parity)); // warp-uniform before tcgen05.ld
    if (ok) parity ^= 1; // on a time-out the phase is still pending: the drain below waits on it
    tc_fence_after();
    if (ok) {
      for (int c = 0; c < 64; c += 16) {
        float v[16];
        tmem_ld16(tmem + lane0 + c, v);
        uint16_t h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) h[j] = tobf(fmaxf(v[j] + bias[c + j], 0.f));
#pragma unroll
        for (int q = 0; q < 2; ++q)
          store_chunk(sm + kOffA, t, c / 8 + q, 64,
                      make_uint4(pack2(h[8 * q], h[8 * q + 1]), pack2(h[8 * q + 2], h[8 * q + 3]),
                                 pack2(h[8 * q + 4], h[8 * q + 5]), pack2(h[8 * q + 6], h[8 * q + 7])));
      }
    }
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
    if (!__syncthreads_and(ok)) break;
    if (t == 0) {
      tc_fence_after();
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tmem, smem_desc(aA + ks * 256, 64), smem_desc(aW2 + ks * 256, 64), idesc_bf16(128, 64), ks > 0);
      mma_commit(barA);
    }
    ok = __all_sync(0xffffffffu, bar_wait(barA, parity)); // warp-uniform before tcgen05.ld
    if (ok) parity ^= 1; // on a time-out the phase is still pending: the drain below waits on it
    tc_fence_after();
    if (ok) {
      for (int c = 0; c < 64; c += 16) {
        float v[16];
        tmem_ld16(tmem + lane0 + c, v);
        uint16_t h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) h[j] = tobf(fmaxf(v[j] + bias[64 + c + j], 0.f));
#pragma unroll
        for (int q = 0; q < 2; ++q)
          store_chunk(sm + kOffA, t, c / 8 + q, 64,
                      make_uint4(pack2(h[8 * q], h[8 * q + 1]), pack2(h[8 * q + 2], h[8 * q + 3]),
                                 pack2(h[8 * q + 4], h[8 * q + 5]), pack2(h[8 * q + 6], h[8 * q + 7])));
      }
    }
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
    if (!__syncthreads_and(ok)) break;
    if (t == 0) {
      tc_fence_after();
      for (int ks = 0; ks < 4; ++ks)
        mma_bf16(tmem, smem_desc(aA + ks * 256, 64), smem_desc(aW3 + ks * 256, 64), idesc_bf16(128, 16), ks > 0);
      mma_commit(barA);
    }
    ok = __all_sync(0xffffffffu, bar_wait(barA, parity)); // warp-uniform before tcgen05.ld
    if (ok) parity ^= 1; // on a time-out the phase is still pending: the drain below waits on it
    tc_fence_after();
    if (ok) {
      float v[16];
      tmem_ld16(tmem + lane0, v);
      int best = 0;
      float bv = -INFINITY;
      for (int o = 0; o < kMlpCls; ++o) {
        const float s = v[o] + bias[128 + o];
        if (logits && i < n) logits[i * kMlpOut + o] = s;
        if (s > bv) bv = s, best = o;
      }
      if (i < n) slot[trk] = (int8_t)(valid ? (best == 8 ? -1 : best) : -1);
    }
    tc_fence_before();
    __syncthreads();
    ok = __syncthreads_and(ok);
  }
  if (!ok) {
    if (t == 0) atomicExch(err, 1);
    // drain: a commit issued before the time-out still arrives on the barrier (bounded)
    bar_wait(barA, parity);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

template <bool Step>
cudaError_t launch_tc(const DevGeom &g, const StepArgs &a, const float *feat, const int32_t *lv, size_t n,
                      const uint16_t *wbf, int8_t *slot, float *logits, int *err, cudaStream_t s)
{
  if (n == 0) return cudaSuccess;
  static int configured = 0, blocks_per_sm = 1;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_propose_tc<Step>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSmemBytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_propose_tc<Step>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    // resident CTAs per SM from shared memory and registers (tensor memory: at most 6 x 64
    // of the 512 columns)
    cudaFuncAttributes fa{};
    int dev0 = 0, smem_sm = 0;
    e = cudaFuncGetAttributes(&fa, k_mlp_propose_tc<Step>);
    if (e == cudaSuccess) e = cudaGetDevice(&dev0);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev0);
    if (e != cudaSuccess) return e;
    const int by_smem = smem_sm / (kSmemBytes + 1024);
    const int by_regs = 65536 / ((fa.numRegs > 0 ? fa.numRegs : 255) * kTile);
    int r             = by_smem < by_regs ? by_smem : by_regs;
    blocks_per_sm     = r < 1 ? 1 : (r > 6 ? 6 : r);
    configured    = 1;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  size_t grid = (size_t)sms * blocks_per_sm, tiles = (n + kTile - 1) / kTile;
  if (grid > tiles) grid = tiles;
  k_mlp_propose_tc<Step><<<(unsigned)grid, kTile, kSmemBytes, s>>>(g, a, feat, lv, n, wbf, slot, logits, err);
  return cudaGetLastError();
}

} // namespace

cudaError_t launch_mlp_propose_tc(const DevGeom &g, const StepArgs &a, const uint16_t *wbf, int8_t *slot, int *err,
                                  cudaStream_t s)
{
  return launch_tc<true>(g, a, nullptr, nullptr, a.n, wbf, slot, nullptr, err, s);
}

cudaError_t launch_mlp_infer_feat_tc(const uint16_t *wbf, const float *feat, const int32_t *lv, size_t n, int8_t *slot,
                                     float *logits, int *err, cudaStream_t s)
{
  return launch_tc<false>(DevGeom{}, StepArgs{}, feat, lv, n, wbf, slot, logits, err, s);
}

} // namespace vg
