// Learned proposal: feature/label generation, training kernels (FP32 forward, backward and
// Adam over the flat parameter vector) and the SIMT BF16 inference kernel used as the
// reference for the tensor-core one.
#define VG_FP64_INT_COMPARE 0 // latency-bound navigation code (fp64_int.cuh)
#include "learn_features.cuh"
#include <cuda_bf16.h>

namespace vg {
namespace {

inline unsigned grid_for(size_t n, int block)
{
  size_t blocks       = (n + block - 1) / block;
  const size_t maxgrd = 152 * 16;
  if (blocks > maxgrd) blocks = maxgrd;
  return (unsigned)(blocks ? blocks : 1);
}

__global__ void __launch_bounds__(256) k_learn_features(const DevGeom g, const StepArgs a, float *__restrict__ feat,
                                                        int32_t *__restrict__ lvout, int8_t *__restrict__ label)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    float f[kMlpIn];
    int lv = -1;
    learn::V3 lp, ld;
    const NavState s = a.in[i];
    const bool ok = learn::features(g, s.navInd, learn::V3{a.x[i], a.y[i], a.z[i]}, learn::V3{a.dx[i], a.dy[i], a.dz[i]},
                                    f, lv, lp, ld);
    float *o = feat + i * kMlpIn;
    for (int k = 0; k < kMlpIn; ++k) o[k] = ok ? f[k] : 0.f;
    lvout[i] = lv;
    if (label) label[i] = (int8_t)(ok ? learn::label_fp64(g, s, lv, lp, ld) : -1);
  }
}

// ---------------------------------------------------------------- training (FP32)
// X[b] = feat[idx[b]] with the embedding of its logical volume in columns [6, 22).
__global__ void k_gather(const float *__restrict__ feat, const int32_t *__restrict__ lv,
                         const int8_t *__restrict__ label, const uint32_t *__restrict__ idx, int nb,
                         const float *__restrict__ emb, float *__restrict__ X, int32_t *__restrict__ y,
                         int32_t *__restrict__ ylv)
{
  const int b = blockIdx.x * blockDim.y + threadIdx.y;
  if (b >= nb) return;
  const uint32_t j = idx[b];
  const int l      = lv[j];
  for (int k = threadIdx.x; k < kMlpIn; k += blockDim.x) {
    float v = feat[(size_t)j * kMlpIn + k];
    if (k >= kMlpEmbOff && k < kMlpEmbOff + kMlpEmb) v = emb[(size_t)l * kMlpEmb + (k - kMlpEmbOff)];
    X[(size_t)b * kMlpIn + k] = v;
  }
  if (threadIdx.x == 0) {
    y[b]   = label[j];
    ylv[b] = l;
  }
}

// Y = act(X W^T + bias) for 32 samples per block; Z keeps the pre-activation.
template <int K, int N>
__global__ void __launch_bounds__(256) k_linear(const float *__restrict__ X, const float *__restrict__ W,
                                                const float *__restrict__ bias, float *__restrict__ Z,
                                                float *__restrict__ Y, int nb, bool relu)
{
  __shared__ float Ws[N][K + 1];
  __shared__ float Xs[32][K + 1];
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) Ws[e / K][e % K] = W[e];
  const int b0 = blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * K; e += blockDim.x) {
    const int r = e / K;
    Xs[r][e % K] = (b0 + r < nb) ? X[(size_t)(b0 + r) * K + e % K] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * N; e += blockDim.x) {
    const int r = e / N, o = e % N;
    if (b0 + r >= nb) continue;
    float sum = bias[o];
    for (int k = 0; k < K; ++k) sum += Xs[r][k] * Ws[o][k];
    const size_t at = (size_t)(b0 + r) * N + o;
    Z[at]           = sum;
    Y[at]           = relu ? fmaxf(sum, 0.f) : sum;
  }
}

// Softmax cross-entropy over the first kMlpCls logits; dZ = (softmax - onehot) / nb.
__global__ void k_xent(const float *__restrict__ Z, const int32_t *__restrict__ y, int nb, float *__restrict__ dZ,
                       float *__restrict__ loss)
{
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const float *z = Z + (size_t)b * kMlpOut;
  float mx       = z[0];
  for (int k = 1; k < kMlpCls; ++k) mx = fmaxf(mx, z[k]);
  float se = 0.f;
  for (int k = 0; k < kMlpCls; ++k) se += expf(z[k] - mx);
  const float lse = mx + logf(se);
  atomicAdd(loss, lse - z[y[b]]);
  float *d = dZ + (size_t)b * kMlpOut;
  for (int k = 0; k < kMlpOut; ++k)
    d[k] = k < kMlpCls ? (expf(z[k] - lse) - (k == y[b] ? 1.f : 0.f)) / (float)nb : 0.f;
}

// dX = dY W, masked by Zprev > 0 when Zprev is given (ReLU of the previous layer).
template <int K, int N>
__global__ void __launch_bounds__(256) k_linear_bwd_x(const float *__restrict__ dY, const float *__restrict__ W,
                                                      const float *__restrict__ Zprev, float *__restrict__ dX, int nb)
{
  __shared__ float Ws[N][K + 1];
  __shared__ float Ds[32][N + 1];
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) Ws[e / K][e % K] = W[e];
  const int b0 = blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * N; e += blockDim.x) {
    const int r = e / N;
    Ds[r][e % N] = (b0 + r < nb) ? dY[(size_t)(b0 + r) * N + e % N] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * K; e += blockDim.x) {
    const int r = e / K, k = e % K;
    if (b0 + r >= nb) continue;
    float sum = 0.f;
    for (int o = 0; o < N; ++o) sum += Ds[r][o] * Ws[o][k];
    const size_t at = (size_t)(b0 + r) * K + k;
    dX[at]          = (Zprev && !(Zprev[at] > 0.f)) ? 0.f : sum;
  }
}

// dW += dY^T X and db += sum dY over 64 samples per block (atomics across blocks).
template <int K, int N>
__global__ void __launch_bounds__(256) k_linear_bwd_w(const float *__restrict__ dY, const float *__restrict__ X,
                                                      float *__restrict__ dW, float *__restrict__ db, int nb)
{
  __shared__ float Ds[64][N];
  __shared__ float Xs[64][K];
  const int b0 = blockIdx.x * 64;
  for (int e = threadIdx.x; e < 64 * N; e += blockDim.x) {
    const int r = e / N;
    Ds[r][e % N] = (b0 + r < nb) ? dY[(size_t)(b0 + r) * N + e % N] : 0.f;
  }
  for (int e = threadIdx.x; e < 64 * K; e += blockDim.x) {
    const int r = e / K;
    Xs[r][e % K] = (b0 + r < nb) ? X[(size_t)(b0 + r) * K + e % K] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) {
    const int o = e / K, k = e % K;
    float sum   = 0.f;
    for (int r = 0; r < 64; ++r) sum += Ds[r][o] * Xs[r][k];
    atomicAdd(&dW[e], sum);
  }
  for (int o = threadIdx.x; o < N; o += blockDim.x) {
    float sum = 0.f;
    for (int r = 0; r < 64; ++r) sum += Ds[r][o];
    atomicAdd(&db[o], sum);
  }
}

__global__ void k_embed_grad(const float *__restrict__ dX, const int32_t *__restrict__ ylv, int nb,
                             float *__restrict__ dE)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nb * kMlpEmb) return;
  const int b = e / kMlpEmb, k = e % kMlpEmb;
  atomicAdd(&dE[(size_t)ylv[b] * kMlpEmb + k], dX[(size_t)b * kMlpIn + kMlpEmbOff + k]);
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                       float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float g = gr[i];
    m[i]          = b1 * m[i] + (1.f - b1) * g;
    v[i]          = b2 * v[i] + (1.f - b2) * g * g;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
  }
}

__global__ void k_to_bf16(const float *__restrict__ p, uint16_t *__restrict__ w, size_t n)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    w[i] = __bfloat16_as_ushort(__float2bfloat16_rn(p[i]));
}

// ---------------------------------------------------------------- SIMT inference
__device__ __forceinline__ float bf(uint16_t u) { return __bfloat162float(__ushort_as_bfloat16(u)); }
__device__ __forceinline__ float rbf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Inference semantics shared with the tensor-core kernel: inputs and hidden activations
// rounded to BF16, BF16 weights and biases, FP32 sums, the bias added after the sum.
// W: the BF16 parameters widened to FP32 (shared memory); the embedding row is read from
// the BF16 table. Returns the slot (0..7) or -1 for "none".
__device__ __forceinline__ int mlp_forward(const float *W, const uint16_t *__restrict__ wbf, const float *feat, int l,
                                          float *logits)
{
  float x[kMlpIn], h1[kMlpHid], h2[kMlpHid];
  for (int k = 0; k < kMlpIn; ++k) {
    const bool e = k >= kMlpEmbOff && k < kMlpEmbOff + kMlpEmb;
    x[k]         = e ? bf(wbf[kMlpE + (size_t)l * kMlpEmb + (k - kMlpEmbOff)]) : rbf(feat[k]);
  }
  for (int o = 0; o < kMlpHid; ++o) {
    float s = 0.f;
    for (int k = 0; k < kMlpIn; ++k) s += W[kMlpW1 + o * kMlpIn + k] * x[k];
    h1[o] = rbf(fmaxf(s + W[kMlpB1 + o], 0.f));
  }
  for (int o = 0; o < kMlpHid; ++o) {
    float s = 0.f;
    for (int k = 0; k < kMlpHid; ++k) s += W[kMlpW2 + o * kMlpHid + k] * h1[k];
    h2[o] = rbf(fmaxf(s + W[kMlpB2 + o], 0.f));
  }
  int best = 0;
  float bv = -INFINITY;
  for (int o = 0; o < kMlpCls; ++o) {
    float s = 0.f;
    for (int k = 0; k < kMlpHid; ++k) s += W[kMlpW3 + o * kMlpHid + k] * h2[k];
    s += W[kMlpB3 + o];
    if (logits) logits[o] = s;
    if (s > bv) bv = s, best = o;
  }
  return best == 8 ? -1 : best;
}

__global__ void __launch_bounds__(128) k_mlp_infer_feat(const uint16_t *__restrict__ wbf, const float *__restrict__ feat,
                                                        const int32_t *__restrict__ lv, size_t n,
                                                        int8_t *__restrict__ slot, float *__restrict__ logits)
{
  __shared__ float W[kMlpE];
  for (int e = threadIdx.x; e < kMlpE; e += blockDim.x) W[e] = bf(wbf[e]);
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int l = lv[i];
    if (l < 0) {
      slot[i] = -1;
      continue;
    }
    slot[i] = (int8_t)mlp_forward(W, wbf, feat + i * kMlpIn, l, logits ? logits + i * kMlpOut : nullptr);
  }
}

// Features + inference for the step: slot[t] for every track t (visited in `order` when
// given, so neighbouring threads share a logical volume).
__global__ void __launch_bounds__(128) k_mlp_propose(const DevGeom g, const StepArgs a, const uint16_t *__restrict__ wbf,
                                                     int8_t *__restrict__ slot)
{
  __shared__ float W[kMlpE];
  for (int e = threadIdx.x; e < kMlpE; e += blockDim.x) W[e] = bf(wbf[e]);
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t n      = a.n_dev && *a.n_dev < a.n ? (size_t)*a.n_dev : a.n;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const size_t t = a.order ? (size_t)__ldg(a.order + i) : i;
    float f[kMlpIn];
    int lv = -1;
    learn::V3 lp, ld;
    const bool ok = learn::features(g, a.in[t].navInd, learn::V3{a.x[t], a.y[t], a.z[t]},
                                    learn::V3{a.dx[t], a.dy[t], a.dz[t]}, f, lv, lp, ld);
    slot[t] = (int8_t)(ok ? mlp_forward(W, wbf, f, lv, nullptr) : -1);
  }
}

} // namespace

cudaError_t launch_learn_features(const DevGeom &g, const StepArgs &a, float *feat, int32_t *lv, int8_t *label,
                                  cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  k_learn_features<<<grid_for(a.n, 256), 256, 0, s>>>(g, a, feat, lv, label);
  return cudaGetLastError();
}

size_t mlp_train_ws_floats(int nb)
{
  // X, dX (80 each), Z1 H1 Z2 H2 dH2 dH1 (64 each), Z3 L dZ3 (16 each), y, ylv
  return (size_t)nb * (2 * kMlpIn + 6 * kMlpHid + 3 * kMlpOut + 2) + 64;
}

cudaError_t launch_mlp_grad(const float *params, int n_lv, const float *feat, const int32_t *lv, const int8_t *label,
                            const uint32_t *idx, int nb, float *grads, float *loss, float *ws, cudaStream_t s)
{
  const size_t P = mlp_param_count(n_lv);
  cudaError_t e  = cudaMemsetAsync(grads, 0, P * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float), s);
  if (e != cudaSuccess) return e;
  if (nb <= 0) return cudaSuccess;
  float *X = ws, *dX = X + (size_t)nb * kMlpIn;
  float *Z1 = dX + (size_t)nb * kMlpIn, *H1 = Z1 + (size_t)nb * kMlpHid;
  float *Z2 = H1 + (size_t)nb * kMlpHid, *H2 = Z2 + (size_t)nb * kMlpHid;
  float *dH2 = H2 + (size_t)nb * kMlpHid, *dH1 = dH2 + (size_t)nb * kMlpHid;
  float *Z3 = dH1 + (size_t)nb * kMlpHid, *L = Z3 + (size_t)nb * kMlpOut, *dZ3 = L + (size_t)nb * kMlpOut;
  int32_t *y = reinterpret_cast<int32_t *>(dZ3 + (size_t)nb * kMlpOut), *ylv = y + nb;
  const unsigned b32 = (unsigned)((nb + 31) / 32), b64 = (unsigned)((nb + 63) / 64);
  k_gather<<<(nb + 7) / 8, dim3(32, 8), 0, s>>>(feat, lv, label, idx, nb, params + kMlpE, X, y, ylv);
  k_linear<kMlpIn, kMlpHid><<<b32, 256, 0, s>>>(X, params + kMlpW1, params + kMlpB1, Z1, H1, nb, true);
  k_linear<kMlpHid, kMlpHid><<<b32, 256, 0, s>>>(H1, params + kMlpW2, params + kMlpB2, Z2, H2, nb, true);
  k_linear<kMlpHid, kMlpOut><<<b32, 256, 0, s>>>(H2, params + kMlpW3, params + kMlpB3, Z3, L, nb, false);
  k_xent<<<(nb + 255) / 256, 256, 0, s>>>(Z3, y, nb, dZ3, loss);
  k_linear_bwd_w<kMlpHid, kMlpOut><<<b64, 256, 0, s>>>(dZ3, H2, grads + kMlpW3, grads + kMlpB3, nb);
  k_linear_bwd_x<kMlpHid, kMlpOut><<<b32, 256, 0, s>>>(dZ3, params + kMlpW3, Z2, dH2, nb);
  k_linear_bwd_w<kMlpHid, kMlpHid><<<b64, 256, 0, s>>>(dH2, H1, grads + kMlpW2, grads + kMlpB2, nb);
  k_linear_bwd_x<kMlpHid, kMlpHid><<<b32, 256, 0, s>>>(dH2, params + kMlpW2, Z1, dH1, nb);
  k_linear_bwd_w<kMlpIn, kMlpHid><<<b64, 256, 0, s>>>(dH1, X, grads + kMlpW1, grads + kMlpB1, nb);
  k_linear_bwd_x<kMlpIn, kMlpHid><<<b32, 256, 0, s>>>(dH1, params + kMlpW1, nullptr, dX, nb);
  k_embed_grad<<<(nb * kMlpEmb + 255) / 256, 256, 0, s>>>(dX, ylv, nb, grads + kMlpE);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *params, const float *grads, float *m, float *v, size_t n, float lr, float b1,
                            float b2, float eps, int t, cudaStream_t s)
{
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  k_adam<<<grid_for(n, 256), 256, 0, s>>>(params, grads, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_mlp_to_bf16(const float *params, uint16_t *wbf, size_t n, cudaStream_t s)
{
  k_to_bf16<<<grid_for(n, 256), 256, 0, s>>>(params, wbf, n);
  return cudaGetLastError();
}

cudaError_t launch_mlp_propose(const DevGeom &g, const StepArgs &a, const uint16_t *wbf, int8_t *slot, cudaStream_t s)
{
  if (a.n == 0) return cudaSuccess;
  k_mlp_propose<<<grid_for(a.n, 128), 128, 0, s>>>(g, a, wbf, slot);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer_feat(const uint16_t *wbf, int n_lv, const float *feat, const int32_t *lv, size_t n,
                                  int8_t *slot, float *logits, cudaStream_t s)
{
  (void)n_lv;
  if (n == 0) return cudaSuccess;
  k_mlp_infer_feat<<<grid_for(n, 128), 128, 0, s>>>(wbf, feat, lv, n, slot, logits);
  return cudaGetLastError();
}

} // namespace vg
