// FP64 issue-rate probe: the peak against which the navigation kernels' FP64 roofline is
// stated. Each thread runs 8 independent chains of explicit fma() (one DFMA each), enough
// warps per SM to keep the FP64 pipe full; the rate is DFMA instructions per second of the
// timed launch (CUDA events on the caller's stream, after one warm-up launch).
#include "../../include/vecgeom_gb300.h"
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_fp64_fma_rate(double *out, int iters, double b, double c)
{
  double a[kChains];
  for (int j = 0; j < kChains; ++j) a[j] = 1.0 + 1e-3 * (threadIdx.x + j);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], b, c);
  double s = 0.;
  for (int j = 0; j < kChains; ++j) s += a[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" int vg_device_fp64_rate(double *fma_per_s, void *stream)
{
  if (!fma_per_s) return VG_EINVAL;
  *fma_per_s = 0.;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return VG_ECUDA;
  const int grid = sms * 8, block = 256, iters = 1024;
  cudaStream_t s = (cudaStream_t)stream;
  double *out    = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaMalloc(&out, sizeof(double) * (size_t)grid * block);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_fp64_fma_rate<<<grid, block, 0, s>>>(out, 16, 1.0000001, 1e-9);
    e = cudaEventRecord(e0, s);
  }
  if (e == cudaSuccess) {
    k_fp64_fma_rate<<<grid, block, 0, s>>>(out, iters, 1.0000001, 1e-9);
    e = cudaEventRecord(e1, s);
  }
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return VG_ECUDA;
  *fma_per_s = (double)grid * block * iters * kChains / (ms * 1e-3);
  return VG_OK;
}
