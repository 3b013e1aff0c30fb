// FP64 FMA throughput probe: the denominator of the FP64-ALU roofline that
// bounds the FP64 form of the force step (the GPU's HBM and tensor peaks do
// not bound these kernels).  Independent FMA chains, fixed trip count.
#include "../../include/reaxgpu.h"
#include "rg_internal.h"

namespace {
__global__ void k_fp64_fma(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int rg_measure_fp64_peak(int device, double *tflops) {
  if (!tflops) return RG_E_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return RG_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256, iters = 20000;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return RG_E_CUDA;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fp64_fma<<<blocks, threads>>>(out, 100, 0.999, 0.001);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(a);
    k_fp64_fma<<<blocks, threads>>>(out, iters, 0.999, 0.001);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return RG_E_CUDA;
  *tflops = 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return RG_OK;
}
