// FP64 throughput of the device, measured with independent DFMA chains.  Used
// as the roofline denominator for the FP64-bound element kernels (the DGEMM of
// cuBLAS runs below the DFMA rate on this part).
#include <cuda_runtime.h>

#include "../../include/muscade_gpu.h"

namespace {
__global__ void dfma_chains(double* out, int iters, double b, double c) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double a0 = tid * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c);
    a1 = fma(a1, b, c);
    a2 = fma(a2, b, c);
    a3 = fma(a3, b, c);
    a4 = fma(a4, b, c);
    a5 = fma(a5, b, c);
    a6 = fma(a6, b, c);
    a7 = fma(a7, b, c);
  }
  out[tid] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
}  // namespace

extern "C" int mgpu_measure_fp64_peak(int32_t device, double* tflops) {
  if (!tflops) return MGPU_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MGPU_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 4, tpb = 256, n = blocks * tpb, iters = 20000;
  double* out = nullptr;
  if (cudaMalloc(&out, size_t(n) * sizeof(double)) != cudaSuccess) return MGPU_ERR_NOMEM;
  cudaEvent_t s, e;
  cudaEventCreate(&s);
  cudaEventCreate(&e);
  dfma_chains<<<blocks, tpb>>>(out, 200, 0.999999, 1e-7);
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(s);
    dfma_chains<<<blocks, tpb>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e);
    cudaEventSynchronize(e);
    float ms = 0;
    cudaEventElapsedTime(&ms, s, e);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(s);
  cudaEventDestroy(e);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return MGPU_ERR_CUDA;
  *tflops = 2.0 * double(n) * iters * 8 / (best * 1e-3) / 1e12;
  return MGPU_OK;
}
