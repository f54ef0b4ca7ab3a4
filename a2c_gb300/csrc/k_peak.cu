// Pipe-peak calibration: the roofline denominators for the FP32 and FP64
// SIMT pipes (the evaluator uses no tensor cores), measured on the device it
// runs on.  Each thread advances 8 independent FMA chains; a block count of
// 8 per SM keeps every scheduler issuing.  Flops counted as 2 per FMA.
#include <cstdio>

#include "internal.cuh"

namespace a2c {
namespace {

template <class T>
__global__ void __launch_bounds__(256) k_fma_chains(T *out, int iters, T seed) {
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + (T)(threadIdx.x + k);
  const T m = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = a[k] * m + c;  // contracted to FMA
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == (T)-12345.678) out[blockIdx.x] = s;  // never true; keeps the chains live
}

template <class T>
a2c_status measure(int device, double *flops) {
  A2C_CUDA(cudaSetDevice(device));
  int sms = 0;
  A2C_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int blocks = sms * 8, threads = 256;
  const int iters = sizeof(T) == 4 ? 16384 : 1024;
  T *out = nullptr;
  A2C_CUDA(cudaMalloc(&out, sizeof(T) * blocks));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)1);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, threads>>>(out, iters, (T)1);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  A2C_CUDA(err);
  *flops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3);
  return A2C_OK;
}

}  // namespace
}  // namespace a2c

extern "C" a2c_status a2c_gpp_peak_flops(int device, int precision, double *flops_per_s) {
  if (!flops_per_s) return A2C_ERR_INVALID;
  return precision == A2C_FP64 ? a2c::measure<double>(device, flops_per_s) : a2c::measure<float>(device, flops_per_s);
}
