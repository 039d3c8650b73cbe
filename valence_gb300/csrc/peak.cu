/*
 * peak.cu -- measured FMA throughput of the device (FP64 and FP32), the
 * roofline denominators for the CUDA-core-bound ERI kernels.  Eight
 * independent dependent-FMA chains per thread, a grid of 4 blocks x 256
 * threads per SM, timed with CUDA events; best of three launches.
 */
#include <cuda_runtime.h>

#include "../../include/vsvb_gpu.h"

namespace {

template <typename T>
__global__ void fma_chain(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int measure(int nsm, int iters, double *flops) {
  const int threads = 256, blocks = nsm * 4;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * threads * blocks) != cudaSuccess) return VSVB_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess) return VSVB_ERR_CUDA;
  *flops = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3);
  return VSVB_OK;
}

}  // namespace

extern "C" int vsvb_gpu_fma_peak(int device, double *fp64, double *fp32) {
  if (cudaSetDevice(device) != cudaSuccess) return VSVB_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return VSVB_ERR_CUDA;
  int rc = measure<double>(prop.multiProcessorCount, 2048, fp64);
  if (rc) return rc;
  return measure<float>(prop.multiProcessorCount, 65536, fp32);
}
