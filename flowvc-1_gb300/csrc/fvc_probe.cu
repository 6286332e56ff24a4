// fvc_probe.cu -- FP64 issue-rate probes: the denominators of the FP64
// roofline the exact advection path is measured against (GB300's FP64 rate
// is a small fraction of its FP32 rate, and no vendor figure is assumed).
#include <cuda_runtime.h>

#include "fvc.h"

namespace {

// 8 independent chains of dependent multiply-adds per thread.
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = threadIdx.x * 1e-9 + c;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// 8 independent chains of IEEE double divisions per thread.
__global__ void k_fp64_div(double* out, int iters, double a) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = 1.0 + threadIdx.x * 1e-9 + c;
#pragma unroll 1
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = a / x[c];
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += x[c];
  if (s == 12345.678) out[0] = s;
}

}  // namespace

// Measured FP64 rates of this device: rates[0] = fused multiply-adds per
// second (each counted as one operation), rates[1] = IEEE divisions per
// second.  Runs on the calling thread's current device, a few milliseconds.
extern "C" fvc_status fvc_probe_fp64(int device, double rates[2]) {
  if (!rates) return FVC_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return FVC_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return FVC_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  const int it_fma = 4096, it_div = 256;
  float ms = 0;
  k_fp64_fma<<<blocks, threads>>>(d, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fp64_fma<<<blocks, threads>>>(d, it_fma, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  rates[0] = (double)blocks * threads * it_fma * 8 / (ms * 1e-3);
  cudaEventRecord(e0);
  k_fp64_div<<<blocks, threads>>>(d, it_div, 1.0000001);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  rates[1] = (double)blocks * threads * it_div * 8 / (ms * 1e-3);
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return err == cudaSuccess ? FVC_OK : FVC_ERR_CUDA;
}
