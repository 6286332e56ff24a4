// fp64_rate.cu -- FP64 issue-rate probe of a device: the denominators of the
// FP64 roofline the exact advection path is measured against (GB300's FP64
// rate is a small fraction of its FP32 rate, and no vendor figure is
// assumed).  A measurement aid of the benchmark, not part of the engine.
//
//   fp64_rate [device]   prints {"fma_per_s": F, "div_per_s": D}
//
// F counts fused multiply-adds (one operation each), D IEEE divisions.
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

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

int fail(const char* what, cudaError_t e) {
  fprintf(stderr, "fp64_rate: %s: %s\n", what, cudaGetErrorString(e));
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  const int device = argc > 1 ? atoi(argv[1]) : 0;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail("cudaSetDevice", e);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* d = nullptr;
  if ((e = cudaMalloc(&d, sizeof(double))) != cudaSuccess) return fail("cudaMalloc", e);
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
  const double fma_s = (double)blocks * threads * it_fma * 8 / (ms * 1e-3);
  cudaEventRecord(e0);
  k_fp64_div<<<blocks, threads>>>(d, it_div, 1.0000001);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  const double div_s = (double)blocks * threads * it_div * 8 / (ms * 1e-3);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("probe kernels", e);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  printf("{\"fma_per_s\": %.6e, \"div_per_s\": %.6e}\n", fma_s, div_s);
  return 0;
}
