// fvc_mixed_kernels.cu -- frame quantisation and position packing for the
// mixed-precision form.
#include <cuda_bf16.h>
#include <string.h>
#include <cuda_fp16.h>

#include "fvc_kernels.h"
#include "fvc_mixed.cuh"

namespace fvc {

static inline unsigned nblk_q(long n, int bs) {
  long b = (n + bs - 1) / bs;
  return (unsigned)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

// max |component| over the frame's nodes, as float bit patterns (the
// order of non-negative floats is that of their bits)
__global__ void k_maxabs(const double4_32a* f, long n, unsigned* out) {
  float m0 = 0.f, m1 = 0.f, m2 = 0.f;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double4_32a v = f[i];
    m0 = fmaxf(m0, fabsf((float)v.x));
    m1 = fmaxf(m1, fabsf((float)v.y));
    m2 = fmaxf(m2, fabsf((float)v.z));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, __float_as_uint(m0));
    atomicMax(out + 1, __float_as_uint(m1));
    atomicMax(out + 2, __float_as_uint(m2));
  }
}

__device__ __forceinline__ unsigned short enc16(float x, int fmt) {
  return fmt == QF_BF16 ? __bfloat16_as_ushort(__float2bfloat16_rn(x)) : __half_as_ushort(__float2half_rn(x));
}

__global__ void k_quantize(const double4_32a* f, long n, int fmt, float i0, float i1, float i2, ushort4* q) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double4_32a v = f[i];
    ushort4 o;
    o.x = enc16((float)v.x * i0, fmt);
    o.y = enc16((float)v.y * i1, fmt);
    o.z = enc16((float)v.z * i2, fmt);
    o.w = 0;
    q[i] = o;
  }
}

int quantize_frame(const double4_32a* f, long n, int fmt, ushort4* q, unsigned* scratch, float scale[3],
                   cudaStream_t s) {
  if (cudaMemsetAsync(scratch, 0, 3 * sizeof(unsigned), s) != cudaSuccess) return -1;
  k_maxabs<<<nblk_q(n, 256), 256, 0, s>>>(f, n, scratch);
  unsigned h[3] = {0, 0, 0};
  if (cudaMemcpyAsync(h, scratch, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
  if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
  float inv[3];
  for (int c = 0; c < 3; c++) {
    float mx;
    memcpy(&mx, &h[c], sizeof(float));
    scale[c] = (mx > 0.f && mx < 3.0e38f) ? mx : 1.0f;
    inv[c] = 1.0f / scale[c];
  }
  k_quantize<<<nblk_q(n, 256), 256, 0, s>>>(f, n, fmt, inv[0], inv[1], inv[2], q);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void k_pair_frames(const ushort4* a, const ushort4* b, long n, uint4* out) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const ushort4 p = a[i], q = b[i];
    out[i] = make_uint4((unsigned)p.x | ((unsigned)p.y << 16), (unsigned)p.z | ((unsigned)q.x << 16),
                        (unsigned)q.y | ((unsigned)q.z << 16), 0u);
  }
}
void pair_frames(const ushort4* a, const ushort4* b, long n, uint4* out, cudaStream_t s) {
  if (n > 0) k_pair_frames<<<nblk_q(n, 256), 256, 0, s>>>(a, b, n, out);
}

__global__ void k_pack_pairs(double* A, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float2 p = split_pos(A[i]);
    reinterpret_cast<float2*>(A)[i] = p;
  }
}
__global__ void k_unpack_pairs(double* A, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    A[i] = join_pos(reinterpret_cast<const float2*>(A)[i]);
}
// unpack the first 3 * (*count) slots (a count on the device)
__global__ void k_unpack_pairs_counted(double* A, const int* count) {
  const long n = 3L * *count;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    A[i] = join_pos(reinterpret_cast<const float2*>(A)[i]);
}
void unpack_pairs_counted(double* A, long max_rows, const int* count, cudaStream_t s) {
  if (max_rows > 0) k_unpack_pairs_counted<<<nblk_q(3 * max_rows, 256), 256, 0, s>>>(A, count);
}
void pack_pairs(double* A, long n, cudaStream_t s) {
  if (n > 0) k_pack_pairs<<<nblk_q(n, 256), 256, 0, s>>>(A, n);
}
void unpack_pairs(double* A, long n, cudaStream_t s) {
  if (n > 0) k_unpack_pairs<<<nblk_q(n, 256), 256, 0, s>>>(A, n);
}

}  // namespace fvc
