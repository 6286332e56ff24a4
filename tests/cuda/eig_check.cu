// Runs the FTLE eigenvalue helpers of fvc_ftle_math.cuh on the GPU over
// symmetric 3x3 matrices read from a file (n x 9 doubles, row-major): for
// each, the closed form's result and whether it accepted the matrix
// (max_eig_closed) and the Jacobi solver's result (max_eig).  Writes n x 3
// doubles (closed or NaN, accepted 1/0, Jacobi) to the output file.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fvc_ftle_math.cuh"

__global__ void k_eig(const double* C, long n, double* out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a[3][3], b[3][3];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) a[r][c] = b[r][c] = C[9 * i + 3 * r + c];
  double lam = 0.0;
  const bool ok = fvc::max_eig_closed(a, lam);
  out[3 * i] = ok ? lam : nan("");
  out[3 * i + 1] = ok ? 1.0 : 0.0;
  out[3 * i + 2] = fvc::max_eig(b);
}

int main(int argc, char** argv) {
  if (argc < 3) return 1;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<double> h;
  double v;
  while (fread(&v, sizeof(double), 1, f) == 1) h.push_back(v);
  fclose(f);
  const long n = (long)(h.size() / 9);
  if (n == 0) return 3;
  double *dC = nullptr, *dO = nullptr;
  if (cudaMalloc(&dC, sizeof(double) * 9 * n) != cudaSuccess) return 4;
  if (cudaMalloc(&dO, sizeof(double) * 3 * n) != cudaSuccess) return 4;
  cudaMemcpy(dC, h.data(), sizeof(double) * 9 * n, cudaMemcpyHostToDevice);
  k_eig<<<(unsigned)((n + 127) / 128), 128>>>(dC, n, dO);
  std::vector<double> o(3 * n);
  if (cudaMemcpy(o.data(), dO, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 5;
  FILE* g = fopen(argv[2], "wb");
  if (!g || fwrite(o.data(), sizeof(double), 3 * n, g) != (size_t)(3 * n)) return 6;
  fclose(g);
  cudaFree(dC);
  cudaFree(dO);
  printf("%ld\n", n);
  return 0;
}
