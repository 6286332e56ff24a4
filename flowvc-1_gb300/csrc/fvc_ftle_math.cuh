// fvc_ftle_math.cuh -- FTLE stencil and largest eigenvalue (device).
#pragma once
#include "fvc_device.cuh"

namespace fvc {

// Largest eigenvalue of a symmetric 3x3 by cyclic Jacobi rotations (Jacobi
// 1846 with Rutishauser's update; Golub & Van Loan section 8.5).
__device__ __forceinline__ double max_eig(double a[3][3]) {
  const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
  for (int sweep = 0; sweep < 32; sweep++) {
    int rotated = 0;
    for (int nn = 0; nn < 3; nn++) {
      int p = P[nn], q = Q[nn], r = 3 - p - q;
      double apq = a[p][q];
      if (apq == 0.0) continue;
      if (fabs(apq) <= 1e-18 * (fabs(a[p][p]) + fabs(a[q][q]))) {
        a[p][q] = a[q][p] = 0.0;
        continue;
      }
      rotated = 1;
      double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
      double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
      if (theta < 0.0) t = -t;
      double cs = 1.0 / sqrt(t * t + 1.0);
      double sn = t * cs;
      double tau = sn / (1.0 + cs);
      a[p][p] = a[p][p] - t * apq;
      a[q][q] = a[q][q] + t * apq;
      a[p][q] = a[q][p] = 0.0;
      double arp = a[r][p], arq = a[r][q];
      a[r][p] = a[p][r] = arp - sn * (arq + tau * arp);
      a[r][q] = a[q][r] = arq + sn * (arp - tau * arq);
    }
    if (!rotated) break;
  }
  return dmax(a[0][0], dmax(a[1][1], a[2][2]));
}

// Cauchy-Green tensor of the central / one-sided flow-map gradient and its
// largest eigenvalue (ompVC/ftle.c:1000-1029, 1159-1189).
__device__ __forceinline__ double stencil_lambda(int dims, const double* L, const double* R, const double* B,
                                 const double* T, const double* Bk, const double* F, double fx,
                                 double fy, double fz, double dx, double dy, double dz) {
  double Dp[3][3], C[3][3];
  if (dims == 3) {
    Dp[0][2] = (F[0] - Bk[0]) / (fz * dz);
    Dp[1][2] = (F[1] - Bk[1]) / (fz * dz);
    Dp[2][0] = (R[2] - L[2]) / (fx * dx);
    Dp[2][1] = (T[2] - B[2]) / (fy * dy);
    Dp[2][2] = (F[2] - Bk[2]) / (fz * dz);
  } else {
    Dp[0][2] = 0;
    Dp[1][2] = 0;
    Dp[2][0] = 0;
    Dp[2][1] = 0;
    Dp[2][2] = 0;
  }
  Dp[0][0] = (R[0] - L[0]) / (fx * dx);
  Dp[0][1] = (T[0] - B[0]) / (fy * dy);
  Dp[1][0] = (R[1] - L[1]) / (fx * dx);
  Dp[1][1] = (T[1] - B[1]) / (fy * dy);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      double acc = 0;
      for (int q = 0; q < 3; q++) acc += Dp[q][a] * Dp[q][b];
      C[a][b] = acc;
    }
  return max_eig(C);
}

}  // namespace fvc
