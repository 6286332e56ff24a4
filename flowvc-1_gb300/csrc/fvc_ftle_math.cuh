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

// The largest eigenvalue of a symmetric 3x3 from the trigonometric solution
// of its characteristic cubic (Smith, "Eigenvalues of a symmetric 3 x 3
// matrix", CACM 4(4), 1961): with q = tr/3, p^2 = |A - qI|_F^2 / 6 and
// r = det((A - qI)/p)/2, the largest root is q + 2p cos(acos(r)/3).  Its
// error is a few ulps of max(|q|, p) except where the two largest
// eigenvalues nearly coincide: there (r near -1) the root's derivative in r
// grows as 1/sqrt(1 - r^2), and below r = -0.999 the function returns false
// for the caller to use the Jacobi solver.  Applied to C - I (the FTLE is
// log1p of the result), its FTLE error on test matrices from the identity
// to strongly stretching ones was below 1e-13 relative.
__device__ __forceinline__ bool max_eig_closed(const double a[3][3], double& lam) {
  const double p1 = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
  const double q = (a[0][0] + a[1][1] + a[2][2]) * (1.0 / 3.0);
  const double b0 = a[0][0] - q, b1 = a[1][1] - q, b2 = a[2][2] - q;
  const double p = sqrt((b0 * b0 + b1 * b1 + b2 * b2 + 2.0 * p1) * (1.0 / 6.0));
  if (p == 0.0) {
    lam = q;
    return true;
  }
  const double ip = 1.0 / p;
  const double c00 = b0 * ip, c11 = b1 * ip, c22 = b2 * ip;
  const double c01 = a[0][1] * ip, c02 = a[0][2] * ip, c12 = a[1][2] * ip;
  const double r =
      0.5 * (c00 * (c11 * c22 - c12 * c12) - c01 * (c01 * c22 - c12 * c02) + c02 * (c01 * c12 - c11 * c02));
  if (!(r >= -0.999)) return false;
  const double phi = r >= 1.0 ? 0.0 : acos(r) * (1.0 / 3.0);
  lam = q + 2.0 * p * cos(phi);
  return true;
}

// Cauchy-Green tensor of the central / one-sided flow-map gradient
// (ompVC/ftle.c:1000-1027, 1159-1187) from the stencil's differences
// d[component][direction] (R - L, T - B, F - Bk), returned minus the
// identity: its largest eigenvalue is then lambda - 1 with an error relative
// to itself, also where the flow map is close to a rigid motion.  The
// differences are scaled by the reciprocal of each spacing (ompVC divides;
// the products differ from the quotients by at most an ulp).
__device__ __forceinline__ void tensor_from_diffs(int dims, const double d[3][3], double fx, double fy, double fz,
                                                  double dx, double dy, double dz, double C[3][3]) {
  double Dp[3][3];
  const double ix = 1.0 / (fx * dx), iy = 1.0 / (fy * dy), iz = dims == 3 ? 1.0 / (fz * dz) : 0.0;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    Dp[q][0] = (dims == 3 || q < 2) ? d[q][0] * ix : 0.0;
    Dp[q][1] = (dims == 3 || q < 2) ? d[q][1] * iy : 0.0;
    Dp[q][2] = dims == 3 ? d[q][2] * iz : 0.0;
  }
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      double acc = 0;
      for (int q = 0; q < 3; q++) acc += Dp[q][a] * Dp[q][b];
      C[a][b] = a == b ? acc - 1.0 : acc;
    }
}

// The same from the six stencil positions.
__device__ __forceinline__ void stencil_tensor(int dims, const double* L, const double* R, const double* B,
                                               const double* T, const double* Bk, const double* F, double fx,
                                               double fy, double fz, double dx, double dy, double dz,
                                               double C[3][3]) {
  double d[3][3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    d[q][0] = R[q] - L[q];
    d[q][1] = T[q] - B[q];
    d[q][2] = F[q] - Bk[q];
  }
  tensor_from_diffs(dims, d, fx, fy, fz, dx, dy, dz, C);
}

// lambda - 1 for the tensor's largest eigenvalue lambda (GetMaxEigenvalue,
// ompVC/ftle.c:1029, 1189): the closed form, else Jacobi.
__device__ __forceinline__ double stencil_lambda_m1(int dims, const double* L, const double* R, const double* B,
                                                    const double* T, const double* Bk, const double* F, double fx,
                                                    double fy, double fz, double dx, double dy, double dz) {
  double C[3][3], lm1;
  stencil_tensor(dims, L, R, B, T, Bk, F, fx, fy, fz, dx, dy, dz, C);
  if (!max_eig_closed(C, lm1)) lm1 = max_eig(C);
  return lm1;
}

}  // namespace fvc
