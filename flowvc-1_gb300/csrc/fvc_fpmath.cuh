// fvc_fpmath.cuh -- two helpers that keep work off the FP64 pipe (GB300's
// FP64 rate is 1/64 of its FP32 rate) without changing a bit of any result.
#pragma once
#include <cuda_runtime.h>

namespace fvc {

// a / b rounded to nearest, given y = RN(1/b) (the IEEE quotient 1.0 / b,
// precomputed once per divisor).  Markstein's correction step:
//   r = a - b q (one FMA), q' = q + r y (one FMA)
// returns RN(a/b) exactly when y is within half an ulp of 1/b and q is
// within one ulp of a/b (P. Markstein, "Computation of elementary functions
// on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; the
// Handbook of Floating-Point Arithmetic, Muller et al., Birkhauser, treats
// the same theorem).  q0 = RN(a y) can be up to two ulps off, so one
// correction first brings it within 2^-104 relative (faithful), and the
// second gives the correctly rounded quotient.  The remainder a - b q is
// exact only without underflow, so numerators outside 2^-400 .. 2^400 in
// magnitude (zero included: IEEE keeps its sign) and divisors without a
// usable reciprocal (y passed as 0) take the IEEE division.  Cost: one DMUL
// and four DFMA, against a reciprocal iteration for the IEEE division.  A
// divisor that is a power of two (a grid spacing of 2^-7, say) has y = 1/b
// exactly, so a y is the quotient itself and its rounding is RN(a/b): one
// DMUL (the test is on b's fraction bits).
__device__ __forceinline__ double div_rn(double a, double b, double y) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff;
  if ((unsigned)(ea - (1023 - 400)) > 800u || __double2hiint(y) == 0) return a / b;
  if (((__double2hiint(b) & 0xfffff) | __double2loint(b)) == 0) return a * y;
  double q = a * y;
  double r = fma(-b, q, a);
  q = fma(r, y, q);
  r = fma(-b, q, a);
  return fma(r, y, q);
}

// x^(1/4) rounded to nearest, for RKF's step-size factor (the reference
// calls pow(x, 0.25), which glibc rounds correctly but for inputs within
// about 0.02 ulp of a rounding boundary).  y = sqrt(sqrt(x)) is within about
// an ulp; its residual y^4 - x is formed with error-free products
// (Dekker's TwoProduct by FMA: y*y = P + p, P*P = Q + q exactly, and Q - x
// exact by Sterbenz's lemma since Q is within a few ulps of x), and one
// Newton step t = y - (y^4 - x) / (4 y^3) lands within about 2^-104 of the
// root, so the final subtraction rounds to RN(x^(1/4)) unless the root lies
// within that distance of a rounding boundary.  Inputs outside
// 2^-960 .. 2^960 (where the products could over- or underflow) use pow.
__device__ __forceinline__ double rn_root4(double x) {
  if (!(x >= 0x1p-960 && x <= 0x1p960)) return pow(x, 0.25);
  const double y = sqrt(sqrt(x));
  const double P = y * y, p = fma(y, y, -P);
  const double Q = P * P, q = fma(P, P, -Q);
  const double r = (Q - x) + (q + (2.0 * P * p + p * p));
  return y - r / (4.0 * y * P);
}

// The reciprocal div_rn wants for divisor b, or 0 when b is outside
// 2^-400 .. 2^400 in magnitude (then div_rn divides).
__host__ __device__ __forceinline__ double rcp_for_div(double b) {
  double ab = b < 0 ? -b : b;
  if (!(ab >= 0x1p-400 && ab <= 0x1p400)) return 0.0;
  return 1.0 / b;
}

// x rounded toward zero to FP32 with integer operations only (no FP64-pipe
// conversion).  For |x| < 2^128 the result f satisfies |x - f| <= 2^-23 |x|
// + 2^-126; larger magnitudes, infinities and NaN give NaN, which fails
// every comparison and so leaves a decision to the FP64 path.
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int fe = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
  const unsigned man = ((hi & 0xfffffu) << 3) | (lo >> 29);
  unsigned bits;
  if (fe <= 0) bits = sign;
  else if (fe >= 255) bits = 0x7fc00000u;
  else bits = sign | ((unsigned)fe << 23) | man;
  return __uint_as_float(bits);
}

// x >= -1e-10 (ge) or x > -1e-10 -- the walk's TINY -- decided on the bit
// pattern with integer instructions (off the FP64 pipe), with the FP64
// comparison's outcome for every x: +0 .. +inf pass; a negative x passes when
// its magnitude is at most (below) 1e-10's; NaNs fail.
__device__ __forceinline__ bool above_neg_tiny(double x, bool ge) {
  // the move through inline PTX keeps the compiler from turning the integer
  // tests back into FP64 comparisons (it recognises the sign-mask idiom)
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  const unsigned long long a = u & 0x7fffffffffffffffull;
  const unsigned long long tiny = 0x3ddb7cdfd9d7bdbbull;  // bits of 1.0e-10
  if (!(u >> 63)) return a <= 0x7ff0000000000000ull;
  return ge ? a <= tiny : a < tiny;
}

// a < b decided on the bit patterns with integer instructions, with the
// FP64 comparison's outcome for every input: +0 == -0, NaN compares false.
// Each pattern maps to a signed key in the doubles' order (a negative
// double's key is minus its magnitude bits, so both zeros map to 0).
__device__ __forceinline__ bool bits_of(double x, long long& key) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  const unsigned long long a = u & 0x7fffffffffffffffull;
  key = (u >> 63) ? -(long long)a : (long long)a;
  return a <= 0x7ff0000000000000ull;  // not NaN
}
__device__ __forceinline__ bool lt_bits(double a, double b) {
  long long ka, kb;
  const bool na = bits_of(a, ka), nb = bits_of(b, kb);
  return na && nb && ka < kb;
}

// (int)floor(x) for 0 <= x < 2^31 (and NaN: 0, as the conversion gives it)
// with integer instructions; ompVC's cell index of a point inside the grid.
__device__ __forceinline__ int floor_nonneg_bits(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  const int e = (int)((u >> 52) & 0x7ff) - 1023;
  if (e < 0 || e > 30) return 0;
  const unsigned long long m = (u & 0xfffffffffffffull) | 0x10000000000000ull;
  return (int)(m >> (52 - e));
}

// A zero with x's sign (x * +0.0 for finite nonzero x), on the bit pattern.
__device__ __forceinline__ double zero_of(double x) {
  unsigned long long u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  u &= 0x8000000000000000ull;
  double z;
  asm("mov.b64 %0, %1;" : "=d"(z) : "l"(u));
  return z;
}

// (double)i for 0 <= i < 2^31, exactly, with integer instructions.
__device__ __forceinline__ double double_of_nonneg(int i) {
  if (i <= 0) return 0.0;
  const int e = 31 - __clz(i);
  const unsigned long long u = ((unsigned long long)(1023 + e) << 52) |
                               (((unsigned long long)i << (52 - e)) & 0xfffffffffffffull);
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
}

}  // namespace fvc
