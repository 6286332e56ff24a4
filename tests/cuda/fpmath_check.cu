// Checks the helpers of fvc_fpmath.cuh on the GPU: div_rn(a, b,
// rcp_for_div(b)) must equal CUDA's IEEE a / b bit for bit, and f32_trunc(x)
// must equal __double2float_rz(x), on many seeded operands from several
// distributions, above_neg_tiny(x) must agree with the FP64 comparisons
// against -1e-10 it stands for, and the integer comparison and conversion
// helpers with the FP64 operations they replace (one line of counts on
// stdout).  With a file argument it
// also writes seeded (x, rn_root4(x)) pairs there for the host to check.
#include <cstdio>
#include <cstdint>
#include <cstring>

#include "fvc_fpmath.cuh"

using namespace fvc;

__device__ __forceinline__ uint64_t mix(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// a double with a random 52-bit fraction, random sign and exponent in [lo, hi]
__device__ __forceinline__ double rnd(uint64_t h, int lo, int hi) {
  uint64_t e = (uint64_t)(lo + (int)((h >> 52) % (uint64_t)(hi - lo + 1))) + 1023;
  uint64_t bits = (h & 0xfffffffffffffull) | (e << 52) | ((h >> 63) << 63);
  return __longlong_as_double((long long)bits);
}

struct Out {
  unsigned long long n_div, bad_div, n_cvt, bad_cvt;
  double a, b;
  int kind;
};

__global__ void k_div(uint64_t seed, long n, Out* o) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t h1 = mix(seed ^ (uint64_t)i), h2 = mix(h1), h3 = mix(h2);
  int kind = (int)(h3 % 7);
  double a, b;
  switch (kind) {
    case 0: a = rnd(h1, -300, 300); b = rnd(h2, -99, 99); break;      // wide exponents
    case 1: a = rnd(h1, -30, -10); b = rnd(h2, -24, -16); break;      // cofactor sums / element volumes
    case 2: b = rnd(h2, -24, -16); a = b * (double)(int)(h1 % 2001 - 1000); break;  // exact quotients
    case 3: {                                                          // quotients near a rounding midpoint
      double q = rnd(h1, -8, 8);
      b = rnd(h2, -20, 20);
      a = fma(b, q, b * ldexp(q, -53));
      break;
    }
    case 4: a = rnd(h1, -60, 60); b = 6.0; break;                      // the RK4 update
    case 5: a = rnd(h1, -60, 60); b = ldexp((h2 & 1) ? -1.0 : 1.0, (int)(h2 % 61) - 30); break;  // powers of two
    default: a = rnd(h1, -400, 400); b = rnd(h2, -400, 400); break;   // the fallback edges
  }
  double want = a / b, got = div_rn(a, b, rcp_for_div(b));
  bool bad = __double_as_longlong(want) != __double_as_longlong(got);
  if (bad && atomicAdd(&o->bad_div, 1ull) == 0) {
    o->a = a;
    o->b = b;
    o->kind = kind;
  }
  double x = rnd(h3, -126, 127);
  float fw = __double2float_rz(x), fg = f32_trunc(x);
  if (__float_as_uint(fw) != __float_as_uint(fg)) atomicAdd(&o->bad_cvt, 1ull);
}

// above_neg_tiny against the FP64 comparisons it replaces, x >= -TINY,
// x > -TINY and the reference's own form (x + TINY) >= 0, on values around
// -TINY, random magnitudes and the special values
__global__ void k_tiny(uint64_t seed, long n, unsigned long long* bad) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double TINY = 1.0e-10;
  uint64_t h = mix(seed ^ (uint64_t)i);
  double x;
  const int kind = (int)(i % 8);
  if (kind == 0) x = rnd(h, -40, -28);                                     // around TINY's exponent
  else if (kind == 1) x = __longlong_as_double(__double_as_longlong(-TINY) + (long long)(h % 65) - 32);
  else if (kind == 2) x = __longlong_as_double(__double_as_longlong(TINY) + (long long)(h % 65) - 32);
  else if (kind == 3) x = rnd(h, -1022, 1023);
  else if (kind == 4) x = __longlong_as_double((long long)h);               // any bit pattern (NaNs, subnormals)
  else {
    const double sp[8] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, -TINY, TINY};
    x = sp[h % 8];
  }
  const bool ge = above_neg_tiny(x, true), gt = above_neg_tiny(x, false);
  if (ge != (x >= -TINY) || ge != ((x + TINY) >= 0) || gt != (x > -TINY)) atomicAdd(bad, 1ull);
}

// lt_bits against a < b, floor_nonneg_bits against (int)floor(x) on
// [0, 2^31), double_of_nonneg against (double)i, zero_of against x * +0.0,
// on random values, neighbours of each other and the special values
__global__ void k_bits(uint64_t seed, long n, unsigned long long* bad) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t h1 = mix(seed ^ (uint64_t)i), h2 = mix(h1);
  const double sp[8] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 1.0, -1.0};
  double a, b;
  const int kind = (int)(i % 6);
  if (kind == 0) { a = rnd(h1, -60, 60); b = rnd(h2, -60, 60); }
  else if (kind == 1) { a = rnd(h1, -1022, 1023); b = __longlong_as_double(__double_as_longlong(a) + (long long)(h2 % 5) - 2); }
  else if (kind == 2) { a = __longlong_as_double((long long)h1); b = __longlong_as_double((long long)h2); }
  else if (kind == 3) { a = sp[h1 % 8]; b = sp[h2 % 8]; }
  else if (kind == 4) { a = sp[h1 % 8]; b = rnd(h2, -10, 10); }
  else { a = rnd(h1, -10, 10); b = -a; }
  if (lt_bits(a, b) != (a < b) || lt_bits(b, a) != (b < a)) atomicAdd(bad, 1ull);
  // cell indices: grid coordinates in [0, 2^31), integers and their neighbours
  const double x = (i & 1) ? fabs(rnd(h1, -30, 30)) * 0.5
                           : __longlong_as_double(__double_as_longlong((double)(h1 % 100000)) + (long long)(h2 % 3) - 1);
  if (x >= 0.0 && x < 2147483648.0 && floor_nonneg_bits(x) != (int)floor(x)) atomicAdd(bad + 1, 1ull);
  const int k = (int)(h2 & 0x7fffffff) >> (int)(h1 % 31);
  if (__double_as_longlong(double_of_nonneg(k)) != __double_as_longlong((double)k)) atomicAdd(bad + 2, 1ull);
  const double y = rnd(h2, -60, 60);
  if (__double_as_longlong(zero_of(y)) != __double_as_longlong(y * 0.0)) atomicAdd(bad + 3, 1ull);
}

__global__ void k_root4(uint64_t seed, long n, double* out) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t h = mix(seed ^ (uint64_t)i);
  // RKF's factor |tol h / (2 err)| spans a few decades around 1; also wide
  double x = (i & 1) ? fabs(rnd(h, -40, 40)) : fabs(rnd(h, -900, 900));
  out[2 * i] = x;
  out[2 * i + 1] = rn_root4(x);
}

int main(int argc, char** argv) {
  long n = argc > 1 ? atol(argv[1]) : (1L << 26);
  int reps = argc > 2 ? atoi(argv[2]) : 4;
  Out* d = nullptr;
  if (cudaMalloc(&d, sizeof(Out)) != cudaSuccess) return 2;
  cudaMemset(d, 0, sizeof(Out));
  for (int r = 0; r < reps; r++) k_div<<<(unsigned)((n + 255) / 256), 256>>>(0x1234567ull + 977ull * r, n, d);
  Out h;
  if (cudaMemcpy(&h, d, sizeof(Out), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  h.n_div = h.n_cvt = (unsigned long long)n * reps;
  unsigned long long* dt = nullptr, bad_tiny = 0;
  if (cudaMalloc(&dt, sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(dt, 0, sizeof(unsigned long long));
  k_tiny<<<(unsigned)((n + 255) / 256), 256>>>(0x5151ull, n, dt);
  if (cudaMemcpy(&bad_tiny, dt, sizeof(bad_tiny), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  cudaFree(dt);
  unsigned long long* db = nullptr, bad_bits[4] = {0, 0, 0, 0};
  if (cudaMalloc(&db, sizeof(bad_bits)) != cudaSuccess) return 2;
  cudaMemset(db, 0, sizeof(bad_bits));
  k_bits<<<(unsigned)((n + 255) / 256), 256>>>(0x7e57ull, n, db);
  if (cudaMemcpy(bad_bits, db, sizeof(bad_bits), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  cudaFree(db);
  printf("{\"n_div\": %llu, \"bad_div\": %llu, \"n_cvt\": %llu, \"bad_cvt\": %llu, \"n_tiny\": %ld, "
         "\"bad_tiny\": %llu, \"n_bits\": %ld, \"bad_lt\": %llu, \"bad_floor\": %llu, \"bad_i2d\": %llu, "
         "\"bad_zero\": %llu, \"first_bad\": [%.17g, %.17g, %d]}\n",
         h.n_div, h.bad_div, h.n_cvt, h.bad_cvt, n, bad_tiny, n, bad_bits[0], bad_bits[1], bad_bits[2],
         bad_bits[3], h.a, h.b, h.kind);
  cudaFree(d);
  if (argc > 3) {
    const long nr = 1L << 18;
    double* dr = nullptr;
    if (cudaMalloc(&dr, 16 * nr) != cudaSuccess) return 4;
    k_root4<<<(unsigned)(nr / 256), 256>>>(0xabcdefull, nr, dr);
    double* hr = (double*)malloc(16 * nr);
    if (!hr || cudaMemcpy(hr, dr, 16 * nr, cudaMemcpyDeviceToHost) != cudaSuccess) return 5;
    FILE* f = fopen(argv[3], "wb");
    if (!f || fwrite(hr, 16, nr, f) != (size_t)nr) return 6;
    fclose(f);
    free(hr);
    cudaFree(dr);
  }
  return 0;
}
