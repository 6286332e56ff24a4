// Checks the helpers of fvc_fpmath.cuh on the GPU: div_rn(a, b,
// rcp_for_div(b)) must equal CUDA's IEEE a / b bit for bit, and f32_trunc(x)
// must equal __double2float_rz(x), on many seeded operands from several
// distributions, and above_neg_tiny(x) must agree with the FP64 comparisons
// against -1e-10 it stands for (one line of counts on stdout).  With a file argument it
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
  int kind = (int)(h3 % 6);
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
  printf("{\"n_div\": %llu, \"bad_div\": %llu, \"n_cvt\": %llu, \"bad_cvt\": %llu, \"n_tiny\": %ld, "
         "\"bad_tiny\": %llu, \"first_bad\": [%.17g, %.17g, %d]}\n",
         h.n_div, h.bad_div, h.n_cvt, h.bad_cvt, n, bad_tiny, h.a, h.b, h.kind);
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
