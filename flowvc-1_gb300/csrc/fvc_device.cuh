// fvc_device.cuh -- device-side FP64 interpolation, point location and
// integrators of the flowVC advection path.
//
// Every expression keeps the operation order of the ompVC routine cited
// beside it, and this file is compiled with --fmad=false, so each multiply
// and add is rounded on its own exactly as gcc -O3 does on x86-64: element
// ids, exit flags and positions come out bit-identical to ompVC.
//
// Layout in HBM (see fvc_state.h):
//   elements  int4 pairs {nodes, neighbours}   32 B per element, one sector
//   geometry  per element the natural-coordinate map (a11..a33, V, x0, y0,
//             z0) precomputed once from the node coordinates; recomputing
//             it gives the same doubles, so precomputing changes no bit
//   frames    double4_32a (u, v, w, 0) per node, one 32 B sector per gather
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fvc_fpmath.cuh"
#include "fvc_state.h"

namespace fvc {

#define FVC_TINY 1.0e-10

// RN(1/6) and RN(1/13), for the RK4 update's division by 6 and RKF's stage
// time 12h/13 through div_rn
constexpr double kRcp6 = 1.0 / 6.0;
constexpr double kRcp13 = 1.0 / 13.0;

struct Pt {
  double X[3];
  double V[3];
  int eid;
  int left;
  double ldt;
};

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dsign(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

// TestOutsideDomain, ompVC/velocity.c:654-669 (the comparisons on the bit
// patterns, off the FP64 pipe, with the FP64 comparisons' outcomes)
__device__ __forceinline__ int outside_domain(const DevMesh& m, const double X[3]) {
  if (lt_bits(X[0], m.bounds[0] - FVC_TINY) || lt_bits(m.bounds[1] + FVC_TINY, X[0])) return 1;
  if (lt_bits(X[1], m.bounds[2] - FVC_TINY) || lt_bits(m.bounds[3] + FVC_TINY, X[1])) return 1;
  if (lt_bits(X[2], m.bounds[4] - FVC_TINY) || lt_bits(m.bounds[5] + FVC_TINY, X[2])) return 1;
  return 0;
}

// ------------------------------------------------------------------ Cartesian

// One axis of TestOutsideCartVelDomain: (int)floor(f) >= 0 and (int)ceil(f)
// <= last hold exactly when 0 <= f <= last (last an integer); a NaN is
// outside, as the x86-64 conversion (INT_MIN) makes it for ompVC.  Decided
// on the bit patterns.
__device__ __forceinline__ bool cell_index_ok(double f, int last) {
  long long kf, kl;
  if (!bits_of(f, kf)) return false;
  bits_of(double_of_nonneg(last), kl);
  return kf >= 0 && kf <= kl;
}

// TestOutsideCartVelDomain, ompVC/velocity.c:624-651: the point's grid
// coordinates f = (X - min) / delta and whether the cell they index lies in
// the grid.  GetVelocity_Cartesian (ompVC/velocity.c:257-457) divides the
// same differences by the same deltas again; the engine keeps the quotients.
template <int DIMS>
__device__ __forceinline__ bool cart_coords(const DevMesh& m, const double X[3], double f[3]) {
  f[0] = div_rn(X[0] - m.xmin, m.dx, m.rdx);
  f[1] = div_rn(X[1] - m.ymin, m.dy, m.rdy);
  f[2] = DIMS == 3 ? div_rn(X[2] - m.zmin, m.dz, m.rdz) : 0.0;
  return cell_index_ok(f[0], m.xres - 1) && cell_index_ok(f[1], m.yres - 1) &&
         (DIMS != 3 || cell_index_ok(f[2], m.zres - 1));
}
template <int DIMS>
__device__ __forceinline__ int outside_cart_grid(const DevMesh& m, const double X[3]) {
  double f[3];
  return !cart_coords<DIMS>(m, X, f);
}

// one 32-byte node record as two read-only 16-byte loads
__device__ __forceinline__ double4_32a ldf(const double4_32a* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 a = __ldg(q), b = __ldg(q + 1);
  return make_double4_32a(a.x, a.y, b.x, b.y);
}

// GetVelocity_Cartesian, ompVC/velocity.c:257-457.  The 16 space-time
// weights and the summation order f0000*V16 + ... + f1111*V1 are the
// reference's.  In 2D the reference's zloc is 0, so the eight weights with a
// zloc factor are exactly zero and adding their zero products leaves every
// partial sum unchanged; the 2D branch skips them.
// tloc of a query time (ompVC/velocity.c:275-277): from the slot table when
// the query is a tabulated stage time, else computed and range-checked.
// The times are compared with integer instructions, off the FP64 pipe: equal
// bit patterns, or both zero (+0 == -0, as the FP64 comparison has it).
__device__ __forceinline__ bool slot_hit(const DevWindow& w, int slot, double tq) {
  if (slot < 0 || slot >= w.nslots) return false;
  const unsigned long long a = (unsigned long long)__double_as_longlong(w.tq[slot]);
  const unsigned long long b = (unsigned long long)__double_as_longlong(tq);
  return a == b || ((a | b) << 1) == 0ull;
}
__device__ __forceinline__ int get_tloc(const DevWindow& w, int slot, double tq, double& tloc) {
  if (slot_hit(w, slot, tq)) {
    tloc = w.tl[slot];
    return 0;
  }
  tloc = div_rn(tq - w.tmin, w.tmax - w.tmin, w.rspan);
  if ((tloc > 1 + FVC_TINY) || (tloc < 0 - FVC_TINY)) return PT_ERR_TLOC;
  return 0;
}

template <int DIMS>
__device__ __forceinline__ int vel_cart(const DevMesh& m, const DevWindow& w, double tq, int tslot,
                                        const double X[3], int& left, double out[3]) {
  double f[3];
  if (!cart_coords<DIMS>(m, X, f)) {
    out[0] = out[1] = out[2] = 0.0;
    left = 1;
    return 0;
  }
  double tloc;
  if (get_tloc(w, tslot, tq, tloc)) return PT_ERR_TLOC;
  // cell indices (int)floor(f) of a point inside the grid, and the offsets
  // X - min - i delta with i converted exactly, on integer instructions
  double xloc, yloc;
  int i = floor_nonneg_bits(f[0]);
  if (i == (m.xres - 1)) {
    i = m.xres - 2;
    xloc = 1.0;
  } else
    xloc = div_rn(X[0] - m.xmin - double_of_nonneg(i) * m.dx, m.dx, m.rdx);
  int j = floor_nonneg_bits(f[1]);
  if (j == (m.yres - 1)) {
    j = m.yres - 2;
    yloc = 1.0;
  } else
    yloc = div_rn(X[1] - m.ymin - double_of_nonneg(j) * m.dy, m.dy, m.rdy);
  const long nx = m.xres, ny = m.yres;
  const double4_32a* A = w.f0;
  const double4_32a* B = w.f1;
  if (DIMS == 3) {
    double zloc;
    int k = floor_nonneg_bits(f[2]);
    if (k == (m.zres - 1)) {
      k = m.zres - 2;
      zloc = 1.0;
    } else
      zloc = div_rn(X[2] - m.zmin - double_of_nonneg(k) * m.dz, m.dz, m.rdz);
    double V1 = (tloc) * (xloc) * (yloc) * (zloc);
    double V2 = (tloc) * (xloc) * (yloc) * (1 - zloc);
    double V3 = (tloc) * (xloc) * (1 - yloc) * (zloc);
    double V4 = (tloc) * (xloc) * (1 - yloc) * (1 - zloc);
    double V5 = (tloc) * (1 - xloc) * (yloc) * (zloc);
    double V6 = (tloc) * (1 - xloc) * (yloc) * (1 - zloc);
    double V7 = (tloc) * (1 - xloc) * (1 - yloc) * (zloc);
    double V8 = (tloc) * (1 - xloc) * (1 - yloc) * (1 - zloc);
    double V9 = (1 - tloc) * (xloc) * (yloc) * (zloc);
    double V10 = (1 - tloc) * (xloc) * (yloc) * (1 - zloc);
    double V11 = (1 - tloc) * (xloc) * (1 - yloc) * (zloc);
    double V12 = (1 - tloc) * (xloc) * (1 - yloc) * (1 - zloc);
    double V13 = (1 - tloc) * (1 - xloc) * (yloc) * (zloc);
    double V14 = (1 - tloc) * (1 - xloc) * (yloc) * (1 - zloc);
    double V15 = (1 - tloc) * (1 - xloc) * (1 - yloc) * (zloc);
    double V16 = (1 - tloc) * (1 - xloc) * (1 - yloc) * (1 - zloc);
    long o000 = ((long)k * ny + j) * nx + i;
    long o100 = o000 + 1, o010 = o000 + nx, o110 = o000 + nx + 1;
    long sk = nx * ny;
    double4_32a a000 = ldf(A + o000), a001 = ldf(A + o000 + sk), a010 = ldf(A + o010), a011 = ldf(A + o010 + sk);
    double4_32a a100 = ldf(A + o100), a101 = ldf(A + o100 + sk), a110 = ldf(A + o110), a111 = ldf(A + o110 + sk);
    double4_32a b000 = ldf(B + o000), b001 = ldf(B + o000 + sk), b010 = ldf(B + o010), b011 = ldf(B + o010 + sk);
    double4_32a b100 = ldf(B + o100), b101 = ldf(B + o100 + sk), b110 = ldf(B + o110), b111 = ldf(B + o110 + sk);
#define FVC_CSUM(c)                                                                                \
  (a000.c * V16 + a001.c * V15 + a010.c * V14 + a011.c * V13 + a100.c * V12 + a101.c * V11 +       \
   a110.c * V10 + a111.c * V9 + b000.c * V8 + b001.c * V7 + b010.c * V6 + b011.c * V5 +            \
   b100.c * V4 + b101.c * V3 + b110.c * V2 + b111.c * V1)
    out[0] = FVC_CSUM(x);
    out[1] = FVC_CSUM(y);
    out[2] = FVC_CSUM(z);
#undef FVC_CSUM
  } else {
    // zloc = 0: (1 - zloc) == 1 exactly, so V2 == tloc*xloc*yloc etc.
    double V2 = (tloc) * (xloc) * (yloc);
    double V4 = (tloc) * (xloc) * (1 - yloc);
    double V6 = (tloc) * (1 - xloc) * (yloc);
    double V8 = (tloc) * (1 - xloc) * (1 - yloc);
    double V10 = (1 - tloc) * (xloc) * (yloc);
    double V12 = (1 - tloc) * (xloc) * (1 - yloc);
    double V14 = (1 - tloc) * (1 - xloc) * (yloc);
    double V16 = (1 - tloc) * (1 - xloc) * (1 - yloc);
    long o000 = (long)j * nx + i;
    double4_32a a000 = ldf(A + o000), a010 = ldf(A + o000 + nx), a100 = ldf(A + o000 + 1), a110 = ldf(A + o000 + nx + 1);
    double4_32a b000 = ldf(B + o000), b010 = ldf(B + o000 + nx), b100 = ldf(B + o000 + 1), b110 = ldf(B + o000 + nx + 1);
#define FVC_CSUM2(c)                                                                               \
  (a000.c * V16 + a010.c * V14 + a100.c * V12 + a110.c * V10 + b000.c * V8 + b010.c * V6 +         \
   b100.c * V4 + b110.c * V2)
    out[0] = FVC_CSUM2(x);
    out[1] = FVC_CSUM2(y);
    out[2] = w.wz ? 0.0 : FVC_CSUM2(z);  // the w sum of all-zero frames is +0.0
#undef FVC_CSUM2
  }
  return 0;
}

// --------------------------------------------------------------- unstructured

// One element's record: the natural-coordinate map precomputed from its node
// coordinates (ompVC/velocity.c:497-510 and 529-535; recomputing it gives the
// same doubles) and its node ids.
//   3D, 16 doubles: a11 a12 a13 a21 a22 a23 a31 a32 a33 V x0 y0 z0 rV | nodes
//   2D, 12 doubles: a11 a12 a21 a22 V x0 y0 rV | nodes | -
// rV is the reciprocal div_rn uses to divide by V.
template <int DIMS>
struct Geo {
  double a[DIMS == 3 ? 9 : 4];
  double V, rV, x0, y0, z0;
  int4 nd;
};

template <int DIMS>
__device__ __forceinline__ void load_geo(const DevMesh& m, int e, Geo<DIMS>& g) {
  if (DIMS == 3) {
    const double2* p = reinterpret_cast<const double2*>(m.geom + (long)e * 16);
    double2 g0 = __ldg(p + 0), g1 = __ldg(p + 1), g2 = __ldg(p + 2), g3 = __ldg(p + 3);
    double2 g4 = __ldg(p + 4), g5 = __ldg(p + 5), g6 = __ldg(p + 6);
    g.nd = __ldg(reinterpret_cast<const int4*>(p + 7));
    g.a[0] = g0.x; g.a[1] = g0.y; g.a[2] = g1.x; g.a[3] = g1.y; g.a[4] = g2.x;
    g.a[5] = g2.y; g.a[6] = g3.x; g.a[7] = g3.y; g.a[8] = g4.x;
    g.V = g4.y; g.x0 = g5.x; g.y0 = g5.y; g.z0 = g6.x; g.rV = g6.y;
  } else {
    const double2* p = reinterpret_cast<const double2*>(m.geom + (long)e * 12);
    double2 g0 = __ldg(p + 0), g1 = __ldg(p + 1), g2 = __ldg(p + 2), g3 = __ldg(p + 3);
    g.nd = __ldg(reinterpret_cast<const int4*>(p + 4));
    g.a[0] = g0.x; g.a[1] = g0.y; g.a[2] = g1.x; g.a[3] = g1.y;
    g.V = g2.x; g.x0 = g2.y; g.y0 = g3.x; g.z0 = 0.0; g.rV = g3.y;
  }
}

// Natural coordinates of X (ompVC/velocity.c:512-517 and 537-542, the same in
// ompVC/mesh.c:542-547 and 587-591).
template <int DIMS>
__device__ __forceinline__ void natural_coords(const Geo<DIMS>& g, const double X[3], double& r, double& s,
                                               double& t, double& wv) {
  if (DIMS == 3) {
    double dx = X[0] - g.x0, dy = X[1] - g.y0, dz = X[2] - g.z0;
    r = div_rn(g.a[0] * dx + g.a[1] * dy + g.a[2] * dz, g.V, g.rV);
    s = div_rn(g.a[3] * dx + g.a[4] * dy + g.a[5] * dz, g.V, g.rV);
    t = div_rn(g.a[6] * dx + g.a[7] * dy + g.a[8] * dz, g.V, g.rV);
    wv = 1 - r - s - t;
  } else {
    double dx = X[0] - g.x0, dy = X[1] - g.y0;
    r = div_rn(g.a[0] * dx + g.a[1] * dy, g.V, g.rV);
    s = div_rn(g.a[2] * dx + g.a[3] * dy, g.V, g.rV);
    t = 0;
    wv = 1 - r - s;
  }
}

// d, the coordinates' minimum, as the reference forms it
template <int DIMS>
__device__ __forceinline__ double natural_min(double r, double s, double t, double wv) {
  return DIMS == 3 ? dmin(r, dmin(s, dmin(t, wv))) : dmin(r, dmin(s, wv));
}

// Natural coordinates of X; returns d, their minimum.
template <int DIMS>
__device__ __forceinline__ double natural_from(const Geo<DIMS>& g, const double X[3], double& r,
                                               double& s, double& t, double& wv) {
  natural_coords<DIMS>(g, X, r, s, t, wv);
  return natural_min<DIMS>(r, s, t, wv);
}

// The containment tests of the walk on the coordinates themselves: the
// reference's (d + TINY) >= 0 (vel_rule) or d > -TINY, with d the minimum.
// For a finite d, d + TINY rounds to a negative number exactly when
// d < -TINY (within a factor two of TINY the sum is exact), so the first
// test is d >= -TINY; a NaN coordinate makes wv, and so d, NaN, and fails
// both forms.  Hence: every coordinate >= -TINY (> -TINY).
template <int DIMS>
__device__ __forceinline__ bool inside_tiny(double r, double s, double t, double wv, bool vel_rule) {
  return above_neg_tiny(r, vel_rule) & above_neg_tiny(s, vel_rule) & (DIMS == 2 || above_neg_tiny(t, vel_rule)) &
         above_neg_tiny(wv, vel_rule);
}

template <int DIMS>
__device__ __forceinline__ double natural(const DevMesh& m, int e, const double X[3], double& r,
                                          double& s, double& t, double& wv) {
  Geo<DIMS> g;
  load_geo<DIMS>(m, e, g);
  return natural_from<DIMS>(g, X, r, s, t, wv);
}

// Natural coordinates computed by the last point location at the current
// position: a walk that tests the same element at the same position gets the
// same doubles, so the first velocity evaluation after a locate reuses them.
struct NatCache {
  int e;
  int4 nd;
  double r, s, t, w;
};

// The node velocities a tabulated stage evaluation interpolates, gathered
// right after the element record so the loads overlap the containment test.
template <int DIMS>
struct NodeVel {
  double u[DIMS == 3 ? 4 : 3], v[DIMS == 3 ? 4 : 3], w[DIMS == 3 ? 4 : 3];
};

template <int DIMS>
__device__ __forceinline__ void load_slot_nodes(const DevWindow& w, int tslot, int4 nd, NodeVel<DIMS>& nv) {
  const int ids[4] = {nd.x, nd.y, nd.z, nd.w};
  const double* F = reinterpret_cast<const double*>(w.vt + (long)tslot * w.vt_stride);
#pragma unroll
  for (int c = 0; c < (DIMS == 3 ? 4 : 3); c++) {
    const double* q = F + 4L * ids[c];
    double2 uv = __ldg(reinterpret_cast<const double2*>(q));
    nv.u[c] = uv.x;
    nv.v[c] = uv.y;
    nv.w[c] = DIMS == 3 ? __ldg(q + 2) : 0.0;
  }
}

// FP32 pre-check of one walk hop.  The reference tests element e with
// natural coordinates computed in FP64 and, when the point is outside by more
// than TINY, steps through the face of the first coordinate within TINY of
// the minimum (ompVC/velocity.c:545-609, mesh.c:549-560).  When the FP32
// coordinates put the point outside by more than their error bound, with one
// coordinate below all others by more than that bound, the FP64 test fails
// and selects that face too, so the hop is taken without the FP64 solve.
// Returns the face slot; -2 when every FP32 coordinate exceeds twice the
// bound, so that every FP64 coordinate is positive and the FP64 test passes
// (callers that need only the element, not its coordinates, stop there);
// or -1 when the FP64 test must decide.
//
// The FP32 offsets are Xf - x0f, with Xf the position truncated to FP32
// (f32_trunc, no FP64 instruction) once per walk and x0f the node rounded to
// FP32.  Per component the offset then errs by at most
//   E = 2^-22 (|Xf| + |x0f| + |dx|) + 2^-125,
// and each coordinate (and 1 - r - s - t) by at most A E, with A = sum |a_ij|
// / |V| stored per element.  The FP32 map, products, sums and 1/V add at most
// 1e-6 (1 + S), S = sum |a_ij dx_j / V|; tol is the sum of the two.
struct PosF {
  float x[3];
  float m;  // max |x_j|
};

__device__ __forceinline__ PosF pos_f32(const double X[3]) {
  PosF P;
  P.x[0] = f32_trunc(X[0]);
  P.x[1] = f32_trunc(X[1]);
  P.x[2] = f32_trunc(X[2]);
  P.m = fmaxf(fabsf(P.x[0]), fmaxf(fabsf(P.x[1]), fabsf(P.x[2])));
  return P;
}

template <int DIMS>
__device__ __forceinline__ int quick_hop(const DevMesh& m, int e, const PosF& P) {
  const float* q = m.geo32 + (long)e * 16;
  if (DIMS == 3) {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    float4 q2 = __ldg(reinterpret_cast<const float4*>(q + 8));
    float2 q3 = __ldg(reinterpret_cast<const float2*>(q + 12));
    // q2 = (a33, 1/V, x0, y0), q3 = (z0, A)
    float dx = P.x[0] - q2.z, dy = P.x[1] - q2.w, dz = P.x[2] - q3.x;
    float iv = q2.y;
    float r0 = q0.x * dx, r1 = q0.y * dy, r2 = q0.z * dz;
    float s0 = q0.w * dx, s1 = q1.x * dy, s2 = q1.y * dz;
    float t0 = q1.z * dx, t1 = q1.w * dy, t2 = q2.x * dz;
    float r = (r0 + r1 + r2) * iv, s = (s0 + s1 + s2) * iv, t = (t0 + t1 + t2) * iv;
    float S = (fabsf(r0) + fabsf(r1) + fabsf(r2) + fabsf(s0) + fabsf(s1) + fabsf(s2) + fabsf(t0) + fabsf(t1) +
               fabsf(t2)) * fabsf(iv);
    float E = 2.4e-7f * (P.m + fmaxf(fabsf(q2.z), fmaxf(fabsf(q2.w), fabsf(q3.x))) +
                         fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)))) + 1e-37f;
    float tol = 1e-6f * (1.0f + S) + 1.01f * q3.y * E;
    float w = 1.0f - r - s - t;
    float c[4] = {r, s, t, w};
    int k = 0;
    float d = c[0];
#pragma unroll
    for (int j = 1; j < 4; j++)
      if (c[j] < d) { d = c[j]; k = j; }
    float second = 3.0e38f;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (j != k) second = fminf(second, c[j]);
    if (d > 2.0f * tol) return -2;
    if (!(d < -(1e-10f + 2.0f * tol)) || !(second - d > 1e-10f + 4.0f * tol)) return -1;
    return k;
  } else {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    // q0 = (a11, a12, a21, a22), q1 = (1/V, x0, y0, A)
    float dx = P.x[0] - q1.y, dy = P.x[1] - q1.z;
    float iv = q1.x;
    float r0 = q0.x * dx, r1 = q0.y * dy, s0 = q0.z * dx, s1 = q0.w * dy;
    float r = (r0 + r1) * iv, s = (s0 + s1) * iv;
    float S = (fabsf(r0) + fabsf(r1) + fabsf(s0) + fabsf(s1)) * fabsf(iv);
    float E = 2.4e-7f * (fmaxf(fabsf(P.x[0]), fabsf(P.x[1])) + fmaxf(fabsf(q1.y), fabsf(q1.z)) +
                         fmaxf(fabsf(dx), fabsf(dy))) + 1e-37f;
    float tol = 1e-6f * (1.0f + S) + 1.01f * q1.w * E;
    float w = 1.0f - r - s;
    float c[3] = {r, s, w};
    int k = 0;
    float d = c[0];
#pragma unroll
    for (int j = 1; j < 3; j++)
      if (c[j] < d) { d = c[j]; k = j; }
    float second = 3.0e38f;
#pragma unroll
    for (int j = 0; j < 3; j++)
      if (j != k) second = fminf(second, c[j]);
    if (d > 2.0f * tol) return -2;
    if (!(d < -(1e-10f + 2.0f * tol)) || !(second - d > 1e-10f + 4.0f * tol)) return -1;
    return k;  // 2D slots: 0 r, 1 s, 2 (1 - r - s)
  }
}

__device__ __forceinline__ int pick(int4 nb, int slot) {
  return slot == 0 ? nb.x : slot == 1 ? nb.y : slot == 2 ? nb.z : nb.w;
}
__device__ __forceinline__ int4 neighbours(const DevMesh& m, int e) { return __ldg(m.elem + 2 * (long)e + 1); }
__device__ __forceinline__ int neighbour(const DevMesh& m, int e, int slot) { return pick(neighbours(m, e), slot); }

// The reference's walk (GetVelocity_Unstructured's loop, ompVC/velocity.c:
// 480-619, with vel_rule; Get_Element_Local_Search, ompVC/mesh.c:510-609,
// without): hops the FP32 pre-check can decide are taken first, then the
// FP64 solve decides at the element reached, so the lanes of a warp run the
// expensive step together.  An element's neighbours are loaded together
// with its records, so a hop costs one memory round trip.  Returns 0 with
// the element's coordinates, or 1 when the walk stops: eid = -1 when it left
// through a boundary face, EID_FAULT when it failed.
//
// nc (velocity walks only): the last locate's element and coordinates at
// this same position.  When the walk reaches that element, the FP64 solve
// there would recompute the cached doubles and pass (the locate's d > -TINY
// implies (d + TINY) >= 0), so the cache stands in for it.  An RK4 step's
// first stage walks from its own hint, which lags the located element
// whenever the previous step crossed a face: without this those walks
// repeated the locate's solve, lane by lane.
//
// coords = false (a locate that wants only the element): an element the
// FP32 pre-check puts inside beyond its error bound ends the walk without
// the FP64 solve (the solve would pass); r, s, t, wv and nd are then unset.
template <int DIMS>
__device__ __forceinline__ int walk(const DevMesh& m, const double X[3], int& eid, bool vel_rule, double& r,
                                    double& s, double& t, double& wv, int4& nd, const NatCache* nc = nullptr,
                                    bool coords = true) {
  const PosF P = pos_f32(X);
  int4 nb = neighbours(m, eid);
  for (int hop = 0; hop < m.max_hops;) {
    int qs;
    while (hop < m.max_hops && (qs = quick_hop<DIMS>(m, eid, P)) >= 0) {
      eid = pick(nb, qs);
      hop++;
      if (eid == -1) return 1;
      nb = neighbours(m, eid);
    }
    if (hop >= m.max_hops) break;
    if (qs == -2 && !coords) return 0;
    if (nc && eid == nc->e) {
      r = nc->r;
      s = nc->s;
      t = nc->t;
      wv = nc->w;
      nd = nc->nd;
      return 0;
    }
    Geo<DIMS> g;
    load_geo<DIMS>(m, eid, g);
    natural_coords<DIMS>(g, X, r, s, t, wv);
    nd = g.nd;
    if (inside_tiny<DIMS>(r, s, t, wv, vel_rule)) return 0;
    // the point is outside: the reference's face choice on d
    const double d = natural_min<DIMS>(r, s, t, wv);
    int slot;
    if (fabs(r - d) < FVC_TINY) slot = 0;
    else if (fabs(s - d) < FVC_TINY) slot = 1;
    else if (DIMS == 3 && fabs(t - d) < FVC_TINY) slot = 2;
    else if (fabs(wv - d) < FVC_TINY) slot = DIMS == 3 ? 3 : 2;
    else break;  // "Indeterminate neighbor"
    eid = pick(nb, slot);
    hop++;
    if (eid == -1) return 1;
    nb = neighbours(m, eid);
  }
  eid = EID_FAULT;
  return 1;
}

// PT_ERR_WALK for the element id a failed walk leaves behind
__device__ __forceinline__ int walk_fault(int eid) { return eid == EID_FAULT ? PT_ERR_WALK : 0; }

// GetVelocity_Unstructured, ompVC/velocity.c:459-621: walk from eid until the
// element passes (d + TINY) >= 0, then P1 in space and linear in time.
template <int DIMS>
__device__ __forceinline__ int vel_unstruct(const DevMesh& m, const DevWindow& w, double tq, int tslot,
                                            const double X[3], int& eid, int& left, double out[3],
                                            const NatCache* nc) {
  if (eid < 0 || eid >= m.nelem) return PT_ERR_WALK;
  const bool tab = slot_hit(w, tslot, tq);
  double tloc = 0.0;
  if (!tab) {
    tloc = div_rn(tq - w.tmin, w.tmax - w.tmin, w.rspan);
    if ((tloc > 1 + FVC_TINY) || (tloc < 0 - FVC_TINY)) return PT_ERR_TLOC;
  }
  double r, s, t, wv;
  int4 nd;
  if (nc && nc->e == eid) {
    // the last locate tested this element at this position (d > -TINY)
    nd = nc->nd;
    r = nc->r;
    s = nc->s;
    t = nc->t;
    wv = nc->w;
  } else {
    if (walk<DIMS>(m, X, eid, true, r, s, t, wv, nd, nc)) {
      // out of the domain, or a failed walk (eid = EID_FAULT): the point stops
      left = 1;
      out[0] = out[1] = out[2] = 0.0;
      return 0;
    }
  }
  NodeVel<DIMS> nv;
  if (tab) {
    load_slot_nodes<DIMS>(w, tslot, nd, nv);
  } else {
    const int ids[4] = {nd.x, nd.y, nd.z, nd.w};
#pragma unroll
    for (int c = 0; c < (DIMS == 3 ? 4 : 3); c++) {
      double4_32a a = ldf(w.f0 + ids[c]), b = ldf(w.f1 + ids[c]);
      nv.u[c] = (1 - tloc) * a.x + tloc * b.x;
      nv.v[c] = (1 - tloc) * a.y + tloc * b.y;
      nv.w[c] = (1 - tloc) * a.z + tloc * b.z;
    }
  }
  if (DIMS == 3) {
    out[0] = nv.u[0] + (nv.u[1] - nv.u[0]) * fabs(r) + (nv.u[2] - nv.u[0]) * fabs(s) + (nv.u[3] - nv.u[0]) * fabs(t);
    out[1] = nv.v[0] + (nv.v[1] - nv.v[0]) * fabs(r) + (nv.v[2] - nv.v[0]) * fabs(s) + (nv.v[3] - nv.v[0]) * fabs(t);
    out[2] = nv.w[0] + (nv.w[1] - nv.w[0]) * fabs(r) + (nv.w[2] - nv.w[0]) * fabs(s) + (nv.w[3] - nv.w[0]) * fabs(t);
  } else {
    out[0] = nv.u[0] + (nv.u[1] - nv.u[0]) * fabs(r) + (nv.u[2] - nv.u[0]) * fabs(s);
    out[1] = nv.v[0] + (nv.v[1] - nv.v[0]) * fabs(r) + (nv.v[2] - nv.v[0]) * fabs(s);
    out[2] = 0.0;
  }
  return 0;
}

// Get_Element_Local_Search, ompVC/mesh.c:496-611: containment d > -TINY;
// returns -1 when the walk leaves through a boundary face (or guess < 0) and
// EID_FAULT when it fails.  On success nc (if given) receives the natural
// coordinates of the element found.
template <int DIMS>
__device__ __forceinline__ int locate_walk(const DevMesh& m, const double X[3], int guess, int& err,
                                           NatCache* nc = nullptr) {
  if (nc) nc->e = -1;
  if (guess < 0) return -1;
  if (guess >= m.nelem) {
    err |= PT_ERR_WALK;
    return -1;
  }
  double r, s, t, wv;
  int4 nd;
  if (walk<DIMS>(m, X, guess, false, r, s, t, wv, nd, nullptr, nc != nullptr))
    return guess == EID_FAULT ? EID_FAULT : -1;
  if (nc) {
    nc->e = guess;
    nc->nd = nd;
    nc->r = r;
    nc->s = s;
    nc->t = t;
    nc->w = wv;
  }
  return guess;
}

// locate_walk for a one-off locate: a failed walk is reported in err and
// answers -1
template <int DIMS>
__device__ __forceinline__ int locate_once(const DevMesh& m, const double X[3], int guess, int& err) {
  const int r = locate_walk<DIMS>(m, X, guess, err);
  if (r != EID_FAULT) return r;
  err |= PT_ERR_WALK;
  return -1;
}

// Containment test of one element (the predicate of
// Get_Element_Global_Search, ompVC/mesh.c:360 and 389).
template <int DIMS>
__device__ __forceinline__ bool contains(const DevMesh& m, int e, const double X[3]) {
  double r, s, t, wv;
  return natural<DIMS>(m, e, X, r, s, t, wv) > -FVC_TINY;
}

// Get_Element_Global_Search (ompVC/mesh.c:304-398): lowest element id whose
// containment test d > -TINY passes, from the point's bucket.  Candidates the
// walk's FP32 pre-check puts outside beyond its error bound are skipped
// without the FP64 test (they would fail it), and one it puts inside beyond
// that bound is taken without it (it would pass).
template <int DIMS>
__device__ __forceinline__ int global_find(const DevMesh& m, const BucketGrid& g, const double X[3]) {
  int c[3];
  for (int a = 0; a < 3; a++) {
    if (a == 2 && DIMS == 2) { c[a] = 0; continue; }
    double f = (X[a] - g.lo[a]) * g.inv[a];
    if (!(f >= 0.0) || f >= (double)g.n[a]) return -1;
    c[a] = min(g.n[a] - 1, (int)f);
  }
  long cell = ((long)c[2] * g.n[1] + c[1]) * g.n[0] + c[0];
  int b = __ldg(g.start + cell), e = __ldg(g.start + cell + 1);
  const PosF P = pos_f32(X);
  for (int i = b; i < e; i++) {
    int el = __ldg(g.ids + i);
    const int qs = quick_hop<DIMS>(m, el, P);
    if (qs >= 0) continue;
    if (qs == -2 || contains<DIMS>(m, el, X)) return el;
  }
  return -1;
}


// GetVelocity dispatch, ompVC/velocity.c:236-247.  tslot names the stage
// time in the call's table (-1: none); nc the last locate's coordinates.
template <int DIMS, int MESH>
__device__ __forceinline__ int velocity(const DevMesh& m, const DevWindow& w, double tq, int tslot,
                                        const double X[3], int& eid, int& left, double out[3],
                                        const NatCache* nc = nullptr) {
  if (MESH == 0) return vel_cart<DIMS>(m, w, tq, tslot, X, left, out);
  return vel_unstruct<DIMS>(m, w, tq, tslot, X, eid, left, out, nc);
}

// ComputeExposureTime, ompVC/exposuretime.c:110-172: credits a step of
// length h from X0 to X1 (X1 in element e1) to the elements it crossed.  If
// both ends lie in one element the whole step goes to it; otherwise the
// straight path is cut into substeps - 1 pieces, each credited with
// h / (substeps - 1) to the element holding its end point (walk from the
// previous piece's element, global search if the walk leaves the mesh;
// pieces outside the mesh are skipped, as ompVC skips them with a warning),
// and every change of element counts an encounter.  Accumulated with
// atomics: the sums' rounding depends on the order the GPU adds them in.
template <int DIMS>
__device__ __noinline__ void cet_step(const DevMesh& m, const CetDev& c, const double* X0, const double* X1,
                                      int e1, double h, int* err) {
  int e0 = locate_once<DIMS>(m, X0, e1, *err);
  if (e0 < 0) {
    e0 = global_find<DIMS>(m, c.g, X0);
    if (e0 < 0) {
      *err |= PT_ERR_CET;  // ompVC: "Point X0 ... appears to be outside of velocity domain"
      return;
    }
  }
  if (e0 == e1) {
    atomicAdd(c.sum + e0, h);
    return;
  }
  int last = e0;
  for (int s = 1; s < c.substeps; s++) {
    const double a = ((double)s) / ((double)(c.substeps - 1));
    double Xt[3];
#pragma unroll
    for (int q = 0; q < 3; q++) Xt[q] = (1 - a) * X0[q] + a * X1[q];
    int et = locate_once<DIMS>(m, Xt, last, *err);
    if (et < 0) {
      et = global_find<DIMS>(m, c.g, Xt);
      if (et < 0) continue;
    }
    atomicAdd(c.sum + et, h / (c.substeps - 1));
    if (et != last) {
      atomicAdd(c.enc + et, 1);
      last = et;
    }
  }
}

// ---------------------------------------------------------------- integrators
//
// Step k of a call evaluates at the stage times of slots 2k (tc), 2k+1
// (tc + h/2) and 2k+2 (tc + h); the slot is only a hint, checked against the
// time it names before its table entry is used.

// velocity at the accepted position for extrapolation (Int_Extrapolate),
// kept out of line: it is off the common path
template <int DIMS, int MESH>
__device__ __noinline__ int velocity_cold(const DevMesh& m, const DevWindow& w, double tq, int tslot,
                                          const double* X, int* eid, int* left, double* out) {
  const int r = velocity<DIMS, MESH>(m, w, tq, tslot, X, *eid, *left, out);
  return MESH == 1 ? r | walk_fault(*eid) : r;
}

// Euler, ompVC/integration.c:222-311
template <int DIMS, int MESH, bool CET = false>
__device__ __noinline__ double euler(const DevMesh& m, const DevWindow& w, const DevInteg& in,
                                     Pt& p, double tstart, double tend, unsigned& steps, int& err,
                                     const CetDev* cet = nullptr, const RecOut* rec = nullptr) {
  double tc = tstart, h = dsign(in.h, tend - tstart), ve[3];
  NatCache nc;
  nc.e = -1;
  int k = 0;
  while ((tc - tend) * (tend - tstart) < 0.0) {
    if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = dsign(tend - tc, tend - tstart);
    if ((err |= velocity<DIMS, MESH>(m, w, tc, 2 * k, p.X, p.eid, p.left, ve, &nc) |
                (MESH == 1 ? walk_fault(p.eid) : 0)))
      return tend;
    p.X[0] = p.X[0] + h * ve[0];
    p.X[1] = p.X[1] + h * ve[1];
    p.X[2] = p.X[2] + h * ve[2];
    tc = tc + h;
    k++;
    if (MESH == 1) p.eid = locate_walk<DIMS>(m, p.X, p.eid, err, &nc);
    if (err) return tend;
    if ((MESH == 0 && outside_domain(m, p.X)) || (MESH == 1 && p.eid < 0)) {
      p.left = 1;
      p.ldt = tc - h;
      p.X[0] = p.X[0] - h * ve[0];
      p.X[1] = p.X[1] - h * ve[1];
      p.X[2] = p.X[2] - h * ve[2];
      return p.ldt;
    }
    steps++;
    if (rec && k <= rec->max) {
      double* o = rec->base + (long)(k - 1) * rec->stride;
      o[0] = p.X[0];
      o[1] = p.X[1];
      o[2] = p.X[2];
    }
    if (in.extrapolate && (err |= velocity_cold<DIMS, MESH>(m, w, tc, 2 * k, p.X, &p.eid, &p.left, p.V)))
      return tend;
    if (CET) {  // ompVC/integration.c:277-299
      const double X0[3] = {p.X[0] - h * ve[0], p.X[1] - h * ve[1], p.X[2] - h * ve[2]};
      cet_step<DIMS>(m, *cet, X0, p.X, p.eid, h, &err);
      if (err) return tend;
    }
  }
  return tend;
}

// The four stage evaluations of one RK4 step (ompVC/integration.c:362-396);
// e[]/l[] are the stage points' persistent element hints and exit flags.
template <int DIMS, int MESH>
__device__ __forceinline__ int rk4_stages(const DevMesh& m, const DevWindow& w, const Pt& p,
                                          double tc, double h, int k, int e[4], int l[4],
                                          double kk[4][3], const NatCache* nc) {
  double M[3];
  int err;
  M[0] = p.X[0];
  M[1] = p.X[1];
  M[2] = p.X[2];
  if ((err = velocity<DIMS, MESH>(m, w, tc, 2 * k, M, e[0], l[0], kk[0], nc))) return err;
  M[0] = p.X[0] + 0.5 * kk[0][0] * h;
  M[1] = p.X[1] + 0.5 * kk[0][1] * h;
  M[2] = p.X[2] + 0.5 * kk[0][2] * h;
  if ((err = velocity<DIMS, MESH>(m, w, tc + h * 0.5, 2 * k + 1, M, e[1], l[1], kk[1]))) return err;
  M[0] = p.X[0] + 0.5 * kk[1][0] * h;
  M[1] = p.X[1] + 0.5 * kk[1][1] * h;
  M[2] = p.X[2] + 0.5 * kk[1][2] * h;
  if ((err = velocity<DIMS, MESH>(m, w, tc + h * 0.5, 2 * k + 1, M, e[2], l[2], kk[2]))) return err;
  M[0] = p.X[0] + kk[2][0] * h;
  M[1] = p.X[1] + kk[2][1] * h;
  M[2] = p.X[2] + kk[2][2] * h;
  return velocity<DIMS, MESH>(m, w, tc + h, 2 * k + 2, M, e[3], l[3], kk[3]);
}

// RK4, ompVC/integration.c:317-462
template <int DIMS, int MESH, bool CET = false>
__device__ __forceinline__ double rk4(const DevMesh& m, const DevWindow& w, const DevInteg& in,
                                      Pt& p, double tstart, double tend, unsigned& steps, int& err,
                                      const CetDev* cet = nullptr, const RecOut* rec = nullptr,
                                      Chk1* chk = nullptr) {
  int e[4] = {p.eid, p.eid, p.eid, p.eid};
  int l[4] = {p.left, p.left, p.left, p.left};
  double kk[4][3];
  NatCache nc;
  nc.e = -1;
  // a planar flow's stages all give w = +0.0 (2D triangles; a 2D grid whose
  // frames carry w = 0): the z increment h (0 + 2*0 + 2*0 + 0) / 6 is then a
  // zero with h's sign, added without the arithmetic
  const bool planar = DIMS == 2 && (MESH == 1 || w.wz);
  double tc = tstart, h = dsign(in.h, tend - tstart);
  int k = 0;
  while ((tc - tend) * (tend - tstart) < 0.0) {
    if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = dsign(tend - tc, tend - tstart);
    if ((err |= rk4_stages<DIMS, MESH>(m, w, p, tc, h, k, e, l, kk, &nc))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++)
      p.X[q] = (q == 2 && planar) ? p.X[2] + zero_of(h)
                                  : p.X[q] + div_rn(h * (kk[0][q] + 2 * kk[1][q] + 2 * kk[2][q] + kk[3][q]), 6.0, kRcp6);
    tc = tc + h;
    k++;
    if (MESH == 1) p.eid = locate_walk<DIMS>(m, p.X, p.eid, err, &nc);
    if (err) return tend;
    if ((MESH == 0 && outside_domain(m, p.X)) || (MESH == 1 && p.eid < 0) || l[0] || l[1] || l[2] ||
        l[3]) {
      if (MESH == 1) err |= walk_fault(e[0]) | walk_fault(e[1]) | walk_fault(e[2]) | walk_fault(e[3]);
      p.left = 1;
      p.ldt = tc - h;
#pragma unroll
      for (int q = 0; q < 3; q++)
        p.X[q] = (q == 2 && planar) ? p.X[2] - zero_of(h)
                                    : p.X[q] - div_rn(h * (kk[0][q] + 2 * kk[1][q] + 2 * kk[2][q] + kk[3][q]), 6.0, kRcp6);
      return p.ldt;
    }
    steps++;
    if (rec && k <= rec->max) {
      double* o = rec->base + (long)(k - 1) * rec->stride;
      o[0] = p.X[0];
      o[1] = p.X[1];
      o[2] = p.X[2];
      if (k == 1 && rec->e1) *rec->e1 = make_int4(e[0] == rec->eid0 ? e[1] : -3, e[2], e[3], p.eid);
    }
    if (chk && k == 1) {
      chk->hit = e[0] == chk->e0 && e[1] == chk->e1.x && e[2] == chk->e1.y && e[3] == chk->e1.z &&
                 p.eid == chk->e1.w;
      if (chk->hit) return tend;
    }
    if (in.extrapolate && (err |= velocity_cold<DIMS, MESH>(m, w, tc, 2 * k, p.X, &p.eid, &p.left, p.V)))
      return tend;
    if (CET) {  // ompVC/integration.c:427-447
      double X0[3];
#pragma unroll
      for (int q = 0; q < 3; q++) X0[q] = p.X[q] - div_rn(h * (kk[0][q] + 2 * kk[1][q] + 2 * kk[2][q] + kk[3][q]), 6.0, kRcp6);
      cet_step<DIMS>(m, *cet, X0, p.X, p.eid, h, &err);
      if (err) return tend;
    }
  }
  return tend;
}

// Two-step Adams-Bashforth (Int_Type 3, cudaVC's numbering,
// cudaVC/src/main.cu:225).  ompVC has no multistep integrator; this is the
// textbook variable-step AB2 X_{n+1} = X_n + h (c1 f_n - c0 f_{n-1}) with
// c0 = h / (2 h_prev), c1 = 1 + c0, bootstrapped by one RK4 step at the start
// of every call and using RK4's clip, relocation and exit rules.
template <int DIMS, int MESH>
__device__ __noinline__ double ab2(const DevMesh& m, const DevWindow& w, const DevInteg& in,
                                   Pt& p, double tstart, double tend, unsigned& steps, int& err) {
  int e[4] = {p.eid, p.eid, p.eid, p.eid};
  int l[4] = {p.left, p.left, p.left, p.left};
  double kk[4][3], fprev[3] = {0, 0, 0}, hprev = 0.0;
  NatCache nc;
  nc.e = -1;
  double tc = tstart, h = dsign(in.h, tend - tstart);
  bool first = true;
  int k = 0;
  while ((tc - tend) * (tend - tstart) < 0.0) {
    if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = dsign(tend - tc, tend - tstart);
    double inc[3], f[3];
    int lf = 0, ef = p.eid;
    if (first) {
      if ((err |= rk4_stages<DIMS, MESH>(m, w, p, tc, h, k, e, l, kk, &nc))) return tend;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        inc[q] = div_rn(h * (kk[0][q] + 2 * kk[1][q] + 2 * kk[2][q] + kk[3][q]), 6.0, kRcp6);
        f[q] = kk[0][q];
      }
      lf = l[0] || l[1] || l[2] || l[3];
    } else {
      if ((err |= velocity<DIMS, MESH>(m, w, tc, 2 * k, p.X, ef, lf, f, &nc))) return tend;
      double c0 = h / (2.0 * hprev), c1 = 1.0 + c0;
#pragma unroll
      for (int q = 0; q < 3; q++) inc[q] = h * (c1 * f[q] - c0 * fprev[q]);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) p.X[q] = p.X[q] + inc[q];
    tc = tc + h;
    k++;
    if (MESH == 1) p.eid = locate_walk<DIMS>(m, p.X, p.eid, err, &nc);
    if (err) return tend;
    if ((MESH == 0 && outside_domain(m, p.X)) || (MESH == 1 && p.eid < 0) || lf) {
      if (MESH == 1)
        err |= walk_fault(ef) | walk_fault(e[0]) | walk_fault(e[1]) | walk_fault(e[2]) | walk_fault(e[3]);
      p.left = 1;
      p.ldt = tc - h;
#pragma unroll
      for (int q = 0; q < 3; q++) p.X[q] = p.X[q] - inc[q];
      return p.ldt;
    }
    steps++;
#pragma unroll
    for (int q = 0; q < 3; q++) fprev[q] = f[q];
    hprev = h;
    first = false;
    if (in.extrapolate && (err |= velocity_cold<DIMS, MESH>(m, w, tc, 2 * k, p.X, &p.eid, &p.left, p.V)))
      return tend;
  }
  return tend;
}

// Advect, ompVC/integration.c:22-45 (Int_Type 0 Euler, 1 RK4, 3 AB2).
// Euler and AB2 are called out of line so that kernels inline only RK4.
// RKF, ompVC/integration.c:464-699: Runge-Kutta-Fehlberg 4(5) with the
// reference's coefficients, error estimate and step-size control, per
// particle.  The stage points keep their element hints and exit flags across
// steps (MP1 .. MP6); a stage outside the domain stops the point at tc
// without moving it.  Stage times vary per particle, so the stages
// interpolate the two frames in time themselves.  The step-size factor is
// the reference's pow(x, 0.25), computed correctly rounded (rn_root4): the
// accept / reject test makes the trajectory depend on its last bit.
template <int DIMS, int MESH, bool CET = false>
__device__ __noinline__ double rkf(const DevMesh& m, const DevWindow& w, const DevInteg& in, Pt& p,
                                   double tstart, double tend, unsigned& steps, int& err,
                                   const CetDev* cet = nullptr) {
  double k[6][3], M[3];
  int e[6], l[6];
#pragma unroll
  for (int j = 0; j < 6; j++) {
    e[j] = p.eid;
    l[j] = p.left;
  }
  const double a3 = 3.0 / 32.0, b3 = 9.0 / 32.0;
  const double a4 = 1932.0 / 2197.0, b4 = -7200.0 / 2197.0, c4 = 7296.0 / 2197.0;
  const double a5 = 439.0 / 216.0, b5 = -8.0, c5 = 3680.0 / 513.0, d5 = -845.0 / 4104.0;
  const double a6 = -8.0 / 27.0, b6 = 2.0, c6 = -3544.0 / 2565.0, d6 = 1859.0 / 4104.0, e6 = -11.0 / 40.0;
  const double a7 = 1.0 / 360.0, b7 = -128.0 / 4275.0, c7 = -2197.0 / 75240.0, d7 = 1.0 / 50.0, e7 = 2.0 / 55.0;
  const double a8 = 25.0 / 216.0, b8 = 1408.0 / 2565.0, c8 = 2197.0 / 4104.0, d8 = -1.0 / 5.0;
  double h = dsign(in.hmax, tend - tstart), tc = tstart, ts, ss;
  // the reference loops until tc reaches tend; a cap on the attempts bounds
  // the kernel when Int_MinTimeStep is tiny against the interval
  for (int attempt = 0; (tc - tend) * (tend - tstart) < 0.0; attempt++) {
    if (attempt >= (1 << 24)) {
      err |= PT_ERR_WALK;
      return tend;
    }
    if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = dsign(tend - tc, tend - tstart);
#pragma unroll
    for (int q = 0; q < 3; q++) M[q] = p.X[q];
    if ((err |= velocity<DIMS, MESH>(m, w, tc, -1, M, e[0], l[0], k[0]))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++) M[q] = p.X[q] + 0.25 * k[0][q] * h;
    ts = tc + 0.25 * h;
    if ((err |= velocity<DIMS, MESH>(m, w, ts, -1, M, e[1], l[1], k[1]))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++) M[q] = p.X[q] + (a3 * k[0][q] + b3 * k[1][q]) * h;
    ts = tc + 0.375 * h;
    if ((err |= velocity<DIMS, MESH>(m, w, ts, -1, M, e[2], l[2], k[2]))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++) M[q] = p.X[q] + (a4 * k[0][q] + b4 * k[1][q] + c4 * k[2][q]) * h;
    ts = tc + div_rn(12.0 * h, 13.0, kRcp13);
    if ((err |= velocity<DIMS, MESH>(m, w, ts, -1, M, e[3], l[3], k[3]))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++) M[q] = p.X[q] + (a5 * k[0][q] + b5 * k[1][q] + c5 * k[2][q] + d5 * k[3][q]) * h;
    ts = tc + h;
    if ((err |= velocity<DIMS, MESH>(m, w, ts, -1, M, e[4], l[4], k[4]))) return tend;
#pragma unroll
    for (int q = 0; q < 3; q++)
      M[q] = p.X[q] + (a6 * k[0][q] + b6 * k[1][q] + c6 * k[2][q] + d6 * k[3][q] + e6 * k[4][q]) * h;
    ts = tc + 0.5 * h;
    if ((err |= velocity<DIMS, MESH>(m, w, ts, -1, M, e[5], l[5], k[5]))) return tend;
    if (l[0] || l[1] || l[2] || l[3] || l[4] || l[5]) {
      if (MESH == 1)
        err |= walk_fault(e[0]) | walk_fault(e[1]) | walk_fault(e[2]) | walk_fault(e[3]) | walk_fault(e[4]) |
               walk_fault(e[5]);
      p.left = 1;
      p.ldt = tc;
      return p.ldt;
    }
    double ex[3];
#pragma unroll
    for (int q = 0; q < 3; q++)
      ex[q] = fabs(a7 * k[0][q] + b7 * k[2][q] + c7 * k[3][q] + d7 * k[4][q] + e7 * k[5][q]);
    const double er = fmax(fmax(ex[0], ex[1]), ex[2]);
    if (er == 0.0) ss = 0.0;
    else ss = rn_root4(fabs((in.acc * h) / (2 * er)));
    if (er < in.acc || fabs(h) <= in.hmin) {
#pragma unroll
      for (int q = 0; q < 3; q++) p.X[q] = p.X[q] + (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
      tc = tc + h;
      if (MESH == 1) p.eid = locate_walk<DIMS>(m, p.X, p.eid, err);
      if (err) return tend;
      if ((MESH == 0 && outside_domain(m, p.X)) || (MESH == 1 && p.eid < 0)) {
        p.left = 1;
        p.ldt = tc - h;
#pragma unroll
        for (int q = 0; q < 3; q++)
          p.X[q] = p.X[q] - (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
        return p.ldt;
      }
      steps++;
      if (in.extrapolate && (err |= velocity_cold<DIMS, MESH>(m, w, tc, -1, p.X, &p.eid, &p.left, p.V)))
        return tend;
      if (CET) {  // ompVC/integration.c:649-669
        double X0[3];
#pragma unroll
        for (int q = 0; q < 3; q++)
          X0[q] = p.X[q] - (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
        cet_step<DIMS>(m, *cet, X0, p.X, p.eid, h, &err);
        if (err) return tend;
      }
      if (fabs(h) > in.hmin && ss > 1.0) {
        ss = (ss > 4.0) ? 4.0 : ss;
        h = dsign((fabs(ss * h) > in.hmax) ? in.hmax : ss * h, tend - tstart);
      }
    } else {
      if (ss < 1.0) {
        ss = (ss < 0.1) ? 0.1 : ss;
        h = dsign((fabs(ss * h) < in.hmin) ? in.hmin : ss * h, tend - tstart);
      } else
        h = dsign((fabs(0.5 * h) < in.hmin) ? in.hmin : 0.5 * h, tend - tstart);
    }
  }
  return tend;
}

// I: the integrator when the kernel is compiled for one (1 = RK4: the other
// integrators' code, and the registers it needs, drop out), or -1 for
// in.type at run time.
template <int DIMS, int MESH, bool CET = false, int I = -1>
__device__ __forceinline__ int advect(const DevMesh& m, const DevWindow& w, const DevInteg& in,
                                      Pt& p, double tstart, double tend, unsigned& steps,
                                      const CetDev* cet = nullptr, const RecOut* rec = nullptr,
                                      Chk1* chk = nullptr) {
  int err = 0;
  if (p.left && in.extrapolate) {
#pragma unroll
    for (int q = 0; q < 3; q++) p.X[q] = p.X[q] + p.V[q] * (tend - tstart);
    return 0;
  }
  if (p.left) return PT_ERR_STATE;  // "integrate point that already left domain"
  if (MESH == 1 && p.eid < 0) return PT_ERR_STATE;
  double stop;
  if (I == 1 || (I < 0 && in.type == 1)) stop = rk4<DIMS, MESH, CET>(m, w, in, p, tstart, tend, steps, err, cet, rec, chk);
  else if (I < 0 && in.type == 2) stop = rkf<DIMS, MESH, CET>(m, w, in, p, tstart, tend, steps, err, cet);
  else if (I < 0 && in.type == 3 && !CET) stop = ab2<DIMS, MESH>(m, w, in, p, tstart, tend, steps, err);
  else stop = euler<DIMS, MESH, CET>(m, w, in, p, tstart, tend, steps, err, cet, rec);
  if (MESH == 1) err |= walk_fault(p.eid);
  if (!err && (fabs(stop - tend) > FVC_TINY) && in.extrapolate) {
#pragma unroll
    for (int q = 0; q < 3; q++) p.X[q] = p.X[q] + p.V[q] * (tend - stop);
  }
  return err;
}

// ------------------------------------------------------------- reductions

// Warp-aggregated accumulation of accepted steps and fault bits.
__device__ __forceinline__ void flush_counters(unsigned long long* step_ctr, int* status,
                                               unsigned steps, int err) {
  unsigned long long s = steps;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  int e = __reduce_or_sync(0xffffffffu, err);
  if ((threadIdx.x & 31) == 0) {
    if (s) atomicAdd(step_ctr, s);
    if (e) atomicOr(status, e);
  }
}

}  // namespace fvc
