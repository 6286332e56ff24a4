// fvc_mixed.cuh -- the mixed-precision form of unstructured advection.
//
// Frames are read as 16-bit values (BF16 or FP16) times a per-frame,
// per-component FP32 scale; point location, the barycentric weights, the
// time interpolation and the Euler / RK4 stages run in FP32; positions are
// FP32 with a Kahan compensation term (the position is X - c).  Within
// FVC_NEAR_FACE of an element face (in natural coordinates) the containment
// test and the walk's face choice are ompVC's FP64 ones
// (ompVC/velocity.c:512-617, ompVC/mesh.c:542-609) on X - c; so is every
// decision whose FP32 coordinates lie within their own error bound of a face
// (nat32's tol, from the element's conditioning).
//
// The step sequence of a call (stage times, step lengths, tloc) is the FP64
// host sequence of the call in a device table (StepM), so the step loop
// issues no FP64 instruction: GB300 runs FP64 at 1/64 of its FP32 rate.
// A particle that leaves records the start time of the step it left in
// (LeftDomainTime), a table time, which later calls use as an end time.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "fvc_device.cuh"

namespace fvc {

#define FVC_NEAR_FACE 1.0e-5f
// resident 128-thread blocks per SM the mixed-form kernels are compiled for
#ifndef FVC_MX_MINBLOCKS
#define FVC_MX_MINBLOCKS 4
#endif
enum { QF_BF16 = 1, QF_FP16 = 2 };  // the FVC_PREC_* codes of fvc.h

struct PtM {
  float X[3];
  float c[3];
  int eid;
  int left;
  double ldt;
};

// In the mixed form a job's FP64 position arrays hold, in each 8-byte slot,
// the float pair (X, c) of one coordinate.
__device__ __forceinline__ void load_pos_pair(const double* A, long p, float X[3], float c[3]) {
  const float2* q = reinterpret_cast<const float2*>(A + 3 * p);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float2 v = q[k];
    X[k] = v.x;
    c[k] = v.y;
  }
}
__device__ __forceinline__ void store_pos_pair(double* A, long p, const float X[3], const float c[3]) {
  float2* q = reinterpret_cast<float2*>(A + 3 * p);
#pragma unroll
  for (int k = 0; k < 3; k++) q[k] = make_float2(X[k], c[k]);
}
// FP64 value <-> pair: X = RN(v), c = RN(X - v); back: X - c
__device__ __forceinline__ float2 split_pos(double v) {
  float x = __double2float_rn(v);
  return make_float2(x, __double2float_rn((double)x - v));
}
__device__ __forceinline__ double join_pos(float2 p) { return (double)p.x - (double)p.y; }

__device__ __forceinline__ float dec16(unsigned short b, int fmt) {
  return fmt == QF_BF16 ? __uint_as_float((unsigned)b << 16) : __half2float(__ushort_as_half(b));
}

// One node's velocity at tloc tl from the two quantised frames.  W is a
// DevWindow or any view with its qp, qs0, qs1 and qfmt members.
template <class W>
__device__ __forceinline__ void node_vel_mx(const W& w, int node, float tl, float out[3]) {
  const uint4 p = __ldg(w.qp + node);
  const float ua = dec16((unsigned short)(p.x & 0xffffu), w.qfmt) * w.qs0[0];
  const float va = dec16((unsigned short)(p.x >> 16), w.qfmt) * w.qs0[1];
  const float wa = dec16((unsigned short)(p.y & 0xffffu), w.qfmt) * w.qs0[2];
  const float ub = dec16((unsigned short)(p.y >> 16), w.qfmt) * w.qs1[0];
  const float vb = dec16((unsigned short)(p.z & 0xffffu), w.qfmt) * w.qs1[1];
  const float wb = dec16((unsigned short)(p.z >> 16), w.qfmt) * w.qs1[2];
  out[0] = fmaf(tl, ub - ua, ua);
  out[1] = fmaf(tl, vb - va, va);
  out[2] = fmaf(tl, wb - wa, wa);
}

// FP32 natural coordinates of X in element e from its 64-byte FP32 record
// (a11..a33, 1/V, x0, y0, z0, A in 3D; a11..a22, 1/V, x0, y0, A in 2D);
// returns their minimum.  tol bounds the coordinates' FP32 error: the
// offsets X - x0 err by at most E = 2^-24 (|X| + |x0| + |dx|) per component
// (half an ulp each for X against X - c, for the rounded x0 and for the
// difference), which moves each coordinate by at
// most A E with A = sum |a_ij| / |V|, and the FP32 products and sums add at
// most 1e-6 (1 + S) with S <= A max |dx| -- the bound of the FP64 form's
// pre-check (fvc_device.cuh, quick_hop).  Ill-conditioned (sliver) elements
// have a large A, so their walk decisions fall to the FP64 test.
template <int D>
__device__ __forceinline__ float nat32(const DevMesh& m, int e, const float X[3], float& r, float& s, float& t,
                                       float& wv, float& tol) {
  const float* q = m.geo32 + (long)e * 16;
  if (D == 3) {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    float4 q2 = __ldg(reinterpret_cast<const float4*>(q + 8));
    float2 q3 = __ldg(reinterpret_cast<const float2*>(q + 12));  // (z0, A)
    float dx = X[0] - q2.z, dy = X[1] - q2.w, dz = X[2] - q3.x;
    r = fmaf(q0.x, dx, fmaf(q0.y, dy, q0.z * dz)) * q2.y;
    s = fmaf(q0.w, dx, fmaf(q1.x, dy, q1.y * dz)) * q2.y;
    t = fmaf(q1.z, dx, fmaf(q1.w, dy, q2.x * dz)) * q2.y;
    wv = 1.0f - r - s - t;
    const float dm = fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)));
    const float xm = fmaxf(fabsf(X[0]), fmaxf(fabsf(X[1]), fabsf(X[2])));
    const float om = fmaxf(fabsf(q2.z), fmaxf(fabsf(q2.w), fabsf(q3.x)));
    tol = fmaf(q3.y, fmaf(6.0e-8f, xm + om + dm, 1e-6f * dm), 1e-6f);
    return fminf(fminf(r, s), fminf(t, wv));
  } else {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    // q1 = (1/V, x0, y0, A)
    float dx = X[0] - q1.y, dy = X[1] - q1.z;
    r = fmaf(q0.x, dx, q0.y * dy) * q1.x;
    s = fmaf(q0.z, dx, q0.w * dy) * q1.x;
    t = 0.0f;
    wv = 1.0f - r - s;
    const float dm = fmaxf(fabsf(dx), fabsf(dy));
    const float xm = fmaxf(fabsf(X[0]), fabsf(X[1]));
    const float om = fmaxf(fabsf(q1.y), fabsf(q1.z));
    tol = fmaf(q1.w, fmaf(6.0e-8f, xm + om + dm, 1e-6f * dm), 1e-6f);
    return fminf(fminf(r, s), wv);
  }
}

// (X - C) - x0 for a position X with compensation C (|C| within an ulp of X)
// and a node x0 = xh + xl held as two floats: X - xh exactly by Knuth's
// TwoSum, the small terms added to its error, one rounding at the end.  The
// result errs by 2^-24 of itself plus about 2^-44 |X| (the small terms'
// roundings), all in FP32.
__device__ __forceinline__ float exact_offset(float X, float C, float xh, float xl) {
  const float s = X - xh;
  const float bb = s - X;
  const float e = (X - (s - bb)) + (-xh - bb);
  return s + ((e - C) - xl);
}

// The same coordinates with exact offsets: (X - C) - x0 formed from the
// element's node in two floats (exact_offset) and rounded once, then the
// FP32 map.  The offsets then err by 2^-24 |dx| instead of by the FP32
// positions' rounding, so tol shrinks to the map's own rounding.  Per
// coordinate, r = fl(fl(fmaf(a11, dx, fmaf(a12, dy, a13 dz))) / V) carries
// seven relative roundings of at most 2^-24 on sums bounded by
// sum_j |a1j dxj| / |V| (the FP32 a1j and 1/V, the offsets, the product and
// two partial sums, the scaling); w = ((1 - r) - s) - t adds three roundings
// of at most 2^-24 (1 + |r| + |s| + |t|) <= 2^-23; exact_offset's absolute
// error, 2^-44 max(|X|, |x0|), adds A times that.  The minimum coordinate
// therefore errs by at most 4.2e-7 A max|dx| + 5.7e-14 A (|X| + max|dx|)
// + 3.6e-7, and tol is set a little above that.
template <int D>
__device__ __forceinline__ float nat32_fine(const DevMesh& m, int e, const float X[3], const float C[3], float& r,
                                            float& s, float& t, float& wv, float& tol) {
  const float* q = m.geo32 + (long)e * 16;
  if (D == 3) {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    float4 q2 = __ldg(reinterpret_cast<const float4*>(q + 8));
    const float4 lo = __ldg(m.geo32lo + e);
    const float dx = exact_offset(X[0], C[0], q2.z, lo.x);
    const float dy = exact_offset(X[1], C[1], q2.w, lo.y);
    const float dz = exact_offset(X[2], C[2], __ldg(q + 12), lo.z);
    const float A = __ldg(q + 13);
    r = fmaf(q0.x, dx, fmaf(q0.y, dy, q0.z * dz)) * q2.y;
    s = fmaf(q0.w, dx, fmaf(q1.x, dy, q1.y * dz)) * q2.y;
    t = fmaf(q1.z, dx, fmaf(q1.w, dy, q2.x * dz)) * q2.y;
    wv = 1.0f - r - s - t;
    const float dm = fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)));
    const float xm = fmaxf(fabsf(X[0]), fmaxf(fabsf(X[1]), fabsf(X[2])));
    tol = fmaf(A, fmaf(4.5e-7f, dm, 6e-14f * (xm + dm)), 4e-7f);
    return fminf(fminf(r, s), fminf(t, wv));
  } else {
    float4 q0 = __ldg(reinterpret_cast<const float4*>(q)), q1 = __ldg(reinterpret_cast<const float4*>(q + 4));
    const float4 lo = __ldg(m.geo32lo + e);
    const float dx = exact_offset(X[0], C[0], q1.y, lo.x);
    const float dy = exact_offset(X[1], C[1], q1.z, lo.y);
    r = fmaf(q0.x, dx, q0.y * dy) * q1.x;
    s = fmaf(q0.z, dx, q0.w * dy) * q1.x;
    t = 0.0f;
    wv = 1.0f - r - s;
    const float dm = fmaxf(fabsf(dx), fabsf(dy));
    const float xm = fmaxf(fabsf(X[0]), fabsf(X[1]));
    tol = fmaf(q1.w, fmaf(4.5e-7f, dm, 6e-14f * (xm + dm)), 4e-7f);
    return fminf(fminf(r, s), wv);
  }
}

// The walk of GetVelocity_Unstructured (vel_rule) / Get_Element_Local_Search
// in the mixed form.  Returns 0 with the FP32 natural coordinates of the
// element found, or 1 when the walk stops: eid = -1 when it left through a
// boundary face, EID_FAULT when it failed.
// ompVC's FP64 containment test of element e at X - C and, when it fails,
// its face choice: returns -2 when the point is inside (coordinates in
// r, s, t, wv), the face slot to step through, or -1 ("Indeterminate
// neighbor").  Out of line so that none of its FP64 work is hoisted into
// the FP32 walk.
template <int D>
__device__ __noinline__ int near_face_fp64(const DevMesh& m, int e, const float* X, const float* C, bool vel_rule,
                                           float* out) {
  const double x[3] = {(double)X[0] - (double)C[0], (double)X[1] - (double)C[1], (double)X[2] - (double)C[2]};
  double R, S, T, W;
  const double dd = natural<D>(m, e, x, R, S, T, W);
  if (vel_rule ? ((dd + FVC_TINY) >= 0) : (dd > -FVC_TINY)) {
    out[0] = (float)R;
    out[1] = (float)S;
    out[2] = (float)T;
    out[3] = (float)W;
    return -2;
  }
  if (fabs(R - dd) < FVC_TINY) return 0;
  if (fabs(S - dd) < FVC_TINY) return 1;
  if (D == 3 && fabs(T - dd) < FVC_TINY) return 2;
  if (fabs(W - dd) < FVC_TINY) return D == 3 ? 3 : 2;
  return -1;
}

// The last locate's element and coordinates at the current position.
struct NatM {
  int e;
  int4 nd;
  float r, s, t;
};

// nc (velocity walks only): as in the FP64 walk, reaching the element the
// last locate found at this position gives that locate's coordinates, which
// the tests below would reproduce there (the locate passed, so the velocity
// rule passes too).
template <int D>
__device__ __forceinline__ int walk_mx(const DevMesh& m, const float X[3], const float C[3], int& eid, bool vel_rule,
                                       float& r, float& s, float& t, float& wv, int4& nd,
                                       const NatM* nc = nullptr) {
  for (int hop = 0; hop < m.max_hops; hop++) {
    if (nc && eid == nc->e) {
      nd = nc->nd;
      r = nc->r;
      s = nc->s;
      t = nc->t;
      wv = 1.0f - r - s - t;
      return 0;
    }
    // the element's node ids and neighbours (one 32-byte sector), loaded
    // beside its record
    nd = __ldg(m.elem + 2 * (long)eid);
    const int4 nb = __ldg(m.elem + 2 * (long)eid + 1);
    float tol;
    float d = nat32<D>(m, eid, X, r, s, t, wv, tol);
    // FP32 decides only outside the band its error bound leaves open; inside
    // it, the coordinates are recomputed from exact offsets first, and the
    // FP64 test decides only inside that narrower band
    float band = fmaxf(FVC_NEAR_FACE, 2.0f * tol);
    if (fabsf(d) <= band) {
      d = nat32_fine<D>(m, eid, X, C, r, s, t, wv, tol);
      band = fmaxf(FVC_NEAR_FACE, 2.0f * tol);
    }
    int slot;
    if (d > band) return 0;
    if (d < -band) {
      // the face of the smallest coordinate, first in r, s, t, 1-r-s-t order
      slot = (r == d) ? 0 : (s == d) ? 1 : (D == 3 && t == d) ? 2 : (D == 3 ? 3 : 2);
    } else {
      float c4[4];
      slot = near_face_fp64<D>(m, eid, X, C, vel_rule, c4);
      if (slot == -2) {
        r = c4[0];
        s = c4[1];
        t = c4[2];
        wv = c4[3];
        return 0;
      }
      if (slot < 0) break;
    }
    eid = pick(nb, slot);
    if (eid == -1) return 1;
  }
  eid = EID_FAULT;
  return 1;
}

// Velocity at X (compensation C) and tloc tl: P1 in space, linear in time.
template <int D, class W>
__device__ __forceinline__ int vel_mx(const DevMesh& m, const W& w, float tl, const float X[3],
                                      const float C[3], int& eid, int& left, float out[3], const NatM* nc) {
  if (eid < 0 || eid >= m.nelem) return PT_ERR_WALK;
  float r, s, t, wv;
  int4 nd;
  if (nc && nc->e == eid) {
    nd = nc->nd;
    r = nc->r;
    s = nc->s;
    t = nc->t;
  } else {
    if (walk_mx<D>(m, X, C, eid, true, r, s, t, wv, nd, nc)) {
      // out of the domain, or a failed walk (eid = EID_FAULT): the point stops
      left = 1;
      out[0] = out[1] = out[2] = 0.0f;
      return 0;
    }
  }
  float u0[3], u1[3], u2[3];
  node_vel_mx(w, nd.x, tl, u0);
  node_vel_mx(w, nd.y, tl, u1);
  node_vel_mx(w, nd.z, tl, u2);
  const float ar = fabsf(r), as = fabsf(s);
  if (D == 3) {
    float u3[3];
    node_vel_mx(w, nd.w, tl, u3);
    const float at = fabsf(t);
#pragma unroll
    for (int c = 0; c < 3; c++) out[c] = fmaf(u3[c] - u0[c], at, fmaf(u2[c] - u0[c], as, fmaf(u1[c] - u0[c], ar, u0[c])));
  } else {
#pragma unroll
    for (int c = 0; c < 2; c++) out[c] = fmaf(u2[c] - u0[c], as, fmaf(u1[c] - u0[c], ar, u0[c]));
    out[2] = 0.0f;
  }
  return 0;
}

template <int D>
__device__ __forceinline__ int locate_mx(const DevMesh& m, const float X[3], const float C[3], int guess, int& err,
                                         NatM* nc) {
  nc->e = -1;
  if (guess < 0) return -1;
  if (guess >= m.nelem) {
    err |= PT_ERR_WALK;
    return -1;
  }
  float r, s, t, wv;
  int4 nd;
  if (walk_mx<D>(m, X, C, guess, false, r, s, t, wv, nd)) return guess == EID_FAULT ? EID_FAULT : -1;
  nc->e = guess;
  nc->nd = nd;
  nc->r = r;
  nc->s = s;
  nc->t = t;
  return guess;
}

// Positions += inc with Kahan compensation.
__device__ __forceinline__ void kahan_add(float X[3], float c[3], const float inc[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float y = inc[k] - c[k];
    const float t = X[k] + y;
    c[k] = (t - X[k]) - y;
    X[k] = t;
  }
}

// Euler or RK4 over table steps [0, kend) (Advect, ompVC/integration.c:
// 22-45, with RK4's exit rules, integration.c:317-462).  A particle that
// leaves keeps its position before the step and records the step's start
// time as LeftDomainTime.
//
// Walk hints.  ompVC starts each RK4 stage's walk from the element that
// stage ended in on the previous step, and the step's locate from the
// point's element; the FP64 form keeps that (its element ids are compared
// bit for bit).  Here each walk starts where the previous one ended: stage
// 1 at the located element (its coordinates are the locate's), stage k + 1
// at stage k's element, the locate at stage 4's.  Consecutive stage points
// lie half a step apart instead of a whole step, so walks hop about half as
// often, and one running hint replaces four.  Only a point within the walk's
// tolerance of a shared face can end in another element, where the P1
// velocity is continuous: the results differ by rounding.  A stage whose
// walk leaves the domain leaves the hint where it was.
template <int D, class W>
__device__ __forceinline__ void advect_mx(const DevMesh& m, const W& w, int type, PtM& p, int kend,
                                          unsigned& steps, int& err, const RecOut* rec = nullptr) {
  if (p.left) return;
  const float zero[3] = {0.0f, 0.0f, 0.0f};
  NatM nc;
  nc.e = -1;
  for (int k = 0; k < kend; k++) {
    const StepM st = w.steps[k];
    const float h = st.h;
    float inc[3];
    int hint = p.eid, out = 0;
    // one stage: velocity at Y (compensation C) from the running hint
    auto stage = [&](float tl, const float* Y, const float* C, const NatM* cache, float v[3]) {
      int e = hint, l = 0;
      err |= vel_mx<D>(m, w, tl, Y, C, e, l, v, cache);
      if (l) {
        err |= walk_fault(e);
        out = 1;
      } else {
        hint = e;
      }
    };
    if (type == 0) {
      float v[3];
      stage(st.tl0, p.X, p.c, &nc, v);
      if (err) return;
#pragma unroll
      for (int q = 0; q < 3; q++) inc[q] = h * v[q];
    } else {
      float kq[3], acc[3], M[3];
      stage(st.tl0, p.X, p.c, &nc, kq);
      if (err) return;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        acc[q] = kq[q];
        M[q] = fmaf(0.5f * h, kq[q], p.X[q]);
      }
      stage(st.tlh, M, zero, nullptr, kq);
      if (err) return;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        acc[q] = acc[q] + 2.0f * kq[q];
        M[q] = fmaf(0.5f * h, kq[q], p.X[q]);
      }
      stage(st.tlh, M, zero, nullptr, kq);
      if (err) return;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        acc[q] = acc[q] + 2.0f * kq[q];
        M[q] = fmaf(h, kq[q], p.X[q]);
      }
      stage(st.tl1, M, zero, nullptr, kq);
      if (err) return;
#pragma unroll
      for (int q = 0; q < 3; q++) inc[q] = h * ((acc[q] + kq[q]) * (1.0f / 6.0f));
    }
    float X0[3] = {p.X[0], p.X[1], p.X[2]}, c0[3] = {p.c[0], p.c[1], p.c[2]};
    kahan_add(p.X, p.c, inc);
    p.eid = locate_mx<D>(m, p.X, p.c, hint, err, &nc);
    if (err) return;
    if (p.eid < 0 || out) {
      err |= walk_fault(p.eid);
      p.left = 1;
      p.ldt = st.tc;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        p.X[q] = X0[q];
        p.c[q] = c0[q];
      }
      return;
    }
    steps++;
    if (rec && k < rec->max) {
      float2* o = reinterpret_cast<float2*>(rec->base + (long)k * rec->stride);
      o[0] = make_float2(p.X[0], p.c[0]);
      o[1] = make_float2(p.X[1], p.c[1]);
      o[2] = make_float2(p.X[2], p.c[2]);
    }
  }
}

// The number of table steps from the call's start to tend, a table time
// (the end of the call or a LeftDomainTime recorded in it); -1 if tend is
// not one.  Compared bit for bit, with integer instructions.
__device__ __forceinline__ int steps_to(const DevWindow& w, double tend) {
  const long long b = __double_as_longlong(tend);
  for (int k = 0; k <= w.nsteps; k++)
    if (__double_as_longlong(w.steps[k].tc) == b) return k;
  return -1;
}

}  // namespace fvc
