// fvc_mixed_impl.cuh -- the kernels of the mixed-precision form (unstructured
// meshes, Euler and RK4), instantiated per dimension in fvc_variant_u2m.cu and
// fvc_variant_u3m.cu.  Same launch interface as Variant<D, 1>; job position
// arrays hold (X, c) float pairs (fvc_mixed.cuh), step-level calls take and
// return FP64 positions.
#pragma once
#include "fvc_advect_impl.cuh"
#include "fvc_mixed.cuh"

namespace fvc {

template <int D>
__global__ void __launch_bounds__(128, FVC_MX_MINBLOCKS) k_advect_mx(DevMesh m, DevWindow w, int type, int n, double* X, int* eid,
                                                   int* left, double* ldt, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned steps = 0;
  int err = 0;
  if (i < n && !left[i]) {
    PtM p;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float2 v = split_pos(X[3 * i + k]);
      p.X[k] = v.x;
      p.c[k] = v.y;
    }
    p.eid = eid[i];
    p.left = 0;
    p.ldt = ldt[i];
    advect_mx<D>(m, w, type, p, w.nsteps, steps, err);
#pragma unroll
    for (int k = 0; k < 3; k++) X[3 * i + k] = join_pos(make_float2(p.X[k], p.c[k]));
    eid[i] = p.eid;
    left[i] = p.left;
    ldt[i] = p.ldt;
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}

template <int D>
__global__ void k_velocity_mx(DevMesh m, DevWindow w, int n, const double* X, int* eid, int* left, float tl,
                              double* out, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (i < n) {
    float x[3], c[3], v[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float2 q = split_pos(X[3 * i + k]);
      x[k] = q.x;
      c[k] = q.y;
    }
    int e = eid[i], l = left[i];
    err = isnan(tl) ? PT_ERR_TLOC : vel_mx<D>(m, w, tl, x, c, e, l, v, nullptr) | walk_fault(e);
    out[3 * i] = v[0];
    out[3 * i + 1] = v[1];
    out[3 * i + 2] = v[2];
    eid[i] = e;
    left[i] = l;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}

template <int D>
__global__ void k_ftle_launch_mx(DevMesh m, DevWindow w, FtleDev f, float tl, DevCounters* ctr) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (p < f.n && !f.left[p]) {
    float x[3], c[3], v[3];
    load_pos_pair(f.X, p, x, c);
    int e = f.eid[p], l = 0;
    err = isnan(tl) ? PT_ERR_TLOC : vel_mx<D>(m, w, tl, x, c, e, l, v, nullptr) | walk_fault(e);
    f.V[3 * p] = v[0];
    f.V[3 * p + 1] = v[1];
    f.V[3 * p + 2] = v[2];
    f.eid[p] = e;
    if (l) f.left[p] = 1;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}

template <int D>
__global__ void __launch_bounds__(128, FVC_MX_MINBLOCKS) k_ftle_pass1_mx(DevMesh m, DevWindow w, int type, FtleDev f,
                                                       DevCounters* ctr) {
  clear_early_counters(ctr);
  const long nlive = *(volatile int*)&ctr->nlive;
  unsigned steps = 0;
  int err = 0;
  for (long base = warp_grab(&ctr->cur[0]); base < nlive; base = warp_grab(&ctr->cur[0])) {
    const long idx = base + (threadIdx.x & 31);
    if (idx >= nlive) continue;
    const long p = f.live[idx];
    PtM t;
    load_pos_pair(f.X, p, t.X, t.c);
    t.eid = f.eid[p];
    t.left = f.left[p];
    t.ldt = f.ldt[p];
    const unsigned before = steps;
    const RecOut r{f.rec + 3 * p, 3L * f.n, f.rec_steps, nullptr, 0};
    advect_mx<D>(m, w, type, t, w.nsteps, steps, err, f.rec ? &r : nullptr);
    if (f.rec) f.kacc[p] = (unsigned char)(steps - before);
    f.flag[p] = 1 | (t.left ? 6 : 0);
    store_pos_pair(f.Xn, p, t.X, t.c);
    f.en[p] = t.eid;
    f.te[p] = t.ldt;
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}

template <int D>
__global__ void __launch_bounds__(128, FVC_MX_MINBLOCKS) k_ftle_tasks_mx(DevMesh m, DevWindow w, int type, FtleDev f, int phase,
                                                       DevCounters* ctr) {
  const long ntask = *(volatile int*)&ctr->tq[phase].ntask;
  int* cursor = &ctr->cur[1 + phase];
  unsigned steps = 0;
  int err = 0;
  for (long base = warp_grab(cursor); base < ntask; base = warp_grab(cursor)) {
    const long idx = base + (threadIdx.x & 31);
    if (idx >= ntask) continue;
    const int2 tk = f.tsorted[idx];
    const long s = tk.x;
    const int c = tk.y & 7;
    const long q = f.served[s], trig = f.trig[s];
    long nb[6];
    int i, j, k;
    served_geometry(f, q, nb, i, j, k);
    const long p = c == 6 ? q : nb[c];
    const double tend = phase == 0 ? f.te[trig] : f.emt[s];
    const int kend = steps_to(w, tend);
    PtM t;
    load_pos_pair(f.X, p, t.X, t.c);
    t.left = f.left[p];
    t.eid = eid_at_trigger(f, p, trig);
    t.ldt = 0.0;
    if (kend < 0) err |= PT_ERR_TLOC;
    else advect_mx<D>(m, w, type, t, kend, steps, err);
    store_pos_pair(f.epos + (s * 7 + c) * 3, 0, t.X, t.c);
    if (phase == 0) f.elt[s * 6 + c] = t.left ? t.ldt : tend;
  }
  flush_counters(&ctr->steps_early, &ctr->status, steps, err);
}

template <int D>
__global__ void k_tracer_launch_mx(DevMesh m, DevWindow w, TracerDev t, float tl, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (i < t.n && !t.left[i]) {
    float x[3], c[3], v[3];
    load_pos_pair(t.X, i, x, c);
    int e = t.eid[i], l = 0;
    err = isnan(tl) ? PT_ERR_TLOC : vel_mx<D>(m, w, tl, x, c, e, l, v, nullptr) | walk_fault(e);
    t.V[3 * i] = v[0];
    t.V[3 * i + 1] = v[1];
    t.V[3 * i + 2] = v[2];
    t.eid[i] = e;
    if (l) t.left[i] = 1;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}

template <int D>
__global__ void __launch_bounds__(128, FVC_MX_MINBLOCKS) k_tracer_advance_mx(DevMesh m, DevWindow w, int type, TracerDev t,
                                                           DevCounters* ctr) {
  const TracerLists L = tracer_lists(t, ctr);
  const long nlive = *(volatile int*)L.cnt;
  unsigned steps = 0;
  int err = 0;
  for (long base = warp_grab(L.cur); base < nlive; base = warp_grab(L.cur)) {
    const long idx = base + (threadIdx.x & 31);
    long i = -1;
    bool keep = false;
    if (idx < nlive) {
      i = t.live[idx];
      PtM p;
      load_pos_pair(t.X, i, p.X, p.c);
      p.eid = t.eid[i];
      p.left = t.left[i];
      p.ldt = t.ldt[i];
      advect_mx<D>(m, w, type, p, w.nsteps, steps, err);
      store_pos_pair(t.X, i, p.X, p.c);
      t.eid[i] = p.eid;
      t.left[i] = p.left;
      t.ldt[i] = p.ldt;
      keep = p.ldt > -FVC_TINY && !p.left;  // the mixed form does not extrapolate
    }
    if (L.next) append_live(t, L, keep, i);
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}

// tloc of a query time for the one-off velocity evaluations (the step loop
// takes its tloc from the step table); a value outside [0, 1] by more than
// TINY is reported as NaN, which the launchers turn into an error.
static inline float host_tloc(const DevWindow& w, double tq) {
  double tl = (tq - w.tmin) / (w.tmax - w.tmin);
  if ((tl > 1 + 1.0e-10) || (tl < 0 - 1.0e-10)) return __builtin_nanf("");
  return (float)tl;
}

template <int D>
struct VariantMx {
  static void advect(const DevMesh& m, const DevWindow& w, const DevInteg& in, int n, double* X, double* V,
                     int* eid, int* left, double* ldt, double t0, double t1, DevCounters* ctr, cudaStream_t s) {
    k_advect_mx<D><<<vblk(n, 128), 128, 0, s>>>(m, w, in.type, n, X, eid, left, ldt, ctr);
  }
  static void velocity(const DevMesh& m, const DevWindow& w, int n, const double* X, int* eid, int* left,
                       double tq, double* out, DevCounters* ctr, cudaStream_t s) {
    k_velocity_mx<D><<<vblk(n, 128), 128, 0, s>>>(m, w, n, X, eid, left, host_tloc(w, tq), out, ctr);
  }
  static void ftle_launch(const DevMesh& m, const DevWindow& w, const FtleDev& f, double t, DevCounters* ctr,
                          cudaStream_t s) {
    k_ftle_launch_mx<D><<<vblk(f.n, 128), 128, 0, s>>>(m, w, f, host_tloc(w, t), ctr);
  }
  static void ftle_pass1(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f, double t1,
                         double t2, DevCounters* ctr, cudaStream_t s) {
    static const unsigned res = resident_blocks(k_ftle_pass1_mx<D>, 128);
    k_ftle_pass1_mx<D><<<capped(f.n, 128, res), 128, 0, s>>>(m, w, in.type, f, ctr);
  }
  // The mixed form runs the task lists in queue order: its advections are
  // bound by gather latency, and grid order keeps a warp's points close
  // together, which pays more here than grouping them by length.
  static void ftle_early(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f, double t1,
                         DevCounters* ctr, bool jacobi, cudaStream_t s) {
    static const unsigned res_nb = resident_blocks(k_ftle_queue_nb<D>, 256);
    static const unsigned res_self = resident_blocks(k_ftle_queue_self<D>, 256);
    static const unsigned res_tasks = resident_blocks(k_ftle_tasks_mx<D>, 128);
    static const unsigned res_final = resident_blocks(k_ftle_early_final<D>, 128);
    static const unsigned res_jacobi = resident_blocks(k_ftle_early_jacobi<D>, 64);
    const double inv_h = 1.0 / fabs(in.h);
    FtleDev g = f;
    g.tsorted = g.tasks;
    // the task counters were cleared with the served count (ftle_triggers)
    k_ftle_queue_nb<D><<<capped(6L * f.n, 256, res_nb), 256, 0, s>>>(f, w, 1, ctr, t1, inv_h);
    k_ftle_tasks_mx<D><<<capped(6L * f.n, 128, res_tasks), 128, 0, s>>>(m, w, in.type, g, 0, ctr);
    k_ftle_queue_self<D><<<capped(7L * f.n, 256, res_self), 256, 0, s>>>(f, w, 1, ctr, t1, inv_h);
    k_ftle_tasks_mx<D><<<capped(7L * f.n, 128, res_tasks), 128, 0, s>>>(m, w, in.type, g, 1, ctr);
    k_ftle_early_final<D><<<capped(f.n, 128, res_final), 128, 0, s>>>(f, ctr);
    if (jacobi) k_ftle_early_jacobi<D><<<capped(f.n, 64, res_jacobi), 64, 0, s>>>(f, ctr);
  }
  static void tracer_launch(const DevMesh& m, const DevWindow& w, const TracerDev& t, double tq, DevCounters* ctr,
                            cudaStream_t s) {
    k_tracer_launch_mx<D><<<vblk(t.n, 128), 128, 0, s>>>(m, w, t, host_tloc(w, tq), ctr);
  }
  static void tracer_advance(const DevMesh& m, const DevWindow& w, const DevInteg& in, const TracerDev& t,
                             double t1, double t2, DevCounters* ctr, cudaStream_t s) {
    static const unsigned res = resident_blocks(k_tracer_advance_mx<D>, 128);
    k_tracer_advance_mx<D><<<capped(t.n, 128, res), 128, 0, s>>>(m, w, in.type, t, ctr);
  }
};

extern template struct VariantMx<2>;
extern template struct VariantMx<3>;

}  // namespace fvc
