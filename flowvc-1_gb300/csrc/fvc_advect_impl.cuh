// fvc_advect_impl.cuh -- kernels that run the integrators, templated on the
// dimension D and mesh type M (0 Cartesian, 1 unstructured).  Each variant is
// instantiated in its own translation unit (fvc_variant_*.cu) so the four
// compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "fvc_device.cuh"
#include "fvc_ftle_math.cuh"
#include "fvc_kernels.h"

namespace fvc {

#ifndef FVC_MINBLOCKS
#define FVC_MINBLOCKS 4
#endif
// the early-FTLE task kernel: divergent short advections, which run better
// with more registers a thread than the main pass (a sweep kept 3)
#ifndef FVC_TASK_MINBLOCKS
#define FVC_TASK_MINBLOCKS 3
#endif

static inline unsigned vblk(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Persistent launches.  Kernels whose item count is only known on the device
// (live lists, task lists) run as many blocks as the GPU holds at once, never
// more than the largest possible count needs; each warp takes the next 32
// items from a cursor in the call's counters, so warps that drew short items
// take more and no block sits idle behind a long one.
template <typename Kern>
static unsigned resident_blocks(Kern k, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, 0);
  long b = (long)(sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  return (unsigned)b;
}
static inline unsigned capped(long n, int bs, unsigned resident) {
  unsigned need = vblk(n, bs);
  return need < resident ? (need > 0 ? need : 1) : resident;
}

// count .. nfall of the counters (the triggers and early-FTLE passes that
// follow the main pass), cleared by the main pass's first block.
__device__ __forceinline__ void clear_early_counters(DevCounters* ctr) {
  constexpr int n = (int)(FVC_EARLY_COUNTERS_BYTES / sizeof(int));
  static_assert(n <= 128, "one store per thread of a 128-thread block");
  if (blockIdx.x == 0 && threadIdx.x < n) (&ctr->count)[threadIdx.x] = 0;
}

// The first of the 32 items the calling warp takes next (all lanes call it).
__device__ __forceinline__ long warp_grab(int* cursor) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(cursor, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

// A tracer advance's lists: the one it takes (count, cursor) and, when the
// advance builds the next call's list itself, the pair it appends to; the
// pair after that is cleared for the call after next.
struct TracerLists {
  int* cnt;
  int* cur;
  int* next;
};
__device__ __forceinline__ TracerLists tracer_lists(const TracerDev& t, DevCounters* ctr) {
  if (!t.live_next) return TracerLists{&ctr->nlive, &ctr->cur[0], nullptr};
  const int a = t.gen % 3;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctr->lcnt[(a + 2) % 3] = 0;
    ctr->lcur[(a + 2) % 3] = 0;
  }
  return TracerLists{&ctr->lcnt[a], &ctr->lcur[a], &ctr->lcnt[(a + 1) % 3]};
}

// Appends the warp's tracers that stay live to the next list (warp ballot,
// one atomic per warp), as compact_live would select them.
__device__ __forceinline__ void append_live(const TracerDev& t, const TracerLists& L, bool keep, long i) {
  const unsigned b = __ballot_sync(0xffffffffu, keep);
  if (!b) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(L.next, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) t.live_next[base + __popc(b & ((1u << lane) - 1u))] = (int)i;
}

__device__ __forceinline__ void load_pt(Pt& p, long i, const double* X, const double* V,
                                        const int* eid, const int* left, const double* ldt) {
  p.X[0] = X[3 * i];
  p.X[1] = X[3 * i + 1];
  p.X[2] = X[3 * i + 2];
  if (V) {
    p.V[0] = V[3 * i];
    p.V[1] = V[3 * i + 1];
    p.V[2] = V[3 * i + 2];
  } else {
    p.V[0] = p.V[1] = p.V[2] = 0.0;
  }
  p.eid = eid ? eid[i] : -1;
  p.left = left[i];
  p.ldt = ldt[i];
}

template <int D, int M, int I>
__global__ void __launch_bounds__(128, FVC_MINBLOCKS) k_advect(DevMesh m, DevWindow w, DevInteg in, int n, double* X, double* V, int* eid,
                         int* left, double* ldt, double t0, double t1, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned steps = 0;
  int err = 0;
  if (i < n) {
    Pt p;
    load_pt(p, i, X, V, eid, left, ldt);
    if (!(p.left && !in.extrapolate)) {
      err = advect<D, M, false, I>(m, w, in, p, t0, t1, steps);
      X[3 * i] = p.X[0];
      X[3 * i + 1] = p.X[1];
      X[3 * i + 2] = p.X[2];
      if (V) {
        V[3 * i] = p.V[0];
        V[3 * i + 1] = p.V[1];
        V[3 * i + 2] = p.V[2];
      }
      if (eid) eid[i] = p.eid;
      left[i] = p.left;
      ldt[i] = p.ldt;
    }
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}


template <int D, int M>
__global__ void k_velocity(DevMesh m, DevWindow w, int n, const double* X, int* eid, int* left,
                           double tq, double* out, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (i < n) {
    double x[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]}, v[3] = {0, 0, 0};
    int e = eid ? eid[i] : -1, l = left[i];
    err = velocity<D, M>(m, w, tq, -1, x, e, l, v) | (M == 1 ? walk_fault(e) : 0);
    out[3 * i] = v[0];
    out[3 * i + 1] = v[1];
    out[3 * i + 2] = v[2];
    if (eid) eid[i] = e;
    left[i] = l;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}



// Launch velocity of a slide (ompVC/ftle.c:84-96): on a Cartesian grid it
// flags points outside the velocity grid.
template <int D, int M>
__global__ void k_ftle_launch(DevMesh m, DevWindow w, FtleDev f, double t, DevCounters* ctr) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (p < f.n && !f.left[p]) {
    double x[3] = {f.X[3 * p], f.X[3 * p + 1], f.X[3 * p + 2]}, v[3];
    int e = f.eid[p], l = 0;
    err = velocity<D, M>(m, w, t, -1, x, e, l, v) | (M == 1 ? walk_fault(e) : 0);
    f.V[3 * p] = v[0];
    f.V[3 * p + 1] = v[1];
    f.V[3 * p + 2] = v[2];
    f.eid[p] = e;
    if (l) f.left[p] = 1;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}


// Pass 1: every live point from its frame-start state (ompVC/ftle.c:109-130),
// one thread per entry of the interval's compacted live list.
template <int D, int M, int I>
__global__ void __launch_bounds__(128, FVC_MINBLOCKS) k_ftle_pass1(DevMesh m, DevWindow w, DevInteg in, FtleDev f,
                                                    double t1, double t2, DevCounters* ctr) {
  clear_early_counters(ctr);
  const long nlive = *(volatile int*)&ctr->nlive;
  const int lane = threadIdx.x & 31;
  unsigned steps = 0;
  int err = 0;
  for (long base = warp_grab(&ctr->cur[0]); base < nlive; base = warp_grab(&ctr->cur[0])) {
    const long idx = base + lane;
    if (idx >= nlive) continue;
    long p = f.live[idx];
    Pt t;
    load_pt(t, p, f.X, in.extrapolate ? f.V : nullptr, f.eid, f.left, f.ldt);
    const unsigned before = steps;
    const RecOut r{f.rec + 3 * p, 3L * f.n, f.rec_steps, f.rec_e1 ? f.rec_e1 + p : nullptr, t.eid};
    err |= advect<D, M, false, I>(m, w, in, t, t1, t2, steps, nullptr, f.rec ? &r : nullptr);
    if (f.rec) f.kacc[p] = (unsigned char)(steps - before);
    f.flag[p] = 1 | ((t.left && !in.extrapolate) ? 2 : 0) | (t.left ? 4 : 0);
    f.Xn[3 * p] = t.X[0];
    f.Xn[3 * p + 1] = t.X[1];
    f.Xn[3 * p + 2] = t.X[2];
    if (in.extrapolate) {
      f.Vn[3 * p] = t.V[0];
      f.Vn[3 * p + 1] = t.V[1];
      f.Vn[3 * p + 2] = t.V[2];
    }
    f.en[p] = t.eid;
    f.te[p] = t.ldt;
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}

// Pass 2b: GetFTLEForPointEarly (ompVC/ftle.c:788-1048) for every served point
// q with its trigger's exit time te.  Its up to thirteen advections are queued
// as tasks so full warps run them:
//   A  each of q's six neighbours from its frame-start state to te
//   B  MinExitTime = min(te, the neighbours' exit times)   (ftle.c:878)
//   C  q itself to MinExitTime, and the neighbours again when MinExitTime
//      differs from te (Advect is deterministic: when it equals te, the
//      positions from A are the ones the reference recomputes)
//   D  the stencil, Cauchy-Green tensor and FTLE          (ftle.c:882-1046)
// Points the serial loop has passed before the trigger carry their
// end-of-interval element into these advections (ftle.c:167-168).
__device__ __forceinline__ void served_geometry(const FtleDev& f, long q, long nb[6], int& i, int& j, int& k) {
  int YZ = f.yr * f.zr, zr = f.zr;
  k = (int)(q % zr);
  j = (int)((q / zr) % f.yr);
  i = (int)(q / YZ);
  nb[0] = i > 0 ? q - YZ : -1;
  nb[1] = i < f.xr - 1 ? q + YZ : -1;
  nb[2] = j > 0 ? q - zr : -1;
  nb[3] = j < f.yr - 1 ? q + zr : -1;
  nb[4] = k > 0 ? q - 1 : -1;
  nb[5] = k < zr - 1 ? q + 1 : -1;
}

__device__ __forceinline__ int eid_at_trigger(const FtleDev& f, long pp, long trig) {
  return (pp < trig && (f.flag[pp] & 1) && !(f.flag[pp] & 2)) ? f.en[pp] : f.eid[pp];
}

// The length bucket of an advection from t1 to tend: its number of steps,
// capped at 7.  Only a sort key: advections of one bucket run together so a
// warp's lanes finish their step loops at about the same time.
__device__ __forceinline__ int length_bucket(double t1, double tend, double inv_h) {
  const double k = fabs(tend - t1) * inv_h + 0.5;
  return k < 7.0 ? (int)k : 7;
}

// Appends (s, c) with its bucket to the task list (the lanes of a warp land
// next to each other) and counts it in its bucket.
__device__ __forceinline__ void append_task(const FtleDev& f, TaskCounters* tc, bool want, int s, int c, int b) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0) base = atomicAdd(&tc->ntask, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (want) f.tasks[base + __popc(m & ((1u << lane) - 1u))] = make_int2(s, c | (b << 3));
  const unsigned peers = __match_any_sync(0xffffffffu, want ? b : -1);
  if (want && lane == __ffs(peers) - 1) atomicAdd(&tc->hist[b], __popc(peers));
}

// Groups the task list by bucket into f.tsorted (order within a bucket
// follows the warps' arrival, roughly the served points' grid order).
template <int D>
__global__ void k_task_sort(FtleDev f, TaskCounters* tc) {
  __shared__ int off[8];
  if (threadIdx.x == 0) {
    int a = 0;
    for (int b = 0; b < 8; b++) {
      off[b] = a;
      a += ((volatile int*)tc->hist)[b];
    }
  }
  __syncthreads();
  const long ntask = *(volatile int*)&tc->ntask;
  const int lane = threadIdx.x & 31;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long base = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < ntask; base += stride) {
    const long i = base + lane;
    const bool ok = i < ntask;
    const int2 t = ok ? f.tasks[i] : make_int2(0, 0);
    const int b = ok ? (t.y >> 3) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    if (ok) {
      const int leader = __ffs(peers) - 1;
      int pos = 0;
      if (lane == leader) pos = atomicAdd(&tc->scat[b], __popc(peers));
      pos = __shfl_sync(peers, pos, leader);
      f.tsorted[off[b] + pos + __popc(peers & ((1u << lane) - 1u))] = t;
    }
  }
}

// Steps of advections read from the record: counted with the early-FTLE
// steps (they are the advections ompVC performs) and on their own.
__device__ __forceinline__ void flush_rec(DevCounters* ctr, unsigned steps) {
  unsigned long long s = steps;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) {
    atomicAdd(&ctr->steps_early, s);
    atomicAdd(&ctr->steps_rec, s);
  }
}

// The index k of a step-start time T in the interval's step sequence (the
// position after k steps is the main pass's record k), or -1: FP64 form, the
// slot table's exact times tc_k = slot 2k; mixed form, the step table.
__device__ __forceinline__ int step_of(const DevWindow& w, int mixed, double T) {
  const long long b = __double_as_longlong(T);
  if (mixed) {
    for (int k = 0; k <= w.nsteps; k++)
      if (__double_as_longlong(w.steps[k].tc) == b) return k;
    return -1;
  }
  for (int k = 0; 2 * k < w.nslots; k++)
    if (__double_as_longlong(w.tq[2 * k]) == b) return k;
  return -1;
}

// The record's answer for an advection of point p from the interval's start
// to the step-start time of step kend (kend within the record; p advected
// this interval and not left before it): the position after min(kend, p's
// accepted steps), exiting on the way exactly when p exited before kend.
// Copies the position to pos, the exit or end time to lt, counts the steps.
__device__ __forceinline__ void from_record(const FtleDev& f, long p, int kend, double tend, double* pos,
                                            double* lt, unsigned* nsteps) {
  const unsigned char fl = f.flag[p];
  const int kx = f.kacc[p];
  const bool exits = (fl & 2) && kx < kend;
  const int k = exits ? kx : kend;
  const double* src = k == 0 ? f.X + 3 * p : f.rec + (long)(k - 1) * 3 * f.n + 3 * p;
  pos[0] = src[0];
  pos[1] = src[1];
  pos[2] = src[2];
  if (lt) *lt = exits ? f.te[p] : tend;
  *nsteps += (unsigned)k;
}

// Whether an early-FTLE advection of point p to the step-start time of step
// kend can be read from the main pass's record.  It repeats the main pass
// exactly when p was advected this interval, starts from its frame-start
// element (the hint eid_at_trigger gives it: not a point the serial loop has
// already moved, ompVC/ftle.c:167-168) and the record reaches kend.  Returns
// 1 with the result (from_record), 0 when it must be computed, and 2 when it
// starts from the interval's end element instead and everything else holds:
// in the FP64 form the walks from there may settle a tie on a shared face
// differently, so it is computed until its step-1 element state can be
// compared with the main pass's (FP64 RK4 with rec_e1; else 0).  The mixed
// form reads the record in that case too (on a shared face the P1 velocity is
// continuous, so the two differ by rounding only).
__device__ __forceinline__ int record_state(const FtleDev& f, long p, long trig, int kend) {
  if (!f.rec || kend < 0 || kend > f.rec_steps) return 0;
  const unsigned char fl = f.flag[p];
  if (!(fl & 1) || f.left[p]) return 0;
  if (!f.mixed && p < trig && !(fl & 2)) return (f.rec_e1 && kend >= 1) ? 2 : 0;
  return 1;
}

__device__ __forceinline__ int recorded(const FtleDev& f, long p, long trig, int kend, double tend, double* pos,
                                        double* lt, unsigned* nsteps) {
  const int r = record_state(f, p, trig, kend);
  if (r == 1) from_record(f, p, kend, tend, pos, lt, nsteps);
  return r;
}

// A: queue the neighbours that exist; boundary slots keep te as exit time.
// The queue kernels walk their items warp by warp (grid-stride, uniform per
// warp) so append_task's ballot always sees the whole warp.
template <int D>
__global__ void k_ftle_queue_nb(FtleDev f, DevWindow w, int mixed, DevCounters* ctr, double t1, double inv_h) {
  const long nserved = *(volatile int*)&ctr->count;
  const long total = 6 * nserved, stride = (long)gridDim.x * blockDim.x;
  unsigned rsteps = 0;
  for (long base = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    long idx = base + (threadIdx.x & 31);
    long s = idx / 6;
    int c = (int)(idx % 6);
    bool want = false;
    int b = 0;
    if (s < nserved) {
      long nb[6];
      int i, j, k;
      served_geometry(f, f.served[s], nb, i, j, k);
      want = nb[c] >= 0;
      const long trig = f.trig[s];
      const double te = f.te[trig];
      int r = 0;
      if (!want) f.elt[s * 6 + c] = te;
      else if (f.rec)
        r = recorded(f, nb[c], trig, step_of(w, mixed, te), te, f.epos + (s * 7 + c) * 3, f.elt + s * 6 + c, &rsteps);
      if (r == 1) want = false;
      // an advection checked after its first step mostly ends there
      b = r == 2 ? 1 : length_bucket(t1, te, inv_h);
    }
    append_task(f, &ctr->tq[0], want, (int)s, c, b);
  }
  flush_rec(ctr, rsteps);
}

// B + C queue: MinExitTime, then q itself and (if it moved) the neighbours.
template <int D>
__global__ void k_ftle_queue_self(FtleDev f, DevWindow w, int mixed, DevCounters* ctr, double t1, double inv_h) {
  unsigned rsteps = 0;
  const long nserved = *(volatile int*)&ctr->count;
  const long total = 7 * nserved, stride = (long)gridDim.x * blockDim.x;
  for (long base = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
  long idx = base + (threadIdx.x & 31);
  long s = idx / 7;
  int c = (int)(idx % 7);
  bool want = false;
  int b = 0;
  if (s < nserved) {
    double te = f.te[f.trig[s]];
    const double* lt = f.elt + s * 6;
    double mt = dmin(te, dmin(lt[5], dmin(lt[4], dmin(lt[3], dmin(lt[2], dmin(lt[1], lt[0]))))));
    b = length_bucket(t1, mt, inv_h);
    long p = -1;
    if (c == 6) {
      f.emt[s] = mt;
      want = true;
      p = f.served[s];
    } else if (mt != te) {
      long nb[6];
      int i, j, k;
      served_geometry(f, f.served[s], nb, i, j, k);
      want = nb[c] >= 0;
      p = nb[c];
    }
    if (want && f.rec) {
      const int r = recorded(f, p, f.trig[s], step_of(w, mixed, mt), mt, f.epos + (s * 7 + c) * 3, nullptr, &rsteps);
      if (r == 1) want = false;
      if (r == 2) b = 1;
    }
  }
  append_task(f, &ctr->tq[1], want, (int)s, c, b);
  }
  flush_rec(ctr, rsteps);
}

// The advections of A (phase 0: to te, recording exit times) and C (phase 1:
// to MinExitTime).
template <int D, int M, int I>
__global__ void __launch_bounds__(128, FVC_TASK_MINBLOCKS) k_ftle_tasks(DevMesh m, DevWindow w, DevInteg in, FtleDev f,
                                                                   double t1, int phase, DevCounters* ctr) {
  const long ntask = *(volatile int*)&ctr->tq[phase].ntask;
  int* cursor = &ctr->cur[1 + phase];
  unsigned steps = 0, rsteps = 0;
  int err = 0;
  for (long base = warp_grab(cursor); base < ntask; base = warp_grab(cursor)) {
    const long idx = base + (threadIdx.x & 31);
    if (idx >= ntask) continue;
    int2 tk = f.tsorted[idx];
    long s = tk.x;
    int c = tk.y & 7;
    long q = f.served[s], trig = f.trig[s];
    long nb[6];
    int i, j, k;
    served_geometry(f, q, nb, i, j, k);
    long p = c == 6 ? q : nb[c];
    double tend = phase == 0 ? f.te[trig] : f.emt[s];
    Pt t;
    t.X[0] = f.X[3 * p];
    t.X[1] = f.X[3 * p + 1];
    t.X[2] = f.X[3 * p + 2];
    t.V[0] = t.V[1] = t.V[2] = 0.0;
    t.left = f.left[p];
    t.eid = eid_at_trigger(f, p, trig);
    t.ldt = 0.0;
    double* pos = f.epos + (s * 7 + c) * 3;
    // started from the interval's end element (recorded() == 2): checked
    // against the main pass after step 1, and read from its record on a match
    const int kend = f.rec_e1 ? step_of(w, 0, tend) : -1;
    Chk1 chk;
    chk.hit = 0;
    const bool check = kend >= 1 && record_state(f, p, trig, kend) == 2;
    if (check) {
      chk.e0 = f.eid[p];
      chk.e1 = f.rec_e1[p];
    }
    unsigned st = 0;
    err |= advect<D, M, false, I>(m, w, in, t, t1, tend, st, nullptr, nullptr, check ? &chk : nullptr);
    if (chk.hit) {
      // step 1 was computed (st = 1); the record has the rest
      double lt;
      unsigned k = 0;
      from_record(f, p, kend, tend, pos, &lt, &k);
      steps += 1;
      rsteps += k - 1;
      if (phase == 0) f.elt[s * 6 + c] = lt;
      continue;
    }
    steps += st;
    pos[0] = t.X[0];
    pos[1] = t.X[1];
    pos[2] = t.X[2];
    if (phase == 0) f.elt[s * 6 + c] = t.left ? t.ldt : tend;
  }
  flush_counters(&ctr->steps_early, &ctr->status, steps, err);
  flush_rec(ctr, rsteps);
}

// (u.x - u.y) - (v.x - v.y) for two (X, c) float pairs, as a double: the
// difference of the X parts exactly by TwoSum, the compensations added to
// its error, the float sum split exactly into two floats (TwoSum again).
__device__ __forceinline__ double pair_diff(float2 u, float2 v) {
  const float s = u.x - v.x;
  const float b1 = s - u.x;
  const float e = (u.x - (s - b1)) + (-v.x - b1);
  const float t = (e - u.y) + v.y;
  const float h = s + t;
  const float b2 = h - s;
  const float l = (s - (h - b2)) + (t - b2);
  return (double)h + (double)l;
}

// GetFTLEForPointEarly's reduction (ompVC/ftle.c:900-1047) for served point
// s.  The eigenvalue comes from the closed form; where that is not accurate
// enough (jacobi false) the point is left for the Jacobi pass and false
// returned.
template <int D>
__device__ __forceinline__ bool early_final_one(const FtleDev& f, long s, bool jacobi) {
  long q = f.served[s];
  double mt = f.emt[s];
  long nb[6];
  int i, j, k;
  served_geometry(f, q, nb, i, j, k);
  // the stencil's positions among the seven (neighbours -x +x -y +y -z +z,
  // then q itself): lo / hi per direction, one-sided at the grid's faces
  int lo[3], hi[3];
  double fs[3];
  const int ext[3] = {i == 0 ? 0 : i == f.xr - 1 ? 2 : 1, j == 0 ? 0 : j == f.yr - 1 ? 2 : 1,
                      D != 3 ? 3 : k == 0 ? 0 : k == f.zr - 1 ? 2 : 1};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    lo[a] = ext[a] == 0 || ext[a] == 3 ? 6 : 2 * a;
    hi[a] = ext[a] == 2 || ext[a] == 3 ? 6 : 2 * a + 1;
    fs[a] = ext[a] == 1 ? 2.0 : 1.0;
  }
  double d[3][3];  // d[component][direction] = hi - lo
  const double* E = f.epos + s * 21;
  if (f.mixed) {
    // (X, c) float pairs, the position X - c: each difference formed in
    // FP32 without error (TwoSum) and carried as two floats
    const float2* E2 = reinterpret_cast<const float2*>(E);
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int c = 0; c < 3; c++) d[c][a] = pair_diff(E2[3 * hi[a] + c], E2[3 * lo[a] + c]);
  } else {
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int c = 0; c < 3; c++) d[c][a] = E[3 * hi[a] + c] - E[3 * lo[a] + c];
  }
  double C[3][3], lm1;  // C - I and lambda - 1
  tensor_from_diffs(D, d, fs[0], fs[1], fs[2], f.dx, f.dy, f.dz, C);
  if (jacobi) lm1 = max_eig(C);
  else if (!max_eig_closed(C, lm1)) return false;
  double wT = 0.0, wN = 0.0;
  if (lm1 > -FVC_TINY && !(fabs(mt - f.start) < FVC_TINY)) {
    wN = 0.5 * log1p(lm1);
    wT = wN / fabs(mt - f.start);
  }
  f.ftT[q] = wT;
  f.ftN[q] = wN;
  f.have[q] = 1;
  return true;
}

// The served points' FTLE by the closed-form eigenvalue; the few it leaves
// are listed (in the task array, free once the task kernels are done) for
// k_ftle_early_jacobi.
template <int D>
__global__ void k_ftle_early_final(FtleDev f, DevCounters* ctr) {
  const long nserved = *(volatile int*)&ctr->count;
  int* fall = reinterpret_cast<int*>(f.tasks);
  for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < nserved; s += (long)gridDim.x * blockDim.x)
    if (!early_final_one<D>(f, s, false)) fall[atomicAdd(&ctr->nfall, 1)] = (int)s;
}

template <int D>
__global__ void k_ftle_early_jacobi(FtleDev f, DevCounters* ctr) {
  const long nfall = *(volatile int*)&ctr->nfall;
  const int* fall = reinterpret_cast<const int*>(f.tasks);
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nfall; i += (long)gridDim.x * blockDim.x)
    early_final_one<D>(f, fall[i], true);
}

template <int D, int M>
__global__ void k_tracer_launch(DevMesh m, DevWindow w, TracerDev t, double tq, DevCounters* ctr) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  int err = 0;
  if (i < t.n && !t.left[i]) {
    double x[3] = {t.X[3 * i], t.X[3 * i + 1], t.X[3 * i + 2]}, v[3];
    int e = t.eid[i], l = 0;
    err = velocity<D, M>(m, w, tq, -1, x, e, l, v) | (M == 1 ? walk_fault(e) : 0);
    t.V[3 * i] = v[0];
    t.V[3 * i + 1] = v[1];
    t.V[3 * i + 2] = v[2];
    t.eid[i] = e;
    if (l) t.left[i] = 1;
  }
  flush_counters(&ctr->steps, &ctr->status, 0, err);
}


template <int D, int M, int I>
__global__ void __launch_bounds__(128, FVC_MINBLOCKS) k_tracer_advance(DevMesh m, DevWindow w, DevInteg in, TracerDev t,
                                                        double t1, double t2, DevCounters* ctr) {
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
      Pt p;
      load_pt(p, i, t.X, t.V, t.eid, t.left, t.ldt);
      err |= advect<D, M, false, I>(m, w, in, p, t1, t2, steps);
      t.X[3 * i] = p.X[0];
      t.X[3 * i + 1] = p.X[1];
      t.X[3 * i + 2] = p.X[2];
      t.V[3 * i] = p.V[0];
      t.V[3 * i + 1] = p.V[1];
      t.V[3 * i + 2] = p.V[2];
      t.eid[i] = p.eid;
      t.left[i] = p.left;
      t.ldt[i] = p.ldt;
      keep = p.ldt > -FVC_TINY && (!p.left || in.extrapolate);
    }
    if (L.next) append_live(t, L, keep, i);
  }
  flush_counters(&ctr->steps, &ctr->status, steps, err);
}



// The advection kernels come in two builds each: RK4 alone (I = 1, the
// common case, without the other integrators' registers and spills) and any
// integrator chosen at run time (I = -1).
template <int D, int M>
struct Variant {
  static void advect(const DevMesh& m, const DevWindow& w, const DevInteg& in, int n, double* X,
                     double* V, int* eid, int* left, double* ldt, double t0, double t1,
                     DevCounters* ctr, cudaStream_t s) {
    if (in.type == 1) k_advect<D, M, 1><<<vblk(n, 128), 128, 0, s>>>(m, w, in, n, X, V, eid, left, ldt, t0, t1, ctr);
    else k_advect<D, M, -1><<<vblk(n, 128), 128, 0, s>>>(m, w, in, n, X, V, eid, left, ldt, t0, t1, ctr);
  }
  static void velocity(const DevMesh& m, const DevWindow& w, int n, const double* X, int* eid,
                       int* left, double tq, double* out, DevCounters* ctr, cudaStream_t s) {
    k_velocity<D, M><<<vblk(n, 128), 128, 0, s>>>(m, w, n, X, eid, left, tq, out, ctr);
  }
  static void ftle_launch(const DevMesh& m, const DevWindow& w, const FtleDev& f, double t,
                          DevCounters* ctr, cudaStream_t s) {
    k_ftle_launch<D, M><<<vblk(f.n, 128), 128, 0, s>>>(m, w, f, t, ctr);
  }
  static void ftle_pass1(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                         double t1, double t2, DevCounters* ctr, cudaStream_t s) {
    static const unsigned res1 = resident_blocks(k_ftle_pass1<D, M, 1>, 128);
    static const unsigned res = resident_blocks(k_ftle_pass1<D, M, -1>, 128);
    if (in.type == 1) k_ftle_pass1<D, M, 1><<<capped(f.n, 128, res1), 128, 0, s>>>(m, w, in, f, t1, t2, ctr);
    else k_ftle_pass1<D, M, -1><<<capped(f.n, 128, res), 128, 0, s>>>(m, w, in, f, t1, t2, ctr);
  }
  static void ftle_early(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                         double t1, DevCounters* ctr, bool jacobi, cudaStream_t s) {
    static const unsigned res_nb = resident_blocks(k_ftle_queue_nb<D>, 256);
    static const unsigned res_self = resident_blocks(k_ftle_queue_self<D>, 256);
    static const unsigned res_tasks1 = resident_blocks(k_ftle_tasks<D, M, 1>, 128);
    static const unsigned res_tasks = resident_blocks(k_ftle_tasks<D, M, -1>, 128);
    static const unsigned res_final = resident_blocks(k_ftle_early_final<D>, 128);
    static const unsigned res_jacobi = resident_blocks(k_ftle_early_jacobi<D>, 64);
    static const unsigned res_sort = resident_blocks(k_task_sort<D>, 256);
    const double inv_h = 1.0 / fabs(in.h);
    // the task counters were cleared with the served count (ftle_triggers)
    k_ftle_queue_nb<D><<<capped(6L * f.n, 256, res_nb), 256, 0, s>>>(f, w, 0, ctr, t1, inv_h);
    k_task_sort<D><<<capped(6L * f.n, 256, res_sort), 256, 0, s>>>(f, &ctr->tq[0]);
    if (in.type == 1) k_ftle_tasks<D, M, 1><<<capped(6L * f.n, 128, res_tasks1), 128, 0, s>>>(m, w, in, f, t1, 0, ctr);
    else k_ftle_tasks<D, M, -1><<<capped(6L * f.n, 128, res_tasks), 128, 0, s>>>(m, w, in, f, t1, 0, ctr);
    k_ftle_queue_self<D><<<capped(7L * f.n, 256, res_self), 256, 0, s>>>(f, w, 0, ctr, t1, inv_h);
    k_task_sort<D><<<capped(7L * f.n, 256, res_sort), 256, 0, s>>>(f, &ctr->tq[1]);
    if (in.type == 1) k_ftle_tasks<D, M, 1><<<capped(7L * f.n, 128, res_tasks1), 128, 0, s>>>(m, w, in, f, t1, 1, ctr);
    else k_ftle_tasks<D, M, -1><<<capped(7L * f.n, 128, res_tasks), 128, 0, s>>>(m, w, in, f, t1, 1, ctr);
    k_ftle_early_final<D><<<capped(f.n, 128, res_final), 128, 0, s>>>(f, ctr);
    if (jacobi) k_ftle_early_jacobi<D><<<capped(f.n, 64, res_jacobi), 64, 0, s>>>(f, ctr);
  }
  static void tracer_launch(const DevMesh& m, const DevWindow& w, const TracerDev& t, double tq,
                            DevCounters* ctr, cudaStream_t s) {
    k_tracer_launch<D, M><<<vblk(t.n, 128), 128, 0, s>>>(m, w, t, tq, ctr);
  }
  static void tracer_advance(const DevMesh& m, const DevWindow& w, const DevInteg& in,
                             const TracerDev& t, double t1, double t2, DevCounters* ctr, cudaStream_t s) {
    static const unsigned res1 = resident_blocks(k_tracer_advance<D, M, 1>, 128);
    static const unsigned res = resident_blocks(k_tracer_advance<D, M, -1>, 128);
    if (in.type == 1) k_tracer_advance<D, M, 1><<<capped(t.n, 128, res1), 128, 0, s>>>(m, w, in, t, t1, t2, ctr);
    else k_tracer_advance<D, M, -1><<<capped(t.n, 128, res), 128, 0, s>>>(m, w, in, t, t1, t2, ctr);
  }
};

extern template struct Variant<2, 0>;
extern template struct Variant<3, 0>;
extern template struct Variant<2, 1>;
extern template struct Variant<3, 1>;

}  // namespace fvc
