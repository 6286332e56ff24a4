// fvc_batch.cu -- batched and served advection: many tracer, residence-time
// and FTLE jobs with their own seeds and integration windows, advanced
// together over the frames resident on the device.
//
// Schedule.  Time advances in ticks.  In one tick every active job runs its
// next frame interval -- exactly the interval ompVC's frame loop would give
// it (ompVC/main.c:170-227: the window [t_k, t_k+1] of two frames, the step
// sequence restarted at the interval's start and clipped at its end) -- so a
// job's arithmetic does not depend on which other jobs share its ticks:
// its results are identical alone and in any mix.  Jobs are admitted
// between ticks as device memory allows (an HBM budget over the jobs'
// footprints) and retired when their window ends; a fixed set of jobs can
// instead be captured whole into one CUDA graph.
//
// Device work per tick: one compaction kernel appends the live points of
// every active job to the tick's work queue (warp ballots, one atomic per
// warp), one persistent kernel advects the queue (each warp takes 32 entries
// at a time from a cursor), then each FTLE job runs its early-FTLE passes
// and update (the per-interval body of ComputeFTLE, ompVC/ftle.c:109-175)
// and, after its last interval, the FTLE reduction.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <deque>
#include <initializer_list>
#include <map>
#include <memory>
#include <vector>

#include "fvc_fpmath.cuh"
#include "fvc_internal.h"
#include "fvc_mixed_impl.cuh"

namespace fvc {

// The mixed form's view of one job's interval: the two frames' quantised
// pair records with their scales, and the interval's step table.
struct WinQ {
  const uint4* qp;
  float qs0[3], qs1[3];
  int qfmt;
  const StepM* steps;
  int nsteps;
};

// One frame interval of a job in a tick: its integration range and window
// (the FP64 form's frames, or the mixed form's pair records and step table).
struct BWin {
  double t1, t2;
  const DevWindow* w;
  WinQ q;
};

// One job's work in one tick, as the kernels see it.
struct BJob {
  int kind;             // 0 tracers (state advanced in place), 1 FTLE pass 1
  int n;                // points
  long long group0;     // first 32-point group of the job in the compaction grid
  double* X;            // positions (FP64, or (X, c) float pairs in the mixed form)
  int* eid;
  int* left;
  double* ldt;
  double* Xn;           // FTLE pass-1 outputs
  int* en;
  double* te;
  unsigned char* flag;
  DevCounters* ctr;     // the job's own counters
  double t1, t2;        // the interval's integration range
  const double4_32a* f0;  // FP64 window
  const double4_32a* f1;
  double tmin, tmax, rspan;
  WinQ q;
  const DevWindow* w;   // FP64 form: the job's window (two frames, no stage table)
  int nwin;             // frame intervals of this tick (tracer jobs may run several)
  const BWin* wins;     // their windows, in order (wins[0] is the one above)
  // FTLE pass 1: the per-step record the early-FTLE tasks read (null: none)
  double* rec;
  unsigned char* kacc;
  int4* rec_e1;
  int rec_steps;
};

struct BatchCtr {
  int nqueue;
  int cursor;
};

// The tick's work queue: (job, point) of every live point of every job
// (ldt > -TINY and not left, ompVC/ftle.c:113, tracers.c:225); FTLE jobs'
// per-interval flags are cleared on the way.
__global__ void k_batch_compact(const BJob* __restrict__ jobs, int njobs, long long ngroups, int2* queue,
                                BatchCtr* bc) {
  const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= ngroups) return;  // uniform per warp
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].group0 <= g) lo = mid;
    else hi = mid - 1;
  }
  const BJob& J = jobs[lo];
  const long i = (long)(g - J.group0) * 32 + lane;
  bool live = false;
  if (i < J.n) {
    live = J.ldt[i] > -FVC_TINY && !J.left[i];
    if (J.kind == 1) J.flag[i] = 0;
  }
  const unsigned b = __ballot_sync(0xffffffffu, live);
  int base = 0;
  if (lane == 0 && b) base = atomicAdd(&bc->nqueue, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (live) queue[base + __popc(b & ((1u << lane) - 1u))] = make_int2(lo, (int)i);
}

// Accepted steps and fault bits of the warp's 32 entries, added to each
// job's counters once per job present in the warp.
__device__ __forceinline__ void flush_jobs(const BJob* jobs, int jid, unsigned steps, int err) {
  const unsigned grp = __match_any_sync(0xffffffffu, jid);
  const unsigned s = __reduce_add_sync(grp, steps);
  const int e = (int)__reduce_or_sync(grp, (unsigned)err);
  if (jid >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) {
    DevCounters* c = jobs[jid].ctr;
    if (s) atomicAdd(&c->steps, (unsigned long long)s);
    if (e) atomicOr(&c->status, e);
  }
}

// The persistent advection of the mixed form over the tick's queue.
template <int D>
__global__ void __launch_bounds__(256, (FVC_MX_MINBLOCKS + 1) / 2) k_batch_advance_mx(DevMesh m, int type, const BJob* __restrict__ jobs,
                                                         const int2* __restrict__ queue, BatchCtr* bc) {
  const long nq = *(volatile int*)&bc->nqueue;
  for (long base = warp_grab(&bc->cursor); base < nq; base = warp_grab(&bc->cursor)) {
    const long idx = base + (threadIdx.x & 31);
    int jid = -1, err = 0;
    unsigned steps = 0;
    if (idx < nq) {
      const int2 e = queue[idx];
      jid = e.x;
      const BJob& J = jobs[jid];
      const long p = e.y;
      PtM t;
      load_pos_pair(J.X, p, t.X, t.c);
      t.eid = J.eid[p];
      t.left = J.left[p];
      t.ldt = J.ldt[p];
      // the job's intervals of this tick in order; a tracer that leaves is
      // not advanced further (the live test of every later interval).  An
      // FTLE job's pass 1 (one interval) writes its per-step record.
      const unsigned before = steps;
      const RecOut r{J.rec + 3 * p, 3L * J.n, J.rec_steps, nullptr, 0};
      const RecOut* rp = (J.kind == 1 && J.rec) ? &r : nullptr;
      for (int k = 0; k < J.nwin; k++) {
        const WinQ w = J.wins[k].q;
        advect_mx<D>(m, w, type, t, w.nsteps, steps, err, rp);
        if (t.left || err) break;
      }
      if (rp) J.kacc[p] = (unsigned char)(steps - before);
      if (J.kind == 0) {
        store_pos_pair(J.X, p, t.X, t.c);
        J.eid[p] = t.eid;
        J.left[p] = t.left;
        J.ldt[p] = t.ldt;
      } else {
        J.flag[p] = 1 | (t.left ? 6 : 0);
        store_pos_pair(J.Xn, p, t.X, t.c);
        J.en[p] = t.eid;
        J.te[p] = t.ldt;
      }
    }
    flush_jobs(jobs, jid, steps, err);
  }
}

// The same in the FP64 form (ompVC's arithmetic): each stage interpolates the
// job's two frames itself (the window carries no stage-time table).  I = 1:
// built for RK4 alone; -1: the integrator chosen at run time.
template <int D, int I>
__global__ void __launch_bounds__(256, FVC_MINBLOCKS / 2) k_batch_advance(DevMesh m, DevInteg in,
                                                                      const BJob* __restrict__ jobs,
                                                                      const int2* __restrict__ queue,
                                                                      BatchCtr* bc) {
  const long nq = *(volatile int*)&bc->nqueue;
  for (long base = warp_grab(&bc->cursor); base < nq; base = warp_grab(&bc->cursor)) {
    const long idx = base + (threadIdx.x & 31);
    int jid = -1, err = 0;
    unsigned steps = 0;
    if (idx < nq) {
      const int2 e = queue[idx];
      jid = e.x;
      const BJob& J = jobs[jid];
      const long p = e.y;
      Pt t;
      load_pt(t, p, J.X, nullptr, J.eid, J.left, J.ldt);
      const unsigned before = steps;
      const RecOut r{J.rec + 3 * p, 3L * J.n, J.rec_steps, J.rec_e1 ? J.rec_e1 + p : nullptr, t.eid};
      const RecOut* rp = (J.kind == 1 && J.rec) ? &r : nullptr;
      for (int k = 0; k < J.nwin; k++) {
        const BWin& W = J.wins[k];
        err |= advect<D, 1, false, I>(m, *W.w, in, t, W.t1, W.t2, steps, nullptr, rp);
        if (t.left || err) break;
      }
      if (rp) J.kacc[p] = (unsigned char)(steps - before);
      if (J.kind == 0) {
        J.X[3 * p] = t.X[0];
        J.X[3 * p + 1] = t.X[1];
        J.X[3 * p + 2] = t.X[2];
        J.eid[p] = t.eid;
        J.left[p] = t.left;
        J.ldt[p] = t.ldt;
      } else {
        J.flag[p] = 1 | (t.left ? 6 : 0);
        J.Xn[3 * p] = t.X[0];
        J.Xn[3 * p + 1] = t.X[1];
        J.Xn[3 * p + 2] = t.X[2];
        J.en[p] = t.eid;
        J.te[p] = t.ldt;
      }
    }
    flush_jobs(jobs, jid, steps, err);
  }
}

// Launch geometry of the persistent advection, chosen by the autotuner.
struct BatchLaunch {
  int threads;  // block size
  int blocks;   // grid (resident blocks, or fewer)
};

static unsigned batch_resident(int dims, int prec, int threads) {
  if (prec) return dims == 3 ? resident_blocks(k_batch_advance_mx<3>, threads)
                             : resident_blocks(k_batch_advance_mx<2>, threads);
  return dims == 3 ? resident_blocks(k_batch_advance<3, 1>, threads) : resident_blocks(k_batch_advance<2, 1>, threads);
}

static void batch_advance(const DevMesh& m, const DevInteg& in, const BJob* jobs, const int2* queue, BatchCtr* bc,
                          const BatchLaunch& L, cudaStream_t s) {
  if (m.prec) {
    if (m.dims == 3) k_batch_advance_mx<3><<<L.blocks, L.threads, 0, s>>>(m, in.type, jobs, queue, bc);
    else k_batch_advance_mx<2><<<L.blocks, L.threads, 0, s>>>(m, in.type, jobs, queue, bc);
  } else {
    if (in.type == 1) {
      if (m.dims == 3) k_batch_advance<3, 1><<<L.blocks, L.threads, 0, s>>>(m, in, jobs, queue, bc);
      else k_batch_advance<2, 1><<<L.blocks, L.threads, 0, s>>>(m, in, jobs, queue, bc);
    } else {
      if (m.dims == 3) k_batch_advance<3, -1><<<L.blocks, L.threads, 0, s>>>(m, in, jobs, queue, bc);
      else k_batch_advance<2, -1><<<L.blocks, L.threads, 0, s>>>(m, in, jobs, queue, bc);
    }
  }
}

// ---- the tick's work queue ordered by job, then by a Z-order of the
// entries' current positions over the mesh's box (2^(3 bits) cells): a
// counting sort, key histogram, scan, scatter.  Entries of one job and cell
// stay together, so warps walk neighbouring elements and read one frame pair
// even after a release has dispersed; the particle arrays are not moved.

__global__ void k_qkeys(const BJob* __restrict__ jobs, const int2* queue, const BatchCtr* bc, int mixed, int bits,
                        double3 lo, double3 inv, int* key, int* hist) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *(volatile const int*)&bc->nqueue) return;
  const int2 e = queue[i];
  const double* X = jobs[e.x].X + 3L * e.y;
  double x[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (mixed) {
      const float2 p = *reinterpret_cast<const float2*>(X + a);
      x[a] = (double)p.x;
    } else {
      x[a] = X[a];
    }
  }
  const double l[3] = {lo.x, lo.y, lo.z}, sc[3] = {inv.x, inv.y, inv.z};
  const unsigned top = (1u << bits) - 1u;
  unsigned code = 0;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double f = (x[a] - l[a]) * sc[a];
    const unsigned c = f < 0.0 ? 0u : f >= (double)top ? top : (unsigned)f;
    for (int b = 0; b < bits; b++) code |= ((c >> b) & 1u) << (3 * b + a);
  }
  const int k = (int)(((unsigned)e.x << (3 * bits)) | code);
  key[i] = k;
  atomicAdd(hist + k, 1);
}

__global__ void k_qscatter(const int2* queue, const BatchCtr* bc, const int* key, const int* off, int* cur,
                           int2* out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *(volatile const int*)&bc->nqueue) return;
  const int k = key[i];
  out[off[k] + atomicAdd(cur + k, 1)] = queue[i];
}

// ---- spatial ordering of a release's tracers (Z-order of 64^3 cells over
// the seeds' box): a warp's 32 tracers then walk neighbouring elements and
// share their records and frame nodes in cache.  Advection is independent
// per tracer, so the order changes no result; results are read back in seed
// order through the permutation.

__device__ __forceinline__ unsigned spread6(unsigned v) {  // 6 bits -> every third bit
  unsigned r = 0;
#pragma unroll
  for (int b = 0; b < 6; b++) r |= ((v >> b) & 1u) << (3 * b);
  return r;
}

__global__ void k_zkeys(const double* X, int n, int packed, double3 lo, double3 inv, int* key, int* hist) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double v = X[3 * i + a];
    if (packed) {
      const float2 p = *reinterpret_cast<const float2*>(&X[3 * i + a]);
      x[a] = (double)p.x - (double)p.y;
    } else {
      x[a] = v;
    }
  }
  const double l[3] = {lo.x, lo.y, lo.z}, s[3] = {inv.x, inv.y, inv.z};
  unsigned c[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double f = (x[a] - l[a]) * s[a];
    c[a] = f < 0.0 ? 0u : f > 63.0 ? 63u : (unsigned)f;
  }
  const int k = (int)(spread6(c[0]) | (spread6(c[1]) << 1) | (spread6(c[2]) << 2));
  key[i] = k;
  atomicAdd(hist + k, 1);
}

__global__ void k_zscatter(const int* key, int n, const int* off, int* cur, int* perm) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = key[i];
  perm[off[k] + atomicAdd(cur + k, 1)] = (int)i;
}

// out[j] = in[perm[j]] for the tracer state (X, V as 3 doubles, eid, left, ldt)
__global__ void k_zgather(TracerDev t, const int* perm, double* X2, double* V2, int* e2, int* l2, double* d2) {
  long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= t.n) return;
  const long i = perm[j];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    X2[3 * j + a] = t.X[3 * i + a];
    V2[3 * j + a] = t.V[3 * i + a];
  }
  e2[j] = t.eid[i];
  l2[j] = t.left[i];
  d2[j] = t.ldt[i];
}

// inv[perm[j]] = j: the device position of each seed
__global__ void k_zinverse(const int* perm, int n, int* inv) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) inv[perm[j]] = (int)j;
}

// A finished tracer job's state in seed order, written straight into the
// result's page-locked block: positions (the mixed form's (X, c) pairs
// joined to FP64, as the host-side unpacking does), exit data and the
// residence times of OutputRT (ompVC/residencetime.c:160-178, as k_residence).
__global__ void k_res_tracer(TracerDev t, const int* inv, int packed, double launch, double stop, double* X,
                             double* ldt, double* rt, int* eid, int* left) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.n) return;
  const long j = inv ? inv[i] : i;
#pragma unroll
  for (int a = 0; a < 3; a++)
    X[3 * i + a] = packed ? join_pos(reinterpret_cast<const float2*>(t.X)[3 * j + a]) : t.X[3 * j + a];
  const double d = t.ldt[j];
  const int l = t.left[j];
  ldt[i] = d;
  rt[i] = fabs(d + 1) < FVC_TINY ? -1.0 : (l ? d : stop) - launch;
  eid[i] = t.eid[j];
  left[i] = l;
}

}  // namespace fvc

// ====================================================================== host

namespace {

constexpr double kTiny = 1.0e-10;

enum { JQ_QUEUED = 0, JQ_ACTIVE = 1, JQ_FINISHING = 2, JQ_DONE = 3, JQ_FAILED = 4, JQ_RELEASED = 5 };

struct HostJob {
  int id = 0;
  int kind = 0;  // FVC_JOB_*
  int state = JQ_QUEUED;
  fvc_batch_job_spec spec{};
  std::vector<double> seeds;
  fvc_job* job = nullptr;
  int slot = -1;
  int dir = 1;
  double stop = 0.0, T = 0.0;
  long long df = 0;      // next frame interval (unwrapped index), moving in dir
  bool launched = false;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
  long long ticks = 0;
  long npts = 0;  // points (work-queue entries at most)
  int* d_inv = nullptr;   // tracers: seed index -> device position (null: seed order)
  int per_tick = 1;       // frame intervals a tick advances the job by
  int res_held = 0;       // result tickets held on the job
  fvc_status err = FVC_OK;
  std::string msg;
};

// A frame pair's quantised records (the mixed form's window of one interval).
struct PairQ {
  uint4* q = nullptr;
  float s0[3], s1[3];
  int fmt = 0;
};

// Per-point device bytes of a job (the carve lists of fvc_tracer_create /
// fvc_ftle_create, rounded up) and the seed-chain scratch.
size_t job_bytes(int kind, long n) {
  if (kind == FVC_JOB_FTLE) return (size_t)n * 560 + (1u << 20);
  return (size_t)n * 134 + (1u << 20);
}

// An FTLE job's per-step record (the steps of one interval, at most 32, as
// the single-job interval keeps it): positions, accepted steps, step-1
// element states.
int rec_steps_of(double tdelta, double h) {
  const double k = ceil(tdelta / fabs(h)) + 1.0;
  return k < 32.0 ? (int)k : 32;
}
size_t rec_bytes_of(long n, int want) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return al(24 * (size_t)n * (size_t)want) + al((size_t)n) + 16 * (size_t)n;
}

}  // namespace

static constexpr int FTLE_SIDE_STREAMS = 4;

struct fvc_batch {
  fvc_ctx* c = nullptr;
  fvc_batch_opts o{};
  std::vector<std::unique_ptr<HostJob>> jobs;
  std::deque<int> queued;
  std::vector<int> active;
  std::vector<int> finishing;
  size_t used = 0;
  int max_jobs = 1024;
  // device state
  DevCounters* d_ctrs = nullptr;  // one block per job slot
  DevCounters* h_ctrs = nullptr;  // pinned copies, written after each job's last tick
  std::vector<int> free_slots;
  BatchCtr* d_bc = nullptr;
  int2* d_queue = nullptr;
  size_t queue_cap = 0;  // entries
  size_t queue_need = 0;
  char* d_tick = nullptr;
  size_t tick_cap = 0;
  char* h_tick[2] = {nullptr, nullptr};
  size_t h_cap[2] = {0, 0};
  cudaEvent_t h_ev[2] = {nullptr, nullptr};
  int hbuf = 0;
  std::map<std::pair<int, int>, PairQ> pairs;
  std::vector<cudaEvent_t> tick_ev;  // ring of the last ticks, for the in-flight limit
  cudaEvent_t t_start = nullptr, t_end = nullptr;
  BatchLaunch launch{128, 0};
  fvc_batch_stats stats{};
  // queue ordering (resort_every > 0): sorted copy of the queue, keys and
  // the counting sort's arrays (room for QSORT_KEYS keys)
  int resort = 0;
  int2* d_queue2 = nullptr;
  int* d_qkey = nullptr;
  size_t qsort_cap = 0;  // entries
  int* d_qhist = nullptr;  // hist, off (+1), cur
  long long* d_qtmp = nullptr;
  // results of finished jobs are read on a stream of their own, after the
  // job's last tick (its done event), so reading them never waits for the
  // ticks still in flight
  cudaStream_t res_stream = nullptr;
  // result tickets: FVC_BATCH_RESULT_SLOTS page-locked blocks for the
  // caller, and one more for the blocking result calls
  struct ResSlot {
    unsigned char* h = nullptr;
    size_t cap = 0;
    cudaEvent_t ev = nullptr;
    long long ticket = -1;
    int job = -1;
    bool busy = false;
    fvc_batch_result r{};
  };
  ResSlot res[FVC_BATCH_RESULT_SLOTS + 1];
  long long res_next = 0;
  // admission (seed upload and location, Z-ordering) runs on a stream of
  // its own, so its waits do not drain the ticks in flight
  cudaStream_t setup_stream = nullptr;
  // the FTLE jobs' per-interval kernels (early FTLE, update) of a tick are
  // spread over these streams, forked after the tick's advection and joined
  // before its end: the jobs' small launches run side by side
  cudaStream_t side[FTLE_SIDE_STREAMS] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[FTLE_SIDE_STREAMS] = {};
};

static constexpr int QSORT_KEYS = 1 << 22;

// ticks a batch may have queued on the GPU before fvc_batch_tick waits for
// the oldest (build knob)
#ifndef FVC_BATCH_INFLIGHT
#define FVC_BATCH_INFLIGHT 2
#endif

using namespace fvc;

static int frame_mod(const fvc_batch* b, long long frame) {
  long long per = b->o.tres - 1;
  long long m = frame % per;
  if (m < 0) m += per;
  return (int)m;
}

static fvc_status batch_fail(fvc_batch* b, fvc_status code, const char* what) {
  return fail(b->c, code, "%s", what);
}

// One interval of a job: (frame_lo, tmin, tmax) of interval df, the
// integration range and whether it is the job's last (flow of
// ompVC/main.c:170-227 with one FTLE slide or one tracer release).
struct Interval {
  long long lo;
  double tmin, tmax, t1, t2;
  bool launch, last;
};

static Interval interval_at(const fvc_batch* b, const HostJob& J, long long df, bool launched) {
  Interval I{};
  I.lo = J.dir > 0 ? df : df - 1;
  I.tmin = b->o.tmin + (double)I.lo * b->o.tdelta;
  I.tmax = I.tmin + b->o.tdelta;
  I.launch = !launched;
  const double t0 = J.spec.t_start;
  I.t1 = I.launch ? t0 : (J.dir > 0 ? I.tmin : I.tmax);
  I.t2 = J.dir > 0 ? std::min(I.tmax, J.stop) : std::max(I.tmin, J.stop);
  I.last = (J.dir > 0 ? (J.stop - I.tmax) : (I.tmin - J.stop)) < kTiny;
  return I;
}

static Interval interval_of(const fvc_batch* b, const HostJob& J) { return interval_at(b, J, J.df, J.launched); }

// The first frame interval of a window starting at t0 (ompVC/parameters.c:
// 322-333 for one slide).
static long long first_interval(const fvc_batch* b, double t0, int dir) {
  double x = (t0 - b->o.tmin) / b->o.tdelta;
  return dir > 0 ? (long long)floor(x) : (long long)ceil(x);
}

// The mixed form's step table of [t1, t2] in the window [tmin, tmax]: the
// stage times of the FP64 step loop (ompVC/integration.c:345-352, 402), as
// the single-job calls build it.
static bool build_steps_for(double h0, double tmin, double tmax, double t1, double t2, std::vector<StepM>& T) {
  T.clear();
  auto tloc = [&](double tq, float& out) {
    double tl = (tq - tmin) / (tmax - tmin);
    if ((tl > 1 + 1.0e-10) || (tl < 0 - 1.0e-10)) return false;
    out = (float)tl;
    return true;
  };
  double tc = t1, h = (t2 - t1) >= 0.0 ? fabs(h0) : -fabs(h0);
  while ((tc - t2) * (t2 - t1) < 0.0) {
    if ((tc + h - t2) * (tc + h - t1) > 0.0) h = (t2 - t1) >= 0.0 ? fabs(t2 - tc) : -fabs(t2 - tc);
    StepM s{};
    s.tc = tc;
    s.h = (float)h;
    if (!tloc(tc, s.tl0) || !tloc(tc + h / 2, s.tlh) || !tloc(tc + h, s.tl1)) return false;
    T.push_back(s);
    tc = tc + h;
  }
  StepM e{};
  e.tc = tc;
  T.push_back(e);
  return true;
}

static fvc_status ensure_pair(fvc_batch* b, int lo, int hi, PairQ** out) {
  fvc_ctx* c = b->c;
  auto key = std::make_pair(lo, hi);
  PairQ& P = b->pairs[key];
  if (!P.q || P.fmt != c->prec) {
    fvc_ctx::QFrame *qa = nullptr, *qb = nullptr;
    if (!c->frames.count(lo) || !c->frames.count(hi)) return fail(c, FVC_ERR_STATE, "frames %d / %d are not resident", lo, hi);
    fvc_status st;
    if ((st = quantised(c, lo, &qa)) || (st = quantised(c, hi, &qb))) return st;
    if (!P.q && cudaMalloc(&P.q, sizeof(uint4) * (size_t)c->frame_nodes) != cudaSuccess) {
      P.q = nullptr;
      return fail(c, FVC_ERR_OOM, "quantised frame pair");
    }
    pair_frames(qa->q, qb->q, c->frame_nodes, P.q, c->stream);
    if ((st = check_launch(c, "pair frames"))) return st;
    for (int k = 0; k < 3; k++) {
      P.s0[k] = qa->s[k];
      P.s1[k] = qb->s[k];
    }
    P.fmt = c->prec;
  }
  *out = &P;
  return FVC_OK;
}

// The host view of a job's window for the per-job kernels (launch velocity,
// early FTLE): FP64 frames without a stage table, or the quantised pair and
// the interval's step table at d_steps.
static fvc_status job_window(fvc_batch* b, const Interval& I, const StepM* d_steps, int nsteps, DevWindow& w,
                             BJob& J) {
  fvc_ctx* c = b->c;
  const int flo = frame_mod(b, I.lo), fhi = frame_mod(b, I.lo + 1);
  auto a = c->frames.find(flo), z = c->frames.find(fhi);
  if (a == c->frames.end() || z == c->frames.end())
    return fail(c, FVC_ERR_STATE, "frames %d / %d are not resident", flo, fhi);
  frame_dep(c, flo);
  frame_dep(c, fhi);
  memset(&w, 0, sizeof(w));
  w.f0 = a->second;
  w.f1 = z->second;
  w.tmin = I.tmin;
  w.tmax = I.tmax;
  w.rspan = rcp_for_div(I.tmax - I.tmin);
  w.nslots = 0;
  J.f0 = w.f0;
  J.f1 = w.f1;
  J.tmin = w.tmin;
  J.tmax = w.tmax;
  J.rspan = w.rspan;
  J.t1 = I.t1;
  J.t2 = I.t2;
  memset(&J.q, 0, sizeof(J.q));
  if (c->prec) {
    PairQ* P = nullptr;
    fvc_status st;
    if ((st = ensure_pair(b, flo, fhi, &P))) return st;
    w.qp = P->q;
    for (int k = 0; k < 3; k++) {
      w.qs0[k] = P->s0[k];
      w.qs1[k] = P->s1[k];
    }
    w.qfmt = c->prec;
    w.steps = d_steps;
    w.nsteps = nsteps;
    J.q.qp = w.qp;
    memcpy(J.q.qs0, w.qs0, sizeof(w.qs0));
    memcpy(J.q.qs1, w.qs1, sizeof(w.qs1));
    J.q.qfmt = w.qfmt;
    J.q.steps = d_steps;
    J.q.nsteps = nsteps;
  }
  return FVC_OK;
}

// ------------------------------------------------------------ admission

// Reorders a located release's tracers along the Z-order curve of 64^3 cells
// over the seeds' bounding box (counting sort: key histogram, scan, scatter,
// gather) and keeps the inverse permutation on the device, for putting
// results back in seed order.
static fvc_status zorder_tracers(fvc_batch* b, HostJob& J) {
  fvc_ctx* c = b->c;
  TracerDev& t = J.job->t;
  const int n = t.n;
  if (n < 64) return FVC_OK;
  int* d_inv = (int*)pool_get(c, 4 * (size_t)n);
  if (!d_inv) return FVC_OK;  // no room: keep seed order
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (long i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) {
      lo[a] = std::min(lo[a], J.seeds[3 * i + a]);
      hi[a] = std::max(hi[a], J.seeds[3 * i + a]);
    }
  double3 dlo = make_double3(lo[0], lo[1], lo[2]), inv;
  double* ip = &inv.x;
  for (int a = 0; a < 3; a++) ip[a] = hi[a] > lo[a] ? 64.0 / (hi[a] - lo[a]) : 0.0;
  const int K = 1 << 18;
  const size_t nb = (size_t)n;
  char* mem = nullptr;
  const size_t bytes = 4 * nb * 2 + 4 * (3 * (size_t)K + 2) + 8 * ((size_t)K / 1024 + 2) + 64 * nb + 256 * 16;
  mem = (char*)pool_get(c, bytes);
  if (!mem) {
    pool_put(c, d_inv, 4 * (size_t)n);
    return FVC_OK;  // no room: keep seed order
  }
  char* q = mem;
  auto take = [&](size_t sz) { char* r = q; q += (sz + 255) & ~(size_t)255; return r; };
  int* key = (int*)take(4 * nb);
  int* perm = (int*)take(4 * nb);
  int* hist = (int*)take(4 * (size_t)K);
  int* off = (int*)take(4 * ((size_t)K + 1));
  int* cur = (int*)take(4 * (size_t)K);
  long long* tmp = (long long*)take(8 * ((size_t)K / 1024 + 2));
  double* X2 = (double*)take(24 * nb);
  double* V2 = (double*)take(24 * nb);
  int* e2 = (int*)take(4 * nb);
  int* l2 = (int*)take(4 * nb);
  double* d2 = (double*)take(8 * nb);
  cudaStream_t s = c->stream;
  const unsigned g = (unsigned)((n + 255) / 256);
  cudaMemsetAsync(hist, 0, 4 * (size_t)K, s);
  cudaMemsetAsync(cur, 0, 4 * (size_t)K, s);
  k_zkeys<<<g, 256, 0, s>>>(t.X, n, J.job->packed ? 1 : 0, dlo, inv, key, hist);
  scan_counts(hist, off, K, tmp, s);
  k_zscatter<<<g, 256, 0, s>>>(key, n, off, cur, perm);
  k_zgather<<<g, 256, 0, s>>>(t, perm, X2, V2, e2, l2, d2);
  cudaMemcpyAsync(t.X, X2, 24 * nb, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(t.V, V2, 24 * nb, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(t.eid, e2, 4 * nb, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(t.left, l2, 4 * nb, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(t.ldt, d2, 8 * nb, cudaMemcpyDeviceToDevice, s);
  k_zinverse<<<g, 256, 0, s>>>(perm, n, d_inv);
  fvc_status st = check_launch(c, "z-order");
  cudaError_t e = cudaStreamSynchronize(s);
  pool_put(c, mem, bytes);
  if (st || e != cudaSuccess) {
    pool_put(c, d_inv, 4 * (size_t)n);
    return st ? st : fail(c, FVC_ERR_CUDA, "z-order: %s", cudaGetErrorString(e));
  }
  J.d_inv = d_inv;
  b->stats.launches += 7;
  return FVC_OK;
}

// The job's device state is made on the batch's setup stream: the creation
// calls wait for their own work (seed location is host-driven), and on the
// context's stream that wait would take the ticks in flight with it.  Every
// creation call returns after its work has completed, so the ticks that use
// the job, issued later on the context's stream, see it.  The blocks the
// creation takes from the context's pool were returned by jobs whose last
// kernels have completed.
struct SetupStream {
  fvc_ctx* c;
  cudaStream_t main;
  SetupStream(fvc_batch* b) : c(b->c), main(b->c->stream) {
    if (b->setup_stream) c->stream = b->setup_stream;
  }
  ~SetupStream() { c->stream = main; }
};

static fvc_status admit_one(fvc_batch* b, HostJob& J) {
  fvc_ctx* c = b->c;
  fvc_status st;
  {
    SetupStream on_setup(b);
    if (J.kind == FVC_JOB_FTLE) {
      fvc_ftle_spec sp = J.spec.grid;
      sp.start_time = J.spec.t_start;
      sp.stop_time = J.stop;
      sp.generate = 1;
      st = fvc_ftle_create(c, &sp, &J.job);
      if (!st) {
        // the main pass's per-step record, from which early-FTLE advections
        // that repeat it are read (without room, they are computed)
        fvc_job* j = J.job;
        const int want = rec_steps_of(b->o.tdelta, c->integ.h);
        const size_t n = (size_t)j->f.n;
        j->rec_bytes = rec_bytes_of((long)n, want);
        j->rec_mem = pool_get(c, j->rec_bytes);
        if (j->rec_mem) {
          j->rec_cap = want;
          const size_t pos = (24 * n * (size_t)want + 255) & ~(size_t)255;
          j->f.rec = nullptr;  // per interval, from the tick's plan
          j->f.kacc = (unsigned char*)j->rec_mem + pos;
          j->f.rec_e1 = (!j->prec && c->integ.type == 1) ? (int4*)((char*)j->rec_mem + pos + ((n + 255) & ~(size_t)255))
                                                          : nullptr;
        } else {
          j->rec_bytes = 0;
          j->f.rec = nullptr;
          j->f.kacc = nullptr;
          j->f.rec_e1 = nullptr;
        }
        j->f.rec_steps = 0;
      }
    } else {
      fvc_tracer_spec sp{};
      sp.local_search_checking = J.spec.local_search_checking;
      sp.seed_chain = 0;
      st = fvc_tracer_create(c, &sp, J.spec.n, J.seeds.data(), &J.job);
      if (!st) st = zorder_tracers(b, J);
    }
  }
  if (st) return st;
  J.slot = b->free_slots.back();
  b->free_slots.pop_back();
  FVC_CUDA(c, cudaMemsetAsync(b->d_ctrs + J.slot, 0, sizeof(DevCounters), c->stream));
  if (!J.done) cudaEventCreateWithFlags(&J.done, cudaEventDisableTiming);
  J.df = first_interval(b, J.spec.t_start, J.dir);
  J.launched = false;
  J.state = JQ_ACTIVE;
  b->used += J.bytes;
  J.npts = J.kind == FVC_JOB_FTLE ? J.job->f.n : J.job->t.n;
  b->queue_need += (size_t)J.npts;
  b->active.push_back(J.id);
  return FVC_OK;
}

// Admits queued jobs in submission order while their footprint fits the
// budget (a job larger than the whole budget runs alone) and slots are free.
static fvc_status admit(fvc_batch* b) {
  while (!b->queued.empty()) {
    HostJob& J = *b->jobs[b->queued.front()];
    const bool alone = b->active.empty() && b->finishing.empty();
    if (b->o.hbm_budget > 0 && b->used + J.bytes > (size_t)b->o.hbm_budget && !alone) break;
    if (b->free_slots.empty()) break;
    b->queued.pop_front();
    fvc_status st = admit_one(b, J);
    if (st) {
      J.state = JQ_FAILED;
      J.err = st;
      J.msg = b->c->err;
      if (J.job) {
        fvc_job_destroy(J.job);
        J.job = nullptr;
      }
    }
  }
  if (b->queue_need > b->queue_cap) {
    fvc_ctx* c = b->c;
    FVC_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(b->d_queue);
    b->d_queue = nullptr;
    size_t cap = std::max(b->queue_need, (size_t)2 * b->queue_cap);
    if (cudaMalloc(&b->d_queue, sizeof(int2) * cap) != cudaSuccess) {
      b->queue_cap = 0;
      return fail(c, FVC_ERR_OOM, "batch work queue (%zu entries)", cap);
    }
    b->queue_cap = cap;
  }
  return FVC_OK;
}

// ------------------------------------------------------------ one tick

// The tick's descriptors (BJob array, then the step tables) in a host blob,
// with the device address each part will have at dev_base.
struct TickPlan {
  std::vector<char> blob;
  std::vector<int> ids;           // job ids in BJob order
  std::vector<Interval> iv;       // per job: its first interval of the tick
  std::vector<int> nint;          // per job: intervals in the tick
  std::vector<int> rec_steps;     // per FTLE job: the record's steps this interval (0: none)
  std::vector<char> last;         // per job: the tick ends the job's window
  std::vector<DevWindow> win;     // per job (launch velocity, early FTLE)
  long long ngroups = 0;
  long long npts = 0;             // points of the tick's jobs (queue entries at most)
};

static size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// The tick's layout: BJob[jobs] | BWin[intervals] | DevWindow[intervals]
// (FP64 form) | step tables (mixed form), one window per interval.
static fvc_status plan_tick(fvc_batch* b, const std::vector<int>& ids, char* dev_base, TickPlan& P) {
  fvc_ctx* c = b->c;
  P.ids = ids;
  const size_t nj = ids.size();
  P.iv.resize(nj);
  P.nint.resize(nj);
  P.rec_steps.assign(nj, 0);
  P.last.resize(nj);
  P.win.resize(nj);
  // every job's intervals of this tick: one for FTLE jobs, up to per_tick
  // for releases, never past the window's last
  std::vector<std::vector<Interval>> ivs(nj);
  size_t nw = 0;
  for (size_t k = 0; k < nj; k++) {
    const HostJob& H = *b->jobs[ids[k]];
    const int K = H.kind == FVC_JOB_FTLE ? 1 : H.per_tick;
    long long df = H.df;
    bool launched = H.launched;
    for (int i = 0; i < K; i++) {
      const Interval I = interval_at(b, H, df, launched);
      ivs[k].push_back(I);
      if (I.last) break;
      df += H.dir;
      launched = true;
    }
    nw += ivs[k].size();
    P.iv[k] = ivs[k].front();
    P.nint[k] = (int)ivs[k].size();
    P.last[k] = ivs[k].back().last;
  }
  size_t off = al16(sizeof(BJob) * nj);
  const size_t bwoff = off;
  off = al16(off + sizeof(BWin) * nw);
  const size_t woff = off;  // FP64 form: the intervals' windows
  if (!c->prec) off = al16(off + sizeof(DevWindow) * nw);
  std::vector<std::vector<StepM>> tabs(nw);
  std::vector<size_t> toff(nw, 0);
  if (c->prec) {
    size_t wi = 0;
    for (size_t k = 0; k < nj; k++)
      for (const Interval& I : ivs[k]) {
        if (!build_steps_for(c->integ.h, I.tmin, I.tmax, I.t1, I.t2, tabs[wi]))
          return fail(c, FVC_ERR_TLOC, "batch job %d: query time outside the loaded frame interval", ids[k]);
        toff[wi] = off;
        off = al16(off + sizeof(StepM) * tabs[wi].size());
        wi++;
      }
  }
  P.blob.assign(off, 0);
  std::vector<BJob> J(nj);
  std::vector<BWin> W(nw);
  long long groups = 0;
  size_t wi = 0;
  for (size_t k = 0; k < nj; k++) {
    HostJob& H = *b->jobs[ids[k]];
    BJob& B = J[k];
    memset(&B, 0, sizeof(B));
    B.nwin = (int)ivs[k].size();
    B.wins = (const BWin*)(dev_base + bwoff + sizeof(BWin) * wi);
    for (size_t i = 0; i < ivs[k].size(); i++, wi++) {
      const StepM* dsteps = c->prec ? (const StepM*)(dev_base + toff[wi]) : nullptr;
      const int nsteps = c->prec ? (int)tabs[wi].size() - 1 : 0;
      DevWindow w;
      BJob tmp;
      memset(&tmp, 0, sizeof(tmp));
      fvc_status st = job_window(b, ivs[k][i], dsteps, nsteps, w, i == 0 ? B : tmp);
      if (st) return st;
      const BJob& src = i == 0 ? B : tmp;
      W[wi].t1 = ivs[k][i].t1;
      W[wi].t2 = ivs[k][i].t2;
      W[wi].q = src.q;
      if (c->prec) {
        memcpy(P.blob.data() + toff[wi], tabs[wi].data(), sizeof(StepM) * tabs[wi].size());
      } else {
        memcpy(P.blob.data() + woff + sizeof(DevWindow) * wi, &w, sizeof(DevWindow));
        W[wi].w = (const DevWindow*)(dev_base + woff + sizeof(DevWindow) * wi);
      }
      if (i == 0) {
        P.win[k] = w;
        B.w = W[wi].w;
      }
    }
    B.ctr = b->d_ctrs + H.slot;
    B.group0 = groups;
    if (H.kind == FVC_JOB_FTLE) {
      // the record's steps this interval (as the single-job interval keeps
      // them: the interval's steps, at most the record's room), for the
      // pass (here) and the job's early-FTLE kernels (enqueue_tick)
      const FtleDev& f = H.job->f;
      int rs = 0;
      if (H.job->rec_mem) {
        int ns;
        if (c->prec) {
          ns = (int)tabs[wi - 1].size() - 1;
        } else {
          std::vector<StepM> T;
          const Interval& I = ivs[k][0];
          ns = build_steps_for(c->integ.h, I.tmin, I.tmax, I.t1, I.t2, T) ? (int)T.size() - 1 : 0;
        }
        const int want = ns < 32 ? ns : 32;
        rs = (want > 0 && H.job->rec_cap >= want) ? want : 0;
      }
      P.rec_steps[k] = rs;
      B.rec = rs > 0 ? (double*)H.job->rec_mem : nullptr;
      B.kacc = f.kacc;
      B.rec_e1 = f.rec_e1;
      B.rec_steps = rs;
      B.kind = 1;
      B.n = f.n;
      B.X = f.X;
      B.eid = f.eid;
      B.left = f.left;
      B.ldt = f.ldt;
      B.Xn = f.Xn;
      B.en = f.en;
      B.te = f.te;
      B.flag = f.flag;
    } else {
      const TracerDev& t = H.job->t;
      B.kind = 0;
      B.n = t.n;
      B.X = t.X;
      B.eid = t.eid;
      B.left = t.left;
      B.ldt = t.ldt;
    }
    groups += (B.n + 31) / 32;
    P.npts += B.n;
  }
  memcpy(P.blob.data(), J.data(), sizeof(BJob) * nj);
  if (nw) memcpy(P.blob.data() + bwoff, W.data(), sizeof(BWin) * nw);
  P.ngroups = groups;
  return FVC_OK;
}

// Enqueues a planned tick whose descriptors are at d_jobs on the stream.
// Room for ordering a queue of `need` entries (outside capture only).
static fvc_status ensure_qsort(fvc_batch* b, size_t need) {
  fvc_ctx* c = b->c;
  if (!b->d_qhist) {
    if (cudaMalloc(&b->d_qhist, sizeof(int) * (3 * (size_t)QSORT_KEYS + 2)) != cudaSuccess ||
        cudaMalloc(&b->d_qtmp, sizeof(long long) * ((size_t)QSORT_KEYS / 1024 + 2)) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "queue ordering arrays");
  }
  if (need > b->qsort_cap) {
    FVC_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(b->d_queue2);
    cudaFree(b->d_qkey);
    b->d_queue2 = nullptr;
    b->d_qkey = nullptr;
    b->qsort_cap = 0;
    if (cudaMalloc(&b->d_queue2, sizeof(int2) * need) != cudaSuccess ||
        cudaMalloc(&b->d_qkey, sizeof(int) * need) != cudaSuccess)
      return fail(c, FVC_ERR_OOM, "queue ordering (%zu entries)", need);
    b->qsort_cap = need;
  }
  return FVC_OK;
}

// Whether tick `t` orders its queue.
static bool resorts(const fvc_batch* b, long long t) { return b->resort > 0 && t % b->resort == 0; }

// Orders the tick's queue (in d_queue) into d_queue2 by job and position.
static bool order_queue(fvc_batch* b, const TickPlan& P, const BJob* d_jobs, cudaStream_t s) {
  fvc_ctx* c = b->c;
  const int nj = (int)P.ids.size();
  int jb = 0;
  while ((1 << jb) < nj) jb++;
  int bits = (22 - jb) / 3;
  if (bits < 1) return false;  // too many jobs for the key range: leave the order
  bits = bits > 6 ? 6 : bits;
  const long long K = (long long)nj << (3 * bits);
  if (K > QSORT_KEYS) return false;
  double3 lo = make_double3(c->node_lo[0], c->node_lo[1], c->node_lo[2]), inv;
  double* ip = &inv.x;
  for (int a = 0; a < 3; a++) {
    const double ext = c->node_hi[a] - c->node_lo[a];
    ip[a] = ext > 0 ? (double)(1 << bits) / ext : 0.0;
  }
  int* hist = b->d_qhist;
  int* off = hist + QSORT_KEYS;
  int* cur = off + QSORT_KEYS + 1;
  cudaMemsetAsync(hist, 0, sizeof(int) * (size_t)K, s);
  cudaMemsetAsync(cur, 0, sizeof(int) * (size_t)K, s);
  const unsigned g = (unsigned)((P.npts + 255) / 256);
  k_qkeys<<<g, 256, 0, s>>>(d_jobs, b->d_queue, b->d_bc, c->prec ? 1 : 0, bits, lo, inv, b->d_qkey, hist);
  scan_counts(hist, off, (int)K, b->d_qtmp, s);
  k_qscatter<<<g, 256, 0, s>>>(b->d_queue, b->d_bc, b->d_qkey, off, cur, b->d_queue2);
  b->stats.launches += 5;
  return true;
}

static fvc_status enqueue_tick(fvc_batch* b, const TickPlan& P, const BJob* d_jobs, bool counters_cleared,
                               long long tick) {
  fvc_ctx* c = b->c;
  cudaStream_t s = c->stream;
  const size_t nj = P.ids.size();
  if (!counters_cleared) FVC_CUDA(c, cudaMemsetAsync(b->d_bc, 0, sizeof(BatchCtr), s));
  // releases / slide launches: the velocity at the start time
  for (size_t k = 0; k < nj; k++) {
    HostJob& H = *b->jobs[P.ids[k]];
    if (!P.iv[k].launch) continue;
    if (H.kind == FVC_JOB_FTLE) ftle_launch(c->mesh, P.win[k], H.job->f, H.job->f.start, b->d_ctrs + H.slot, s);
    else tracer_launch_vel(c->mesh, P.win[k], H.job->t, H.spec.t_start, b->d_ctrs + H.slot, s);
    b->stats.launches++;
  }
  if (P.ngroups > 0) {
    const unsigned nb = (unsigned)((P.ngroups + 7) / 8);
    k_batch_compact<<<nb, 256, 0, s>>>(d_jobs, (int)nj, P.ngroups, b->d_queue, b->d_bc);
    const int2* q = b->d_queue;
    if (resorts(b, tick) && b->qsort_cap >= (size_t)P.npts && order_queue(b, P, d_jobs, s)) q = b->d_queue2;
    batch_advance(c->mesh, c->integ, d_jobs, q, b->d_bc, b->launch, s);
    b->stats.launches += 2;
  }
  // the FTLE jobs' per-interval work, spread over the side streams
  int nftle = 0;
  for (size_t k = 0; k < nj; k++) nftle += b->jobs[P.ids[k]]->kind == FVC_JOB_FTLE;
  const int nside = std::min(nftle > 1 ? nftle : 0, FTLE_SIDE_STREAMS);
  if (nside) {
    FVC_CUDA(c, cudaEventRecord(b->fork, s));
    for (int q = 0; q < nside; q++) FVC_CUDA(c, cudaStreamWaitEvent(b->side[q], b->fork, 0));
  }
  int fj = 0;
  for (size_t k = 0; k < nj; k++) {
    HostJob& H = *b->jobs[P.ids[k]];
    if (H.kind != FVC_JOB_FTLE) continue;
    cudaStream_t s = nside ? b->side[fj++ % nside] : c->stream;
    DevCounters* ctr = b->d_ctrs + H.slot;
    FtleDev f = H.job->f;  // with this interval's record, which the pass wrote
    f.rec = P.rec_steps[k] > 0 ? (double*)H.job->rec_mem : nullptr;
    f.rec_steps = P.rec_steps[k];
    // the task lists' work cursors start at 0 every interval
    FVC_CUDA(c, cudaMemsetAsync(ctr->cur, 0, sizeof(ctr->cur), s));
    ftle_triggers(f, ctr, false, s);
    ftle_early(c->mesh, P.win[k], c->integ, f, P.iv[k].t1, ctr, true, s);
    ftle_update(c->mesh, c->integ, f, nullptr, s);
    b->stats.launches += 2 + (H.job->prec ? 6 : 8);
    if (P.last[k]) {
      if (H.job->packed) {
        unpack_pairs(H.job->f.X, 3L * f.n, s);
        H.job->packed = false;
        b->stats.launches++;
      }
      ftle_final(f, c->mesh.dims, H.T, s);
      b->stats.launches++;
    }
  }
  for (int q = 0; q < nside; q++) {
    FVC_CUDA(c, cudaEventRecord(b->join[q], b->side[q]));
    FVC_CUDA(c, cudaStreamWaitEvent(c->stream, b->join[q], 0));
  }
  return check_launch(c, "batch tick");
}

// Bookkeeping after a tick was planned and enqueued: interval cursors, jobs
// whose window ended move to the finishing list with an event behind them.
static void advance_cursors(fvc_batch* b, const TickPlan& P) {
  std::vector<int> still;
  for (size_t k = 0; k < P.ids.size(); k++) {
    HostJob& H = *b->jobs[P.ids[k]];
    H.launched = true;
    H.df += (long long)H.dir * P.nint[k];
    H.ticks += P.nint[k];
    if (P.last[k]) {
      cudaMemcpyAsync(b->h_ctrs + H.slot, b->d_ctrs + H.slot, sizeof(DevCounters), cudaMemcpyDeviceToHost,
                      b->c->stream);
      cudaEventRecord(H.done, b->c->stream);
      H.state = JQ_FINISHING;
      b->queue_need -= (size_t)H.npts;
      b->finishing.push_back(H.id);
    } else {
      still.push_back(H.id);
    }
  }
  b->active.swap(still);
}

// Device room for a tick's descriptors (waits for the ticks in flight when
// it has to grow).
static fvc_status ensure_tick_cap(fvc_batch* b, size_t bytes) {
  fvc_ctx* c = b->c;
  if (bytes > b->tick_cap) {
    FVC_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(b->d_tick);
    b->d_tick = nullptr;
    size_t cap = std::max(bytes, (size_t)2 * b->tick_cap);
    if (cudaMalloc(&b->d_tick, cap) != cudaSuccess) {
      b->tick_cap = 0;
      return fail(c, FVC_ERR_OOM, "batch descriptors");
    }
    b->tick_cap = cap;
  }
  return FVC_OK;
}

static fvc_status stage_upload(fvc_batch* b, const std::vector<char>& blob) {
  fvc_ctx* c = b->c;
  const size_t bytes = blob.size();
  fvc_status st;
  if ((st = ensure_tick_cap(b, bytes))) return st;
  int k = b->hbuf;
  b->hbuf ^= 1;
  FVC_CUDA(c, cudaEventSynchronize(b->h_ev[k]));
  if (bytes > b->h_cap[k]) {
    cudaFreeHost(b->h_tick[k]);
    b->h_tick[k] = nullptr;
    size_t cap = std::max(bytes, (size_t)2 * b->h_cap[k]);
    if (cudaMallocHost(&b->h_tick[k], cap) != cudaSuccess) {
      b->h_cap[k] = 0;
      return fail(c, FVC_ERR_OOM, "pinned batch staging");
    }
    b->h_cap[k] = cap;
  }
  memcpy(b->h_tick[k], blob.data(), bytes);
  FVC_CUDA(c, cudaMemcpyAsync(b->d_tick, b->h_tick[k], bytes, cudaMemcpyHostToDevice, c->stream));
  FVC_CUDA(c, cudaEventRecord(b->h_ev[k], c->stream));
  return FVC_OK;
}

// Retires finishing jobs whose last tick has completed: reads their counters
// and marks them done (or failed with the counters' fault).
static void retire(fvc_batch* b, bool wait) {
  std::vector<int> still;
  for (int id : b->finishing) {
    HostJob& H = *b->jobs[id];
    cudaError_t q = wait ? cudaEventSynchronize(H.done) : cudaEventQuery(H.done);
    if (q == cudaErrorNotReady) {
      still.push_back(id);
      continue;
    }
    const DevCounters h = b->h_ctrs[H.slot];
    H.job->stats.steps_main += (long long)h.steps;
    H.job->stats.steps_early += (long long)h.steps_early;
    H.job->stats.intervals += H.ticks;
    b->stats.steps += (long long)(h.steps + h.steps_early);
    b->stats.jobs_done++;
    if (q != cudaSuccess) {
      H.state = JQ_FAILED;
      H.err = FVC_ERR_CUDA;
      H.msg = cudaGetErrorString(q);
    } else if (h.status) {
      H.state = JQ_FAILED;
      H.err = (h.status & PT_ERR_STATE) ? FVC_ERR_STATE : (h.status & PT_ERR_TLOC) ? FVC_ERR_TLOC : FVC_ERR_WALK;
      H.msg = "device fault while advancing the job";
    } else {
      H.state = JQ_DONE;
    }
  }
  b->finishing.swap(still);
}

static fvc_status tick(fvc_batch* b) {
  fvc_ctx* c = b->c;
  fvc_status st;
  if ((st = use_device(c))) return st;
  retire(b, false);
  if ((st = admit(b))) return st;
  if (b->active.empty()) return FVC_OK;
  TickPlan P;
  if ((st = plan_tick(b, b->active, b->d_tick, P))) return st;
  // the step tables' device addresses depend on where the blob lands
  if (P.blob.size() > b->tick_cap) {
    if ((st = ensure_tick_cap(b, P.blob.size()))) return st;
    if ((st = plan_tick(b, b->active, b->d_tick, P))) return st;
  }
  if ((st = stage_upload(b, P.blob))) return st;
  if (b->resort > 0 && (st = ensure_qsort(b, (size_t)P.npts))) return st;
  if ((st = enqueue_tick(b, P, (const BJob*)b->d_tick, false, b->stats.ticks))) return st;
  advance_cursors(b, P);
  // at most two ticks in flight: the host plans the next while one runs
  cudaEvent_t& e = b->tick_ev[b->stats.ticks % b->tick_ev.size()];
  if (b->stats.ticks >= (long long)b->tick_ev.size()) FVC_CUDA(c, cudaEventSynchronize(e));
  FVC_CUDA(c, cudaEventRecord(e, c->stream));
  b->stats.ticks++;
  return FVC_OK;
}

// --------------------------------------------------------------- autotune

// Times the persistent advection of one planned tick for each candidate
// block size (and half occupancy) on a copy of the jobs' state and keeps the
// fastest.  The state is restored afterwards, so tuning changes no result.
static fvc_status autotune(fvc_batch* b) {
  fvc_ctx* c = b->c;
  if (b->active.empty()) return FVC_OK;
  fvc_status st;
  TickPlan P;
  if ((st = plan_tick(b, b->active, b->d_tick, P))) return st;
  if (P.blob.size() > b->tick_cap) {
    if ((st = ensure_tick_cap(b, P.blob.size()))) return st;
    if ((st = plan_tick(b, b->active, b->d_tick, P))) return st;
  }
  if ((st = stage_upload(b, P.blob))) return st;
  // snapshot every job's mutable state
  std::vector<std::pair<void*, size_t>> regions;
  size_t total = 0;
  for (int id : b->active) {
    HostJob& H = *b->jobs[id];
    size_t n = H.kind == FVC_JOB_FTLE ? (size_t)H.job->f.n : (size_t)H.job->t.n;
    if (H.kind == FVC_JOB_FTLE) {
      regions.push_back({H.job->f.Xn, 24 * n});
      regions.push_back({H.job->f.en, 4 * n});
      regions.push_back({H.job->f.te, 8 * n});
      regions.push_back({H.job->f.flag, n});
    } else {
      regions.push_back({H.job->t.X, 24 * n});
      regions.push_back({H.job->t.eid, 4 * n});
      regions.push_back({H.job->t.left, 4 * n});
      regions.push_back({H.job->t.ldt, 8 * n});
    }
    regions.push_back({b->d_ctrs + H.slot, sizeof(DevCounters)});
  }
  for (auto& r : regions) total += r.second;
  char* save = nullptr;
  if (cudaMalloc(&save, total) != cudaSuccess) return FVC_OK;  // no room to tune: keep the default
  size_t o = 0;
  for (auto& r : regions) {
    cudaMemcpyAsync(save + o, r.first, r.second, cudaMemcpyDeviceToDevice, c->stream);
    o += r.second;
  }
  const BJob* dj = (const BJob*)b->d_tick;
  const int cand_threads[3] = {64, 128, 256};
  float best = 1e30f;
  BatchLaunch bestL = b->launch;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int ti = 0; ti < 3; ti++) {
    const unsigned res = batch_resident(c->mesh.dims, c->prec, cand_threads[ti]);
    for (int half = 0; half < 2; half++) {
      BatchLaunch L{cand_threads[ti], (int)std::max(1u, half ? res / 2 : res)};
      cudaMemsetAsync(b->d_bc, 0, sizeof(BatchCtr), c->stream);
      const unsigned nb = (unsigned)((P.ngroups + 7) / 8);
      k_batch_compact<<<nb, 256, 0, c->stream>>>(dj, (int)P.ids.size(), P.ngroups, b->d_queue, b->d_bc);
      cudaEventRecord(e0, c->stream);
      batch_advance(c->mesh, c->integ, dj, b->d_queue, b->d_bc, L, c->stream);
      cudaEventRecord(e1, c->stream);
      // restore before the next candidate
      o = 0;
      for (auto& r : regions) {
        cudaMemcpyAsync(r.first, save + o, r.second, cudaMemcpyDeviceToDevice, c->stream);
        o += r.second;
      }
      if (cudaStreamSynchronize(c->stream) != cudaSuccess) break;
      float ms = ev_ms(e0, e1);
      if (ms > 0 && ms < best) {
        best = ms;
        bestL = L;
      }
    }
  }
  // the re-sort interval, when left to the tuner: the best shape once more
  // with the queue ordered (ordering included in the time); ordering every
  // tick is kept only if that is faster
  if (b->o.resort_every == -1) {
    fvc_status qs = ensure_qsort(b, (size_t)P.npts);
    b->resort = 0;
    if (!qs) {
      cudaMemsetAsync(b->d_bc, 0, sizeof(BatchCtr), c->stream);
      const unsigned nb = (unsigned)((P.ngroups + 7) / 8);
      k_batch_compact<<<nb, 256, 0, c->stream>>>(dj, (int)P.ids.size(), P.ngroups, b->d_queue, b->d_bc);
      cudaEventRecord(e0, c->stream);
      const bool ordered = order_queue(b, P, dj, c->stream);
      batch_advance(c->mesh, c->integ, dj, ordered ? b->d_queue2 : b->d_queue, b->d_bc, bestL, c->stream);
      cudaEventRecord(e1, c->stream);
      o = 0;
      for (auto& r : regions) {
        cudaMemcpyAsync(r.first, save + o, r.second, cudaMemcpyDeviceToDevice, c->stream);
        o += r.second;
      }
      if (cudaStreamSynchronize(c->stream) == cudaSuccess && ordered) {
        const float ms = ev_ms(e0, e1);
        if (ms > 0 && ms < 0.97f * best) b->resort = 1;
      }
    }
    b->stats.tuned_resort = b->resort;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(save);
  b->launch = bestL;
  b->stats.tuned_threads = bestL.threads;
  b->stats.tuned_blocks = bestL.blocks;
  return check_launch(c, "batch autotune");
}

// ============================================================== C ABI

extern "C" fvc_status fvc_batch_create(fvc_ctx* c, const fvc_batch_opts* o, fvc_batch** out) {
  if (!c || !o || !out) return FVC_ERR_ARG;
  *out = nullptr;
  fvc_status st;
  if ((st = use_device(c))) return st;
  if (!c->mesh_set || c->mesh.mesh_type != 1) return fail(c, FVC_ERR_STATE, "the batch form needs an unstructured mesh");
  if (o->tres < 2 || !(o->tdelta > 0)) return fail(c, FVC_ERR_ARG, "batch time axis: tres >= 2 and tdelta > 0");
  if (c->integ.type != 0 && c->integ.type != 1) return fail(c, FVC_ERR_ARG, "the batch form runs Euler (0) or RK4 (1)");
  if (c->integ.extrapolate) return fail(c, FVC_ERR_ARG, "the batch form does not extrapolate");
  if ((st = mixed_ok(c))) return st;
  fvc_batch* b = new fvc_batch();
  b->c = c;
  b->o = *o;
  b->max_jobs = o->max_jobs > 0 ? o->max_jobs : 1024;
  if (cudaMalloc(&b->d_ctrs, sizeof(DevCounters) * (size_t)b->max_jobs) != cudaSuccess ||
      cudaMallocHost(&b->h_ctrs, sizeof(DevCounters) * (size_t)b->max_jobs) != cudaSuccess ||
      cudaMalloc(&b->d_bc, sizeof(BatchCtr)) != cudaSuccess) {
    fvc_batch_destroy(b);
    return fail(c, FVC_ERR_OOM, "batch counters");
  }
  for (int k = b->max_jobs - 1; k >= 0; k--) b->free_slots.push_back(k);
  for (int k = 0; k < 2; k++) cudaEventCreateWithFlags(&b->h_ev[k], cudaEventDisableTiming);
  b->tick_ev.resize(FVC_BATCH_INFLIGHT);
  for (auto& e : b->tick_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  cudaEventCreate(&b->t_start);
  cudaEventCreate(&b->t_end);
  b->launch.threads = 128;
  b->launch.blocks = (int)batch_resident(c->mesh.dims, c->prec, 128);
  b->resort = o->resort_every > 0 ? o->resort_every : 0;
  b->stats.tuned_resort = b->resort;
  if (cudaStreamCreateWithFlags(&b->res_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->setup_stream, cudaStreamNonBlocking) != cudaSuccess) {
    fvc_batch_destroy(b);
    return fail(c, FVC_ERR_CUDA, "batch result / setup stream");
  }
  bool side_ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < FTLE_SIDE_STREAMS && side_ok; k++)
    side_ok = cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming) == cudaSuccess;
  if (!side_ok) {
    fvc_batch_destroy(b);
    return fail(c, FVC_ERR_CUDA, "batch side streams");
  }
  *out = b;
  return check_launch(c, "batch create");
}

extern "C" void fvc_batch_destroy(fvc_batch* b) {
  if (!b) return;
  fvc_ctx* c = b->c;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (b->res_stream) cudaStreamSynchronize(b->res_stream);
  for (auto& J : b->jobs) {
    if (J->job) {
      if (J->d_inv) pool_put(c, J->d_inv, 4 * (size_t)J->job->t.n);
      fvc_job_destroy(J->job);
    }
    if (J->done) cudaEventDestroy(J->done);
  }
  for (auto& kv : b->pairs) cudaFree(kv.second.q);
  cudaFree(b->d_queue2);
  cudaFree(b->d_qkey);
  cudaFree(b->d_qhist);
  cudaFree(b->d_qtmp);
  cudaFree(b->d_ctrs);
  cudaFreeHost(b->h_ctrs);
  cudaFree(b->d_bc);
  cudaFree(b->d_queue);
  cudaFree(b->d_tick);
  for (int k = 0; k < 2; k++) {
    cudaFreeHost(b->h_tick[k]);
    if (b->h_ev[k]) cudaEventDestroy(b->h_ev[k]);
  }
  for (auto& e : b->tick_ev) cudaEventDestroy(e);
  if (b->t_start) cudaEventDestroy(b->t_start);
  if (b->t_end) cudaEventDestroy(b->t_end);
  if (b->res_stream) {
    cudaStreamSynchronize(b->res_stream);
    cudaStreamDestroy(b->res_stream);
  }
  if (b->setup_stream) {
    cudaStreamSynchronize(b->setup_stream);
    cudaStreamDestroy(b->setup_stream);
  }
  for (int k = 0; k < FTLE_SIDE_STREAMS; k++) {
    if (b->side[k]) {
      cudaStreamSynchronize(b->side[k]);
      cudaStreamDestroy(b->side[k]);
    }
    if (b->join[k]) cudaEventDestroy(b->join[k]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  for (auto& r : b->res) {
    cudaFreeHost(r.h);
    if (r.ev) cudaEventDestroy(r.ev);
  }
  delete b;
}

extern "C" fvc_status fvc_batch_submit(fvc_batch* b, const fvc_batch_job_spec* sp, int* id) {
  if (!b || !sp || !id) return FVC_ERR_ARG;
  fvc_ctx* c = b->c;
  if (sp->kind != FVC_JOB_TRACERS && sp->kind != FVC_JOB_RESIDENCE && sp->kind != FVC_JOB_FTLE)
    return fail(c, FVC_ERR_ARG, "unknown job kind %d", sp->kind);
  if (!(sp->t_stop != sp->t_start)) return fail(c, FVC_ERR_ARG, "empty integration window");
  if (sp->kind == FVC_JOB_RESIDENCE && sp->t_stop < sp->t_start)
    return fail(c, FVC_ERR_ARG, "residence time is computed forward in time (ompVC/parameters.c:541-542)");
  if (sp->kind != FVC_JOB_FTLE && (sp->n < 0 || (sp->n > 0 && !sp->seeds)))
    return fail(c, FVC_ERR_ARG, "bad seed array");
  std::unique_ptr<HostJob> J(new HostJob());
  J->id = (int)b->jobs.size();
  J->kind = sp->kind;
  J->spec = *sp;
  J->dir = sp->t_stop > sp->t_start ? 1 : -1;
  J->T = fabs(sp->t_stop - sp->t_start);
  const double tmax = b->o.tmin + (b->o.tres - 1) * b->o.tdelta;
  J->stop = sp->t_stop;
  if (!b->o.periodic) {
    if (sp->t_start < b->o.tmin || sp->t_start > tmax) return fail(c, FVC_ERR_ARG, "start time outside the data range");
    J->stop = std::max(std::min(sp->t_stop, tmax), b->o.tmin);
  }
  long n;
  if (sp->kind == FVC_JOB_FTLE) {
    const fvc_ftle_spec& g = sp->grid;
    n = (long)g.xres * g.yres * (c->mesh.dims == 3 ? g.zres : 1);
    if (g.xres < 2 || g.yres < 2 || (c->mesh.dims == 3 && g.zres < 2)) return fail(c, FVC_ERR_ARG, "FTLE grid too small");
  } else {
    n = sp->n;
    J->seeds.assign(sp->seeds, sp->seeds + 3 * (size_t)sp->n);
  }
  J->spec.seeds = nullptr;
  J->bytes = job_bytes(sp->kind, n);
  if (sp->kind == FVC_JOB_FTLE) J->bytes += rec_bytes_of(n, rec_steps_of(b->o.tdelta, c->integ.h));
  if (sp->kind != FVC_JOB_FTLE && b->o.tick_intervals > 0) {
    // the frame intervals the window touches, at most; a long release runs
    // several of them per tick
    const double nint = ceil(fabs(J->stop - sp->t_start) / b->o.tdelta) + 1.0;
    J->per_tick = (int)std::min(64.0, std::max(1.0, ceil(nint / (double)b->o.tick_intervals)));
  }
  *id = J->id;
  b->queued.push_back(J->id);
  b->jobs.push_back(std::move(J));
  b->stats.jobs_submitted++;
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_tick(fvc_batch* b, int* pending) {
  if (!b) return FVC_ERR_ARG;
  fvc_status st = tick(b);
  if (pending) *pending = (int)(b->queued.size() + b->active.size() + b->finishing.size());
  return st;
}

extern "C" fvc_status fvc_batch_autotune(fvc_batch* b) {
  if (!b) return FVC_ERR_ARG;
  fvc_status st;
  if ((st = use_device(b->c))) return st;
  if ((st = admit(b))) return st;
  return autotune(b);
}

extern "C" fvc_status fvc_batch_run(fvc_batch* b, int graph) {
  if (!b) return FVC_ERR_ARG;
  fvc_ctx* c = b->c;
  fvc_status st;
  if ((st = use_device(c))) return st;
  cudaEventRecord(b->t_start, c->stream);
  if ((st = admit(b))) return st;
  if (graph && b->queued.empty() && !b->active.empty()) {
    // the whole remaining schedule is fixed: plan every tick, upload all
    // descriptors once, capture the ticks into one graph and launch it
    std::vector<TickPlan> plans;
    std::vector<size_t> offs;
    size_t total = 0;
    // plan with cursors moved on a copy of the host state
    std::vector<HostJob> saved;
    for (int id : b->active) saved.push_back(*b->jobs[id]);
    std::vector<int> act = b->active;
    while (!act.empty()) {
      plans.emplace_back();
      offs.push_back(total);
      if ((st = plan_tick(b, act, nullptr, plans.back()))) break;  // sizes and pairs
      total = al16(total + plans.back().blob.size());
      std::vector<int> still;
      for (size_t k = 0; k < act.size(); k++) {
        HostJob& H = *b->jobs[act[k]];
        H.launched = true;
        H.df += (long long)H.dir * plans.back().nint[k];
        if (!plans.back().last[k]) still.push_back(act[k]);
      }
      act.swap(still);
    }
    for (size_t k = 0; k < saved.size(); k++) {  // restore the cursors
      HostJob& H = *b->jobs[saved[k].id];
      H.df = saved[k].df;
      H.launched = saved[k].launched;
    }
    if (st) return st;
    char* d_all = nullptr;
    if (cudaMalloc(&d_all, total ? total : 16) != cudaSuccess) return fail(c, FVC_ERR_OOM, "graph descriptors");
    std::vector<char> all(total);
    act = b->active;
    for (size_t t = 0; t < plans.size(); t++) {
      if ((st = plan_tick(b, act, d_all + offs[t], plans[t]))) break;
      memcpy(all.data() + offs[t], plans[t].blob.data(), plans[t].blob.size());
      std::vector<int> still;
      for (size_t k = 0; k < act.size(); k++) {
        HostJob& H = *b->jobs[act[k]];
        H.launched = true;
        H.df += (long long)H.dir * plans[t].nint[k];
        if (!plans[t].last[k]) still.push_back(act[k]);
      }
      act.swap(still);
    }
    for (size_t k = 0; k < saved.size(); k++) {
      HostJob& H = *b->jobs[saved[k].id];
      H.df = saved[k].df;
      H.launched = saved[k].launched;
    }
    if (st) {
      cudaFree(d_all);
      return st;
    }
    if (b->resort > 0) {
      long long most = 0;
      for (auto& pl : plans) most = std::max(most, pl.npts);
      if ((st = ensure_qsort(b, (size_t)most))) {
        cudaFree(d_all);
        return st;
      }
    }
    FVC_CUDA(c, cudaMemcpyAsync(d_all, all.data(), total, cudaMemcpyHostToDevice, c->stream));
    FVC_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    FVC_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    fvc_status cst = FVC_OK;
    for (size_t t = 0; t < plans.size() && !cst; t++) {
      cst = enqueue_tick(b, plans[t], (const BJob*)(d_all + offs[t]), false, (long long)t);
      if (!cst) advance_cursors(b, plans[t]);
    }
    cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (cst || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaFree(d_all);
      return cst ? cst : fail(c, FVC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&ge, g, 0);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(ge, c->stream);
    // the done events recorded during capture are graph nodes; record them again after the graph
    for (int id : b->finishing) cudaEventRecord(b->jobs[id]->done, c->stream);
    b->stats.ticks += (long long)plans.size();
    b->stats.graphs++;
    cudaError_t se = cudaStreamSynchronize(c->stream);
    if (ge) cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    cudaFree(d_all);
    if (ce != cudaSuccess || se != cudaSuccess)
      return fail(c, FVC_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce != cudaSuccess ? ce : se));
  }
  while (!b->queued.empty() || !b->active.empty()) {
    if ((st = tick(b))) return st;
  }
  retire(b, true);
  cudaEventRecord(b->t_end, c->stream);
  FVC_CUDA(c, cudaEventSynchronize(b->t_end));
  b->stats.ms_run += ev_ms(b->t_start, b->t_end);
  return FVC_OK;
}

static HostJob* job_of(fvc_batch* b, int id) {
  if (!b || id < 0 || id >= (int)b->jobs.size()) return nullptr;
  return b->jobs[id].get();
}

extern "C" fvc_status fvc_batch_poll(fvc_batch* b, int id, int* state) {
  HostJob* J = job_of(b, id);
  if (!J || !state) return FVC_ERR_ARG;
  if (J->state == JQ_FINISHING) retire(b, false);
  *state = J->state == JQ_DONE ? FVC_BATCH_DONE
         : J->state == JQ_FAILED ? FVC_BATCH_FAILED
         : J->state == JQ_RELEASED ? FVC_BATCH_RELEASED
         : J->state == JQ_QUEUED ? FVC_BATCH_QUEUED : FVC_BATCH_RUNNING;
  if (J->state == JQ_FAILED) return fail(b->c, J->err, "batch job %d: %s", id, J->msg.c_str());
  return FVC_OK;
}

static fvc_status job_ready(fvc_batch* b, HostJob* J, int kind_ok) {
  if (!J) return FVC_ERR_ARG;
  if (J->state == JQ_FINISHING) retire(b, true);
  if (J->state == JQ_FAILED) return fail(b->c, J->err, "batch job %d: %s", J->id, J->msg.c_str());
  if (J->state != JQ_DONE) return fail(b->c, FVC_ERR_STATE, "batch job %d has not finished", J->id);
  if (!(kind_ok & (1 << J->kind))) return fail(b->c, FVC_ERR_ARG, "batch job %d is of another kind", J->id);
  return FVC_OK;
}

// ------------------------------------------------------------ results

// Queues a finished job's results into a free result block (slot k) on the
// result stream, after the job's last tick: the tracer state in seed order
// with its residence times (k_res_tracer writes the page-locked block
// directly), or the FTLE fields (copied).
static fvc_status result_begin(fvc_batch* b, HostJob* J, int k, long long* ticket) {
  fvc_ctx* c = b->c;
  fvc_status st;
  if ((st = use_device(c))) return st;
  auto& S = b->res[k];
  const bool ftle = J->kind == FVC_JOB_FTLE;
  const size_t n = ftle ? (size_t)J->job->f.n : (size_t)J->job->t.n;
  const size_t need = std::max<size_t>((ftle ? 16 : 48) * n, 256);
  if (need > S.cap) {
    if (S.h) {
      cudaEventSynchronize(S.ev);  // a released ticket's copy may still run
      cudaFreeHost(S.h);
      S.h = nullptr;
      S.cap = 0;
    }
    const size_t cap = need + need / 4;
    if (cudaMallocHost(&S.h, cap) != cudaSuccess) {
      S.h = nullptr;
      return fail(c, FVC_ERR_OOM, "batch result block (page-locked, %zu bytes)", cap);
    }
    S.cap = cap;
  }
  if (!S.ev && cudaEventCreateWithFlags(&S.ev, cudaEventDisableTiming) != cudaSuccess)
    return fail(c, FVC_ERR_CUDA, "batch result event");
  cudaStream_t s = b->res_stream;
  FVC_CUDA(c, cudaStreamWaitEvent(s, J->done, 0));
  fvc_batch_result r{};
  r.kind = J->kind;
  r.n = (long long)n;
  if (ftle) {
    double* w = reinterpret_cast<double*>(S.h);
    if (n) {
      FVC_CUDA(c, cudaMemcpyAsync(w, J->job->f.out, 8 * n, cudaMemcpyDeviceToHost, s));
      FVC_CUDA(c, cudaMemcpyAsync(w + n, J->job->f.out + n, 8 * n, cudaMemcpyDeviceToHost, s));
    }
    r.ftle_wT = w;
    r.ftle_woT = w + n;
  } else {
    double* X = reinterpret_cast<double*>(S.h);
    double* ldt = X + 3 * n;
    double* rt = ldt + n;
    int* eid = reinterpret_cast<int*>(rt + n);
    int* left = eid + n;
    if (n) {
      const TracerDev& t = J->job->t;
      k_res_tracer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(t, J->d_inv, J->job->packed ? 1 : 0, J->spec.t_start,
                                                      J->stop, X, ldt, rt, eid, left);
      if ((st = check_launch(c, "batch result"))) return st;
    }
    r.X = X;
    r.ldt = ldt;
    r.rt = rt;
    r.eid = eid;
    r.left = left;
  }
  FVC_CUDA(c, cudaEventRecord(S.ev, s));
  S.r = r;
  S.job = J->id;
  S.ticket = b->res_next++;
  S.busy = true;
  J->res_held++;
  *ticket = S.ticket;
  return FVC_OK;
}

static int res_slot(fvc_batch* b, long long ticket) {
  for (int k = 0; k <= FVC_BATCH_RESULT_SLOTS; k++)
    if (b->res[k].busy && b->res[k].ticket == ticket) return k;
  return -1;
}

static fvc_status result_get(fvc_batch* b, int k, fvc_batch_result* out) {
  auto& S = b->res[k];
  if (cudaEventSynchronize(S.ev) != cudaSuccess) return fail(b->c, FVC_ERR_CUDA, "batch result copy failed");
  *out = S.r;
  return FVC_OK;
}

static void result_release(fvc_batch* b, int k) {
  auto& S = b->res[k];
  cudaEventSynchronize(S.ev);  // the job's memory stays read until the copy ends
  HostJob* J = job_of(b, S.job);
  if (J && J->res_held > 0) J->res_held--;
  S.busy = false;
  S.ticket = -1;
  S.job = -1;
}

extern "C" fvc_status fvc_batch_result_begin(fvc_batch* b, int id, long long* ticket) {
  if (!b || !ticket) return FVC_ERR_ARG;
  HostJob* J = job_of(b, id);
  fvc_status st = job_ready(b, J, (1 << FVC_JOB_TRACERS) | (1 << FVC_JOB_RESIDENCE) | (1 << FVC_JOB_FTLE));
  if (st) return st;
  for (int k = 0; k < FVC_BATCH_RESULT_SLOTS; k++)
    if (!b->res[k].busy) return result_begin(b, J, k, ticket);
  return fail(b->c, FVC_ERR_STATE, "all %d batch result blocks are held: release a ticket first",
              FVC_BATCH_RESULT_SLOTS);
}

extern "C" fvc_status fvc_batch_result_ready(fvc_batch* b, long long ticket, int* ready) {
  if (!b || !ready) return FVC_ERR_ARG;
  const int k = res_slot(b, ticket);
  if (k < 0) return fail(b->c, FVC_ERR_STATE, "no batch result with ticket %lld is held", ticket);
  const cudaError_t e = cudaEventQuery(b->res[k].ev);
  if (e == cudaErrorNotReady) {
    cudaGetLastError();  // not an error
    *ready = 0;
    return FVC_OK;
  }
  if (e != cudaSuccess) return fail(b->c, FVC_ERR_CUDA, "batch result copy: %s", cudaGetErrorString(e));
  *ready = 1;
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_result_get(fvc_batch* b, long long ticket, fvc_batch_result* out) {
  if (!b || !out) return FVC_ERR_ARG;
  const int k = res_slot(b, ticket);
  if (k < 0) return fail(b->c, FVC_ERR_STATE, "no batch result with ticket %lld is held", ticket);
  return result_get(b, k, out);
}

extern "C" fvc_status fvc_batch_result_release(fvc_batch* b, long long ticket) {
  if (!b) return FVC_ERR_ARG;
  const int k = res_slot(b, ticket);
  if (k < 0) return fail(b->c, FVC_ERR_STATE, "no batch result with ticket %lld is held", ticket);
  result_release(b, k);
  return FVC_OK;
}

// The blocking result calls: the same path through the batch's own block,
// then copied into the caller's arrays.
static fvc_status result_now(fvc_batch* b, int id, int kinds, fvc_batch_result* r, int* slot) {
  HostJob* J = job_of(b, id);
  fvc_status st = job_ready(b, J, kinds);
  if (st) return st;
  const int k = FVC_BATCH_RESULT_SLOTS;
  long long t;
  if ((st = result_begin(b, J, k, &t))) return st;
  if ((st = result_get(b, k, r))) {
    result_release(b, k);
    return st;
  }
  *slot = k;
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_tracer_result(fvc_batch* b, int id, double* X, int* eid, int* left, double* ldt) {
  if (!b) return FVC_ERR_ARG;
  fvc_batch_result r;
  int k;
  fvc_status st = result_now(b, id, (1 << FVC_JOB_TRACERS) | (1 << FVC_JOB_RESIDENCE), &r, &k);
  if (st) return st;
  const size_t n = (size_t)r.n;
  if (X) memcpy(X, r.X, 24 * n);
  if (eid) memcpy(eid, r.eid, 4 * n);
  if (left) memcpy(left, r.left, 4 * n);
  if (ldt) memcpy(ldt, r.ldt, 8 * n);
  result_release(b, k);
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_residence_result(fvc_batch* b, int id, double* rt) {
  if (!b) return FVC_ERR_ARG;
  if (!rt) return FVC_ERR_ARG;
  fvc_batch_result r;
  int k;
  fvc_status st = result_now(b, id, (1 << FVC_JOB_TRACERS) | (1 << FVC_JOB_RESIDENCE), &r, &k);
  if (st) return st;
  memcpy(rt, r.rt, 8 * (size_t)r.n);
  result_release(b, k);
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_ftle_result(fvc_batch* b, int id, double* wT, double* wN) {
  if (!b) return FVC_ERR_ARG;
  fvc_batch_result r;
  int k;
  fvc_status st = result_now(b, id, 1 << FVC_JOB_FTLE, &r, &k);
  if (st) return st;
  const size_t n = (size_t)r.n;
  if (wT) memcpy(wT, r.ftle_wT, 8 * n);
  if (wN) memcpy(wN, r.ftle_woT, 8 * n);
  result_release(b, k);
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_job_stats(fvc_batch* b, int id, fvc_job_stats* out) {
  HostJob* J = job_of(b, id);
  if (!J || !out) return FVC_ERR_ARG;
  if (J->state == JQ_FINISHING) retire(b, true);
  memset(out, 0, sizeof(*out));
  if (J->job) *out = J->job->stats;
  if (J->state == JQ_ACTIVE && J->slot >= 0) {
    // a running job: its step counters as the ticks completed so far left them
    DevCounters h;
    if (cudaMemcpyAsync(&h, b->d_ctrs + J->slot, sizeof(h), cudaMemcpyDeviceToHost, b->res_stream) == cudaSuccess &&
        cudaStreamSynchronize(b->res_stream) == cudaSuccess) {
      out->steps_main += (long long)h.steps;
      out->steps_early += (long long)h.steps_early;
      out->intervals += J->ticks;
    }
  }
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_release(fvc_batch* b, int id) {
  HostJob* J = job_of(b, id);
  if (!J) return FVC_ERR_ARG;
  if (J->state == JQ_QUEUED || J->state == JQ_ACTIVE)
    return fail(b->c, FVC_ERR_STATE, "batch job %d is still running", id);
  if (J->res_held > 0)
    return fail(b->c, FVC_ERR_STATE, "batch job %d still has %d result ticket(s) held", id, J->res_held);
  if (J->state == JQ_FINISHING) retire(b, true);
  if (J->job) {
    // the job's last tick has completed (done or failed) and result reads
    // waited for their own stream: nothing queued uses its memory, so it
    // goes back to the pool without draining the ticks in flight
    if (J->d_inv) pool_put(b->c, J->d_inv, 4 * (size_t)J->job->t.n);
    J->d_inv = nullptr;
    job_destroy_idle(J->job);
    J->job = nullptr;
    b->used -= J->bytes;
  }
  if (J->slot >= 0) {
    b->free_slots.push_back(J->slot);
    J->slot = -1;
  }
  J->seeds.clear();
  J->seeds.shrink_to_fit();
  if (J->state != JQ_FAILED) J->state = JQ_RELEASED;
  return FVC_OK;
}

extern "C" fvc_status fvc_batch_get_stats(fvc_batch* b, fvc_batch_stats* out) {
  if (!b || !out) return FVC_ERR_ARG;
  *out = b->stats;
  out->hbm_used = (long long)b->used;
  return FVC_OK;
}
