// fvc_kernels.h -- host-side launch wrappers for the engine's kernels.
// Each wrapper launches on the given stream and returns immediately; all
// pointers are device pointers.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "fvc_state.h"

namespace fvc {

// One early-FTLE task list's counters.
struct TaskCounters {
  int ntask;    // advections queued
  int hist[8];  // queued advections per length bucket (steps, capped at 7)
  int scat[8];  // fill cursors of the buckets in the sorted list
};

// Scratch counters shared by the launches of one call.  steps .. changed
// (and steps_rec) are the accumulated figures a job's wait takes and clears.
struct DevCounters {
  unsigned long long steps;
  unsigned long long steps_early;  // accepted steps of the early-FTLE advections
  int status;
  int changed;
  int nlive;   // live points of the current advection call
  int cur[4];  // work cursors of the persistent launches: 0 live list, 1-2 task lists (after nlive: cleared with it)
  // count .. nfall are cleared together before an interval's early-FTLE passes
  int count;   // points served an early FTLE this interval
  TaskCounters tq[2];  // the task lists: 0 neighbours to the exit time, 1 to MinExitTime
  int nfall;   // served points whose eigenvalue falls back to the Jacobi solver
  unsigned long long steps_rec;  // early-FTLE steps read from the main pass's record
  // a tracer job's live lists built by its advances: three (count, cursor)
  // pairs in rotation (the call with generation g reads pair g % 3, appends
  // to (g + 1) % 3 and clears (g + 2) % 3, which the call before read)
  int lcnt[3];
  int lcur[3];
};
#define FVC_EARLY_COUNTERS_BYTES (offsetof(DevCounters, nfall) + sizeof(int) - offsetof(DevCounters, count))
static_assert(offsetof(DevCounters, cur) == offsetof(DevCounters, nlive) + sizeof(int),
              "the live-list kernels clear nlive and the cursors as one run of ints");

// ---- mesh preprocessing
// the mesh's element records from the caller's connectivity and adjacency
// (4 ints each per element) with the ids range-checked (*bad: the lowest
// element out of range, untouched if none)
void pack_elements(const int4* conn, const int4* adj, int nelem, int nnodes, int nv, int4* elem, int* bad,
                   cudaStream_t s);
// geo32 holds 16 floats per element followed by the float4 low parts (geo32lo)
void launch_geometry(const DevMesh& m, double* geom, float* geo32, cudaStream_t s);

// Builds the grid into caller-owned buffers; returns the number of entries
// written to ids (the caller sizes ids with bucket_count first).
long long bucket_count(const DevMesh& m, BucketGrid& g, int* cell_count, int ncells, int* d_total,
                       cudaStream_t s);
void bucket_fill(const DevMesh& m, const BucketGrid& g, int* cell_start, int* cursor, int* ids,
                 int ncells, int* scan_tmp, cudaStream_t s);

void scan_counts(const int* in, int* out, int n, long long* tmp, cudaStream_t s);

// ---- step level
void launch_advect(const DevMesh& m, const DevWindow& w, const DevInteg& in, int n, double* X,
                   double* V, int* eid, int* left, double* ldt, double t0, double t1,
                   DevCounters* ctr, cudaStream_t s);
void launch_velocity(const DevMesh& m, const DevWindow& w, int n, const double* X, int* eid,
                     int* left, double tq, double* out, DevCounters* ctr, cudaStream_t s);
void launch_local_search(const DevMesh& m, int n, const double* X, const int* guess, int* out,
                         DevCounters* ctr, cudaStream_t s);
void launch_global_search(const DevMesh& m, const BucketGrid& g, int n, const double* X,
                          const int* skip, int* out, cudaStream_t s);

// ---- seed location chains (element ids of seeds with ompVC's guess chain)
struct ChainArgs {
  int kind;        // 0 FTLE grid (ftle.c:455-602), 1 tracer list (tracers.c:1107-1251),
                   // 2 generated tracer grid (tracers.c:1340-1530)
  int n;
  int res[3];      // FTLE: XRes, YRes, ZRes (i outer, k fastest)
  int lsc;         // LocalSearchChecking
  int center_eid;  // global search of the grid centre (kinds 0 and 2), else -1
};
// left0: 1 for points outside Data_MeshBounds.  On return eid holds the
// element or -1 for points the chain could not place.  Returns the number of
// fixed-point rounds, or -1 on a device fault.
int locate_chain(const DevMesh& m, const BucketGrid& g, const ChainArgs& a, const double* X,
                 const int* left0, int* eid, int* work, DevCounters* ctr, cudaStream_t s);
// ints of scratch locate_chain needs in `work`
size_t chain_words(const ChainArgs& a);

// ---- FTLE slide
struct FtleDev {
  int n, xr, yr, zr;
  int mixed;             // 1: X, Xn and epos hold (X, c) float pairs (mixed-precision form)
  double dx, dy, dz;     // FTLE_CartMesh deltas
  double start;          // StartTime
  double* X;             // n x 3
  double* V;             // n x 3
  double* ldt;
  double* ftT;
  double* ftN;
  int* eid;
  int* left;
  int* have;
  // per-interval scratch
  double* Xn;
  double* Vn;
  double* te;
  int* en;
  unsigned char* flag;   // bit0 integrated, bit1 exited, bit2 left after step
  int* served;           // compacted list of points given an early FTLE
  int* trig;
  double* epos;          // early FTLE: 7 positions (6 neighbours, self) per served point
  double* elt;           // early FTLE: the neighbours' exit times
  double* emt;           // early FTLE: MinExitTime
  int2* tasks;           // early FTLE: queued advections (served index, 0-5 neighbour / 6 self | bucket << 3)
  int2* tsorted;         // the same, grouped by length bucket
  int* live;             // points advected this interval, in grid order
  int* block_cnt;        // compaction scratch
  double* out;           // 2 x n, output order
  // the main pass's record of the interval (null: not kept): the position
  // after k accepted steps at rec + (k - 1) 3n (k = 1 .. rec_steps; k = 0 is
  // X), and each point's accepted steps in kacc
  double* rec;
  unsigned char* kacc;
  int rec_steps;
  // FP64 RK4: each point's element state after step 1 of the main pass
  // (RecOut::e1), against which early-FTLE advections that start from
  // another element hint are checked (null: not kept)
  int4* rec_e1;
};

void ftle_seed_grid(const DevMesh& m, const FtleDev& f, double xmin, double ymin, double zmin,
                    int* left0, cudaStream_t s);
void ftle_mark_outside(const FtleDev& f, cudaStream_t s);
void ftle_launch(const DevMesh& m, const DevWindow& w, const FtleDev& f, double t, DevCounters* ctr,
                 cudaStream_t s);
void ftle_pass1(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                double t1, double t2, DevCounters* ctr, cudaStream_t s);
// cleared: the early-FTLE counters (count .. nfall) were cleared by the
// interval's main pass; else they are cleared here
void ftle_triggers(const FtleDev& f, DevCounters* ctr, bool cleared, cudaStream_t s);
// the number of served points is read on the device from ctr->count
// jacobi false: the points the closed-form eigenvalue leaves are solved by
// the update kernel that follows (ftle_update with ctr)
void ftle_early(const DevMesh& m, const DevWindow& w, const DevInteg& in, const FtleDev& f,
                double t1, DevCounters* ctr, bool jacobi, cudaStream_t s);
// ctr: also build the next interval's live list (f.live, ctr->nlive), clear
// the work cursors for it and solve the early-FTLE points the closed-form
// eigenvalue left (ctr->nfall; the list is in f.tasks)
void ftle_update(const DevMesh& m, const DevInteg& in, const FtleDev& f, DevCounters* ctr, cudaStream_t s);
// the live list of the current state (every flag and the work cursors
// cleared)
void ftle_live(const DevInteg& in, const FtleDev& f, DevCounters* ctr, cudaStream_t s);
void ftle_final(const FtleDev& f, int dims, double int_t, cudaStream_t s);

// ---- tracers
struct TracerDev {
  int n;
  double* X;
  double* V;
  double* ldt;
  int* eid;
  int* left;
  double* outX;
  int* block_cnt;
  int* live;             // tracers advected by the current call
  int* live_next;        // non-null: the advance appends the tracers still live to it (the next call's list)
  int gen;               // the advance's generation (the rotation of DevCounters::lcnt / lcur)
};

// Compacts the indices of live points (LeftDomainTime > -TINY and, unless
// extrapolating, not left: ompVC/ftle.c:113, tracers.c:225) in order into
// live[], the count into ctr->nlive; clears flag[] (may be null).
void compact_live(int n, const double* ldt, const int* left, int extrapolate, int* live,
                  unsigned char* flag, int* block_cnt, DevCounters* ctr, cudaStream_t s);
void tracer_launch_vel(const DevMesh& m, const DevWindow& w, const TracerDev& t, double tq,
                       DevCounters* ctr, cudaStream_t s);
void tracer_advance(const DevMesh& m, const DevWindow& w, const DevInteg& in, const TracerDev& t,
                    double t1, double t2, DevCounters* ctr, cudaStream_t s);
void tracer_init_ldt(const TracerDev& t, cudaStream_t s);
// Compacts the selected tracers' positions (in seed order) into t.outX;
// the count lands in ctr->count.  unpack: the mixed form's (X, c) pairs are
// written as FP64 positions.  Returns the kernels launched.
int tracer_compact(const TracerDev& t, int always, DevCounters* ctr, cudaStream_t s, bool unpack = false);

// ---- tracer side analyses (fvc_cet.cu), unstructured meshes, FP64 form
// tracer_advance with the exposure-time accumulation after every step
void tracer_advance_cet(const DevMesh& m, const DevWindow& w, const DevInteg& in, const TracerDev& t, double t1,
                        double t2, const CetDev& cet, DevCounters* ctr, cudaStream_t s);
// one encounter for the element of every tracer of a release inside the domain
void cet_release(const TracerDev& t, const CetDev& cet, cudaStream_t s);
// normalised exposure times: out = CET[nelem] then MET[nelem]
void cet_results(const DevMesh& m, const CetDev& cet, int ntracers, double* out, cudaStream_t s);
// residence time of every tracer of a release
void tracer_residence(const TracerDev& t, double launch, double stop, double* rt, cudaStream_t s);

// left = outside the domain or not placed by the seed chain; LeftDomainTime
// as ompVC initialises it for each seeding routine
void ftle_init_marks(const DevMesh& m, const FtleDev& f, const int* left0, cudaStream_t s);
void tracer_init_marks(const DevMesh& m, const TracerDev& t, const int* left0, int chain_kind,
                       cudaStream_t s);

// Time-interpolated node velocities of every slot of w (unstructured meshes).
void time_fields(const DevMesh& m, const DevWindow& w, double4_32a* vt, cudaStream_t s);

// ---- mixed-precision form
// Quantises one frame to 16 bits a component (fmt 1 BF16, 2 FP16) with a
// per-component scale (max |component|, returned in scale); synchronises
// the stream.  Returns 0 on success.
int quantize_frame(const double4_32a* f, long n, int fmt, ushort4* q, unsigned* scratch, float scale[3],
                   cudaStream_t s);
// The window's two quantised frames interleaved per node (DevWindow::qp).
void pair_frames(const ushort4* a, const ushort4* b, long n, uint4* out, cudaStream_t s);
// FP64 values <-> (X, c) float pairs in place (X = RN(v), c = RN(X - v)).
void pack_pairs(double* A, long n, cudaStream_t s);
void unpack_pairs(double* A, long n, cudaStream_t s);
// unpack_pairs over the first *count rows of 3 slots (count on the device,
// at most max_rows)
void unpack_pairs_counted(double* A, long max_rows, const int* count, cudaStream_t s);

// ---- utilities
void outside_domain_flags(const DevMesh& m, int n, const double* X, int* left0, cudaStream_t s);
void pack_frame(const double* uvw, double4_32a* out, long n, cudaStream_t s);

}  // namespace fvc
