// fvc_internal.h -- library-internal state shared by the C-ABI translation
// units (fvc_api.cu, fvc_batch.cu): the context and job structures and the
// helpers both use.  Not part of the public interface (include/fvc.h).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "fvc.h"
#include "fvc_kernels.h"

using namespace fvc;

struct fvc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevMesh mesh{};
  bool mesh_set = false;
  DevInteg integ{1, 0.01, 0, 0.0, 0.0, 0.0};
  bool integ_set = false;
  DevWindow window{};
  bool window_set = false;
  long frame_nodes = 0;  // nodes per frame
  // window-level launches (stage-time fields, quantised frame pairs) not yet
  // counted in a job's statistics; the next FTLE interval takes them over
  long long aux_launches = 0;
  double node_lo[3] = {0, 0, 0}, node_hi[3] = {0, 0, 0};  // bounding box of the mesh nodes
  // device buffers
  int4* d_elem = nullptr;
  double* d_geom = nullptr;
  float* d_geo32 = nullptr;
  double4_32a* d_nodes = nullptr;
  int* d_cell_start = nullptr;
  int* d_cell_ids = nullptr;
  BucketGrid grid{};
  std::unordered_map<int, double4_32a*> frames;
  // Cartesian 2D: frames whose w components are all +0.0 (bit pattern 0)
  std::unordered_map<int, bool> frame_wzero;
  double* d_stage = nullptr;  // frame upload staging, 3 doubles a node
  DevCounters* d_ctr = nullptr;
  double4_32a* d_vt = nullptr;  // stage-time node velocities
  int vt_slots = 0;
  // scratch for array calls
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  // mixed-precision form: quantised frames by frame id, the call's step table
  int prec = 0;
  struct QFrame {
    ushort4* q = nullptr;
    float s[3] = {1.f, 1.f, 1.f};
    int fmt = 0;
    unsigned ver = 0;  // counts the quantisations (a pair made from an older one is stale)
  };
  std::unordered_map<int, QFrame> qframes;
  unsigned* d_qscratch = nullptr;
  uint4* d_qpair = nullptr;  // the window's two quantised frames, interleaved
  // interleaved pairs kept per (frame_lo, frame_hi), so a window set again
  // (every interval of a slide or release) reuses its records
  struct QPair {
    uint4* q = nullptr;
    unsigned va = 0, vb = 0;
    int fmt = 0;
  };
  std::map<std::pair<int, int>, QPair> qpairs;
  size_t qpair_bytes = 0;
  std::vector<StepM> h_steps;
  StepM* d_steps = nullptr;
  size_t steps_cap = 0;
  // step tables staged through page-locked memory (a pageable copy would
  // synchronise the stream): a ring of tables, each slot reused after the
  // event of its last upload
  StepM* h_ring = nullptr;
  StepM* d_ring = nullptr;
  int ring_k = 0;
  std::vector<cudaEvent_t> ring_ev;
  int window_lo = -1, window_hi = -1;
  // asynchronous frame uploads: a side stream, a two-buffer staging ring and
  // per frame the event its upload recorded
  cudaStream_t up_stream = nullptr;
  double* d_up_stage[2] = {nullptr, nullptr};
  int up_k = 0;
  cudaEvent_t up_after = nullptr;  // compute-stream point an upload must follow
  std::unordered_map<int, cudaEvent_t> frame_ev;
  // device blocks freed by jobs, kept for later jobs on this context: a
  // cudaFree synchronises the device, and FTLE windows allocate the same
  // sizes again and again; reuse is ordered by the context's stream
  std::multimap<size_t, void*> pool;
  size_t pool_bytes = 0;
  // asynchronous tracer outputs: a ring of FVC_TRACER_OUTPUT_SLOTS slots,
  // each a device buffer for one compacted output and a page-locked host
  // copy, filled on a side stream; tickets number the outputs of the context
  struct OutSlot {
    double* d = nullptr;        // compacted positions (device)
    double* h = nullptr;        // page-locked copy
    int* hc = nullptr;          // page-locked [count, status]
    cudaEvent_t compacted = nullptr;  // the compaction into d finished (context stream)
    cudaEvent_t copied = nullptr;     // the copy to h finished (side stream)
    const void* tag = nullptr;  // the job the output came from (compared, never dereferenced)
    long long ticket = -1;      // output in the slot, -1 none
    long long rows = 0;         // rows the side-stream copy moved
    long long n = 0;            // tracers of the output's job (its largest count)
    bool busy = false;          // begun and not released
  };
  OutSlot out[FVC_TRACER_OUTPUT_SLOTS];
  size_t out_rows_cap = 0;      // rows each slot has room for
  long long out_next = 0;       // the next ticket
  cudaStream_t out_stream = nullptr;
  std::mutex out_mu;            // the slots' ticket / busy state (waits may come from another thread)
  // exposure time (Trace_CETCompute): per-element sums shared by all releases
  double* d_cet_sum = nullptr;
  int* d_cet_enc = nullptr;
  int cet_sub = 0;  // Trace_CETSubsteps; 0 = off
  std::string err;
};

struct fvc_job {
  fvc_ctx* ctx = nullptr;
  size_t mem_bytes = 0;     // size of mem (returned to the context's pool)
  size_t rec_bytes = 0;     // size of rec_mem
  int kind = 0;  // 0 FTLE, 1 tracers
  FtleDev f{};
  TracerDev t{};
  void* mem = nullptr;  // one allocation for all per-job arrays
  int prec = 0;         // arithmetic form the job was created with
  bool packed = false;  // positions held as (X, c) float pairs
  bool live_ready = false;  // FTLE: f.live holds the next interval's live points
  // tracers: the other live list, which each advance fills for the next
  // one, and its state (valid until the tracers' state changes otherwise)
  int* live_alt = nullptr;
  int tgen = 0;
  bool tlive_ready = false;
  int tlive_extrap = 0;
  fvc_job_stats stats{};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  void* rec_mem = nullptr;  // FTLE: the main pass's per-step record
  int rec_cap = 0;          // steps it has room for
  // FTLE intervals run asynchronously on the job's own counters; the
  // events of each interval not yet accounted (main start, main end, early
  // end) and recycled events
  DevCounters* d_ctr = nullptr;
  std::vector<cudaEvent_t> pend;
  std::vector<cudaEvent_t> spare;
  // tracers: the largest output count a completed output of this job had
  // (outputs only shrink: a tracer that left stays left), -1 unknown
  long long out_bound = -1;
};

// ---- helpers defined in fvc_api.cu
// records the message on the context and returns code
fvc_status fail(fvc_ctx* c, fvc_status code, const char* fmt, ...);
fvc_status use_device(fvc_ctx* c);
fvc_status check_launch(fvc_ctx* c, const char* what);
// the quantised copy of resident frame `id` in the context's 16-bit format
fvc_status quantised(fvc_ctx* c, int id, fvc_ctx::QFrame** out);
// the integrator / precision combination is one the form supports
fvc_status mixed_ok(fvc_ctx* c);
void job_events(fvc_job* j);
// frees a job whose GPU work has all completed, without a stream wait
void job_destroy_idle(fvc_job* j);
// (X, c) float pairs copied to the host back to FP64 positions X - c
void unpack_host(double* A, size_t n);
// device memory from / back to the context's pool of freed blocks (a block
// of at least `bytes` and at most twice that, else cudaMalloc)
void* pool_get(fvc_ctx* c, size_t bytes);
void pool_put(fvc_ctx* c, void* p, size_t bytes);
// orders the context's stream after a pending asynchronous upload of frame id
void frame_dep(fvc_ctx* c, int id);
float ev_ms(cudaEvent_t a, cudaEvent_t b);

#define FVC_CUDA(c, x)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (x);                                                                \
    if (e_ != cudaSuccess) return fail((c), FVC_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
  } while (0)
