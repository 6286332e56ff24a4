/*
 * fvc.h -- C ABI of the GB300 flowVC advection engine (libfvc.so).
 *
 * The engine replaces the hot path of ompVC (flowVC's OpenMP program):
 * tracer and FTLE-grid advection through a time-interpolated velocity field
 * on Cartesian grids or unstructured triangle / tetrahedral meshes, point
 * location, and the FTLE reduction.  ompVC has no plugin layer; the entry
 * points below replace the internal calls its driver makes once per frame
 * interval, and each cites the ompVC routine it stands in for.
 *
 * Conventions
 *   - Plain pointers and sizes only.  Host arrays are read or written during
 *     the call and never retained; the library keeps its own device copies.
 *   - Every call returns an fvc_status; fvc_last_error() gives the text of
 *     the last failure on a context.  Nothing calls exit().
 *   - A context owns one CUDA stream on one device.  Calls on one context
 *     must not overlap; separate contexts may be used from separate threads.
 *   - Arithmetic is IEEE FP64 in ompVC's operation order: element ids, exit
 *     flags and positions are bit-identical to ompVC built for x86-64.
 *     fvc_set_precision selects the mixed-precision form instead.
 *   - Point arrays are n x 3 doubles (x, y, z interleaved), as in ompVC's
 *     LagrangianPoint.X.
 */
#ifndef FVC_H
#define FVC_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FVC_ABI_VERSION 3

typedef int fvc_status;
enum {
  FVC_OK = 0,
  FVC_ERR_IO = 1,      /* file or host I/O failure */
  FVC_ERR_ARG = 2,     /* invalid argument or unsupported option */
  FVC_ERR_OOM = 3,     /* device or host allocation failed */
  FVC_ERR_WALK = 4,    /* neighbour walk hit its hop cap or an indeterminate
                          neighbour (ompVC: FatalError "Indeterminate neighbor") */
  FVC_ERR_TIMEOUT = 5, /* a bounded device wait gave up */
  FVC_ERR_CUDA = 6,    /* CUDA runtime error */
  FVC_ERR_STATE = 7,   /* call out of order, or a point that left was advected */
  FVC_ERR_TLOC = 8     /* query time outside the loaded frame interval
                          (ompVC: FatalError "tloc must be between 0 and 1") */
};

typedef struct fvc_ctx fvc_ctx;
typedef struct fvc_job fvc_job;

typedef struct {
  int device;    /* CUDA device ordinal */
  int dims;      /* Dimensions: 2 or 3 */
  int mesh_type; /* Data_MeshType: 0 Cartesian, 1 unstructured */
  int max_hops;  /* neighbour-walk cap per point location, 0 = 65536 */
} fvc_opts;

int fvc_abi_version(void);

/* Context lifetime.  Replaces ompVC's process globals (ompVC/globals.h:17-168). */
fvc_status fvc_create(fvc_ctx **ctx, const fvc_opts *opts);
void fvc_destroy(fvc_ctx *ctx);
const char *fvc_last_error(const fvc_ctx *ctx);

/* Cartesian velocity grid; replaces LoadCartMeshData (ompVC/mesh.c:67-122).
 * The deltas are derived exactly as ompVC derives them. */
fvc_status fvc_set_cart_mesh(fvc_ctx *ctx, double xmin, double xmax, int xres, double ymin,
                             double ymax, int yres, double zmin, double zmax, int zres);

/* Unstructured mesh; replaces LoadUnstructMeshData (ompVC/mesh.c:124-213).
 * xyz: nnodes x 3; conn, adj: nelem x 4 in ompVC's layout (triangles: 4th
 * connectivity slot -1).  Also builds the bucket grid used by global search.
 * Every node id must lie in [0, nnodes) and every neighbour id in
 * [-1, nelem): otherwise FVC_ERR_ARG names the lowest bad element and the
 * context keeps its previous mesh. */
fvc_status fvc_set_unstruct_mesh(fvc_ctx *ctx, int nnodes, const double *xyz, int nelem,
                                 const int *conn, const int *adj);

/* Data_MeshBounds: xmin xmax ymin ymax zmin zmax (TestOutsideDomain,
 * ompVC/velocity.c:654-669). */
fvc_status fvc_set_bounds(fvc_ctx *ctx, const double bounds[6]);

/* Int_Type (0 Euler, 1 RK4, 2 Runge-Kutta-Fehlberg, 3 two-step
 * Adams-Bashforth), Int_TimeStep and Int_Extrapolate; replaces the globals
 * Advect reads (ompVC/integration.c:22-45). */
fvc_status fvc_set_integrator(fvc_ctx *ctx, int int_type, double h, int extrapolate);

/* Int_Accuracy, Int_MinTimeStep and Int_MaxTimeStep of RKF (ompVC/
 * integration.c:464-699, checked as CheckParameters does,
 * ompVC/parameters.c:462-463); required before advecting with Int_Type 2. */
fvc_status fvc_set_rkf(fvc_ctx *ctx, double accuracy, double min_step, double max_step);

/* Velocity frames.  uvw is one frame as stored in a <prefix>_vel.<n>.bin file
 * after its time stamp: (u, v, w) per node, Cartesian nodes in k, j, i order
 * with i fastest.  Frames stay resident on the device under the caller's
 * frame_id (0 <= frame_id < 65536) until replaced; replaces
 * Load{Cart,Unstruct}VelDataFrame (ompVC/velocity.c:61-234). */
fvc_status fvc_upload_frame(fvc_ctx *ctx, int frame_id, const double *uvw);

/* The frame pipeline: fvc_upload_frame without waiting.  The copy and the
 * repacking run on a side stream while the context's stream computes; every
 * later use of the frame (fvc_set_window, the mixed form's quantiser, batch
 * ticks) waits for it on the device, in stream order, and work already queued
 * that reads the frame id being replaced finishes first.  uvw must stay
 * unchanged until fvc_frame_ready reports 1 or fvc_frame_wait returns; from
 * pinned memory (fvc_host_alloc) the copy overlaps the computation, from
 * pageable memory it does not.  Replaces the blocking read-and-load of
 * Load{Cart,Unstruct}VelDataFrame (ompVC/velocity.c:61-234) in the frame loop
 * (ompVC/main.c:188-199). */
fvc_status fvc_upload_frame_async(fvc_ctx *ctx, int frame_id, const double *uvw);
fvc_status fvc_frame_ready(fvc_ctx *ctx, int frame_id, int *ready);
fvc_status fvc_frame_wait(fvc_ctx *ctx, int frame_id);
/* Page-locked host memory for frame staging (cudaMallocHost); no reference
 * counterpart. */
fvc_status fvc_host_alloc(void **ptr, size_t bytes);
void fvc_host_free(void *ptr);

/* Select the two resident frames bracketing [tmin, tmax] (Data_LoadedTMin /
 * Data_LoadedTMax, ompVC/main.c:188-195); frame_lo is the frame at tmin. */
fvc_status fvc_set_window(fvc_ctx *ctx, int frame_lo, int frame_hi, double tmin, double tmax);

/* Arithmetic form.  ompVC has FP64 only; the mixed forms are this engine's
 * own, for unstructured meshes with Euler or RK4 and no extrapolation:
 *   FVC_PREC_FP64  (default) ompVC's FP64 arithmetic, bit-exact.
 *   FVC_PREC_BF16  frames stored as BF16 (FVC_PREC_FP16: FP16) with one FP32
 *                  scale per frame and component; point location,
 *                  interpolation and the integrator's stages in FP32;
 *                  positions accumulated in FP32 with Kahan compensation.
 *                  Near an element face (within the element's own FP32
 *                  error bound, at least 1e-5) the containment test is the
 *                  FP64 one; the FTLE stencil and eigenvalue stay FP64.
 * Results differ from the FP64 form by the quantisation of the frames and
 * FP32 rounding.  Set it before creating jobs; jobs keep the form they were
 * created with. */
enum { FVC_PREC_FP64 = 0, FVC_PREC_BF16 = 1, FVC_PREC_FP16 = 2 };
fvc_status fvc_set_precision(fvc_ctx *ctx, int precision);

/* ---- step level ------------------------------------------------------- */

/* Advect n points from t0 to t1: ompVC's Advect (ompVC/integration.c:22-45)
 * over arrays.  X (n x 3), V (n x 3, may be NULL unless extrapolating), eid
 * (may be NULL on Cartesian meshes), left and ldt (LeftDomainTime) are
 * updated in place; points with left set are skipped unless extrapolating.
 * steps (may be NULL) receives the number of accepted integration steps. */
fvc_status fvc_advect(fvc_ctx *ctx, int n, double *X, double *V, int *eid, int *left, double *ldt,
                      double t0, double t1, long long *steps);

/* The same on arrays already in device memory (d-prefixed pointers), on the
 * context's stream; returns after the work completes. */
fvc_status fvc_advect_device(fvc_ctx *ctx, int n, double *dX, double *dV, int *deid, int *dleft,
                             double *dldt, double t0, double t1, long long *steps);

/* fvc_advect without any device allocation.  This entry point has no
 * counterpart in the reference: ompVC advects in host memory and never
 * allocates on a GPU.  It is for callers that must not allocate device
 * memory while they run, e.g. a host application that has handed the rest
 * of the GPU's memory to its own pool allocator, or one that advects from a
 * code path where a cudaMalloc (which can synchronise the device) is not
 * allowed.  Arguments, results and errors are those of fvc_advect; results
 * are identical to it.
 *
 * Its device scratch (the staging copies of the point arrays, the step
 * counters and as much of the stage-time velocity table as fits) lives in
 * one fixed array of FVC_NOALLOC_SCRATCH_BYTES that the library declares at
 * file scope: every GPU that loads libfvc holds that much memory until the
 * process exits, whether or not this function is called.
 *   - n above FVC_NOALLOC_MAX_POINTS is refused with FVC_ERR_ARG.
 *   - The first call on a device looks the array's device address up (one
 *     cudaGetSymbolAddress, which loads the library's device code if it is
 *     not loaded yet); make that first call before any stream capture.
 *   - That address is kept until the process exits.  It does not survive a
 *     cudaDeviceReset (or any other teardown of the device's primary
 *     context): the array may then load elsewhere, so a process that resets
 *     a device must not call this function on that device again.
 *   - All calls, from every context on a device, share the one array and
 *     it keeps the last call's contents.  Calls whose GPU work overlaps
 *     (from several threads, or several contexts on other streams) race and
 *     corrupt each other's results: serialise them. */
#define FVC_NOALLOC_MAX_POINTS 131072
#define FVC_NOALLOC_SCRATCH_BYTES (32u << 20)
fvc_status fvc_advect_noalloc(fvc_ctx *ctx, int n, double *X, double *V, int *eid, int *left,
                              double *ldt, double t0, double t1, long long *steps);

/* GetVelocity (ompVC/velocity.c:236-247) at time tq for n points; eid walks
 * and left is set as the reference does.  out: n x 3. */
fvc_status fvc_velocity(fvc_ctx *ctx, int n, const double *X, int *eid, int *left, double tq,
                        double *out);

/* Get_Element_Local_Search (ompVC/mesh.c:496-611) from guess[i]. */
fvc_status fvc_local_search(fvc_ctx *ctx, int n, const double *X, const int *guess, int *out);

/* Get_Element_Global_Search (ompVC/mesh.c:304-398): the lowest element id
 * containing each point, -1 if none; answered from a uniform bucket grid. */
fvc_status fvc_global_search(fvc_ctx *ctx, int n, const double *X, int *out);

/* ---- FTLE job: one output slide of ompVC's FTLE computation ------------ */

typedef struct {
  /* FTLE_CartMesh: seed grid bounds and resolution (ZRes = 1 in 2D) */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  int xres, yres, zres;
  int local_search_checking; /* LocalSearchChecking */
  double start_time;         /* FTLE_Launches[ss].StartTime */
  double stop_time;          /* FTLE_Launches[ss].StopTime */
  int generate;              /* 1: seed the grid and locate it on the device
                                (InitializeFTLEArray, ompVC/ftle.c:383-628);
                                0: state comes from fvc_ftle_set_state */
} fvc_ftle_spec;

fvc_status fvc_ftle_create(fvc_ctx *ctx, const fvc_ftle_spec *spec, fvc_job **job);

/* FTLEPoint state in the seed grid's (i, j, k) order, k fastest
 * (ompVC/ftle.c:616-624); any pointer may be NULL to skip that field. */
fvc_status fvc_ftle_set_state(fvc_job *job, const double *X, const int *eid, const int *left,
                              const double *ldt, const int *have, const double *ftle_wT,
                              const double *ftle_woT);
fvc_status fvc_ftle_get_state(fvc_job *job, double *X, int *eid, int *left, double *ldt, int *have,
                              double *ftle_wT, double *ftle_woT);

/* One frame interval of the slide: ComputeFTLE's body for one slide
 * (ompVC/ftle.c:72-176) on the context's current window.  launch = 1 on the
 * slide's first interval (evaluates the launch velocity, ftle.c:80-99).
 * Points that leave get their FTLE early (GetFTLEForPointEarly,
 * ftle.c:788-1048) with the result of ompVC's serial loop order.
 * With steps != NULL the call waits for the interval and returns its
 * accepted steps; with steps == NULL it returns once the work is queued on
 * the context's stream, and device faults of such intervals are returned by
 * the job's next call that waits (fvc_ftle_reduce, fvc_ftle_get_state,
 * fvc_ftle_set_state, fvc_job_get_stats). */
fvc_status fvc_ftle_interval(fvc_job *job, int launch, double t1, double t2, long long *steps);

/* FTLE of every point still without one (GetFTLEForPoint, ftle.c:1050-1203)
 * and the two output fields in output order (k, j, i with i fastest,
 * OutputFTLE, ftle.c:1304-1315). */
fvc_status fvc_ftle_reduce(fvc_job *job, double int_t, double *ftle_wT, double *ftle_woT);

/* ---- tracer job: one release of ompVC's tracer computation ------------- */

typedef struct {
  int local_search_checking; /* LocalSearchChecking */
  int seed_chain;            /* element-location chain for the seeds:
                                0 list order (ReadInTraceMesh, ompVC/tracers.c:1107-1251)
                                1 generated grid (GenerateTracerMesh, ompVC/tracers.c:1314-1533) */
  double center[3];          /* grid centre used by chain 1 */
} fvc_tracer_spec;

/* Seeds n x 3; points outside Data_MeshBounds or the mesh are marked as
 * left, as ompVC marks them. */
fvc_status fvc_tracer_create(fvc_ctx *ctx, const fvc_tracer_spec *spec, int n, const double *seeds,
                             fvc_job **job);
/* Release velocity at t_start (ompVC/tracers.c:190-207). */
fvc_status fvc_tracer_launch(fvc_job *job, double t_start);
/* Advect live tracers over [t1, t2] (ompVC/tracers.c:217-240).  With
 * steps != NULL the call waits and returns the accepted steps; with NULL it
 * returns once the work is queued, and device faults are returned by the
 * job's next call that waits (fvc_tracer_output_wait, fvc_tracer_snapshot,
 * fvc_tracer_get_state, fvc_tracer_residence, fvc_job_get_stats). */
fvc_status fvc_tracer_advance(fvc_job *job, double t1, double t2, long long *steps);
/* Positions of the tracers ompVC writes at an output time, in seed order
 * (ompVC/tracers.c:243-256): LeftDomainTime > -TINY and (not left or
 * always_output).  X_out must hold n x 3; *count receives the number. */
fvc_status fvc_tracer_snapshot(fvc_job *job, int always_output, double *X_out, long long *count);
fvc_status fvc_tracer_get_state(fvc_job *job, double *X, int *eid, int *left, double *ldt);

/* Asynchronous tracer outputs: the output step of Compute_Tracer
 * (ompVC/tracers.c:243-256, written by OutputTracers,
 * ompVC/tracers.c:1763-1816) without a wait on the GPU.
 * fvc_tracer_output_begin queues, behind the job's queued advances, the
 * compaction of the tracers fvc_tracer_snapshot would return into a slot
 * of the context's output ring and their copy to page-locked host memory on
 * a side stream, and returns at once with a ticket.
 * fvc_tracer_output_wait waits for that output only and gives its
 * positions (count x 3, seed order) in library-owned page-locked memory,
 * valid until fvc_tracer_output_release frees the slot.  A context has
 * FVC_TRACER_OUTPUT_SLOTS slots: begin returns FVC_ERR_STATE while all
 * are held (release one first).  wait and release touch only the ring and
 * may be called from another thread (a file writer) while the context's
 * thread makes other calls; their failures return a status without
 * setting fvc_last_error.  A device fault of the advances before the
 * output is returned by wait.  fvc_tracer_advance with steps == NULL
 * queues its work without waiting (its steps are counted in the job's
 * statistics), so a release loop of advances and outputs never waits for
 * the GPU. */
#define FVC_TRACER_OUTPUT_SLOTS 4
fvc_status fvc_tracer_output_begin(fvc_job *job, int always_output, long long *ticket);
fvc_status fvc_tracer_output_wait(fvc_ctx *ctx, long long ticket, const double **X, long long *count);
fvc_status fvc_tracer_output_release(fvc_ctx *ctx, long long ticket);

/* ---- tracer side analyses (unstructured meshes, FP64 form) ------------- */

/* Exposure time (Trace_CETCompute, ompVC/exposuretime.c:110-172): while
 * enabled, every accepted Euler / RK4 / RKF step of fvc_tracer_advance
 * credits its duration to the elements its straight path crosses, sampled
 * at `substeps` points (Trace_CETSubsteps >= 2), and every release counts
 * one encounter for each tracer's starting element (ompVC/tracers.c:180-185).
 * The per-element sums live on the device, shared by all releases on the
 * context; enabling clears them, substeps = 0 disables and frees them.  The
 * GPU adds with atomics, so sums can differ from ompVC's serial order in
 * their last bits; encounter counts are exact.  Velocity-mesh only (ompVC's
 * Trace_CETAuxillaryMesh is not supported). */
fvc_status fvc_cet_enable(fvc_ctx *ctx, int substeps);
/* OutputCET's fields (ompVC/exposuretime.c:175-246), nelem values each, any
 * pointer may be NULL: cet = sum / xc / ntracers and met = sum / xc /
 * encounters where sum > TINY, else 0 (xc = 1 in 3D, as the reference's
 * pow(vol, 1/3) with integer 1/3 evaluates; sqrt(area) in 2D); enc the
 * encounter counts. */
fvc_status fvc_cet_results(fvc_ctx *ctx, int ntracers, double *cet, double *met, int *enc);

/* Residence time of a release (OutputRT, ompVC/residencetime.c:160-178),
 * in seed order: -1 for tracers never inside the domain, else
 * LeftDomainTime - launch_time for tracers that left and stop_time -
 * launch_time for the rest.  rt must hold n doubles. */
fvc_status fvc_tracer_residence(fvc_job *job, double launch_time, double stop_time, double *rt);

/* Counters of a job since its creation, from CUDA events recorded on the
 * context's stream around each launch. */
typedef struct {
  long long intervals;     /* frame intervals (or advance calls) run */
  long long steps_main;    /* accepted steps of the main advection pass */
  long long steps_early;   /* accepted steps of the early-FTLE advections */
  double ms_main;          /* device time of the main advection kernel */
  double ms_early;         /* device time of trigger search + early FTLE */
  double ms_reduce;        /* device time of the FTLE reduction */
  double ms_setup;         /* device time of seeding and seed location */
  long long launches;      /* kernels launched on the job's behalf */
  long long steps_early_recorded; /* of steps_early, those read from the main
                                     pass's per-step record instead of
                                     recomputed (identical results) */
} fvc_job_stats;
fvc_status fvc_job_get_stats(fvc_job *job, fvc_job_stats *out);

/* ---- batched and served form ------------------------------------------ */

/* Many tracer, residence-time and FTLE jobs, each with its own seeds and
 * integration window, advanced together over velocity frames resident on
 * the device.  No counterpart in ompVC, which runs one window per process;
 * each job is computed exactly as the single-job calls above compute it (the
 * same frame intervals, step sequences and kernels' arithmetic), so its
 * results are identical alone and in any mix of jobs, in either arithmetic
 * form of the context.
 *
 * Time advances in ticks; in one tick every active job runs its next frame
 * interval: one kernel builds the tick's work queue from all jobs' live
 * points, one persistent kernel advects it, then FTLE jobs run their
 * per-interval early-FTLE passes.  Jobs are admitted between ticks, in
 * submission order, while their device footprint fits hbm_budget; results
 * stay on the device until read or released.  Unstructured meshes, Euler or
 * RK4, no extrapolation.  Frames 0 .. tres-1 must be resident
 * (fvc_upload_frame) under their file index, frame k at tmin + k tdelta;
 * with periodic data frame indices wrap modulo tres - 1 as ompVC wraps them
 * (ompVC/velocity.c:77-80). */
typedef struct fvc_batch fvc_batch;
typedef struct {
  double tmin;           /* Data_TMin: time of frame 0 */
  double tdelta;         /* Data_TDelta */
  int tres;              /* Data_TRes */
  int periodic;          /* Data_TPeriodic */
  long long hbm_budget;  /* device bytes the admitted jobs may hold; 0 = no limit */
  int max_jobs;          /* jobs admitted at once; 0 = 1024 */
  int resort_every;      /* order each tick's work queue by job and position
                            (Z-order over the mesh's box) every this many
                            ticks, so a warp's tracers walk neighbouring
                            elements after releases disperse; 0 = never,
                            -1 = chosen by fvc_batch_autotune (default 0) */
  int tick_intervals;    /* tracer and residence-time jobs advance
                            ceil(their frame intervals / tick_intervals)
                            intervals per tick (in one launch, each interval
                            exactly as alone), so that a long release takes
                            about this many ticks, like an FTLE job of as many
                            intervals; 0 = one interval per tick */
} fvc_batch_opts;

enum { FVC_JOB_TRACERS = 0, FVC_JOB_RESIDENCE = 1, FVC_JOB_FTLE = 2 };
typedef struct {
  int kind;                  /* FVC_JOB_* */
  double t_start, t_stop;    /* integration window; backward when t_stop < t_start
                                (residence time: forward only) */
  /* tracers / residence time: n seeds (n x 3), located with ompVC's list chain */
  int n;
  const double *seeds;
  int local_search_checking;
  /* FTLE: the seed grid (start_time, stop_time and generate are set from
     the window) */
  fvc_ftle_spec grid;
} fvc_batch_job_spec;

enum { FVC_BATCH_QUEUED = 0, FVC_BATCH_RUNNING = 1, FVC_BATCH_DONE = 2, FVC_BATCH_FAILED = 3,
       FVC_BATCH_RELEASED = 4 };

typedef struct {
  long long ticks;           /* ticks run (graph ticks included) */
  long long graphs;          /* CUDA graphs launched */
  long long launches;        /* kernels launched by ticks */
  long long steps;           /* accepted steps of retired jobs */
  long long jobs_submitted;
  long long jobs_done;
  double ms_run;             /* device time inside fvc_batch_run */
  int tuned_threads;         /* block size the autotuner chose (0 = not tuned) */
  int tuned_blocks;          /* grid the autotuner chose */
  int tuned_resort;          /* re-sort interval in use (ticks; 0 = never) */
  long long hbm_used;        /* footprint of the jobs holding device memory */
} fvc_batch_stats;

fvc_status fvc_batch_create(fvc_ctx *ctx, const fvc_batch_opts *opts, fvc_batch **batch);
void fvc_batch_destroy(fvc_batch *batch);
/* Queues a job (the seeds are copied); returns its id. */
fvc_status fvc_batch_submit(fvc_batch *batch, const fvc_batch_job_spec *spec, int *id);
/* Admits what fits, then enqueues one tick and returns without waiting for
 * the GPU (at most two ticks in flight).  *pending = jobs not yet finished. */
fvc_status fvc_batch_tick(fvc_batch *batch, int *pending);
/* Runs until every submitted job has finished.  graph = 1: when every job
 * fits at once, the whole schedule is captured into one CUDA graph and
 * launched as one. */
fvc_status fvc_batch_run(fvc_batch *batch, int graph);
/* Times the persistent kernel's launch shapes on the next tick of the
 * admitted jobs (their state restored after each trial) and keeps the
 * fastest. */
fvc_status fvc_batch_autotune(fvc_batch *batch);
/* *state = FVC_BATCH_*; a failed job returns its error. */
fvc_status fvc_batch_poll(fvc_batch *batch, int id, int *state);
/* Results of a finished job (waits for it): tracer state in seed order
 * (as fvc_tracer_get_state), residence times (as fvc_tracer_residence with
 * the job's window), FTLE fields in output order (as fvc_ftle_reduce). */
fvc_status fvc_batch_tracer_result(fvc_batch *batch, int id, double *X, int *eid, int *left, double *ldt);
fvc_status fvc_batch_residence_result(fvc_batch *batch, int id, double *rt);
fvc_status fvc_batch_ftle_result(fvc_batch *batch, int id, double *ftle_wT, double *ftle_woT);
/* A job's statistics; for a job still running, the steps of the ticks that
 * have completed so far. */
fvc_status fvc_batch_job_stats(fvc_batch *batch, int id, fvc_job_stats *out);

/* Asynchronous results, for a request loop that must go on ticking while
 * results travel.  fvc_batch_result_begin queues a finished job's results on
 * the batch's result stream, after the job's last tick, into a page-locked
 * block the batch owns (tracer state put back in seed order and residence
 * times on the device, or the two FTLE fields) and returns a ticket at once.
 * fvc_batch_result_ready polls it; fvc_batch_result_get waits for it and
 * fills *out with pointers into the block, valid until the ticket is
 * released; fvc_batch_result_release gives the block back.  At most
 * FVC_BATCH_RESULT_SLOTS tickets are held at a time (begin refuses another
 * with FVC_ERR_STATE), and a job holding a ticket cannot be released.  The
 * blocking result calls above stay available beside these. */
#define FVC_BATCH_RESULT_SLOTS 8
typedef struct {
  int kind;               /* FVC_JOB_* of the job */
  long long n;            /* tracers, or FTLE points */
  const double *X;        /* tracer kinds: n x 3 positions, seed order */
  const int *eid;         /* tracer kinds */
  const int *left;        /* tracer kinds */
  const double *ldt;      /* tracer kinds: LeftDomainTime */
  const double *rt;       /* tracer kinds: residence times over the job's window */
  const double *ftle_wT;  /* FTLE: fields in output order */
  const double *ftle_woT;
} fvc_batch_result;
fvc_status fvc_batch_result_begin(fvc_batch *batch, int id, long long *ticket);
fvc_status fvc_batch_result_ready(fvc_batch *batch, long long ticket, int *ready);
fvc_status fvc_batch_result_get(fvc_batch *batch, long long ticket, fvc_batch_result *out);
fvc_status fvc_batch_result_release(fvc_batch *batch, long long ticket);

/* Frees a finished job's device memory (its results become unavailable). */
fvc_status fvc_batch_release(fvc_batch *batch, int id);
fvc_status fvc_batch_get_stats(fvc_batch *batch, fvc_batch_stats *out);


/* The context's CUDA stream (a cudaStream_t), for callers that record their
 * own events on it or order their work after the engine's. */
void *fvc_stream(fvc_ctx *ctx);

void fvc_job_destroy(fvc_job *job);

#ifdef __cplusplus
}
#endif
#endif
