/*
 * fvcflow.c -- "fvcflow <file.in>": flowVC's FTLE / tracer run on the GPU.
 *
 * A drop-in for ompVC's driver (ompVC/main.c:34-305) on the engine's path:
 * it reads the same .in file, mesh and velocity files, runs the same frame
 * loop and writes the same output files, with the bodies of ComputeFTLE and
 * Compute_Tracer replaced by calls into libfvc (include/fvc.h).
 *
 * Differences from ompVC, by design:
 *   - every velocity frame the run needs is uploaded once and stays resident
 *     in device memory; no per-interval temporary files are written;
 *   - out-of-scope options (inertial particles, staggered release, the
 *     activation-potential analysis, an auxiliary exposure-time mesh,
 *     velocity resampling) are refused with an error instead of being
 *     computed;
 *   - errors return a non-zero exit status with a message instead of
 *     exiting from inside the computation.
 *
 * Options after the .in file:  --device N   --stats (print a JSON line of
 * step counts and timings on stdout)   --dump-state DIR (write the final FTLE
 * grid state of every output: n, X, element ids, left flags, have flags)
 * --precision fp64|bf16|fp16 (the arithmetic form, fvc_set_precision; fp64,
 * ompVC's, by default).
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "fvc.h"
#include "fvc_params.h"

#define TINY 1.0e-10
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))

static double wall(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static int die(const char *what, fvc_ctx *c, int rc)
{
    fprintf(stderr, "\nERROR:\n%s (status %d)%s%s\n", what, rc, c ? ": " : "", c ? fvc_last_error(c) : "");
    return 1;
}

/* LagrangianPoint / FTLEPoint as ompVC writes them (ompVC/structs.h:21-36) */
typedef struct {
    double X[3], V[3];
    int eid, aux, left, pad;
    double ldt, scalar;
} disk_lpt;
typedef struct {
    disk_lpt pt;
    int have, pad;
    double ftT, ftN;
} disk_fpt;

typedef struct {
    fvcp_params P;
    fvc_ctx *ctx;
    long frame_len; /* doubles per frame */
    double *frame_buf;
    unsigned char *resident;
    long long steps;
    double t_compute;
    const char *dump_dir; /* --dump-state: final FTLE grid state per output */
    long nelem;           /* elements of the unstructured mesh */
    struct frame_pipe *pipe;  /* frame reader ahead of the computation */
} run_t;

/* frame index -> file index with ompVC's wrap (ompVC/velocity.c:77-80) */
static int frame_mod(const fvcp_params *P, int frame)
{
    int mod = (int)fmod((double)frame, (double)(P->tres - 1));
    if (mod < 0) mod += P->tres - 1;
    return mod;
}

static int load_mesh(run_t *R)
{
    fvcp_params *P = &R->P;
    char path[2 * FVCP_STR];
    int rc;
    if (P->mesh_type == 0) {
        snprintf(path, sizeof(path), "%s%s_Cartesian.bin", P->path_data, P->prefix);
        FILE *f = fopen(path, "rb");
        if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        double v[6];
        int r[3];
        int ok = fread(&v[0], 8, 2, f) == 2 && fread(&r[0], 4, 1, f) == 1 && fread(&v[2], 8, 2, f) == 2 &&
                 fread(&r[1], 4, 1, f) == 1 && fread(&v[4], 8, 2, f) == 2 && fread(&r[2], 4, 1, f) == 1;
        fclose(f);
        if (!ok) { fprintf(stderr, "Could not read %s\n", path); return 1; }
        if ((rc = fvc_set_cart_mesh(R->ctx, v[0], v[1], r[0], v[2], v[3], r[1], v[4], v[5], r[2])))
            return die("Cartesian mesh", R->ctx, rc);
        R->frame_len = 3L * r[0] * r[1] * (P->dims == 3 ? r[2] : 1);
    } else {
        int n = 0, e = 0, e2 = 0;
        snprintf(path, sizeof(path), "%s%s_coordinates.bin", P->path_data, P->prefix);
        FILE *f = fopen(path, "rb");
        if (!f || fread(&n, 4, 1, f) != 1 || n <= 0) { fprintf(stderr, "Could not read number of mesh nodes from %s\n", path); if (f) fclose(f); return 1; }
        double *xyz = (double *)malloc(24 * (size_t)n);
        if (!xyz || fread(xyz, 8, 3 * (size_t)n, f) != 3 * (size_t)n) { fprintf(stderr, "Could not read nodal coordinates completely from %s\n", path); fclose(f); free(xyz); return 1; }
        fclose(f);
        snprintf(path, sizeof(path), "%s%s_connectivity.bin", P->path_data, P->prefix);
        f = fopen(path, "rb");
        if (!f || fread(&e, 4, 1, f) != 1 || e <= 0) { fprintf(stderr, "Could not read number of mesh elements from %s\n", path); if (f) fclose(f); free(xyz); return 1; }
        int *conn = (int *)malloc(16 * (size_t)e), *adj = (int *)malloc(16 * (size_t)e);
        if (!conn || !adj || fread(conn, 4, 4 * (size_t)e, f) != 4 * (size_t)e) { fprintf(stderr, "Could not read connectivity from %s\n", path); fclose(f); free(xyz); free(conn); free(adj); return 1; }
        fclose(f);
        snprintf(path, sizeof(path), "%s%s_adjacency.bin", P->path_data, P->prefix);
        f = fopen(path, "rb");
        if (!f || fread(&e2, 4, 1, f) != 1 || e2 != e || fread(adj, 4, 4 * (size_t)e, f) != 4 * (size_t)e) {
            fprintf(stderr, "Could not read adjacency from %s (or element counts differ)\n", path);
            if (f) fclose(f);
            free(xyz); free(conn); free(adj);
            return 1;
        }
        fclose(f);
        rc = fvc_set_unstruct_mesh(R->ctx, n, xyz, e, conn, adj);
        R->nelem = e;
        free(xyz); free(conn); free(adj);
        if (rc) return die("unstructured mesh", R->ctx, rc);
        R->frame_len = 3L * n;
    }
    R->frame_buf = (double *)malloc(8 * (size_t)R->frame_len);
    R->resident = (unsigned char *)calloc((size_t)P->tres, 1);
    return (!R->frame_buf || !R->resident) ? (fprintf(stderr, "out of memory\n"), 1) : 0;
}

/* ---- frame pipeline: a reader thread reads the frame files in the order
 * the frame loop first needs them into a ring of page-locked buffers, and
 * the main thread uploads each one asynchronously (fvc_upload_frame_async)
 * as soon as it is read, so file reads and host-to-device copies overlap
 * the kernels of earlier intervals.  A ring slot returns to the reader once
 * its upload has completed (fvc_frame_ready / fvc_frame_wait). */
#define PIPE_SLOTS 4

typedef struct frame_pipe {
    run_t *R;
    int n;            /* frames in first-use order */
    int *seq;         /* file index of each */
    int *pos;         /* file index -> position in seq, -1 if unused */
    double *buf;      /* PIPE_SLOTS page-locked frames */
    int nread, up, rel, err, stop;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    pthread_t th;
    int started;
} frame_pipe;

static int read_frame_file(const fvcp_params *P, int mod, double *dst, long len)
{
    char path[2 * FVCP_STR];
    snprintf(path, sizeof(path), "%s%s_vel.%d.bin", P->path_data, P->prefix, P->suffix_tmin + mod * P->suffix_tdelta);
    FILE *f = fopen(path, "rb");
    double ts;
    if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
    if (fread(&ts, 8, 1, f) != 1 || (long)fread(dst, 8, (size_t)len, f) != len) {
        fclose(f);
        fprintf(stderr, "Could not load velocity data from %s\n", path);
        return 1;
    }
    fclose(f);
    return 0;
}

static void *pipe_reader(void *arg)
{
    frame_pipe *F = (frame_pipe *)arg;
    for (int i = 0; i < F->n; i++) {
        pthread_mutex_lock(&F->mu);
        while (!F->stop && i - F->rel >= PIPE_SLOTS) pthread_cond_wait(&F->cv, &F->mu);
        int stop = F->stop;
        pthread_mutex_unlock(&F->mu);
        if (stop) break;
        int bad = read_frame_file(&F->R->P, F->seq[i], F->buf + (long)(i % PIPE_SLOTS) * F->R->frame_len,
                                  F->R->frame_len);
        pthread_mutex_lock(&F->mu);
        if (bad) F->err = 1;
        else F->nread = i + 1;
        pthread_cond_broadcast(&F->cv);
        pthread_mutex_unlock(&F->mu);
        if (bad) break;
    }
    return NULL;
}

/* The frame files of intervals first .. last (exclusive) in first-use order. */
static int pipe_start(run_t *R)
{
    fvcp_params *P = &R->P;
    frame_pipe *F = (frame_pipe *)calloc(1, sizeof(frame_pipe));
    if (!F) return 1;
    F->R = R;
    int nfiles = P->tres;
    F->pos = (int *)malloc(sizeof(int) * (size_t)nfiles);
    F->seq = (int *)malloc(sizeof(int) * (size_t)nfiles);
    if (!F->pos || !F->seq) return 1;
    for (int k = 0; k < nfiles; k++) F->pos[k] = -1;
    for (int df = P->first_frame; df != P->last_frame; df += P->int_dir) {
        int lo = P->int_dir > 0 ? df : df - 1;
        for (int e = 0; e < 2; e++) {
            int mod = frame_mod(P, lo + e);
            if (F->pos[mod] < 0) { F->pos[mod] = F->n; F->seq[F->n++] = mod; }
        }
    }
    if (fvc_host_alloc((void **)&F->buf, sizeof(double) * (size_t)R->frame_len * PIPE_SLOTS)) {
        fprintf(stderr, "could not allocate page-locked frame buffers\n");
        return 1;
    }
    pthread_mutex_init(&F->mu, NULL);
    pthread_cond_init(&F->cv, NULL);
    if (pthread_create(&F->th, NULL, pipe_reader, F)) return 1;
    F->started = 1;
    R->pipe = F;
    return 0;
}

static void pipe_stop(run_t *R)
{
    frame_pipe *F = R->pipe;
    if (!F) return;
    if (F->started) {
        pthread_mutex_lock(&F->mu);
        F->stop = 1;
        pthread_cond_broadcast(&F->cv);
        pthread_mutex_unlock(&F->mu);
        pthread_join(F->th, NULL);
        pthread_mutex_destroy(&F->mu);
        pthread_cond_destroy(&F->cv);
    }
    /* page-locked buffers may still be read by uploads in flight */
    for (int i = F->rel; i < F->up; i++) fvc_frame_wait(R->ctx, F->seq[i]);
    fvc_host_free(F->buf);
    free(F->seq);
    free(F->pos);
    free(F);
    R->pipe = NULL;
}

/* Uploads every frame read so far, returns slots whose uploads finished, and
 * returns once the frame at position `need` is uploaded (need < 0: no wait). */
static int pipe_pump(run_t *R, int need)
{
    frame_pipe *F = R->pipe;
    pthread_mutex_lock(&F->mu);
    for (;;) {
        int ready = 1;
        while (F->rel < F->up && !fvc_frame_ready(R->ctx, F->seq[F->rel], &ready) && ready) {
            F->rel++;
            pthread_cond_broadcast(&F->cv);
        }
        while (F->up < F->nread) {
            int rc = fvc_upload_frame_async(R->ctx, F->seq[F->up], F->buf + (long)(F->up % PIPE_SLOTS) * R->frame_len);
            if (rc) { pthread_mutex_unlock(&F->mu); return die("frame upload", R->ctx, rc); }
            F->up++;
        }
        if (need < 0 || F->up > need) break;
        if (F->err) { pthread_mutex_unlock(&F->mu); return 1; }
        if (F->nread - F->rel >= PIPE_SLOTS) {
            /* the reader waits for a slot: free the oldest */
            int mod = F->seq[F->rel];
            pthread_mutex_unlock(&F->mu);
            int rc = fvc_frame_wait(R->ctx, mod);
            pthread_mutex_lock(&F->mu);
            if (rc) { pthread_mutex_unlock(&F->mu); return die("frame upload", R->ctx, rc); }
            F->rel++;
            pthread_cond_broadcast(&F->cv);
            continue;
        }
        pthread_cond_wait(&F->cv, &F->mu);
    }
    pthread_mutex_unlock(&F->mu);
    return 0;
}

/* Upload the file behind frame index `frame` once; it stays resident under
 * its file index (Load*VelDataFrame, ompVC/velocity.c:61-234). */
static int ensure_frame(run_t *R, int frame)
{
    fvcp_params *P = &R->P;
    int mod = frame_mod(P, frame);
    if (R->resident[mod]) return 0;
    if (R->pipe && R->pipe->pos[mod] >= 0) {
        if (pipe_pump(R, R->pipe->pos[mod])) return 1;
        R->resident[mod] = 1;
        return 0;
    }
    char path[2 * FVCP_STR];
    snprintf(path, sizeof(path), "%s%s_vel.%d.bin", P->path_data, P->prefix, P->suffix_tmin + mod * P->suffix_tdelta);
    FILE *f = fopen(path, "rb");
    double ts;
    if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
    if (fread(&ts, 8, 1, f) != 1 || (long)fread(R->frame_buf, 8, (size_t)R->frame_len, f) != R->frame_len) {
        fclose(f);
        fprintf(stderr, "Could not load velocity data from %s\n", path);
        return 1;
    }
    fclose(f);
    int rc = fvc_upload_frame(R->ctx, mod, R->frame_buf);
    if (rc) return die("frame upload", R->ctx, rc);
    R->resident[mod] = 1;
    return 0;
}

/* Data_LoadedTMin / TMax for interval df (ompVC/main.c:188-195) and the
 * window of frames bracketing it. */
static int set_window(run_t *R, int df, double *tmin, double *tmax)
{
    fvcp_params *P = &R->P;
    int lo = P->int_dir > 0 ? df : df - 1;
    if (ensure_frame(R, lo) || ensure_frame(R, lo + 1)) return 1;
    *tmin = P->tmin + (P->int_dir > 0 ? df : df - 1) * P->tdelta;
    *tmax = *tmin + P->tdelta;
    int rc = fvc_set_window(R->ctx, frame_mod(P, lo), frame_mod(P, lo + 1), *tmin, *tmax);
    return rc ? die("frame window", R->ctx, rc) : 0;
}

/* =========================================================== FTLE */

typedef struct {
    fvc_job *job;
    double start, stop;
    int status; /* 0 unlaunched, 1 launched, 2 complete */
} slide_t;

static int write_ftle_ic(run_t *R, int n, const double *X, const int *eid, const int *left, const double *ldt,
                         const int *have, const double *wT, const double *wN)
{
    fvcp_params *P = &R->P;
    char path[2 * FVCP_STR];
    snprintf(path, sizeof(path), "%s%s", P->path_data, P->ftle_ic);
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
    fwrite(&P->fres[0], 4, 1, f);
    fwrite(&P->fres[1], 4, 1, f);
    fwrite(&P->fres[2], 4, 1, f);
    disk_fpt r;
    for (int p = 0; p < n; p++) {
        memset(&r, 0, sizeof(r));
        memcpy(r.pt.X, X + 3 * (long)p, 24);
        r.pt.eid = eid[p];
        r.pt.left = left[p];
        r.pt.ldt = ldt[p];
        r.have = have[p];
        r.ftT = wT[p];
        r.ftN = wN[p];
        if (fwrite(&r, sizeof(r), 1, f) != 1) { fclose(f); fprintf(stderr, "Could not write %s\n", path); return 1; }
    }
    fclose(f);
    return 0;
}

static int read_ftle_ic(run_t *R, int n, double *X, int *eid, int *left, double *ldt, int *have, double *wT, double *wN)
{
    fvcp_params *P = &R->P;
    char path[2 * FVCP_STR];
    snprintf(path, sizeof(path), "%s%s", P->path_data, P->ftle_ic);
    FILE *f = fopen(path, "rb");
    if (!f) {
        fprintf(stderr, "Error: Could not open file %s (file must be generated by flowVC with FTLE_GenerateMesh = 0)\n", path);
        return 1;
    }
    int r3[3];
    if (fread(r3, 4, 3, f) != 3 || r3[0] != P->fres[0] || r3[1] != P->fres[1] || r3[2] != P->fres[2]) {
        fclose(f);
        fprintf(stderr, "FTLE IC file %s does not match FTLE_CartMesh\n", path);
        return 1;
    }
    disk_fpt r;
    for (int p = 0; p < n; p++) {
        if (fread(&r, sizeof(r), 1, f) != 1) { fclose(f); fprintf(stderr, "Could not completely read %s\n", path); return 1; }
        memcpy(X + 3 * (long)p, r.pt.X, 24);
        eid[p] = r.pt.eid;
        left[p] = r.pt.left;
        ldt[p] = r.pt.ldt;
        have[p] = r.have;
        wT[p] = r.ftT;
        wN[p] = r.ftN;
    }
    fclose(f);
    return 0;
}

/* OutputFTLE, ompVC/ftle.c:1244-1329 */
static int output_ftle(run_t *R, slide_t *s, int ss, double IntT, int *numout, double *buf)
{
    fvcp_params *P = &R->P;
    char path[2 * FVCP_STR];
    int n = P->fres[0] * P->fres[1] * P->fres[2], rc;
    if ((ss == 0 && !P->ftle_var) || (P->ftle_var && !*numout)) {
        snprintf(path, sizeof(path), "%s%s.info", P->path_output, P->ftle_prefix);
        FILE *f = fopen(path, "w");
        if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        fprintf(f, "Int_Type\t\t=\t%10d\n", P->int_type);
        fprintf(f, "Int_TimeStep\t\t=\t%10g\n", P->int_h);
        fprintf(f, "Int_Accuracy\t\t=\t%10g\n", P->int_acc);
        fprintf(f, "Int_MinTimeStep\t\t=\t%10g\n", P->int_hmin);
        fprintf(f, "Int_MaxTimeStep\t\t=\t%10g\n", P->int_hmax);
        fprintf(f, "Int_TimeDirection\t=\t%10d\n", P->int_dir);
        fprintf(f, "Int_NormalFlow\t\t=\t%10d\n", P->normal_flow);
        fprintf(f, "Int_NormalFlowScaling\t=\t%10g\n\n", P->normal_scale);
        fprintf(f, "LocalSearchChecking\t=\t%10d\n\n", P->lsc);
        fprintf(f, "FTLE_GenerateMesh\t=\t%10d\n", P->ftle_genmesh);
        fprintf(f, "FTLE_ICFile\t\t=\t%s\n", P->ftle_ic);
        fprintf(f, "FTLE_IntTLength\t\t=\t%10g\n", P->ftle_T);
        fclose(f);
        snprintf(path, sizeof(path), "%s%s_Cartesian.bin", P->path_output, P->ftle_prefix);
        f = fopen(path, "wb");
        if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        fwrite(&P->fb[0], 8, 1, f); fwrite(&P->fb[1], 8, 1, f); fwrite(&P->fres[0], 4, 1, f);
        fwrite(&P->fb[2], 8, 1, f); fwrite(&P->fb[3], 8, 1, f); fwrite(&P->fres[1], 4, 1, f);
        fwrite(&P->fb[4], 8, 1, f); fwrite(&P->fb[5], 8, 1, f); fwrite(&P->fres[2], 4, 1, f);
        fclose(f);
    }
    double t0 = wall();
    if ((rc = fvc_ftle_reduce(s->job, IntT, buf, buf + n))) return die("FTLE reduction", R->ctx, rc);
    R->t_compute += wall() - t0;
    int id = P->ftle_var ? *numout : (P->int_dir > 0 ? ss : (P->out_tres - 1 - ss));
    if (R->dump_dir) {
        double *X = (double *)malloc(24 * (size_t)n);
        int *e = (int *)malloc(12 * (size_t)n);
        if (!X || !e || (rc = fvc_ftle_get_state(s->job, X, e, e + n, NULL, e + 2 * (long)n, NULL, NULL))) {
            free(X); free(e);
            return die("FTLE state", R->ctx, X && e ? rc : FVC_ERR_OOM);
        }
        snprintf(path, sizeof(path), "%s/state.%d.bin", R->dump_dir, id);
        FILE *f = fopen(path, "wb");
        if (f) {
            fwrite(&n, 4, 1, f);
            fwrite(X, 8, 3 * (size_t)n, f);
            fwrite(e, 4, 3 * (size_t)n, f);
            fclose(f);
        }
        free(X); free(e);
    }
    for (int which = 0; which < 2; which++) {
        snprintf(path, sizeof(path), which ? "%s%s_noT.%d.bin" : "%s%s.%d.bin", P->path_output, P->ftle_prefix, id);
        FILE *f = fopen(path, "wb");
        if (!f) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        int ok = fwrite(&s->start, 8, 1, f) == 1 && fwrite(buf + (which ? n : 0), 8, (size_t)n, f) == (size_t)n;
        fclose(f);
        if (!ok) { fprintf(stderr, "Could not write %s\n", path); return 1; }
    }
    if (P->ftle_var) (*numout)++;
    return 0;
}

static int run_ftle(run_t *R)
{
    fvcp_params *P = &R->P;
    int nsl = P->out_tres, rc, n = P->fres[0] * P->fres[1] * P->fres[2], numout = 0;
    slide_t *sl = (slide_t *)calloc((size_t)nsl, sizeof(slide_t));
    double *X = (double *)malloc(24 * (size_t)n), *ldt = (double *)malloc(8 * (size_t)n);
    double *wT = (double *)malloc(8 * (size_t)n), *wN = (double *)malloc(8 * (size_t)n);
    int *eid = (int *)malloc(4 * (size_t)n), *left = (int *)malloc(4 * (size_t)n), *have = (int *)malloc(4 * (size_t)n);
    double *buf = (double *)malloc(16 * (size_t)n);
    if (!sl || !X || !ldt || !wT || !wN || !eid || !left || !have || !buf) { fprintf(stderr, "out of memory\n"); return 1; }
    fvc_ftle_spec sp;
    memset(&sp, 0, sizeof(sp));
    sp.xmin = P->fb[0]; sp.xmax = P->fb[1]; sp.ymin = P->fb[2]; sp.ymax = P->fb[3]; sp.zmin = P->fb[4]; sp.zmax = P->fb[5];
    sp.xres = P->fres[0]; sp.yres = P->fres[1]; sp.zres = P->fres[2];
    sp.local_search_checking = P->lsc;
    double t0 = wall();
    for (int ss = 0; ss < nsl; ss++) {
        slide_t *s = &sl[ss];
        /* FTLE_Launches, ompVC/ftle.c:671-683 */
        s->start = P->out_tstart + ss * P->int_dir * P->out_tdelta;
        if (!P->periodic) {
            s->stop = MIN(P->out_tstart + ss * P->int_dir * P->out_tdelta + (double)P->int_dir * P->ftle_T, P->data_tmax);
            s->stop = MAX(s->stop, P->tmin);
            if (fabs(s->stop - s->start) < P->ftle_T - TINY)
                fprintf(stderr, "Warning: FTLE at time %f will have a maximum integration length of %f\n", s->start, fabs(s->stop - s->start));
        } else
            s->stop = P->out_tstart + ss * P->int_dir * P->out_tdelta + (double)P->int_dir * P->ftle_T;
        sp.start_time = s->start;
        sp.stop_time = s->stop;
        sp.generate = (ss == 0 && P->ftle_genmesh);
        if ((rc = fvc_ftle_create(R->ctx, &sp, &s->job))) return die("FTLE grid", R->ctx, rc);
        if (ss == 0) {
            if (P->ftle_genmesh) {
                if ((rc = fvc_ftle_get_state(s->job, X, eid, left, ldt, have, wT, wN))) return die("FTLE state", R->ctx, rc);
                if (write_ftle_ic(R, n, X, eid, left, ldt, have, wT, wN)) return 1;
            } else if (read_ftle_ic(R, n, X, eid, left, ldt, have, wT, wN)) return 1;
        }
        if (ss > 0 || !P->ftle_genmesh)
            if ((rc = fvc_ftle_set_state(s->job, X, eid, left, ldt, have, wT, wN))) return die("FTLE state", R->ctx, rc);
    }
    R->t_compute += wall() - t0;
    for (int df = P->first_frame; df != P->last_frame; df = df + P->int_dir) {
        double tmin, tmax;
        if (set_window(R, df, &tmin, &tmax)) return 1;
        printf("Data loaded in memory spans t = %g to %g\n", tmin, tmax);
        for (int ss = 0; ss < nsl; ss++) {
            slide_t *s = &sl[ss];
            if (s->status == 2 || !(s->status == 1 || (s->start <= tmax + TINY && s->start >= tmin - TINY))) continue;
            int launch = s->status == 0;
            double t1 = launch ? s->start : (P->int_dir > 0 ? tmin : tmax);
            double t2 = P->int_dir > 0 ? MIN(tmax, s->stop) : MAX(tmin, s->stop);
            s->status = 1;
            t0 = wall();
            /* queued without waiting; the slide's output (or the stats
               below) waits for it and reports device faults */
            if ((rc = fvc_ftle_interval(s->job, launch, t1, t2, NULL))) return die("FTLE interval", R->ctx, rc);
            R->t_compute += wall() - t0;
            if (((P->int_dir > 0) ? (s->stop - tmax) : (tmin - s->stop)) < TINY) {
                if (output_ftle(R, s, ss, P->ftle_T, &numout, buf)) return 1;
                s->status = 2;
            } else if (P->ftle_var && !fmod(df - P->first_frame, P->ftle_varfreq)) {
                if (output_ftle(R, s, ss, fabs(t2 - s->start), &numout, buf)) return 1;
            }
        }
    }
    for (int ss = 0; ss < nsl; ss++) {
        fvc_job_stats js;
        if ((rc = fvc_job_get_stats(sl[ss].job, &js))) return die("FTLE interval", R->ctx, rc);
        R->steps += js.steps_main + js.steps_early;
        fvc_job_destroy(sl[ss].job);
    }
    free(sl); free(X); free(ldt); free(wT); free(wN); free(eid); free(left); free(have); free(buf);
    return 0;
}

/* ========================================================= tracers */

static int read_seeds(run_t *R, int *nout, double **out, double center[3])
{
    fvcp_params *P = &R->P;
    double *pts = NULL;
    int n = 0;
    if (P->tr_genmesh) {
        /* GenerateTracerMesh, ompVC/tracers.c:1308-1347: kk, jj, ii order */
        n = P->tres3[0] * P->tres3[1] * P->tres3[2];
        pts = (double *)malloc(24 * (size_t)(n ? n : 1));
        if (!pts) return 1;
        long c = 0;
        for (int kk = 0; kk < P->tres3[2]; kk++)
            for (int jj = 0; jj < P->tres3[1]; jj++)
                for (int ii = 0; ii < P->tres3[0]; ii++) {
                    pts[3 * c] = P->tb[0] + ii * P->tdelta3[0];
                    pts[3 * c + 1] = P->tb[2] + jj * P->tdelta3[1];
                    pts[3 * c + 2] = P->tb[4] + kk * P->tdelta3[2];
                    c++;
                }
        center[0] = P->tb[0] + ((int)(P->tres3[0] / 2)) * P->tdelta3[0];
        center[1] = P->tb[2] + ((int)(P->tres3[1] / 2)) * P->tdelta3[1];
        center[2] = P->tb[4] + ((int)(P->tres3[2] / 2)) * P->tdelta3[2];
    } else {
        char path[2 * FVCP_STR];
        snprintf(path, sizeof(path), "%s%s", P->path_data, P->tr_infile);
        if (P->tr_format == 4) {
            FILE *f = fopen(path, "rb");
            if (!f || fread(&n, 4, 1, f) != 1 || n < 0) { fprintf(stderr, "Could not read Trace_NumTracers from %s\n", path); if (f) fclose(f); return 1; }
            pts = (double *)calloc((size_t)(n ? n : 1), 24);
            if (!pts) { fclose(f); return 1; }
            for (int i = 0; i < n; i++)
                if ((int)fread(pts + 3 * (long)i, 8, (size_t)P->dims, f) < P->dims) {
                    fprintf(stderr, "Could not read TraceIC_Array[%d].X from %s\n", i, path);
                    fclose(f); free(pts); return 1;
                }
            fclose(f);
        } else {
            FILE *f = fopen(path, "r");
            if (!f || fscanf(f, "%d\n", &n) != 1 || n < 0) { fprintf(stderr, "Could not read tracer count from %s\n", path); if (f) fclose(f); return 1; }
            pts = (double *)calloc((size_t)(n ? n : 1), 24);
            if (!pts) { fclose(f); return 1; }
            for (int i = 0; i < n; i++) {
                double *x = pts + 3 * (long)i;
                int r = P->dims == 3 ? fscanf(f, "%lf %lf %lf\n", &x[0], &x[1], &x[2]) : fscanf(f, "%lf %lf\n", &x[0], &x[1]);
                if (r != P->dims) { fprintf(stderr, "bad tracer line %d in %s\n", i, path); fclose(f); free(pts); return 1; }
            }
            fclose(f);
        }
        if (P->dims == 2)
            for (int i = 0; i < n; i++) pts[3 * (long)i + 2] = 0;
    }
    *nout = n;
    *out = pts;
    return 0;
}

/* OutputRT, ompVC/residencetime.c:21-185 (generated grids and seed lists):
 * <RT>_Cartesian.bin (the seed grid's bounds and resolution) or
 * <RT>_coordinates.bin (count, then the located seeds' positions), and per
 * release <RT>.<ss>.bin: its release time, then the residence time of each
 * tracer in seed order (fvc_tracer_residence). */
static int output_rt(run_t *R, int n, const double *icX, fvc_job **rel, const double *stop)
{
    fvcp_params *P = &R->P;
    char path[2 * FVCP_STR];
    FILE *f;
    if (P->tr_genmesh) {
        snprintf(path, sizeof(path), "%s%s_Cartesian.bin", P->path_output, P->tr_rtprefix);
        if (!(f = fopen(path, "wb"))) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        for (int a = 0; a < 3; a++) {
            fwrite(&P->tb[2 * a], 8, 1, f);
            fwrite(&P->tb[2 * a + 1], 8, 1, f);
            fwrite(&P->tres3[a], 4, 1, f);
        }
        fclose(f);
    } else {
        snprintf(path, sizeof(path), "%s%s_coordinates.bin", P->path_output, P->tr_rtprefix);
        if (!(f = fopen(path, "wb"))) { fprintf(stderr, "Could not open file %s\n", path); return 1; }
        fwrite(&n, 4, 1, f);
        fwrite(icX, 24, (size_t)n, f);
        fclose(f);
    }
    double *rt = (double *)malloc(8 * (size_t)(n ? n : 1));
    if (!rt) return 1;
    for (int ss = 0; ss < P->tr_nlaunch; ss++) {
        double time = P->out_tstart + ss * P->tr_spacing;
        int rc = fvc_tracer_residence(rel[ss], time, stop[ss], rt);
        if (rc) { free(rt); return die("residence time", R->ctx, rc); }
        snprintf(path, sizeof(path), "%s%s.%d.bin", P->path_output, P->tr_rtprefix, ss);
        if (!(f = fopen(path, "wb"))) { free(rt); fprintf(stderr, "Could not open file %s\n", path); return 1; }
        fwrite(&time, 8, 1, f);
        fwrite(rt, 8, (size_t)n, f);
        fclose(f);
    }
    free(rt);
    return 0;
}

/* OutputCET, ompVC/exposuretime.c:175-302: <RT>_CET.0.bin and <RT>_MET.0.bin
 * (time stamp -1, then a double per element) and <RT>_ENC.0.bin (time stamp
 * -1, then an int per element), from fvc_cet_results. */
static int output_cet(run_t *R, int ntracers)
{
    fvcp_params *P = &R->P;
    long E = R->nelem;
    double *cet = (double *)malloc(8 * (size_t)E), *met = (double *)malloc(8 * (size_t)E);
    int *enc = (int *)malloc(4 * (size_t)E);
    if (!cet || !met || !enc) return 1;
    int rc = fvc_cet_results(R->ctx, ntracers, cet, met, enc);
    if (rc) return die("exposure time", R->ctx, rc);
    const char *suffix[3] = {"CET", "MET", "ENC"};
    double t = -1.0;
    for (int k = 0; k < 3; k++) {
        char path[2 * FVCP_STR];
        snprintf(path, sizeof(path), "%s%s_%s.0.bin", P->path_output, P->tr_rtprefix, suffix[k]);
        FILE *f = fopen(path, "wb");
        if (!f) { fprintf(stderr, "Could not open %s\n", path); return 1; }
        fwrite(&t, 8, 1, f);
        if (k == 0) fwrite(cet, 8, (size_t)E, f);
        else if (k == 1) fwrite(met, 8, (size_t)E, f);
        else fwrite(enc, 4, (size_t)E, f);
        fclose(f);
    }
    free(cet); free(met); free(enc);
    return 0;
}

/* Tracer outputs are written by a thread of their own (OutputTracers,
 * ompVC/tracers.c:1763-1816): the release loop queues each output with
 * fvc_tracer_output_begin and goes on advancing; the writer waits for the
 * outputs in ticket order, appends each to its output file (created when
 * the first release with tracers to write reaches it, as ompVC creates it)
 * and frees the slot.  At most FVC_TRACER_OUTPUT_SLOTS outputs are
 * outstanding. */
typedef struct {
    long long ticket;
    int frame;
    double time;
} wr_item;

typedef struct {
    fvc_ctx *ctx;
    const char *dir, *prefix;
    wr_item q[FVC_TRACER_OUTPUT_SLOTS];
    int head, count, inflight, stop, err;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    pthread_t th;
    FILE *fo;
    int fo_frame;
    char msg[256];
} writer_t;

static void *writer_main(void *arg)
{
    writer_t *W = (writer_t *)arg;
    for (;;) {
        pthread_mutex_lock(&W->mu);
        while (W->count == 0 && !W->stop) pthread_cond_wait(&W->cv, &W->mu);
        if (W->count == 0) {
            pthread_mutex_unlock(&W->mu);
            break;
        }
        wr_item it = W->q[W->head];
        W->head = (W->head + 1) % FVC_TRACER_OUTPUT_SLOTS;
        W->count--;
        int err = W->err;
        pthread_mutex_unlock(&W->mu);
        const double *X = NULL;
        long long cnt = 0;
        int rc = err ? 0 : fvc_tracer_output_wait(W->ctx, it.ticket, &X, &cnt);
        if (!err && rc) {
            err = rc;
            snprintf(W->msg, sizeof(W->msg), "tracer output %d: status %d", it.frame, rc);
        }
        if (!err && W->fo && W->fo_frame != it.frame) {
            fclose(W->fo);
            W->fo = NULL;
        }
        if (!err && cnt > 0) {
            if (!W->fo) {
                char path[2 * FVCP_STR];
                snprintf(path, sizeof(path), "%s%s.%d.bin", W->dir, W->prefix, it.frame);
                W->fo = fopen(path, "wb");
                W->fo_frame = it.frame;
                if (!W->fo || fwrite(&it.time, 8, 1, W->fo) != 1) {
                    err = FVC_ERR_IO;
                    snprintf(W->msg, sizeof(W->msg), "Could not open file %s", path);
                }
            }
            if (!err && fwrite(X, 24, (size_t)cnt, W->fo) != (size_t)cnt) {
                err = FVC_ERR_IO;
                snprintf(W->msg, sizeof(W->msg), "Could not write output %d", it.frame);
            }
        }
        fvc_tracer_output_release(W->ctx, it.ticket);
        pthread_mutex_lock(&W->mu);
        W->inflight--;
        if (err && !W->err) W->err = err;
        pthread_cond_broadcast(&W->cv);
        pthread_mutex_unlock(&W->mu);
    }
    if (W->fo) fclose(W->fo);
    W->fo = NULL;
    return NULL;
}

static int writer_start(writer_t *W, fvc_ctx *ctx, const char *dir, const char *prefix)
{
    memset(W, 0, sizeof(*W));
    W->ctx = ctx;
    W->dir = dir;
    W->prefix = prefix;
    W->fo_frame = -1;
    pthread_mutex_init(&W->mu, NULL);
    pthread_cond_init(&W->cv, NULL);
    return pthread_create(&W->th, NULL, writer_main, W) ? 1 : 0;
}

/* queues output `frame` of job (waits while every slot is taken) */
static int writer_submit(writer_t *W, fvc_job *job, int always, int frame, double time)
{
    pthread_mutex_lock(&W->mu);
    while (W->inflight >= FVC_TRACER_OUTPUT_SLOTS && !W->err) pthread_cond_wait(&W->cv, &W->mu);
    int err = W->err;
    if (!err) W->inflight++;
    pthread_mutex_unlock(&W->mu);
    if (err) return err;
    long long ticket = 0;
    int rc = fvc_tracer_output_begin(job, always, &ticket);
    pthread_mutex_lock(&W->mu);
    if (rc) {
        W->inflight--;
    } else {
        wr_item it = {ticket, frame, time};
        W->q[(W->head + W->count) % FVC_TRACER_OUTPUT_SLOTS] = it;
        W->count++;
        pthread_cond_broadcast(&W->cv);
    }
    pthread_mutex_unlock(&W->mu);
    return rc;
}

/* drains the queue and joins the thread; returns the first failure */
static int writer_stop(writer_t *W)
{
    pthread_mutex_lock(&W->mu);
    W->stop = 1;
    pthread_cond_broadcast(&W->cv);
    pthread_mutex_unlock(&W->mu);
    pthread_join(W->th, NULL);
    pthread_mutex_destroy(&W->mu);
    pthread_cond_destroy(&W->cv);
    if (W->err) fprintf(stderr, "%s\n", W->msg[0] ? W->msg : "tracer output failed");
    return W->err;
}

static int run_tracers(run_t *R)
{
    fvcp_params *P = &R->P;
    int n = 0, rc, nl = P->tr_nlaunch;
    double *seeds = NULL, center[3] = {0, 0, 0};
    if (read_seeds(R, &n, &seeds, center)) return 1;
    fvc_tracer_spec sp;
    memset(&sp, 0, sizeof(sp));
    sp.local_search_checking = P->lsc;
    sp.seed_chain = P->tr_genmesh ? 1 : 0;
    memcpy(sp.center, center, sizeof(center));
    fvc_job **rel = (fvc_job **)calloc((size_t)nl, sizeof(fvc_job *));
    double *start = (double *)calloc((size_t)nl, 8), *stop = (double *)calloc((size_t)nl, 8);
    int *status = (int *)calloc((size_t)nl, sizeof(int));
    if (!rel || !start || !stop || !status) { fprintf(stderr, "out of memory\n"); return 1; }
    double t0 = wall();
    for (int ss = 0; ss < nl; ss++) {
        if ((rc = fvc_tracer_create(R->ctx, &sp, n, seeds, &rel[ss]))) return die("tracer seeds", R->ctx, rc);
        start[ss] = P->out_tstart + P->int_dir * ss * P->tr_spacing;
        stop[ss] = P->int_dir > 0 ? MIN(start[ss] + P->tr_T, P->out_tend) : MAX(start[ss] - P->tr_T, P->out_tend);
    }
    if (P->tr_cet && (rc = fvc_cet_enable(R->ctx, P->tr_cetsub))) return die("exposure time", R->ctx, rc);
    R->t_compute += wall() - t0;
    double *icX = (double *)malloc(24 * (size_t)(n ? n : 1));
    if (!icX) { fprintf(stderr, "out of memory\n"); return 1; }
    {   /* the located seeds, as ompVC stores them (ompVC/tracers.c:1258-1272) */
        char path[2 * FVCP_STR];
        snprintf(path, sizeof(path), "%s%s.IC", P->path_data, P->tr_prefix);
        int *eid = (int *)malloc(4 * (size_t)(n ? n : 1)), *left = (int *)malloc(4 * (size_t)(n ? n : 1));
        double *X = icX, *ldt = (double *)malloc(8 * (size_t)(n ? n : 1));
        if ((rc = fvc_tracer_get_state(rel[0], X, eid, left, ldt))) return die("tracer seeds", R->ctx, rc);
        FILE *f = fopen(path, "wb");
        if (f && eid && left && ldt) {
            fwrite(&n, 4, 1, f);
            disk_lpt r;
            for (int i = 0; i < n; i++) {
                memset(&r, 0, sizeof(r));
                memcpy(r.X, X + 3 * (long)i, 24);
                r.eid = eid[i]; r.left = left[i]; r.ldt = ldt[i];
                fwrite(&r, sizeof(r), 1, f);
            }
        }
        if (f) fclose(f);
        free(eid); free(left); free(ldt);
    }
    int outputframe = 0;
    double next = P->out_tstart;
    writer_t W;
    if (writer_start(&W, R->ctx, P->path_output, P->tr_prefix)) { fprintf(stderr, "writer thread\n"); return 1; }
    for (int df = P->first_frame; df != P->last_frame; df = df + P->int_dir) {
        double tmin, tmax;
        if (set_window(R, df, &tmin, &tmax)) return 1;
        /* Compute_Tracer, ompVC/tracers.c:25-289 */
        double t1 = P->int_dir > 0 ? tmin : tmax, t2;
        while (((P->int_dir > 0) ? (t1 - tmax) : (tmin - t1)) < 0) {
            t2 = P->int_dir > 0 ? MIN(next, tmax) : MAX(tmin, next);
            int out_now = fabs(next - t2) < TINY && outputframe < P->out_tres;
            for (int ss = 0; ss < nl; ss++) {
                if (status[ss] != 2 && (status[ss] == 1 || (start[ss] <= MAX(t1, t2) && start[ss] >= MIN(t1, t2)))) {
                    t0 = wall();
                    if (status[ss] == 0) {
                        status[ss] = 1;
                        t1 = start[ss];
                        if ((rc = fvc_tracer_launch(rel[ss], start[ss]))) { writer_stop(&W); return die("tracer release", R->ctx, rc); }
                    }
                    /* queued, not waited for: its steps are counted from the job's statistics */
                    if ((rc = fvc_tracer_advance(rel[ss], t1, t2, NULL))) { writer_stop(&W); return die("tracer advection", R->ctx, rc); }
                    /* OutputTracers, ompVC/tracers.c:1777-1804, on the writer thread */
                    double time = P->out_tstart + outputframe * P->int_dir * P->out_tdelta;
                    if (out_now && (rc = writer_submit(&W, rel[ss], P->tr_always, outputframe, time))) {
                        writer_stop(&W);
                        return die("tracer output", R->ctx, rc);
                    }
                    R->t_compute += wall() - t0;
                }
                if (((P->int_dir > 0) ? (stop[ss] - t2) : (t2 - stop[ss])) < TINY) status[ss] = 2;
            }
            if (fabs(t2 - next) < TINY) {
                next += P->int_dir * P->out_tdelta;
                outputframe++;
                if (outputframe >= P->out_tres) break;
            }
            t1 = t2;
        }
    }
    if (writer_stop(&W)) return 1;
    for (int ss = 0; ss < nl; ss++) {
        fvc_job_stats js;
        if ((rc = fvc_job_get_stats(rel[ss], &js))) return die("tracer advection", R->ctx, rc);
        R->steps += js.steps_main;
    }
    if (P->tr_rt && output_rt(R, n, icX, rel, stop)) return 1;
    if (P->tr_cet && output_cet(R, n)) return 1;
    for (int ss = 0; ss < nl; ss++) fvc_job_destroy(rel[ss]);
    free(rel); free(start); free(stop); free(status); free(seeds); free(icX);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s inputfile [--device N] [--stats] [--dump-state DIR] [--precision fp64|bf16|fp16]\n",
                argv[0]);
        return 1;
    }
    int device = 0, stats = 0, prec = FVC_PREC_FP64;
    run_t R;
    memset(&R, 0, sizeof(R));
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--stats")) stats = 1;
        else if (!strcmp(argv[i], "--dump-state") && i + 1 < argc) R.dump_dir = argv[++i];
        else if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
            const char *p = argv[++i];
            if (!strcmp(p, "fp64")) prec = FVC_PREC_FP64;
            else if (!strcmp(p, "bf16")) prec = FVC_PREC_BF16;
            else if (!strcmp(p, "fp16")) prec = FVC_PREC_FP16;
            else {
                fprintf(stderr, "unknown precision '%s' (fp64, bf16 or fp16)\n", p);
                return 1;
            }
        }
    }
    char err[1024];
    double t_start = wall();
    if (fvcp_read(argv[1], &R.P, err, sizeof(err)) || fvcp_check_derive(&R.P, err, sizeof(err))) {
        fprintf(stderr, "\nERROR:\n%s\n", err);
        return 1;
    }
    fvc_opts o;
    memset(&o, 0, sizeof(o));
    o.device = device;
    o.dims = R.P.dims;
    o.mesh_type = R.P.mesh_type;
    int rc = fvc_create(&R.ctx, &o);
    if (rc) return die("could not create a GPU context", NULL, rc);
    double bounds[6];
    memcpy(bounds, R.P.bounds, sizeof(bounds));
    if ((rc = fvc_set_bounds(R.ctx, bounds)) || (rc = fvc_set_integrator(R.ctx, R.P.int_type, R.P.int_h, R.P.extrapolate)))
        return die("settings", R.ctx, rc);
    if (R.P.int_type == 2 && (rc = fvc_set_rkf(R.ctx, R.P.int_acc, R.P.int_hmin, R.P.int_hmax)))
        return die("RKF settings", R.ctx, rc);
    if (prec != FVC_PREC_FP64 && (rc = fvc_set_precision(R.ctx, prec)))
        return die("precision", R.ctx, rc);
    int bad = load_mesh(&R);
    if (!bad) bad = pipe_start(&R);
    if (!bad) bad = R.P.ftle_compute ? run_ftle(&R) : run_tracers(&R);
    pipe_stop(&R);
    if (!bad && stats)
        printf("{\"steps\": %lld, \"compute_seconds\": %.6f, \"total_seconds\": %.6f}\n", R.steps, R.t_compute, wall() - t_start);
    free(R.frame_buf);
    free(R.resident);
    fvc_destroy(R.ctx);
    if (!bad) printf("\nSimulation complete!\n");
    return bad;
}
