/*
 * orc_jobs.c -- CPU oracle: FTLE and tracer jobs and the full .in run.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h).
 *
 * FTLE follows ompVC/ftle.c with one restatement: the serial (i,j,k) loop of
 * ComputeFTLE (ompVC/ftle.c:109-173), whose early-exit FTLE depends on the
 * loop order, is computed in two passes:
 *   pass 1  advects every live point over the interval from its frame-start
 *           state and records exits (parallel);
 *   pass 2  gives every point q without an FTLE value the early FTLE of its
 *           trigger, the exiting member of {q} + its 6 grid neighbours with the
 *           smallest linear index (i*YRes + j)*ZRes + k -- the point whose
 *           GetFTLEForPointEarly call reaches q first in the serial loop.
 *           Points the serial loop has already passed carry their updated
 *           element index when the trigger is processed (ftle.c:167-168);
 *           pass 2 hands the same index to the advections it repeats.
 * The result is identical to the serial loop for every point.
 */
#include <math.h>
#include <omp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "orc_int.h"
#include "orc_params.h"

/* ---------------------------------------------------------------- helpers */

static int set_err(char *err, int errlen, int code, const char *fmt, ...)
{
    if (err && errlen > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)errlen, fmt, ap);
        va_end(ap);
    }
    return code;
}

static double now_s(void) { return omp_get_wtime(); }

/* On-disk LagrangianPoint / FTLEPoint (ompVC/structs.h:21-36): 80 and 104 B. */
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
    orc_ctx ctx;
    orc_params P;
    double *frame_lo, *frame_hi;
    int lo_id, hi_id;             /* frame indices held (before wrap) */
    long frame_len;               /* doubles per frame */
} orc_run_state;

/* frame index -> file suffix with ompVC's wrap (ompVC/velocity.c:174-177) */
static int frame_suffix(const orc_params *P, int frame)
{
    int mod = (int)fmod((double)frame, (double)(P->tres - 1));
    if (mod < 0) mod += P->tres - 1;
    return P->suffix_tmin + mod * P->suffix_tdelta;
}

static int load_frame(orc_run_state *S, int frame, double *dst, char *err, int errlen)
{
    char path[2 * ORC_STR];
    snprintf(path, sizeof(path), "%s%s_vel.%d.bin", S->P.path_data, S->P.prefix, frame_suffix(&S->P, frame));
    FILE *f = fopen(path, "rb");
    if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
    double ts;
    if (fread(&ts, 8, 1, f) != 1 || (long)fread(dst, 8, (size_t)S->frame_len, f) != S->frame_len) {
        fclose(f);
        return set_err(err, errlen, ORC_ERR_IO, "Could not read velocity data from %s", path);
    }
    fclose(f);
    return ORC_OK;
}

/* Make the frames at LoadedTMin / LoadedTMax resident (the two-slot window
 * of ompVC/main.c:170-195). */
static int window(orc_run_state *S, int df, char *err, int errlen)
{
    const orc_params *P = &S->P;
    int lo = P->int_dir > 0 ? df : df - 1, hi = lo + 1, rc;
    if (!(S->lo_id == lo && S->hi_id == hi)) {
        if (S->hi_id == lo || S->lo_id == hi) {
            double *t = S->frame_lo; S->frame_lo = S->frame_hi; S->frame_hi = t;
            int ti = S->lo_id; S->lo_id = S->hi_id; S->hi_id = ti;
        }
        if (S->lo_id != lo) { if ((rc = load_frame(S, lo, S->frame_lo, err, errlen))) return rc; S->lo_id = lo; }
        if (S->hi_id != hi) { if ((rc = load_frame(S, hi, S->frame_hi, err, errlen))) return rc; S->hi_id = hi; }
    }
    if (P->int_dir > 0) {
        S->ctx.tmin = P->tmin + df * P->tdelta;
        S->ctx.tmax = S->ctx.tmin + P->tdelta;
    } else {
        S->ctx.tmin = P->tmin + (df - 1) * P->tdelta;
        S->ctx.tmax = S->ctx.tmin + P->tdelta;
    }
    S->ctx.f0 = S->frame_lo;
    S->ctx.f1 = S->frame_hi;
    return ORC_OK;
}

static int load_mesh(orc_run_state *S, char *err, int errlen)
{
    orc_params *P = &S->P;
    orc_ctx *c = &S->ctx;
    char path[2 * ORC_STR];
    memset(c, 0, sizeof(*c));
    c->dims = P->dims;
    c->mesh_type = P->mesh_type;
    memcpy(c->bounds, P->bounds, sizeof(c->bounds));
    c->int_type = (P->int_type >= 1 && P->int_type <= 3) ? P->int_type : 0;
    c->h = P->int_h;
    c->acc = P->int_acc;
    c->hmin = P->int_hmin;
    c->hmax = P->int_hmax;
    c->extrapolate = P->extrapolate;
    if (P->mesh_type == 0) {
        snprintf(path, sizeof(path), "%s%s_Cartesian.bin", P->path_data, P->prefix);
        FILE *f = fopen(path, "rb");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        double v[6];
        int r[3];
        int ok = fread(&v[0], 8, 2, f) == 2 && fread(&r[0], 4, 1, f) == 1 && fread(&v[2], 8, 2, f) == 2 &&
                 fread(&r[1], 4, 1, f) == 1 && fread(&v[4], 8, 2, f) == 2 && fread(&r[2], 4, 1, f) == 1;
        fclose(f);
        if (!ok) return set_err(err, errlen, ORC_ERR_IO, "Could not read %s", path);
        orc_grid *g = &c->g;
        g->xmin = v[0]; g->xmax = v[1]; g->xres = r[0];
        g->ymin = v[2]; g->ymax = v[3]; g->yres = r[1];
        g->zmin = v[4]; g->zmax = v[5]; g->zres = r[2];
        if (g->xres < 2 || g->xmin >= g->xmax) return set_err(err, errlen, ORC_ERR_ARG, "Insufficient resolution of velocity data in x-direction");
        g->dx = (g->xmax - g->xmin) / (g->xres - 1);
        if (g->yres < 2 || g->ymin >= g->ymax) return set_err(err, errlen, ORC_ERR_ARG, "Insufficient resolution of velocity data in y-direction");
        g->dy = (g->ymax - g->ymin) / (g->yres - 1);
        if (P->dims == 3) {
            if (g->zres < 2 || g->zmin >= g->zmax) return set_err(err, errlen, ORC_ERR_ARG, "Insufficient resolution of velocity data in z-direction");
            g->dz = (g->zmax - g->zmin) / (g->zres - 1);
        } else {
            g->zmin = 0; g->zmax = 0; g->zres = 1; g->dz = 0;
        }
        S->frame_len = 3L * g->xres * g->yres * g->zres;
    } else {
        int n, e, e2;
        snprintf(path, sizeof(path), "%s%s_coordinates.bin", P->path_data, P->prefix);
        FILE *f = fopen(path, "rb");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        if (fread(&n, 4, 1, f) != 1 || n <= 0) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "bad node count in %s", path); }
        c->xyz = (double *)malloc(sizeof(double) * 3 * (size_t)n);
        if (!c->xyz || (long)fread(c->xyz, 8, 3 * (size_t)n, f) != 3L * n) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "Could not read %s", path); }
        fclose(f);
        snprintf(path, sizeof(path), "%s%s_connectivity.bin", P->path_data, P->prefix);
        f = fopen(path, "rb");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        if (fread(&e, 4, 1, f) != 1 || e <= 0) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "bad element count in %s", path); }
        c->conn = (int *)malloc(sizeof(int) * 4 * (size_t)e);
        if (!c->conn || (long)fread(c->conn, 4, 4 * (size_t)e, f) != 4L * e) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "Could not read %s", path); }
        fclose(f);
        snprintf(path, sizeof(path), "%s%s_adjacency.bin", P->path_data, P->prefix);
        f = fopen(path, "rb");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        if (fread(&e2, 4, 1, f) != 1 || e2 != e) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "Incompatible number of elements listed in connectivity and adjacency files"); }
        c->adj = (int *)malloc(sizeof(int) * 4 * (size_t)e);
        if (!c->adj || (long)fread(c->adj, 4, 4 * (size_t)e, f) != 4L * e) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "Could not read %s", path); }
        fclose(f);
        c->nnodes = n;
        c->nelem = e;
        S->frame_len = 3L * n;
    }
    S->frame_lo = (double *)malloc(sizeof(double) * (size_t)S->frame_len);
    S->frame_hi = (double *)malloc(sizeof(double) * (size_t)S->frame_len);
    if (!S->frame_lo || !S->frame_hi) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    S->lo_id = S->hi_id = -0x7fffffff;
    return ORC_OK;
}

static void free_state(orc_run_state *S)
{
    free(S->ctx.xyz); free(S->ctx.conn); free(S->ctx.adj);
    free(S->frame_lo); free(S->frame_hi);
}

/* ======================================================================= FTLE */

typedef struct {
    int n, xr, yr, zr;
    double *X, *V, *ldt, *ftT, *ftN;
    int *eid, *left, *have;
    double start, stop;
    int status; /* 0 unlaunched, 1 launched, 2 complete */
    int nout;   /* FTLE_NumOutput (variation mode) */
} ftle_slide;

/* scratch for one interval */
typedef struct {
    double *Xn, *Vn, *te;
    int *en, *ln, *integ, *exited;
} ftle_scratch;

static void mark_outside(ftle_slide *s, int i, int j, int k, int *have, int *left, double *ldt, double *ftT, double *ftN)
{
    int YZ = s->yr * s->zr, p = (i * s->yr + j) * s->zr + k;
    left[p] = 1; ldt[p] = -1.0; ftT[p] = -1.0; ftN[p] = -1.0; have[p] = 1;
    if (i > 0) have[p - YZ] = 1;
    if (i < s->xr - 1) have[p + YZ] = 1;
    if (j > 0) have[p - s->zr] = 1;
    if (j < s->yr - 1) have[p + s->zr] = 1;
    if (k > 0) have[p - 1] = 1;
    if (k < s->zr - 1) have[p + 1] = 1;
}

/* InitializeFTLEArray, ompVC/ftle.c:383-628 (FTLE_GenerateMesh = 1), with the
 * same serial guess chain for locating seeds on an unstructured mesh. */
static int ftle_seed(orc_run_state *S, ftle_slide *s, long long *ngs)
{
    const orc_params *P = &S->P;
    const orc_ctx *c = &S->ctx;
    int xr = s->xr, yr = s->yr, zr = s->zr;
    for (int i = 0; i < xr; i++)
        for (int j = 0; j < yr; j++)
            for (int k = 0; k < zr; k++) {
                int p = (i * yr + j) * zr + k;
                s->X[3 * p] = P->fb[0] + i * P->fdelta[0];
                s->X[3 * p + 1] = P->fb[2] + j * P->fdelta[1];
                s->X[3 * p + 2] = P->fb[4] + k * P->fdelta[2];
                s->ftT[p] = 0.0; s->ftN[p] = 0.0; s->have[p] = 0; s->left[p] = 0; s->ldt[p] = 0.0;
                s->eid[p] = -1;
                s->V[3 * p] = s->V[3 * p + 1] = s->V[3 * p + 2] = 0.0;
            }
    for (int i = 0; i < xr; i++)
        for (int j = 0; j < yr; j++)
            for (int k = 0; k < zr; k++) {
                int p = (i * yr + j) * zr + k;
                if (orc_outside_domain(c, &s->X[3 * p])) mark_outside(s, i, j, k, s->have, s->left, s->ldt, s->ftT, s->ftN);
            }
    if (c->mesh_type != 1) return ORC_OK;
    double Xs[3];
    Xs[0] = P->fb[0] + ((int)(xr / 2)) * P->fdelta[0];
    Xs[1] = P->fb[2] + ((int)(yr / 2)) * P->fdelta[1];
    Xs[2] = P->fb[4] + ((int)(zr / 2)) * P->fdelta[2];
    int seed = orc_global(c, Xs), guess = -1, err = 0;
    if (seed >= 0) guess = seed;
    int iguess = -1, jguess = -1;
    for (int i = 0; i < xr; i++) {
        iguess = -1;
        for (int j = 0; j < yr; j++) {
            jguess = -1;
            for (int k = 0; k < zr; k++) {
                int p = (i * yr + j) * zr + k;
                if (s->left[p]) continue;
                double *X = &s->X[3 * p];
                if (seed < 0) {
                    seed = orc_global(c, X);
                    (*ngs)++;
                    if (seed < 0) mark_outside(s, i, j, k, s->have, s->left, s->ldt, s->ftT, s->ftN);
                    else { s->eid[p] = seed; guess = seed; jguess = seed; iguess = seed; }
                    continue;
                }
                int index = orc_local(c, X, guess, &err);
                if (index < 0) index = orc_local(c, X, seed, &err);
                if (index < 0 && P->lsc) { index = orc_global(c, X); (*ngs)++; }
                if (index < 0) { mark_outside(s, i, j, k, s->have, s->left, s->ldt, s->ftT, s->ftN); continue; }
                s->eid[p] = index;
                guess = index;
                if (jguess < 0) jguess = index;
                if (iguess < 0) iguess = index;
            }
        }
        /* ompVC/ftle.c:597-598 stand after the j loop (the indentation there
         * suggests a restart per row): within a plane the guess runs on from
         * row to row, and the next plane starts from the first element found
         * in this plane's last row */
        if (jguess >= 0) guess = jguess;
    }
    if (iguess >= 0) guess = iguess; /* ompVC/ftle.c:600-601, after the i loop: no effect */
    return err ? ORC_ERR_WALK : ORC_OK;
}

static int write_ic(orc_run_state *S, ftle_slide *s, char *err, int errlen)
{
    char path[2 * ORC_STR];
    snprintf(path, sizeof(path), "%s%s", S->P.path_data, S->P.ftle_ic);
    FILE *f = fopen(path, "wb");
    if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
    fwrite(&s->xr, 4, 1, f); fwrite(&s->yr, 4, 1, f); fwrite(&s->zr, 4, 1, f);
    disk_fpt r;
    for (int p = 0; p < s->n; p++) {
        memset(&r, 0, sizeof(r));
        memcpy(r.pt.X, &s->X[3 * p], 24);
        r.pt.eid = s->eid[p]; r.pt.left = s->left[p]; r.pt.ldt = s->ldt[p];
        r.have = s->have[p]; r.ftT = s->ftT[p]; r.ftN = s->ftN[p];
        if (fwrite(&r, sizeof(r), 1, f) != 1) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "write failed %s", path); }
    }
    fclose(f);
    return ORC_OK;
}

static int read_ic(orc_run_state *S, ftle_slide *s, char *err, int errlen)
{
    char path[2 * ORC_STR];
    snprintf(path, sizeof(path), "%s%s", S->P.path_data, S->P.ftle_ic);
    FILE *f = fopen(path, "rb");
    if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
    int r3[3];
    if (fread(r3, 4, 3, f) != 3 || r3[0] != s->xr || r3[1] != s->yr || r3[2] != s->zr) {
        fclose(f); return set_err(err, errlen, ORC_ERR_IO, "FTLE IC file %s does not match the FTLE grid", path);
    }
    disk_fpt r;
    for (int p = 0; p < s->n; p++) {
        if (fread(&r, sizeof(r), 1, f) != 1) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "short read %s", path); }
        memcpy(&s->X[3 * p], r.pt.X, 24); memcpy(&s->V[3 * p], r.pt.V, 24);
        s->eid[p] = r.pt.eid; s->left[p] = r.pt.left; s->ldt[p] = r.pt.ldt;
        s->have[p] = r.have; s->ftT[p] = r.ftT; s->ftN[p] = r.ftN;
    }
    fclose(f);
    return ORC_OK;
}

/* Advect_FTLEPoint (ompVC/ftle.c:1205-1227) for point p with element eid. */
static int adv_point(const orc_ctx *c, const ftle_slide *s, int p, int eid, double t1, double t2, orc_pt *out, long long *steps)
{
    out->X[0] = s->X[3 * p]; out->X[1] = s->X[3 * p + 1]; out->X[2] = s->X[3 * p + 2];
    out->V[0] = s->V[3 * p]; out->V[1] = s->V[3 * p + 1]; out->V[2] = s->V[3 * p + 2];
    out->left = s->left[p];
    out->eid = eid;
    out->ldt = 0.0;
    return orc_advect_pt(c, out, t1, t2, steps);
}

/* Cauchy-Green tensor and FTLE from the six stencil positions, in the order
 * of ompVC/ftle.c:1000-1044 and 1159-1197.  Returns lambda. */
static double stencil_lambda(int dims, const double *L, const double *R, const double *B, const double *T,
                             const double *Bk, const double *F, double fx, double fy, double fz,
                             double dx, double dy, double dz)
{
    double D[3][3], C[9];
    if (dims == 3) {
        D[0][2] = (F[0] - Bk[0]) / (fz * dz);
        D[1][2] = (F[1] - Bk[1]) / (fz * dz);
        D[2][0] = (R[2] - L[2]) / (fx * dx);
        D[2][1] = (T[2] - B[2]) / (fy * dy);
        D[2][2] = (F[2] - Bk[2]) / (fz * dz);
    } else {
        D[0][2] = 0; D[1][2] = 0; D[2][0] = 0; D[2][1] = 0; D[2][2] = 0;
    }
    D[0][0] = (R[0] - L[0]) / (fx * dx);
    D[0][1] = (T[0] - B[0]) / (fy * dy);
    D[1][0] = (R[1] - L[1]) / (fx * dx);
    D[1][1] = (T[1] - B[1]) / (fy * dy);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            double acc = 0;
            for (int m = 0; m < 3; m++) acc += D[m][a] * D[m][b];
            C[3 * a + b] = acc;
        }
    return orc_max_eig(C);
}

/* GetFTLEForPointEarly, ompVC/ftle.c:788-1048, for point q served by trigger
 * trig exiting at te.  eid_of gives the element the serial loop would hold
 * for each point when trig is processed. */
static int early_ftle(const orc_run_state *S, ftle_slide *s, const ftle_scratch *w, int q, int trig,
                      double t1, double te, long long *steps)
{
    const orc_ctx *c = &S->ctx;
    int xr = s->xr, yr = s->yr, zr = s->zr, YZ = yr * zr;
    int k = q % zr, j = (q / zr) % yr, i = q / YZ;
    int nb[6] = {i > 0 ? q - YZ : -1, i < xr - 1 ? q + YZ : -1, j > 0 ? q - zr : -1,
                 j < yr - 1 ? q + zr : -1, k > 0 ? q - 1 : -1, k < zr - 1 ? q + 1 : -1};
#define EID_OF(p) (((p) < trig && w->integ[p] && !w->exited[p]) ? w->en[p] : s->eid[p])
    orc_pt tmp, at_te[6];
    double lt[6];
    int rc = 0;
    for (int n = 0; n < 6; n++) {
        lt[n] = te;
        if (nb[n] < 0) continue;
        if ((rc = adv_point(c, s, nb[n], EID_OF(nb[n]), t1, te, &at_te[n], steps))) return rc;
        if (at_te[n].left) lt[n] = at_te[n].ldt;
    }
    double mt = ORC_MIN(te, ORC_MIN(lt[5], ORC_MIN(lt[4], ORC_MIN(lt[3], ORC_MIN(lt[2], ORC_MIN(lt[1], lt[0]))))));
    orc_pt self;
    if ((rc = adv_point(c, s, q, EID_OF(q), t1, mt, &self, steps))) return rc;
    /* neighbours at the minimum exit time; Advect is deterministic, so when
     * mt == te the positions computed above are the ones the reference gets */
    double pos[6][3];
    for (int n = 0; n < 6; n++) {
        if (nb[n] < 0) continue;
        const orc_pt *src = &at_te[n];
        if (mt != te) {
            if ((rc = adv_point(c, s, nb[n], EID_OF(nb[n]), t1, mt, &tmp, steps))) return rc;
            src = &tmp;
        }
        memcpy(pos[n], src->X, 24);
    }
#undef EID_OF
    const double *L, *R, *B, *T, *Bk, *F;
    double fx, fy, fz;
    if (i == 0) { L = self.X; R = pos[1]; fx = 1.0; }
    else if (i == xr - 1) { L = pos[0]; R = self.X; fx = 1.0; }
    else { L = pos[0]; R = pos[1]; fx = 2.0; }
    if (j == 0) { B = self.X; T = pos[3]; fy = 1.0; }
    else if (j == yr - 1) { B = pos[2]; T = self.X; fy = 1.0; }
    else { B = pos[2]; T = pos[3]; fy = 2.0; }
    if (c->dims == 3) {
        if (k == 0) { Bk = self.X; F = pos[5]; fz = 1.0; }
        else if (k == zr - 1) { Bk = pos[4]; F = self.X; fz = 1.0; }
        else { Bk = pos[4]; F = pos[5]; fz = 2.0; }
    } else { Bk = F = self.X; fz = 1.0; }
    double lam = stencil_lambda(c->dims, L, R, B, T, Bk, F, fx, fy, fz, S->P.fdelta[0], S->P.fdelta[1], S->P.fdelta[2]);
    if (lam > 1.0 - ORC_TINY) {
        if (fabs(mt - s->start) < ORC_TINY) { s->ftT[q] = 0.0; s->ftN[q] = 0.0; }
        else {
            s->ftT[q] = (0.5 * log(lam)) / fabs(mt - s->start);
            s->ftN[q] = 0.5 * log(lam);
        }
    } else { s->ftT[q] = 0.0; s->ftN[q] = 0.0; }
    return 0;
}

/* GetFTLEForPoint, ompVC/ftle.c:1050-1203 */
static void final_ftle(const orc_run_state *S, ftle_slide *s, int q, double IntT)
{
    int xr = s->xr, yr = s->yr, zr = s->zr, YZ = yr * zr;
    int k = q % zr, j = (q / zr) % yr, i = q / YZ;
    if (IntT < ORC_TINY) { s->ftT[q] = 0.0; s->ftN[q] = 0.0; return; }
    const double *X = s->X;
    const double *L, *R, *B, *T, *Bk, *F;
    double fx, fy, fz;
    if (i == 0) { L = &X[3 * q]; R = &X[3 * (q + YZ)]; fx = 1.0; }
    else if (i == xr - 1) { L = &X[3 * (q - YZ)]; R = &X[3 * q]; fx = 1.0; }
    else { L = &X[3 * (q - YZ)]; R = &X[3 * (q + YZ)]; fx = 2.0; }
    if (j == 0) { B = &X[3 * q]; T = &X[3 * (q + zr)]; fy = 1.0; }
    else if (j == yr - 1) { B = &X[3 * (q - zr)]; T = &X[3 * q]; fy = 1.0; }
    else { B = &X[3 * (q - zr)]; T = &X[3 * (q + zr)]; fy = 2.0; }
    if (S->ctx.dims == 3) {
        if (k == 0) { Bk = &X[3 * q]; F = &X[3 * (q + 1)]; fz = 1.0; }
        else if (k == zr - 1) { Bk = &X[3 * (q - 1)]; F = &X[3 * q]; fz = 1.0; }
        else { Bk = &X[3 * (q - 1)]; F = &X[3 * (q + 1)]; fz = 2.0; }
    } else { Bk = F = &X[3 * q]; fz = 1.0; }
    double lam = stencil_lambda(S->ctx.dims, L, R, B, T, Bk, F, fx, fy, fz, S->P.fdelta[0], S->P.fdelta[1], S->P.fdelta[2]);
    if (lam > 1.0 - ORC_TINY) {
        s->ftT[q] = (0.5 * log(lam)) / IntT;
        s->ftN[q] = 0.5 * log(lam);
    } else { s->ftT[q] = 0.0; s->ftN[q] = 0.0; }
}

/* OutputFTLE, ompVC/ftle.c:1244-1329 */
static int output_ftle(orc_run_state *S, ftle_slide *s, int ss, double IntT, char *err, int errlen)
{
    const orc_params *P = &S->P;
    char path[2 * ORC_STR];
    if ((ss == 0 && !P->ftle_var) || (P->ftle_var && !s->nout)) {
        snprintf(path, sizeof(path), "%s%s.info", P->path_output, P->ftle_prefix);
        FILE *f = fopen(path, "w");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
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
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        fwrite(&P->fb[0], 8, 1, f); fwrite(&P->fb[1], 8, 1, f); fwrite(&P->fres[0], 4, 1, f);
        fwrite(&P->fb[2], 8, 1, f); fwrite(&P->fb[3], 8, 1, f); fwrite(&P->fres[1], 4, 1, f);
        fwrite(&P->fb[4], 8, 1, f); fwrite(&P->fb[5], 8, 1, f); fwrite(&P->fres[2], 4, 1, f);
        fclose(f);
    }
    int id = P->ftle_var ? s->nout : (P->int_dir > 0 ? ss : (P->out_tres - 1 - ss));
    for (int q = 0; q < s->n; q++)
        if (!s->have[q]) final_ftle(S, s, q, IntT);
    const char *dump = getenv("ORC_DUMP_STATE");
    if (dump && *dump) {
        snprintf(path, sizeof(path), "%s/state.%d.bin", dump, id);
        FILE *f = fopen(path, "wb");
        if (f) {
            fwrite(&s->n, 4, 1, f);
            fwrite(s->X, 8, 3 * (size_t)s->n, f);
            fwrite(s->eid, 4, (size_t)s->n, f);
            fwrite(s->left, 4, (size_t)s->n, f);
            fwrite(s->have, 4, (size_t)s->n, f);
            fclose(f);
        }
    }
    double *buf = (double *)malloc(sizeof(double) * (size_t)s->n * 2);
    if (!buf) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    long m = 0;
    for (int k = 0; k < s->zr; k++)
        for (int j = 0; j < s->yr; j++)
            for (int i = 0; i < s->xr; i++) {
                int q = (i * s->yr + j) * s->zr + k;
                buf[m] = s->ftT[q];
                buf[s->n + m] = s->ftN[q];
                m++;
            }
    for (int which = 0; which < 2; which++) {
        snprintf(path, sizeof(path), which ? "%s%s_noT.%d.bin" : "%s%s.%d.bin", P->path_output, P->ftle_prefix, id);
        FILE *f = fopen(path, "wb");
        if (!f) { free(buf); return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path); }
        fwrite(&s->start, 8, 1, f);
        fwrite(buf + (which ? s->n : 0), 8, (size_t)s->n, f);
        fclose(f);
    }
    free(buf);
    if (P->ftle_var) s->nout++;
    return ORC_OK;
}

/* One frame interval of one slide: ComputeFTLE's body for slide ss
 * (ompVC/ftle.c:72-192) as the two passes described at the top. */
static int ftle_interval(orc_run_state *S, ftle_slide *s, ftle_scratch *w, int ss, int df,
                         long long *steps, char *err, int errlen)
{
    orc_ctx *c = &S->ctx;
    const orc_params *P = &S->P;
    double t1, t2;
    int n = s->n, rc = 0;
    if (s->status == 0) {
        s->status = 1;
        t1 = s->start;
        /* launch velocity (ftle.c:84-96); on a Cartesian grid it flags
         * points outside the velocity grid */
        for (int p = 0; p < n; p++)
            if (!s->left[p]) {
                int l = 0, e = s->eid[p];
                double v[3];
                if ((rc = orc_vel(c, s->start, &s->X[3 * p], &e, &l, v)))
                    return set_err(err, errlen, ORC_ERR_WALK, "launch velocity failed (%d)", rc);
                memcpy(&s->V[3 * p], v, 24);
                s->eid[p] = e;
                if (l) s->left[p] = 1;
            }
    } else t1 = (P->int_dir > 0) ? c->tmin : c->tmax;
    t2 = (P->int_dir > 0) ? ORC_MIN(c->tmax, s->stop) : ORC_MAX(c->tmin, s->stop);

    long long st = 0;
    int fault = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : st) reduction(| : fault)
    for (int p = 0; p < n; p++) {
        w->integ[p] = 0;
        w->exited[p] = 0;
        if (!(s->ldt[p] > -ORC_TINY && (!s->left[p] || P->extrapolate))) continue;
        orc_pt t;
        memcpy(t.X, &s->X[3 * p], 24);
        memcpy(t.V, &s->V[3 * p], 24);
        t.left = s->left[p];
        t.ldt = s->ldt[p];
        t.eid = s->eid[p];
        fault |= orc_advect_pt(c, &t, t1, t2, &st);
        w->integ[p] = 1;
        w->exited[p] = t.left && !P->extrapolate;
        w->te[p] = t.ldt;
        memcpy(&w->Xn[3 * p], t.X, 24);
        memcpy(&w->Vn[3 * p], t.V, 24);
        w->en[p] = t.eid;
        w->ln[p] = t.left;
    }
    if (fault) return set_err(err, errlen, ORC_ERR_WALK, "advection fault in slide %d, frame %d", ss, df);

    if (!P->extrapolate) {
        int YZ = s->yr * s->zr, zr = s->zr;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : st) reduction(| : fault)
        for (int q = 0; q < n; q++) {
            if (s->have[q]) continue;
            int k = q % zr, j = (q / zr) % s->yr, i = q / YZ;
            int cand[7] = {i > 0 ? q - YZ : -1, j > 0 ? q - zr : -1, k > 0 ? q - 1 : -1, q,
                           k < zr - 1 ? q + 1 : -1, j < s->yr - 1 ? q + zr : -1, i < s->xr - 1 ? q + YZ : -1};
            int trig = -1;
            for (int m = 0; m < 7; m++)
                if (cand[m] >= 0 && w->exited[cand[m]]) { trig = cand[m]; break; }
            if (trig < 0) continue;
            fault |= early_ftle(S, s, w, q, trig, t1, w->te[trig], &st);
            s->have[q] = 2; /* served this interval; finalised below */
        }
        if (fault) return set_err(err, errlen, ORC_ERR_STATE, "early FTLE advected a point that had left (slide %d)", ss);
    }
    for (int p = 0; p < n; p++) {
        if (s->have[p] == 2) s->have[p] = 1;
        if (!w->integ[p]) continue;
        if (w->exited[p]) { s->left[p] = 1; continue; }
        memcpy(&s->X[3 * p], &w->Xn[3 * p], 24);
        memcpy(&s->V[3 * p], &w->Vn[3 * p], 24);
        if (P->extrapolate) s->left[p] = w->ln[p];
        if (c->mesh_type == 1) s->eid[p] = w->en[p];
    }
    *steps += st;
    if (((P->int_dir > 0) ? (s->stop - c->tmax) : (c->tmin - s->stop)) < ORC_TINY) {
        if ((rc = output_ftle(S, s, ss, P->ftle_T, err, errlen))) return rc;
        s->status = 2;
    } else if (P->ftle_var && !fmod(df - P->first_frame, P->ftle_varfreq)) {
        if ((rc = output_ftle(S, s, ss, fabs(t2 - s->start), err, errlen))) return rc;
    }
    return ORC_OK;
}

static int run_ftle(orc_run_state *S, double *secs, long long *steps, char *err, int errlen)
{
    orc_params *P = &S->P;
    int nsl = P->out_tres, rc = 0;
    int xr = P->fres[0], yr = P->fres[1], zr = P->fres[2], n = xr * yr * zr;
    ftle_slide *sl = (ftle_slide *)calloc((size_t)nsl, sizeof(ftle_slide));
    ftle_scratch w;
    w.Xn = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    w.Vn = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    w.te = (double *)malloc(sizeof(double) * (size_t)n);
    w.en = (int *)malloc(sizeof(int) * (size_t)n);
    w.ln = (int *)malloc(sizeof(int) * (size_t)n);
    w.integ = (int *)malloc(sizeof(int) * (size_t)n);
    w.exited = (int *)malloc(sizeof(int) * (size_t)n);
    if (!sl || !w.Xn || !w.Vn || !w.te || !w.en || !w.ln || !w.integ || !w.exited)
        return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    for (int ss = 0; ss < nsl; ss++) {
        ftle_slide *s = &sl[ss];
        s->n = n; s->xr = xr; s->yr = yr; s->zr = zr;
        s->X = (double *)malloc(sizeof(double) * 3 * (size_t)n);
        s->V = (double *)malloc(sizeof(double) * 3 * (size_t)n);
        s->ldt = (double *)malloc(sizeof(double) * (size_t)n);
        s->ftT = (double *)malloc(sizeof(double) * (size_t)n);
        s->ftN = (double *)malloc(sizeof(double) * (size_t)n);
        s->eid = (int *)malloc(sizeof(int) * (size_t)n);
        s->left = (int *)malloc(sizeof(int) * (size_t)n);
        s->have = (int *)malloc(sizeof(int) * (size_t)n);
        if (!s->X || !s->V || !s->ldt || !s->ftT || !s->ftN || !s->eid || !s->left || !s->have)
            return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    }
    /* the first frame window is needed for seeding-independent data only */
    if (P->ftle_genmesh) {
        long long ngs = 0;
        if ((rc = ftle_seed(S, &sl[0], &ngs))) return set_err(err, errlen, rc, "seed location failed");
        if ((rc = write_ic(S, &sl[0], err, errlen))) return rc;
    } else if ((rc = read_ic(S, &sl[0], err, errlen))) return rc;
    for (int ss = 0; ss < nsl; ss++) {
        ftle_slide *s = &sl[ss];
        if (ss > 0) {
            memcpy(s->X, sl[0].X, sizeof(double) * 3 * (size_t)n);
            memcpy(s->V, sl[0].V, sizeof(double) * 3 * (size_t)n);
            memcpy(s->ldt, sl[0].ldt, sizeof(double) * (size_t)n);
            memcpy(s->ftT, sl[0].ftT, sizeof(double) * (size_t)n);
            memcpy(s->ftN, sl[0].ftN, sizeof(double) * (size_t)n);
            memcpy(s->eid, sl[0].eid, sizeof(int) * (size_t)n);
            memcpy(s->left, sl[0].left, sizeof(int) * (size_t)n);
            memcpy(s->have, sl[0].have, sizeof(int) * (size_t)n);
        }
        s->status = 0;
        s->start = P->out_tstart + ss * P->int_dir * P->out_tdelta;
        if (!P->periodic) {
            s->stop = ORC_MIN(P->out_tstart + ss * P->int_dir * P->out_tdelta + (double)P->int_dir * P->ftle_T, P->data_tmax);
            s->stop = ORC_MAX(s->stop, P->tmin);
        } else s->stop = P->out_tstart + ss * P->int_dir * P->out_tdelta + (double)P->int_dir * P->ftle_T;
    }
    double tsum = 0;
    for (int df = P->first_frame; df != P->last_frame; df = df + P->int_dir) {
        if ((rc = window(S, df, err, errlen))) return rc;
        double t0 = now_s();
        for (int ss = 0; ss < nsl; ss++) {
            ftle_slide *s = &sl[ss];
            if (s->status != 2 && (s->status == 1 || (s->start <= S->ctx.tmax + ORC_TINY && s->start >= S->ctx.tmin - ORC_TINY)))
                if ((rc = ftle_interval(S, s, &w, ss, df, steps, err, errlen))) return rc;
        }
        tsum += now_s() - t0;
    }
    *secs = tsum;
    for (int ss = 0; ss < nsl; ss++) {
        ftle_slide *s = &sl[ss];
        free(s->X); free(s->V); free(s->ldt); free(s->ftT); free(s->ftN); free(s->eid); free(s->left); free(s->have);
    }
    free(sl);
    free(w.Xn); free(w.Vn); free(w.te); free(w.en); free(w.ln); free(w.integ); free(w.exited);
    return ORC_OK;
}

/* ==================================================================== tracers */

typedef struct {
    double start, stop;
    int status;
} launch_t;

/* ReadInTraceMesh (ompVC/tracers.c:998-1296) for ASCII (1) and binary (4)
 * lists and GenerateTracerMesh (ompVC/tracers.c:1298-1577), each with the
 * reference's seed-location chain. */
static int tracer_seed(orc_run_state *S, int *nout, orc_pt **out, char *err, int errlen)
{
    const orc_params *P = &S->P;
    const orc_ctx *c = &S->ctx;
    orc_pt *pts = NULL;
    int n = 0, e = 0;
    char path[2 * ORC_STR];
    if (P->tr_genmesh) {
        n = P->tres3[0] * P->tres3[1] * P->tres3[2];
        pts = (orc_pt *)calloc((size_t)n, sizeof(orc_pt));
        if (!pts) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
        int seed = -1, guess = -1, cnt = 0;
        if (c->mesh_type == 1) {
            double Xs[3] = {P->tb[0] + ((int)(P->tres3[0] / 2)) * P->tdelta3[0],
                            P->tb[2] + ((int)(P->tres3[1] / 2)) * P->tdelta3[1],
                            P->tb[4] + ((int)(P->tres3[2] / 2)) * P->tdelta3[2]};
            seed = orc_global(c, Xs);
            if (seed >= 0) guess = seed;
        }
        for (int kk = 0; kk < P->tres3[2]; kk++)
            for (int jj = 0; jj < P->tres3[1]; jj++)
                for (int ii = 0; ii < P->tres3[0]; ii++) {
                    orc_pt *t = &pts[cnt++];
                    t->X[0] = P->tb[0] + ii * P->tdelta3[0];
                    t->X[1] = P->tb[2] + jj * P->tdelta3[1];
                    t->X[2] = P->tb[4] + kk * P->tdelta3[2];
                    t->eid = -1;
                    t->ldt = 0.0;
                    t->left = orc_outside_domain(c, t->X);
                    if (t->left || c->mesh_type != 1) continue;
                    if (seed < 0) {
                        seed = orc_global(c, t->X);
                        if (seed < 0) { t->left = 1; t->ldt = -1.0; t->eid = -1; }
                        else { t->eid = seed; guess = seed; }
                        continue;
                    }
                    int index = orc_local(c, t->X, guess, &e);
                    if (index < 0) index = orc_local(c, t->X, seed, &e);
                    if (index < 0 && P->lsc) index = orc_global(c, t->X);
                    if (index < 0) { t->left = 1; t->ldt = -1.0; t->eid = -1; }
                    else { t->eid = index; t->left = 0; t->ldt = 0.0; guess = index; }
                }
    } else {
        snprintf(path, sizeof(path), "%s%s", P->path_data, P->tr_infile);
        if (P->tr_format == 4) {
            FILE *f = fopen(path, "rb");
            if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
            if (fread(&n, 4, 1, f) != 1 || n < 0) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "Could not read Trace_NumTracers from %s", path); }
            pts = (orc_pt *)calloc((size_t)(n ? n : 1), sizeof(orc_pt));
            if (!pts) { fclose(f); return set_err(err, errlen, ORC_ERR_OOM, "out of memory"); }
            for (int i = 0; i < n; i++) {
                if ((int)fread(pts[i].X, 8, (size_t)P->dims, f) < P->dims) { fclose(f); free(pts); return set_err(err, errlen, ORC_ERR_IO, "Could not read TraceIC_Array[%d].X from %s", i, path); }
                if (P->dims == 2) pts[i].X[2] = 0;
            }
            fclose(f);
        } else {
            FILE *f = fopen(path, "r");
            if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
            if (fscanf(f, "%d\n", &n) != 1 || n < 0) { fclose(f); return set_err(err, errlen, ORC_ERR_IO, "bad tracer count in %s", path); }
            pts = (orc_pt *)calloc((size_t)(n ? n : 1), sizeof(orc_pt));
            if (!pts) { fclose(f); return set_err(err, errlen, ORC_ERR_OOM, "out of memory"); }
            for (int i = 0; i < n; i++) {
                int r = P->dims == 3 ? fscanf(f, "%lf %lf %lf\n", &pts[i].X[0], &pts[i].X[1], &pts[i].X[2])
                                     : fscanf(f, "%lf %lf\n", &pts[i].X[0], &pts[i].X[1]);
                if (r != P->dims) { fclose(f); free(pts); return set_err(err, errlen, ORC_ERR_IO, "bad tracer line %d in %s", i, path); }
                if (P->dims == 2) pts[i].X[2] = 0;
            }
            fclose(f);
        }
        int found = 0, guess = -1;
        for (int i = 0; i < n; i++) {
            orc_pt *t = &pts[i];
            t->eid = -1;
            t->left = orc_outside_domain(c, t->X);
            if (c->mesh_type == 1 && !t->left) {
                if (!found) {
                    int index = orc_global(c, t->X);
                    if (index < 0) { t->left = 1; t->eid = -1; }
                    else { t->eid = index; guess = index; found++; }
                } else {
                    int index = orc_local(c, t->X, guess, &e);
                    if (index < 0 && P->lsc) index = orc_global(c, t->X);
                    if (index < 0) { t->left = 1; t->eid = -1; }
                    else { t->eid = index; t->left = 0; guess = index; found++; }
                }
            }
            t->ldt = t->left ? -1.0 : 0.0;
        }
    }
    if (e) { free(pts); return set_err(err, errlen, ORC_ERR_WALK, "walk fault while locating tracers"); }
    *nout = n;
    *out = pts;
    return ORC_OK;
}

/* OutputRT, ompVC/residencetime.c:21-185, for generated grids and seed
 * lists: the seed grid's parameters (<RT>_Cartesian.bin) or the located
 * seeds' positions (<RT>_coordinates.bin: count, then X per seed), and per
 * release <RT>.<ss>.bin: the release time, then per tracer -1 if it never was
 * in the domain, else (LeftDomainTime if it left, the release's stop time if
 * not) minus the release time. */
static int output_rt(orc_run_state *S, int n, const orc_pt *ic, orc_pt **rel, const launch_t *L, char *err,
                     int errlen)
{
    const orc_params *P = &S->P;
    char path[2 * ORC_STR];
    FILE *f;
    if (P->tr_genmesh) {
        snprintf(path, sizeof(path), "%s%s_Cartesian.bin", P->path_output, P->tr_rtprefix);
        if (!(f = fopen(path, "wb"))) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        for (int a = 0; a < 3; a++) {
            fwrite(&P->tb[2 * a], 8, 1, f);
            fwrite(&P->tb[2 * a + 1], 8, 1, f);
            fwrite(&P->tres3[a], 4, 1, f);
        }
        fclose(f);
    } else {
        snprintf(path, sizeof(path), "%s%s_coordinates.bin", P->path_output, P->tr_rtprefix);
        if (!(f = fopen(path, "wb"))) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        fwrite(&n, 4, 1, f);
        for (int i = 0; i < n; i++) fwrite(ic[i].X, 8, 3, f);
        fclose(f);
    }
    for (int ss = 0; ss < P->tr_nlaunch; ss++) {
        snprintf(path, sizeof(path), "%s%s.%d.bin", P->path_output, P->tr_rtprefix, ss);
        if (!(f = fopen(path, "wb"))) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        double time = P->out_tstart + ss * P->tr_spacing;
        fwrite(&time, 8, 1, f);
        for (int i = 0; i < n; i++) {
            const orc_pt *t = &rel[ss][i];
            double rt = fabs(t->ldt + 1) < ORC_TINY ? -1.0 : (t->left ? t->ldt : L[ss].stop) - time;
            fwrite(&rt, 8, 1, f);
        }
        fclose(f);
    }
    return ORC_OK;
}

/* OutputCET, ompVC/exposuretime.c:175-302: per element CET = sum / xc /
 * Trace_NumTracers and MET = sum / xc / encounters where the sum exceeds
 * TINY, else 0, with xc = pow(vol, (1/3)) in 3D -- the integer quotient 1/3
 * is 0, so xc = 1 -- and sqrt(triangle area) in 2D; the files
 * <RT>_CET.0.bin, <RT>_MET.0.bin (time stamp -1, then doubles) and
 * <RT>_ENC.0.bin (time stamp -1, then ints). */
static int output_cet(orc_run_state *S, int ntracers, char *err, int errlen)
{
    const orc_params *P = &S->P;
    const orc_ctx *c = &S->ctx;
    long E = c->nelem;
    double *cet = (double *)calloc((size_t)E, 8), *met = (double *)calloc((size_t)E, 8);
    if (!cet || !met) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    for (long e = 0; e < E; e++) {
        if (c->cet_sum[e] > ORC_TINY) {
            double xc = 1.0;
            if (c->dims == 2) {
                const double *X1 = c->xyz + 3L * c->conn[4 * e], *X2 = c->xyz + 3L * c->conn[4 * e + 1],
                             *X3 = c->xyz + 3L * c->conn[4 * e + 2];
                double A0 = X2[0] - X1[0], A1 = X2[1] - X1[1], B0 = X3[0] - X1[0], B1 = X3[1] - X1[1];
                xc = sqrt(fabs(A0 * B1 - A1 * B0) / 2);
            }
            cet[e] = c->cet_sum[e] / xc / ntracers;
            met[e] = c->cet_sum[e] / xc / c->cet_enc[e];
        }
    }
    const char *suffix[3] = {"CET", "MET", "ENC"};
    double t = -1.0;
    for (int k = 0; k < 3; k++) {
        char path[2 * ORC_STR];
        snprintf(path, sizeof(path), "%s%s_%s.0.bin", P->path_output, P->tr_rtprefix, suffix[k]);
        FILE *f = fopen(path, "wb");
        if (!f) { free(cet); free(met); return set_err(err, errlen, ORC_ERR_IO, "Could not open %s", path); }
        fwrite(&t, 8, 1, f);
        if (k == 0) fwrite(cet, 8, (size_t)E, f);
        else if (k == 1) fwrite(met, 8, (size_t)E, f);
        else fwrite(c->cet_enc, 4, (size_t)E, f);
        fclose(f);
    }
    free(cet);
    free(met);
    return ORC_OK;
}

static int run_tracers(orc_run_state *S, double *secs, long long *steps, char *err, int errlen)
{
    orc_params *P = &S->P;
    orc_ctx *c = &S->ctx;
    int n = 0, rc, nl = P->tr_nlaunch;
    orc_pt *ic = NULL;
    if ((rc = tracer_seed(S, &n, &ic, err, errlen))) return rc;
    launch_t *L = (launch_t *)calloc((size_t)nl, sizeof(launch_t));
    orc_pt **rel = (orc_pt **)calloc((size_t)nl, sizeof(orc_pt *));
    long *cnt = (long *)calloc((size_t)P->out_tres, sizeof(long));
    double **outbuf = (double **)calloc((size_t)P->out_tres, sizeof(double *));
    if (!L || !rel || !cnt || !outbuf) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
    for (int ss = 0; ss < nl; ss++) {
        L[ss].start = P->out_tstart + P->int_dir * ss * P->tr_spacing;
        L[ss].stop = (P->int_dir > 0) ? ORC_MIN(L[ss].start + P->tr_T, P->out_tend) : ORC_MAX(L[ss].start - P->tr_T, P->out_tend);
        L[ss].status = 0;
        rel[ss] = (orc_pt *)malloc(sizeof(orc_pt) * (size_t)(n ? n : 1));
        if (!rel[ss]) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
        memcpy(rel[ss], ic, sizeof(orc_pt) * (size_t)n);
    }
    if (P->tr_cet) {
        c->cet_sum = (double *)calloc((size_t)c->nelem, sizeof(double));
        c->cet_enc = (int *)calloc((size_t)c->nelem, sizeof(int));
        if (!c->cet_sum || !c->cet_enc) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
        c->cet_sub = P->tr_cetsub;
    }
    int outputframe = 0;
    double next = P->out_tstart, tsum = 0;
    for (int df = P->first_frame; df != P->last_frame; df = df + P->int_dir) {
        if ((rc = window(S, df, err, errlen))) return rc;
        double t0 = now_s();
        /* Compute_Tracer, ompVC/tracers.c:25-289 (TRACER_LOWERLOOP) */
        double t1 = (P->int_dir > 0) ? c->tmin : c->tmax, t2;
        while (((P->int_dir > 0) ? (t1 - c->tmax) : (c->tmin - t1)) < 0) {
            t2 = (P->int_dir > 0) ? ORC_MIN(next, c->tmax) : ORC_MAX(c->tmin, next);
            for (int ss = 0; ss < nl; ss++) {
                if (L[ss].status != 2 && (L[ss].status == 1 || (L[ss].start <= ORC_MAX(t1, t2) && L[ss].start >= ORC_MIN(t1, t2)))) {
                    orc_pt *T = rel[ss];
                    if (L[ss].status == 0) {
                        L[ss].status = 1;
                        /* the release's first encounters, ompVC/tracers.c:180-185 */
                        if (c->cet_sub)
                            for (int i = 0; i < n; i++)
                                if (!T[i].left) c->cet_enc[T[i].eid]++;
                        t1 = L[ss].start;
                        for (int i = 0; i < n; i++)
                            if (!T[i].left) {
                                double v[3];
                                int r2 = orc_vel(c, L[ss].start, T[i].X, &T[i].eid, &T[i].left, v);
                                if (r2) return set_err(err, errlen, ORC_ERR_WALK, "launch velocity failed");
                                memcpy(T[i].V, v, 24);
                            }
                    }
                    long long st = 0;
                    int fault = 0;
                    /* exposure-time sums are added in tracer order, as ompVC's
                     * loop on one thread adds them */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : st) reduction(| : fault) if (!c->cet_sub)
                    for (int i = 0; i < n; i++)
                        if (T[i].ldt > -ORC_TINY && (!T[i].left || P->extrapolate))
                            fault |= orc_advect_pt(c, &T[i], t1, t2, &st);
                    if (fault) return set_err(err, errlen, ORC_ERR_WALK, "advection fault (release %d)", ss);
                    *steps += st;
                    if (fabs(next - t2) < ORC_TINY && outputframe < P->out_tres) {
                        long add = 0;
                        for (int i = 0; i < n; i++)
                            if (T[i].ldt > -ORC_TINY && (!T[i].left || P->tr_always)) add++;
                        double *b = (double *)realloc(outbuf[outputframe], sizeof(double) * 3 * (size_t)(cnt[outputframe] + add + 1));
                        if (!b) return set_err(err, errlen, ORC_ERR_OOM, "out of memory");
                        outbuf[outputframe] = b;
                        for (int i = 0; i < n; i++)
                            if (T[i].ldt > -ORC_TINY && (!T[i].left || P->tr_always)) {
                                memcpy(&b[3 * cnt[outputframe]], T[i].X, 24);
                                cnt[outputframe]++;
                            }
                    }
                }
                if (((P->int_dir > 0) ? (L[ss].stop - t2) : (t2 - L[ss].stop)) < ORC_TINY) L[ss].status = 2;
            }
            if (fabs(t2 - next) < ORC_TINY) {
                next += P->int_dir * P->out_tdelta;
                outputframe++;
                if (outputframe >= P->out_tres) break;
            }
            t1 = t2;
        }
        tsum += now_s() - t0;
    }
    *secs = tsum;
    /* OutputTracers, ompVC/tracers.c:1763-1816 */
    char path[2 * ORC_STR];
    for (int i = 0; i < P->out_tres; i++) {
        if (cnt[i] <= 0) continue;
        snprintf(path, sizeof(path), "%s%s.%d.bin", P->path_output, P->tr_prefix, i);
        FILE *f = fopen(path, "wb");
        if (!f) return set_err(err, errlen, ORC_ERR_IO, "Could not open file %s", path);
        double time = P->out_tstart + i * P->int_dir * P->out_tdelta;
        fwrite(&time, 8, 1, f);
        fwrite(outbuf[i], 8, 3 * (size_t)cnt[i], f);
        fclose(f);
    }
    if (P->tr_rt && (rc = output_rt(S, n, ic, rel, L, err, errlen))) return rc;
    if (P->tr_cet && (rc = output_cet(S, n, err, errlen))) return rc;
    for (int i = 0; i < P->out_tres; i++) free(outbuf[i]);
    for (int ss = 0; ss < nl; ss++) free(rel[ss]);
    free(outbuf); free(cnt); free(rel); free(L); free(ic);
    free(c->cet_sum); free(c->cet_enc);
    c->cet_sum = NULL; c->cet_enc = NULL; c->cet_sub = 0;
    return ORC_OK;
}

/* ====================================================================== run */

int orc_run(const char *in_path, int nthreads, double *advect_seconds, long long *steps, char *errbuf, int errlen)
{
    orc_run_state S;
    memset(&S, 0, sizeof(S));
    int rc;
    if ((rc = orc_read_params(in_path, &S.P, errbuf, errlen))) return rc;
    if ((rc = orc_check_derive(&S.P, errbuf, errlen))) return rc;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    else if (S.P.nthreads > 0) omp_set_num_threads(S.P.nthreads);
    if ((rc = load_mesh(&S, errbuf, errlen))) { free_state(&S); return rc; }
    double secs = 0;
    long long st = 0;
    if (S.P.ftle_compute) rc = run_ftle(&S, &secs, &st, errbuf, errlen);
    else rc = run_tracers(&S, &secs, &st, errbuf, errlen);
    if (advect_seconds) *advect_seconds = secs;
    if (steps) *steps = st;
    free_state(&S);
    return rc;
}
