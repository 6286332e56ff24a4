/*
 * orc_core.c -- CPU oracle: interpolation, point location and integrators.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h).  Each routine restates the ompVC
 * routine cited beside it, keeping the reference's expression order so that
 * IEEE double results are bit-identical (build with -ffp-contract=off).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc_int.h"

/* ------------------------------------------------------------------ domain */

/* TestOutsideDomain, ompVC/velocity.c:654-669 */
int orc_outside_domain(const orc_ctx *c, const double X[3])
{
    const double *b = c->bounds;
    if (X[0] < (b[0] - ORC_TINY) || X[0] > (b[1] + ORC_TINY)) return 1;
    if (X[1] < (b[2] - ORC_TINY) || X[1] > (b[3] + ORC_TINY)) return 1;
    if (X[2] < (b[4] - ORC_TINY) || X[2] > (b[5] + ORC_TINY)) return 1;
    return 0;
}

/* TestOutsideCartVelDomain, ompVC/velocity.c:624-651 */
static int outside_cart_grid(const orc_ctx *c, const double X[3])
{
    const orc_grid *g = &c->g;
    int imin = (int)floor((X[0] - g->xmin) / g->dx);
    int jmin = (int)floor((X[1] - g->ymin) / g->dy);
    int kmin = c->dims == 3 ? (int)floor((X[2] - g->zmin) / g->dz) : 0;
    int imax = (int)ceil((X[0] - g->xmin) / g->dx);
    int jmax = (int)ceil((X[1] - g->ymin) / g->dy);
    int kmax = c->dims == 3 ? (int)ceil((X[2] - g->zmin) / g->dz) : 0;
    return imin < 0 || imax > (g->xres - 1) || jmin < 0 || jmax > (g->yres - 1) || kmin < 0 ||
           kmax > (g->zres - 1);
}

/* ------------------------------------------------------- Cartesian velocity */

/* GetVelocity_Cartesian, ompVC/velocity.c:257-457: space-time quadrilinear
 * interpolation with the reference's 16 weights and summation order. */
static int vel_cart(const orc_ctx *c, double tq, const double X[3], int *left, double out[3])
{
    const orc_grid *g = &c->g;
    if (outside_cart_grid(c, X)) {
        out[0] = out[1] = out[2] = 0.0;
        *left = 1;
        return 0;
    }
    double tloc = (tq - c->tmin) / (c->tmax - c->tmin);
    if ((tloc > 1 + ORC_TINY) || (tloc < 0 - ORC_TINY)) return ORC_PT_ERR_TLOC;
    double xloc, yloc, zloc;
    int i = (int)floor((X[0] - g->xmin) / g->dx);
    if (i == (g->xres - 1)) { i = g->xres - 2; xloc = 1.0; }
    else xloc = (X[0] - g->xmin - i * g->dx) / g->dx;
    int j = (int)floor((X[1] - g->ymin) / g->dy);
    if (j == (g->yres - 1)) { j = g->yres - 2; yloc = 1.0; }
    else yloc = (X[1] - g->ymin - j * g->dy) / g->dy;
    int k, k1;
    if (c->dims == 3) {
        k = (int)floor((X[2] - g->zmin) / g->dz);
        if (k == (g->zres - 1)) { k = g->zres - 2; zloc = 1.0; }
        else zloc = (X[2] - g->zmin - k * g->dz) / g->dz;
        k1 = k + 1;
    } else {
        k = 0; k1 = 0; zloc = 0.0;
    }
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
    /* node offsets in file order (k, j, i with i fastest), 3 values a node */
    long nx = g->xres, ny = g->yres;
#define CIDX(ii, jj, kk) ((((long)(kk) * ny + (jj)) * nx + (ii)) * 3)
    long o000 = CIDX(i, j, k), o001 = CIDX(i, j, k1), o010 = CIDX(i, j + 1, k),
         o011 = CIDX(i, j + 1, k1), o100 = CIDX(i + 1, j, k), o101 = CIDX(i + 1, j, k1),
         o110 = CIDX(i + 1, j + 1, k), o111 = CIDX(i + 1, j + 1, k1);
#undef CIDX
    for (int q = 0; q < 3; q++) {
        const double *A = c->f0 + q, *B = c->f1 + q;
        out[q] = A[o000] * V16 + A[o001] * V15 + A[o010] * V14 + A[o011] * V13 + A[o100] * V12 +
                 A[o101] * V11 + A[o110] * V10 + A[o111] * V9 + B[o000] * V8 + B[o001] * V7 +
                 B[o010] * V6 + B[o011] * V5 + B[o100] * V4 + B[o101] * V3 + B[o110] * V2 +
                 B[o111] * V1;
    }
    return 0;
}

/* ----------------------------------------------------- barycentric geometry */

/* Natural coordinates of X in element e (ompVC/velocity.c:481-543, the same
 * expressions in ompVC/mesh.c:511-591).  Returns d = min of the coordinates;
 * r, s, t and the fourth coordinate w are returned for the tie-break. */
static inline double natural(const orc_ctx *c, int e, const double X[3], double *r_, double *s_,
                             double *t_, double *w_)
{
    const int *nd = c->conn + 4 * (long)e;
    const double *p0 = c->xyz + 3 * (long)nd[0], *p1 = c->xyz + 3 * (long)nd[1],
                 *p2 = c->xyz + 3 * (long)nd[2];
    double x = X[0], y = X[1], z = X[2];
    double r, s, t, d, w;
    if (c->dims == 3) {
        const double *p3 = c->xyz + 3 * (long)nd[3];
        double x0 = p0[0], y0 = p0[1], z0 = p0[2], x1 = p1[0], y1 = p1[1], z1 = p1[2];
        double x2 = p2[0], y2 = p2[1], z2 = p2[2], x3 = p3[0], y3 = p3[1], z3 = p3[2];
        double a11 = (z3 - z0) * (y2 - y3) - (z2 - z3) * (y3 - y0);
        double a21 = (z3 - z0) * (y0 - y1) - (z0 - z1) * (y3 - y0);
        double a31 = (z1 - z2) * (y0 - y1) - (z0 - z1) * (y1 - y2);
        double a12 = (x3 - x0) * (z2 - z3) - (x2 - x3) * (z3 - z0);
        double a22 = (x3 - x0) * (z0 - z1) - (x0 - x1) * (z3 - z0);
        double a32 = (x1 - x2) * (z0 - z1) - (x0 - x1) * (z1 - z2);
        double a13 = (y3 - y0) * (x2 - x3) - (y2 - y3) * (x3 - x0);
        double a23 = (y3 - y0) * (x0 - x1) - (y0 - y1) * (x3 - x0);
        double a33 = (y1 - y2) * (x0 - x1) - (y0 - y1) * (x1 - x2);
        double V = (x1 - x0) * ((y2 - y0) * (z3 - z0) - (z2 - z0) * (y3 - y0)) +
                   (x2 - x0) * ((y0 - y1) * (z3 - z0) - (z0 - z1) * (y3 - y0)) +
                   (x3 - x0) * ((y1 - y0) * (z2 - z0) - (z1 - z0) * (y2 - y0));
        r = (a11 * (x - x0) + a12 * (y - y0) + a13 * (z - z0)) / V;
        s = (a21 * (x - x0) + a22 * (y - y0) + a23 * (z - z0)) / V;
        t = (a31 * (x - x0) + a32 * (y - y0) + a33 * (z - z0)) / V;
        w = 1 - r - s - t;
        d = ORC_MIN(r, ORC_MIN(s, ORC_MIN(t, w)));
    } else {
        double x0 = p0[0], y0 = p0[1], x1 = p1[0], y1 = p1[1], x2 = p2[0], y2 = p2[1];
        double a11 = y2 - y0, a12 = x0 - x2, a21 = y0 - y1, a22 = x1 - x0;
        double V = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
        r = (a11 * (x - x0) + a12 * (y - y0)) / V;
        s = (a21 * (x - x0) + a22 * (y - y0)) / V;
        t = 0;
        w = 1 - r - s;
        d = ORC_MIN(r, ORC_MIN(s, w));
    }
    *r_ = r; *s_ = s; *t_ = t; *w_ = w;
    return d;
}

/* Neighbour slot for the walk step: the first coordinate within TINY of the
 * minimum in the order r, s, t, w (ompVC/velocity.c:588-609). */
static inline int walk_slot(int dims, double r, double s, double t, double w, double d)
{
    if (fabs(r - d) < ORC_TINY) return 0;
    if (fabs(s - d) < ORC_TINY) return 1;
    if (dims == 3) {
        if (fabs(t - d) < ORC_TINY) return 2;
        if (fabs(w - d) < ORC_TINY) return 3;
    } else {
        if (fabs(d - w) < ORC_TINY) return 2;
    }
    return -1; /* "Indeterminate neighbor" */
}

/* GetVelocity_Unstructured, ompVC/velocity.c:459-621: walk from *eid until
 * the element passes (d + TINY) >= 0, then P1-in-space, linear-in-time. */
static int vel_unstruct(const orc_ctx *c, double tq, const double X[3], int *eid, int *left,
                        double out[3])
{
    if (*eid < 0) return ORC_PT_ERR_WALK;
    double tloc = (tq - c->tmin) / (c->tmax - c->tmin);
    if ((tloc > 1 + ORC_TINY) || (tloc < 0 - ORC_TINY)) return ORC_PT_ERR_TLOC;
    for (long hop = 0; hop < ORC_MAX_HOPS; hop++) {
        double r, s, t, w;
        double d = natural(c, *eid, X, &r, &s, &t, &w);
        if ((d + ORC_TINY) >= 0) {
            const int *nd = c->conn + 4 * (long)(*eid);
            const double *A = c->f0, *B = c->f1;
            double U1t = (1 - tloc) * A[3 * (long)nd[0]] + tloc * B[3 * (long)nd[0]];
            double V1t = (1 - tloc) * A[3 * (long)nd[0] + 1] + tloc * B[3 * (long)nd[0] + 1];
            double U2t = (1 - tloc) * A[3 * (long)nd[1]] + tloc * B[3 * (long)nd[1]];
            double V2t = (1 - tloc) * A[3 * (long)nd[1] + 1] + tloc * B[3 * (long)nd[1] + 1];
            double U3t = (1 - tloc) * A[3 * (long)nd[2]] + tloc * B[3 * (long)nd[2]];
            double V3t = (1 - tloc) * A[3 * (long)nd[2] + 1] + tloc * B[3 * (long)nd[2] + 1];
            if (c->dims == 3) {
                double W1t = (1 - tloc) * A[3 * (long)nd[0] + 2] + tloc * B[3 * (long)nd[0] + 2];
                double W2t = (1 - tloc) * A[3 * (long)nd[1] + 2] + tloc * B[3 * (long)nd[1] + 2];
                double W3t = (1 - tloc) * A[3 * (long)nd[2] + 2] + tloc * B[3 * (long)nd[2] + 2];
                double U4t = (1 - tloc) * A[3 * (long)nd[3]] + tloc * B[3 * (long)nd[3]];
                double V4t = (1 - tloc) * A[3 * (long)nd[3] + 1] + tloc * B[3 * (long)nd[3] + 1];
                double W4t = (1 - tloc) * A[3 * (long)nd[3] + 2] + tloc * B[3 * (long)nd[3] + 2];
                out[0] = U1t + (U2t - U1t) * fabs(r) + (U3t - U1t) * fabs(s) + (U4t - U1t) * fabs(t);
                out[1] = V1t + (V2t - V1t) * fabs(r) + (V3t - V1t) * fabs(s) + (V4t - V1t) * fabs(t);
                out[2] = W1t + (W2t - W1t) * fabs(r) + (W3t - W1t) * fabs(s) + (W4t - W1t) * fabs(t);
            } else {
                out[0] = U1t + (U2t - U1t) * fabs(r) + (U3t - U1t) * fabs(s);
                out[1] = V1t + (V2t - V1t) * fabs(r) + (V3t - V1t) * fabs(s);
                out[2] = 0.0;
            }
            return 0;
        }
        int slot = walk_slot(c->dims, r, s, t, w, d);
        if (slot < 0) return ORC_PT_ERR_WALK;
        *eid = c->adj[4 * (long)(*eid) + slot];
        if (*eid == -1) {
            *left = 1;
            out[0] = out[1] = out[2] = 0.0;
            return 0;
        }
    }
    return ORC_PT_ERR_WALK;
}

int orc_vel(const orc_ctx *c, double tq, double X[3], int *eid, int *left, double out[3])
{
    if (c->mesh_type == 0) return vel_cart(c, tq, X, left, out);
    return vel_unstruct(c, tq, X, eid, left, out);
}

/* ------------------------------------------------------------ point location */

/* Get_Element_Local_Search, ompVC/mesh.c:496-611.  Returns the element, -1
 * when the walk leaves through a boundary face; *err set on a walk fault. */
int orc_local(const orc_ctx *c, const double X[3], int guess, int *err)
{
    if (guess < 0) return -1;
    for (long hop = 0; hop < ORC_MAX_HOPS; hop++) {
        double r, s, t, w;
        double d = natural(c, guess, X, &r, &s, &t, &w);
        if (d > -ORC_TINY) return guess;
        int slot;
        if (fabs(r - d) < ORC_TINY) slot = 0;
        else if (fabs(s - d) < ORC_TINY) slot = 1;
        else if (c->dims == 3 && fabs(t - d) < ORC_TINY) slot = 2;
        else if (fabs(d - w) < ORC_TINY) slot = c->dims == 3 ? 3 : 2;
        else { if (err) *err |= ORC_PT_ERR_WALK; return -1; }
        guess = c->adj[4 * (long)guess + slot];
        if (guess == -1) return -1;
    }
    if (err) *err |= ORC_PT_ERR_WALK;
    return -1;
}

/* Get_Element_Global_Search, ompVC/mesh.c:304-398: first element by id with
 * d > -TINY, else -1. */
int orc_global(const orc_ctx *c, const double X[3])
{
    for (int e = 0; e < c->nelem; e++) {
        double r, s, t, w;
        if (natural(c, e, X, &r, &s, &t, &w) > -ORC_TINY) return e;
    }
    return -1;
}

/* ComputeExposureTime, ompVC/exposuretime.c:110-172: the step from X0 to X1
 * (X1 in element e1) of length h.  Same element at both ends: all of h to
 * it.  Otherwise the straight path is sampled at substeps points; each
 * sample after the first credits h / (substeps - 1) to the element holding
 * it (walk from the previous sample's element, global search when the walk
 * leaves; samples outside the mesh are skipped) and a change of element
 * counts an encounter. */
static void cet_step(const orc_ctx *c, const double X0[3], const double X1[3], int e1, double h, int *err)
{
    int e0 = orc_local(c, X0, e1, err);
    if (e0 < 0) {
        e0 = orc_global(c, X0);
        if (e0 < 0) { *err |= ORC_PT_ERR_CET; return; }
    }
    if (e0 == e1) {
        c->cet_sum[e0] = c->cet_sum[e0] + h;
        return;
    }
    int last = e0;
    for (int s = 1; s < c->cet_sub; s++) {
        double a = ((double)s) / ((double)(c->cet_sub - 1)), Xt[3];
        for (int q = 0; q < 3; q++) Xt[q] = (1 - a) * X0[q] + a * X1[q];
        int et = orc_local(c, Xt, last, err);
        if (et < 0) {
            et = orc_global(c, Xt);
            if (et < 0) continue;
        }
        c->cet_sum[et] = c->cet_sum[et] + (h / (c->cet_sub - 1));
        if (et != last) {
            c->cet_enc[et]++;
            last = et;
        }
    }
}

/* -------------------------------------------------------------- integrators */

/* Euler, ompVC/integration.c:222-311 */
static double euler(const orc_ctx *c, orc_pt *p, double tstart, double tend, long long *steps, int *err)
{
    double tc = tstart, h = ORC_SIGN(c->h, tend - tstart), ve[3];
    int unst = c->mesh_type == 1;
    while ((tc - tend) * (tend - tstart) < 0.0) {
        if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = ORC_SIGN(tend - tc, tend - tstart);
        if ((*err |= orc_vel(c, tc, p->X, &p->eid, &p->left, ve))) return tend;
        p->X[0] = p->X[0] + h * ve[0];
        p->X[1] = p->X[1] + h * ve[1];
        p->X[2] = p->X[2] + h * ve[2];
        tc = tc + h;
        if (unst) p->eid = orc_local(c, p->X, p->eid, err);
        if (*err) return tend;
        if ((!unst && orc_outside_domain(c, p->X)) || (unst && p->eid < 0)) {
            p->left = 1;
            p->ldt = tc - h;
            p->X[0] = p->X[0] - h * ve[0];
            p->X[1] = p->X[1] - h * ve[1];
            p->X[2] = p->X[2] - h * ve[2];
            return p->ldt;
        }
        (*steps)++;
        if (c->extrapolate && (*err |= orc_vel(c, tc, p->X, &p->eid, &p->left, p->V))) return tend;
        if (c->cet_sub) {   /* ompVC/integration.c:277-299 */
            double X0[3] = {p->X[0] - h * ve[0], p->X[1] - h * ve[1], p->X[2] - h * ve[2]};
            cet_step(c, X0, p->X, p->eid, h, err);
            if (*err) return tend;
        }
    }
    return tend;
}

/* One classic RK4 step from (tc, p->X) with stage hints e[4] / left flags
 * l[4] (ompVC/integration.c:362-401).  k receives k1..k4. */
static int rk4_stages(const orc_ctx *c, const orc_pt *p, double tc, double h, int e[4], int l[4],
                      double k[4][3])
{
    double M[3];
    int err = 0;
    M[0] = p->X[0]; M[1] = p->X[1]; M[2] = p->X[2];
    if ((err = orc_vel(c, tc, M, &e[0], &l[0], k[0]))) return err;
    M[0] = p->X[0] + 0.5 * k[0][0] * h;
    M[1] = p->X[1] + 0.5 * k[0][1] * h;
    M[2] = p->X[2] + 0.5 * k[0][2] * h;
    if ((err = orc_vel(c, tc + h / 2, M, &e[1], &l[1], k[1]))) return err;
    M[0] = p->X[0] + 0.5 * k[1][0] * h;
    M[1] = p->X[1] + 0.5 * k[1][1] * h;
    M[2] = p->X[2] + 0.5 * k[1][2] * h;
    if ((err = orc_vel(c, tc + h / 2, M, &e[2], &l[2], k[2]))) return err;
    M[0] = p->X[0] + k[2][0] * h;
    M[1] = p->X[1] + k[2][1] * h;
    M[2] = p->X[2] + k[2][2] * h;
    return orc_vel(c, tc + h, M, &e[3], &l[3], k[3]);
}

/* RK4, ompVC/integration.c:317-462, with the stage points' element hints
 * persisting across the steps of one call (integration.c:323-342). */
static double rk4(const orc_ctx *c, orc_pt *p, double tstart, double tend, long long *steps, int *err)
{
    int e[4] = {p->eid, p->eid, p->eid, p->eid}, l[4] = {p->left, p->left, p->left, p->left};
    double k[4][3], tc = tstart, h = ORC_SIGN(c->h, tend - tstart);
    int unst = c->mesh_type == 1;
    while ((tc - tend) * (tend - tstart) < 0.0) {
        if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = ORC_SIGN(tend - tc, tend - tstart);
        if ((*err |= rk4_stages(c, p, tc, h, e, l, k))) return tend;
        for (int q = 0; q < 3; q++)
            p->X[q] = p->X[q] + h * (k[0][q] + 2 * k[1][q] + 2 * k[2][q] + k[3][q]) / 6;
        tc = tc + h;
        if (unst) p->eid = orc_local(c, p->X, p->eid, err);
        if (*err) return tend;
        if ((!unst && orc_outside_domain(c, p->X)) || (unst && p->eid < 0) || l[0] || l[1] ||
            l[2] || l[3]) {
            p->left = 1;
            p->ldt = tc - h;
            for (int q = 0; q < 3; q++)
                p->X[q] = p->X[q] - h * (k[0][q] + 2 * k[1][q] + 2 * k[2][q] + k[3][q]) / 6;
            return p->ldt;
        }
        (*steps)++;
        if (c->extrapolate && (*err |= orc_vel(c, tc, p->X, &p->eid, &p->left, p->V))) return tend;
        if (c->cet_sub) {   /* ompVC/integration.c:427-447 */
            double X0[3];
            for (int q = 0; q < 3; q++)
                X0[q] = p->X[q] - h * (k[0][q] + 2 * k[1][q] + 2 * k[2][q] + k[3][q]) / 6;
            cet_step(c, X0, p->X, p->eid, h, err);
            if (*err) return tend;
        }
    }
    return tend;
}

/* Two-step Adams-Bashforth (Int_Type 3; cudaVC's numbering, cudaVC/src/main.cu:225).
 * ompVC has no multistep integrator; this is the textbook variable-step AB2,
 * X_{n+1} = X_n + h (c1 f_n - c0 f_{n-1}), c0 = h / (2 h_prev), c1 = 1 + c0,
 * bootstrapped by one RK4 step at the start of every call, with RK4's clip,
 * relocation and exit rules. */
static double ab2(const orc_ctx *c, orc_pt *p, double tstart, double tend, long long *steps, int *err)
{
    int e[4] = {p->eid, p->eid, p->eid, p->eid}, l[4] = {p->left, p->left, p->left, p->left};
    double k[4][3], fprev[3] = {0, 0, 0}, hprev = 0.0, tc = tstart, h = ORC_SIGN(c->h, tend - tstart);
    int unst = c->mesh_type == 1, first = 1;
    while ((tc - tend) * (tend - tstart) < 0.0) {
        if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = ORC_SIGN(tend - tc, tend - tstart);
        double inc[3], f[3];
        int lf = 0;
        if (first) {
            if ((*err |= rk4_stages(c, p, tc, h, e, l, k))) return tend;
            for (int q = 0; q < 3; q++) {
                inc[q] = h * (k[0][q] + 2 * k[1][q] + 2 * k[2][q] + k[3][q]) / 6;
                f[q] = k[0][q];
            }
            lf = l[0] || l[1] || l[2] || l[3];
        } else {
            int ef = p->eid;
            if ((*err |= orc_vel(c, tc, p->X, &ef, &lf, f))) return tend;
            double c0 = h / (2.0 * hprev), c1 = 1.0 + c0;
            for (int q = 0; q < 3; q++) inc[q] = h * (c1 * f[q] - c0 * fprev[q]);
        }
        for (int q = 0; q < 3; q++) p->X[q] = p->X[q] + inc[q];
        tc = tc + h;
        if (unst) p->eid = orc_local(c, p->X, p->eid, err);
        if (*err) return tend;
        if ((!unst && orc_outside_domain(c, p->X)) || (unst && p->eid < 0) || lf) {
            p->left = 1;
            p->ldt = tc - h;
            for (int q = 0; q < 3; q++) p->X[q] = p->X[q] - inc[q];
            return p->ldt;
        }
        (*steps)++;
        for (int q = 0; q < 3; q++) fprev[q] = f[q];
        hprev = h;
        first = 0;
        if (c->extrapolate && (*err |= orc_vel(c, tc, p->X, &p->eid, &p->left, p->V))) return tend;
    }
    return tend;
}

/* Advect, ompVC/integration.c:22-45 */
/* RKF, ompVC/integration.c:464-699: Runge-Kutta-Fehlberg 4(5) with the
 * reference's coefficients, error estimate and step-size control; the
 * stage points keep their element hints and exit flags across steps (MP1 ..
 * MP6).  A stage outside the domain stops the point at tc without moving
 * it. */
static double rkf(const orc_ctx *c, orc_pt *p, double tstart, double tend, long long *steps, int *err)
{
    double k[6][3], M[3];
    int e[6], l[6];
    for (int j = 0; j < 6; j++) {
        e[j] = p->eid;
        l[j] = p->left;
    }
    const double a3 = 3.0 / 32.0, b3 = 9.0 / 32.0;
    const double a4 = 1932.0 / 2197.0, b4 = -7200.0 / 2197.0, c4 = 7296.0 / 2197.0;
    const double a5 = 439.0 / 216.0, b5 = -8.0, c5 = 3680.0 / 513.0, d5 = -845.0 / 4104.0;
    const double a6 = -8.0 / 27.0, b6 = 2.0, c6 = -3544.0 / 2565.0, d6 = 1859.0 / 4104.0, e6 = -11.0 / 40.0;
    const double a7 = 1.0 / 360.0, b7 = -128.0 / 4275.0, c7 = -2197.0 / 75240.0, d7 = 1.0 / 50.0, e7 = 2.0 / 55.0;
    const double a8 = 25.0 / 216.0, b8 = 1408.0 / 2565.0, c8 = 2197.0 / 4104.0, d8 = -1.0 / 5.0;
    double h = ORC_SIGN(c->hmax, tend - tstart), hmax = c->hmax, tol = c->acc, tc = tstart, ts, ss;
    int unst = c->mesh_type == 1;
    while ((tc - tend) * (tend - tstart) < 0.0) {
        if ((tc + h - tend) * (tc + h - tstart) > 0.0) h = ORC_SIGN(tend - tc, tend - tstart);
        for (int q = 0; q < 3; q++) M[q] = p->X[q];
        if ((*err |= orc_vel(c, tc, M, &e[0], &l[0], k[0]))) return tend;
        for (int q = 0; q < 3; q++) M[q] = p->X[q] + 0.25 * k[0][q] * h;
        ts = tc + 0.25 * h;
        if ((*err |= orc_vel(c, ts, M, &e[1], &l[1], k[1]))) return tend;
        for (int q = 0; q < 3; q++) M[q] = p->X[q] + (a3 * k[0][q] + b3 * k[1][q]) * h;
        ts = tc + 0.375 * h;
        if ((*err |= orc_vel(c, ts, M, &e[2], &l[2], k[2]))) return tend;
        for (int q = 0; q < 3; q++) M[q] = p->X[q] + (a4 * k[0][q] + b4 * k[1][q] + c4 * k[2][q]) * h;
        ts = tc + (12.0 * h) / 13.0;
        if ((*err |= orc_vel(c, ts, M, &e[3], &l[3], k[3]))) return tend;
        for (int q = 0; q < 3; q++)
            M[q] = p->X[q] + (a5 * k[0][q] + b5 * k[1][q] + c5 * k[2][q] + d5 * k[3][q]) * h;
        ts = tc + h;
        if ((*err |= orc_vel(c, ts, M, &e[4], &l[4], k[4]))) return tend;
        for (int q = 0; q < 3; q++)
            M[q] = p->X[q] + (a6 * k[0][q] + b6 * k[1][q] + c6 * k[2][q] + d6 * k[3][q] + e6 * k[4][q]) * h;
        ts = tc + 0.5 * h;
        if ((*err |= orc_vel(c, ts, M, &e[5], &l[5], k[5]))) return tend;
        if (l[0] || l[1] || l[2] || l[3] || l[4] || l[5]) {
            p->left = 1;
            p->ldt = tc;
            return p->ldt;
        }
        double ex[3];
        for (int q = 0; q < 3; q++)
            ex[q] = fabs(a7 * k[0][q] + b7 * k[2][q] + c7 * k[3][q] + d7 * k[4][q] + e7 * k[5][q]);
        double er = fmax(fmax(ex[0], ex[1]), ex[2]);
        if (er == 0.0) ss = 0.0;
        else ss = pow(fabs((tol * h) / (2 * er)), 0.25);
        if (er < tol || fabs(h) <= c->hmin) {
            for (int q = 0; q < 3; q++)
                p->X[q] = p->X[q] + (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
            tc = tc + h;
            if (unst) p->eid = orc_local(c, p->X, p->eid, err);
            if (*err) return tend;
            if ((!unst && orc_outside_domain(c, p->X)) || (unst && p->eid < 0)) {
                p->left = 1;
                p->ldt = tc - h;
                for (int q = 0; q < 3; q++)
                    p->X[q] = p->X[q] - (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
                return p->ldt;
            }
            (*steps)++;
            if (c->extrapolate && (*err |= orc_vel(c, tc, p->X, &p->eid, &p->left, p->V))) return tend;
            if (c->cet_sub) {   /* ompVC/integration.c:649-669 */
                double X0[3];
                for (int q = 0; q < 3; q++)
                    X0[q] = p->X[q] - (a8 * k[0][q] + b8 * k[2][q] + c8 * k[3][q] + d8 * k[4][q]) * h;
                cet_step(c, X0, p->X, p->eid, h, err);
                if (*err) return tend;
            }
            if (fabs(h) > c->hmin && ss > 1.0) {
                ss = (ss > 4.0) ? 4.0 : ss;
                h = ORC_SIGN((fabs(ss * h) > hmax) ? hmax : ss * h, tend - tstart);
            }
        } else {
            if (ss < 1.0) {
                ss = (ss < 0.1) ? 0.1 : ss;
                h = ORC_SIGN((fabs(ss * h) < c->hmin) ? c->hmin : ss * h, tend - tstart);
            } else
                h = ORC_SIGN((fabs(0.5 * h) < c->hmin) ? c->hmin : 0.5 * h, tend - tstart);
        }
    }
    return tend;
}

int orc_advect_pt(const orc_ctx *c, orc_pt *p, double tstart, double tend, long long *steps)
{
    int err = 0;
    if (p->left && c->extrapolate) {
        for (int q = 0; q < 3; q++) p->X[q] = p->X[q] + p->V[q] * (tend - tstart);
        return 0;
    }
    if (p->left) return ORC_PT_ERR_WALK; /* "integrate point that already left" */
    if (c->mesh_type == 1 && p->eid < 0) return ORC_PT_ERR_WALK;
    double stop;
    if (c->int_type == 1) stop = rk4(c, p, tstart, tend, steps, &err);
    else if (c->int_type == 2) stop = rkf(c, p, tstart, tend, steps, &err);
    else if (c->int_type == 3) stop = ab2(c, p, tstart, tend, steps, &err);
    else stop = euler(c, p, tstart, tend, steps, &err);
    if (!err && (fabs(stop - tend) > ORC_TINY) && c->extrapolate)
        for (int q = 0; q < 3; q++) p->X[q] = p->X[q] + p->V[q] * (tend - stop);
    return err;
}

/* ------------------------------------------------------------ eigenvalue */

/* Largest eigenvalue of a symmetric 3x3 by cyclic Jacobi rotations
 * (Jacobi 1846; Rutishauser's stable update, Golub & Van Loan 8.5).  The
 * reference uses a Householder + QL routine instead; both agree to a few
 * ulps of the largest eigenvalue. */
double orc_max_eig(const double ain[9])
{
    double a[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[i][j] = ain[3 * i + j];
    static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
    for (int sweep = 0; sweep < 32; sweep++) {
        int rotated = 0;
        for (int n = 0; n < 3; n++) {
            int p = P[n], q = Q[n], r = 3 - p - q;
            double apq = a[p][q];
            if (apq == 0.0) continue;
            if (fabs(apq) <= 1e-18 * (fabs(a[p][p]) + fabs(a[q][q]))) {
                a[p][q] = a[q][p] = 0.0;
                continue;
            }
            rotated = 1;
            double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
            double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
            if (theta < 0.0) t = -t;
            double cs = 1.0 / sqrt(t * t + 1.0);
            double sn = t * cs;
            double tau = sn / (1.0 + cs);
            a[p][p] = a[p][p] - t * apq;
            a[q][q] = a[q][q] + t * apq;
            a[p][q] = a[q][p] = 0.0;
            double arp = a[r][p], arq = a[r][q];
            a[r][p] = a[p][r] = arp - sn * (arq + tau * arp);
            a[r][q] = a[q][r] = arq + sn * (arp - tau * arq);
        }
        if (!rotated) break;
    }
    return ORC_MAX(a[0][0], ORC_MAX(a[1][1], a[2][2]));
}
