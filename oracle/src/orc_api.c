/*
 * orc_api.c -- array-level entry points of the CPU oracle (test
 * infrastructure): the same per-point operations as the engine's C-ABI,
 * restated on the CPU so tests can compare them call for call.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc_int.h"

orc_ctx *orc_create(int dims, int mesh_type)
{
    if ((dims != 2 && dims != 3) || (mesh_type != 0 && mesh_type != 1)) return NULL;
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    if (!c) return NULL;
    c->dims = dims;
    c->mesh_type = mesh_type;
    c->int_type = 1;
    c->h = 0.01;
    c->bounds[0] = c->bounds[2] = c->bounds[4] = -1e300;
    c->bounds[1] = c->bounds[3] = c->bounds[5] = 1e300;
    return c;
}

void orc_destroy(orc_ctx *c)
{
    if (!c) return;
    free(c->xyz);
    free(c->conn);
    free(c->adj);
    free(c);
}

/* Vel_CartMesh set-up, ompVC/mesh.c:101-121 */
int orc_set_cart(orc_ctx *c, double xmin, double xmax, int xres, double ymin, double ymax, int yres,
                 double zmin, double zmax, int zres)
{
    if (!c || c->mesh_type != 0 || xres < 2 || yres < 2 || xmin >= xmax || ymin >= ymax) return ORC_ERR_ARG;
    orc_grid *g = &c->g;
    g->xmin = xmin; g->xmax = xmax; g->xres = xres; g->dx = (xmax - xmin) / (xres - 1);
    g->ymin = ymin; g->ymax = ymax; g->yres = yres; g->dy = (ymax - ymin) / (yres - 1);
    if (c->dims == 3) {
        if (zres < 2 || zmin >= zmax) return ORC_ERR_ARG;
        g->zmin = zmin; g->zmax = zmax; g->zres = zres; g->dz = (zmax - zmin) / (zres - 1);
    } else {
        g->zmin = 0; g->zmax = 0; g->zres = 1; g->dz = 0;
    }
    return ORC_OK;
}

int orc_set_unstruct(orc_ctx *c, int nnodes, const double *xyz, int nelem, const int *conn, const int *adj)
{
    if (!c || c->mesh_type != 1 || nnodes <= 0 || nelem <= 0) return ORC_ERR_ARG;
    free(c->xyz); free(c->conn); free(c->adj);
    c->xyz = (double *)malloc(sizeof(double) * 3 * (size_t)nnodes);
    c->conn = (int *)malloc(sizeof(int) * 4 * (size_t)nelem);
    c->adj = (int *)malloc(sizeof(int) * 4 * (size_t)nelem);
    if (!c->xyz || !c->conn || !c->adj) return ORC_ERR_OOM;
    memcpy(c->xyz, xyz, sizeof(double) * 3 * (size_t)nnodes);
    memcpy(c->conn, conn, sizeof(int) * 4 * (size_t)nelem);
    memcpy(c->adj, adj, sizeof(int) * 4 * (size_t)nelem);
    c->nnodes = nnodes;
    c->nelem = nelem;
    return ORC_OK;
}

int orc_set_bounds(orc_ctx *c, const double b[6])
{
    if (!c) return ORC_ERR_ARG;
    memcpy(c->bounds, b, sizeof(c->bounds));
    return ORC_OK;
}

int orc_set_frames(orc_ctx *c, const double *uvw0, const double *uvw1, double tmin, double tmax)
{
    if (!c || !uvw0 || !uvw1) return ORC_ERR_ARG;
    c->f0 = uvw0;
    c->f1 = uvw1;
    c->tmin = tmin;
    c->tmax = tmax;
    return ORC_OK;
}

int orc_set_integrator(orc_ctx *c, int int_type, double h, int extrapolate)
{
    if (!c || (int_type < 0 || int_type > 3) || !(h > 0)) return ORC_ERR_ARG;
    c->int_type = int_type;
    c->h = h;
    c->extrapolate = extrapolate;
    return ORC_OK;
}

int orc_set_rkf(orc_ctx *c, double accuracy, double min_step, double max_step)
{
    if (!c || !(accuracy > 0) || !(min_step > 0) || !(max_step > 0)) return ORC_ERR_ARG;
    c->acc = accuracy;
    c->hmin = min_step;
    c->hmax = max_step;
    return ORC_OK;
}

int orc_advect(orc_ctx *c, int n, double *X, double *V, int *eid, int *left, double *ldt, double t0,
               double t1, long long *steps)
{
    if (!c || !c->f0) return ORC_ERR_STATE;
    long long st = 0;
    int fault = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : st) reduction(| : fault)
    for (int i = 0; i < n; i++) {
        orc_pt p;
        memcpy(p.X, &X[3 * i], 24);
        if (V) memcpy(p.V, &V[3 * i], 24);
        else p.V[0] = p.V[1] = p.V[2] = 0.0;
        p.eid = eid ? eid[i] : -1;
        p.left = left[i];
        p.ldt = ldt[i];
        if (p.left && !c->extrapolate) continue;
        fault |= orc_advect_pt(c, &p, t0, t1, &st);
        memcpy(&X[3 * i], p.X, 24);
        if (V) memcpy(&V[3 * i], p.V, 24);
        if (eid) eid[i] = p.eid;
        left[i] = p.left;
        ldt[i] = p.ldt;
    }
    if (steps) *steps = st;
    return fault ? ORC_ERR_WALK : ORC_OK;
}

int orc_velocity(orc_ctx *c, int n, const double *X, int *eid, int *left, double tq, double *out)
{
    if (!c || !c->f0) return ORC_ERR_STATE;
    int fault = 0;
    for (int i = 0; i < n; i++) {
        double x[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
        int e = eid ? eid[i] : -1;
        fault |= orc_vel(c, tq, x, &e, &left[i], &out[3 * i]);
        if (eid) eid[i] = e;
    }
    return fault ? ORC_ERR_WALK : ORC_OK;
}

int orc_local_search(orc_ctx *c, int n, const double *X, const int *guess, int *out)
{
    if (!c || c->mesh_type != 1) return ORC_ERR_STATE;
    int err = 0;
    for (int i = 0; i < n; i++) out[i] = orc_local(c, &X[3 * i], guess[i], &err);
    return err ? ORC_ERR_WALK : ORC_OK;
}

int orc_global_search(orc_ctx *c, int n, const double *X, int *out)
{
    if (!c || c->mesh_type != 1) return ORC_ERR_STATE;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) out[i] = orc_global(c, &X[3 * i]);
    return ORC_OK;
}
