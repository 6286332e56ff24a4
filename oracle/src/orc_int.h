/* orc_int.h -- internal state of the CPU oracle (test infrastructure). */
#ifndef ORC_INT_H
#define ORC_INT_H

#include "orc.h"

#define ORC_MAX_HOPS (1 << 22)

/* min/max with the reference's macro semantics (ompVC/macros.h:33-34). */
#define ORC_MIN(a, b) ((a) < (b) ? (a) : (b))
#define ORC_MAX(a, b) ((a) > (b) ? (a) : (b))
#define ORC_SIGN(a, b) ((b) >= 0.0 ? fabs(a) : -fabs(a))

typedef struct {
    double xmin, xmax, dx;
    double ymin, ymax, dy;
    double zmin, zmax, dz;
    int xres, yres, zres;
} orc_grid;

struct orc_ctx {
    int dims, mesh_type;
    orc_grid g;                 /* Cartesian velocity grid (Vel_CartMesh) */
    int nnodes, nelem;
    double *xyz;                /* nnodes x 3 */
    int *conn, *adj;            /* nelem x 4 */
    double bounds[6];           /* Data_MeshBounds */
    const double *f0, *f1;      /* velocity slots 0 and 1, file order */
    double tmin, tmax;          /* Data_LoadedTMin / TMax */
    int int_type;               /* 0 Euler, 1 RK4, 2 RKF, 3 Adams-Bashforth 2 */
    double h;
    int extrapolate;
    double acc, hmin, hmax;     /* Int_Accuracy, Int_MinTimeStep, Int_MaxTimeStep (RKF) */
    /* exposure time (Trace_CETArray, ompVC/exposuretime.c): per-element sums
     * and encounters; cet_sub = Trace_CETSubsteps, 0 when off */
    double *cet_sum;
    int *cet_enc;
    int cet_sub;
};

/* One Lagrangian point as the integrators see it (the fields of
 * LagrangianPoint, ompVC/structs.h:21-29, that the hot path touches). */
typedef struct {
    double X[3];
    double V[3];
    int eid;
    int left;
    double ldt;
} orc_pt;

/* status bits a point can raise */
#define ORC_PT_ERR_WALK 1
#define ORC_PT_ERR_TLOC 2
#define ORC_PT_ERR_CET 4

int orc_outside_domain(const orc_ctx *c, const double X[3]);
int orc_vel(const orc_ctx *c, double tq, double X[3], int *eid, int *left, double out[3]);
int orc_local(const orc_ctx *c, const double X[3], int guess, int *err);
int orc_global(const orc_ctx *c, const double X[3]);
/* Advect; returns 0 or an ORC_PT_ERR_* bit set; *steps += accepted steps */
int orc_advect_pt(const orc_ctx *c, orc_pt *p, double t0, double t1, long long *steps);

#endif
