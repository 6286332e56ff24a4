/*
 * orc.h -- CPU oracle for the flowVC advection / FTLE hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C with OpenMP,
 * the algorithm of ompVC (flowVC's OpenMP program) for tracer and FTLE-grid
 * advection.  It is the checker the GPU engine is compared against and the
 * CPU baseline it is timed beside; nothing in the engine links or calls it.
 *
 * All arithmetic is IEEE double in the operation order of the reference
 * (compile with -ffp-contract=off so no multiply-add is fused), which makes
 * positions, element ids and exit flags bit-identical to ompVC.
 */
#ifndef ORC_H
#define ORC_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_TINY 1.0e-10

enum { ORC_OK = 0, ORC_ERR_IO = 1, ORC_ERR_ARG = 2, ORC_ERR_OOM = 3, ORC_ERR_WALK = 4,
       ORC_ERR_TLOC = 5, ORC_ERR_STATE = 6 };

typedef struct orc_ctx orc_ctx;

/* Context holding one mesh, a two-frame velocity window and integrator
 * settings (the state ompVC keeps in globals, ompVC/globals.h:17-168). */
orc_ctx *orc_create(int dims, int mesh_type /*0 Cartesian, 1 unstructured*/);
void orc_destroy(orc_ctx *c);
int orc_set_cart(orc_ctx *c, double xmin, double xmax, int xres, double ymin, double ymax,
                 int yres, double zmin, double zmax, int zres);
int orc_set_unstruct(orc_ctx *c, int nnodes, const double *xyz, int nelem, const int *conn,
                     const int *adj);
int orc_set_bounds(orc_ctx *c, const double b[6]);
/* uvw0 is the frame at tmin (slot 0), uvw1 the frame at tmax (slot 1); both
 * in file order (interleaved u,v,w per node, Cartesian k,j,i i fastest). */
int orc_set_frames(orc_ctx *c, const double *uvw0, const double *uvw1, double tmin, double tmax);
int orc_set_integrator(orc_ctx *c, int int_type, double h, int extrapolate);
/* Int_Accuracy, Int_MinTimeStep, Int_MaxTimeStep of RKF (Int_Type 2) */
int orc_set_rkf(orc_ctx *c, double accuracy, double min_step, double max_step);

/* Advect n points from t0 to t1 in place (ompVC Advect, integration.c:22-45).
 * X is n x 3, V n x 3 (extrapolation velocity), eid/left per point, ldt the
 * LeftDomainTime.  Points with left set are skipped unless extrapolating.
 * steps (may be NULL) receives the accepted step count. */
int orc_advect(orc_ctx *c, int n, double *X, double *V, int *eid, int *left, double *ldt,
               double t0, double t1, long long *steps);

/* Velocity at (tq, X) as GetVelocity (velocity.c:236-247); eid walks. */
int orc_velocity(orc_ctx *c, int n, const double *X, int *eid, int *left, double tq, double *out);

/* Neighbour walk (mesh.c:496-611) and brute-force first-id search
 * (mesh.c:304-398). */
int orc_local_search(orc_ctx *c, int n, const double *X, const int *guess, int *out);
int orc_global_search(orc_ctx *c, int n, const double *X, int *out);

/* Largest eigenvalue of a symmetric 3x3 (row-major) by cyclic Jacobi. */
double orc_max_eig(const double a[9]);

/* Full ompVC-equivalent run of an .in file: FTLE or tracers, writing the
 * same output files.  nthreads <= 0 uses OpenMP's default.  Timing of the
 * advection phase (seconds) and the accepted step count are returned. */
int orc_run(const char *in_path, int nthreads, double *advect_seconds, long long *steps,
            char *errbuf, int errlen);

#ifdef __cplusplus
}
#endif
#endif
