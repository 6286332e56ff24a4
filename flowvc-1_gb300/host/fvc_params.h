/* fvc_params.h -- flowVC run parameters as read from an ompVC .in file.
 *
 * Field order follows the positional order of ompVC/parameters.c:30-138;
 * derived fields follow SetDerivedParameters (ompVC/parameters.c:294-430). */
#ifndef FVC_PARAMS_H
#define FVC_PARAMS_H

#define FVCP_STR 512

typedef struct {
    char path_data[FVCP_STR], path_output[FVCP_STR];
    int dims, mesh_type;
    char prefix[FVCP_STR];
    int suffix_tmin, suffix_tdelta, tres;
    double tdelta, tmin;
    int periodic;
    double bounds[6];
    double fluid_density, fluid_viscosity;
    double out_tstart;
    int out_tres;
    double out_tdelta;
    int int_type;
    double int_h, int_acc, int_hmin, int_hmax;
    int int_dir, normal_flow;
    double normal_scale;
    int extrapolate;
    double p_radius, p_density;
    int p_ictype;
    double gravity[3];
    int lsc, nthreads;
    int ftle_compute, ftle_genmesh;
    char ftle_ic[FVCP_STR];
    double fb[6];
    int fres[3];
    double ftle_T;
    int ftle_var, ftle_varfreq;
    char ftle_prefix[FVCP_STR];
    int tr_compute, tr_strategy;
    double tr_release_tmax;
    int tr_genmesh;
    char tr_infile[FVCP_STR];
    int tr_multi, tr_format;
    char tr_prefix[FVCP_STR];
    int tr_nlaunch;
    double tr_spacing, tr_T;
    int tr_always;
    double tb[6];
    int tres3[3];
    int tr_ap, tr_cet, tr_cetaux;
    char tr_cetprefix[FVCP_STR];
    int tr_cetsub, tr_rt;
    char tr_rtprefix[FVCP_STR];
    int vo_compute, vo_genmesh;
    char vo_infile[FVCP_STR];
    int vo_format;
    char vo_prefix[FVCP_STR];
    double vb[6];
    int vres[3];
    /* derived */
    double data_tmax, out_tend;
    double fdelta[3], tdelta3[3];
    int first_frame, last_frame;
} fvcp_params;

/* 0 on success; on failure err holds ompVC's message for the same case. */
int fvcp_read(const char *path, fvcp_params *p, char *err, int errlen);
int fvcp_check_derive(fvcp_params *p, char *err, int errlen);

#endif
