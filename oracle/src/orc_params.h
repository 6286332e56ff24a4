/* orc_params.h -- the oracle's copy of ompVC's run parameters (test
 * infrastructure).  Field order follows the positional .in order of
 * ompVC/parameters.c:30-138. */
#ifndef ORC_PARAMS_H
#define ORC_PARAMS_H

#define ORC_STR 512

typedef struct {
    char path_data[ORC_STR], path_output[ORC_STR];
    int dims, mesh_type;
    char prefix[ORC_STR];
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
    char ftle_ic[ORC_STR];
    double fb[6];
    int fres[3];
    double ftle_T;
    int ftle_var, ftle_varfreq;
    char ftle_prefix[ORC_STR];
    int tr_compute, tr_strategy;
    double tr_release_tmax;
    int tr_genmesh;
    char tr_infile[ORC_STR];
    int tr_multi, tr_format;
    char tr_prefix[ORC_STR];
    int tr_nlaunch;
    double tr_spacing, tr_T;
    int tr_always;
    double tb[6];
    int tres3[3];
    int tr_ap, tr_cet, tr_cetaux;
    char tr_cetprefix[ORC_STR];
    int tr_cetsub, tr_rt;
    char tr_rtprefix[ORC_STR];
    int vo_compute, vo_genmesh;
    char vo_infile[ORC_STR];
    int vo_format;
    char vo_prefix[ORC_STR];
    double vb[6];
    int vres[3];
    /* derived (ompVC/parameters.c:294-430) */
    double data_tmax, out_tend;
    double fdelta[3], tdelta3[3];
    int first_frame, last_frame;
} orc_params;

int orc_read_params(const char *path, orc_params *p, char *err, int errlen);
int orc_check_derive(orc_params *p, char *err, int errlen);

#endif
