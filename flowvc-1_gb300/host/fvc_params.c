/*
 * fvc_params.c -- reader for ompVC's .in parameter files.
 *
 * The format is positional (ReadInNextValue, ompVC/parameters.c:258-292):
 * blank lines and lines starting with '#' are skipped; every other line is
 * "KEY = VALUE", the key is ignored and the value is taken in ompVC's fixed
 * order, so existing .in files run unchanged.
 */
#include "fvc_params.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#define P_TINY 1.0e-10
#define P_MIN(a, b) ((a) < (b) ? (a) : (b))
#define P_MAX(a, b) ((a) > (b) ? (a) : (b))

static int perr(char *err, int errlen, const char *fmt, ...)
{
    if (err && errlen > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)errlen, fmt, ap);
        va_end(ap);
    }
    return 1;
}

static int next_value(FILE *f, void *dst, char type)
{
    char key[FVCP_STR];
    for (;;) {
        int c = fgetc(f);
        if (c == EOF) return -1;
        if (c == ' ' || c == '\n' || c == '\r') continue;
        if (c == '#') {
            while (c != '\n' && c != EOF) c = fgetc(f);
            if (c == EOF) return -1;
            continue;
        }
        ungetc(c, f);
        if (fscanf(f, "%511s %*s", key) != 1) return -1;
        int r;
        switch (type) {
        case 's': r = fscanf(f, "%511s\n", (char *)dst); break;
        case 'd': r = fscanf(f, "%d\n", (int *)dst); break;
        default: r = fscanf(f, "%lf\n", (double *)dst); break;
        }
        return r == 1 ? 0 : -1;
    }
}

int fvcp_read(const char *path, fvcp_params *p, char *err, int errlen)
{
    FILE *f = fopen(path, "r");
    if (!f) return perr(err, errlen, "Could not open input file %s", path);
    memset(p, 0, sizeof(*p));
    struct { void *dst; char type; } v[] = {
        {p->path_data, 's'}, {p->path_output, 's'}, {&p->dims, 'd'}, {&p->mesh_type, 'd'},
        {p->prefix, 's'}, {&p->suffix_tmin, 'd'}, {&p->suffix_tdelta, 'd'}, {&p->tres, 'd'},
        {&p->tdelta, 'f'}, {&p->tmin, 'f'}, {&p->periodic, 'd'},
        {&p->bounds[0], 'f'}, {&p->bounds[1], 'f'}, {&p->bounds[2], 'f'}, {&p->bounds[3], 'f'},
        {&p->bounds[4], 'f'}, {&p->bounds[5], 'f'},
        {&p->fluid_density, 'f'}, {&p->fluid_viscosity, 'f'},
        {&p->out_tstart, 'f'}, {&p->out_tres, 'd'}, {&p->out_tdelta, 'f'},
        {&p->int_type, 'd'}, {&p->int_h, 'f'}, {&p->int_acc, 'f'}, {&p->int_hmin, 'f'},
        {&p->int_hmax, 'f'}, {&p->int_dir, 'd'}, {&p->normal_flow, 'd'}, {&p->normal_scale, 'f'},
        {&p->extrapolate, 'd'},
        {&p->p_radius, 'f'}, {&p->p_density, 'f'}, {&p->p_ictype, 'd'},
        {&p->gravity[0], 'f'}, {&p->gravity[1], 'f'}, {&p->gravity[2], 'f'},
        {&p->lsc, 'd'}, {&p->nthreads, 'd'},
        {&p->ftle_compute, 'd'}, {&p->ftle_genmesh, 'd'}, {p->ftle_ic, 's'},
        {&p->fb[0], 'f'}, {&p->fb[1], 'f'}, {&p->fb[2], 'f'}, {&p->fb[3], 'f'}, {&p->fb[4], 'f'},
        {&p->fb[5], 'f'}, {&p->fres[0], 'd'}, {&p->fres[1], 'd'}, {&p->fres[2], 'd'},
        {&p->ftle_T, 'f'}, {&p->ftle_var, 'd'}, {&p->ftle_varfreq, 'd'}, {p->ftle_prefix, 's'},
        {&p->tr_compute, 'd'}, {&p->tr_strategy, 'd'}, {&p->tr_release_tmax, 'f'},
        {&p->tr_genmesh, 'd'}, {p->tr_infile, 's'}, {&p->tr_multi, 'd'}, {&p->tr_format, 'd'},
        {p->tr_prefix, 's'}, {&p->tr_nlaunch, 'd'}, {&p->tr_spacing, 'f'}, {&p->tr_T, 'f'},
        {&p->tr_always, 'd'},
        {&p->tb[0], 'f'}, {&p->tb[1], 'f'}, {&p->tb[2], 'f'}, {&p->tb[3], 'f'}, {&p->tb[4], 'f'},
        {&p->tb[5], 'f'}, {&p->tres3[0], 'd'}, {&p->tres3[1], 'd'}, {&p->tres3[2], 'd'},
        {&p->tr_ap, 'd'}, {&p->tr_cet, 'd'}, {&p->tr_cetaux, 'd'}, {p->tr_cetprefix, 's'},
        {&p->tr_cetsub, 'd'}, {&p->tr_rt, 'd'}, {p->tr_rtprefix, 's'},
        {&p->vo_compute, 'd'}, {&p->vo_genmesh, 'd'}, {p->vo_infile, 's'}, {&p->vo_format, 'd'},
        {p->vo_prefix, 's'},
        {&p->vb[0], 'f'}, {&p->vb[1], 'f'}, {&p->vb[2], 'f'}, {&p->vb[3], 'f'}, {&p->vb[4], 'f'},
        {&p->vb[5], 'f'}, {&p->vres[0], 'd'}, {&p->vres[1], 'd'}, {&p->vres[2], 'd'},
    };
    int n = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n; i++)
        if (next_value(f, v[i].dst, v[i].type)) {
            fclose(f);
            return perr(err, errlen, "%s: could not read parameter %d of %d", path, i + 1, n);
        }
    fclose(f);
    return 0;
}

static void fix_path(char *s)
{
    if (strcmp(s, "pwd")) {
        size_t n = strlen(s);
        if ((n == 0 || s[n - 1] != '/') && n + 1 < FVCP_STR) { s[n] = '/'; s[n + 1] = 0; }
    } else {
        strcpy(s, "./");
    }
}

/* CheckParameters (ompVC/parameters.c:432-567) and SetDerivedParameters
 * (ompVC/parameters.c:294-430).  Options outside the engine's scope
 * (inertial particles, staggered release, side analyses) are refused. */
int fvcp_check_derive(fvcp_params *p, char *err, int errlen)
{
    if (p->dims != 2 && p->dims != 3) return perr(err, errlen, "Dimensions must be equal to 2 or 3");
    if (p->mesh_type != 0 && p->mesh_type != 1) return perr(err, errlen, "Unsupported Data_MeshType");
    if (p->tres < 2) return perr(err, errlen, "Data_TRes must be 2 or greater.");
    if (p->tdelta <= 0) return perr(err, errlen, "Data_TDelta <= 0");
    if (p->periodic != 0 && p->periodic != 1) return perr(err, errlen, "Data_TPeriodic should be 0 or 1");
    if (p->bounds[0] >= p->bounds[1]) return perr(err, errlen, "Data_MeshBounds.XMin >= Data_MeshBounds.XMax");
    if (p->bounds[2] >= p->bounds[3]) return perr(err, errlen, "Data_MeshBounds.YMin >= Data_MeshBounds.YMax");
    if (p->bounds[4] > p->bounds[5]) return perr(err, errlen, "Data_MeshBounds.ZMin > Data_MeshBounds.ZMax");
    if (p->out_tres < 1) return perr(err, errlen, "Output_TRes < 1");
    if (p->out_tdelta < P_TINY && p->out_tres > 1) return perr(err, errlen, "Output_TDelta must be positive");
    if (p->int_type < 0 || p->int_type > 3) p->int_type = 0; /* as Advect's fallback */
    if (p->int_h < P_TINY && p->int_type != 2) return perr(err, errlen, "Int_TimeStep must be positive");
    if ((p->int_hmin < P_TINY || p->int_hmax < P_TINY || p->int_acc < P_TINY) && p->int_type == 2)
        return perr(err, errlen, "RKF integration parameters must be positive");
    if (p->int_dir != 1 && p->int_dir != -1) return perr(err, errlen, "Unsupported Int_TimeDirection value, must be -1 or 1");
    if (p->p_radius > P_TINY) return perr(err, errlen, "Particle_Radius > 0 (inertial particles) is not supported");
    if (p->normal_flow) return perr(err, errlen, "Int_NormalFlow is not supported");
    if (p->ftle_compute && p->tr_compute)
        return perr(err, errlen, "Both FTLE_Compute = 1 and Trace_Compute = 1 cannot be handled concurrently");
    if (p->ftle_compute) {
        if (p->fb[0] >= p->fb[1]) return perr(err, errlen, "FTLE_CartMesh.XMin >= FTLE_CartMesh.XMax");
        if (p->fb[2] >= p->fb[3]) return perr(err, errlen, "FTLE_CartMesh.YMin >= FTLE_CartMesh.YMax");
        if (p->fb[4] > p->fb[5]) return perr(err, errlen, "FTLE_CartMesh.ZMin > FTLE_CartMesh.ZMax");
        if (p->fres[0] < 2) return perr(err, errlen, "FTLE_CartMesh.XRes < 2");
        if (p->fres[1] < 2) return perr(err, errlen, "FTLE_CartMesh.YRes < 2");
        if (p->fres[2] < 2 && ((p->dims == 2 && p->fres[2]) < 1 || p->dims == 3))
            return perr(err, errlen, "FTLE_CartMesh.ZRes insufficient");
        if (p->ftle_T < P_TINY) return perr(err, errlen, "FTLE_IntTLength must be positive");
        if (p->ftle_var) {
            if (p->out_tres != 1) return perr(err, errlen, "Output_TRes has to be 1 if FTLE_ComputeVariation = 1");
            if (p->ftle_varfreq < 1) return perr(err, errlen, "FTLE_VariationOutFreq < 1");
        }
    }
    if (p->tr_compute) {
        if (p->tr_strategy == 1) return perr(err, errlen, "Trace_ReleaseStrategy = 1 (staggered release) is not supported");
        if (p->tr_ap) return perr(err, errlen, "Trace_APCompute (activation potential) is not supported");
        /* CheckParameters, ompVC/parameters.c:535-542 */
        if (p->tr_cet) {
            if (p->tr_rt) return perr(err, errlen, "Cannot compute exposure times and residence times concurrently");
            if (p->tr_cetsub < 2) return perr(err, errlen, "Trace_CETSubsteps must be greater than 1");
            if (p->mesh_type != 1) return perr(err, errlen, "exposure time needs an unstructured velocity mesh");
            if (p->tr_cetaux) return perr(err, errlen, "Trace_CETAuxillaryMesh is not supported");
            if (p->int_type == 3) return perr(err, errlen, "exposure time needs Int_Type 0, 1 or 2");
        }
        if ((p->tr_rt || p->tr_cet) && p->int_dir < 0)
            return perr(err, errlen, "Residence/Exposure time computations not supported for backward time integrations");
        if (p->tr_genmesh) {
            if (p->tb[0] > p->tb[1]) return perr(err, errlen, "Trace_CartMesh.XMin > Trace_CartMesh.XMax");
            if (p->tb[2] > p->tb[3]) return perr(err, errlen, "Trace_CartMesh.YMin > Trace_CartMesh.YMax");
            if (p->tb[4] > p->tb[5]) return perr(err, errlen, "Trace_CartMesh.ZMin > Trace_CartMesh.ZMax");
            if (p->tres3[0] < 1 || p->tres3[1] < 1 || p->tres3[2] < 1) return perr(err, errlen, "Trace_CartMesh resolution < 1");
        } else if (p->tr_format != 1 && p->tr_format != 4) {
            return perr(err, errlen, "Trace_InFileFormat %d is not supported (1 ASCII list, 4 binary list)", p->tr_format);
        }
        if (p->tr_multi) return perr(err, errlen, "Trace_MultipleInFiles is not supported");
        if (p->tr_nlaunch < 1) return perr(err, errlen, "Trace_NumLaunchTimes < 1");
        if (p->tr_spacing < P_TINY && p->tr_nlaunch > 1) return perr(err, errlen, "Trace_LaunchTimeSpacing must be positive");
        if (p->tr_T < 0) return perr(err, errlen, "Trace_IntTLength < 0");
    }
    if (!p->ftle_compute && !p->tr_compute) return perr(err, errlen, "nothing to compute (FTLE_Compute = Trace_Compute = 0)");

    p->data_tmax = p->tmin + (p->tres - 1) * p->tdelta;
    if ((p->out_tstart < p->tmin || p->out_tstart > p->data_tmax) && !p->periodic)
        return perr(err, errlen, "Output_TStart outside data range");
    p->out_tend = p->out_tstart + (p->out_tres - 1) * p->int_dir * p->out_tdelta;
    if ((p->out_tend > p->data_tmax || p->out_tend < p->tmin) && !p->periodic)
        return perr(err, errlen, "Output_TEnd outside data range");
    if (p->ftle_compute) {
        p->fdelta[0] = (p->fb[1] - p->fb[0]) / (p->fres[0] - 1);
        p->fdelta[1] = (p->fb[3] - p->fb[2]) / (p->fres[1] - 1);
        if (p->dims == 3) p->fdelta[2] = (p->fb[5] - p->fb[4]) / (p->fres[2] - 1);
        else { p->fb[4] = 0; p->fb[5] = 0; p->fdelta[2] = 0; p->fres[2] = 1; }
        double tminreq = P_MIN(p->out_tstart, p->out_tend + p->int_dir * p->ftle_T);
        if (tminreq < p->tmin && !p->periodic) tminreq = p->tmin;
        double tmaxreq = P_MAX(p->out_tstart, p->out_tend + p->int_dir * p->ftle_T);
        if (tmaxreq > p->data_tmax && !p->periodic) tmaxreq = p->data_tmax;
        p->first_frame = p->int_dir > 0 ? (int)floor((tminreq - p->tmin) / p->tdelta) : (int)ceil((tmaxreq - p->tmin) / p->tdelta);
        p->last_frame = p->int_dir > 0 ? (int)ceil((tmaxreq - p->tmin) / p->tdelta) : (int)floor((tminreq - p->tmin) / p->tdelta);
    } else {
        p->first_frame = p->int_dir > 0 ? (int)floor((p->out_tstart - p->tmin) / p->tdelta) : (int)ceil((p->out_tstart - p->tmin) / p->tdelta);
        p->last_frame = p->int_dir > 0 ? (int)ceil((p->out_tend - p->tmin) / p->tdelta) : (int)floor((p->out_tend - p->tmin) / p->tdelta);
    }
    if (p->tr_genmesh) {
        for (int a = 0; a < 3; a++) {
            if (p->tres3[a] == 1) p->tdelta3[a] = 0.0;
            else if (a == 2 && p->dims != 3) { p->tb[4] = 0; p->tb[5] = 0; p->tdelta3[2] = 0; p->tres3[2] = 1; }
            else p->tdelta3[a] = (p->tb[2 * a + 1] - p->tb[2 * a]) / ((double)p->tres3[a] - 1.0);
        }
    }
    fix_path(p->path_output);
    fix_path(p->path_data);
    return 0;
}
