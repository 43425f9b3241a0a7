/* model.in / argv parsing, units and constants: read_model (core.c:4-72),
 * set_units (grmhd.c:17-33), set_constants (utilities.c:17-45), and the
 * frequency ladder of main.c:128-132. */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "raptor_host.h"

#define C_GGRAV 6.6742e-8
#define C_CLIGHT 2.99792458e10
#define C_PMASS 1.67262171e-24
#define C_EMASS 9.1093826e-28
#define C_PI 3.14159265358979323846
#define SOURCE_DIST 2.6228263e22 /* parameters.h:144 */
#define HORIZON_MARG 1e-1        /* parameters.h:185 */

static const char *env_or(const char *name, const char *dflt)
{
    const char *v = getenv(name);
    return (v && *v) ? v : dflt;
}

int raptor_read_model(int argc, char **argv, raptor_model *m, char *err, size_t errlen)
{
    memset(m, 0, sizeof *m);
    if (argc < 8) {
        snprintf(err, errlen, "usage: %s model.in dump M_UNIT INCLINATION R_HIGH R_LOW TIME_INIT",
                 argc > 0 ? argv[0] : "raptor_gb300");
        return -1;
    }
    FILE *in = fopen(argv[1], "r");
    if (!in) {
        snprintf(err, errlen, "Cannot read input file %s", argv[1]);
        return -1;
    }
    char t1[128], t2[128];
    int ok = 0;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->MBH) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->M_UNIT) == 3;
    ok += fscanf(in, "%127s %127s %d", t1, t2, &m->ABSORPTION) == 3;
    ok += fscanf(in, "%127s %127s %d", t1, t2, &m->IMG_WIDTH) == 3;
    ok += fscanf(in, "%127s %127s %d", t1, t2, &m->IMG_HEIGHT) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->CAM_SIZE_X) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->CAM_SIZE_Y) == 3;
    ok += fscanf(in, "%127s %127s %d", t1, t2, &m->FREQS_PER_DEC) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->FREQ_MIN) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->FREQ_MAX) == 3;
    ok += fscanf(in, "%127s %127s %lf", t1, t2, &m->STEPSIZE) == 3;
    fclose(in);
    if (ok != 11) {
        snprintf(err, errlen, "%s: expected 11 'NAME (unit) value' lines, parsed %d", argv[1], ok);
        return -1;
    }
    snprintf(m->GRMHD_FILE, sizeof m->GRMHD_FILE, "%s", argv[2]);
    /* argv[3] overrides model.in's M_UNIT (core.c:38) */
    if (sscanf(argv[3], "%lf", &m->M_UNIT) != 1 || sscanf(argv[4], "%lf", &m->INCLINATION) != 1 ||
        sscanf(argv[5], "%lf", &m->R_HIGH) != 1 || sscanf(argv[6], "%lf", &m->R_LOW) != 1 ||
        sscanf(argv[7], "%lf", &m->TIME_INIT) != 1) {
        snprintf(err, errlen, "M_UNIT INCLINATION R_HIGH R_LOW TIME_INIT must be numbers");
        return -1;
    }
    if (m->IMG_WIDTH <= 0 || m->IMG_HEIGHT <= 0 || !(m->STEPSIZE > 0) || m->FREQS_PER_DEC <= 0) {
        snprintf(err, errlen, "model.in: image size, STEPSIZE and FREQS_PER_DEC must be positive");
        return -1;
    }
    m->num_indices = atoi(env_or("RAPTOR_NUM_INDICES", "1"));
    if (m->num_indices < 1 || m->num_indices > RAPTOR_MAX_FREQS) {
        snprintf(err, errlen, "RAPTOR_NUM_INDICES must be 1..%d", RAPTOR_MAX_FREQS);
        return -1;
    }
    const char *im = env_or("RAPTOR_INT_METHOD", "RK4");
    if (!strcasecmp(im, "RK4"))
        m->integrator = RAPTOR_RK4;
    else if (!strcasecmp(im, "RK2"))
        m->integrator = RAPTOR_RK2;
    else {
        snprintf(err, errlen, "RAPTOR_INT_METHOD must be RK4 or RK2");
        return -1;
    }
    const char *cam = env_or("RAPTOR_CAMERA", "linear");
    if (!strcasecmp(cam, "linear"))
        m->camera = RAPTOR_CAM_LINEAR;
    else if (!strcasecmp(cam, "log"))
        m->camera = RAPTOR_CAM_LOG;
    else {
        snprintf(err, errlen, "RAPTOR_CAMERA must be linear or log");
        return -1;
    }
    const char *pr = env_or("RAPTOR_PRECISION", "fp64");
    if (!strcasecmp(pr, "fp64"))
        m->precision = RAPTOR_PREC_FP64;
    else if (!strcasecmp(pr, "mixed"))
        m->precision = RAPTOR_PREC_MIXED;
    else if (!strcasecmp(pr, "mixed_df"))
        m->precision = RAPTOR_PREC_MIXED_DF;
    else {
        snprintf(err, errlen, "RAPTOR_PRECISION must be fp64, mixed or mixed_df");
        return -1;
    }
    m->device = atoi(env_or("RAPTOR_DEVICE", "0"));
    snprintf(m->output_dir, sizeof m->output_dir, "%s", env_or("RAPTOR_OUTPUT_DIR", "output"));

    fprintf(stderr, "Model parameters:\n");
    fprintf(stderr, "MBH \t\t= %g \n", m->MBH);
    fprintf(stderr, "M_UNIT \t\t= %g \n", m->M_UNIT);
    fprintf(stderr, "R_HIGH \t\t= %g \n", m->R_HIGH);
    fprintf(stderr, "R_LOW \t\t= %g \n", m->R_LOW);
    fprintf(stderr, "INCLINATION \t= %g \n", m->INCLINATION);
    fprintf(stderr, "ABSORPTION \t= %d \n", m->ABSORPTION);
    fprintf(stderr, "\nObserver parameters:\n");
    fprintf(stderr, "IMG_WIDTH \t= %d \n", m->IMG_WIDTH);
    fprintf(stderr, "IMG_HEIGHT \t= %d \n", m->IMG_HEIGHT);
    fprintf(stderr, "CAM_SIZE_X \t= %g \n", m->CAM_SIZE_X);
    fprintf(stderr, "CAM_SIZE_Y \t= %g \n", m->CAM_SIZE_Y);
    fprintf(stderr, "FREQS_PER_DEC \t= %d \n", m->FREQS_PER_DEC);
    fprintf(stderr, "FREQ_MIN \t= %.03g \n", m->FREQ_MIN);
    fprintf(stderr, "FREQ_MAX \t= %.03g \n", m->FREQ_MIN * pow(10, (m->num_indices - 1.) / m->FREQS_PER_DEC));
    fprintf(stderr, "NUM OF FREQS \t= %d \n", m->num_indices);
    fprintf(stderr, "STEPSIZE \t= %g \n", m->STEPSIZE);
    return 0;
}

void raptor_set_units(const raptor_model *m, raptor_units *u)
{
    u->L_unit = C_GGRAV * m->MBH / (C_CLIGHT * C_CLIGHT);
    u->T_unit = u->L_unit / C_CLIGHT;
    u->RHO_unit = m->M_UNIT / pow(u->L_unit, 3);
    u->U_unit = u->RHO_unit * C_CLIGHT * C_CLIGHT;
    u->B_unit = C_CLIGHT * sqrt(4. * C_PI * u->RHO_unit);
    u->Ne_unit = u->RHO_unit / (C_PMASS + C_EMASS);
    fprintf(stderr, "\nUNITS\n");
    fprintf(stderr, "L,T,M: %g %g %g\n", u->L_unit, u->T_unit, m->M_UNIT);
    fprintf(stderr, "rho,u,B: %g %g %g\n", u->RHO_unit, u->U_unit, u->B_unit);
}

void raptor_set_constants(const raptor_model *m, double a, raptor_units *u)
{
    u->Rh = 1. + sqrt(1. - a * a);
    u->cutoff_inner = u->Rh * (1. + HORIZON_MARG);
    u->R_GRAV = C_GGRAV * m->MBH / C_CLIGHT / C_CLIGHT;
    double Z1 = 1. + pow(1. - a * a, 1. / 3.) * (pow(1. + a, 1. / 3.) + pow(1. - a, 1. / 3.));
    double Z2 = pow(3. * a * a + Z1 * Z1, 0.5);
    double retro = a < 0. ? 1. : -1.;
    u->R_ISCO = 3. + Z2 + retro * pow((3. - Z1) * (3. + Z1 + 2. * Z2), 0.5);
    /* pixel solid angle, utilities.c:32-42: LINEAR_IMPACT_CAM from the
     * camera size; LOG_IMPACT_CAM folds it into the image (core.c:123-133) */
    double pixsize = 1.;
    if (m->camera == RAPTOR_CAM_LINEAR) {
        double d_x = m->CAM_SIZE_X * u->R_GRAV, d_y = m->CAM_SIZE_Y * u->R_GRAV;
        double delta_x = d_x / SOURCE_DIST, delta_y = d_y / SOURCE_DIST;
        pixsize = (delta_x / (double)m->IMG_WIDTH) * (delta_y / (double)m->IMG_HEIGHT);
    }
    u->JANSKY_FACTOR = 1.e23 * pixsize;
}

void raptor_frequencies(const raptor_model *m, double *freq)
{
    for (int f = 0; f < m->num_indices; f++)
        freq[f] = m->FREQ_MIN * pow(10., (double)f / (double)m->FREQS_PER_DEC);
}
