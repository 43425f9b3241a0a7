/* Host side of the drop-in: everything the reference does around
 * calculate_image, rewritten for the GB300 engine.  The command line,
 * model.in, the HARM dump format and the output files are the reference's:
 *
 *   raptor_gb300 model.in dump M_UNIT INCLINATION R_HIGH R_LOW TIME_INIT
 *
 * (main.c:95-167, run.sh:5).  Engine choices that the reference fixes at
 * compile time are environment variables here:
 *   RAPTOR_INT_METHOD   RK4 (default) or RK2        parameters.h:189
 *   RAPTOR_NUM_INDICES  frequencies, 1..8 (def. 1) parameters.h:215
 *   RAPTOR_PRECISION    fp64 (default), mixed or mixed_df
 *   RAPTOR_CAMERA       linear (default) or log     parameters.h:54-55
 *   RAPTOR_DEVICE       CUDA device ordinal (default 0)
 *   RAPTOR_OUTPUT_DIR   output folder (default "output", core.c:157)
 */
#ifndef RAPTOR_HOST_H
#define RAPTOR_HOST_H

#include <stdio.h>

#include "raptor_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct raptor_model {
    /* model.in, core.c:22-34 */
    double MBH, M_UNIT;
    int ABSORPTION;
    int IMG_WIDTH, IMG_HEIGHT;
    double CAM_SIZE_X, CAM_SIZE_Y;
    int FREQS_PER_DEC;
    double FREQ_MIN, FREQ_MAX, STEPSIZE;
    /* argv, core.c:37-42 */
    char GRMHD_FILE[256];
    double INCLINATION, R_HIGH, R_LOW, TIME_INIT;
    /* engine settings (environment) */
    int num_indices, integrator, precision, device;
    int camera; /* RAPTOR_CAM_LINEAR or RAPTOR_CAM_LOG (parameters.h:54-55) */
    char output_dir[256];
} raptor_model;

typedef struct raptor_units {
    double L_unit, T_unit, RHO_unit, U_unit, B_unit, Ne_unit; /* grmhd.c:17-33 */
    double Rh, cutoff_inner, R_GRAV, R_ISCO, JANSKY_FACTOR;   /* utilities.c:17-45 */
} raptor_units;

typedef struct raptor_dump {
    raptor_grid_geom geom;
    double t, gam, Rin, Rout;
    double *prims; /* [8][n1][n2] */
    double dMact, Ladv;
} raptor_dump;

/* model_io.c */
int raptor_read_model(int argc, char **argv, raptor_model *m, char *err, size_t errlen);
void raptor_set_units(const raptor_model *m, raptor_units *u);
void raptor_set_constants(const raptor_model *m, double a, raptor_units *u);
void raptor_frequencies(const raptor_model *m, double *freq);

/* harm_io.c */
int raptor_read_dump(const char *path, double M_UNIT, double T_unit, raptor_dump *d, char *err, size_t errlen);
void raptor_free_dump(raptor_dump *d);
int raptor_write_image(FILE *f, const double *field, int width, int height, int nfreq, int freq_index,
                       double scalefactor);
int raptor_output_files(const raptor_model *m, const raptor_units *u, const double *field,
                        const double *spectrum, const double *freq);

#ifdef __cplusplus
}
#endif
#endif
