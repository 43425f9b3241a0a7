/* Drop-in for the reference program (main.c:95-167): same command line,
 * model.in, HARM dump and output files; calculate_image (core.c:74-152)
 * runs on the GPU through the engine's C ABI.
 *
 *   raptor_gb300 model.in dump M_UNIT INCLINATION R_HIGH R_LOW TIME_INIT
 *
 * Differences from the reference, all deliberate: every pixel is rendered
 * (the reference drops pixels past index 1e6, core.c:81-83); errors return
 * a non-zero exit status instead of continuing; the integrator, the
 * camera map and the number of frequencies are run-time settings
 * (raptor_host.h). */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "raptor_host.h"

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* calculate_image on the GPU: fills field[W*H][F] (nu^3-scaled, as
 * core.c:136) and spectrum[F] (core.c:146-150). */
static int calculate_image_gpu(const raptor_model *m, const raptor_dump *d, const double *freq, double *field,
                               double *spectrum)
{
    raptor_gpu_options opt;
    memset(&opt, 0, sizeof opt);
    opt.device = m->device;
    raptor_gpu_ctx *ctx = NULL;
    int rc = raptor_gpu_init(&opt, &ctx);
    if (rc != RAPTOR_OK) {
        fprintf(stderr, "raptor_gpu_init failed (%d): no usable GPU\n", rc);
        return rc;
    }
    int gid = -1;
    rc = raptor_gpu_upload_grid(ctx, d->prims, &d->geom, &gid);
    if (rc == RAPTOR_OK) {
        raptor_image_desc img;
        memset(&img, 0, sizeof img);
        img.width = m->IMG_WIDTH;
        img.height = m->IMG_HEIGHT;
        img.cam_size_x = m->CAM_SIZE_X;
        img.cam_size_y = m->CAM_SIZE_Y;
        img.inclination = m->INCLINATION;
        img.mbh = m->MBH;
        img.m_unit = m->M_UNIT;
        img.r_high = m->R_HIGH;
        img.r_low = m->R_LOW;
        img.stepsize = m->STEPSIZE;
        img.integrator = m->integrator;
        img.camera = m->camera;
        img.grid = gid;
        img.n_freq = m->num_indices;
        for (int f = 0; f < m->num_indices; f++)
            img.freq[f] = freq[f];
        rc = raptor_gpu_render(ctx, &img, 1, m->precision, field, spectrum);
    }
    if (rc < 0) {
        fprintf(stderr, "engine error (%d): %s\n", rc, raptor_gpu_last_error(ctx));
    } else {
        /* a positive status is a warning: the image is complete */
        if (rc > 0)
            fprintf(stderr, "engine warning (%d): %s\n", rc, raptor_gpu_last_error(ctx));
        rc = RAPTOR_OK;
        raptor_gpu_stats st;
        raptor_gpu_get_stats(ctx, &st);
        printf("Done: 1e+02 %%, speed: %.3g [geodesics/sec] (%lld steps, kernel %.1f ms)\n",
               st.rays / (st.kernel_ms * 1e-3), st.steps, st.kernel_ms);
    }
    raptor_gpu_destroy(ctx);
    return rc;
}

int main(int argc, char **argv)
{
    fprintf(stderr, "WELCOME TO RAPTOR 1.0 (GB300 engine)\n\n");
    double t0 = now_s();
    char err[512];
    raptor_model m;
    if (raptor_read_model(argc, argv, &m, err, sizeof err)) {
        fprintf(stderr, "%s\n", err);
        return 1;
    }
    raptor_units u;
    raptor_set_units(&m, &u);
    raptor_dump d;
    if (raptor_read_dump(m.GRMHD_FILE, m.M_UNIT, u.T_unit, &d, err, sizeof err)) {
        fprintf(stderr, "%s\n", err);
        return 1;
    }
    fprintf(stderr, "\nREADING HARM2D SIMULATION DATA\n");
    raptor_set_constants(&m, d.geom.a, &u);
    fprintf(stderr, "\nFinished initialization. (%.3f s)\n", now_s() - t0);

    double freq[RAPTOR_MAX_FREQS], spectrum[RAPTOR_MAX_FREQS];
    raptor_frequencies(&m, freq);
    size_t npix = (size_t)m.IMG_WIDTH * m.IMG_HEIGHT;
    double *field = (double *)calloc(npix * m.num_indices, sizeof(double));
    if (!field) {
        fprintf(stderr, "out of memory for the image\n");
        return 1;
    }
    int rc = calculate_image_gpu(&m, &d, freq, field, spectrum);
    raptor_free_dump(&d);
    if (rc != RAPTOR_OK) {
        free(field);
        return 2;
    }
    fprintf(stderr, "\nFinished ray tracing calculations. (%.3f s)\n", now_s() - t0);
    rc = raptor_output_files(&m, &u, field, spectrum, freq);
    fprintf(stderr, "\nFinished writing output files. (%.3f s)\n", now_s() - t0);
    free(field);
    return rc ? 3 : 0;
}
