/* In-process driver for the reference RAPTOR build (oracle test
 * infrastructure; never part of the shipped engine).
 *
 * It replays the reference's own start-up sequence, main.c:104-145:
 *   read_model(argv)        core.c:4-72    model.in + argv[2..7]
 *   init_model()            raptor_harm_model.c:59-66 (units + HARM dump)
 *   set_constants(TIME_INIT) utilities.c:17-45
 * and then renders either with the stock serial calculate_image
 * (core.c:74-152) or with an OpenMP loop over integrate_geodesic
 * (integrator.c:149-289) that follows the loop body of core.c:107-114 and
 * the LINEAR_IMPACT_CAM post-scale of core.c:136.  Results are handed back
 * as raw float64, because the image file keeps only six digits
 * (utilities.c:61). */
#include "functions.h"
#include "parameters.h"
#include "constants.h"
#include "raptor_harm_model.h"
#include <omp.h>

static void fmt_arg(char *dst, size_t n, double v) { snprintf(dst, n, "%.17g", v); }

/* argv layout of run.sh:5: RAPTOR model.in dump M_UNIT INCLINATION R_HIGH R_LOW TIME_INIT */
int ref_setup(const char *model_in, const char *dump, double m_unit,
              double inclination, double r_high, double r_low, double time_init)
{
    static char a1[256], a2[256], a3[64], a4[64], a5[64], a6[64], a7[64];
    if (strlen(model_in) >= 99 || strlen(dump) >= 255)
        return -1; /* read_model copies argv[1] into char[100] (core.c:5) */
    snprintf(a1, sizeof a1, "%s", model_in);
    snprintf(a2, sizeof a2, "%s", dump);
    fmt_arg(a3, sizeof a3, m_unit);
    fmt_arg(a4, sizeof a4, inclination);
    fmt_arg(a5, sizeof a5, r_high);
    fmt_arg(a6, sizeof a6, r_low);
    fmt_arg(a7, sizeof a7, time_init);
    char *argv[9] = {"RAPTOR", a1, a2, a3, a4, a5, a6, a7, NULL};
    read_model(argv);
    init_model();
    set_constants(TIME_INIT);
    return 0;
}

/* Stock path: calculate_image exactly as main.c:122-145 calls it, with one
 * frequency.  out[W*H] receives intensityfield[k][0] (already scaled by
 * nu^3 inside calculate_image), spectrum[0] the unscaled pixel sum. */
int ref_render_serial(double freq, double *out, double *spectrum)
{
    int npix = IMG_WIDTH * IMG_HEIGHT;
    if ((long)npix > (long)maxsize)
        return -2;
    real energy_spectrum[num_indices];
    real frequencies[num_indices];
    real **field = (real **)malloc((size_t)npix * sizeof(real *));
    real *store = (real *)calloc((size_t)npix * num_indices, sizeof(real));
    if (!field || !store)
        return -3;
    for (int i = 0; i < npix; i++)
        field[i] = store + (size_t)i * num_indices;
    frequencies[0] = freq;
    energy_spectrum[0] = 0.0;
    /* calculate_image frees the top-level grid pointer (core.c:143) */
    real ***keep[NPRIM];
    for (int q = 0; q < NPRIM; q++)
        keep[q] = p[q];
    calculate_image(field, energy_spectrum, frequencies);
    for (int i = 0; i < npix; i++)
        out[i] = field[i][0];
    spectrum[0] = energy_spectrum[0];
    free(field);
    free(store);
    for (int q = 0; q < NPRIM; q++) {
        for (int i = 0; i <= N1; i++) {
            for (int j = 0; j <= N2; j++)
                free(keep[q][i][j]);
            free(keep[q][i]);
        }
        free(keep[q]);
    }
    p = NULL;
    return 0;
}

/* Multi-threaded path over an arbitrary pixel list (pixel = x + y*W, as
 * core.c:108-109).  The global Newton-Raphson RNG (rcarry.c:20-21) is
 * shared between threads exactly as it would be with the core.c:105
 * pragma enabled; it only seeds the camera-angle root solve. */
int ref_render_pixels(const int *pixels, int n, double freq, double *out, int nthreads)
{
    if (!p)
        return -4;
    real (*buf)[num_indices] = malloc((size_t)(n > 0 ? n : 1) * sizeof(*buf));
    if (!buf)
        return -3;
    real frequencies[num_indices];
    frequencies[0] = freq;
    double nu3 = pow(freq, 3.);
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
    for (int k = 0; k < n; k++) {
        int i = pixels[k];
        int y = i / IMG_WIDTH;
        int x = i % IMG_WIDTH;
        integrate_geodesic(k, x, y, buf, frequencies, p, TIME_INIT, Xcam, Ucam);
    }
    for (int k = 0; k < n; k++)
        out[k] = buf[k][0] * nu3;
    free(buf);
    return 0;
}

double ref_wtime(void) { return omp_get_wtime(); }
int ref_grid_n1(void) { return N1; }
int ref_grid_n2(void) { return N2; }
int ref_int_method(void) { return int_method; }

/* Write the reference's own output files (core.c:154-200) for a given
 * image, into ./output of the current directory.  field[W*H] holds
 * intensityfield[k][0]; spectrum is energy_spectrum[0]. */
int ref_output_files(const double *field, double spectrum, double freq)
{
    int npix = IMG_WIDTH * IMG_HEIGHT;
    real **f = (real **)malloc((size_t)npix * sizeof(real *));
    real *store = (real *)malloc((size_t)npix * num_indices * sizeof(real));
    if (!f || !store)
        return -3;
    for (int i = 0; i < npix; i++) {
        f[i] = store + (size_t)i * num_indices;
        f[i][0] = field[i];
    }
    real energy_spectrum[num_indices];
    real frequencies[num_indices];
    energy_spectrum[0] = spectrum;
    frequencies[0] = freq;
    output_files(f, energy_spectrum, frequencies);
    free(f);
    free(store);
    return 0;
}

/* Scale one primitive of one cell of the loaded grid, p[q][i][j][0]
 * (grmhd.c:76-91), for finite-difference checks of per-cell gradients. */
int ref_scale_prim(int q, int i, int j, double factor)
{
    if (!p || q < 0 || q >= NPRIM || i < 0 || i >= N1 || j < 0 || j >= N2)
        return -1;
    p[q][i][j][0] *= factor;
    return 0;
}

/* The reference's kappa-distribution fits (j_nu.c:28-106), which its
 * emission_coeff does not call: out[0] = emission_coeff_kappa_FIT,
 * out[1] = absorption_coeff_kappa_FIT at one plasma state (theta: the
 * cosine of the pitch angle, as radiative_transfer.c:67 passes it; beta is
 * unused by both). */
void ref_kappa_coeffs(double nu, double ne, double thetae, double B, double theta, double *out)
{
    out[0] = emission_coeff_kappa_FIT(nu, ne, thetae, B, 0.0, theta);
    out[1] = absorption_coeff_kappa_FIT(nu, ne, thetae, B, 0.0, theta);
}
