/* HARM dump ingest and image/spectrum output for the drop-in host.
 *
 * Ingest reads the format of init_harm_data (raptor_harm_model.c:68-187):
 * a 26-field header, then N1*N2 cell records of 34 numbers, i outer / j
 * inner.  The file is read in one piece; when it holds one record per line
 * (as HARM writes it) the lines are parsed in parallel, otherwise the
 * tokens are parsed in order as fscanf would.  The primitives land directly
 * in [8][N1][N2] - the layout raptor_gpu_upload_grid takes - instead of the
 * reference's pointer-chased p[q][i][j][0] (grmhd.c:76-91).  Unlike the
 * reference, a header whose N1/N2 do not match the body, a truncated body
 * or a non-finite primitive is an error (raptor_harm_model.c:116-119 only
 * prints).
 *
 * Output writes the reference's files byte for byte (core.c:154-200,
 * utilities.c:47-64): "%+.5e" per pixel, x outer / y inner; the formatting
 * is split over threads by image column and concatenated in order. */
#define _POSIX_C_SOURCE 200809L
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "raptor_host.h"

#define NVALS 34
#define C_PI 3.14159265358979323846
#define MSUN 1.989e33
#define YEAR 31536000.

static char *slurp(const char *path, size_t *len)
{
    FILE *f = fopen(path, "rb");
    if (!f)
        return NULL;
    if (fseek(f, 0, SEEK_END) != 0) {
        fclose(f);
        return NULL;
    }
    long n = ftell(f);
    rewind(f);
    char *buf = (char *)malloc((size_t)n + 1);
    if (!buf) {
        fclose(f);
        return NULL;
    }
    size_t got = fread(buf, 1, (size_t)n, f);
    fclose(f);
    buf[got] = 0;
    *len = got;
    return buf;
}

static int is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

/* parse up to n doubles from [p, end); returns count, *next after the last */
static int parse_doubles(const char *p, const char *end, double *out, int n, const char **next)
{
    int k = 0;
    while (k < n) {
        while (p < end && is_space(*p))
            p++;
        if (p >= end)
            break;
        char *e;
        double v = strtod(p, &e);
        if (e == p)
            break;
        out[k++] = v;
        p = e;
    }
    if (next)
        *next = p;
    return k;
}

static void store_cell(raptor_dump *d, long k, const double *v)
{
    const long plane = (long)d->geom.n1 * d->geom.n2;
    for (int q = 0; q < 8; q++)
        d->prims[q * plane + k] = v[4 + q];
}

int raptor_read_dump(const char *path, double M_UNIT, double T_unit, raptor_dump *d, char *err, size_t errlen)
{
    memset(d, 0, sizeof *d);
    fprintf(stderr, "Use slice %s\n", path);
    size_t len = 0;
    char *buf = slurp(path, &len);
    if (!buf) {
        snprintf(err, errlen, "can't open sim data file %s: %s", path, strerror(errno));
        return -1;
    }
    fprintf(stderr, "successfully opened %s\n", path);
    const char *p = buf, *end = buf + len;
    double h[26];
    const char *body;
    if (parse_doubles(p, end, h, 26, &body) != 26) {
        snprintf(err, errlen, "%s: truncated header", path);
        free(buf);
        return -1;
    }
    /* header order, raptor_harm_model.c:90-115 */
    d->t = h[0];
    int n1 = (int)h[1], n2 = (int)h[2];
    d->geom.n1 = n1;
    d->geom.n2 = n2;
    d->geom.startx1 = h[3];
    d->geom.startx2 = h[4];
    d->geom.dx1 = h[5];
    d->geom.dx2 = h[6];
    d->geom.a = h[9];
    d->gam = h[10];
    d->Rin = h[22];
    d->Rout = h[23];
    d->geom.hslope = h[24];
    d->geom.R0 = h[25];
    if (n1 < 2 || n2 < 2 || h[1] != n1 || h[2] != n2 || (long)n1 * n2 > (1L << 28)) {
        snprintf(err, errlen, "%s: bad grid size %g x %g in header", path, h[1], h[2]);
        free(buf);
        return -1;
    }
    const long ncell = (long)n1 * n2;
    fprintf(stderr, "Sim range x1, x2:  %g %g, %g %g\n", d->geom.startx1, d->geom.startx1 + n1 * d->geom.dx1,
            d->geom.startx2, d->geom.startx2 + n2 * d->geom.dx2);
    d->prims = (double *)malloc(sizeof(double) * 8 * (size_t)ncell);
    if (!d->prims) {
        snprintf(err, errlen, "out of memory for a %dx%d grid", n1, n2);
        free(buf);
        return -1;
    }
    /* one record per line? index the lines of the body */
    long nl = 0, cap = ncell + 16;
    const char **line = (const char **)malloc(sizeof(char *) * (size_t)cap);
    const char *q = body;
    int per_line = line != NULL;
    while (per_line && q < end) {
        while (q < end && is_space(*q) && *q != '\n')
            q++;
        if (q < end && *q == '\n') {
            q++;
            continue;
        }
        if (q >= end)
            break;
        if (nl >= cap) {
            per_line = 0;
            break;
        }
        line[nl++] = q;
        const char *nx = memchr(q, '\n', (size_t)(end - q));
        q = nx ? nx + 1 : end;
    }
    if (per_line && nl != ncell)
        per_line = 0;
    long bad = -1, short_rec = -1;
    double dM = 0., La = 0.;
    if (per_line) {
#pragma omp parallel for schedule(static) reduction(+ : dM, La)
        for (long k = 0; k < ncell; k++) {
            double v[NVALS];
            const char *le = (k + 1 < ncell) ? line[k + 1] : end;
            const char *nxt;
            if (parse_doubles(line[k], le, v, NVALS, &nxt) != NVALS) {
#pragma omp critical
                short_rec = k;
                continue;
            }
            store_cell(d, k, v);
            for (int m = 4; m < 12; m++)
                if (!isfinite(v[m])) {
#pragma omp critical
                    bad = k;
                }
            long i = k / n2;
            if (i <= 20)
                dM += v[33] * v[4] * v[14];
            if (i >= 20 && i < 40)
                La += v[33] * v[5] * v[14] * v[17];
        }
    } else {
        const char *c = body;
        for (long k = 0; k < ncell; k++) {
            double v[NVALS];
            if (parse_doubles(c, end, v, NVALS, &c) != NVALS) {
                short_rec = k;
                break;
            }
            store_cell(d, k, v);
            for (int m = 4; m < 12; m++)
                if (!isfinite(v[m]))
                    bad = k;
            long i = k / n2;
            if (i <= 20)
                dM += v[33] * v[4] * v[14];
            if (i >= 20 && i < 40)
                La += v[33] * v[5] * v[14] * v[17];
        }
    }
    free(line);
    free(buf);
    if (short_rec >= 0) {
        snprintf(err, errlen, "%s: cell record %ld is short: truncated or malformed dump", path, short_rec);
        raptor_free_dump(d);
        return -1;
    }
    if (bad >= 0) {
        snprintf(err, errlen, "%s: non-finite primitive in cell record %ld", path, bad);
        raptor_free_dump(d);
        return -1;
    }
    /* accretion-rate diagnostics, raptor_harm_model.c:171-182 */
    double dx2 = d->geom.dx2, dx3 = 2. * C_PI;
    d->dMact = dM * dx3 * dx2 / 21.;
    d->Ladv = La * dx3 * dx2 / 21.;
    fprintf(stderr, "dMact: %g Macc: %e [Msun/year], Ladv: %g\n", d->dMact,
            d->dMact * M_UNIT / T_unit / (MSUN / YEAR), d->Ladv);
    fprintf(stderr, "Done reading data\n\n");
    return 0;
}

void raptor_free_dump(raptor_dump *d)
{
    free(d->prims);
    d->prims = NULL;
}

/* write_image (utilities.c:47-64): x outer, y inner, "%+.5e\n". */
int raptor_write_image(FILE *f, const double *field, int width, int height, int nfreq, int fi, double scale)
{
    const int line_max = 32;
    int nthr = 1;
#ifdef _OPENMP
    nthr = omp_get_max_threads();
#endif
    if ((long)width * height < 65536)
        nthr = 1;
    int nchunk = nthr < width ? nthr : width;
    char **chunk = (char **)calloc((size_t)nchunk, sizeof(char *));
    size_t *clen = (size_t *)calloc((size_t)nchunk, sizeof(size_t));
    if (!chunk || !clen) {
        free(chunk);
        free(clen);
        return -1;
    }
    int fail = 0;
#pragma omp parallel for schedule(static) num_threads(nchunk) reduction(| : fail)
    for (int c = 0; c < nchunk; c++) {
        int x0 = (int)((long)width * c / nchunk), x1 = (int)((long)width * (c + 1) / nchunk);
        size_t cap = (size_t)(x1 - x0) * height * line_max + 1;
        char *b = (char *)malloc(cap);
        if (!b) {
            fail = 1;
            continue;
        }
        size_t n = 0;
        for (int i = x0; i < x1; i++)
            for (int j = 0; j < height; j++)
                n += (size_t)snprintf(b + n, cap - n, "%+.5e\n",
                                      scale * field[((size_t)i + (size_t)j * width) * nfreq + fi]);
        chunk[c] = b;
        clen[c] = n;
    }
    for (int c = 0; c < nchunk && !fail; c++)
        if (fwrite(chunk[c], 1, clen[c], f) != clen[c])
            fail = 1;
    for (int c = 0; c < nchunk; c++)
        free(chunk[c]);
    free(chunk);
    free(clen);
    return fail ? -1 : 0;
}

/* output_files (core.c:154-200) */
int raptor_output_files(const raptor_model *m, const raptor_units *u, const double *field, const double *spectrum,
                        const double *freq)
{
    struct stat st;
    if (stat(m->output_dir, &st) == -1)
        mkdir(m->output_dir, 0700);
    char name[1024];
    snprintf(name, sizeof name, "%s/spectrum_%d_%.02lf.dat", m->output_dir, (int)m->TIME_INIT, m->INCLINATION);
    FILE *spec = fopen(name, "w");
    if (!spec) {
        fprintf(stderr, "cannot write %s\n", name);
        return -1;
    }
    int rc = 0;
    for (int f = 0; f < m->num_indices; f++) {
        snprintf(name, sizeof name, "%s/img_data_%d_%e_%.02lf.dat", m->output_dir, (int)m->TIME_INIT, freq[f],
                 m->INCLINATION);
        FILE *img = fopen(name, "w");
        if (!img) {
            fprintf(stderr, "cannot write %s\n", name);
            rc = -1;
            continue;
        }
        printf("%s\n", m->GRMHD_FILE);
        fprintf(img, "%d %d %e %e %s %e %e %e %e\n", m->IMG_WIDTH, m->IMG_HEIGHT, u->JANSKY_FACTOR * spectrum[f],
                freq[f], m->GRMHD_FILE, m->M_UNIT, m->INCLINATION, m->R_LOW, m->R_HIGH);
        if (raptor_write_image(img, field, m->IMG_WIDTH, m->IMG_HEIGHT, m->num_indices, f, u->JANSKY_FACTOR))
            rc = -1;
        fclose(img);
        fprintf(stderr, "Frequency %.5e Integrated flux density = %.5e\n", freq[f], u->JANSKY_FACTOR * spectrum[f]);
        fprintf(spec, "%+.15e\t%+.15e\n", freq[f], u->JANSKY_FACTOR * spectrum[f]);
    }
    fclose(spec);
    return rc;
}
