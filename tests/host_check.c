/* Test driver for the drop-in host's ingest and output code
 * (raptor_gb300/host/harm_io.c, model_io.c), without a GPU.
 *
 *   host_check parse <dump> <out.bin>
 *       read the dump; write n1, n2 (int32) then prims [8][n1][n2] float64
 *   host_check write <field.bin> <spectrum> model.in dump M_UNIT INCL R_HIGH R_LOW TIME_INIT
 *       write the reference-format output files for field [W*H] float64
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "raptor_host.h"

int main(int argc, char **argv)
{
    char err[512];
    if (argc == 4 && !strcmp(argv[1], "parse")) {
        raptor_dump d;
        if (raptor_read_dump(argv[2], 1e19, 22.171, &d, err, sizeof err)) {
            fprintf(stderr, "%s\n", err);
            return 2;
        }
        FILE *f = fopen(argv[3], "wb");
        fwrite(&d.geom.n1, sizeof(int), 1, f);
        fwrite(&d.geom.n2, sizeof(int), 1, f);
        fwrite(d.prims, sizeof(double), (size_t)8 * d.geom.n1 * d.geom.n2, f);
        fclose(f);
        raptor_free_dump(&d);
        return 0;
    }
    if (argc == 11 && !strcmp(argv[1], "write")) {
        raptor_model m;
        if (raptor_read_model(argc - 3, argv + 3, &m, err, sizeof err)) {
            fprintf(stderr, "%s\n", err);
            return 2;
        }
        size_t n = (size_t)m.IMG_WIDTH * m.IMG_HEIGHT;
        double *field = malloc(n * sizeof(double));
        FILE *f = fopen(argv[2], "rb");
        if (!f || fread(field, sizeof(double), n, f) != n)
            return 3;
        fclose(f);
        raptor_units u;
        raptor_set_units(&m, &u);
        raptor_set_constants(&m, 0.9375, &u);
        double freq[RAPTOR_MAX_FREQS], spec[1];
        spec[0] = strtod(argv[3], NULL);
        raptor_frequencies(&m, freq);
        int rc = raptor_output_files(&m, &u, field, spec, freq);
        free(field);
        return rc ? 4 : 0;
    }
    fprintf(stderr, "usage: see the header comment\n");
    return 1;
}
