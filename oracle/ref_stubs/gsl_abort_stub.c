/* Definition for the one GSL symbol the reference links against
 * (j_nu.c:89-96, kappa absorptivity only).  The thermal-synchrotron path
 * never calls it; if it ever is called the oracle must not return a
 * made-up number, so it aborts. */
#include <stdio.h>
#include <stdlib.h>

double gsl_sf_hyperg_2F1(double a, double b, double c, double x)
{
    (void)a; (void)b; (void)c; (void)x;
    fprintf(stderr, "oracle: gsl_sf_hyperg_2F1 reached (kappa path is out of scope)\n");
    abort();
}
