/* Definition for the one GSL symbol the reference links against,
 * gsl_sf_hyperg_2F1 (called only from the kappa-distribution absorptivity,
 * j_nu.c:85-96; GSL is not installed here).  The Gauss hypergeometric
 * function by its power series sum_n (a)_n (b)_n / ((c)_n n!) x^n for
 * 0 <= x <= 1/2 and Pfaff's transformation
 * 2F1(a, b; c; x) = (1 - x)^-a 2F1(a, c - b; c; x / (x - 1)) for
 * -1 <= x < 0 - the two ranges the reference's call sites reach.  Outside
 * them the oracle must not return a made-up number, so it aborts.  Checked
 * against scipy's hyp2f1 through the oracle port's copy of the same method
 * (tests/test_oracle.py). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

double gsl_sf_hyperg_2F1(double a, double b, double c, double x)
{
    if (x < -1.0 || x > 0.5) {
        fprintf(stderr, "oracle: gsl_sf_hyperg_2F1 outside [-1, 1/2] (x = %g)\n", x);
        abort();
    }
    if (x < 0)
        return pow(1 - x, -a) * gsl_sf_hyperg_2F1(a, c - b, c, x / (x - 1));
    double term = 1.0, sum = 1.0;
    for (int n = 0; n < 400; n++) {
        term *= (a + n) * (b + n) / ((c + n) * (n + 1)) * x;
        sum += term;
        if (fabs(term) <= 1e-17 * fabs(sum))
            break;
    }
    return sum;
}
