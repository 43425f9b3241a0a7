/* Prototype-only stand-in for GSL's hypergeometric header.  The reference
 * calls gsl_sf_hyperg_2F1 only from the kappa-distribution absorptivity
 * (j_nu.c:85-96), which the thermal hot path never reaches.  GSL is not
 * installed here; gsl_hyperg_stub.c supplies a definition (power series and
 * Pfaff's transformation on the ranges the reference reaches). */
#ifndef RAPTOR_ORACLE_GSL_HYPERG_STUB_H
#define RAPTOR_ORACLE_GSL_HYPERG_STUB_H
double gsl_sf_hyperg_2F1(double a, double b, double c, double x);
#endif
