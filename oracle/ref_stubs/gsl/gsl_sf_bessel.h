/* Empty stand-in: j_nu.c:13 includes it, j_nu.c:146 replaced the call. */
#ifndef RAPTOR_ORACLE_GSL_BESSEL_STUB_H
#define RAPTOR_ORACLE_GSL_BESSEL_STUB_H
#endif
