/* Empty stand-in: metric.c:11 includes it and calls nothing from it. */
#ifndef RAPTOR_ORACLE_GSL_LINALG_STUB_H
#define RAPTOR_ORACLE_GSL_LINALG_STUB_H
#endif
