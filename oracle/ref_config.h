/* Forced-include header (gcc -include) for building the reference RAPTOR
 * sources unmodified, straight from where they lie.
 *
 * It pulls in the reference's parameters.h once (its include guard then
 * swallows every later #include of it) and overrides the compile-time
 * switches that the reference only offers as #defines:
 *
 *   int_method  parameters.h:189  RK2 in the stock build; RK4 for the
 *                                  benchmark configurations
 *   N1, N2      parameters.h:76-77 grid size of the dump being read
 *   maxsize     parameters.h:52   image buffer; 1e6 silently drops pixels
 *                                  of images larger than 1000x1000
 *                                  (core.c:76,81-83), so it is raised to
 *                                  at least W*H
 *   LOG_IMPACT_CAM / LINEAR_IMPACT_CAM  parameters.h:54-55, swapped when
 *                                  REF_LOG_CAM is defined
 *
 * num_indices (parameters.h:215) stays 1: transfer is independent per
 * frequency (radiative_transfer.c:71-98), so the oracle runs one
 * frequency per call. */
#ifndef RAPTOR_ORACLE_REF_CONFIG_H
#define RAPTOR_ORACLE_REF_CONFIG_H
#include "parameters.h"

#ifndef REF_INT_METHOD
#define REF_INT_METHOD RK4
#endif
#ifndef REF_N1
#define REF_N1 256
#endif
#ifndef REF_N2
#define REF_N2 256
#endif
#ifndef REF_MAXSIZE
#define REF_MAXSIZE 4194304
#endif

#undef int_method
#define int_method (REF_INT_METHOD)
#undef N1
#define N1 (REF_N1)
#undef N2
#define N2 (REF_N2)
#undef maxsize
#define maxsize (REF_MAXSIZE)
#ifdef REF_LOG_CAM
#undef LOG_IMPACT_CAM
#define LOG_IMPACT_CAM (1)
#undef LINEAR_IMPACT_CAM
#define LINEAR_IMPACT_CAM (0)
#endif
#endif
