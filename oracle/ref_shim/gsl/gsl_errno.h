/* Minimal restatement of the GSL error interface that the reference's minimiser uses
 * (GSL >= 1.16 public API: error codes and the GSL_ERROR macro).  Test infrastructure: it
 * exists only so that the reference's own src/lib/util/gsl/conjugate_gradient.cpp compiles
 * into oracle/_ref without GSL installed. */
#ifndef RDXG_REF_GSL_ERRNO_H
#define RDXG_REF_GSL_ERRNO_H
#include <stdio.h>

enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_ENOMEM = 8, GSL_ENOPROG = 27 };

#define GSL_ERROR(reason, gsl_errno)                                  \
    do {                                                              \
        fprintf(stderr, "gsl: %s:%d: %s\n", __FILE__, __LINE__, reason); \
        return gsl_errno;                                             \
    } while (0)

#endif
