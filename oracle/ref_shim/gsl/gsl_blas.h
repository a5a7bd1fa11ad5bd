/* Minimal restatement of the GSL level-1 BLAS calls the reference's minimiser makes
 * (gsl_blas_dnrm2, gsl_blas_ddot, gsl_blas_daxpy), following GSL's own CBLAS.  Test
 * infrastructure for oracle/_ref. */
#ifndef RDXG_REF_GSL_BLAS_H
#define RDXG_REF_GSL_BLAS_H
#include "gsl_vector.h"

double gsl_blas_dnrm2(const gsl_vector* x);
int gsl_blas_ddot(const gsl_vector* x, const gsl_vector* y, double* result);
int gsl_blas_daxpy(double alpha, const gsl_vector* x, gsl_vector* y);

#endif
