/* Minimal restatement of GSL's gsl_vector (public API; unit stride only).  Test
 * infrastructure for oracle/_ref. */
#ifndef RDXG_REF_GSL_VECTOR_H
#define RDXG_REF_GSL_VECTOR_H
#include <stddef.h>

typedef struct {
    size_t size;
    size_t stride;
    double* data;
    void* block;
    int owner;
} gsl_vector;

gsl_vector* gsl_vector_alloc(size_t n);
gsl_vector* gsl_vector_calloc(size_t n);
void gsl_vector_free(gsl_vector* v);
int gsl_vector_memcpy(gsl_vector* dest, const gsl_vector* src);
void gsl_vector_set_zero(gsl_vector* v);

#endif
