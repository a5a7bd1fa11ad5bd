/* Minimal restatement of GSL's multimin "fdf" minimiser interface (public API of GSL >= 1.16:
 * the function object, the minimiser type table and the framework calls).  Test
 * infrastructure: with it the reference's own conjugate_rdx minimiser type compiles into
 * oracle/_ref, driven by oracle/ref_driver.cpp. */
#ifndef RDXG_REF_GSL_MULTIMIN_H
#define RDXG_REF_GSL_MULTIMIN_H
#include <math.h>
#include <stddef.h>

#include "gsl_errno.h"
#include "gsl_vector.h"

struct gsl_multimin_function_fdf_struct {
    double (*f)(const gsl_vector* x, void* params);
    void (*df)(const gsl_vector* x, void* params, gsl_vector* df);
    void (*fdf)(const gsl_vector* x, void* params, double* f, gsl_vector* df);
    size_t n;
    void* params;
};
typedef struct gsl_multimin_function_fdf_struct gsl_multimin_function_fdf;

#define GSL_MULTIMIN_FN_EVAL_F(F, x) (*((F)->f))(x, (F)->params)
#define GSL_MULTIMIN_FN_EVAL_DF(F, x, g) (*((F)->df))(x, (F)->params, (g))
#define GSL_MULTIMIN_FN_EVAL_F_DF(F, x, y, g) (*((F)->fdf))(x, (F)->params, (y), (g))

typedef struct {
    const char* name;
    size_t size;
    int (*alloc)(void* state, size_t n);
    int (*set)(void* state, gsl_multimin_function_fdf* fdf, const gsl_vector* x, double* f, gsl_vector* gradient,
               double step_size, double tol);
    int (*iterate)(void* state, gsl_multimin_function_fdf* fdf, gsl_vector* x, double* f, gsl_vector* gradient,
                   gsl_vector* dx);
    int (*restart)(void* state);
    void (*free)(void* state);
} gsl_multimin_fdfminimizer_type;

typedef struct {
    const gsl_multimin_fdfminimizer_type* type;
    gsl_multimin_function_fdf* fdf;
    double f;
    gsl_vector* x;
    gsl_vector* gradient;
    gsl_vector* dx;
    void* state;
} gsl_multimin_fdfminimizer;

gsl_multimin_fdfminimizer* gsl_multimin_fdfminimizer_alloc(const gsl_multimin_fdfminimizer_type* T, size_t n);
int gsl_multimin_fdfminimizer_set(gsl_multimin_fdfminimizer* s, gsl_multimin_function_fdf* fdf,
                                  const gsl_vector* x, double step_size, double tol);
int gsl_multimin_fdfminimizer_iterate(gsl_multimin_fdfminimizer* s);
void gsl_multimin_fdfminimizer_free(gsl_multimin_fdfminimizer* s);

#endif
