/* Stand-in for <gsl/gsl_monte.h>: the Monte Carlo routines of
 * orthogonalisation.c / calculate_eigen.c (calculate_ortho_mc and friends)
 * are declared so the files compile; the grid paths used here never call
 * them, and the link stubs in ref_glue.c abort if they are. */
#ifndef REFSHIM_GSL_MONTE_H
#define REFSHIM_GSL_MONTE_H
#include <stddef.h>
typedef struct { double (*f)(double *x, size_t dim, void *params); size_t dim; void *params; } gsl_monte_function;
typedef struct refshim_rng_type gsl_rng_type;
typedef struct refshim_rng gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
const gsl_rng_type *gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
#endif
