/* Stand-in for <gsl/gsl_monte_plain.h> (see gsl_monte.h). */
#ifndef REFSHIM_GSL_MONTE_PLAIN_H
#define REFSHIM_GSL_MONTE_PLAIN_H
#include "gsl_monte.h"
typedef struct refshim_monte_plain gsl_monte_plain_state;
gsl_monte_plain_state *gsl_monte_plain_alloc(size_t dim);
int gsl_monte_plain_integrate(const gsl_monte_function *f, const double xl[], const double xu[], size_t dim,
                              size_t calls, gsl_rng *r, gsl_monte_plain_state *state, double *result, double *abserr);
void gsl_monte_plain_free(gsl_monte_plain_state *s);
#endif
