/* Stand-in for <gsl/gsl_integration.h>: orthogonalisation_late.c allocates a
 * fixed Gauss-Legendre table it never uses; the stand-in returns NULL. */
#ifndef REFSHIM_GSL_INTEGRATION_H
#define REFSHIM_GSL_INTEGRATION_H
#include <stddef.h>
typedef struct refshim_glfixed gsl_integration_glfixed_table;
gsl_integration_glfixed_table *gsl_integration_glfixed_table_alloc(size_t n);
void gsl_integration_glfixed_table_free(gsl_integration_glfixed_table *t);
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
#endif
