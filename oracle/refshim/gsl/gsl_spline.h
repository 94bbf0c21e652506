/* Stand-in for <gsl/gsl_spline.h>: global.h includes it.  calculate_gamma.c's
 * calculate_gamma() uses a GSL cubic spline; that routine is not exercised by
 * the oracle (its default path calculate_gamma_2d integrates with its own
 * integrate_cubic_spline), so in libmodalref these entry points are link stubs
 * that report misuse if called.  fixed_data.c's spectrum readers interpolate
 * with gsl_interp_cspline; in libmodalfiles a natural cubic spline of this
 * repository's own (files_glue.c) stands in for it. */
#ifndef REFSHIM_GSL_SPLINE_H
#define REFSHIM_GSL_SPLINE_H
#include <stddef.h>
typedef struct refshim_spline gsl_spline;
typedef struct refshim_interp_accel gsl_interp_accel;
typedef struct refshim_interp_type gsl_interp_type;
extern const gsl_interp_type *gsl_interp_cspline;
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n);
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n);
double gsl_spline_eval_integ(const gsl_spline *s, double a, double b, gsl_interp_accel *acc);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *acc);
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
#endif
