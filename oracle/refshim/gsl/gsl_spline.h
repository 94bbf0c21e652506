/* Stand-in for <gsl/gsl_spline.h>: global.h includes it; the compiled subset
 * only needs the type names. */
#ifndef REFSHIM_GSL_SPLINE_H
#define REFSHIM_GSL_SPLINE_H
typedef struct refshim_spline gsl_spline;
typedef struct refshim_interp_accel gsl_interp_accel;
#endif
