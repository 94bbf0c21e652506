/* Stand-in for <gsl/gsl_sf_bessel.h>: GSL's regular cylindrical Bessel
 * functions J0, J1, Jn, forwarded to the C library's j0/j1/jn. */
#ifndef REFSHIM_GSL_SF_BESSEL_H
#define REFSHIM_GSL_SF_BESSEL_H
double gsl_sf_bessel_J0(double x);
double gsl_sf_bessel_J1(double x);
double gsl_sf_bessel_Jn(int n, double x);
#endif
