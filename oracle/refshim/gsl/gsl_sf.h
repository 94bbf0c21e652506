/* Stand-in for <gsl/gsl_sf.h>: Bessel J (above) and the Legendre polynomial
 * P_l(x), evaluated like GSL's gsl_sf_legendre_Pl for l < 100000 (upward
 * three-term recurrence from P_0 = 1, P_1 = x, with P_2 in closed form). */
#ifndef REFSHIM_GSL_SF_H
#define REFSHIM_GSL_SF_H
#include "gsl_sf_bessel.h"
double gsl_sf_legendre_Pl(int l, double x);
#endif
