/* Stand-in for <gsl/gsl_math.h>: the reference only needs M_PI from it. */
#include <math.h>
