/* Stand-in for <gsl/gsl_monte_miser.h> (see gsl_monte.h). */
#include "gsl_monte.h"
