/* Stand-in for <gsl/gsl_monte_vegas.h> (see gsl_monte.h). */
#include "gsl_monte.h"
