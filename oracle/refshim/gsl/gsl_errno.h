/* Stand-in for <gsl/gsl_errno.h> (nothing used by the compiled subset). */
