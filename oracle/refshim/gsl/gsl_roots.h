/* GSL's bracketing root-solver interface as find_root_vr uses it
 * (cmc_nr.c:500-603), for oracle/ref.mk (TEST INFRASTRUCTURE).  The one
 * solver type, "brent", is Brent's method restated from Brent (1973),
 * "Algorithms for Minimization without Derivatives", ch. 4 (oracle/brent1973.h),
 * the same restatement cmc_oracle.c uses; GSL's sources are not part of the
 * reference and are not used. */
#ifndef CMCREF_SHIM_GSL_ROOTS_H
#define CMCREF_SHIM_GSL_ROOTS_H
#include "gsl_math.h"
#include "gsl_errno.h"
typedef struct { const char *name; } gsl_root_fsolver_type;
typedef struct gsl_root_fsolver gsl_root_fsolver;
extern const gsl_root_fsolver_type *gsl_root_fsolver_brent;
gsl_root_fsolver *gsl_root_fsolver_alloc(const gsl_root_fsolver_type *T);
void gsl_root_fsolver_free(gsl_root_fsolver *s);
int gsl_root_fsolver_set(gsl_root_fsolver *s, gsl_function *f, double x_lower, double x_upper);
int gsl_root_fsolver_iterate(gsl_root_fsolver *s);
double gsl_root_fsolver_root(const gsl_root_fsolver *s);
double gsl_root_fsolver_x_lower(const gsl_root_fsolver *s);
double gsl_root_fsolver_x_upper(const gsl_root_fsolver *s);
int gsl_root_test_interval(double x_lower, double x_upper, double epsabs, double epsrel);
int gsl_root_test_delta(double x1, double x0, double epsabs, double epsrel);
#endif
