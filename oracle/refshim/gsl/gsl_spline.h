/* GSL interpolation handles named by comp_multi_mass_percent (cmc_utils.c),
 * which the Henon step does not reach; oracle/ref.mk (TEST INFRASTRUCTURE)
 * links aborting definitions. */
#ifndef CMCREF_SHIM_GSL_SPLINE_H
#define CMCREF_SHIM_GSL_SPLINE_H
typedef struct { const char *name; } gsl_interp_type;
typedef struct gsl_spline { const gsl_interp_type *type; } gsl_spline;
typedef struct gsl_interp_accel { unsigned long cache; } gsl_interp_accel;
extern const gsl_interp_type *gsl_interp_linear;
extern const gsl_interp_type *gsl_interp_cspline;
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, unsigned long n);
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], unsigned long n);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
#endif
