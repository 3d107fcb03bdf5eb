/* GSL random-generator handles, for oracle/ref.mk (TEST INFRASTRUCTURE).
 * The Henon step draws from the reference's own taus113 state (curr_st); the
 * gsl_rng objects it allocates are never drawn from on that path, so these
 * handles carry no generator. */
#ifndef CMCREF_SHIM_GSL_RNG_H
#define CMCREF_SHIM_GSL_RNG_H
#include "gsl_math.h"
typedef struct { const char *name; } gsl_rng_type;
typedef struct { const gsl_rng_type *type; unsigned long seed; } gsl_rng;
extern const gsl_rng_type *gsl_rng_taus2;
extern const gsl_rng_type *gsl_rng_default;
extern const gsl_rng_type *gsl_rng_mt19937;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
const gsl_rng_type *gsl_rng_env_setup(void);
#endif
