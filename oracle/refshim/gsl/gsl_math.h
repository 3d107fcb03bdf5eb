/* The subset of GSL's math header the reference's hot-path TUs use, for
 * oracle/ref.mk (TEST INFRASTRUCTURE).  GSL itself is not in this image;
 * these are the documented meanings of the names, written here. */
#ifndef CMCREF_SHIM_GSL_MATH_H
#define CMCREF_SHIM_GSL_MATH_H
#include <float.h>
#include <math.h>
#define GSL_POSINF (INFINITY)
#define GSL_NEGINF (-INFINITY)
#define GSL_NAN (NAN)
#define GSL_SIGN(x) ((x) >= 0.0 ? 1 : -1)
#define GSL_MAX(a, b) ((a) > (b) ? (a) : (b))
#define GSL_MIN(a, b) ((a) < (b) ? (a) : (b))
typedef struct {
    double (*function)(double x, void *params);
    void *params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
#endif
