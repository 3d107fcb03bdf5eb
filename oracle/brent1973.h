/* Brent's method for a bracketed zero, restated from R. P. Brent, "Algorithms
 * for Minimization without Derivatives" (1973), ch. 4, procedure zero (TEST
 * INFRASTRUCTURE).
 *
 * One interpolation or bisection step per call, the bracket kept as [b, c].
 * The reference's find_root_vr (cmc_nr.c:500-603) drives GSL's Brent solver,
 * whose sources are not part of the reference; this one restatement stands in
 * for it in both the oracle (cmc_oracle.c) and the GSL shim that the
 * reference's own cmc_nr.c is compiled against (refshim/refshim.c), so the two
 * agree with each other by construction on that branch. */
#ifndef CMC_BRENT1973_H
#define CMC_BRENT1973_H
#include <float.h>
#include <math.h>

typedef struct {
    double a, b, c, d, e, fa, fb, fc;
    int exact; /* f(b) == 0: the bracket collapses to [b, b] */
} brent_t;

static inline int brent_set(brent_t *z, double fl, double fu, double lo, double hi)
{
    z->a = lo;
    z->fa = fl;
    z->b = hi;
    z->fb = fu;
    z->c = hi;
    z->fc = fu;
    z->d = hi - lo;
    z->e = hi - lo;
    z->exact = 0;
    if ((fl < 0.0 && fu < 0.0) || (fl > 0.0 && fu > 0.0)) return 1;
    return 0;
}

static inline void brent_fix_bracket(brent_t *z)
{
    if ((z->fb < 0.0 && z->fc < 0.0) || (z->fb > 0.0 && z->fc > 0.0)) {
        z->c = z->a;
        z->fc = z->fa;
        z->d = z->b - z->a;
        z->e = z->b - z->a;
    }
    if (fabs(z->fc) < fabs(z->fb)) {
        z->a = z->b;
        z->b = z->c;
        z->c = z->a;
        z->fa = z->fb;
        z->fb = z->fc;
        z->fc = z->fa;
    }
}

/* returns the new abscissa at which the caller must evaluate f */
static inline double brent_propose(brent_t *z)
{
    brent_fix_bracket(z);
    double tol = 0.5 * DBL_EPSILON * fabs(z->b);
    double m = 0.5 * (z->c - z->b);
    if (z->fb == 0.0 || fabs(m) <= tol) return z->b;
    if (fabs(z->e) < tol || fabs(z->fa) <= fabs(z->fb)) {
        z->d = m;
        z->e = m;
    } else {
        double p, q, r, s = z->fb / z->fa;
        if (z->a == z->c) {
            p = 2.0 * m * s;
            q = 1.0 - s;
        } else {
            q = z->fa / z->fc;
            r = z->fb / z->fc;
            p = s * (2.0 * m * q * (q - r) - (z->b - z->a) * (r - 1.0));
            q = (q - 1.0) * (r - 1.0) * (s - 1.0);
        }
        if (p > 0.0)
            q = -q;
        else
            p = -p;
        double min1 = 3.0 * m * q - fabs(tol * q), min2 = fabs(z->e * q);
        if (2.0 * p < (min1 < min2 ? min1 : min2)) {
            z->e = z->d;
            z->d = p / q;
        } else {
            z->d = m;
            z->e = m;
        }
    }
    z->a = z->b;
    z->fa = z->fb;
    if (fabs(z->d) > tol)
        z->b += z->d;
    else
        z->b += (m > 0 ? tol : -tol);
    return z->b;
}

static inline void brent_accept(brent_t *z, double fb)
{
    z->fb = fb;
    if (fb == 0.0) {
        z->exact = 1;
        return;
    }
    brent_fix_bracket(z);
}

#endif
