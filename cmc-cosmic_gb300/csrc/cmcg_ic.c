/*
 * cmcg_ic.c -- seeded synthetic star clusters in CMC's N-body units.
 *
 * The reference reads its initial models from HDF5 files written by COSMIC's
 * sampler or by its own src/utils generators.  Neither HDF5 nor COSMIC is
 * available here, so this file generates the same kinds of models from the
 * formulas of the reference's in-tree generators:
 *   Plummer sphere       src/utils/mkplummer/mkplummer.c:63-106 (M(r)), 151-170
 *                        (von Neumann speeds on q^2 (1-q^2)^{7/2}), 234-274 (scaling)
 *   King model (W0)      src/utils/mkking/mkking.c:61-88 (ODE), 330-394 (RKF45),
 *                        398-443 (radii), 446-465 (speeds), 105-150 (scaling)
 *   Kroupa 2001 IMF      two power-law segments, slope 1.3 on [0.08, 0.5] and
 *                        2.3 on [0.5, 150] Msun (src/utils/setimf/genimf.c:23-111)
 * Radii are drawn as sorted uniforms pushed through the mass profile (as both
 * generators do), masses independently of radius, and the model is scaled to
 * N-body units (G = M = 1, E = -1/4) with the generators' own energy sums.
 * Random numbers come from xoshiro256** seeded by SplitMix64 (Blackman and
 * Vigna), so a seed names one model on every host.
 */
#include "cmcgpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    uint64_t s[4];
} xo256;

static uint64_t splitmix64(uint64_t *x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void xo_seed(xo256 *g, uint64_t seed)
{
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) g->s[i] = splitmix64(&x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t xo_next(xo256 *g)
{
    uint64_t *s = g->s;
    uint64_t result = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
}

/* uniform in (0,1): 53 random bits, never exactly 0 */
static double xo_unif(xo256 *g) { return ((xo_next(g) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

uint64_t cmcg_derive_seed(uint64_t master, uint64_t index)
{
    uint64_t x = master ^ (0xD1B54A32D192ED03ull * (index + 1));
    splitmix64(&x);
    return splitmix64(&x);
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* Kroupa (2001) two-segment IMF, dN/dm ~ m^-1.3 on [0.08,0.5], m^-2.3 on [0.5,150],
 * continuous at 0.5.  Inverse-CDF sampling within the chosen segment. */
static double kroupa_draw(xo256 *g)
{
    const double m0 = 0.08, m1 = 0.5, m2 = 150.0, a1 = 1.3, a2 = 2.3;
    /* segment normalisations with continuity: k2 = k1 * m1^(a2-a1) */
    const double k1 = 1.0, k2 = pow(m1, a2 - a1);
    const double w1 = k1 * (pow(m1, 1.0 - a1) - pow(m0, 1.0 - a1)) / (1.0 - a1);
    const double w2 = k2 * (pow(m2, 1.0 - a2) - pow(m1, 1.0 - a2)) / (1.0 - a2);
    double u = xo_unif(g) * (w1 + w2), v = xo_unif(g);
    if (u < w1) {
        double lo = pow(m0, 1.0 - a1), hi = pow(m1, 1.0 - a1);
        return pow(lo + v * (hi - lo), 1.0 / (1.0 - a1));
    }
    double lo = pow(m1, 1.0 - a2), hi = pow(m2, 1.0 - a2);
    return pow(lo + v * (hi - lo), 1.0 / (1.0 - a2));
}

/* mkplummer.c / mkking.c scale_pos_and_vel: PE from the sorted-shell recursion,
 * r *= -2 PE, v *= 1/sqrt(4 KE), which gives PE = -1/2, KE = 1/4. */
static void scale_to_nbody(long N, double *r, const double *m, double *vr, double *vt, double *rfac_out)
{
    double PE = 0.0, KE = 0.0, U = 0.0, MM = 1.0;
    for (long i = N - 1; i >= 0; i--) {
        double rnext = (i + 1 < N) ? r[i + 1] : INFINITY;
        U -= MM * (1.0 / r[i] - 1.0 / rnext);
        double T = 0.5 * (vr[i] * vr[i] + vt[i] * vt[i]);
        MM -= m[i];
        PE += 0.5 * U * m[i];
        KE += T * m[i];
    }
    double rfac = -PE * 2.0, vfac = 1.0 / sqrt(4.0 * KE);
    for (long i = 0; i < N; i++) {
        r[i] *= rfac;
        vr[i] *= vfac;
        vt[i] *= vfac;
    }
    if (rfac_out) *rfac_out = rfac;
}

/* Masses: equal (imf = 0) or Kroupa (imf = 1), with a fraction of composite
 * binaries (m = m1 + m2); normalised to unit total mass. */
static void draw_masses(xo256 *g, long N, int imf, double binary_fraction, double *m)
{
    double tot = 0.0;
    for (long i = 0; i < N; i++) {
        double mi = imf ? kroupa_draw(g) : 1.0;
        if (binary_fraction > 0.0 && xo_unif(g) < binary_fraction) mi += imf ? kroupa_draw(g) : 1.0;
        m[i] = mi;
        tot += mi;
    }
    if (!imf && binary_fraction <= 0.0) {
        for (long i = 0; i < N; i++) m[i] = 1.0 / (double)N;
        return;
    }
    for (long i = 0; i < N; i++) m[i] /= tot;
}

static void sorted_uniforms(xo256 *g, long N, double lo, double hi, double *X)
{
    for (long i = 0; i < N; i++) X[i] = lo + (hi - lo) * xo_unif(g);
    qsort(X, (size_t)N, sizeof(double), cmp_double);
    /* no duplicates: a repeated value would give two stars the same radius */
    for (long i = 1; i < N; i++)
        if (X[i] <= X[i - 1]) X[i] = nextafter(X[i - 1], 2.0);
}

static int plummer(const cmcg_ic_spec *spec, cmcg_ic *out)
{
    const long N = spec->N;
    xo256 g;
    xo_seed(&g, spec->seed);
    /* r_max = 300 Plummer radii before scaling; M(r) = r^3 (1+r^2)^-3/2 */
    const double rmax = 300.0;
    const double Mmax = rmax * rmax * rmax * pow(1.0 + rmax * rmax, -1.5);
    sorted_uniforms(&g, N, 0.0, Mmax, out->r);
    for (long i = 0; i < N; i++) {
        double u = out->r[i];
        out->r[i] = 1.0 / sqrt(pow(u, -2.0 / 3.0) - 1.0); /* inverse of M(r) */
    }
    for (long i = 0; i < N; i++) {
        double r = out->r[i], vesc = sqrt(2.0 / sqrt(1.0 + r * r)), q, gq;
        do {
            double X1 = xo_unif(&g), X2 = xo_unif(&g);
            q = X1;
            gq = q * q * pow(1.0 - q * q, 3.5);
            if (!(0.1 * X2 > gq)) break;
        } while (1);
        double v = q * vesc, X3 = xo_unif(&g);
        out->vr[i] = (1.0 - 2.0 * X3) * v;
        out->vt[i] = sqrt(v * v - out->vr[i] * out->vr[i]);
    }
    draw_masses(&g, N, spec->imf, spec->binary_fraction, out->m);
    scale_to_nbody(N, out->r, out->m, out->vr, out->vt, NULL);
    out->rtid = 1.0e6; /* mkplummer.c:212 */
    return 0;
}

/* King (1966) model: x = Psi/sigma^2 as a function of t = r/r0 from
 * x'' = -9 rho(x)/rho(W0) - 2 x'/t, rho(x) = e^x erf(sqrt x) - sqrt(4x/pi)(1+2x/3). */
static double king_rho(double x)
{
    if (x <= 0.0) return 0.0;
    return exp(x) * erf(sqrt(x)) - sqrt(4.0 * x / 3.14159265358979323846) * (1.0 + 2.0 * x / 3.0);
}

static double king_f1(double t, double x, double y, double rho0)
{
    double res = -9.0 * king_rho(x) / rho0;
    if (fabs(y) < 2.220446049250313e-16 && fabs(t) < 2.220446049250313e-16)
        res /= 3.0;
    else
        res -= 2.0 * y / t;
    return res;
}

static int king(const cmcg_ic_spec *spec, cmcg_ic *out)
{
    const long N = spec->N;
    const double w0 = spec->w0, tol = 1e-10, hmax = 0.01, hmin = 1e-11, rho0 = king_rho(w0);
    xo256 g;
    xo_seed(&g, spec->seed);
    long cap = 4096, n = 0;
    double *pos = malloc(cap * sizeof(double)), *den = malloc(cap * sizeof(double)),
           *pot = malloc(cap * sizeof(double));
    if (!pos || !den || !pot) return -1;
    double t = 0.0, x = w0, y = 0.0, h = tol;
    /* adaptive Runge-Kutta-Fehlberg 4(5), step halving/doubling on the x error */
    while (x > 0 && king_rho(x) / rho0 > 0) {
        if (n >= cap) {
            cap *= 2;
            pos = realloc(pos, cap * sizeof(double));
            den = realloc(den, cap * sizeof(double));
            pot = realloc(pot, cap * sizeof(double));
            if (!pos || !den || !pot) return -1;
        }
        pos[n] = t;
        den[n] = king_rho(x) / rho0;
        pot[n] = x;
        n++;
        double k1 = h * y, l1 = h * king_f1(t, x, y, rho0);
        double x2 = x + k1 / 4, y2 = y + l1 / 4;
        double k2 = h * y2, l2 = h * king_f1(t + h / 4, x2, y2, rho0);
        double x3 = x + 3.0 / 32 * k1 + 9.0 / 32 * k2, y3 = y + 3.0 / 32 * l1 + 9.0 / 32 * l2;
        double k3 = h * y3, l3 = h * king_f1(t + 3.0 / 8 * h, x3, y3, rho0);
        double x4 = x + 1932.0 / 2197 * k1 - 7200.0 / 2197 * k2 + 7296.0 / 2197 * k3;
        double y4 = y + 1932.0 / 2197 * l1 - 7200.0 / 2197 * l2 + 7296.0 / 2197 * l3;
        double k4 = h * y4, l4 = h * king_f1(t + 12.0 / 13 * h, x4, y4, rho0);
        double x5 = x + 439.0 / 216 * k1 - 8.0 * k2 + 3680.0 / 513 * k3 - 845.0 / 4104 * k4;
        double y5 = y + 439.0 / 216 * l1 - 8.0 * l2 + 3680.0 / 513 * l3 - 845.0 / 4104 * l4;
        double k5 = h * y5, l5 = h * king_f1(t + h, x5, y5, rho0);
        double x6 = x - 8.0 / 27 * k1 + 2.0 * k2 - 3544.0 / 2565 * k3 + 1859.0 / 4104 * k4 - 11.0 / 40 * k5;
        double y6 = y - 8.0 / 27 * l1 + 2.0 * l2 - 3544.0 / 2565 * l3 + 1859.0 / 4104 * l4 - 11.0 / 40 * l5;
        double k6 = h * y6, l6 = h * king_f1(t + h / 2, x6, y6, rho0);
        (void)l6;
        double err = 1.0 / 360 * k1 - 128.0 / 4275 * k3 - 2197.0 / 75240 * k4 + 1.0 / 50 * k5 + 2.0 / 55 * k6;
        if (isnan(k2 + k3 + k4 + k5 + k6) && h > hmin) {
            h *= 0.5;
            n--;
            continue;
        }
        if (err > tol && h > hmin) {
            h *= 0.5;
            n--;
            continue;
        }
        x += 25.0 / 216 * k1 + 1408.0 / 2565 * k3 + 2197.0 / 4104 * k4 - 1.0 / 5 * k5;
        y += 25.0 / 216 * l1 + 1408.0 / 2565 * l3 + 2197.0 / 4104 * l4 - 1.0 / 5 * l5;
        t += h;
        if (err < tol / 2 && h < hmax / 2) h *= 2.0;
    }
    if (n < 3) return -1;
    double rt = pos[n - 1];
    /* cumulative mass on the tabulated radii (trapezoid in rho r^2) */
    double *mR = malloc(n * sizeof(double));
    if (!mR) return -1;
    mR[0] = 0.0;
    for (long i = 1; i < n; i++)
        mR[i] = mR[i - 1] + (pos[i] - pos[i - 1]) * (den[i] * pos[i] * pos[i] + den[i - 1] * pos[i - 1] * pos[i - 1]) / 2.0;
    for (long i = 0; i < n; i++) mR[i] /= mR[n - 1];
    double *psi = malloc(N * sizeof(double));
    if (!psi) return -1;
    sorted_uniforms(&g, N, 0.0, 1.0, out->r);
    for (long i = 0; i < N; i++) {
        double X = out->r[i];
        long jmin = 0, jmax = n - 2;
        while (jmin != jmax) {
            long jtry = (jmin + jmax + 1) / 2;
            if (mR[jtry] > X)
                jmax = jtry - 1;
            else
                jmin = jtry;
        }
        double f = (X - mR[jmin]) / (mR[jmin + 1] - mR[jmin]);
        out->r[i] = pos[jmin] + (pos[jmin + 1] - pos[jmin]) * f;
        psi[i] = pot[jmin] + (pot[jmin + 1] - pot[jmin]) * f;
        if (out->r[i] <= 0.0) out->r[i] = 1e-12 * (i + 1);
        if (psi[i] < 0.0) psi[i] = 0.0;
    }
    for (long i = 1; i < N; i++)
        if (out->r[i] <= out->r[i - 1]) out->r[i] = nextafter(out->r[i - 1], INFINITY);
    /* speeds: rejection on the lowered-isothermal DF, f(v) ~ (e^{psi - v^2/2} - 1) v^2 */
    for (long i = 0; i < N; i++) {
        double ps = psi[i], F = (exp(ps) - 1.0) * 2.0 * ps, v0 = 0.0;
        if (ps > 0.0) {
            for (int it = 0; it < 100000; it++) {
                double X1 = xo_unif(&g), X2 = xo_unif(&g);
                v0 = X1 * sqrt(2.0 * ps);
                double f0 = X2 * F, fv = (exp(ps - v0 * v0 / 2.0) - 1.0) * v0 * v0;
                if (!(f0 > fv)) break;
            }
        }
        double X3 = xo_unif(&g);
        out->vr[i] = (1.0 - 2.0 * X3) * v0;
        out->vt[i] = sqrt(fmax(v0 * v0 - out->vr[i] * out->vr[i], 0.0));
        if (out->vt[i] == 0.0 && out->vr[i] == 0.0) out->vt[i] = 1e-6;
    }
    draw_masses(&g, N, spec->imf, spec->binary_fraction, out->m);
    double rfac;
    scale_to_nbody(N, out->r, out->m, out->vr, out->vt, &rfac);
    out->rtid = rt * rfac;
    free(pos);
    free(den);
    free(pot);
    free(mR);
    free(psi);
    return 0;
}

int cmcg_ic_generate(const cmcg_ic_spec *spec, cmcg_ic *out)
{
    if (!spec || !out || spec->N < 2 || !out->r || !out->m || !out->vr || !out->vt) return CMCG_ERR_ARG;
    int rc = (spec->model == CMCG_MODEL_KING) ? king(spec, out) : plummer(spec, out);
    if (rc) return CMCG_ERR_ARG;
    if (out->id)
        for (long i = 0; i < spec->N; i++) out->id[i] = i + 1;
    return CMCG_OK;
}
