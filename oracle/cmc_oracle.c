/*
 * cmc_oracle.c -- CPU oracle for the CMC Henon step (TEST INFRASTRUCTURE ONLY).
 *
 * A single-rank restatement of the reference's plain-dynamics step.  Each
 * function names the reference function and file:line it follows; operation
 * order, `long double` usage and branch structure are kept so that results can
 * be compared with the GPU kernels bit for bit where the arithmetic is IEEE
 * basic operations (+ - * / sqrt) and within stated tolerances elsewhere.
 * Build with -O2 -ffp-contract=off -fno-fast-math.
 *
 * Scope: the branches reachable with PERTURB=RELAXATION=1 and BINBIN =
 * BINSINGLE = SS_COLLISION = STELLAR_EVOLUTION = THREEBODYBINARIES = 0,
 * no search grid, no central black hole loss cone.
 */
#include "cmc_oracle.h"

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include "brent1973.h"
#include "philox.h"

/* include/cmc/cmc.h:58-64 */
#define SF_INFINITY 1.0e10
#define ZERO 1.0e-20
#define PI 3.14159265358979323

struct ostar {
    double r, m, vr, vt, E, J;
    double rnew, vrnew, vtnew, rOld;
    double X, Y, r_peri, r_apo;
    double vrold, vtold, Uoldrold, Uoldrnew, EI;
    int64_t id;
    int interacted;
};

struct ocmc_state {
    ocmc_params P;
    long cap;
    struct ostar *star;               /* 0 .. cap+1 */
    double *star_r, *star_m, *star_phi;
    double *sigma_r, *sigma;
    long sigma_n;
    long N_STAR, N_MAX, N_MAX_NEW;
    double Mtotal, Rtidal, orbit_r, madhoc;
    double cenma_m, cenma_m_new, cenma_E, cenma_E_new;
    double Dt, Prev_Dt, TotalTime, max_r;
    double TidalMassLoss, TidalMassLoss_old, OldTidalMassLoss, DTidalMassLoss;
    double Eescaped, Jescaped, Eintescaped, Ebescaped, Etidal, Eoops;
    double Eescaped_old, Jescaped_old, Eintescaped_old, Ebescaped_old, Etidal_old;
    double Etot, KE, PE, Etot_ini;
    long tcount;
    long Nrel, Nrelbeta[4];
    long n_root_vr; /* find_root_vr calls: apsides outside the closed form's interval */
    double qaverelbeta[4], maverelbeta[4], raverelbeta[4];
    uint32_t taus[4];
    int err;
    long err_index;
};

static double sqr(double x) { return x * x; }       /* cmc_utils.c:27 */
static double cub(double x) { return x * x * x; }   /* cmc_utils.c:39 */
#define OMIN(a, b) ((a) <= (b) ? (a) : (b))          /* cmc.h:2242 */
#define OMAX(a, b) ((a) >= (b) ? (a) : (b))          /* cmc.h:2241 */

static int fail(ocmc_state *s, int code, long idx)
{
    if (!s->err) {
        s->err = code;
        s->err_index = idx;
    }
    return code;
}

/* ---------------------------------------------------------------- RNG ---- */

/* Philox4x32-10: philox.h */
void ocmc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    philox4x32_10(ctr_in, key_in, out);
}

/* taus113 (L'Ecuyer 1999), seeding by the 69069 LCG with minimum-bit fixes and
 * ten warm-up draws, as src/libs/taus113-v2.c:196-215 does. */
static uint32_t lcg69069(uint32_t n) { return (uint32_t)(69069u * n); }

void ocmc_taus113_seed(uint32_t z[4], unsigned long s)
{
    uint32_t s32 = (uint32_t)s;
    if (s32 == 0) s32 = 1u;
    z[0] = lcg69069(s32);
    if (z[0] < 2u) z[0] += 2u;
    z[1] = lcg69069(z[0]);
    if (z[1] < 8u) z[1] += 8u;
    z[2] = lcg69069(z[1]);
    if (z[2] < 16u) z[2] += 16u;
    z[3] = lcg69069(z[2]);
    if (z[3] < 128u) z[3] += 128u;
    for (int i = 0; i < 10; ++i) ocmc_taus113_next(z);
}

uint32_t ocmc_taus113_next(uint32_t z[4])
{
    uint32_t b;
    b = ((z[0] << 6) ^ z[0]) >> 13;
    z[0] = ((z[0] & 4294967294u) << 18) ^ b;
    b = ((z[1] << 2) ^ z[1]) >> 27;
    z[1] = ((z[1] & 4294967288u) << 2) ^ b;
    b = ((z[2] << 13) ^ z[2]) >> 21;
    z[2] = ((z[2] & 4294967280u) << 7) ^ b;
    b = ((z[3] << 3) ^ z[3]) >> 12;
    z[3] = ((z[3] & 4294967168u) << 13) ^ b;
    return z[0] ^ z[1] ^ z[2] ^ z[3];
}

/* Counter-draw keying: key = (seed lo, seed hi ^ tcount), ctr = (id lo, id hi,
 * site, n).  Returns word `word` of the Philox block scaled by 2^-32, the same
 * 32-bit resolution as rng_t113_dbl_new (taus113-v2.c:186). */
double ocmc_draw(const ocmc_state *s, int site, int64_t id, uint32_t n, int word)
{
    if (s->P.draw_mode == OCMC_DRAW_TAUS113) {
        return ocmc_taus113_next(((ocmc_state *)s)->taus) / 4294967296.0;
    }
    uint32_t key[2] = {(uint32_t)s->P.seed, (uint32_t)(s->P.seed >> 32) ^ (uint32_t)s->tcount};
    uint64_t uid = (uint64_t)id;
    uint32_t ctr[4] = {(uint32_t)uid, (uint32_t)(uid >> 32), (uint32_t)site, n};
    uint32_t out[4];
    ocmc_philox4x32_10(ctr, key, out);
    return out[word & 3] / 4294967296.0;
}

/* ---------------------------------------------------------- lifecycle ---- */

void ocmc_default_params(ocmc_params *p)
{
    memset(p, 0, sizeof(*p));
    p->N_STAR = 0;
    p->AVEKERNEL = 20;                /* cmc_io.c:1749 */
    p->GAMMA = 0.1;                   /* examples/PlummerSphere.ini */
    p->THETASEMAX = 1.412;            /* cmc_io.c:1671 */
    p->PERTURB = 1;
    p->RELAXATION = 1;
    p->TIDALLY_STRIP_STARS = 1;
    p->TIDAL_TREATMENT = 1;
    p->orbit_r = 1.0e6;
    p->cenma_m = 0.0;
    p->apsides_max_iter = 100;        /* cmc_io.c:1753 */
    p->apsides_precision = 1.0e-11;   /* cmc_io.c:1752 */
    p->apsides_convergence = 5.0e-13; /* cmc_io.c:1754 */
    p->n_try = 50000;                 /* cmc.h:64 */
    p->seed = 0;
    p->draw_mode = OCMC_DRAW_COUNTER;
}

ocmc_state *ocmc_create(const ocmc_params *p, long N, const double *r, const double *m,
                        const double *vr, const double *vt, const int64_t *id)
{
    if (N < 2 * p->AVEKERNEL + 2) return NULL;
    ocmc_state *s = (ocmc_state *)calloc(1, sizeof(*s));
    if (!s) return NULL;
    s->P = *p;
    s->cap = N;
    s->star = (struct ostar *)calloc((size_t)N + 2, sizeof(struct ostar));
    s->star_r = (double *)calloc((size_t)N + 3, sizeof(double));
    s->star_m = (double *)calloc((size_t)N + 3, sizeof(double));
    s->star_phi = (double *)calloc((size_t)N + 3, sizeof(double));
    s->sigma_r = (double *)calloc((size_t)N + 2, sizeof(double));
    s->sigma = (double *)calloc((size_t)N + 2, sizeof(double));
    if (!s->star || !s->star_r || !s->star_m || !s->star_phi || !s->sigma_r || !s->sigma) {
        ocmc_destroy(s);
        return NULL;
    }
    s->N_STAR = p->N_STAR > 0 ? p->N_STAR : N;
    /* cmc_fits.c:98-136: masses stored x N_STAR, sentinels r[0]=ZERO, r[N+1]=inf */
    for (long i = 1; i <= N; ++i) {
        struct ostar *st = &s->star[i];
        st->m = m[i - 1] * ((double)s->N_STAR);
        st->r = r[i - 1];
        st->vr = vr[i - 1];
        st->vt = vt[i - 1];
        st->id = id ? id[i - 1] : (int64_t)i;
        s->star_m[i] = st->m;
        s->star_r[i] = st->r;
    }
    s->star_r[0] = ZERO;
    s->star_r[N + 1] = SF_INFINITY;
    s->Mtotal = 1.0;
    s->cenma_m = p->cenma_m;
    s->star_m[0] = 0.0;
    s->N_MAX = N;
    s->N_MAX_NEW = N;
    s->orbit_r = p->orbit_r;
    s->madhoc = 1.0 / ((double)s->N_STAR); /* cmc_utils.c:1183 */
    s->tcount = 1;
    ocmc_taus113_seed(s->taus, (unsigned long)p->seed);
    return s;
}

void ocmc_destroy(ocmc_state *s)
{
    if (!s) return;
    free(s->star);
    free(s->star_r);
    free(s->star_m);
    free(s->star_phi);
    free(s->sigma_r);
    free(s->sigma);
    free(s);
}

/* ------------------------------------------------------ potential ------- */

/* potential_calculate, cmc_utils.c:675-736 */
int ocmc_calc_potential(ocmc_state *s)
{
    long k = 1;
    double mprev = 0.0;
    while (s->star_r[k] < SF_INFINITY && k <= s->N_MAX) {
        mprev += s->star_m[k];
        if (isnan(mprev)) return fail(s, OCMC_ERR_NAN_MASS, k);
        k++;
    }
    s->N_MAX = k - 1;
    s->cenma_m += s->cenma_m_new;
    s->cenma_m_new = 0.0;
    s->Mtotal = mprev * s->madhoc + s->cenma_m * s->madhoc;
    s->Rtidal = s->orbit_r * pow(s->Mtotal, 1.0 / 3.0);
    s->star_r[s->N_MAX + 1] = SF_INFINITY;
    s->star_phi[s->N_MAX + 1] = 0.0;
    mprev = s->Mtotal;
    for (k = s->N_MAX; k >= 1; k--) {
        s->star_phi[k] = s->star_phi[k + 1] - mprev * (1.0 / s->star_r[k] - 1.0 / s->star_r[k + 1]);
        mprev -= s->star_m[k] / s->N_STAR;
        if (isnan(s->star_phi[k])) return fail(s, OCMC_ERR_NAN_PHI, k);
    }
    s->star_phi[0] = s->star_phi[1] + s->cenma_m * s->madhoc / s->star_r[1];
    if (isnan(s->star_phi[0])) return fail(s, OCMC_ERR_NAN_PHI, 0);
    return OCMC_OK;
}

/* FindZero_r, cmc_nr.c:62-82 */
static long find_zero_r(const ocmc_state *s, long kmin, long kmax, double r)
{
    long ktry;
    do {
        ktry = (kmin + kmax + 1) / 2;
        if (s->star_r[ktry] < r) {
            kmin = ktry;
        } else {
            kmax = ktry - 1;
        }
    } while (kmax != kmin);
    return kmin;
}

/* potential, cmc_utils.c:112-164 (SEARCH_GRID = 0) */
static double potential_checked(ocmc_state *s, double r, int *ok)
{
    long i, kmax, kmin;
    *ok = 1;
    if (r == 0.0) return s->star_phi[0];
    if (r < s->star_r[1]) return s->star_phi[0] - (s->star_phi[0] - s->star_phi[1]) * s->star_r[1] / r;
    kmax = s->N_MAX + 1;
    kmin = 1;
    if (kmin == kmax - 1) {
        i = kmin;
    } else {
        i = find_zero_r(s, kmin, kmax, r);
    }
    if (s->star_r[i] > r || s->star_r[i + 1] < r) {
        *ok = 0;
        fail(s, OCMC_ERR_FINDZERO_R, i);
        return 0.0;
    }
    if (i == 0) return s->star_phi[1];
    return s->star_phi[i] + (s->star_phi[i + 1] - s->star_phi[i]) * (1.0 / s->star_r[i] - 1.0 / r) /
                                (1.0 / s->star_r[i] - 1.0 / s->star_r[i + 1]);
}

double ocmc_potential(ocmc_state *s, double r)
{
    int ok;
    return potential_checked(s, r, &ok);
}

/* MPI_PHI_S, cmc.h:2175: self-potential correction of star j at radius rad */
static double phi_s(const ocmc_state *s, double rad, long j)
{
    return (rad >= s->star_r[j] ? s->star_m[j] / rad : s->star_m[j] / s->star_r[j]) * (1.0 / s->N_STAR);
}

/* ---------------------------------------------------------- time step --- */

/* calc_n_local, cmc_dynamics_helper.c:768-786 */
static double calc_n_local(const ocmc_state *s, long k, long p, long N_LIMIT)
{
    long kmin = k - p, kmax = k + p;
    if (kmin < 0) {
        kmin = 0;
        kmax = 2 * p + 1;
    } else if (kmax > N_LIMIT) {
        kmax = N_LIMIT;
        kmin = N_LIMIT - 2 * p - 1;
    }
    return (2.0 * ((double)p)) * 3.0 / (4.0 * PI * (cub(s->star_r[kmax]) - cub(s->star_r[kmin])));
}

/* simul_relax_new, cmc_dynamics_helper.c:2526-2579 (single rank) */
static double simul_relax_new(ocmc_state *s)
{
    long p = s->P.AVEKERNEL, N = s->N_MAX;
    double dtmin = INFINITY;
    for (long si = 1 + p; si < N + 1 - p; si += 2 * p) {
        long simin = si - p, simax = simin + (2 * p - 1);
        double Mv2ave = 0.0, Mave = 0.0, M2ave = 0.0;
        for (long k = simin; k <= simax; k++) {
            double tmp = s->star_m[k] * s->madhoc;
            Mv2ave += tmp * (sqr(s->star[k].vr) + sqr(s->star[k].vt));
            Mave += tmp;
            M2ave += sqr(tmp);
        }
        Mv2ave /= (double)(2 * p);
        Mave /= (double)(2 * p);
        M2ave /= (double)(2 * p);
        double sigma = sqrt(Mv2ave / Mave);
        double W = 4.0 * sigma / sqrt(3.0 * PI);
        double n_local = calc_n_local(s, si, p, s->N_MAX);
        double dt = sqr(2.0 * s->P.THETASEMAX / PI) * (PI / 32.0) * cub(W) /
                    (((double)s->N_STAR) * n_local * (4.0 * M2ave));
        dtmin = OMIN(dtmin, dt);
    }
    return dtmin;
}

/* calc_timestep, cmc_utils.c:2132-2148 with GetTimeStep, cmc_evolution_thr.c:317-438
 * reduced to the relaxation term (collisions, binaries, SE and aging are off). */
int ocmc_calc_timestep(ocmc_state *s)
{
    double Dt = (s->P.RELAXATION) ? simul_relax_new(s) : INFINITY;
    if (isinf(Dt)) Dt = 0.001;
    if ((s->TidalMassLoss_old - s->OldTidalMassLoss) > 0.01) {
        Dt = s->Prev_Dt * 0.8;
    } else if (Dt > 1.1 * s->Prev_Dt && s->Prev_Dt > 0 && (s->TidalMassLoss - s->OldTidalMassLoss) > 0.02) {
        Dt = s->Prev_Dt * 1.1;
    }
    s->Dt = Dt;
    s->TotalTime += Dt;
    return OCMC_OK;
}

/* ---------------------------------------------------------- relaxation -- */

/* calc_sigma_r, cmc_dynamics_helper.c:2821-2986, single rank (no ghosts used) */
static void calc_sigma_r(ocmc_state *s, long p, long N_LIMIT)
{
    long siminlast = 1, simaxlast = 0, simin, simax;
    double Mv2ave = 0.0, Mave = 0.0;
    s->sigma_n = N_LIMIT;
    for (long si = 1; si <= N_LIMIT; si++) {
        simin = si - p;
        simax = simin + (2 * p - 1);
        if (simin < 1) {
            simin = 1;
            simax = simin + (2 * p - 1);
        } else if (simax > s->N_MAX) {
            simax = N_LIMIT;
            simin = simax - (2 * p - 1);
        }
        for (long k = siminlast; k < simin; k++) {
            double vr = s->star[k].vr, vt = s->star[k].vt;
            Mv2ave -= s->star_m[k] * s->madhoc * (sqr(vr) + sqr(vt));
            Mave -= s->star_m[k] * s->madhoc;
        }
        for (long k = simaxlast + 1; k <= simax; k++) {
            double vr = s->star[k].vr, vt = s->star[k].vt;
            Mv2ave += s->star_m[k] * s->madhoc * (sqr(vr) + sqr(vt));
            Mave += s->star_m[k] * s->madhoc;
        }
        s->sigma_r[si] = s->star_r[si];
        s->sigma[si] = sqrt(Mv2ave / Mave);
        siminlast = simin;
        simaxlast = simax;
    }
}

/* set_star_EJ, cmc_dynamics_helper.c:878-882 */
static void set_star_EJ(ocmc_state *s, long k)
{
    s->star[k].E = s->star_phi[k] + 0.5 * (sqr(s->star[k].vr) + sqr(s->star[k].vt));
    s->star[k].J = s->star_r[k] * s->star[k].vt;
}

/* dynamics_apply, cmc_dynamics.c:17-542: the two-body relaxation branch with the
 * encounter dyns of cmc_dynamics_helper.c:831-871. */
int ocmc_dynamics_apply(ocmc_state *s, double dt)
{
    const long p = s->P.AVEKERNEL;
    const long N = s->N_MAX; /* mpiEnd - mpiBegin + 1 */
    const double relbeta[4] = {PI / 2.0, PI / 4.0, PI / 8.0, PI / 16.0};
    double SaveDt = dt;

    calc_sigma_r(s, p, N);

    s->Nrel = 0;
    for (int i = 0; i < 4; i++) {
        s->Nrelbeta[i] = 0;
        s->qaverelbeta[i] = s->maverelbeta[i] = s->raverelbeta[i] = 0.0;
    }
    const long N_LIMIT = s->N_MAX;
    long si = 1;
    while (si <= N - N % 2 - 1) {
        double v[4], vp[4], w[4], W, rcm, vcm[4], n_local, mass_k, mass_kp, S, P_enc;
        dt = SaveDt;
        long k = si, kp = si + 1;
        si += 2;
        struct ostar *sk = &s->star[k], *skp = &s->star[kp];

        /* calc_encounter_dyns, cmc_dynamics_helper.c:831-871 */
        sk->Y = ocmc_draw(s, OCMC_SITE_Y, sk->id, 0, 0);
        skp->Y = sk->Y;
        double phi = sk->Y * 2.0 * PI;
        v[1] = sk->vt;
        v[2] = 0.0;
        v[3] = sk->vr;
        vp[1] = skp->vt * cos(phi);
        vp[2] = skp->vt * sin(phi);
        vp[3] = skp->vr;
        for (int j = 1; j <= 3; j++) w[j] = vp[j] - v[j];
        W = sqrt(sqr(w[1]) + sqr(w[2]) + sqr(w[3]));
        if (W == 0.0) return fail(s, OCMC_ERR_W_ZERO, k);
        rcm = (s->star_m[k] * s->star_r[k] + s->star_m[kp] * s->star_r[kp]) / (s->star_m[k] + s->star_m[kp]);
        for (int j = 1; j <= 3; j++)
            vcm[j] = (s->star_m[k] * v[j] + s->star_m[kp] * vp[j]) / (s->star_m[k] + s->star_m[kp]);
        (void)vcm;

        n_local = calc_n_local(s, k, p, N_LIMIT);
        mass_k = s->star_m[k];
        mass_kp = s->star_m[kp];
        S = 0.0; /* single-single with SS_COLLISION = 0 (cmc_dynamics.c:392-394) */
        P_enc = n_local * W * S * (dt * ((double)s->N_STAR) / log(s->P.GAMMA * ((double)s->N_STAR)));

        if (ocmc_draw(s, OCMC_SITE_PENC, sk->id, 0, 0) < P_enc) {
            /* strong encounter branch: host-only physics, unreachable with S = 0 */
            continue;
        } else if (s->P.RELAXATION) {
            double Trel12, beta, wp, w1[4], w2[4], psi, w_new[4], v_new[4], vp_new[4];
            Trel12 = (PI / 32.0) * cub(W) / (((double)s->N_STAR) * n_local * sqr((mass_k + mass_kp) * s->madhoc));
            beta = (PI / 2.0) * sqrt(dt / Trel12);
            s->Nrel++;
            for (int i = 0; i < 4; i++) {
                if (beta > relbeta[i]) {
                    s->Nrelbeta[i]++;
                    s->qaverelbeta[i] += OMAX(mass_k, mass_kp) / OMIN(mass_k, mass_kp);
                    s->maverelbeta[i] += (mass_k + mass_kp) / 2.0;
                    s->raverelbeta[i] += rcm;
                }
            }
            if (beta > PI / 2.0) beta = PI / 2.0;
            wp = sqrt(sqr(w[1]) + sqr(w[2]));
            if (wp == 0.0) return fail(s, OCMC_ERR_WP_ZERO, k);
            w1[1] = -w[2] * W / wp;
            w1[2] = w[1] * W / wp;
            w1[3] = 0.0;
            w2[1] = -w[1] * w[3] / wp;
            w2[2] = -w[2] * w[3] / wp;
            w2[3] = wp;
            psi = ocmc_draw(s, OCMC_SITE_PSI, sk->id, 0, 0) * 2 * PI;
            for (int j = 1; j <= 3; j++)
                w_new[j] = w[j] * cos(beta) + w1[j] * sin(beta) * cos(psi) + w2[j] * sin(beta) * sin(psi);
            for (int j = 1; j <= 3; j++) {
                v_new[j] = v[j] - mass_kp / (mass_k + mass_kp) * (w_new[j] - w[j]);
                vp_new[j] = vp[j] + mass_k / (mass_k + mass_kp) * (w_new[j] - w[j]);
            }
            sk->vr = v_new[3];
            sk->vt = sqrt(sqr(v_new[1]) + sqr(v_new[2]));
            skp->vr = vp_new[3];
            skp->vt = sqrt(sqr(vp_new[1]) + sqr(vp_new[2]));
            set_star_EJ(s, k);
            set_star_EJ(s, kp);
        }
    }
    return OCMC_OK;
}

/* energy_conservation1, cmc_utils.c:2153-2174 */
int ocmc_energy_conservation1(ocmc_state *s)
{
    for (long i = 1; i <= s->N_MAX_NEW; i++) {
        s->star[i].vtold = s->star[i].vt;
        s->star[i].vrold = s->star[i].vr;
        s->star[i].Uoldrold = s->star_phi[i] + phi_s(s, s->star_r[i], i);
    }
    return OCMC_OK;
}

/* ------------------------------------------------------------ orbits ---- */

/* zero_star + destroy_obj + remove_star_center, cmc_dynamics_helper.c:19-73,131-150;
 * cmc_evolution_thr.c:766-771 */
static void destroy_obj(ocmc_state *s, long i)
{
    double r = s->star_r[i], phi = s->star_phi[i];
    struct ostar *st = &s->star[i];
    memset(st, 0, sizeof(*st));
    s->star_r[i] = r;
    s->star_phi[i] = phi;
    st->rnew = SF_INFINITY;
    s->star_m[i] = DBL_MIN;
    st->vrnew = 0.0;
    st->vtnew = 0.0;
}

/* remove_star, cmc_evolution_thr.c:655-716 (logging omitted) */
static void remove_star(ocmc_state *s, long j)
{
    double E = s->star[j].E, J = s->star[j].J, m;
    s->star[j].rnew = SF_INFINITY;
    s->star[j].vrnew = 0.0;
    s->star[j].vtnew = 0.0;
    m = s->star_m[j];
    s->Eescaped += E * m / s->N_STAR;
    s->Jescaped += J * m / s->N_STAR;
    s->TidalMassLoss += m / s->N_STAR;
    s->Etidal += E * m / s->N_STAR;
    destroy_obj(s, j);
}

/* function_q, cmc_utils.c:1654-1662.  SQR() stores its argument in a static
 * double (cmc.h:2030-2031), so J/r is rounded to double before squaring. */
static double function_q(const ocmc_state *s, long j, long double r, long double pot, long double E,
                         long double J)
{
    double res;
    long double Jr, phis;
    double sqrarg = (double)((J) / (r));
    Jr = (sqrarg == 0.0 ? 0.0 : sqrarg * sqrarg);
    phis = ((r) >= s->star_r[j] ? s->star_m[j] / (r) : (long double)(s->star_m[j] / s->star_r[j])) *
           (1.0 / s->N_STAR);
    res = (2.0 * ((E) - (pot + phis)) - Jr);
    return res;
}

/* get_positive_Q_index, cmc_orbit.c:30-59 (no new particles on one rank) */
static long get_positive_Q_index(const ocmc_state *s, long index, double E, double J)
{
    long ktemp = index;
    double Qtemp = function_q(s, index, s->star_r[ktemp], s->star_phi[ktemp], E, J);
    if (Qtemp <= 0.0) {
        ktemp = -1;
        do {
            ktemp++;
            Qtemp = function_q(s, index, s->star_r[ktemp], s->star_phi[ktemp], E, J);
        } while (Qtemp <= 0.0 && ktemp <= s->N_MAX);
        if (ktemp >= s->N_MAX) return -1;
    }
    return ktemp;
}

/* find_zero_Q, cmc_nr.c:316-383 */
static long find_zero_Q(const ocmc_state *s, long j, long kmin, long kmax, long double E, long double J)
{
    long ktry;
    long double rmax, pot_max, rmin, pot_min, rtry, pot_try, qmin, qmax, qtry;
    rmax = s->star_r[kmax];
    pot_max = s->star_phi[kmax];
    rmin = s->star_r[kmin];
    pot_min = s->star_phi[kmin];
    qmin = function_q(s, j, rmin, pot_min, E, J);
    qmax = function_q(s, j, rmax, pot_max, E, J);
    if (qmin < qmax) {
        do {
            ktry = (kmin + kmax + 1) / 2;
            rtry = s->star_r[ktry];
            pot_try = s->star_phi[ktry];
            qtry = function_q(s, j, rtry, pot_try, E, J);
            if (qtry < 0.e0) {
                kmin = ktry;
            } else {
                kmax = ktry - 1;
            }
        } while (kmax != kmin);
    } else {
        do {
            ktry = (kmin + kmax + 1) / 2;
            rtry = s->star_r[ktry];
            pot_try = s->star_phi[ktry];
            qtry = function_q(s, j, rtry, pot_try, E, J);
            if (qtry > 0.e0) {
                kmin = ktry;
            } else {
                kmax = ktry - 1;
            }
        } while (kmax != kmin);
    }
    return kmin;
}

/* set_a_b, cmc_orbit.c:722-740 */
static void set_a_b(const ocmc_state *s, long index, long k, double *a, double *b)
{
    if (k == 0) {
        *a = -s->cenma_m * s->madhoc;
        *b = s->star_phi[1] + s->cenma_m * s->madhoc / s->star_r[1] + s->star_m[index] * s->madhoc / s->star_r[index];
    } else {
        double rk = s->star_r[k], rk1 = s->star_r[k + 1];
        double Uk = s->star_phi[k] + phi_s(s, rk, index);
        double Uk1 = s->star_phi[k + 1] + phi_s(s, rk1, index);
        *a = (Uk1 - Uk) / (1. / rk1 - 1. / rk);
        *b = (Uk / rk1 - Uk1 / rk) / (1. / rk1 - 1. / rk);
    }
}

/* calc_pot_within_interval, cmc_nr.c:230-259 */
static double calc_pot_within_interval(ocmc_state *s, double r, long k, int *ok)
{
    *ok = 1;
    if (r < (s->star_r[k] - DBL_EPSILON) || r > s->star_r[k + 1] + DBL_EPSILON) {
        *ok = 0;
        fail(s, OCMC_ERR_POT_INTERVAL, k);
        return 0.0;
    }
    if (fabs(r - s->star_r[k]) < DBL_EPSILON) return s->star_phi[k];
    if (fabs(r - s->star_r[k + 1]) < DBL_EPSILON) return s->star_phi[k + 1];
    if (r < s->star_r[1]) return s->star_phi[0] - s->cenma_m * s->madhoc / r;
    return (s->star_phi[k] + (s->star_phi[k + 1] - s->star_phi[k]) * (1.0 / s->star_r[k] - 1.0 / r) /
                                 (1.0 / s->star_r[k] - 1.0 / s->star_r[k + 1]));
}

/* calc_vr_within_interval, cmc_nr.c:267-278 */
static double vr2_in_interval(ocmc_state *s, double r, long index, long k, double E, double J, int *ok)
{
    double pot = calc_pot_within_interval(s, r, k, ok);
    return function_q(s, index, r, pot, E, J);
}

/* Brent (1973): oracle/brent1973.h */

/* find_root_vr, cmc_nr.c:500-603 */
static double find_root_vr(ocmc_state *s, long index, long k, double E, double J)
{
    s->n_root_vr++;
    const double prec = s->P.apsides_precision, conv = s->P.apsides_convergence;
    int ok = 1, not_converged = 1;
    long iter = s->P.apsides_max_iter;
    double r_low = -1.0, r_high = -1.0, apsis, prev_apsis = -1.0;
    double flo = vr2_in_interval(s, s->star_r[k], index, k, E, J, &ok);
    double fhi = vr2_in_interval(s, s->star_r[k + 1], index, k, E, J, &ok);
    if (!ok) return 0.0;
    /* GSL_SIGN(x) = (x >= 0 ? 1 : -1) */
    if ((flo >= 0.0 ? 1 : -1) == (fhi >= 0.0 ? 1 : -1)) {
        fail(s, OCMC_ERR_ROOT_SIGNS, index);
        return 0.0;
    }
    brent_t z;
    brent_set(&z, flo, fhi, s->star_r[k], s->star_r[k + 1]);
    while (not_converged && iter) {
        double x = brent_propose(&z);
        double fx = vr2_in_interval(s, x, index, k, E, J, &ok);
        if (!ok) return 0.0;
        if (!isfinite(fx)) {
            fail(s, OCMC_ERR_ROOT_NOCONV, index);
            return 0.0;
        }
        brent_accept(&z, fx);
        if (z.exact) {
            r_low = r_high = z.b;
        } else {
            r_low = z.b < z.c ? z.b : z.c;
            r_high = z.b < z.c ? z.c : z.b;
        }
        /* gsl_root_test_interval: |hi - lo| < epsabs + epsrel * min(|lo|, |hi|) */
        not_converged = !(fabs(r_high - r_low) < prec + prec * OMIN(fabs(r_low), fabs(r_high)));
        iter--;
        if (iter < 10) {
            if (prev_apsis < 0.) {
                prev_apsis = z.b;
            } else {
                apsis = z.b;
                /* gsl_root_test_delta: |x1 - x0| < epsabs + epsrel * |x1| */
                not_converged = not_converged && !(fabs(apsis - prev_apsis) < conv + conv * fabs(apsis));
                prev_apsis = apsis;
            }
        }
    }
    if (not_converged) {
        fail(s, OCMC_ERR_ROOT_NOCONV, index);
        return 0.0;
    }
    apsis = z.b;
    if (vr2_in_interval(s, apsis, index, k, E, J, &ok) < 0.) {
        if (vr2_in_interval(s, r_low, index, k, E, J, &ok) < 0.) apsis = r_high;
        if (vr2_in_interval(s, r_high, index, k, E, J, &ok) < 0.) apsis = r_low;
    }
    if (vr2_in_interval(s, apsis, index, k, E, J, &ok) < 0.) {
        fail(s, OCMC_ERR_ROOT_NEG, index);
        return 0.0;
    }
    return apsis;
}

typedef struct {
    double rp, ra, dQdrp, dQdra;
    long kmin, kmax;
    int circular_flag;
} orbit_rs_t;

/* calc_orbit_new, cmc_orbit.c:413-540 */
static orbit_rs_t calc_orbit_new(ocmc_state *s, long index, double E, double J)
{
    orbit_rs_t o;
    long ktemp, kmin, kmax;
    double rmin, rmax, rkmin, rk1min, rkmax, rk1max, a, b, dQdr_min, dQdr_max;
    int circular = 0;

    ktemp = get_positive_Q_index(s, index, E, J);
    if (ktemp <= -1) {
        o.rp = o.ra = s->star_r[index];
        o.kmin = o.kmax = index;
        o.dQdrp = o.dQdra = 0.0;
        o.circular_flag = 1;
        return o;
    }
    kmin = find_zero_Q(s, index, 0, ktemp, E, J);
    kmax = find_zero_Q(s, index, ktemp, s->N_MAX + 1, E, J);
    rkmin = s->star_r[kmin];
    rk1min = s->star_r[kmin + 1];
    rkmax = s->star_r[kmax];
    rk1max = s->star_r[kmax + 1];

    double inside_sqrt;
    set_a_b(s, index, kmin, &a, &b);
    inside_sqrt = a * a - 2.0 * J * J * (b - E);
    if (inside_sqrt < 0.0) {
        rmin = -1.0 * J * J / a;
        if ((rmin < rkmin) || (rmin > rk1min)) rmin = find_root_vr(s, index, kmin, E, J);
    } else {
        rmin = J * J / (-a + sqrt(inside_sqrt));
    }
    dQdr_min = 2.0 * J * J / (rmin * rmin * rmin) + 2.0 * a / (rmin * rmin);

    set_a_b(s, index, kmax, &a, &b);
    inside_sqrt = a * a - 2.0 * J * J * (b - E);
    if (inside_sqrt < 0.0) {
        rmax = -a / (2.0 * (b - E));
        if ((rmax < rkmax) || (rmax > rk1max)) rmax = find_root_vr(s, index, kmax, E, J);
    } else {
        rmax = (-a + sqrt(inside_sqrt)) / (2.0 * (b - E));
    }
    dQdr_max = 2.0 * J * J / (rmax * rmax * rmax) + 2.0 * a / (rmax * rmax);

    if ((rmin > rmax) || (dQdr_min <= 0.) || (dQdr_max >= 0.)) circular = 1;
    if (circular) {
        o.rp = o.ra = s->star_r[index];
        o.kmin = o.kmax = index;
        o.dQdrp = o.dQdra = 0.0;
        o.circular_flag = 1;
    } else {
        o.rp = rmin;
        o.ra = rmax;
        o.kmin = kmin;
        o.kmax = kmax;
        o.dQdrp = dQdr_min;
        o.dQdra = dQdr_max;
        o.circular_flag = 0;
    }
    return o;
}

/* get_positions_loop, cmc_evolution_thr.c:784-937 */
static int get_positions(ocmc_state *s)
{
    double max_rad = 0.0;
    int ok;
    /* get_positions, cmc_evolution_thr.c:963-964 */
    (void)potential_checked(s, s->Rtidal, &ok);
    (void)potential_checked(s, 0.0, &ok);
    for (long si = 1; si <= s->N_MAX_NEW; si++) {
        long j = si, k;
        double E = s->star[j].E + phi_s(s, s->star_r[j], j);
        double J = s->star[j].J;
        double r = 0.0, vr = 0.0, vt, rmin, rmax, g1, g2, F, s0, g0, drds, pot, X = 0.0, Q;
        if (s->star_m[j] < ZERO) {
            destroy_obj(s, j);
            continue;
        }
        if (E >= 0.0) {
            remove_star(s, j);
            continue;
        }
        orbit_rs_t o = calc_orbit_new(s, j, E, J);
        if (s->err) return s->err;
        if (o.circular_flag == 1) {
            s->star[j].rnew = s->star_r[j];
            s->star[j].vrnew = s->star[j].vr;
            s->star[j].vtnew = s->star[j].vt;
            continue;
        }
        rmin = o.rp;
        rmax = o.ra;
        if (rmax >= s->Rtidal) {
            s->star[j].r_apo = rmax;
            s->star[j].r_peri = rmin;
            remove_star(s, j);
            continue;
        }
        g1 = sqrt(3.0 * (rmax - rmin) / o.dQdrp);
        g2 = sqrt(-3.0 * (rmax - rmin) / o.dQdra);
        F = 1.2 * OMAX(g1, g2);
        const int64_t id = s->star[j].id;
        for (k = 1; k <= s->P.n_try; k++) {
            X = ocmc_draw(s, OCMC_SITE_TRIAL, id, (uint32_t)(k - 1), 0);
            s0 = 2.0 * X - 1.0;
            g0 = F * ocmc_draw(s, OCMC_SITE_TRIAL, id, (uint32_t)(k - 1), 1);
            r = 0.5 * (rmin + rmax) + 0.25 * (rmax - rmin) * (3.0 * s0 - s0 * s0 * s0);
            pot = potential_checked(s, r, &ok) + phi_s(s, r, j);
            if (!ok) return s->err;
            drds = 0.25 * (rmax - rmin) * (3.0 - 3.0 * s0 * s0);
            Q = 2.0 * E - 2.0 * pot - J * J / r / r;
            if (Q >= 0.0) {
                vr = sqrt(Q);
            } else {
                if (isnan(Q)) return fail(s, OCMC_ERR_Q_NAN, j);
                vr = 0;
            }
            if (g0 < 1.0 / vr * drds) break;
        }
        if (k == s->P.n_try + 1) return fail(s, OCMC_ERR_NTRY, j);
        s->star[j].X = X;
        s->star[j].r_peri = rmin;
        s->star[j].r_apo = rmax;
        if (ocmc_draw(s, OCMC_SITE_SIGN, id, 0, 0) < 0.5) vr = -vr;
        vt = J / r;
        s->star[j].rnew = r;
        s->star[j].vrnew = vr;
        s->star[j].vtnew = vt;
        if (r > max_rad) max_rad = r;
    }
    s->max_r = max_rad;
    return OCMC_OK;
}

/* new_orbits_calculate, cmc_utils.c:2194-2211 */
int ocmc_new_orbits_calculate(ocmc_state *s)
{
    s->OldTidalMassLoss = s->TidalMassLoss_old;
    int rc = get_positions(s);
    if (rc) return rc;
    s->TidalMassLoss += s->TidalMassLoss_old;
    return OCMC_OK;
}

/* energy_conservation2, cmc_utils.c:2218-2228 */
int ocmc_energy_conservation2(ocmc_state *s)
{
    int ok;
    for (long i = 1; i <= s->N_MAX_NEW; i++) {
        double rn = s->star[i].rnew;
        s->star[i].Uoldrnew = potential_checked(s, rn, &ok) + phi_s(s, rn, i);
        if (!ok) return s->err;
    }
    return OCMC_OK;
}

/* tidally_strip_stars, cmc_evolution_thr.c:443-646 (logging omitted) */
int ocmc_tidally_strip_stars(ocmc_state *s)
{
    if (!s->P.TIDALLY_STRIP_STARS) return OCMC_OK;
    int ok;
    s->Etidal = 0.0;
    s->DTidalMassLoss = s->TidalMassLoss - s->OldTidalMassLoss;
    do {
        s->Rtidal = s->orbit_r * pow(s->Mtotal - (s->TidalMassLoss - s->OldTidalMassLoss), 1.0 / 3.0);
        double phi_rtidal = potential_checked(s, s->Rtidal, &ok);
        (void)potential_checked(s, 0.0, &ok);
        s->DTidalMassLoss = 0.0;
        double gierszalpha = 1.5 - 3.0 * pow(log(s->P.GAMMA * ((double)s->N_STAR)) / ((double)s->N_STAR), 0.25);
        for (long i = 1; i <= s->N_MAX_NEW; i++) {
            double m = s->star_m[i];
            struct ostar *st = &s->star[i];
            int strip;
            if (s->P.TIDAL_TREATMENT == 0)
                strip = (st->r_apo > s->Rtidal && st->rnew < 1000000);
            else
                strip = (st->E > gierszalpha * phi_rtidal && st->rnew < 1000000);
            if (strip) {
                st->rnew = SF_INFINITY;
                st->vrnew = 0.0;
                st->vtnew = 0.0;
                s->Eescaped += st->E * m / s->N_STAR;
                s->Jescaped += st->J * m / s->N_STAR;
                s->DTidalMassLoss += m / s->N_STAR;
                s->Etidal += st->E * m / s->N_STAR;
                destroy_obj(s, i);
            }
        }
        s->TidalMassLoss += s->DTidalMassLoss;
    } while (s->DTidalMassLoss > 0);
    return OCMC_OK;
}

/* ComputeIntermediateEnergy, cmc_utils.c:368-391 */
int ocmc_compute_intermediate_energy(ocmc_state *s)
{
    int ok;
    for (long j = 1; j <= s->N_MAX_NEW; j++) {
        if (s->star[j].rnew < 1.0e6) {
            s->star[j].EI = sqr(s->star[j].vr) + sqr(s->star[j].vt) + s->star_phi[j] - potential_checked(s, s->star[j].rnew, &ok);
            if (!ok) return s->err;
        }
    }
    for (long j = 1; j <= s->N_MAX_NEW; j++) {
        s->star[j].rOld = s->star_r[j];
        s->star[j].r = s->star[j].rnew;
        s->star[j].m = s->star_m[j];
        s->star[j].vr = s->star[j].vrnew;
        s->star[j].vt = s->star[j].vtnew;
    }
    return OCMC_OK;
}

/* compare_type, cmc_sort.c:245-250 */
static int compare_r(const void *a, const void *b)
{
    double ka = ((const struct ostar *)a)->r, kb = ((const struct ostar *)b)->r;
    if (ka < kb) return -1;
    if (ka > kb) return 1;
    return 0;
}

/* qsorts_new + sample_sort on one rank + post_sort_comm:
 * cmc_utils.c:2232-2288, cmc_sort.c:375-420 (local qsort, remove_stripped_stars). */
int ocmc_qsorts_new(ocmc_state *s)
{
    long n = s->N_MAX_NEW;
    qsort(&s->star[1], (size_t)n, sizeof(struct ostar), compare_r);
    long i = n; /* remove_stripped_stars, cmc_sort.c:343-354 */
    while (i >= 1 && s->star[i].r == SF_INFINITY) {
        n--;
        i--;
    }
    s->N_MAX = n;
    s->N_MAX_NEW = n;
    for (i = 1; i <= n; i++) {
        s->star_r[i] = s->star[i].r;
        s->star_m[i] = s->star[i].m;
    }
    return OCMC_OK;
}

/* set_velocities3, cmc_utils.c:254-349, single rank (the excess pass between
 * ranks starts from zero and therefore changes nothing). */
int ocmc_energy_conservation3(ocmc_state *s)
{
    const double q = 0.5, E_dump_factor = 0.8;
    double Eexcess = 0.0;
    int ok;
    for (long i = 1; i <= s->N_MAX_NEW; i++) {
        struct ostar *st = &s->star[i];
        double m = s->star_m[i];
        if (st->interacted == 0) {
            double Unewrold = potential_checked(s, st->rOld, &ok) + phi_s(s, st->rOld, i);
            if (!ok) return s->err;
            double Unewrnew = s->star_phi[i] + phi_s(s, s->star_r[i], i);
            double vold2 = st->vtold * st->vtold + st->vrold * st->vrold;
            double vnew2 = vold2 + 2.0 * (1.0 - q) * (st->Uoldrold - st->Uoldrnew) + 2.0 * q * (Unewrold - Unewrnew);
            if (vnew2 <= 0.0) {
                Eexcess += 0.5 * (sqr(st->vr) + sqr(st->vt) - vnew2) * m;
            } else {
                double alpha = sqrt(vnew2 / (sqr(st->vr) + sqr(st->vt)));
                st->vr *= alpha;
                st->vt *= alpha;
                double v2 = sqr(st->vr) + sqr(st->vt);
                st->vrnew = st->vr;
                st->vtnew = st->vt;
                double E_dump_capacity = E_dump_factor * 0.5 * m * v2;
                double E_dump = OMIN(E_dump_capacity, Eexcess);
                if (Eexcess > 0) {
                    double exc_ratio = sqrt((v2 - 2 * E_dump / m) / v2);
                    st->vr *= exc_ratio;
                    st->vt *= exc_ratio;
                    Eexcess -= E_dump;
                }
            }
        }
    }
    /* cmc_utils.c:313-348 on one rank: Eexcess is replaced by the (zero) value
     * received from the previous rank, so the remainder is dropped. */
    s->Eoops += -0.0 * s->madhoc;
    return OCMC_OK;
}

/* compute_energy_new + ComputeEnergy, cmc_utils.c:2018-2028, 604-656 */
int ocmc_compute_energy(ocmc_state *s)
{
    s->Eescaped += s->Eescaped_old;
    s->Jescaped += s->Jescaped_old;
    s->Eintescaped += s->Eintescaped_old;
    s->Ebescaped += s->Ebescaped_old;
    s->Etidal += s->Etidal_old;
    double K = 0.0, P = 0.0, phi0 = s->star_phi[0];
    for (long i = 1; i <= s->N_MAX; i++) {
        s->star[i].E = s->star_phi[i] + 0.5 * (sqr(s->star[i].vr) + sqr(s->star[i].vt));
        s->star[i].J = s->star_r[i] * s->star[i].vt;
    }
    for (long i = 1; i <= s->N_MAX; i++) {
        K += 0.5 * (sqr(s->star[i].vr) + sqr(s->star[i].vt)) * s->star_m[i] * s->madhoc;
        P += s->star_phi[i] * s->star_m[i] * s->madhoc;
        P += phi0 * s->cenma_m * s->madhoc / s->N_MAX;
    }
    P *= 0.5;
    s->KE = K;
    s->PE = P;
    s->cenma_E += s->cenma_E_new;
    s->cenma_E_new = 0.0;
    s->Etot = K + P + 0.0 + 0.0;
    s->Etot += s->cenma_E + s->Eescaped + s->Ebescaped + s->Eintescaped;
    return OCMC_OK;
}

/* cmc.c:246-257 */
int ocmc_begin_step(ocmc_state *s)
{
    s->Eescaped_old = s->Eescaped;
    s->Jescaped_old = s->Jescaped;
    s->Eintescaped_old = s->Eintescaped;
    s->Ebescaped_old = s->Ebescaped;
    s->TidalMassLoss_old = s->TidalMassLoss;
    s->Etidal_old = s->Etidal;
    s->Eescaped = s->Jescaped = s->Eintescaped = s->Ebescaped = 0.0;
    s->TidalMassLoss = 0.0;
    s->Etidal = 0.0;
    s->N_MAX_NEW = s->N_MAX;
    return OCMC_OK;
}

int ocmc_end_step(ocmc_state *s)
{
    for (long i = 1; i <= s->N_MAX_NEW; i++) s->star[i].interacted = 0;
    s->tcount++;
    return OCMC_OK;
}

/* cmc.c:152-167: potential, then energies (set_energy_vars zeroes the tallies) */
int ocmc_initialize(ocmc_state *s)
{
    int rc = ocmc_calc_potential(s);
    if (rc) return rc;
    s->Eescaped = s->Jescaped = s->Eintescaped = s->Ebescaped = s->Eoops = 0.0;
    rc = ocmc_compute_energy(s);
    s->Etot_ini = s->Etot;
    return rc;
}

#define STEP(call)                     \
    do {                               \
        int rc_ = (call);              \
        if (rc_) return rc_;           \
        if (s->err) return s->err;     \
    } while (0)

/* The main loop body, cmc.c:240-407, restricted to the plain-dynamics path. */
int ocmc_step(ocmc_state *s)
{
    STEP(ocmc_begin_step(s));
    STEP(ocmc_calc_timestep(s));
    if (s->P.PERTURB > 0) STEP(ocmc_dynamics_apply(s, s->Dt));
    s->Prev_Dt = s->Dt;
    STEP(ocmc_energy_conservation1(s));
    STEP(ocmc_new_orbits_calculate(s));
    STEP(ocmc_energy_conservation2(s));
    STEP(ocmc_tidally_strip_stars(s));
    STEP(ocmc_compute_intermediate_energy(s));
    STEP(ocmc_qsorts_new(s));
    STEP(ocmc_calc_potential(s));
    STEP(ocmc_energy_conservation3(s));
    STEP(ocmc_compute_energy(s));
    STEP(ocmc_end_step(s));
    return OCMC_OK;
}

/* ------------------------------------------------------------ access ---- */

/* ------------------------------------------------------- diagnostics ---- */
/* comp_mass_percent (cmc_utils.c:872-968), one rank: the radius at which the
 * forward mass sum first exceeds each fraction of Mtotal, with the running
 * kinetic sums there; at most one fraction is assigned per star (an if, not
 * a while).  clusdyn_calculate (cmc_utils.c:1613-1624): rh = star_r just past
 * half the mass.  central_calculate (cmc_utils.c:1239-1345): Casertano & Hut
 * (1985) local densities over the J = 6 neighbours of every star out to that
 * index, and their density-weighted averages. */
int ocmc_diagnostics(ocmc_state *s, const double *mass_pc, int n_pc, int bh_include, double minimum_r,
                     ocmc_diag *d)
{
    memset(d, 0, sizeof(*d));
    if (n_pc < 0 || n_pc > OCMC_MASS_PC_MAX) return fail(s, OCMC_ERR_CAPACITY, n_pc);
    d->n_pc = n_pc;
    const double madhoc = s->madhoc, Mtotal = s->Mtotal;
    const long J = 6;
    /* central_calculate: nave just beyond the half-mass radius */
    double m = 0.0;
    long nave = 1;
    while (m < 0.5 * Mtotal) {
        m += s->star_m[nave] / s->N_STAR;
        nave++;
    }
    if (s->N_STAR <= 2 * J || nave >= s->N_STAR - 6) return fail(s, OCMC_ERR_CAPACITY, nave);
    d->nave = nave;
    double rhojsum = 0.0, rhoj2sum = 0.0, rho = 0.0, v_rms = 0.0, rc = 0.0, rc_nb = 0.0, m_ave = 0.0;
    for (long i = 1; i <= nave; i++) {
        const long jmin = (i - J / 2 > 1) ? i - J / 2 : 1, jmax = jmin + J;
        double mrho = 0.0;
        for (long j = jmin + 1; j <= jmax - 1; j++) mrho += s->star_m[j] * madhoc;
        const double Vrj = 4.0 / 3.0 * PI * (cub(s->star_r[jmax]) - cub(s->star_r[jmin]));
        const double rhoj = mrho / Vrj;
        rhojsum += rhoj;
        rhoj2sum += sqr(rhoj);
        rho += sqr(rhoj);
        v_rms += rhoj * (sqr(s->star[i].vr) + sqr(s->star[i].vt));
        rc += rhoj * s->star_r[i];
        rc_nb += sqr(rhoj * s->star_r[i]);
        m_ave += rhoj * s->star_m[i] * madhoc;
    }
    rho /= rhojsum;
    rho *= 4.0 / 5.0;
    rho *= 2.0;
    v_rms /= rhojsum;
    v_rms = sqrt(v_rms);
    rc /= rhojsum;
    rc_nb = sqrt(rc_nb / rhoj2sum);
    m_ave /= rhojsum;
    d->rho = rho;
    d->v_rms = v_rms;
    d->rc = rc;
    d->rc_nb = rc_nb;
    d->m_ave = m_ave;
    d->n = rho / m_ave;
    d->rc_spitzer = sqrt(3.0 * sqr(v_rms) / (4.0 * PI * rho));
    d->N_core = 4.0 / 3.0 * PI * cub(rc) * (d->n / 2.0);
    d->N_core_nb = 4.0 / 3.0 * PI * cub(rc_nb) * (d->n / 2.0);
    d->Trc = 0.065 * cub(v_rms) / (rho * m_ave);
    /* clusdyn_calculate */
    m = 0.0;
    long k = 1;
    while (m < 0.5 * Mtotal) {
        m += s->star_m[k] / s->N_STAR;
        k++;
    }
    d->rh = s->star_r[k];
    /* comp_mass_percent */
    double mprev;
    long mcount = 0;
    if (bh_include) {
        mprev = s->cenma_m * madhoc;
        for (mcount = 0; mcount < n_pc; mcount++) {
            if (mprev / Mtotal > mass_pc[mcount]) {
                d->mass_r[mcount] = minimum_r;
            } else {
                break;
            }
        }
    } else {
        mprev = 0.0;
    }
    const long NN = s->N_MAX_NEW;
    double *kr = calloc((size_t)NN + 1, sizeof(double)), *kt = calloc((size_t)NN + 1, sizeof(double));
    double *vr2 = calloc((size_t)NN + 1, sizeof(double)), *vt2 = calloc((size_t)NN + 1, sizeof(double));
    if (!kr || !kt || !vr2 || !vt2) {
        free(kr);
        free(kt);
        free(vr2);
        free(vt2);
        return fail(s, OCMC_ERR_CAPACITY, NN);
    }
    for (k = 1; k <= NN; k++) {
        const struct ostar *st = &s->star[k];
        kr[k] = kr[k - 1] + 0.5 * s->star_m[k] * madhoc * st->vr * st->vr;
        kt[k] = kt[k - 1] + 0.5 * s->star_m[k] * madhoc * st->vt * st->vt;
        vr2[k] = vr2[k - 1] + st->vr * st->vr;
        vt2[k] = vt2[k - 1] + st->vt * st->vt;
    }
    if (mcount < n_pc) {
        for (k = 1; k <= s->N_MAX; k++) {
            mprev += s->star_m[k] / s->N_STAR;
            if (mprev > mass_pc[mcount] * Mtotal) {
                d->mass_r[mcount] = s->star_r[k];
                d->ave_mass_r[mcount] = mprev / Mtotal / k * 1.0;  /* initial_total_mass = 1 */
                d->no_star_r[mcount] = k;
                d->densities_r[mcount] = mprev / (4.0 / 3.0 * PI * pow(s->star_r[k], 3));
                d->ke_rad_r[mcount] = kr[k];
                d->ke_tan_r[mcount] = kt[k];
                d->v2_rad_r[mcount] = vr2[k];
                d->v2_tan_r[mcount] = vt2[k];
                mcount++;
                if (mcount == n_pc) break;
            }
        }
    }
    free(kr);
    free(kt);
    free(vr2);
    free(vt2);
    return 0;
}

static double *global_array(const ocmc_state *s, const char *name)
{
    if (!strcmp(name, "star_r")) return s->star_r;
    if (!strcmp(name, "star_m")) return s->star_m;
    if (!strcmp(name, "star_phi")) return s->star_phi;
    if (!strcmp(name, "sigma_r")) return s->sigma_r;
    if (!strcmp(name, "sigma")) return s->sigma;
    return NULL;
}

static long star_field_offset(const char *name)
{
#define F(n)                                                     \
    if (!strcmp(name, #n)) return (long)offsetof(struct ostar, n);
    F(r) F(m) F(vr) F(vt) F(E) F(J) F(rnew) F(vrnew) F(vtnew) F(rOld) F(X) F(Y) F(r_peri) F(r_apo)
    F(vrold) F(vtold) F(Uoldrold) F(Uoldrnew) F(EI)
#undef F
    return -1;
}

long ocmc_get_field(const ocmc_state *s, const char *name, double *out, long cap)
{
    double *g = global_array(s, name);
    if (g) {
        long n = s->N_MAX + 2;
        if (n > cap) n = cap;
        memcpy(out, g, (size_t)n * sizeof(double));
        return n;
    }
    long off = star_field_offset(name);
    if (off < 0) return -1;
    long n = s->N_MAX_NEW;
    if (n > cap) n = cap;
    for (long i = 0; i < n; i++) out[i] = *(const double *)((const char *)&s->star[i + 1] + off);
    return n;
}

long ocmc_set_field(ocmc_state *s, const char *name, const double *in, long n)
{
    double *g = global_array(s, name);
    if (g) {
        if (n > s->cap + 2) n = s->cap + 2;
        memcpy(g, in, (size_t)n * sizeof(double));
        return n;
    }
    long off = star_field_offset(name);
    if (off < 0) return -1;
    if (n > s->N_MAX_NEW) n = s->N_MAX_NEW;
    for (long i = 0; i < n; i++) *(double *)((char *)&s->star[i + 1] + off) = in[i];
    return n;
}

long ocmc_get_ids(const ocmc_state *s, int64_t *out, long cap)
{
    long n = s->N_MAX_NEW;
    if (n > cap) n = cap;
    for (long i = 0; i < n; i++) out[i] = s->star[i + 1].id;
    return n;
}

double ocmc_get_scalar(const ocmc_state *s, const char *name)
{
#define S(n) \
    if (!strcmp(name, #n)) return (double)s->n;
    S(N_STAR) S(N_MAX) S(N_MAX_NEW) S(Mtotal) S(Rtidal) S(orbit_r) S(madhoc) S(cenma_m) S(Dt) S(Prev_Dt)
    S(TotalTime) S(max_r) S(TidalMassLoss) S(OldTidalMassLoss) S(TidalMassLoss_old) S(Eescaped) S(Jescaped)
    S(Etidal) S(Eoops) S(Etot) S(KE) S(PE) S(Etot_ini) S(tcount) S(Nrel) S(sigma_n) S(n_root_vr)
#undef S
    if (!strcmp(name, "Nrelbeta0")) return (double)s->Nrelbeta[0];
    if (!strcmp(name, "Nrelbeta1")) return (double)s->Nrelbeta[1];
    if (!strcmp(name, "Nrelbeta2")) return (double)s->Nrelbeta[2];
    if (!strcmp(name, "Nrelbeta3")) return (double)s->Nrelbeta[3];
    return NAN;
}

int ocmc_set_scalar(ocmc_state *s, const char *name, double v)
{
#define S(n)                \
    if (!strcmp(name, #n)) { \
        s->n = v;           \
        return 0;           \
    }
    S(Mtotal) S(Rtidal) S(orbit_r) S(Dt) S(Prev_Dt) S(TotalTime) S(TidalMassLoss) S(OldTidalMassLoss)
    S(TidalMassLoss_old)
#undef S
    if (!strcmp(name, "tcount")) {
        s->tcount = (long)v;
        return 0;
    }
    return -1;
}

long ocmc_nstars(const ocmc_state *s) { return s->N_MAX_NEW; }
int ocmc_last_error(const ocmc_state *s) { return s->err; }
long ocmc_last_error_index(const ocmc_state *s) { return s->err_index; }
