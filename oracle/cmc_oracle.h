/*
 * cmc_oracle.h -- CPU oracle for the CMC Henon step (TEST INFRASTRUCTURE).
 *
 * This is a plain-C restatement of the reference's single-rank Henon step
 * (sort -> potential -> relaxation -> new orbits, plus the host glue the
 * reference runs between them), written to follow the reference's operation
 * order, `long double` usage and branch structure so that it can serve as the
 * parity checker for the GPU kernels.  Every function cites the reference
 * file:line it restates (paths relative to the CMC-COSMIC source tree).
 *
 * Only the test suite, the smoke check and bench.py's CPU-baseline leg use
 * this library.  The GPU product never links or calls it.
 *
 * Pinning: the taus113 generator is pinned to the reference's own known-answer
 * test (seed 123456, 2^20 steps -> 3511752030) and to the reference's
 * taus113-v2.c compiled in place; the physics (potential, relaxation, orbits)
 * has no golden vectors in the reference, so its parity is "unpinned" beyond
 * the statistical fixtures (initial virial energies, Plummer Lagrange radii).
 *
 * Uniform draws come from one of two sources:
 *   OCMC_DRAW_COUNTER  Philox4x32-10 keyed (seed, tcount, star id, site, n):
 *                      the same counter-based draws the GPU kernels make
 *                      ("draw injection"), so oracle and GPU are comparable
 *                      star by star;
 *   OCMC_DRAW_TAUS113  the reference's sequential taus113 stream seeded with
 *                      IDUM ("untouched" reference behaviour, used for the
 *                      timed CPU baseline).
 */
#ifndef CMC_ORACLE_H
#define CMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OCMC_DRAW_COUNTER = 0, OCMC_DRAW_TAUS113 = 1 };

/* Draw sites: the six rng_t113_dbl_new() call sites on the plain path. */
enum {
    OCMC_SITE_Y = 1,     /* cmc_dynamics_helper.c:839  random angle Y       */
    OCMC_SITE_PENC = 2,  /* cmc_dynamics.c:406         encounter test       */
    OCMC_SITE_PSI = 3,   /* cmc_dynamics.c:465         deflection azimuth   */
    OCMC_SITE_TRIAL = 4, /* cmc_evolution_thr.c:863/867 X and g0 per trial  */
    OCMC_SITE_SIGN = 5   /* cmc_evolution_thr.c:923    sign of vr           */
};

/* Error codes (the reference calls exit_cleanly(); the oracle returns). */
enum {
    OCMC_OK = 0,
    OCMC_ERR_NAN_MASS = 1,      /* cmc_utils.c:688  NaN (2) detected          */
    OCMC_ERR_NAN_PHI = 2,       /* cmc_utils.c:718/731                        */
    OCMC_ERR_W_ZERO = 3,        /* cmc_dynamics_helper.c:858                  */
    OCMC_ERR_WP_ZERO = 4,       /* cmc_dynamics.c:450                         */
    OCMC_ERR_NTRY = 5,          /* cmc_evolution_thr.c:890                    */
    OCMC_ERR_Q_NAN = 6,         /* cmc_evolution_thr.c:877                    */
    OCMC_ERR_ROOT_SIGNS = 7,    /* cmc_nr.c:515                               */
    OCMC_ERR_ROOT_NOCONV = 8,   /* cmc_nr.c:572                               */
    OCMC_ERR_ROOT_NEG = 9,      /* cmc_nr.c:594                               */
    OCMC_ERR_FINDZERO_R = 10,   /* cmc_utils.c:146 binary search failed       */
    OCMC_ERR_POT_INTERVAL = 11, /* cmc_nr.c:240                               */
    OCMC_ERR_CAPACITY = 12
};

typedef struct {
    long N_STAR;             /* clus.N_STAR: initial number of stars          */
    long AVEKERNEL;          /* p, sliding window half-width (default 20)     */
    double GAMMA;            /* Coulomb logarithm factor                       */
    double THETASEMAX;       /* max scattering angle for the time step         */
    int PERTURB, RELAXATION;
    int TIDALLY_STRIP_STARS, TIDAL_TREATMENT;
    double orbit_r;          /* R_MAX from the initial model (Rtid)            */
    double cenma_m;          /* central mass, stored x N                       */
    long apsides_max_iter;   /* APSIDES_MAX_ITER (100)                         */
    double apsides_precision;   /* APSIDES_PRECISION (1e-11)                  */
    double apsides_convergence; /* APSIDES_CONVERGENCE (5e-13)                */
    long n_try;              /* N_TRY (50000)                                  */
    uint64_t seed;           /* IDUM                                           */
    int draw_mode;           /* OCMC_DRAW_COUNTER or OCMC_DRAW_TAUS113         */
} ocmc_params;

typedef struct ocmc_state ocmc_state;

void ocmc_default_params(ocmc_params *p);

/* Creates the state from an initial model.  r, vr, vt are per star (index 0..N-1,
 * sorted by radius), m is the mass in N-body units (sum 1); it is stored x N as
 * the reference does (cmc_fits.c:99,123).  id may be NULL (ids 1..N). */
ocmc_state *ocmc_create(const ocmc_params *p, long N, const double *r, const double *m,
                        const double *vr, const double *vt, const int64_t *id);
void ocmc_destroy(ocmc_state *s);

/* Reference initialisation after loading (cmc.c:152-167): potential, energies. */
int ocmc_initialize(ocmc_state *s);

/* Phase functions, in main-loop order (cmc.c:240-407). */
int ocmc_begin_step(ocmc_state *s);               /* cmc.c:246-257          */
int ocmc_calc_timestep(ocmc_state *s);            /* cmc_utils.c:2132       */
int ocmc_dynamics_apply(ocmc_state *s, double dt);/* cmc_dynamics.c:17      */
int ocmc_energy_conservation1(ocmc_state *s);     /* cmc_utils.c:2153       */
int ocmc_new_orbits_calculate(ocmc_state *s);     /* cmc_utils.c:2194       */
int ocmc_energy_conservation2(ocmc_state *s);     /* cmc_utils.c:2218       */
int ocmc_tidally_strip_stars(ocmc_state *s);      /* cmc_evolution_thr.c:443*/
int ocmc_compute_intermediate_energy(ocmc_state *s); /* cmc_utils.c:368     */
int ocmc_qsorts_new(ocmc_state *s);               /* cmc_utils.c:2232+2259  */
int ocmc_calc_potential(ocmc_state *s);           /* cmc_utils.c:675        */
int ocmc_energy_conservation3(ocmc_state *s);     /* cmc_utils.c:254        */
int ocmc_compute_energy(ocmc_state *s);           /* cmc_utils.c:2018+604   */
int ocmc_end_step(ocmc_state *s);                 /* tcount++               */
/* The whole step in the order above. */
int ocmc_step(ocmc_state *s);

/* Point queries. */
double ocmc_potential(ocmc_state *s, double r);   /* cmc_utils.c:112        */

/* Per-step diagnostics of the dyn.dat and lagrad.dat outputs: the
 * density-weighted core of central_calculate (cmc_utils.c:1239-1345),
 * clusdyn_calculate's half-mass radius (cmc_utils.c:1613-1624) and
 * comp_mass_percent (cmc_utils.c:872-968), single rank, sequential sums. */
#define OCMC_MASS_PC_MAX 64
typedef struct {
    long nave;                 /* index just beyond the half-mass radius      */
    double rh;                 /* clusdyn.rh                                  */
    double rho, v_rms, rc, rc_nb, m_ave, n, rc_spitzer;  /* central.*         */
    double N_core, N_core_nb, Trc;
    int n_pc;
    double mass_r[OCMC_MASS_PC_MAX], ave_mass_r[OCMC_MASS_PC_MAX], no_star_r[OCMC_MASS_PC_MAX];
    double densities_r[OCMC_MASS_PC_MAX], ke_rad_r[OCMC_MASS_PC_MAX], ke_tan_r[OCMC_MASS_PC_MAX];
    double v2_rad_r[OCMC_MASS_PC_MAX], v2_tan_r[OCMC_MASS_PC_MAX];
} ocmc_diag;
int ocmc_diagnostics(ocmc_state *s, const double *mass_pc, int n_pc, int bh_include, double minimum_r,
                     ocmc_diag *d);
double ocmc_draw(const ocmc_state *s, int site, int64_t id, uint32_t n, int word);

/* Field access.  Per-star fields (index 1..N_MAX_NEW) are copied into out[0..n-1];
 * global arrays ("star_r", "star_m", "star_phi", "sigma_r", "sigma") copy
 * indices 0..N_MAX+1. Returns the number of values copied or -1. */
long ocmc_get_field(const ocmc_state *s, const char *name, double *out, long cap);
long ocmc_get_ids(const ocmc_state *s, int64_t *out, long cap);
long ocmc_set_field(ocmc_state *s, const char *name, const double *in, long n);
double ocmc_get_scalar(const ocmc_state *s, const char *name);
int ocmc_set_scalar(ocmc_state *s, const char *name, double v);
long ocmc_nstars(const ocmc_state *s);  /* clus.N_MAX_NEW */
int ocmc_last_error(const ocmc_state *s);
long ocmc_last_error_index(const ocmc_state *s);

/* RNG primitives (exposed for known-answer tests). */
void ocmc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void ocmc_taus113_seed(uint32_t z[4], unsigned long s);
uint32_t ocmc_taus113_next(uint32_t z[4]);

#ifdef __cplusplus
}
#endif
#endif
