/* Driver of the reference's own Henon step (TEST INFRASTRUCTURE; never part
 * of the product).
 *
 * oracle/ref.mk compiles the reference's hot-path TUs unmodified, in place,
 * against the single-rank MPI / GSL / HDF5 shims beside this file, and links
 * them with this driver into oracle/_ref/libcmcref.so.  The driver sets the
 * reference's globals as its parser and loader would (one rank, the plain
 * dynamics configuration), loads a model through the reference's own
 * load_fits_file_data (cmc_fits.c:63), and then calls the reference's
 * functions in its main loop's order (cmc.c:240-407).  Its API mirrors the
 * oracle's (cmc_oracle.h) phase by phase, so that tests drive both the same
 * way and compare them field by field.
 *
 * The reference keeps its state in globals, so there is one cluster per
 * process at a time.  Draws: counter mode keys Philox4x32-10 exactly as the
 * oracle and the kernels do (cmcref_draw); taus113 mode runs the reference's
 * own generator untouched.  A reference exit()/MPI_Abort returns here through
 * longjmp with the error code; the reference's exit_cleanly() has by then
 * freed its arrays, so the instance is closed. */
#include <math.h>
#include <setjmp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cmc.h"
#include "cmc_vars.h"

#include "../philox.h"

/* same layout as ocmc_params (cmc_oracle.h) */
typedef struct {
    long N_STAR, AVEKERNEL;
    double GAMMA, THETASEMAX;
    int PERTURB, RELAXATION, TIDALLY_STRIP_STARS, TIDAL_TREATMENT;
    double orbit_r, cenma_m;
    long apsides_max_iter;
    double apsides_precision, apsides_convergence;
    long n_try;
    uint64_t seed;
    int draw_mode;
} cmcref_params;

enum { DRAW_COUNTER = 0, DRAW_TAUS113 = 1 };
enum { SITE_Y = 1, SITE_PENC = 2, SITE_PSI = 3, SITE_TRIAL = 4, SITE_SIGN = 5 };

static jmp_buf g_jmp;
static int g_in_call, g_live, g_err;
static long g_err_line;
static char g_err_what[160];
static cmcref_params g_p;
static gsl_rng *g_rng;
static double g_Etot_ini;

void cmcref_exit(int code)
{
    if (!g_in_call) {
        fprintf(stderr, "cmcref: exit(%d) outside a driver call\n", code);
        abort();
    }
    longjmp(g_jmp, code ? code : -1);
}

void cmcref_unreachable(const char *what)
{
    snprintf(g_err_what, sizeof g_err_what, "%s", what);
    cmcref_exit(-100);
}

/* The reference's log macros (parafprintf, cmc.h:2200-2204) append to these
 * MPI-IO string buffers, which its output routines flush; nothing is written
 * here, so every driver call starts them empty. */
static void reset_file_buffers(void)
{
#define R(f)                                   \
    if (mpi_##f##file_wrbuf) {                \
        mpi_##f##file_wrbuf[0] = 0;           \
        mpi_##f##file_len = 0;                \
    }
    R(bhmerger) R(bhsummary) R(binint) R(collision) R(escbhsummary) R(esc) R(lightcollision) R(log) R(morecoll) R(morepulsar) R(newbh) R(newns) R(pulsar) R(relaxation) R(removestar) R(semergedisrupt) R(tde) R(threebbdebug) R(threebb) R(threebbprobability) R(tidalcapture) R(triple)
#undef R
}

/* ------------------------------------------------------------- draws ---- */

static double counter_draw(int site, int64_t id, uint32_t n, int word)
{
    uint32_t key[2] = {(uint32_t)g_p.seed, (uint32_t)(g_p.seed >> 32) ^ (uint32_t)tcount};
    uint64_t uid = (uint64_t)id;
    uint32_t ctr[4] = {(uint32_t)uid, (uint32_t)(uid >> 32), (uint32_t)site, n};
    uint32_t out[4];
    philox4x32_10(ctr, key, out);
    return out[word & 3] / 4294967296.0;
}

/* (TU, line) -> (site, draw number, word); see cmcref_inject.h */
double cmcref_draw(int tu, int line, long idx, long trial)
{
    int site = 0, word = 0;
    uint32_t n = 0;
    if (tu == 1 && line == 406) site = SITE_PENC;
    else if (tu == 1 && line == 465) site = SITE_PSI;
    else if (tu == 2 && line == 839) site = SITE_Y;
    else if (tu == 3 && line == 863) site = SITE_TRIAL, n = (uint32_t)(trial - 1), word = 0;
    else if (tu == 3 && line == 867) site = SITE_TRIAL, n = (uint32_t)(trial - 1), word = 1;
    else if (tu == 3 && line == 923) site = SITE_SIGN;
    if (!site) {
        snprintf(g_err_what, sizeof g_err_what, "draw at TU %d line %d is off the Henon-step path", tu, line);
        g_err_line = line;
        cmcref_exit(-101);
    }
    if (g_p.draw_mode == DRAW_TAUS113) return rng_t113_dbl_new(curr_st);
    if (idx < 0) cmcref_unreachable("draw site without a star index");
    return counter_draw(site, star[idx].id, n, word);
}

/* --------------------------------------------------------- lifecycle ---- */

#define CALL_BEGIN                                \
    if (!g_live) return -200;                     \
    reset_file_buffers();                         \
    g_in_call = 1;                                \
    {                                             \
        int rc_ = setjmp(g_jmp);                  \
        if (rc_) {                                \
            g_in_call = 0;                        \
            g_live = 0;                           \
            g_err = rc_;                          \
            return rc_;                           \
        }                                         \
    }
#define CALL_END    \
    g_in_call = 0;  \
    return 0;

static void *xcalloc(size_t n, size_t sz)
{
    void *p = calloc(n ? n : 1, sz);
    if (!p) {
        fprintf(stderr, "cmcref: out of memory\n");
        abort();
    }
    return p;
}

/* Parameters as the reference's parser sets them (cmc_io.c CHECK_PARSED
 * defaults) for the plain-dynamics configuration: relaxation and tidal
 * stripping on; strong encounters, stellar evolution, three-body binaries,
 * loss cone, search grid and tidal-tensor files off. */
static void set_parameters(const cmcref_params *p, long N)
{
    quiet = 1;
    debug = 0;
    PERTURB = p->PERTURB;
    RELAXATION = p->RELAXATION;
    TIDALLY_STRIP_STARS = p->TIDALLY_STRIP_STARS;
    THETASEMAX = p->THETASEMAX;
    TIDAL_TREATMENT = p->TIDAL_TREATMENT;
    GAMMA = p->GAMMA;
    AVEKERNEL = p->AVEKERNEL;
    MIN_CHUNK_SIZE = 40;
    BH_AVEKERNEL = 10;
    APSIDES_PRECISION = p->apsides_precision;
    APSIDES_MAX_ITER = p->apsides_max_iter;
    APSIDES_CONVERGENCE = p->apsides_convergence;
    IDUM = (long)p->seed;
    STELLAR_EVOLUTION = 0;
    SS_COLLISION = 0;
    TIDAL_CAPTURE = 0;
    BH_CAPTURE = 0;
    STAR_AGING_SCHEME = 0;
    PREAGING = 0;
    BINBIN = 0;
    BINSINGLE = 0;
    STREAMS = 1;
    THREEBODYBINARIES = 0;
    BH_LOSS_CONE = 0;
    MINIMUM_R = 0.0;
    BH_R_DISRUPT_NB = 0.0;
    CIRC_PERIOD_THRESHOLD = 1e-18;
    USE_TT_FILE = 0;
    USE_DF_CUTOFF = 0;
    SEARCH_GRID = 0;
    FORCE_RLX_STEP = 0;
    DT_HARD_BINARIES = 0;
    HARD_BINARY_KT = 1;
    BH_LC_FDT = 0.0;
    NUM_CENTRAL_STARS = 300;
    MASS_PC_BH_INCLUDE = 1;
    WIND_FACTOR = 1.0;
    TC_FACTOR = 1.0;
    COLL_FACTOR = 1.0;
    SAMPLESIZE = 1024;
    T_MAX = 20.0;
    T_MAX_COUNT = 1000000;
    MASS_PC_COUNT = 1;
    NO_MASS_BINS = 1;
    (void)N;
}

int cmcref_create(const cmcref_params *p, long N, const double *r, const double *m, const double *vr,
                  const double *vt, const int64_t *id)
{
    if (g_live || N < 2 * p->AVEKERNEL + 2) return -1;
    g_p = *p;
    g_err = 0;
    g_err_what[0] = 0;
    g_live = 1;
    g_in_call = 1;
    int rc = setjmp(g_jmp);
    if (rc) {
        g_in_call = 0;
        g_live = 0;
        g_err = rc;
        return rc;
    }
    /* main(), cmc.c:84-95: one rank */
    procs = 1;
    myid = 0;
    mpiDisp = (int *)xcalloc(1, sizeof(int));
    mpiLen = (int *)xcalloc(1, sizeof(int));
    mpiAllocFileBuffers();
    reset_file_buffers();
    set_global_vars1();
    set_parameters(p, N);
    g_rng = gsl_rng_alloc(gsl_rng_mt19937);

    /* parser(), cmc_io.c:2056-2104: the model as the input file would give it */
    cfd.NOBJ = N;
    cfd.NBINARY = 0;
    cfd.Mclus = 1.0e5;
    cfd.Rvir = 1.0;
    cfd.Rtid = p->orbit_r;
    cfd.Z = 0.001;
    cfd.obj_id = (long *)xcalloc((size_t)N + 2, sizeof(long));
    cfd.obj_k = (int *)xcalloc((size_t)N + 2, sizeof(int));
    cfd.obj_m = (double *)xcalloc((size_t)N + 2, sizeof(double));
    cfd.obj_Reff = (double *)xcalloc((size_t)N + 2, sizeof(double));
    cfd.obj_r = (double *)xcalloc((size_t)N + 2, sizeof(double));
    cfd.obj_vr = (double *)xcalloc((size_t)N + 2, sizeof(double));
    cfd.obj_vt = (double *)xcalloc((size_t)N + 2, sizeof(double));
    cfd.obj_binind = (long *)xcalloc((size_t)N + 2, sizeof(long));
    cfd.bs_index = (long *)xcalloc(1, sizeof(long));
    cfd.bs_id1 = (long *)xcalloc(1, sizeof(long));
    cfd.bs_k1 = (int *)xcalloc(1, sizeof(int));
    cfd.bs_m1 = (double *)xcalloc(1, sizeof(double));
    cfd.bs_Reff1 = (double *)xcalloc(1, sizeof(double));
    cfd.bs_id2 = (long *)xcalloc(1, sizeof(long));
    cfd.bs_k2 = (int *)xcalloc(1, sizeof(int));
    cfd.bs_m2 = (double *)xcalloc(1, sizeof(double));
    cfd.bs_Reff2 = (double *)xcalloc(1, sizeof(double));
    cfd.bs_a = (double *)xcalloc(1, sizeof(double));
    cfd.bs_e = (double *)xcalloc(1, sizeof(double));
    /* element 0 is the central mass (stored x 1/N like every mass, cmc_fits.c:128) */
    cfd.obj_m[0] = p->cenma_m / (double)(p->N_STAR > 0 ? p->N_STAR : N);
    cfd.obj_r[N + 1] = SF_INFINITY;
    for (long i = 1; i <= N; ++i) {
        cfd.obj_id[i] = (long)id[i - 1];
        cfd.obj_m[i] = m[i - 1];
        cfd.obj_r[i] = r[i - 1];
        cfd.obj_vr[i] = vr[i - 1];
        cfd.obj_vt[i] = vt[i - 1];
    }
    clus.N_STAR = N;
    clus.N_BINARY = 0;
    R_MAX = cfd.Rtid;
    METALLICITY = cfd.Z;
    clus.N_STAR_NEW = clus.N_STAR;
    N_STAR_DIM = 2 + clus.N_STAR;
    N_BIN_DIM = 2 + clus.N_STAR / 2;
    N_STAR_DIM = (long)floor(1.1 * ((double)N_STAR_DIM));
    N_BIN_DIM = (long)floor(1.1 * ((double)N_BIN_DIM));
    sigma_array.n = 0;
    N_STAR_DIM_OPT = (long)floor(1.5 * ((double)(1 + clus.N_STAR)));
    N_BIN_DIM_OPT = (long)floor(1.5 * ((double)(clus.N_STAR / 2)));
    star = (star_t *)xcalloc((size_t)N_STAR_DIM_OPT, sizeof(star_t));
    binary = (binary_t *)xcalloc((size_t)N_BIN_DIM_OPT, sizeof(binary_t));
    sigma_array.r = (double *)xcalloc((size_t)N_STAR_DIM_OPT, sizeof(double));
    sigma_array.sigma = (double *)xcalloc((size_t)N_STAR_DIM_OPT, sizeof(double));
    mass_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    ave_mass_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    no_star_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    densities_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    ke_rad_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    ke_tan_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    v2_rad_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    v2_tan_r = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    mass_pc = (double *)xcalloc(MASS_PC_COUNT, sizeof(double));
    mass_bins = (double *)xcalloc(NO_MASS_BINS, sizeof(double));
    mass_pc[0] = 0.5;

    /* main(), cmc.c:126-137 */
    Start = (int *)xcalloc(1, sizeof(int));
    End = (int *)xcalloc(1, sizeof(int));
    findLimits(cfd.NOBJ, MIN_CHUNK_SIZE);
    /* get_star_data(), cmc_io.c:3384-3426 */
    q_root = gsl_root_fsolver_alloc(gsl_root_fsolver_brent);
    star_r = (double *)xcalloc((size_t)N_STAR_DIM, sizeof(double));
    star_m = (double *)xcalloc((size_t)N_STAR_DIM, sizeof(double));
    star_phi = (double *)xcalloc((size_t)N_STAR_DIM, sizeof(double));
    load_fits_file_data();
    set_global_vars2();
    reset_rng_t113(IDUM);
    clus.N_MAX = clus.N_STAR;
    N_b = clus.N_BINARY;
    set_rng_states();
    orbit_r = R_MAX;
    g_in_call = 0;
    return 0;
}

static void free_inputs(void)
{
    free(cfd.obj_id), free(cfd.obj_k), free(cfd.obj_m), free(cfd.obj_Reff), free(cfd.obj_r), free(cfd.obj_vr);
    free(cfd.obj_vt), free(cfd.obj_binind), free(cfd.bs_index), free(cfd.bs_id1), free(cfd.bs_k1);
    free(cfd.bs_m1), free(cfd.bs_Reff1), free(cfd.bs_id2), free(cfd.bs_k2), free(cfd.bs_m2), free(cfd.bs_Reff2);
    free(cfd.bs_a), free(cfd.bs_e);
    memset(&cfd, 0, sizeof(cfd));
}

void cmcref_destroy(void)
{
    if (g_live) {
        free(star), free(binary), free(star_r), free(star_m), free(star_phi);
        free(sigma_array.r), free(sigma_array.sigma);
        free(mass_r), free(ave_mass_r), free(no_star_r), free(densities_r), free(ke_rad_r), free(ke_tan_r);
        free(v2_rad_r), free(v2_tan_r), free(mass_pc), free(mass_bins);
        free(curr_st), free(q_root);
        mpiFreeFileBuffers();
    }
    star = NULL, binary = NULL, star_r = star_m = star_phi = NULL;
    free(Start), free(End), free(mpiDisp), free(mpiLen);
    Start = End = mpiDisp = mpiLen = NULL;
    if (g_rng) gsl_rng_free(g_rng);
    g_rng = NULL;
    free_inputs();
    g_live = 0;
}

/* main(), cmc.c:152-183 up to the loop, plain dynamics */
int cmcref_initialize(void)
{
    CALL_BEGIN
    calc_potential_new();
    calc_sigma_new();
    central_calculate();
    bin_vars_calculate();
    set_energy_vars();
    compute_energy_new();
    clus.N_MAX_NEW = mpiEnd - mpiBegin + 1;
    DMse = 0.0;
    update_vars();
    central_calculate();
    calc_clusdyn_new();
    g_Etot_ini = Etotal.tot;
    CALL_END
}

/* cmc.c:246-257 */
int cmcref_begin_step(void)
{
    CALL_BEGIN
    Eescaped_old = Eescaped;
    Jescaped_old = Jescaped;
    Eintescaped_old = Eintescaped;
    Ebescaped_old = Ebescaped;
    TidalMassLoss_old = TidalMassLoss;
    Etidal_old = Etidal;
    Eescaped = Jescaped = Eintescaped = Ebescaped = 0.0;
    TidalMassLoss = 0.0;
    Etidal = 0.0;
    CALL_END
}

/* cmc.c:260-275: central_calculate, calc_timestep, N_MAX_NEW */
int cmcref_calc_timestep(void)
{
    CALL_BEGIN
    central_calculate();
    calc_timestep(g_rng);
    clus.N_MAX_NEW = mpiEnd - mpiBegin + 1;
    CALL_END
}

int cmcref_dynamics_apply(double dt)
{
    CALL_BEGIN
    dynamics_apply(dt, g_rng);
    CALL_END
}

/* cmc.c:289-302 */
int cmcref_energy_conservation1(void)
{
    CALL_BEGIN
    Prev_Dt = Dt;
    DMse = 0.0;
    energy_conservation1();
    toy_rejuvenation();
    CALL_END
}

int cmcref_new_orbits_calculate(void)
{
    CALL_BEGIN
    new_orbits_calculate();
    CALL_END
}

int cmcref_energy_conservation2(void)
{
    CALL_BEGIN
    energy_conservation2();
    CALL_END
}

int cmcref_tidally_strip_stars(void)
{
    CALL_BEGIN
    if (TIDALLY_STRIP_STARS > 0) tidally_strip_stars();
    CALL_END
}

int cmcref_compute_intermediate_energy(void)
{
    CALL_BEGIN
    ComputeIntermediateEnergy();
    CALL_END
}

/* cmc.c:326-332 */
int cmcref_qsorts_new(void)
{
    CALL_BEGIN
    qsorts_new();
    post_sort_comm();
    CALL_END
}

/* cmc.c:335-339 */
int cmcref_calc_potential(void)
{
    CALL_BEGIN
    calc_potential_new();
    findLimits(clus.N_MAX, MIN_CHUNK_SIZE);
    CALL_END
}

int cmcref_energy_conservation3(void)
{
    CALL_BEGIN
    energy_conservation3();
    CALL_END
}

/* cmc.c:343-355 (the mass-percent outputs are diagnostics and skipped) */
int cmcref_compute_energy(void)
{
    CALL_BEGIN
    compute_energy_new();
    CALL_END
}

/* cmc.c:355-382 */
int cmcref_end_step(void)
{
    CALL_BEGIN
    reset_interaction_flags();
    update_vars();
    calc_clusdyn_new();
    tcount++;
    CALL_END
}

int cmcref_step(void)
{
    int rc;
    if ((rc = cmcref_begin_step())) return rc;
    if ((rc = cmcref_calc_timestep())) return rc;
    if (PERTURB > 0 && (rc = cmcref_dynamics_apply(Dt))) return rc;
    if ((rc = cmcref_energy_conservation1())) return rc;
    if ((rc = cmcref_new_orbits_calculate())) return rc;
    if ((rc = cmcref_energy_conservation2())) return rc;
    if ((rc = cmcref_tidally_strip_stars())) return rc;
    if ((rc = cmcref_compute_intermediate_energy())) return rc;
    if ((rc = cmcref_qsorts_new())) return rc;
    if ((rc = cmcref_calc_potential())) return rc;
    if ((rc = cmcref_energy_conservation3())) return rc;
    if ((rc = cmcref_compute_energy())) return rc;
    return cmcref_end_step();
}

double cmcref_potential(double r)
{
    if (!g_live) return NAN;
    g_in_call = 1;
    if (setjmp(g_jmp)) {
        g_in_call = 0;
        g_live = 0;
        return NAN;
    }
    double v = potential(r);
    g_in_call = 0;
    return v;
}

/* ------------------------------------------------------------ access ---- */

static double *global_array(const char *name)
{
    if (!strcmp(name, "star_r")) return star_r;
    if (!strcmp(name, "star_m")) return star_m;
    if (!strcmp(name, "star_phi")) return star_phi;
    if (!strcmp(name, "sigma_r")) return sigma_array.r;
    if (!strcmp(name, "sigma")) return sigma_array.sigma;
    return NULL;
}

static long star_field_offset(const char *name)
{
#define F(n) \
    if (!strcmp(name, #n)) return (long)offsetof(star_t, n);
    F(r) F(m) F(vr) F(vt) F(E) F(J) F(rnew) F(vrnew) F(vtnew) F(rOld) F(X) F(Y) F(r_peri) F(r_apo)
    F(vrold) F(vtold) F(Uoldrold) F(Uoldrnew) F(EI)
#undef F
    return -1;
}

long cmcref_get_field(const char *name, double *out, long cap)
{
    if (!g_live) return -2;
    double *g = global_array(name);
    if (g) {
        long n = clus.N_MAX + 2;
        if (n > cap) n = cap;
        memcpy(out, g, (size_t)n * sizeof(double));
        return n;
    }
    long off = star_field_offset(name);
    if (off < 0) return -1;
    long n = clus.N_MAX_NEW;
    if (n > cap) n = cap;
    for (long i = 0; i < n; i++) out[i] = *(const double *)((const char *)&star[i + 1] + off);
    return n;
}

long cmcref_set_field(const char *name, const double *in, long n)
{
    if (!g_live) return -2;
    double *g = global_array(name);
    if (g) {
        if (n > N_STAR_DIM) n = N_STAR_DIM;
        memcpy(g, in, (size_t)n * sizeof(double));
        return n;
    }
    long off = star_field_offset(name);
    if (off < 0) return -1;
    if (n > clus.N_MAX_NEW) n = clus.N_MAX_NEW;
    for (long i = 0; i < n; i++) *(double *)((char *)&star[i + 1] + off) = in[i];
    return n;
}

long cmcref_get_ids(int64_t *out, long cap)
{
    if (!g_live) return -2;
    long n = clus.N_MAX_NEW;
    if (n > cap) n = cap;
    for (long i = 0; i < n; i++) out[i] = (int64_t)star[i + 1].id;
    return n;
}

double cmcref_get_scalar(const char *name)
{
#define S(n, v) \
    if (!strcmp(name, n)) return (double)(v);
    S("N_STAR", clus.N_STAR) S("N_MAX", clus.N_MAX) S("N_MAX_NEW", clus.N_MAX_NEW) S("Mtotal", Mtotal)
    S("Rtidal", Rtidal) S("orbit_r", orbit_r) S("madhoc", madhoc) S("cenma_m", cenma.m) S("Dt", Dt)
    S("Prev_Dt", Prev_Dt) S("TotalTime", TotalTime) S("max_r", max_r) S("TidalMassLoss", TidalMassLoss)
    S("OldTidalMassLoss", OldTidalMassLoss) S("TidalMassLoss_old", TidalMassLoss_old) S("Eescaped", Eescaped)
    S("Jescaped", Jescaped) S("Etidal", Etidal) S("Eoops", Eoops) S("Etot", Etotal.tot) S("KE", Etotal.K)
    S("PE", Etotal.P) S("Etot_ini", g_Etot_ini) S("tcount", tcount) S("sigma_n", sigma_array.n)
    S("rh", clusdyn.rh) S("rho_core", rho_core) S("core_radius", core_radius)
#undef S
    return NAN;
}

int cmcref_set_scalar(const char *name, double v)
{
#define S(n, lv)             \
    if (!strcmp(name, n)) { \
        lv = v;             \
        return 0;           \
    }
    S("Mtotal", Mtotal) S("Rtidal", Rtidal) S("orbit_r", orbit_r) S("Dt", Dt) S("Prev_Dt", Prev_Dt)
    S("TotalTime", TotalTime) S("TidalMassLoss", TidalMassLoss) S("OldTidalMassLoss", OldTidalMassLoss)
    S("TidalMassLoss_old", TidalMassLoss_old)
#undef S
    if (!strcmp(name, "tcount")) {
        tcount = (long)v;
        return 0;
    }
    return -1;
}

long cmcref_nstars(void) { return g_live ? clus.N_MAX_NEW : -1; }
int cmcref_last_error(void) { return g_err; }
const char *cmcref_last_error_what(void) { return g_err_what; }
int cmcref_sizeof_star(void) { return (int)sizeof(star_t); }
