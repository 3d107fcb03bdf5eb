/*
 * cmcgpu.h -- C ABI of libcmcgpu.so: CMC's Henon relaxation step on one GB300.
 *
 * The library keeps one or more star clusters resident in GPU memory as
 * structure-of-arrays (FP64 radius, mass, velocities, energies, potential) and
 * runs the reference's per-step hot path on them with hand-written sm_103a
 * kernels: radius sort, potential prefix scan, fused relaxation, new orbits.
 * The host glue between those phases (time step, Stodolkiewicz energy
 * conservation, tidal stripping, energy sums) runs on the device as well, so a
 * whole step needs no host round trip.
 *
 * Each phase entry point corresponds to one function of the reference's main
 * loop (src/cmc/cmc.c:240-407); its comment names the reference definition it
 * replaces.  The reference-named drop-in symbols (qsorts_new, dynamics_apply,
 * get_positions, ...) that bind a host `star[]` array live in cmc_dropin.h.
 *
 * Conventions
 *  - All functions return 0 (CMCG_OK) or a negative host error, or a positive
 *    physics error raised on the device (the same conditions on which the
 *    reference calls exit_cleanly(); the codes are listed below).
 *  - Per-star arrays passed in or out are 0-based over the N current stars in
 *    radial order; the library's internal arrays keep the reference's 1-based
 *    layout with sentinels at 0 and N+1.
 *  - Masses are passed in N-body units (total 1) and stored x N_STAR, as the
 *    reference does (src/cmc/cmc_fits.c:99,123).
 *  - A context is used from one host thread; calls are asynchronous on the
 *    context's CUDA stream except where they return data.
 *  - There is no CPU fallback: without a usable GPU, cmcg_create fails.
 */
#ifndef CMCGPU_H
#define CMCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status ---- */
enum {
    CMCG_OK = 0,
    CMCG_ERR_ARG = -1,
    CMCG_ERR_CUDA = -2,
    CMCG_ERR_CAPACITY = -3,
    CMCG_ERR_NOMEM = -4,
    CMCG_ERR_STATE = -5,
    CMCG_ERR_IO = -6,          /* a file could not be opened or read               */
    CMCG_ERR_FORMAT = -7,      /* a file's contents are not the layout expected    */
    /* device-side physics errors; the reference site each one mirrors: */
    CMCG_ERR_NAN_MASS = 1,      /* cmc_utils.c:688   NaN in the mass sum        */
    CMCG_ERR_NAN_PHI = 2,       /* cmc_utils.c:718   NaN in the potential       */
    CMCG_ERR_W_ZERO = 3,        /* cmc_dynamics_helper.c:858  W = 0             */
    CMCG_ERR_WP_ZERO = 4,       /* cmc_dynamics.c:450  wp = 0                   */
    CMCG_ERR_NTRY = 5,          /* cmc_evolution_thr.c:890  N_TRY exceeded      */
    CMCG_ERR_Q_NAN = 6,         /* cmc_evolution_thr.c:877  vr^2 is NaN         */
    CMCG_ERR_ROOT_SIGNS = 7,    /* cmc_nr.c:515   no sign change of vr^2        */
    CMCG_ERR_ROOT_NOCONV = 8,   /* cmc_nr.c:572   apsis root not converged      */
    CMCG_ERR_ROOT_NEG = 9,      /* cmc_nr.c:594   negative residual at apsis    */
    CMCG_ERR_FINDZERO_R = 10,   /* cmc_utils.c:146  radius search failed        */
    CMCG_ERR_POT_INTERVAL = 11, /* cmc_nr.c:240   radius outside interval       */
    CMCG_ERR_ENCOUNTER = 12,    /* a strong-encounter draw hit (host physics)   */
    CMCG_ERR_SPIN = 20,         /* a bounded cross-block wait gave up           */
    CMCG_ERR_TIDAL_ITER = 21,   /* tidal stripping did not settle               */
    CMCG_ERR_BOUNDS = 22,       /* a star count or index outside the cluster's
                                   capacity was refused (access skipped)        */
    CMCG_ERR_FILTER = 23        /* check_filters: a certified FP32 decision
                                   disagreed with the exact evaluation         */
};

/* ------------------------------------------------------- parameters ----- */
typedef struct {
    long N_STAR;               /* clus.N_STAR; 0 = the N of the loaded model      */
    long AVEKERNEL;            /* sliding-window half width p (default 20)        */
    double GAMMA;              /* Coulomb logarithm factor (default 0.1)          */
    double THETASEMAX;         /* max deflection for the time step (1.412)        */
    int PERTURB, RELAXATION;   /* default 1, 1                                    */
    int TIDALLY_STRIP_STARS;   /* default 1                                       */
    int TIDAL_TREATMENT;       /* 0 = apocentre cut, 1 = Giersz energy cut (1)    */
    double orbit_r;            /* R_MAX, the initial tidal radius                 */
    double cenma_m;            /* central mass, stored x N (0)                    */
    long apsides_max_iter;     /* APSIDES_MAX_ITER (100)                          */
    double apsides_precision;  /* APSIDES_PRECISION (1e-11)                       */
    double apsides_convergence;/* APSIDES_CONVERGENCE (5e-13)                     */
    long n_try;                /* N_TRY (50000)                                   */
    uint64_t seed;             /* IDUM: keys the counter-based draws              */
    int relax_fp32;            /* 1 = FP32 relaxation kinematics, FP64 energies   */
    int phi_sequential;        /* 1 = potential by the plain one-thread loop
                                  instead of the parallel exact replay (both give
                                  the reference's bits; for testing)              */
    int check_filters;         /* 1 = every certified FP32 accept/reject of an
                                  orbit trial is also evaluated exactly; a
                                  disagreement is CMCG_ERR_FILTER (for testing)   */
    int relax_trig32;          /* 1 = the FP64 relaxation's sines and cosines on
                                  the FP32 pipe in double-float (within 2e-14 of
                                  sin/cos instead of an ulp; 11% faster
                                  relaxation); 0 = FP64 sincos (default)         */
} cmcg_params;

void cmcg_default_params(cmcg_params *p);

/* ----------------------------------------------- synthetic clusters ----- */
enum { CMCG_MODEL_PLUMMER = 0, CMCG_MODEL_KING = 1 };
typedef struct {
    int model;                 /* CMCG_MODEL_PLUMMER or CMCG_MODEL_KING           */
    long N;                    /* number of objects                               */
    double w0;                 /* King concentration W0                           */
    int imf;                   /* 0 = equal masses, 1 = Kroupa (2001)             */
    double binary_fraction;    /* fraction of composite (m1 + m2) objects         */
    uint64_t seed;
} cmcg_ic_spec;
typedef struct {
    double *r, *m, *vr, *vt;   /* caller-allocated, N each; sorted by r on return */
    int64_t *id;               /* caller-allocated or NULL; ids 1..N              */
    double rtid;               /* tidal radius of the model (R_MAX)               */
} cmcg_ic;

/* Seeded initial model in N-body units (E = -1/4). Host only, no GPU needed. */
int cmcg_ic_generate(const cmcg_ic_spec *spec, cmcg_ic *out);
/* Per-cluster seed for cluster `index` of an ensemble drawn from one master seed. */
uint64_t cmcg_derive_seed(uint64_t master, uint64_t index);

/* The CMC initial-conditions file that COSMIC's InitialCMCTable writes (HDF5,
 * pandas fixed format), read without the HDF5 library.  Replaces
 * cmc_read_hdf5_file (src/libs/fitslib.c:209-455): obj receives
 * CLUS_OBJ_DATA/block0_values, one row per object with the columns
 * id, k, m, Reff, r, vr, vt, binind (row 0 the central mass, row NOBJ+1 the
 * outer sentinel, as cmc_fits.c:63-136 reads them); bin receives
 * CLUS_BINARY_DATA/block0_values, one row per binary with the columns
 * index, id1, k1, m1, Reff1, id2, k2, m2, Reff2, a, e.  Call with obj and bin
 * NULL to learn the shapes; then with row capacities of at least obj_rows and
 * bin_rows.  Returns CMCG_ERR_IO, CMCG_ERR_FORMAT (a storage layout or number
 * type this reader does not take: chunked or filtered data, big-endian or
 * non-8-byte numbers), CMCG_ERR_CAPACITY.  Host only, no GPU needed. */
typedef struct {
    long nobj, nbinary;          /* the NOBJ and NBINARY attributes                */
    double mclus, rvir, rtid, z; /* MCLUS, RVIR, RTID (N-body units), Z             */
    long obj_rows, obj_cols;     /* shape of CLUS_OBJ_DATA/block0_values (cols 8)   */
    long bin_rows, bin_cols;     /* shape of CLUS_BINARY_DATA/block0_values (11)    */
} cmcg_cmc_hdf5_info;
int cmcg_read_cmc_hdf5(const char *path, cmcg_cmc_hdf5_info *info, double *obj, long obj_cap_rows, double *bin,
                       long bin_cap_rows);

/* ---------------------------------------------------------- context ----- */
typedef struct cmcg_ctx cmcg_ctx;

/* One context holds `nclusters` independent clusters; every phase call runs
 * all of them in one launch per kernel.  capacity[c] bounds cluster c's N. */
int cmcg_create(cmcg_ctx **out, int nclusters, const long *capacity, const cmcg_params *params);
int cmcg_destroy(cmcg_ctx *ctx);
/* Copies a model (host memory, pinned or pageable) into cluster c. */
int cmcg_load(cmcg_ctx *ctx, int cluster, long N, const double *r, const double *m, const double *vr,
              const double *vt, const int64_t *id);
/* Start-up sequence of cmc.c:152-167: potential, then E, J and energies. */
int cmcg_initialize(cmcg_ctx *ctx);
/* Host-owned star state for cluster c, as the reference's host loop keeps it:
 * per star r (star_r), m (star_m, i.e. x N_STAR), vr, vt, E, J, id; 0-based, N
 * stars.  put replaces the device copy (scalars are kept), get reads it back
 * and returns N.  Both are asynchronous when the buffers are pinned: put's
 * arrays must stay unchanged until the context's stream has read them
 * (cmcg_synchronize, or any call that synchronises); get synchronises before
 * returning. */
int cmcg_put_stars(cmcg_ctx *ctx, int cluster, long N, const double *r, const double *m, const double *vr,
                   const double *vt, const double *E, const double *J, const int64_t *id);
long cmcg_get_stars(cmcg_ctx *ctx, int cluster, long cap, double *r, double *m, double *vr, double *vt, double *E,
                    double *J, int64_t *id);

/* ------------------------------------------------ step phases (all clusters) */
int cmcg_begin_step(cmcg_ctx *ctx);                /* cmc.c:246-257 tallies      */
int cmcg_calc_timestep(cmcg_ctx *ctx);             /* cmc_utils.c:2132 calc_timestep */
/* cmc_dynamics.c:17 dynamics_apply; dt < 0 uses the device time step. */
int cmcg_dynamics_apply(cmcg_ctx *ctx, double dt);
/* cmc_utils.c:2194 new_orbits_calculate (get_positions, cmc_evolution_thr.c:944)
 * fused with energy_conservation1/2 (cmc_utils.c:2153, 2218). */
int cmcg_new_orbits_calculate(cmcg_ctx *ctx);
int cmcg_tidally_strip_stars(cmcg_ctx *ctx);       /* cmc_evolution_thr.c:443    */
/* ComputeIntermediateEnergy's transfer (cmc_utils.c:368) + qsorts_new
 * (cmc_utils.c:2232) + post_sort_comm (cmc_utils.c:2259). */
int cmcg_qsorts_new(cmcg_ctx *ctx);
int cmcg_calc_potential(cmcg_ctx *ctx);            /* cmc_utils.c:675 potential_calculate */
int cmcg_energy_conservation3(cmcg_ctx *ctx);      /* cmc_utils.c:254 set_velocities3 */
int cmcg_compute_energy(cmcg_ctx *ctx);            /* cmc_utils.c:2018 compute_energy_new */
int cmcg_end_step(cmcg_ctx *ctx);                  /* tcount++                    */
/* One whole step in main-loop order; with graphs enabled it replays a captured
 * CUDA graph of the whole step. */
int cmcg_step(cmcg_ctx *ctx);
int cmcg_run(cmcg_ctx *ctx, int nsteps);
int cmcg_use_graph(cmcg_ctx *ctx, int enable);
int cmcg_synchronize(cmcg_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or record events against the library's launches. */
void *cmcg_stream(cmcg_ctx *ctx);

/* ------------------------------------------------------------ queries --- */
/* potential(r) of cmc_utils.c:112 for cluster c (synchronous). */
int cmcg_potential(cmcg_ctx *ctx, int cluster, double r, double *out);
/* Copies a per-star field (0-based, N_MAX_NEW values) or a global array
 * ("star_r", "star_m", "star_phi", "sigma_r", "sigma": indices 0..N_MAX+1). */
long cmcg_get_field(cmcg_ctx *ctx, int cluster, const char *name, double *out, long cap);
long cmcg_set_field(cmcg_ctx *ctx, int cluster, const char *name, const double *in, long n);
long cmcg_get_ids(cmcg_ctx *ctx, int cluster, int64_t *out, long cap);
int cmcg_get_scalar(cmcg_ctx *ctx, int cluster, const char *name, double *out);
int cmcg_set_scalar(cmcg_ctx *ctx, int cluster, const char *name, double v);
long cmcg_nstars(cmcg_ctx *ctx, int cluster);
/* First device error since the last call (0 if none), with cluster and star index. */
int cmcg_last_error(cmcg_ctx *ctx, int *cluster, long *index);
/* Kernel launches issued by the last cmcg_step / cmcg_run (graph nodes count). */
long cmcg_launch_count(cmcg_ctx *ctx);
/* Duration of the last launch of one kernel family, from CUDA events on the
 * context stream ("sort", "potential", "relax", "orbit", ...); needs
 * cmcg_profile(ctx, 1) before the step. */
int cmcg_profile(cmcg_ctx *ctx, int enable);
int cmcg_kernel_time(cmcg_ctx *ctx, const char *family, double *ms_total, long *launches);
/* Counter-based uniform draw the kernels use (site, star id, n, word). */
double cmcg_draw(uint64_t seed, long tcount, int site, int64_t id, uint32_t n, int word);
/* Diagnostic: the sign of function_q (cmc_utils.c:1654) at n points
 * (r_k, Phi_k) for stars (E, J, r_j, m_j), E including PHI_S(r_j), from each
 * stage of the certified test the apsis bisections use: out[4i + s] for
 * s = 0 FP32, 1 float-float, 2 FP64 (+1 / -1, or 0 = undecided) and s = 3 the
 * double-double evaluation (always decided).  Host arrays; runs on the
 * current device and waits for it. */
int cmcg_sign_stages(const double *E, const double *J, const double *rj, const double *mj, double invN,
                     const double *rk, const double *phik, long n, int *out);
/* Diagnostic: the sines and cosines the relaxation forms on the FP32 pipe
 * (double-float arithmetic): for i < n, out[2i], out[2i + 1] = sin, cos of
 * 2 pi w[i] 2^-32 (a uniform draw's angle); for j < nb, out[2n + 2j],
 * out[2n + 2j + 1] = sin, cos of beta[j] in [0, pi/2] (CMCG_ERR_ARG outside).
 * Host arrays; runs on the current device and waits for it. */
int cmcg_trig_check(const unsigned int *w, long n, const double *beta, long nb, double *out);
/* Diagnostic: how often the orbit phase took its rare branches, summed over
 * every launch on the current device since the last reset (all contexts):
 *   out[CMCG_ORBIT_SIGN_F64]  table probes of the apsis bisections
 *                             (find_zero_Q, cmc_nr.c:316) whose sign the FP32
 *                             and float-float stages left undecided;
 *   out[CMCG_ORBIT_SIGN_DD]   of those, probes the FP64 stage also left
 *                             undecided (evaluated in double-double);
 *   out[CMCG_ORBIT_ROOT_VR]   apsides outside the closed form's interval,
 *                             found by the root finder that stands in for
 *                             GSL's Brent in find_root_vr (cmc_nr.c:500),
 *                             which agrees with it to APSIDES_PRECISION.
 * Waits for the device; reset != 0 zeroes the counts after reading them. */
enum { CMCG_ORBIT_SIGN_F64 = 0, CMCG_ORBIT_SIGN_DD = 1, CMCG_ORBIT_ROOT_VR = 2, CMCG_ORBIT_NCOUNTERS = 4 };
int cmcg_orbit_counters(unsigned long long out[CMCG_ORBIT_NCOUNTERS], int reset);

/* ------------------------------------------------- learned proposal ---
 * An optional proposal for the orbit sampler's rejection loop
 * (get_positions_loop, cmc_evolution_thr.c:855-926).  A network 8 -> 64 ->
 * 64 -> 33 (ReLU; BF16 weights and activations, FP32 accumulation on the
 * tensor cores) maps a star's orbit features (rmin / rmax, ln rmax / 8,
 * E / Phi_a, J^2 / (2 rmin^2 (E - Phi_a)) and the potential's shape at four
 * table points between the apsides, Phi_a being the table value below rmin)
 * to a 32-bin piecewise-constant density q in the reference's sampling
 * variable X (s0 = 2X - 1), mixed with 1/64 of the uniform density, and to P,
 * the predicted acceptance probability of a plain trial.  A proposal trial
 * draws X from q and g0 uniform under kappa F P q(X), and accepts when
 * g0 < min(g(s0), F): the density the plain sampler draws from (its g
 * clipped at its envelope F).  The sampled distribution is therefore the
 * plain sampler's wherever kappa F P q >= min(g, F).  A trial that finds that
 * envelope below the density sends the star back to the plain sampler, which
 * then runs from its first trial with the plain draws (so with kappa small
 * enough every star takes exactly the plain result).
 * Modes: CMCG_LEARN_OFF (the plain sampler only), CMCG_LEARN_ON, and
 * CMCG_LEARN_COLLECT (the plain sampler through the learned launch sequence,
 * recording each sampled star's features, accepted X and trial count:
 * training data).  The network is trained by cmcg_mlp_train (Adam, on the
 * GPU) on (features, floor(32 X), trials) records, minimising
 * -log softmax(z)_bin - (k - 1) log(1 - P) - log P averaged over the batch. */
enum { CMCG_LEARN_OFF = 0, CMCG_LEARN_ON = 1, CMCG_LEARN_COLLECT = 2 };
#define CMCG_MLP_NPARAM 6881  /* W1[64][8], b1[64], W2[64][64], b2[64], W3[33][64], b3[33] */
#define CMCG_MLP_NIN 8
#define CMCG_MLP_NOUT 33
enum {
    CMCG_LSTAT_TRIALS = 0,       /* proposal trials up to each star's decision  */
    CMCG_LSTAT_ACCEPT = 1,       /* stars accepted by a proposal trial          */
    CMCG_LSTAT_FAIL = 2,         /* stars sent back to the plain sampler        */
    CMCG_LSTAT_STARS = 3,        /* stars that started with the proposal        */
    CMCG_LSTAT_PLAIN_TRIALS = 4, /* plain trials of stars the plain sampler did */
    CMCG_LSTAT_PLAIN_STARS = 5,  /* stars the plain sampler did                 */
    CMCG_LSTAT_N = 8
};
/* Select the orbit sampler for the following steps; kappa is the envelope factor (> 0). */
int cmcg_set_learned(cmcg_ctx *ctx, int mode, double kappa);
int cmcg_mlp_init(cmcg_ctx *ctx, uint64_t seed);
int cmcg_mlp_set_params(cmcg_ctx *ctx, const float *params /* CMCG_MLP_NPARAM */);
int cmcg_mlp_get_params(cmcg_ctx *ctx, float *params);
/* The network on n feature rows (n x 8): the 33 logits (n x 33) and/or the
 * stored proposal (n x 32: C_1 .. C_31 of the CDF, then P); either may be NULL. */
int cmcg_mlp_forward(cmcg_ctx *ctx, const float *feat, long n, float *z_out, float *prop_out);
/* Mean loss gradient over the n records (CMCG_MLP_NPARAM values) followed by
 * the two mean loss terms (bins, trial count): no update. */
int cmcg_mlp_gradient(cmcg_ctx *ctx, const float *feat, const int *bin, const int *ntrial, long n, float *grad);
/* `steps` Adam steps (beta 0.9, 0.999) on minibatches of `batch` records drawn
 * with replacement (keyed by seed and step); loss (2 x steps, or NULL). */
int cmcg_mlp_train(cmcg_ctx *ctx, const float *feat, const int *bin, const int *ntrial, long n, int steps,
                   int batch, double lr, uint64_t seed, float *loss);
/* After a step: the records of cluster k's sampled stars (features n x 8,
 * accepted X, trials: plain k > 0, proposal -k); returns their number (at
 * most cap written). */
long cmcg_learned_samples(cmcg_ctx *ctx, int k, float *feat, double *X, int *ntrial, long cap);
int cmcg_learned_stats(cmcg_ctx *ctx, uint64_t *out /* CMCG_LSTAT_N */);

/* --------------------------------------------------- host exchange -----
 * One step on host star arrays, one cmcg_stars per cluster: in[k] (N stars,
 * 0-based, as cmcg_put_stars takes them) is uploaded, the step runs, and
 * out[k] receives the stars after it (out[k].N set; out[k].cap >= in[k].N).
 * E and J go up while the relaxation runs; r, m and id are read back while
 * the potential, energy conservation and energies still run; graphs are
 * used when enabled.
 * in and out may be the same arrays, and the same cmcg_stars array: each
 * in[k].N is read before any out[k].N is written, so a step in place leaves
 * the next step's input counts behind.  Pinned host memory gives full copy
 * speed.  The call returns once every copy has finished, on errors too.
 * Equivalent to cmcg_put_stars + cmcg_step + cmcg_get_stars. */
typedef struct {
    long N;                    /* stars (in), stars after the step (out)          */
    long cap;                  /* capacity of the out arrays                       */
    double *r, *m, *vr, *vt, *E, *J;
    int64_t *id;
} cmcg_stars;
int cmcg_step_host(cmcg_ctx *ctx, const cmcg_stars *in, cmcg_stars *out);

/* ------------------------------------------------------- autotuner -----
 * Launch variants with bit-identical results, chosen by measurement on the
 * context's own clusters: "orbit" (5 or 4 blocks per SM, i.e. register
 * budgets of 102 or 128, each also as a persistent grid: variants 0-3),
 * "relax" (5 or 4 blocks per SM), "orbit_learn" (the same for the learned
 * sampling pass), "mlp_grid" (persistent CTAs per SM of the network's
 * inference: 4, 2, 3, 6), "sort_tile" (keys per tile of the radius sort's
 * digit passes: 4096, 2048, 1024) and "gather_tile" (stars per block of the
 * sort's payload gather: 256, 128, 1024).  cmcg_autotune times every variant of the
 * launches the current configuration uses over `steps` steps each (plus one
 * untimed step), keeps the fastest, and writes a one-line report (may be
 * NULL).  The tuning steps are real steps of the run. */
int cmcg_autotune(cmcg_ctx *ctx, int steps, char *report, long report_len);
int cmcg_set_variant(cmcg_ctx *ctx, const char *name, int variant);
int cmcg_get_variant(cmcg_ctx *ctx, const char *name);   /* the variant, or CMCG_ERR_ARG */

/* ------------------------------------------------- step diagnostics ---
 * What the reference writes to dyn.dat and lagrad.dat every step
 * (PrintFileOutput, cmc_io.c:260-323), reduced on the device from the
 * cluster's current state:
 *   central_calculate (cmc_utils.c:1239-1345): Casertano & Hut local
 *     densities out to the half-mass radius and their density-weighted
 *     averages (core density, rms velocity, core radius, rc_nb, N_core);
 *   clusdyn_calculate (cmc_utils.c:1613-1624): the half-mass radius rh;
 *   comp_mass_percent (cmc_utils.c:872-968): Lagrange radii and the running
 *     kinetic sums at each mass fraction.
 * The reference takes central_calculate at the start of a step and the rest
 * after energy_conservation3, so a dyn.dat line for a step takes its core
 * quantities from a call made before the step and the rest from one made
 * after it (cmcg_format_dyn_line has a parameter for each).  Sums are tree
 * sums: they agree with the reference's sequential ones to a few ulps of
 * their magnitude.  The kernels use the potential's and the sort's scratch
 * arrays, so call between steps. */
#define CMCG_MASS_PC_MAX 64
typedef struct {
    /* the step (dyn.dat columns; cmc_io.c:320-323) */
    double TotalTime, Dt;
    long tcount, N_MAX;
    double Mtotal, Etot, KE, PE, E_cenma, Eescaped, Eoops, max_r;
    /* central_calculate and clusdyn_calculate */
    long nave;                 /* index just beyond the half-mass radius       */
    double rh;                 /* clusdyn.rh                                   */
    double rho_0, v0_rms, core_radius, rc_nb, m_ave, n_central, rc_spitzer;
    double N_core, N_core_nb, Trc;
    /* comp_mass_percent, one entry per mass fraction */
    int n_pc;                  /* fractions asked for                          */
    int n_set;                 /* fractions reached (the rest are left at 0)   */
    double mass_pc[CMCG_MASS_PC_MAX];
    double mass_r[CMCG_MASS_PC_MAX], ave_mass_r[CMCG_MASS_PC_MAX], no_star_r[CMCG_MASS_PC_MAX];
    double densities_r[CMCG_MASS_PC_MAX], ke_rad_r[CMCG_MASS_PC_MAX], ke_tan_r[CMCG_MASS_PC_MAX];
    double v2_rad_r[CMCG_MASS_PC_MAX], v2_tan_r[CMCG_MASS_PC_MAX];
} cmcg_diag;

/* mass_pc: n_pc <= CMCG_MASS_PC_MAX fractions in non-decreasing order (the
 * .ini key MASS_PC); bh_include and minimum_r: MASS_PC_BH_INCLUDE and
 * MINIMUM_R.  Returns CMCG_ERR_STATE where central_calculate would stop
 * (cmc_utils.c:1254). */
int cmcg_diagnostics(cmcg_ctx *ctx, int cluster, const double *mass_pc, int n_pc, int bh_include, double minimum_r,
                     cmcg_diag *out);
/* One line of dyn.dat (the 28 columns of cmc_io.c:320-323): core quantities
 * from `start` (a call before the step), everything else from `end`.
 * Columns this build does not model (binary and internal energies, stellar
 * evolution mass loss) are 0, as the reference writes them without those
 * physics.  Returns the length written (with the newline), or -1 if `cap`
 * is too small. */
long cmcg_format_dyn_line(const cmcg_diag *start, const cmcg_diag *end, char *buf, long cap);
/* One line of lagrad.dat (cmc_io.c:266, 287, 301). */
long cmcg_format_lagrad_line(const cmcg_diag *d, char *buf, long cap);
/* The files' header lines (cmc_io.c:2294-2347). */
long cmcg_format_dyn_header(char *buf, long cap);
long cmcg_format_lagrad_header(const double *mass_pc, int n_pc, char *buf, long cap);

/* --------------------------------------------- allocation-free variant ---
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory once running -- a host code embedding this library in a process
 * whose GPU memory another runtime owns, or a long run on a shared GPU that
 * must not risk a failed allocation mid-simulation -- this is the stable
 * radius sort of cmcg_qsorts_new on caller-provided device arrays, with its
 * working memory in a fixed file-scope device array instead of the heap.
 *   d_r      device pointer, n radii (escapers at SF_INFINITY = 1e10 sort last)
 *   d_perm   device pointer, n outputs: 0-based input position of the i-th
 *            smallest radius (ties keep input order)
 *   n_bound  optional host pointer: count of radii below SF_INFINITY.  With
 *            it the call waits for the sort to finish and also returns any
 *            error the sort kernels recorded on the device; without it the
 *            call only queues the work on `stream` and reports host-side
 *            errors alone
 *   stream   a cudaStream_t, or NULL for the default stream
 * n may not exceed CMCG_NOALLOC_MAX_STARS (CMCG_ERR_CAPACITY otherwise).  Each
 * call looks up the array's device address on the current device; the first
 * call on a device also loads the module there and must come before any
 * stream capture.  Every GPU that loads the library holds the array (about
 * 34 MB) until the process exits.  All calls share it, so calls that overlap
 * on the GPU race. */
#define CMCG_NOALLOC_MAX_STARS (1L << 20)
int cmcg_sort_radii_noalloc(const double *d_r, long n, uint32_t *d_perm, long *n_bound, void *stream);

#ifdef __cplusplus
}
#endif
#endif
