/*
 * cmc_dropin.h -- the reference's hot-path functions under their own names
 * and prototypes (include/cmc/cmc.h), implemented on libcmcgpu.so, for
 * linking in place of their definitions in the reference's host program.
 *
 * The reference's functions work on process globals: the star[] array of
 * star_t records, star_r/star_m/star_phi, clus.N_MAX/N_MAX_NEW and a set of
 * scalars.  This library cannot include the reference's headers, so the host
 * describes where those live once, with cmcx_bind(): the base of star[],
 * sizeof(star_t) and offsetof(star_t, field) of the fields the hot path
 * reads or writes, and pointers to the arrays and scalars.  The glue is one
 * small C file compiled with the reference's headers: it fills cmcx_host with
 * &star[0], sizeof(star_t), offsetof(star_t, ...) and the globals' addresses.
 *
 * Ownership and sync.  cmcx_bind() copies star[1..N] to the GPU, which is
 * then authoritative for the hot fields.  With sync_each = 1 (the default
 * of cmcx_default_host) every function below leaves the host memory as the
 * reference's definition would -- the fields that function writes are copied
 * back into star[] / star_r / star_m / star_phi and the bound scalars -- so
 * any host code may run between calls.  With sync_each = 0 only the bound
 * scalars are copied back; call cmcx_download() before host code reads
 * star[] and cmcx_upload() after host code changes it.
 *
 * Errors.  Where the reference calls exit_cleanly(code, __FUNCTION__), these
 * functions call the handler set by cmcx_set_abort() with the device status
 * code (cmcgpu.h) and the function name; the default handler prints the
 * error and calls exit(code).
 *
 * RNG.  The gsl_rng argument is ignored, as on the reference's own hot path,
 * which draws from curr_st; the device draws are counter-based, keyed by
 * (seed, tcount, star id, site, n).
 */
#ifndef CMC_DROPIN_H
#define CMC_DROPIN_H

#include <stddef.h>
#include <stdint.h>

#include "cmcgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    /* star[] (array of star_t, index 0 and N+1 are the reference's sentinels) */
    void *star;
    size_t star_size;                 /* sizeof(star_t) */
    /* offsetof(star_t, f) of each field; required: r, vr, vt, m, E, J, id.
     * The others may be -1 if the host never reads them. */
    long off_r, off_vr, off_vt, off_m, off_E, off_J, off_id;
    long off_rnew, off_vrnew, off_vtnew, off_rOld, off_X, off_Y, off_r_peri, off_r_apo;
    int id_bytes;                     /* sizeof(star[0].id): 4 or 8 */
    /* global arrays, N_STAR_DIM doubles each */
    double *star_r, *star_m, *star_phi;
    long N_STAR_DIM;                  /* capacity of star[] and the arrays */
    /* clus.N_MAX and clus.N_MAX_NEW */
    long *N_MAX, *N_MAX_NEW;
    /* scalars copied back after the functions that set them (any may be NULL) */
    double *Dt, *Mtotal, *Rtidal, *max_r;
    double *Eescaped, *Jescaped, *TidalMassLoss, *Etidal;
    double *Etot, *KE, *PE;
    long *tcount;                     /* read at calc_timestep: keys the device draws */
    int sync_each;                    /* 1: every call mirrors its outputs into star[] */
} cmcx_host;

/* A host description with every offset -1, every pointer NULL, sync_each = 1. */
void cmcx_default_host(cmcx_host *h);

/* Binds the host state, creates the device context (capacity N_STAR_DIM)
 * and copies star[1..*N_MAX] to it (the masses as stored, i.e. x N_STAR).
 * params->N_STAR must be the run's clus.N_STAR.  Returns a cmcgpu.h status. */
int cmcx_bind(const cmcx_host *h, const cmcg_params *params);
void cmcx_unbind(void);
/* host star[] -> device (after host code changed star[]) */
int cmcx_upload(void);
/* device -> host star[] (every bound field), star_r, star_m, star_phi, N_MAX, scalars */
int cmcx_download(void);
/* replaces exit_cleanly for device errors */
void cmcx_set_abort(void (*handler)(int code, const char *where));
/* the device context, for callers that also use the cmcg_* API directly */
cmcg_ctx *cmcx_context(void);

/* ---- the reference's functions (prototypes as in include/cmc/cmc.h) ----
 * A file that also includes the reference's cmc.h defines
 * CMCX_NO_REFERENCE_PROTOTYPES first and takes these from there (cmc.h types
 * the rng argument as gsl_rng *; it is passed through untouched). */
#ifndef CMCX_NO_REFERENCE_PROTOTYPES
/* cmc_utils.c:2132 calc_timestep.  On the device it first closes the
 * previous step (Prev_Dt = Dt, tcount; the host's tcount wins if bound),
 * then does the step's tallies of cmc.c:246-257; sets Dt */
void calc_timestep(void *rng);
/* cmc_dynamics.c:17; writes star[].vr, vt, E, J, Y */
void dynamics_apply(double dt, void *rng);
/* cmc_utils.c:2153 and 2218: fused into the orbit kernel on the device;
 * these only keep the call sequence */
void energy_conservation1(void);
void energy_conservation2(void);
/* cmc_utils.c:2194; sets max_r and star[].rnew, vrnew, vtnew, X, r_peri, r_apo */
void new_orbits_calculate(void);
/* cmc_evolution_thr.c:944; the same, returning max_r */
double get_positions(void);
/* cmc_evolution_thr.c:443; star[].rnew of stripped stars, Rtidal, mass loss */
void tidally_strip_stars(void);
/* cmc_utils.c:368: its transfer rnew -> r runs inside qsorts_new on the device */
void ComputeIntermediateEnergy(void);
/* cmc_utils.c:2232; star[] records reordered by radius (whole records, every
 * field), escapers removed, N_MAX and N_MAX_NEW set */
void qsorts_new(void);
/* cmc_utils.c:2259; star_r, star_m from star[] */
void post_sort_comm(void);
/* cmc_utils.c:675; star_phi, N_MAX, Mtotal, Rtidal; returns N_MAX */
long potential_calculate(void);
/* cmc_utils.c:2006 */
void calc_potential_new(void);
/* cmc_utils.c:254 set_velocities3 via energy_conservation3 (cmc_utils.c:344);
 * star[].vr, vt */
void energy_conservation3(void);
/* cmc_utils.c:2018 compute_energy_new; star[].E, J and the energy scalars */
void compute_energy_new(void);
/* cmc_utils.c:112 */
double potential(double r);
#endif /* CMCX_NO_REFERENCE_PROTOTYPES */

#ifdef __cplusplus
}
#endif

#endif /* CMC_DROPIN_H */
