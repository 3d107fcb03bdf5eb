/* cmc_gpu_glue.c -- the one file a maintainer adds to the reference's build
 * (as src/cmc/cmc_gpu_glue.c) to run its Henon step on libcmcgpu.so through
 * libcmc_dropin.so.  It is compiled with the reference's own headers and is
 * not part of this repository's libraries; tests/test_cpu_glue.py compiles it
 * against include/cmc/cmc.h and links it with the reference's objects.
 *
 * cmc_gpu_bind() describes where the reference keeps its host state (star[],
 * star_r/m/phi, clus, the step scalars, the .ini parameters) and binds it;
 * call it once after parser(), get_star_data() and the tidal radius set-up,
 * before the first calc_potential_new() (cmc.c:153). */
#include <stddef.h>
#include "cmc.h"
#include "cmc_vars.h"
#define CMCX_NO_REFERENCE_PROTOTYPES  /* cmc.h already declares the replaced functions */
#include "cmc_dropin.h"          /* from this repository's include/ */

static void gpu_abort(int code, const char *where) { exit_cleanly(code, (char *)where); }

/* after parser(), get_star_data() and the tidal radius set-up, before the
 * first calc_potential_new() of cmc.c:153 */
void cmc_gpu_bind(void) {
    cmcx_host h;
    cmcx_default_host(&h);
    h.star = star;  h.star_size = sizeof(star_t);
    h.off_r = offsetof(star_t, r);         h.off_vr = offsetof(star_t, vr);
    h.off_vt = offsetof(star_t, vt);       h.off_m = offsetof(star_t, m);
    h.off_E = offsetof(star_t, E);         h.off_J = offsetof(star_t, J);
    h.off_id = offsetof(star_t, id);       h.id_bytes = sizeof(star[0].id);
    h.off_rnew = offsetof(star_t, rnew);   h.off_vrnew = offsetof(star_t, vrnew);
    h.off_vtnew = offsetof(star_t, vtnew); h.off_rOld = offsetof(star_t, rOld);
    h.off_X = offsetof(star_t, X);         h.off_Y = offsetof(star_t, Y);
    h.off_r_peri = offsetof(star_t, r_peri); h.off_r_apo = offsetof(star_t, r_apo);
    h.star_r = star_r; h.star_m = star_m; h.star_phi = star_phi;
    h.N_STAR_DIM = N_STAR_DIM;
    h.N_MAX = &clus.N_MAX; h.N_MAX_NEW = &clus.N_MAX_NEW; h.tcount = &tcount;
    h.Dt = &Dt; h.Mtotal = &Mtotal; h.Rtidal = &Rtidal; h.max_r = &max_r;
    h.Eescaped = &Eescaped; h.Jescaped = &Jescaped; h.TidalMassLoss = &TidalMassLoss;
    h.Etidal = &Etidal;
    h.sync_each = 1;            /* 0 + cmcx_download() before output, when SE/encounters are off */

    cmcg_params p;
    cmcg_default_params(&p);
    p.N_STAR = clus.N_STAR; p.AVEKERNEL = AVEKERNEL; p.GAMMA = GAMMA;
    p.THETASEMAX = THETASEMAX; p.PERTURB = PERTURB; p.RELAXATION = RELAXATION;
    p.TIDALLY_STRIP_STARS = TIDALLY_STRIP_STARS; p.TIDAL_TREATMENT = TIDAL_TREATMENT;
    p.orbit_r = orbit_r; p.cenma_m = cenma.m; p.seed = IDUM;
    p.apsides_max_iter = APSIDES_MAX_ITER; p.apsides_precision = APSIDES_PRECISION;
    p.apsides_convergence = APSIDES_CONVERGENCE;

    cmcx_set_abort(gpu_abort);
    if (cmcx_bind(&h, &p)) exit_cleanly(-1, __FUNCTION__);
}
