/* Force-included into every reference TU that oracle/ref.mk compiles (TEST
 * INFRASTRUCTURE; never part of the product).
 *
 * Draw injection.  ref.mk compiles each TU with
 *     -DCMCREF_DRAW_ARGS='TU,__LINE__,IDX,TRIAL'
 * and the macro below turns every rng_t113_dbl_new(st) of the TU into
 * cmcref_draw(TU, __LINE__, IDX, TRIAL), where IDX names the star whose draw it is at that TU's hot-path sites and
 * TRIAL the rejection-loop counter (0 where there is none):
 *
 *   TU 1 cmc_dynamics.c         :406 P_enc, :465 psi        IDX = k
 *   TU 2 cmc_dynamics_helper.c  :839 Y                      IDX = k
 *   TU 3 cmc_evolution_thr.c    :863 X, :867 g0, :923 sign  IDX = j, TRIAL = k
 *
 * cmcref_draw maps (TU, line) to the counter-draw site, star[IDX].id and draw
 * number that the oracle and the kernels key Philox4x32-10 with, or, in the
 * untouched mode, forwards to the reference's own rng_t113_dbl_new(curr_st).
 * Any other draw site of these TUs aborts: none is reached on the plain
 * Henon step.  The file-scope j and k below only give the macro a name to
 * bind in functions that have no local j or k; a local always shadows them,
 * and cmcref_draw refuses every site outside the table above. */
#ifndef CMCREF_INJECT_H
#define CMCREF_INJECT_H
#include <stdlib.h>
#include <string.h>

/* the generator's own declarations first (the header is guarded), so that
 * only the calls are rerouted */
#include "taus113-v2.h"

double cmcref_draw(int tu, int line, long idx, long trial);
#define rng_t113_dbl_new(st) cmcref_draw(CMCREF_DRAW_ARGS)

static long j __attribute__((unused)) = -1;
static long k __attribute__((unused)) = -1;

/* exit() inside the reference's TUs (find_root_vr, for one) returns control to
 * the driver instead of ending the test process; see refdrive.c. */
void cmcref_exit(int code) __attribute__((noreturn));
#endif
