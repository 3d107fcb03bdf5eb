/* Definitions for the symbols the reference's hot-path TUs name but that live
 * in TUs oracle/ref.mk does not compile (TEST INFRASTRUCTURE).  They belong to
 * subsystems the plain Henon step never enters -- strong encounters
 * (Fewbody), stellar evolution (BSE), the search grid, the black-hole loss
 * cone, snapshots -- so each one stops the driver call with its name.
 * close_buffers() is the exception: exit_cleanly() calls it before
 * MPI_Abort, and with no output files open it has nothing to do. */
void cmcref_unreachable(const char *what) __attribute__((noreturn));

void close_buffers(void) {}

#define UNREACHABLE(name) \
    void name(void) { cmcref_unreachable(#name); }

UNREACHABLE(bh_rand_walk)
UNREACHABLE(binbin)
UNREACHABLE(binsingle)
UNREACHABLE(compress_binary)
UNREACHABLE(cp_SEvars_to_newbinary)
UNREACHABLE(cp_SEvars_to_newstar)
UNREACHABLE(cp_SEvars_to_star)
UNREACHABLE(cp_binmemb_to_star)
UNREACHABLE(cp_m_to_newstar)
UNREACHABLE(cp_m_to_star)
UNREACHABLE(cp_starSEvars_to_binmember)
UNREACHABLE(cp_starmass_to_binmember)
UNREACHABLE(fb_bh_merger)
UNREACHABLE(fb_downsync)
UNREACHABLE(fb_free_hier)
UNREACHABLE(fb_malloc_hier)
UNREACHABLE(fb_n_hier)
UNREACHABLE(fb_sprint_hier)
UNREACHABLE(fb_sprint_hier_hr)
UNREACHABLE(merge_two_stars)
UNREACHABLE(print_2Dsnapshot)
UNREACHABLE(remove_old_star)
UNREACHABLE(search_grid_get_interval)
UNREACHABLE(sscollision_do)
