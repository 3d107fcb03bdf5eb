/* Single-rank MPI, the GSL subset and the HDF5 names that the reference's
 * hot-path TUs link against (TEST INFRASTRUCTURE for oracle/ref.mk; never
 * part of the product).
 *
 * MPI: one process.  Every collective hands back the caller's own
 * contribution (nothing to do with MPI_IN_PLACE); point-to-point calls reach
 * only rank 0 itself.  MPI_Abort returns control to the driver.
 *
 * GSL: the bracketing root solver find_root_vr drives (cmc_nr.c:500-603), as
 * Brent's method from brent1973.h, and inert gsl_rng handles (the step draws
 * from the reference's own taus113 state, never from a gsl_rng). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gsl/gsl_errno.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_roots.h"
#include "gsl/gsl_spline.h"
#include "mpi.h"

#include "../brent1973.h"

void cmcref_exit(int code) __attribute__((noreturn));
void cmcref_unreachable(const char *what) __attribute__((noreturn));

/* ------------------------------------------------------------------ MPI -- */

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm comm, int code) { (void)comm; cmcref_exit(code ? code : -1); }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void own_copy(const void *s, void *r, long bytes)
{
    if (s != MPI_IN_PLACE && s != r && bytes > 0) memmove(r, s, (size_t)bytes);
}

int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{
    (void)buf; (void)count; (void)t; (void)root; (void)comm;
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm;
    own_copy(s, r, (long)count * t);
    return MPI_SUCCESS;
}

int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
    (void)op; (void)root; (void)comm;
    own_copy(s, r, (long)count * t);
    return MPI_SUCCESS;
}

/* rank 0's receive buffer is undefined after an exclusive scan; left as is */
int MPI_Exscan(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)s; (void)r; (void)count; (void)t; (void)op; (void)comm;
    return MPI_SUCCESS;
}

int MPI_Gather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)root; (void)comm;
    own_copy(s, r, (long)sc * st);
    return MPI_SUCCESS;
}

int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)comm;
    own_copy(s, r, (long)sc * st);
    return MPI_SUCCESS;
}

int MPI_Allgatherv(const void *s, int sc, MPI_Datatype st, void *r, const int *rcs, const int *displs,
                   MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcs; (void)comm;
    if (s != MPI_IN_PLACE) own_copy(s, (char *)r + (long)displs[0] * rt, (long)sc * st);
    return MPI_SUCCESS;
}

int MPI_Alltoall(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)comm;
    own_copy(s, r, (long)sc * st);
    return MPI_SUCCESS;
}

int MPI_Alltoallv(const void *s, const int *scs, const int *sdispls, MPI_Datatype st, void *r, const int *rcs,
                  const int *rdispls, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcs; (void)comm;
    own_copy((const char *)s + (long)sdispls[0] * st, (char *)r + (long)rdispls[0] * rt, (long)scs[0] * st);
    return MPI_SUCCESS;
}

/* Point-to-point with one rank: a message to oneself is buffered until the
 * matching receive (as MPI's eager protocol delivers a short self-send; the
 * reference's calc_sigma_r exchanges its ghost stars that way, sending to and
 * receiving from rank (myid +- 1) % procs = 0).  Any other partner aborts. */
#define SELF_QUEUE 8
static struct {
    int tag;
    long bytes;
    void *data;
} self_q[SELF_QUEUE];
static int self_n;

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
    (void)comm;
    if (dest != 0 || self_n == SELF_QUEUE) cmcref_unreachable("MPI_Send to another rank");
    long bytes = (long)count * t;
    void *copy = malloc(bytes > 0 ? (size_t)bytes : 1);
    if (!copy) cmcref_unreachable("MPI_Send: out of memory");
    if (bytes > 0) memcpy(copy, buf, (size_t)bytes);
    self_q[self_n].tag = tag;
    self_q[self_n].bytes = bytes;
    self_q[self_n].data = copy;
    self_n++;
    return MPI_SUCCESS;
}

int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st)
{
    (void)comm;
    if (src != 0) cmcref_unreachable("MPI_Recv from another rank");
    for (int i = 0; i < self_n; ++i) {
        if (self_q[i].tag != tag) continue;
        long bytes = self_q[i].bytes, cap = (long)count * t;
        if (bytes > cap) cmcref_unreachable("MPI_Recv: message longer than the buffer");
        if (bytes > 0) memcpy(buf, self_q[i].data, (size_t)bytes);
        free(self_q[i].data);
        for (int j = i + 1; j < self_n; ++j) self_q[j - 1] = self_q[j];
        self_n--;
        if (st) st->MPI_SOURCE = 0, st->MPI_TAG = tag, st->MPI_ERROR = MPI_SUCCESS;
        return MPI_SUCCESS;
    }
    cmcref_unreachable("MPI_Recv with no matching send (one rank would block forever)");
}

int MPI_Sendrecv(const void *s, int sc, MPI_Datatype st, int dest, int stag, void *r, int rc, MPI_Datatype rt,
                 int src, int rtag, MPI_Comm comm, MPI_Status *status)
{
    (void)s; (void)sc; (void)st; (void)dest; (void)stag; (void)r; (void)rc; (void)rt; (void)src; (void)rtag;
    (void)comm; (void)status;
    cmcref_unreachable("MPI_Sendrecv with one rank");
}

int MPI_Comm_group(MPI_Comm comm, MPI_Group *g)
{
    (void)comm; (void)g;
    cmcref_unreachable("MPI_Comm_group");
}
int MPI_Group_incl(MPI_Group g, int n, const int ranks[], MPI_Group *out)
{
    (void)g; (void)n; (void)ranks; (void)out;
    cmcref_unreachable("MPI_Group_incl");
}
int MPI_Comm_create(MPI_Comm comm, MPI_Group g, MPI_Comm *out)
{
    (void)comm; (void)g; (void)out;
    cmcref_unreachable("MPI_Comm_create");
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *t)
{
    *t = (MPI_Datatype)count * old;
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype *t) { *t = MPI_DATATYPE_NULL; return MPI_SUCCESS; }
int MPI_Type_size(MPI_Datatype t, int *size) { *size = (int)t; return MPI_SUCCESS; }

/* ------------------------------------------------------------ GSL rng ---- */

static const gsl_rng_type taus2_type = {"taus2"}, mt_type = {"mt19937"};
const gsl_rng_type *gsl_rng_taus2 = &taus2_type;
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;
const gsl_rng_type *gsl_rng_default = &mt_type;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
    if (r) r->type = T;
    return r;
}
void gsl_rng_set(const gsl_rng *r, unsigned long seed) { ((gsl_rng *)r)->seed = seed; }
void gsl_rng_free(gsl_rng *r) { free(r); }
const gsl_rng_type *gsl_rng_env_setup(void) { return gsl_rng_default; }
double gsl_rng_uniform(const gsl_rng *r) { (void)r; cmcref_unreachable("gsl_rng_uniform"); }
unsigned long gsl_rng_get(const gsl_rng *r) { (void)r; cmcref_unreachable("gsl_rng_get"); }

gsl_error_handler_t *gsl_set_error_handler_off(void) { return NULL; }
const char *gsl_strerror(int gsl_errno) { (void)gsl_errno; return "gsl error"; }

/* ---------------------------------------------------------- GSL roots ---- */

struct gsl_root_fsolver {
    gsl_function *f;
    brent_t z;
    double root, x_lower, x_upper;
};

static const gsl_root_fsolver_type brent_type = {"brent"};
const gsl_root_fsolver_type *gsl_root_fsolver_brent = &brent_type;

gsl_root_fsolver *gsl_root_fsolver_alloc(const gsl_root_fsolver_type *T)
{
    (void)T;
    return (gsl_root_fsolver *)calloc(1, sizeof(gsl_root_fsolver));
}

void gsl_root_fsolver_free(gsl_root_fsolver *s) { free(s); }

int gsl_root_fsolver_set(gsl_root_fsolver *s, gsl_function *f, double x_lower, double x_upper)
{
    if (x_lower > x_upper) return GSL_EINVAL;
    s->f = f;
    s->root = 0.5 * (x_lower + x_upper);
    s->x_lower = x_lower;
    s->x_upper = x_upper;
    double fl = GSL_FN_EVAL(f, x_lower), fu = GSL_FN_EVAL(f, x_upper);
    if (!isfinite(fl) || !isfinite(fu)) return GSL_EBADFUNC;
    return brent_set(&s->z, fl, fu, x_lower, x_upper) ? GSL_EINVAL : GSL_SUCCESS;
}

/* one step: new abscissa, one evaluation there, then the bracket [b, c] */
int gsl_root_fsolver_iterate(gsl_root_fsolver *s)
{
    double x = brent_propose(&s->z);
    double fx = GSL_FN_EVAL(s->f, x);
    if (!isfinite(fx)) return GSL_EBADFUNC;
    brent_accept(&s->z, fx);
    s->root = s->z.b;
    if (s->z.exact) {
        s->x_lower = s->x_upper = s->z.b;
    } else {
        s->x_lower = s->z.b < s->z.c ? s->z.b : s->z.c;
        s->x_upper = s->z.b < s->z.c ? s->z.c : s->z.b;
    }
    return GSL_SUCCESS;
}

double gsl_root_fsolver_root(const gsl_root_fsolver *s) { return s->root; }
double gsl_root_fsolver_x_lower(const gsl_root_fsolver *s) { return s->x_lower; }
double gsl_root_fsolver_x_upper(const gsl_root_fsolver *s) { return s->x_upper; }

/* documented tests: |hi - lo| < epsabs + epsrel * min(|lo|, |hi|) (an
 * interval straddling zero uses 0 for the minimum); |x1 - x0| < epsabs +
 * epsrel * |x1| */
int gsl_root_test_interval(double x_lower, double x_upper, double epsabs, double epsrel)
{
    double al = fabs(x_lower), au = fabs(x_upper);
    double min_abs = ((x_lower > 0.0 && x_upper > 0.0) || (x_lower < 0.0 && x_upper < 0.0)) ? (al < au ? al : au)
                                                                                           : 0.0;
    return fabs(x_upper - x_lower) < epsabs + epsrel * min_abs ? GSL_SUCCESS : GSL_CONTINUE;
}

int gsl_root_test_delta(double x1, double x0, double epsabs, double epsrel)
{
    return fabs(x1 - x0) < epsabs + epsrel * fabs(x1) ? GSL_SUCCESS : GSL_CONTINUE;
}

/* --------------------------------------------------------- GSL spline ---- */

static const gsl_interp_type linear_type = {"linear"}, cspline_type = {"cspline"};
const gsl_interp_type *gsl_interp_linear = &linear_type;
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, unsigned long n)
{
    (void)T; (void)n;
    cmcref_unreachable("gsl_spline_alloc");
}
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], unsigned long n)
{
    (void)s; (void)xa; (void)ya; (void)n;
    cmcref_unreachable("gsl_spline_init");
}
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a)
{
    (void)s; (void)x; (void)a;
    cmcref_unreachable("gsl_spline_eval");
}
void gsl_spline_free(gsl_spline *s) { (void)s; }
gsl_interp_accel *gsl_interp_accel_alloc(void) { cmcref_unreachable("gsl_interp_accel_alloc"); }
void gsl_interp_accel_free(gsl_interp_accel *a) { (void)a; }
