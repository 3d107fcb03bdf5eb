// cmc_dropin.cpp -- the reference's hot-path functions under their own names
// (include/cmc_dropin.h), on the public C ABI of libcmcgpu.so.
//
// Each function runs its device phase and then, with sync_each, writes the
// host memory the reference's definition writes: the star[] fields listed in
// the header, star_r / star_m / star_phi, clus.N_MAX / N_MAX_NEW and the bound
// scalars.  qsorts_new reorders whole star_t records (every field the device
// does not hold travels with its star), matching records by star id.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "cmc_dropin.h"

namespace {

struct State {
    cmcx_host h{};
    cmcg_ctx *ctx = nullptr;
    bool stepped = false;
    void (*abort_fn)(int, const char *) = nullptr;
    std::vector<double> buf;
    std::vector<int64_t> ids;
};
State S;

void default_abort(int code, const char *where)
{
    fprintf(stderr, "cmc_dropin: %s: device error %d\n", where, code);
    exit(code > 0 ? code : 1);
}

void fail(int code, const char *where) { (S.abort_fn ? S.abort_fn : default_abort)(code, where); }

char *rec(long i) { return (char *)S.h.star + (size_t)i * S.h.star_size; }
double &fld(long i, long off) { return *(double *)(rec(i) + off); }

int64_t get_id(long i)
{
    if (S.h.id_bytes == 4) {
        int32_t v;
        memcpy(&v, rec(i) + S.h.off_id, 4);
        return v;
    }
    int64_t v;
    memcpy(&v, rec(i) + S.h.off_id, 8);
    return v;
}

void set_id(long i, int64_t v)
{
    if (S.h.id_bytes == 4) {
        const int32_t w = (int32_t)v;
        memcpy(rec(i) + S.h.off_id, &w, 4);
    } else {
        memcpy(rec(i) + S.h.off_id, &v, 8);
    }
}

// First device error since the last call -> the abort handler.
bool check(const char *where, int rc = 0)
{
    if (rc) {
        fail(rc, where);
        return false;
    }
    int c = 0;
    long idx = 0;
    const int e = cmcg_last_error(S.ctx, &c, &idx);
    if (e) {
        fail(e, where);
        return false;
    }
    return true;
}

double scalar(const char *name)
{
    double v = 0.0;
    cmcg_get_scalar(S.ctx, 0, name, &v);
    return v;
}

void put_scalar(double *dst, const char *name)
{
    if (dst) *dst = scalar(name);
}

long nstars() { return cmcg_nstars(S.ctx, 0); }

// per-star device field (stars 1..N) -> star[i].off
void pull_field(const char *name, long off)
{
    if (off < 0) return;
    const long n = nstars();
    S.buf.resize((size_t)n + 2);
    const long got = cmcg_get_field(S.ctx, 0, name, S.buf.data(), n + 2);
    for (long i = 0; i < got; ++i) fld(i + 1, off) = S.buf[(size_t)i];
}

// global device array (indices 0..N+1) -> host array
void pull_global(const char *name, double *dst)
{
    if (!dst) return;
    S.buf.resize((size_t)S.h.N_STAR_DIM);
    const long got = cmcg_get_field(S.ctx, 0, name, S.buf.data(), S.h.N_STAR_DIM);
    if (got > 0) memcpy(dst, S.buf.data(), (size_t)got * sizeof(double));
}

void pull_counts()
{
    const long n = nstars();
    if (S.h.N_MAX) *S.h.N_MAX = (long)scalar("N_MAX");
    if (S.h.N_MAX_NEW) *S.h.N_MAX_NEW = n;
}

int push_stars()
{
    const long N = *S.h.N_MAX_NEW;
    std::vector<double> r(N), m(N), vr(N), vt(N), E(N), J(N);
    std::vector<int64_t> id(N);
    for (long i = 1; i <= N; ++i) {
        r[i - 1] = fld(i, S.h.off_r);
        m[i - 1] = fld(i, S.h.off_m);
        vr[i - 1] = fld(i, S.h.off_vr);
        vt[i - 1] = fld(i, S.h.off_vt);
        E[i - 1] = fld(i, S.h.off_E);
        J[i - 1] = fld(i, S.h.off_J);
        id[i - 1] = get_id(i);
    }
    return cmcg_put_stars(S.ctx, 0, N, r.data(), m.data(), vr.data(), vt.data(), E.data(), J.data(), id.data());
}

}  // namespace

extern "C" {

void cmcx_default_host(cmcx_host *h)
{
    memset(h, 0, sizeof(*h));
    h->off_r = h->off_vr = h->off_vt = h->off_m = h->off_E = h->off_J = h->off_id = -1;
    h->off_rnew = h->off_vrnew = h->off_vtnew = h->off_rOld = h->off_X = h->off_Y = -1;
    h->off_r_peri = h->off_r_apo = -1;
    h->id_bytes = 8;
    h->sync_each = 1;
}

void cmcx_set_abort(void (*handler)(int, const char *)) { S.abort_fn = handler; }

cmcg_ctx *cmcx_context(void) { return S.ctx; }

int cmcx_bind(const cmcx_host *h, const cmcg_params *params)
{
    if (!h || !params || !h->star || h->star_size == 0 || !h->N_MAX || !h->N_MAX_NEW) return CMCG_ERR_ARG;
    if (h->off_r < 0 || h->off_vr < 0 || h->off_vt < 0 || h->off_m < 0 || h->off_E < 0 || h->off_J < 0 ||
        h->off_id < 0 || (h->id_bytes != 4 && h->id_bytes != 8))
        return CMCG_ERR_ARG;
    if (params->N_STAR < 1 || h->N_STAR_DIM < *h->N_MAX + 2) return CMCG_ERR_ARG;
    cmcx_unbind();
    S.h = *h;
    S.stepped = false;
    const long N = *h->N_MAX, cap = h->N_STAR_DIM - 2;
    int rc = cmcg_create(&S.ctx, 1, &cap, params);
    if (rc) return rc;
    // cmcg_load sets the cluster's scalars (N_STAR, madhoc, sentinels); the
    // stars are then replaced bit for bit by the stored values
    std::vector<double> r(N), m(N), vr(N), vt(N);
    std::vector<int64_t> id(N);
    const double NSTAR = (double)params->N_STAR;
    for (long i = 1; i <= N; ++i) {
        r[i - 1] = fld(i, h->off_r);
        m[i - 1] = fld(i, h->off_m) / NSTAR;
        vr[i - 1] = fld(i, h->off_vr);
        vt[i - 1] = fld(i, h->off_vt);
        id[i - 1] = get_id(i);
    }
    rc = cmcg_load(S.ctx, 0, N, r.data(), m.data(), vr.data(), vt.data(), id.data());
    if (!rc) rc = push_stars();
    if (!rc) rc = cmcg_synchronize(S.ctx);
    if (rc) cmcx_unbind();
    return rc;
}

void cmcx_unbind(void)
{
    if (S.ctx) cmcg_destroy(S.ctx);
    S.ctx = nullptr;
}

int cmcx_upload(void)
{
    if (!S.ctx) return CMCG_ERR_STATE;
    return push_stars();
}

int cmcx_download(void)
{
    if (!S.ctx) return CMCG_ERR_STATE;
    const cmcx_host &h = S.h;
    pull_field("r", h.off_r);
    pull_field("m", h.off_m);
    pull_field("vr", h.off_vr);
    pull_field("vt", h.off_vt);
    pull_field("E", h.off_E);
    pull_field("J", h.off_J);
    pull_field("rnew", h.off_rnew);
    pull_field("vrnew", h.off_vrnew);
    pull_field("vtnew", h.off_vtnew);
    pull_field("rOld", h.off_rOld);
    pull_field("X", h.off_X);
    pull_field("Y", h.off_Y);
    pull_field("r_peri", h.off_r_peri);
    pull_field("r_apo", h.off_r_apo);
    const long n = nstars();
    S.ids.resize((size_t)n + 1);
    const long got = cmcg_get_ids(S.ctx, 0, S.ids.data(), n + 1);
    for (long i = 0; i < got; ++i) set_id(i + 1, S.ids[(size_t)i]);
    pull_global("star_r", h.star_r);
    pull_global("star_m", h.star_m);
    pull_global("star_phi", h.star_phi);
    pull_counts();
    put_scalar(h.Dt, "Dt");
    put_scalar(h.Mtotal, "Mtotal");
    put_scalar(h.Rtidal, "Rtidal");
    put_scalar(h.max_r, "max_r");
    put_scalar(h.Etot, "Etot");
    put_scalar(h.KE, "KE");
    put_scalar(h.PE, "PE");
    return CMCG_OK;
}

void calc_timestep(void *rng)
{
    (void)rng;
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (S.stepped && !check(__func__, cmcg_end_step(S.ctx))) return;
    if (S.h.tcount && !check(__func__, cmcg_set_scalar(S.ctx, 0, "tcount", (double)*S.h.tcount))) return;
    if (!check(__func__, cmcg_begin_step(S.ctx))) return;
    if (!check(__func__, cmcg_calc_timestep(S.ctx))) return;
    S.stepped = true;
    put_scalar(S.h.Dt, "Dt");
}

void dynamics_apply(double dt, void *rng)
{
    (void)rng;
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (!check(__func__, cmcg_dynamics_apply(S.ctx, dt))) return;
    if (!S.h.sync_each) return;
    pull_field("vr_rel", S.h.off_vr);
    pull_field("vt_rel", S.h.off_vt);
    pull_field("E", S.h.off_E);
    pull_field("J", S.h.off_J);
    pull_field("Y", S.h.off_Y);
}

void energy_conservation1(void) {}
void energy_conservation2(void) {}
void ComputeIntermediateEnergy(void) {}

double get_positions(void)
{
    if (!S.ctx) {
        fail(CMCG_ERR_STATE, __func__);
        return 0.0;
    }
    if (!check(__func__, cmcg_new_orbits_calculate(S.ctx))) return 0.0;
    const double max_r = scalar("max_r");
    if (S.h.max_r) *S.h.max_r = max_r;
    if (S.h.sync_each) {
        pull_field("rnew", S.h.off_rnew);
        pull_field("vrnew", S.h.off_vrnew);
        pull_field("vtnew", S.h.off_vtnew);
        pull_field("X", S.h.off_X);
        pull_field("r_peri", S.h.off_r_peri);
        pull_field("r_apo", S.h.off_r_apo);
    }
    return max_r;
}

void new_orbits_calculate(void) { (void)get_positions(); }

void tidally_strip_stars(void)
{
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (!check(__func__, cmcg_tidally_strip_stars(S.ctx))) return;
    put_scalar(S.h.Rtidal, "Rtidal");
    put_scalar(S.h.TidalMassLoss, "TidalMassLoss");
    put_scalar(S.h.Eescaped, "Eescaped");
    put_scalar(S.h.Jescaped, "Jescaped");
    put_scalar(S.h.Etidal, "Etidal");
    if (S.h.sync_each) pull_field("rnew", S.h.off_rnew);
}

void qsorts_new(void)
{
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    const long nold = *S.h.N_MAX_NEW;
    std::unordered_map<int64_t, long> where;
    if (S.h.sync_each) {
        where.reserve((size_t)nold * 2);
        for (long i = 1; i <= nold; ++i) where.emplace(get_id(i), i);
    }
    if (!check(__func__, cmcg_qsorts_new(S.ctx))) return;
    const long n = nstars();
    if (S.h.sync_each) {
        // whole records in the new order, then the fields the device changed
        S.ids.resize((size_t)n + 1);
        const long got = cmcg_get_ids(S.ctx, 0, S.ids.data(), n + 1);
        std::vector<char> old((size_t)nold * S.h.star_size);
        memcpy(old.data(), rec(1), old.size());
        for (long i = 0; i < got; ++i) {
            auto it = where.find(S.ids[(size_t)i]);
            if (it == where.end()) return fail(CMCG_ERR_STATE, __func__);
            memcpy(rec(i + 1), old.data() + (size_t)(it->second - 1) * S.h.star_size, S.h.star_size);
        }
        pull_field("r", S.h.off_r);
        pull_field("m", S.h.off_m);
        pull_field("vr", S.h.off_vr);
        pull_field("vt", S.h.off_vt);
        pull_field("rOld", S.h.off_rOld);
    }
    if (S.h.N_MAX) *S.h.N_MAX = n;
    if (S.h.N_MAX_NEW) *S.h.N_MAX_NEW = n;
}

void post_sort_comm(void)
{
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (!S.h.sync_each) return;
    pull_global("star_r", S.h.star_r);
    pull_global("star_m", S.h.star_m);
}

long potential_calculate(void)
{
    if (!S.ctx) {
        fail(CMCG_ERR_STATE, __func__);
        return 0;
    }
    if (!check(__func__, cmcg_calc_potential(S.ctx))) return 0;
    const long N = (long)scalar("N_MAX");
    if (S.h.N_MAX) *S.h.N_MAX = N;
    put_scalar(S.h.Mtotal, "Mtotal");
    put_scalar(S.h.Rtidal, "Rtidal");
    if (S.h.sync_each) pull_global("star_phi", S.h.star_phi);
    return N;
}

void calc_potential_new(void) { (void)potential_calculate(); }

void energy_conservation3(void)
{
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (!check(__func__, cmcg_energy_conservation3(S.ctx))) return;
    if (!S.h.sync_each) return;
    pull_field("vr", S.h.off_vr);
    pull_field("vt", S.h.off_vt);
}

void compute_energy_new(void)
{
    if (!S.ctx) return fail(CMCG_ERR_STATE, __func__);
    if (!check(__func__, cmcg_compute_energy(S.ctx))) return;
    put_scalar(S.h.Etot, "Etot");
    put_scalar(S.h.KE, "KE");
    put_scalar(S.h.PE, "PE");
    put_scalar(S.h.Eescaped, "Eescaped");
    put_scalar(S.h.Jescaped, "Jescaped");
    put_scalar(S.h.Etidal, "Etidal");
    if (!S.h.sync_each) return;
    pull_field("E", S.h.off_E);
    pull_field("J", S.h.off_J);
}

double potential(double r)
{
    double v = 0.0;
    if (!S.ctx) {
        fail(CMCG_ERR_STATE, __func__);
        return v;
    }
    check(__func__, cmcg_potential(S.ctx, 0, r, &v));
    return v;
}

}  // extern "C"
