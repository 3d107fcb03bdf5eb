// cmcg_orbit.cu -- new orbits (get_positions) and tidal stripping.
//
// k_orbit restates get_positions_loop (cmc_evolution_thr.c:784-937) with
// calc_orbit_new (cmc_orbit.c:413-540), get_positive_Q_index (30-59),
// find_zero_Q (cmc_nr.c:316-383), set_a_b (cmc_orbit.c:722-740), and replaces
// the GSL Brent search of find_root_vr (cmc_nr.c:500-603) by a safeguarded
// Newton/bisection iteration with the same bracket, tolerance and residual
// checks.  One thread owns one star; the Q sign tests of the bisections are
// evaluated in double-double because the reference evaluates them in long
// double.  It also folds in energy_conservation1/2 (cmc_utils.c:2153-2228):
// the one quantity set_velocities3 later needs from them,
//   ec_pre = vold^2 + 2(1-q)(Uoldrold - Uoldrnew),  q = 1/2,
// is formed here, evaluated exactly as the reference's first partial sum.
//
// k_tidal restates the iteration of tidally_strip_stars
// (cmc_evolution_thr.c:443-646) in one cooperative launch, its passes
// separated by a bounded grid barrier.
#include <cuda_bf16.h>
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {

constexpr int BISECT_LIMIT = 80;

// Counts of the orbit phase's rare branches over every launch on this device
// since the last reset (cmcg_orbit_counters): table probes whose sign the
// FP32 and float-float stages left to the FP64 stage, probes that went on to
// double-double, and apsides outside their closed-form interval (the
// find_root_vr fallback).  A file-scope array, so that the hot kernels carry
// no extra pointer; the increments sit only on those branches.
__device__ unsigned long long g_orbit_rare[CMCG_ORBIT_NCOUNTERS];

struct OrbitCtx {
    const double *__restrict__ r, *__restrict__ phi, *__restrict__ inv_r;
    const float4 *__restrict__ rphif;
    long long N_MAX, j;
    double E, J, rj, mj, invN, cenma_m, madhoc;
    QF32 s;
};

static __device__ __forceinline__ double fq(const OrbitCtx &o, long long k)
{
    return function_q_dd(__ldg(o.r + k), __ldg(o.phi + k), o.E, o.J, o.rj, o.mj, o.invN);
}

// Sign of function_q at table point k: certified FP32 first, then certified
// float-float (still on the FP32 pipe), then certified FP64 from the 1/r
// table, double-double only when all lie within their error bounds (a table
// point within ~1e-15 of a root).
static __device__ __forceinline__ int fq_sign_at(const OrbitCtx &o, long long k, float4 rp)
{
    const bool ge = k >= o.j;
    int s = fq_sign_f32(o.s, rp, ge);
    if (s) return s;
    s = fq_sign_ff(o.s, rp, ge);
    if (s) return s;
    atomicAdd(&g_orbit_rare[CMCG_ORBIT_SIGN_F64], 1ull);
    s = fq_sign_f64(o.s, __ldg(o.inv_r + k), __ldg(o.phi + k), ge);
    if (s) return s;
    atomicAdd(&g_orbit_rare[CMCG_ORBIT_SIGN_DD], 1ull);
    const double q = fq(o, k);
    return (q > 0.0) - (q < 0.0);
}

static __device__ __forceinline__ int fq_sign(const OrbitCtx &o, long long k)
{
    return fq_sign_at(o, k, __ldg(o.rphif + k));
}

// Pull a table entry into L2 (no register holds it).  In clusters whose
// tables exceed L2 (from PREFETCH_MIN_STARS stars: a 64 MB FP32 table beside
// 192 MB of FP64 ones), the bisections ask for the two entries their next
// round can probe while this round's probe is in flight, so that the next
// probe finds its sector in L2 instead of waiting on DRAM.  At 10^7 stars the
// orbit kernel took 11.16 against 11.38 ms a step with them; at 10^6 stars,
// where the tables sit in L2, the extra L2 requests cost 4.6%, and at 10^8
// stars, where the unused half of the prefetched sectors competes for DRAM
// bandwidth, 202 against 138 ms: hence both bounds.
constexpr long long PREFETCH_MIN_STARS = 1ll << 22, PREFETCH_MAX_STARS = 1ll << 24;
static __device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// find_zero_Q, cmc_nr.c:316-383 (bounded; returns -1 if it does not terminate).
// The reference compares the end-point values to choose the direction; when
// their signs differ the signs decide it, and only same-signed ends are
// evaluated in double-double and compared.  The bisection only needs signs.
// (Fetching several levels of probes at once measured slower: the extra
// live entries cost occupancy and spills that outweigh the shorter chain.)
static __device__ long long find_zero_Q(const OrbitCtx &o, long long kmin, long long kmax)
{
    const int smin = fq_sign(o, kmin), smax = fq_sign(o, kmax);
    const bool up = (smin != smax) ? (smin < smax) : (fq(o, kmin) < fq(o, kmax));
    const bool pf = o.N_MAX >= PREFETCH_MIN_STARS && o.N_MAX < PREFETCH_MAX_STARS;
    int it = 0;
    if (up) {
        do {
            const long long ktry = (kmin + kmax + 1) / 2;
            if (pf) {  // the next probe, either way (within [kmin, kmax])
                prefetch_l2(o.rphif + (ktry + kmax + 1) / 2);
                prefetch_l2(o.rphif + (kmin + ktry) / 2);
            }
            if (fq_sign(o, ktry) < 0)
                kmin = ktry;
            else
                kmax = ktry - 1;
            if (++it > BISECT_LIMIT) return -1;
        } while (kmax != kmin);
    } else {
        do {
            const long long ktry = (kmin + kmax + 1) / 2;
            if (pf) {
                prefetch_l2(o.rphif + (ktry + kmax + 1) / 2);
                prefetch_l2(o.rphif + (kmin + ktry) / 2);
            }
            if (fq_sign(o, ktry) > 0)
                kmin = ktry;
            else
                kmax = ktry - 1;
            if (++it > BISECT_LIMIT) return -1;
        } while (kmax != kmin);
    }
    return kmin;
}

// set_a_b, cmc_orbit.c:722-740; 1/r from the reciprocal table (same rounding)
static __device__ __forceinline__ void set_a_b(const OrbitCtx &o, long long k, double *a, double *b)
{
    if (k == 0) {
        *a = -o.cenma_m * o.madhoc;
        *b = o.phi[1] + o.cenma_m * o.madhoc / o.r[1] + o.mj * o.madhoc / o.rj;
    } else {
        // the divisions by r_k and r_k+1 use the stored reciprocals (div_rcp)
        const double rk = o.r[k], rk1 = o.r[k + 1], ik = o.inv_r[k], ik1 = o.inv_r[k + 1];
        const long long rjb = dbits(o.rj);  // positive radii compare as their bit patterns
        const double Uk = o.phi[k] + ((dbits(rk) >= rjb) ? __dmul_rn(div_rcp(o.mj, rk, ik), o.invN) : o.s.pjd);
        const double Uk1 = o.phi[k + 1] + ((dbits(rk1) >= rjb) ? __dmul_rn(div_rcp(o.mj, rk1, ik1), o.invN) : o.s.pjd);
        const double den = ik1 - ik;
        *a = (Uk1 - Uk) / den;
        *b = (div_rcp(Uk, rk1, ik1) - div_rcp(Uk1, rk, ik)) / den;
    }
}

// calc_pot_within_interval, cmc_nr.c:230-259
static __device__ __forceinline__ double pot_within(const OrbitCtx &o, double x, long long k, bool *ok)
{
    const double rk = o.r[k], rk1 = o.r[k + 1];
    if (x < (rk - CMCG_DBL_EPSILON) || x > rk1 + CMCG_DBL_EPSILON) {
        *ok = false;
        return 0.0;
    }
    if (fabs(x - rk) < CMCG_DBL_EPSILON) return o.phi[k];
    if (fabs(x - rk1) < CMCG_DBL_EPSILON) return o.phi[k + 1];
    if (x < o.r[1]) return o.phi[0] - o.cenma_m * o.madhoc / x;
    return o.phi[k] + (o.phi[k + 1] - o.phi[k]) * (o.inv_r[k] - 1.0 / x) / (o.inv_r[k] - o.inv_r[k + 1]);
}

// vr^2 within interval k (calc_vr_within_interval, cmc_nr.c:267-278)
static __device__ __forceinline__ double vr2_in(const OrbitCtx &o, double x, long long k, bool *ok)
{
    const double pot = pot_within(o, x, k, ok);
    return function_q_dd(x, pot, o.E, o.J, o.rj, o.mj, o.invN);
}

// d(vr^2)/dr inside interval k, for the Newton step
static __device__ __forceinline__ double dvr2_in(const OrbitCtx &o, double x, long long k)
{
    const double ix = 1.0 / x;
    double dpot;
    if (x < o.r[1])
        dpot = o.cenma_m * o.madhoc * ix * ix;
    else
        dpot = (o.phi[k + 1] - o.phi[k]) / (o.inv_r[k] - o.inv_r[k + 1]) * ix * ix;
    const double dphis = (x >= o.rj) ? -o.mj * o.invN * ix * ix : 0.0;
    return -2.0 * (dpot + dphis) + 2.0 * o.J * o.J * ix * ix * ix;
}

// Root of vr^2 in [r_k, r_k+1]: safeguarded Newton with bisection fallback,
// converged when the bracket satisfies |hi-lo| < eps + eps*min(|lo|,|hi|)
// (the gsl_root_test_interval criterion of cmc_nr.c:535), then the residual
// checks of cmc_nr.c:584-597.
static __device__ double find_root_vr(const OrbitCtx &o, long long k, double prec, long long maxit, int *err)
{
    atomicAdd(&g_orbit_rare[CMCG_ORBIT_ROOT_VR], 1ull);
    bool ok = true;
    double lo = o.r[k], hi = o.r[k + 1];
    double flo = vr2_in(o, lo, k, &ok), fhi = vr2_in(o, hi, k, &ok);
    if (!ok) {
        *err = CMCG_ERR_POT_INTERVAL;
        return 0.0;
    }
    if ((flo >= 0.0 ? 1 : -1) == (fhi >= 0.0 ? 1 : -1)) {
        *err = CMCG_ERR_ROOT_SIGNS;
        return 0.0;
    }
    const double a0 = lo, b0 = hi;
    double x = (fabs(flo) < fabs(fhi)) ? lo : hi, fx = (fabs(flo) < fabs(fhi)) ? flo : fhi;
    bool conv = false;
    for (long long it = 0; it < maxit; ++it) {
        if (fabs(hi - lo) < prec + prec * fmin(fabs(lo), fabs(hi))) {
            conv = true;
            break;
        }
        const double d = dvr2_in(o, x, k);
        double xn = (d != 0.0) ? x - fx / d : 0.5 * (lo + hi);
        // bisect when Newton leaves the bracket or lands on an end
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        // close the bracket from the far side once Newton steps become tiny
        const double tol = 0.25 * (prec + prec * fmin(fabs(lo), fabs(hi)));
        if (fabs(xn - x) < tol) xn = (fabs(xn - lo) < fabs(hi - xn)) ? fmin(xn + tol, 0.5 * (xn + hi)) : fmax(xn - tol, 0.5 * (xn + lo));
        x = xn;
        fx = vr2_in(o, x, k, &ok);
        if (!ok) {
            *err = CMCG_ERR_POT_INTERVAL;
            return 0.0;
        }
        if (fx == 0.0) {
            lo = hi = x;
            conv = true;
            break;
        }
        if ((fx >= 0.0) == (flo >= 0.0)) {
            lo = x;
            flo = fx;
        } else {
            hi = x;
            fhi = fx;
        }
    }
    if (!conv) {
        *err = CMCG_ERR_ROOT_NOCONV;
        return 0.0;
    }
    (void)a0;
    (void)b0;
    double apsis = x;
    if (vr2_in(o, apsis, k, &ok) < 0.0) {
        if (vr2_in(o, lo, k, &ok) < 0.0) apsis = hi;
        if (vr2_in(o, hi, k, &ok) < 0.0) apsis = lo;
    }
    if (vr2_in(o, apsis, k, &ok) < 0.0) {
        *err = CMCG_ERR_ROOT_NEG;
        return 0.0;
    }
    return apsis;
}

// The per-star context of the orbit computation (E includes PHI_S(r_j)).
static __device__ __forceinline__ OrbitCtx make_orbit_ctx(const Cluster &C, const Fields &f, long long j, double E,
                                                          double J, double rj, double mj, double ps)
{
    const Scalars *sc = C.sc;
    const long long off = C.off;
    OrbitCtx o;
    o.r = f.r + off;
    o.phi = f.phi + off;
    o.inv_r = f.inv_r + off;
    o.rphif = f.rphif + off;
    o.N_MAX = sc->N_MAX;
    o.j = j;
    o.E = E;
    o.J = J;
    o.rj = rj;
    o.mj = mj;
    o.invN = sc->madhoc;
    o.cenma_m = sc->cenma_m;
    o.madhoc = sc->madhoc;
    // the float pairs (hardware conversions here: the integer split of f2_split
    // measured no faster in this kernel, where it adds registers)
    o.s.E = (float)E;
    o.s.El = (float)(E - (double)o.s.E);
    o.s.J = (float)J;
    o.s.Jl = (float)(J - (double)o.s.J);
    const double mjN = mj * o.invN;
    o.s.mjN = (float)mjN;
    o.s.mjNl = (float)(mjN - (double)o.s.mjN);
    o.s.pj = (float)ps;  // PHI_S(r_j) = (m_j / r_j) / N_STAR
    o.s.pjl = (float)(ps - (double)o.s.pj);
    o.s.rj = rj;
    o.s.Ed = E;
    o.s.Jd = J;
    o.s.mjNd = mj * o.invN;
    o.s.pjd = ps;
    return o;
}

struct OrbitRs {
    double rp, ra, dQdrp, dQdra;
    long long kmin, kmax;  // the table intervals holding the apsides
    int circular;
};

// calc_orbit_new, cmc_orbit.c:413-540.  kpos is get_positive_Q_index's
// answer (cmc_orbit.c:30-59) when already known: j when Q(j) > 0, or the
// first index with Q > 0 found by k_posq_scan; -1 makes this thread scan.
static __device__ OrbitRs calc_orbit_new(const OrbitCtx &o, long long j, long long kpos, double prec,
                                         long long maxit, int *err)
{
    OrbitRs res;
    res.circular = 1;
    res.rp = res.ra = o.rj;
    res.dQdrp = res.dQdra = 0.0;
    long long ktemp = j;
    if (kpos != j) {
        if (kpos >= 0) {
            ktemp = kpos;
        } else {
            ktemp = -1;
            int sgn;
            do {
                ktemp++;
                sgn = fq_sign(o, ktemp);
            } while (sgn <= 0 && ktemp <= o.N_MAX);
        }
        if (ktemp >= o.N_MAX) return res;
    }
    const long long kmin = find_zero_Q(o, 0, ktemp);
    const long long kmax = find_zero_Q(o, ktemp, o.N_MAX + 1);
    if (kmin < 0 || kmax < 0 || kmin > o.N_MAX || kmax > o.N_MAX) {
        *err = CMCG_ERR_ROOT_NOCONV;
        return res;
    }
    const double rkmin = o.r[kmin], rk1min = o.r[kmin + 1], rkmax = o.r[kmax], rk1max = o.r[kmax + 1];
    const double E = o.E, J = o.J;
    double a, b, rmin, rmax, inside_sqrt;
    set_a_b(o, kmin, &a, &b);
    inside_sqrt = a * a - 2.0 * J * J * (b - E);
    if (lt0(inside_sqrt)) {
        rmin = -1.0 * J * J / a;
        if ((rmin < rkmin) || (rmin > rk1min)) {
            rmin = find_root_vr(o, kmin, prec, maxit, err);
            if (*err) return res;
        }
    } else {
        rmin = J * J / (-a + sqrt(inside_sqrt));
    }
    const double dQdr_min = 2.0 * J * J / (rmin * rmin * rmin) + 2.0 * a / (rmin * rmin);
    set_a_b(o, kmax, &a, &b);
    inside_sqrt = a * a - 2.0 * J * J * (b - E);
    if (lt0(inside_sqrt)) {
        rmax = -a / (2.0 * (b - E));
        if ((rmax < rkmax) || (rmax > rk1max)) {
            rmax = find_root_vr(o, kmax, prec, maxit, err);
            if (*err) return res;
        }
    } else {
        rmax = (-a + sqrt(inside_sqrt)) / (2.0 * (b - E));
    }
    const double dQdr_max = 2.0 * J * J / (rmax * rmax * rmax) + 2.0 * a / (rmax * rmax);
    if ((rmin > rmax) || le0(dQdr_min) || ge0(dQdr_max)) return res;
    res.circular = 0;
    res.kmin = kmin;
    res.kmax = kmax;
    res.rp = rmin;
    res.ra = rmax;
    res.dQdrp = dQdr_min;
    res.dQdra = dQdr_max;
    return res;
}

// destroy_obj (cmc_dynamics_helper.c:131-150) on the device arrays: zero the
// record, keep r and phi, send the star to SF_INFINITY with mass DBL_MIN.
static __device__ __forceinline__ void destroy_obj(const Fields &f, long long g)
{
    f.E[g] = 0.0;
    f.J[g] = 0.0;
    f.X[g] = 0.0;
    f.Y[g] = 0.0;
    f.r_peri[g] = 0.0;
    f.r_apo[g] = 0.0;
    f.id[g] = 0;
    f.ec_pre[g] = 0.0;
    f.rnew[g] = CMCG_SF_INFINITY;
    f.vrnew[g] = 0.0;
    f.vtnew[g] = 0.0;
    f.m[g] = CMCG_DBL_MIN;
}

// The sampling state of a block's stars that still sample their position,
// and the lists of its rounds (sample_rounds).
struct SampleSmem {
    double rmin[ORB_T], rmax[ORB_T], F[ORB_T], E[ORB_T], J[ORB_T], rj[ORB_T], mj[ORB_T], vold2[ORB_T],
        Uold[ORB_T], ps[ORB_T];
    double c0[ORB_T], c1[ORB_T];  // 0.5 (rmin + rmax), 0.25 (rmax - rmin): the reference's factors
    long long id[ORB_T];
    long long rjb[ORB_T];         // bits of r_j (r >= r_j compared on bit patterns)
    float fE[ORB_T], fEl[ORB_T], fJ[ORB_T], fmjN[ORB_T], fpj[ORB_T], fF[ORB_T], fc1[ORB_T];
    int next[ORB_T];   // the star's next trial number (1-based)
    int first[ORB_T];  // the first trial of this round the filter did not reject (INT_MAX: none)
    int list[2][ORB_T];
    int wl[ORB_T];     // this round's candidates, one slot per star
    double wX[ORB_T], wr[ORB_T];  // a candidate's X and r, as its filter pass formed them
    long long wi[ORB_T];          // and its radius-table interval (-1: not searched)
    unsigned int wuy[ORB_T];      // and its second draw word
    int n[2], nw;
};

constexpr int TRIAL_REJECT = 0, TRIAL_ACCEPT = 1;  // anything else is a device status code
constexpr int TRIAL_UNSURE = -1;                  // filter only: left to the exact evaluation

struct Trial {
    double X, r, ir, vr, pot;
    double g;  // 1 / vr * drds, the reference's g(s0)
    int code;
};

// A trial's draws and radius (cmc_evolution_thr.c:860-870), and the table
// interval holding r once a search has found it (i = -1 before).
struct TrialIn {
    double X, r;
    long long i;
    unsigned int ux, uy;
};

static __device__ __forceinline__ TrialIn trial_input(const Cluster &C, const Scalars *sc, const SampleSmem &sm,
                                                      int s, int k)
{
    const uint4 u = draw_block(C.seed, sc->tcount, SITE_TRIAL, sm.id[s], (unsigned int)(k - 1));
    TrialIn in;
    in.X = u01(u.x);
    const double s0 = 2.0 * in.X - 1.0;
    in.r = sm.c0[s] + sm.c1[s] * (3.0 * s0 - s0 * s0 * s0);  // 0.5 (rmin + rmax) + 0.25 (rmax - rmin) (...)
    in.i = -1;
    in.ux = u.x;
    in.uy = u.y;
    return in;
}

// The radius of a trial of star slot s, evaluated exactly as the reference
// does (potential, Q, vr and g = 1 / vr * drds), without writing anything;
// code TRIAL_REJECT when that succeeded, else a device status.  Radii are
// positive, so they are compared on their bit patterns (integer
// instructions, as the FP64 comparisons would decide).
static __device__ __forceinline__ Trial eval_core(const Cluster &C, const Scalars *sc, const Fields &f,
                                                  const SampleSmem &sm, int s, const TrialIn &in, double invN)
{
    Trial t;
    const long long off = C.off, N_MAX = sc->N_MAX;
    const double E = sm.E[s], J = sm.J[s], mj = sm.mj[s], c1 = sm.c1[s];
    const double X = in.X, r = in.r;
    const double s0 = 2.0 * X - 1.0;
    // one correctly rounded 1/r serves every division by r below (div_rcp)
    const double ir = __drcp_rn(r);
    int pok = 1;
    const double *rt = f.r + off, *pt = f.phi + off, *it = f.inv_r + off;
    const long long rb = dbits(r);
    double pot;
    if (rb >= dbits(__ldg(rt + 1))) {
        const long long i = in.i >= 0 ? in.i : potential_index(rt, N_MAX, r, ridx_of(C, f));
        if (i > N_MAX || dbits(__ldg(rt + i)) > rb || dbits(__ldg(rt + i + 1)) < rb) {
            pok = 0;
            pot = 0.0;
        } else {
            const double pi = __ldg(pt + i), pi1 = __ldg(pt + i + 1), ii = __ldg(it + i), ii1 = __ldg(it + i + 1);
            pot = __dadd_rn(pi, __ddiv_rn(__dmul_rn(__dsub_rn(pi1, pi), __dsub_rn(ii, ir)), __dsub_rn(ii, ii1)));
        }
    } else {
        pot = potential_at(rt, pt, it, N_MAX, r, &pok);
    }
    pot += (rb >= sm.rjb[s]) ? __dmul_rn(div_rcp(mj, r, ir), invN) : sm.ps[s];
    t.X = X;
    t.r = r;
    t.ir = ir;
    t.pot = pot;
    t.vr = 0.0;
    if (!pok) {
        t.code = CMCG_ERR_FINDZERO_R;
        return t;
    }
    const double drds = c1 * (3.0 - 3.0 * s0 * s0);  // 0.25 (rmax - rmin) (3 - 3 s0^2)
    const double Q = 2.0 * E - 2.0 * pot - div_rcp(div_rcp(J * J, r, ir), r, ir);
    double vr;
    if (ge0(Q)) {
        vr = sqrt(Q);
    } else {
        if (isnan(Q)) {
            t.code = CMCG_ERR_Q_NAN;
            return t;
        }
        vr = 0;
    }
    t.vr = vr;
    t.g = 1.0 / vr * drds;
    t.code = TRIAL_REJECT;
    return t;
}

// A plain trial (cmc_evolution_thr.c:860-885): accepted when g0 = F u < g(s0).
static __device__ __forceinline__ Trial eval_trial(const Cluster &C, const Scalars *sc, const Fields &f,
                                                   const SampleSmem &sm, int s, const TrialIn &in, double invN)
{
    Trial t = eval_core(C, sc, f, sm, s, in, invN);
    if (t.code == TRIAL_REJECT) t.code = (sm.F[s] * u01(in.uy) < t.g) ? TRIAL_ACCEPT : TRIAL_REJECT;
    return t;
}

// Certified FP32 decision of trial k: TRIAL_ACCEPT or TRIAL_REJECT where the
// exact evaluation must agree, TRIAL_UNSURE otherwise.  Only r is formed in
// FP64 (as the reference forms it, so the radius search is the reference's);
// the rest works on floats.
//  * The interpolated potential lies between the two table values around r:
//    the reference's weight RN(1/r_i - 1/r) / RN(1/r_i - 1/r_i+1) is in [0, 1]
//    because RN is monotone, so Q is bracketed by its values at those two
//    potentials.  Each end, formed from the float pairs of E and the table's
//    float Phi, is within 2^-20.7 M of the reference's (M = |E| + |Phi| +
//    phis + |A| + (J/r)^2, A = E - Phi - phis); the bracket is widened by
//    2^-18 M.
//  * Accepted when g0^2 Qmax < drds^2 (1 - eta), rejected when g0^2 Qmin >
//    drds^2 (1 + eta): g0, drds and the products carry at most 2^-19.5 of
//    their value in float; the reference's 3 - 3 s0^2 loses up to
//    2^-51 / (1 - s0^2) to cancellation, and 1 - s0^2 = 4 X (1 - X) is formed
//    from the integer draw without it.  eta = 2^-17 + 2^-48 / (1 - s0^2).
//  * Q < 0 for certain: vr = 0 and 1/vr * drds is +inf (drds > 0 unless the
//    draw is 0), so the trial is accepted.
// Radii at or below r_1, a failed search, neighbours within 4 ulps (whose
// reciprocals may round equal) and non-finite values are unsure.
// The bracket [Qlo, Qhi] (first point above); false where it cannot be
// formed (the trial is then unsure).  Sets in.i once the radius is searched.
static __device__ __forceinline__ bool q_bracket(const Cluster &C, const Scalars *sc, const Fields &f,
                                                 const SampleSmem &sm, int s, TrialIn &in, float &Qlo, float &Qhi)
{
    const double r = in.r;
    const long long off = C.off, N_MAX = sc->N_MAX;
    const double *rt = f.r + off;
    const long long rb = dbits(r);
    if (rb <= dbits(__ldg(rt + 1))) return false;
    const long long i = potential_index(rt, N_MAX, r, ridx_of(C, f));
    in.i = i;
    if (i < 1 || i > N_MAX) return false;
    const long long bi = dbits(__ldg(rt + i)), bi1 = dbits(__ldg(rt + i + 1));
    if (bi >= rb || bi1 < rb || bi1 - bi <= 4) return false;
    const float4 ta = __ldg(f.rphif + off + i), tb = __ldg(f.rphif + off + i + 1);
    const float plo = fminf(ta.y, tb.y), phi = fmaxf(ta.y, tb.y);
    const float irf = __frcp_rn((float)r);
    const float phis = (rb >= sm.rjb[s]) ? __fmul_rn(sm.fmjN[s], irf) : sm.fpj[s];
    const float q = __fmul_rn(sm.fJ[s], irf);
    const float B = __fmul_rn(q, q);
    const float2 dlo = ff_two_sum(sm.fE[s], -phi), dhi = ff_two_sum(sm.fE[s], -plo);
    const float Alo = __fsub_rn(__fadd_rn(dlo.x, __fadd_rn(dlo.y, sm.fEl[s])), phis);
    const float Ahi = __fsub_rn(__fadd_rn(dhi.x, __fadd_rn(dhi.y, sm.fEl[s])), phis);
    const float M = fabsf(sm.fE[s]) + fmaxf(fabsf(plo), fabsf(phi)) + phis + B + fmaxf(fabsf(Alo), fabsf(Ahi));
    const float eQ = __fmul_rn(0x1p-18f, M);
    Qlo = __fsub_rn(__fsub_rn(__fmul_rn(2.0f, Alo), B), eQ);
    Qhi = __fadd_rn(__fsub_rn(__fmul_rn(2.0f, Ahi), B), eQ);
    return fabsf(Qlo) <= 1e30f && fabsf(Qhi) <= 1e30f;
}

static __device__ __forceinline__ int filter_trial(const Cluster &C, const Scalars *sc, const Fields &f,
                                                   const SampleSmem &sm, int s, TrialIn &in)
{
    const float fc1 = sm.fc1[s];
    if (in.ux == 0u || !(fc1 > 0.0f)) return TRIAL_UNSURE;
    float Qlo, Qhi;
    if (!q_bracket(C, sc, f, sm, s, in, Qlo, Qhi)) return TRIAL_UNSURE;
    if (Qhi < 0.0f) return TRIAL_ACCEPT;
    if (!(Qlo > 0.0f)) return TRIAL_UNSURE;
    // 1 - s0^2 = 4 X (1 - X) = u (2^32 - u) 2^-62
    const float w = __fmul_rn(__fmul_rn((float)in.ux, (float)(0u - in.ux)), 0x1p-62f);
    const float drds = __fmul_rn(__fmul_rn(3.0f, fc1), w);
    const float g0 = __fmul_rn(sm.fF[s], __fmul_rn((float)in.uy, 0x1p-32f));
    const float eta = __fadd_rn(0x1p-17f, __fmul_rn(0x1p-48f, __frcp_rn(w)));
    const float g2 = __fmul_rn(g0, g0), d2 = __fmul_rn(drds, drds);
    if (!(g2 <= 1e30f) || !(d2 <= 1e30f) || !(d2 > 1e-30f)) return TRIAL_UNSURE;
    if (__fmul_rn(g2, Qhi) < __fmul_rn(d2, __fsub_rn(1.0f, eta))) return TRIAL_ACCEPT;
    if (__fmul_rn(g2, Qlo) > __fmul_rn(d2, __fadd_rn(1.0f, eta))) return TRIAL_REJECT;
    return TRIAL_UNSURE;
}

// The accepted trial's outputs (cmc_evolution_thr.c:918-935).
static __device__ __forceinline__ void commit_trial(const Cluster &C, const Scalars *sc, const Fields &f,
                                                    const SampleSmem &sm, int s, long long g, const Trial &t,
                                                    double *max_rad)
{
    f.X[g] = t.X;
    f.r_peri[g] = sm.rmin[s];
    f.r_apo[g] = sm.rmax[s];
    double vr = t.vr;
    if (u01(draw_block(C.seed, sc->tcount, SITE_SIGN, sm.id[s], 0u).x) < 0.5) vr = -vr;
    f.rnew[g] = t.r;
    f.vrnew[g] = vr;
    f.vtnew[g] = div_rcp(sm.J[s], t.r, t.ir);
    if (dbits(t.r) > dbits(*max_rad)) *max_rad = t.r;  // both non-negative
    // energy_conservation2: Uoldrnew = potential(rnew) + PHI_S(rnew)
    f.ec_pre[g] = sm.vold2[s] + 2.0 * (1.0 - 0.5) * (sm.Uold[s] - t.pot);
}

// Stars whose Q(j) <= 0 (a turning point: vr rounds to zero) need the first
// table index with Q > 0, which get_positive_Q_index finds by a linear scan
// from the centre.  k_orbit_pre marks them; k_posq_scan spreads each scan
// over the whole grid (atomicMin of the indices with Q > 0; a thread skips
// chunks above the minimum already found); k_orbit takes the answer.
__global__ void __launch_bounds__(ORB_T) k_orbit_pre(const Cluster *__restrict__ cls, Tiles tm, Fields f, PosQ pq)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const Scalars *sc = C.sc;
    const long long off = C.off;
    const long long j = 1 + (long long)ct.y * ORB_T + threadIdx.x;
    if (j > sc->N_MAX_NEW) return;
    const long long g = off + j;
    const double Ej = f.E[g], rj = f.r[g], mj = f.m[g];
    const double ps = __dmul_rn(div_rcp(mj, rj, f.inv_r[g]), sc->madhoc);
    const double E = Ej + ps;
    int slot = PQ_POSITIVE;
    if (!lt_pos(mj, CMCG_ZERO) && lt0(E)) {
        // the FP32 stage from the few floats it reads; the whole certified test
        // (and its context) only when that stage is undecided
        QF32 q;
        f2_split(E, q.E, q.El);
        q.J = d2f_rn(f.J[g]);
        q.mjN = d2f_rn(mj * sc->madhoc);
        q.pj = d2f_rn(ps);
        int sg = fq_sign_f32(q, __ldg(f.rphif + g), true);
        if (sg == 0) {
            const OrbitCtx o = make_orbit_ctx(C, f, j, E, f.J[g], rj, mj, ps);
            sg = fq_sign(o, j);
        }
        if (sg <= 0) {
            const unsigned int e = atomicAdd(pq.count, 1u);
            if (e < PQ_CAP) {
                pq.cl[e] = ct.x;
                pq.j[e] = j;
                pq.res[e] = sc->N_MAX + 1;  // none found: the reference's scan ends past N_MAX
                slot = (int)e;
            } else {
                slot = PQ_SCAN_HERE;  // list full: k_orbit scans in the thread
            }
        }
    }
    pq.slot[g] = slot;
}

__global__ void __launch_bounds__(256) k_posq_scan(const Cluster *__restrict__ cls, Fields f, PosQ pq)
{
    const unsigned int n = min(*(volatile unsigned int *)pq.count, (unsigned int)PQ_CAP);
    const long long T = (long long)gridDim.x * blockDim.x, gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (unsigned int e = 0; e < n; ++e) {
        const Cluster &C = cls[pq.cl[e]];
        const Scalars *sc = C.sc;
        const long long j = pq.j[e], g = C.off + j, N_MAX = sc->N_MAX;
        const double rj = f.r[g], mj = f.m[g];
        const double ps = __dmul_rn(div_rcp(mj, rj, f.inv_r[g]), sc->madhoc);
        const OrbitCtx o = make_orbit_ctx(C, f, j, f.E[g] + ps, f.J[g], rj, mj, ps);
        for (long long base = 0; base <= N_MAX; base += T) {
            if (*(volatile long long *)&pq.res[e] < base) break;
            const long long k = base + gt;
            if (k <= N_MAX && fq_sign(o, k) > 0) atomicMin(&pq.res[e], k);
        }
    }
}

// The per-star part of the learned proposal: the orbit's features for the
// network (normalised, as BF16): rmin / rmax, ln(rmax) / 8, E / Phi_a,
// J^2 / (2 rmin^2 (E - Phi_a)), and the potential's shape across the orbit,
// (Phi_k - Phi_a) / (Phi_b - Phi_a) at four table points evenly spaced in
// index between a = kmin and b = kmax + 1, the table points bracketing the
// apsides (table reads only: no radius search).
static __device__ __forceinline__ uint4 orbit_features(const OrbitCtx &o, const OrbitRs &orb)
{
    const long long ka = orb.kmin, kb = orb.kmax + 1;
    const double pa = __ldg(o.phi + ka), pb = __ldg(o.phi + kb), d = pb - pa;
    float x[MLP_IN];
    x[0] = (float)(orb.rp / orb.ra);
    x[1] = 0.125f * logf((float)orb.ra);
    x[2] = (float)(o.E / pa);
    x[3] = (float)(o.J * o.J / (2.0 * orb.rp * orb.rp * (o.E - pa)));
#pragma unroll
    for (int i = 1; i <= 4; ++i) {
        const long long k = ka + ((kb - ka) * i) / 5;
        x[3 + i] = d > 0.0 ? (float)((__ldg(o.phi + k) - pa) / d) : 0.0f;
    }
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float a = isfinite(x[2 * i]) ? x[2 * i] : 0.0f, b = isfinite(x[2 * i + 1]) ? x[2 * i + 1] : 0.0f;
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        w[i] = *reinterpret_cast<uint32_t *>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

struct LearnSmem {
    float cdf[MLP_BINS - 1][ORB_T];  // C_1 .. C_31 of each star's proposal
    float P[ORB_T];                  // its predicted acceptance probability of a plain trial
    double wenv[ORB_T];              // a candidate's envelope kappa F P q(X)
    int fb[ORB_T];                   // stars sent back to the plain sampler
    int nfb;
};
constexpr int TRIAL_FAIL = -2;  // a proposal trial found the envelope below the density

// Trial k of the proposal for star slot s, with draws of its own site keyed
// by (star id, k): X from the 32-bin density q by inverting its CDF (density
// 32 (C_b+1 - C_b) on bin b, with the stored knots), and the envelope
// kappa F P q(X) under which g0 is drawn uniformly.
static __device__ __forceinline__ TrialIn learned_input(const Cluster &C, const Scalars *sc, const SampleSmem &sm,
                                                        const LearnSmem &ls, int s, int k, double kappa,
                                                        double *env)
{
    const uint4 u = draw_block(C.seed, sc->tcount, SITE_LTRIAL, sm.id[s], (unsigned int)(k - 1));
    const double U = u01(u.x);
    int b = 0;  // the last bin whose lower knot is <= U (C_0 = 0)
#pragma unroll
    for (int h = 16; h > 0; h >>= 1)
        if (b + h <= MLP_BINS - 1 && (double)ls.cdf[b + h - 1][s] <= U) b += h;
    const double lo = b > 0 ? (double)ls.cdf[b - 1][s] : 0.0;
    const double hi = b < MLP_BINS - 1 ? (double)ls.cdf[b][s] : 1.0;
    const double pb = hi - lo;
    double X = ((double)b + (U - lo) / pb) * (1.0 / MLP_BINS);
    if (!(X < 1.0)) X = 0x1.fffffffffffffp-1;
    TrialIn in;
    in.X = X;
    const double s0 = 2.0 * X - 1.0;
    in.r = sm.c0[s] + sm.c1[s] * (3.0 * s0 - s0 * s0 * s0);  // the reference's map from s0 to r
    in.i = -1;
    in.ux = u.x;
    in.uy = u.y;
    *env = kappa * sm.F[s] * (double)ls.P[s] * ((double)MLP_BINS * pb);
    return in;
}

// Exact decision of a proposal trial: accepted when g0 = env u < min(g(s0), F),
// the density the plain sampler samples (its g clipped at its envelope F);
// TRIAL_FAIL where min(g, F) exceeds the envelope (the star then goes back to
// the plain sampler).
static __device__ __forceinline__ Trial learned_eval(const Cluster &C, const Scalars *sc, const Fields &f,
                                                     const SampleSmem &sm, int s, const TrialIn &in, double env,
                                                     double invN)
{
    Trial t = eval_core(C, sc, f, sm, s, in, invN);
    if (t.code != TRIAL_REJECT) return t;  // a device error
    const double F = sm.F[s];
    const double g = isnan(t.g) ? 0.0 : t.g;  // 0 * inf: the reference's comparison rejects
    const double h = g < F ? g : F;
    if (h > env)
        t.code = TRIAL_FAIL;
    else
        t.code = (env * u01(in.uy) < h) ? TRIAL_ACCEPT : TRIAL_REJECT;
    return t;
}

// Certified FP32 decision of a proposal trial, from filter_trial's bracket of
// Q: TRIAL_ACCEPT or TRIAL_REJECT only where the exact evaluation must agree
// and the envelope certainly holds (F <= env, or g < env for every Q in the
// bracket), TRIAL_UNSURE otherwise.  1 - s0^2 = 4 X (1 - X) is formed in FP64
// from X (within 2^-51 of its value), so filter_trial's margin eta holds.
static __device__ __forceinline__ int learned_filter(const Cluster &C, const Scalars *sc, const Fields &f,
                                                     const SampleSmem &sm, int s, TrialIn &in, double env)
{
    const float fc1 = sm.fc1[s];
    const double X = in.X;
    if (!(X > 0.0) || !(X < 1.0) || !(fc1 > 0.0f)) return TRIAL_UNSURE;
    float Qlo, Qhi;
    if (!q_bracket(C, sc, f, sm, s, in, Qlo, Qhi)) return TRIAL_UNSURE;
    const double F = sm.F[s];
    const double g0 = env * u01(in.uy);  // as the exact decision forms it
    const bool holds_at_F = F <= env;     // min(g, F) <= F <= env
    if (Qhi < 0.0f) {                     // vr = 0, g = +inf: min(g, F) = F
        if (!holds_at_F) return TRIAL_UNSURE;
        return g0 < F ? TRIAL_ACCEPT : TRIAL_REJECT;
    }
    if (!(Qlo > 0.0f)) return TRIAL_UNSURE;
    const float w = (float)(4.0 * X * (1.0 - X));
    const float drds = __fmul_rn(__fmul_rn(3.0f, fc1), w);
    const float eta = __fadd_rn(0x1p-17f, __fmul_rn(0x1p-48f, __frcp_rn(w)));
    const float d2 = __fmul_rn(drds, drds);
    if (!(d2 <= 1e30f) || !(d2 > 1e-30f)) return TRIAL_UNSURE;
    if (!holds_at_F) {  // g < env for certain: env^2 Qlo > drds^2 (1 + eta)
        const float e = (float)env, e2 = __fmul_rn(e, e);
        if (!(e2 <= 1e30f) || !(__fmul_rn(e2, Qlo) > __fmul_rn(d2, __fadd_rn(1.0f, eta)))) return TRIAL_UNSURE;
    }
    if (g0 >= F) return TRIAL_REJECT;  // min(g, F) <= F <= g0
    const float gf = (float)g0, g2 = __fmul_rn(gf, gf);
    if (!(g2 <= 1e30f)) return TRIAL_UNSURE;
    if (__fmul_rn(g2, Qhi) < __fmul_rn(d2, __fsub_rn(1.0f, eta))) return TRIAL_ACCEPT;
    if (__fmul_rn(g2, Qlo) > __fmul_rn(d2, __fadd_rn(1.0f, eta))) return TRIAL_REJECT;
    return TRIAL_UNSURE;
}

// Per-thread counters of the learned sampler (block sums go to Learn::stats).
struct LStat {
    unsigned int trials = 0, acc = 0, fail = 0, ptrials = 0, pstars = 0;
};

// The rounds of a block's rejection loop (get_positions_loop,
// cmc_evolution_thr.c:855-926) over the sm.n[0] stars listed in sm.list[0]
// (state staged, next = 1, first = INT_MAX).  A star's trial k uses draws
// keyed by (star id, k), so its trials are independent of one another and of
// the order they run in.  Each round gives every pending star m = ORB_T / n
// threads (n pending stars), which test its next m trials at once with a
// certified FP32 filter; the first trial the filter does not reject is the
// only candidate for the star's outcome in the reference's sequential loop,
// and those candidates, one per star, are then evaluated exactly in FP64 by
// threads packed into full warps.  A candidate the exact evaluation rejects
// (the filter was unsure) puts the star back with its next trial.  Rounds
// stay full of threads, their number falls to about the log of the longest
// trial sequence, and the FP64 evaluation runs about once per star instead
// of once per trial.  LEARN: the proposal's trials; a star whose envelope
// fails, or whose n_try proposal trials are all rejected, is listed in
// ls->fb for the plain rounds that follow.
template <int MODE, bool LEARN>
static __device__ __forceinline__ void sample_rounds(const Cluster &C, Scalars *sc, const Fields &f, SampleSmem &sm,
                                                     LearnSmem *ls, const Learn &L, long long j0, double invN,
                                                     double *max_rad, LStat &st)
{
    const int t = threadIdx.x;
    const long long off = C.off, n_try = C.n_try;
    const bool check = C.check_filters != 0;
    for (int cur = 0;; cur ^= 1) {
        const int n = sm.n[cur];
        if (n == 0) break;
        const int m = ORB_T / n;  // trials per pending star this round
        if (t == 0) {
            sm.n[cur ^ 1] = 0;  // last read at the top of the previous round
            sm.nw = 0;
        }
        // 1. the filter on each star's next m trials
        int slot = -1, k = 0, kb = 0;
        TrialIn in;
        double env = 0.0;
        if (t < n * m) {
            slot = sm.list[cur][t / m];
            kb = sm.next[slot];
            k = kb + t % m;
            if (k <= n_try) {
                int dec;
                if (LEARN) {
                    in = learned_input(C, sc, sm, *ls, slot, k, L.kappa, &env);
                    dec = learned_filter(C, sc, f, sm, slot, in, env);
                    if (check && dec != TRIAL_UNSURE && learned_eval(C, sc, f, sm, slot, in, env, invN).code != dec)
                        set_error(sc, CMCG_ERR_FILTER, j0 + slot);
                } else {
                    in = trial_input(C, sc, sm, slot, k);
                    dec = filter_trial(C, sc, f, sm, slot, in);
                    if (check && dec != TRIAL_UNSURE && eval_trial(C, sc, f, sm, slot, in, invN).code != dec)
                        set_error(sc, CMCG_ERR_FILTER, j0 + slot);
                }
                if (dec != TRIAL_REJECT) atomicMin(&sm.first[slot], k);
            }
        }
        __syncthreads();
        // 2. candidates listed (with their inputs); stars whose m trials were all rejected go on
        if (slot >= 0) {
            const int fst = sm.first[slot];
            if (k == fst) {
                sm.wX[slot] = in.X;
                sm.wr[slot] = in.r;
                sm.wi[slot] = in.i;
                sm.wuy[slot] = in.uy;
                if (LEARN) ls->wenv[slot] = env;
                sm.wl[atomicAdd(&sm.nw, 1)] = slot;
            } else if (t % m == 0 && fst == INT_MAX) {
                if (kb + m - 1 >= n_try) {
                    if (LEARN) {  // the proposal's trials ran out: the plain sampler decides
                        ls->fb[atomicAdd(&ls->nfb, 1)] = slot;
                        st.trials += (unsigned int)n_try;
                        st.fail++;
                    } else {
                        set_error(sc, CMCG_ERR_NTRY, j0 + slot);  // n_try trials, none accepted
                    }
                } else {
                    sm.next[slot] = kb + m;
                    sm.list[cur ^ 1][atomicAdd(&sm.n[cur ^ 1], 1)] = slot;
                }
            }
        }
        __syncthreads();
        // 3. the candidates evaluated exactly, one star per thread
        if (t < sm.nw) {
            const int s = sm.wl[t];
            const int kk = sm.first[s];
            TrialIn cin;
            cin.X = sm.wX[s];
            cin.r = sm.wr[s];
            cin.i = sm.wi[s];
            cin.uy = sm.wuy[s];
            cin.ux = 0u;  // not used by the exact evaluation
            const Trial tr = LEARN ? learned_eval(C, sc, f, sm, s, cin, ls->wenv[s], invN)
                                   : eval_trial(C, sc, f, sm, s, cin, invN);
            if (tr.code == TRIAL_ACCEPT) {
                commit_trial(C, sc, f, sm, s, off + j0 + s, tr, max_rad);
                if (MODE == 2) {
                    L.ntrial[off + j0 + s] = LEARN ? -kk : kk;
                    if (LEARN) {
                        st.trials += (unsigned int)kk;
                        st.acc++;
                    } else {
                        st.ptrials += (unsigned int)kk;
                        st.pstars++;
                    }
                }
            } else if (LEARN && (tr.code == TRIAL_FAIL || (tr.code == TRIAL_REJECT && kk >= n_try))) {
                ls->fb[atomicAdd(&ls->nfb, 1)] = s;
                st.trials += (unsigned int)kk;
                st.fail++;
            } else if (tr.code != TRIAL_REJECT) {
                set_error(sc, tr.code, j0 + s);
            } else if (kk >= n_try) {
                set_error(sc, CMCG_ERR_NTRY, j0 + s);
            } else {
                // the filter was unsure and the trial is rejected: go on from the next one
                sm.first[s] = INT_MAX;
                sm.next[s] = kk + 1;
                sm.list[cur ^ 1][atomicAdd(&sm.n[cur ^ 1], 1)] = s;
            }
        }
        __syncthreads();
    }
}

// One star's sampling state in the block's shared memory.
static __device__ __forceinline__ void stage_star(SampleSmem &sm, int ts, const OrbitCtx &o, double rmin,
                                                  double rmax, double F, double E, double J, double rj, double mj,
                                                  double vold2, double Uoldrold, long long idj, double ps)
{
    sm.rmin[ts] = rmin;
    sm.rmax[ts] = rmax;
    sm.F[ts] = F;
    sm.E[ts] = E;
    sm.J[ts] = J;
    sm.rj[ts] = rj;
    sm.mj[ts] = mj;
    sm.vold2[ts] = vold2;
    sm.Uold[ts] = Uoldrold;
    sm.id[ts] = idj;
    sm.ps[ts] = ps;
    sm.c0[ts] = 0.5 * (rmin + rmax);
    sm.c1[ts] = 0.25 * (rmax - rmin);
    sm.rjb[ts] = dbits(rj);
    // the filter's floats: E as a float pair, the rest rounded once
    sm.fE[ts] = o.s.E;
    sm.fEl[ts] = o.s.El;
    sm.fJ[ts] = o.s.J;
    sm.fmjN[ts] = o.s.mjN;
    sm.fpj[ts] = o.s.pj;
    sm.fF[ts] = (float)F;
    sm.fc1[ts] = (float)sm.c1[ts];
}

// Sum of a per-thread counter over the block, added to a global counter by one thread.
static __device__ __forceinline__ void add_stat(unsigned long long *dst, unsigned int v, unsigned int *s_w)
{
    const unsigned int w = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        for (int q = 0; q < ORB_T / 32; ++q) s += s_w[q];
        if (s) atomicAdd(dst, s);
    }
    __syncthreads();
}

// MODE 0: the whole of get_positions_loop for the block's stars (k_orbit).
// MODE 1: everything up to the rejection loop (k_orbit_aps): stars that still
//         sample a position leave their envelope F and features for the
//         network (apsides in r_peri / r_apo, which the accepted trial writes
//         again unchanged); escapers, circular orbits and errors are final.
// MODE 2: the rejection loop of those stars (k_orbit_learn): proposal trials
//         first (Learn::mode LEARN_ON), stars whose envelope failed then take
//         the plain trials of MODE 0 from the first, as every star does in
//         LEARN_COLLECT.
template <int MODE>
static __device__ __forceinline__ void orbit_body(const Cluster *__restrict__ cls, Tiles tm, const Fields &f,
                                                  double *partials, unsigned int *tickets, const PosQ &pq,
                                                  const Learn &L, SampleSmem &sm, LearnSmem *ls, int tile)
{
    __shared__ double red[ORB_T / 32];
    const int2 ct = tm.tiles[tile];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long off = C.off;
    const long long N_MAX = sc->N_MAX, N_NEW = sc->N_MAX_NEW;
    const double invN = sc->madhoc;  // 1.0 / N_STAR, as the reference forms it (cmc_utils.c:1183)
    const double Rtidal = sc->Rtidal;
    const long long j = 1 + (long long)ct.y * ORB_T + threadIdx.x;
    const long long g = off + j;

    double acc_E = 0.0, acc_J = 0.0, acc_M = 0.0, acc_Et = 0.0, max_rad = 0.0;
    bool pend = false;
    if (MODE == 1 && j <= C.cap) {  // this step's records only (every slot of the cluster)
        L.F[g] = 0.0;
        L.feat[g] = make_uint4(0u, 0u, 0u, 0u);
        L.ntrial[g] = 0;
    }
    if (j <= N_NEW) {
        const double Ej = f.E[g], Jj = f.J[g], rj = f.r[g], mj = f.m[g], phij = f.phi[g];
        const double vr0 = f.vr_rel[g], vt0 = f.vt_rel[g];
        const long long idj = f.id[g];
        const double ps = __dmul_rn(div_rcp(mj, rj, f.inv_r[g]), invN);  // PHI_S(r_j) (cmc.h:2175)
        const double E = Ej + ps;
        const double J = Jj;
        // energy_conservation1: vtold, vrold, Uoldrold
        const double Uoldrold = phij + ps;
        const double vold2 = vt0 * vt0 + vr0 * vr0;
        if (MODE == 2) {
            const double F = L.F[g];
            if (F > 0.0 && C.n_try >= 1) {  // left to sample by the apsides pass
                const OrbitCtx o = make_orbit_ctx(C, f, j, E, J, rj, mj, ps);
                stage_star(sm, threadIdx.x, o, f.r_peri[g], f.r_apo[g], F, E, J, rj, mj, vold2, Uoldrold, idj, ps);
                if (L.mode == LEARN_ON) {
#pragma unroll
                    for (int b = 0; b < MLP_BINS - 1; ++b) ls->cdf[b][threadIdx.x] = L.prop[b * L.stride + g];
                    ls->P[threadIdx.x] = L.prop[(MLP_BINS - 1) * L.stride + g];
                }
                pend = true;
            }
        } else {
            if (lt_pos(mj, CMCG_ZERO)) {  // mj < ZERO, E >= 0 (integer forms of the comparisons)
                destroy_obj(f, g);
            } else if (ge0(E)) {
                // remove_star, cmc_evolution_thr.c:655-716
                acc_E = Ej * mj / (double)sc->N_STAR;
                acc_J = Jj * mj / (double)sc->N_STAR;
                acc_M = mj / (double)sc->N_STAR;
                acc_Et = Ej * mj / (double)sc->N_STAR;
                destroy_obj(f, g);
            } else {
                const OrbitCtx o = make_orbit_ctx(C, f, j, E, J, rj, mj, ps);
                int err = 0;
                // Q(j) > 0, or the index the grid-wide scan found (k_orbit_pre, k_posq_scan)
                const int slot = pq.slot[g];
                const long long kpos = (slot == PQ_POSITIVE) ? j : (slot >= 0 ? pq.res[slot] : -1);
                const OrbitRs orb = calc_orbit_new(o, j, kpos, C.apsides_precision, C.apsides_max_iter, &err);
                if (err) {
                    set_error(sc, err, j);
                } else if (orb.circular) {
                    // cmc_evolution_thr.c:835-840: position and velocities unchanged
                    f.rnew[g] = rj;
                    f.vrnew[g] = vr0;
                    f.vtnew[g] = vt0;
                    bool ok = true;
                    int pok = 1;
                    const double Uoldrnew =
                        potential_at(o.r, o.phi, o.inv_r, N_MAX, rj, &pok, ridx_of(C, f)) + ps;
                    ok = pok;
                    if (!ok) set_error(sc, CMCG_ERR_FINDZERO_R, j);
                    f.ec_pre[g] = vold2 + 2.0 * (1.0 - 0.5) * (Uoldrold - Uoldrnew);
                } else if (ge_pos(orb.ra, Rtidal)) {  // Rtidal > 0
                    acc_E = Ej * mj / (double)sc->N_STAR;
                    acc_J = Jj * mj / (double)sc->N_STAR;
                    acc_M = mj / (double)sc->N_STAR;
                    acc_Et = Ej * mj / (double)sc->N_STAR;
                    destroy_obj(f, g);
                } else {
                    const double rmin = orb.rp, rmax = orb.ra;
                    const double g1 = sqrt(3.0 * (rmax - rmin) / orb.dQdrp);
                    const double g2 = sqrt(-3.0 * (rmax - rmin) / orb.dQdra);
                    const double F = 1.2 * (g1 >= g2 ? g1 : g2);
                    if (C.n_try < 1) {
                        set_error(sc, CMCG_ERR_NTRY, j);  // no trial allowed (cmc_evolution_thr.c:888)
                    } else if (MODE == 1) {
                        f.r_peri[g] = rmin;
                        f.r_apo[g] = rmax;
                        L.F[g] = F;
                        L.feat[g] = orbit_features(o, orb);
                    } else {
                        stage_star(sm, threadIdx.x, o, rmin, rmax, F, E, J, rj, mj, vold2, Uoldrold, idj, ps);
                        pend = true;
                    }
                }
            }
        }
    }
    const int t = threadIdx.x;
    const long long j0 = 1 + (long long)ct.y * ORB_T;
    if (MODE == 2 && L.mode == LEARN_ON && t == 0 && ct.y == 0 && *L.mlp_status != 0)
        set_error(sc, CMCG_ERR_SPIN, 0);  // the network's inference gave up: its proposals are not valid
    // rejection sampling in rounds over the block's pending stars
    if (t == 0) {
        sm.n[0] = 0;
        if (MODE == 2) ls->nfb = 0;
    }
    __syncthreads();
    if (pend) {
        const int p = atomicAdd(&sm.n[0], 1);
        sm.list[0][p] = t;
        sm.next[t] = 1;
        sm.first[t] = INT_MAX;
    }
    __syncthreads();
    LStat st;
    if (MODE == 2 && L.mode == LEARN_ON) {
        sample_rounds<MODE, true>(C, sc, f, sm, ls, L, j0, invN, &max_rad, st);
        // the stars sent back start the plain trials from the first
        const int nfb = ls->nfb;
        if (t < nfb) {
            const int s = ls->fb[t];
            sm.list[0][t] = s;
            sm.next[s] = 1;
            sm.first[s] = INT_MAX;
        }
        __syncthreads();
        if (t == 0) sm.n[0] = nfb;
        __syncthreads();
    }
    sample_rounds<MODE, false>(C, sc, f, sm, ls, L, j0, invN, &max_rad, st);
    if (MODE == 2) {
        __shared__ unsigned int s_w[ORB_T / 32];
        add_stat(L.stats + LSTAT_TRIALS, st.trials, s_w);
        add_stat(L.stats + LSTAT_ACCEPT, st.acc, s_w);
        add_stat(L.stats + LSTAT_FAIL, st.fail, s_w);
        add_stat(L.stats + LSTAT_STARS, (L.mode == LEARN_ON && pend) ? 1u : 0u, s_w);
        add_stat(L.stats + LSTAT_PLAIN_TRIALS, st.ptrials, s_w);
        add_stat(L.stats + LSTAT_PLAIN_STARS, st.pstars, s_w);
    }
    // escapers are rare: most warps skip the sums (block_sums)
    __shared__ double s_acc[ORB_T / 32][4];
    __shared__ long long s_max[ORB_T / 32];
    double acc[4] = {acc_E, acc_J, acc_M, acc_Et};
    block_sums<ORB_T>(acc, s_acc);
    const double tmax = block_max_nonneg<ORB_T>(max_rad, s_max);
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        double *slot = partials + (size_t)tile * ORB_NPART;
        slot[0] = acc[0];
        slot[1] = acc[1];
        slot[2] = acc[2];
        slot[3] = acc[3];
        slot[4] = tmax;
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        double a[ORB_NPART];
        const int b0 = tm.first[ct.x], nb = tm.count[ct.x];
        for (int q = 0; q < 4; ++q) a[q] = reduce_partials_sum<ORB_T>(partials, b0, nb, ORB_NPART, q, red);
        a[4] = reduce_partials_max<ORB_T>(partials, b0, nb, ORB_NPART, 4, red);
        if (threadIdx.x == 0) {
            if (MODE == 2) {
                // the apsides pass set max_r from the stars it finished (none sampled there)
                if (a[4] > sc->max_r) sc->max_r = a[4];
            } else {
                // new_orbits_calculate, cmc_utils.c:2197-2210
                sc->OldTidalMassLoss = sc->TidalMassLoss_old;
                sc->Eescaped += a[0];
                sc->Jescaped += a[1];
                sc->TidalMassLoss += a[2];
                sc->Etidal += a[3];
                sc->max_r = a[4];
                sc->TidalMassLoss += sc->TidalMassLoss_old;
            }
        }
    }
}

// Five blocks per SM (at most 102 registers a thread; a few bytes spill) keep
// more warps on the FP64 pipe than the four that 116 registers allow.
__global__ void __launch_bounds__(ORB_T, 5) k_orbit(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                 double *partials, unsigned int *tickets, PosQ pq)
{
    __shared__ SampleSmem sm;
    const Learn none{};
    orbit_body<0>(cls, tm, f, partials, tickets, pq, none, sm, nullptr, blockIdx.x);
}

// The same kernel with room for 128 registers a thread (four blocks per SM):
// an autotuner candidate, with bit-identical results.
__global__ void __launch_bounds__(ORB_T, 4) k_orbit_lb4(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                     double *partials, unsigned int *tickets, PosQ pq)
{
    __shared__ SampleSmem sm;
    const Learn none{};
    orbit_body<0>(cls, tm, f, partials, tickets, pq, none, sm, nullptr, blockIdx.x);
}

// The persistent forms: a grid of (blocks per SM) x (SMs) blocks, each taking
// tiles from a counter (zeroed before the launch) until none are left, in
// the order the per-tile grid runs them.  The same tiles, partial slots and
// per-cluster last-arriver reductions: bit-identical results.  Autotuner
// candidates beside the one-block-per-tile grids above.
static __device__ __forceinline__ void orbit_persistent(const Cluster *__restrict__ cls, Tiles tm, const Fields &f,
                                                        double *partials, unsigned int *tickets, const PosQ &pq,
                                                        unsigned int *next, SampleSmem &sm)
{
    __shared__ int s_tile;
    const Learn none{};
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(next, 1u);
        __syncthreads();
        const int b = s_tile;
        if (b >= tm.ntiles) break;
        orbit_body<0>(cls, tm, f, partials, tickets, pq, none, sm, nullptr, b);
        __syncthreads();  // s_tile and the sampling state are the next tile's
    }
}

__global__ void __launch_bounds__(ORB_T, 5) k_orbit_pers(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                      double *partials, unsigned int *tickets, PosQ pq,
                                                      unsigned int *next)
{
    __shared__ SampleSmem sm;
    orbit_persistent(cls, tm, f, partials, tickets, pq, next, sm);
}

__global__ void __launch_bounds__(ORB_T, 4) k_orbit_pers_lb4(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                          double *partials, unsigned int *tickets, PosQ pq,
                                                          unsigned int *next)
{
    __shared__ SampleSmem sm;
    orbit_persistent(cls, tm, f, partials, tickets, pq, next, sm);
}

__global__ void __launch_bounds__(ORB_T, 5) k_orbit_aps(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                     double *partials, unsigned int *tickets, PosQ pq, Learn L)
{
    __shared__ SampleSmem sm;
    orbit_body<1>(cls, tm, f, partials, tickets, pq, L, sm, nullptr, blockIdx.x);
}

__global__ void __launch_bounds__(ORB_T, 5) k_orbit_learn(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                       double *partials, unsigned int *tickets, PosQ pq, Learn L)
{
    __shared__ SampleSmem sm;
    __shared__ LearnSmem ls;
    orbit_body<2>(cls, tm, f, partials, tickets, pq, L, sm, &ls, blockIdx.x);
}

__global__ void __launch_bounds__(ORB_T, 4) k_orbit_learn_lb4(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                           double *partials, unsigned int *tickets, PosQ pq, Learn L)
{
    __shared__ SampleSmem sm;
    __shared__ LearnSmem ls;
    orbit_body<2>(cls, tm, f, partials, tickets, pq, L, sm, &ls, blockIdx.x);
}

// Grid-wide barrier for a co-resident (cooperatively launched) grid:
// bar[0] counts arrivals, bar[1] is the generation.  The wait is bounded; on
// timeout the caller records CMCG_ERR_SPIN and the kernel stops iterating.
static __device__ __forceinline__ bool grid_barrier(unsigned int *bar, unsigned int &gen, int *s_ok)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int want = gen + 1u;
        int ok = 1;
        if (atomicAdd(&bar[0], 1u) + 1u == gridDim.x) {
            bar[0] = 0u;
            __threadfence();
            atomicExch(&bar[1], want);
        } else {
            long long spins = 0;
            while (*(volatile unsigned int *)&bar[1] != want) {
                if (++spins > CMCG_SPIN_LIMIT) {
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        gen = want;
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Tidal radius and its potential for the coming pass of cluster c
// (cmc_evolution_thr.c:459-466).
static __device__ __forceinline__ void tidal_radius(const Cluster &C, const Fields &f)
{
    Scalars *sc = C.sc;
    const double Rt = sc->orbit_r * pow(sc->Mtotal - (sc->TidalMassLoss - sc->OldTidalMassLoss), 1.0 / 3.0);
    int pok = 1;
    const double phi = potential_at(f.r + C.off, f.phi + C.off, f.inv_r + C.off, sc->N_MAX, Rt, &pok, ridx_of(C, f));
    if (!pok) set_error(sc, CMCG_ERR_FINDZERO_R, 0);
    sc->tid_Rt = Rt;
    sc->tid_phirt = phi;
}

// tidally_strip_stars, cmc_evolution_thr.c:443-646: the iteration in one
// cooperative launch.  Each pass scans every tile of every cluster not yet
// settled (tiles strided over the co-resident grid, per-tile partials), then
// one block per cluster sums its tiles in tile order, records the pass
// (Rtidal, tallies) and either settles the cluster or prepares the next
// radius.  At most TIDAL_PASSES passes; a cluster still shedding mass after
// them is an error (CMCG_ERR_TIDAL_ITER).
__global__ void __launch_bounds__(TID_THREADS) k_tidal(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                       double *partials, unsigned int *bar, int nclusters)
{
    __shared__ double s_acc[TID_THREADS / 32][TID_NPART];
    __shared__ int s_ok;
    unsigned int gen = 0;
    if (threadIdx.x == 0) gen = *(volatile unsigned int *)&bar[1];
    for (int c = blockIdx.x; c < nclusters; c += gridDim.x) {
        const Cluster &C = cls[c];
        if (threadIdx.x == 0 && counts_ok(C) && !C.sc->tidal_done) tidal_radius(C, f);
    }
    if (!grid_barrier(bar, gen, &s_ok)) {
        if (threadIdx.x == 0) set_error(cls[0].sc, CMCG_ERR_SPIN, 0);
        return;
    }
    for (int pass = 0; pass < TIDAL_PASSES; ++pass) {
        for (int b = blockIdx.x; b < tm.ntiles; b += gridDim.x) {
            const int2 ct = tm.tiles[b];
            const Cluster &C = cls[ct.x];
            Scalars *sc = C.sc;
            if (*(volatile int *)&sc->tidal_done || !counts_ok(C)) continue;
            const long long off = C.off;
            const double NSTAR = (double)sc->N_STAR;
            const double phi_rtidal = *(volatile double *)&sc->tid_phirt, Rtidal = *(volatile double *)&sc->tid_Rt;
            const double gierszalpha = sc->tid_alpha;
            double acc[TID_NPART] = {0.0, 0.0, 0.0, 0.0};  // E, J, M, Etidal
            const long long N_NEW = sc->N_MAX_NEW;
            // the tile's (rnew, criterion) pairs are loaded before any test, so
            // their latencies overlap; stars past N_MAX_NEW read as never stripped
            constexpr int IT = TID_T / TID_THREADS;
            const long long i0 = 1 + (long long)ct.y * TID_T + threadIdx.x;
            const double *crit = (C.TIDAL_TREATMENT == 0) ? f.r_apo : f.E;
            const double bound = (C.TIDAL_TREATMENT == 0) ? Rtidal : gierszalpha * phi_rtidal;
            const long long kbound = bound_key(bound);  // the tests below are integer ones
            double rnv[IT], cv[IT];
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                const long long i = i0 + it * TID_THREADS;
                const bool in = i <= N_NEW;
                rnv[it] = in ? f.rnew[off + i] : CMCG_SF_INFINITY;
                cv[it] = in ? crit[off + i] : 0.0;
            }
#pragma unroll
            for (int it = 0; it < IT; ++it) {
                const long long g = off + i0 + it * TID_THREADS;
                // r_apo > Rtidal (treatment 0) or E > gierszalpha * phi_rtidal, and rnew < 1e6
                if (gt_key(cv[it], kbound) && lt_pos(rnv[it], 1000000.0)) {
                    const double m = f.m[g], E = f.E[g], J = f.J[g];
                    acc[0] += E * m / NSTAR;
                    acc[1] += J * m / NSTAR;
                    acc[2] += m / NSTAR;
                    acc[3] += E * m / NSTAR;
                    destroy_obj(f, g);
                }
            }
            __syncthreads();  // s_acc is reused tile after tile
            block_sums<TID_THREADS>(acc, s_acc);  // stripped stars are few: most warps skip
            if (threadIdx.x == 0) {
                double *slot = partials + (size_t)b * TID_NPART;
                for (int q = 0; q < TID_NPART; ++q) slot[q] = acc[q];
            }
        }
        if (!grid_barrier(bar, gen, &s_ok)) {
            if (threadIdx.x == 0) set_error(cls[0].sc, CMCG_ERR_SPIN, pass);
            return;
        }
        // one block per cluster: the pass's sums in tile order
        for (int c = blockIdx.x; c < nclusters; c += gridDim.x) {
            const Cluster &C = cls[c];
            Scalars *sc = C.sc;
            if (*(volatile int *)&sc->tidal_done || !counts_ok(C)) continue;
            // the cluster's tiles in a fixed order: strided per thread, then block_sums
            double a[TID_NPART] = {0.0, 0.0, 0.0, 0.0};
            for (int t = threadIdx.x; t < tm.count[c]; t += TID_THREADS) {
                const double *pt = partials + (size_t)(tm.first[c] + t) * TID_NPART;
                for (int q = 0; q < TID_NPART; ++q) a[q] += __ldcg(pt + q);
            }
            __syncthreads();
            block_sums<TID_THREADS>(a, s_acc);
            if (threadIdx.x == 0) {
                if (sc->tidal_iters == 0) sc->Etidal = 0.0;  // cmc_evolution_thr.c:452
                sc->Rtidal = sc->tid_Rt;
                sc->phi_rtidal = sc->tid_phirt;
                sc->Eescaped += a[0];
                sc->Jescaped += a[1];
                sc->Etidal += a[3];
                sc->DTidalMassLoss = a[2];
                sc->TidalMassLoss += a[2];
                sc->tidal_iters += 1;
                if (!(a[2] > 0)) {
                    sc->tidal_done = 1;
                } else if (pass + 1 == TIDAL_PASSES) {
                    set_error(sc, CMCG_ERR_TIDAL_ITER, sc->tidal_iters);
                } else {
                    tidal_radius(C, f);
                }
            }
            __syncthreads();
        }
        if (!grid_barrier(bar, gen, &s_ok)) {
            if (threadIdx.x == 0) set_error(cls[0].sc, CMCG_ERR_SPIN, pass);
            return;
        }
        int open = 0;
        for (int c = 0; c < nclusters && !open; ++c) open = !*(volatile int *)&cls[c].sc->tidal_done;
        if (!open) break;
    }
}

// potential(r) for one radius of cluster c (host queries, energy bookkeeping).
__global__ void k_potential_query(const Cluster *__restrict__ cls, Fields f, int c, double x, double *out)
{
    const Cluster &C = cls[c];
    if (!counts_ok(C)) {
        out[0] = 0.0;
        out[1] = 1.0;
        return;
    }
    int ok = 1;
    out[0] = potential_at(f.r + C.off, f.phi + C.off, f.inv_r + C.off, C.sc->N_MAX, x, &ok, ridx_of(C, f));
    out[1] = ok ? 0.0 : 1.0;
}

// Every stage of the certified sign test at one point (cmcg_sign_stages).
__global__ void k_sign_stages(const double *E, const double *J, const double *rj, const double *mj, double invN,
                              const double *rk, const double *phik, long long n, int *out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double r = rk[i], ph = phik[i];
    const double ps = __dmul_rn(__ddiv_rn(mj[i], rj[i]), invN);
    OrbitCtx o;
    o.invN = invN;
    // the per-star constants exactly as make_orbit_ctx forms them
    o.s.E = (float)E[i];
    o.s.El = (float)(E[i] - (double)o.s.E);
    o.s.J = (float)J[i];
    o.s.Jl = (float)(J[i] - (double)o.s.J);
    const double mjN = mj[i] * invN;
    o.s.mjN = (float)mjN;
    o.s.mjNl = (float)(mjN - (double)o.s.mjN);
    o.s.pj = (float)ps;
    o.s.pjl = (float)(ps - (double)o.s.pj);
    o.s.rj = rj[i];
    o.s.Ed = E[i];
    o.s.Jd = J[i];
    o.s.mjNd = mjN;
    o.s.pjd = ps;
    const bool ge = r >= rj[i];
    const float4 rp = rphi_entry(r, ph);
    out[4 * i + 0] = fq_sign_f32(o.s, rp, ge);
    out[4 * i + 1] = fq_sign_ff(o.s, rp, ge);
    out[4 * i + 2] = fq_sign_f64(o.s, __drcp_rn(r), ph, ge);
    const double q = function_q_dd(r, ph, E[i], J[i], rj[i], mj[i], invN);
    out[4 * i + 3] = (q > 0.0) - (q < 0.0);
}

}  // namespace cmcg

extern "C" int cmcg_sign_stages(const double *E, const double *J, const double *rj, const double *mj, double invN,
                                const double *rk, const double *phik, long n, int *out)
{
    using namespace cmcg;
    if (n < 0 || (n > 0 && (!E || !J || !rj || !mj || !rk || !phik || !out))) return CMCG_ERR_ARG;
    if (n == 0) return CMCG_OK;
    const size_t nd = (size_t)n * sizeof(double);
    double *d = nullptr;
    int *dout = nullptr;
    if (cudaMalloc(&d, 6 * nd) != cudaSuccess) return CMCG_ERR_NOMEM;
    if (cudaMalloc(&dout, 4 * (size_t)n * sizeof(int)) != cudaSuccess) {
        cudaFree(d);
        return CMCG_ERR_NOMEM;
    }
    const double *src[6] = {E, J, rj, mj, rk, phik};
    int rc = CMCG_OK;
    for (int a = 0; a < 6 && rc == CMCG_OK; ++a)
        if (cudaMemcpy(d + (size_t)a * n, src[a], nd, cudaMemcpyHostToDevice) != cudaSuccess) rc = CMCG_ERR_CUDA;
    if (rc == CMCG_OK) {
        k_sign_stages<<<(unsigned)((n + 255) / 256), 256>>>(d, d + n, d + 2 * n, d + 3 * n, invN, d + 4 * n, d + 5 * n,
                                                           n, dout);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(out, dout, 4 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = CMCG_ERR_CUDA;
    }
    cudaFree(d);
    cudaFree(dout);
    return rc;
}

extern "C" int cmcg_orbit_counters(unsigned long long out[CMCG_ORBIT_NCOUNTERS], int reset)
{
    using namespace cmcg;
    if (!out) return CMCG_ERR_ARG;
    if (cudaDeviceSynchronize() != cudaSuccess) return CMCG_ERR_CUDA;
    if (cudaMemcpyFromSymbol(out, g_orbit_rare, sizeof(g_orbit_rare)) != cudaSuccess) return CMCG_ERR_CUDA;
    if (reset) {
        const unsigned long long zero[CMCG_ORBIT_NCOUNTERS] = {0, 0, 0, 0};
        if (cudaMemcpyToSymbol(g_orbit_rare, zero, sizeof(zero)) != cudaSuccess) return CMCG_ERR_CUDA;
    }
    return CMCG_OK;
}
