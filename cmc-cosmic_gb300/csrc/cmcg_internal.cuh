// cmcg_internal.cuh -- device data layout and shared device helpers.
//
// Layout in HBM.  Every cluster of a context owns a contiguous slice of each
// structure-of-arrays field: element k of cluster c lives at off[c] + k, with
// k = 0 and k = N+1 the reference's sentinels (star_r[0] = 1e-20,
// star_r[N+1] = 1e10) and stars at 1..N in radial order.  Slices start on
// 256-byte boundaries so a tile of doubles is one aligned 128-bit-vector run.
// Kernels map blocks to (cluster, tile) pairs through a per-tile-size table,
// so one launch covers an ensemble of clusters with uneven N and no tile ever
// straddles two clusters.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CMCG_SF_INFINITY 1.0e10      /* include/cmc/cmc.h:58 */
#define CMCG_ZERO 1.0e-20            /* include/cmc/cmc.h:60 */
#define CMCG_PI 3.14159265358979323  /* include/cmc/cmc.h:62 */
#define CMCG_DBL_EPSILON 2.2204460492503131e-16
#define CMCG_DBL_MIN 2.2250738585072014e-308

// Bounded waits: every cross-block spin gives up after this many polls and
// records CMCG_ERR_SPIN instead of hanging the GPU.
#define CMCG_SPIN_LIMIT (1 << 22)

namespace cmcg {

// Per-cluster scalar state (the reference's globals for one cluster).
struct Scalars {
    long long N_MAX, N_MAX_NEW, N_STAR, tcount;
    double Mtotal, Rtidal, orbit_r, madhoc, cenma_m, cenma_E;
    double Dt, Prev_Dt, TotalTime, max_r;
    double TidalMassLoss, TidalMassLoss_old, OldTidalMassLoss, DTidalMassLoss;
    double Eescaped, Jescaped, Etidal, Eoops, Eescaped_old, Jescaped_old, Etidal_old;
    double Etot, KE, PE, Etot_ini;
    long long Nrel, Nrelbeta[4];
    double qaverelbeta[4], maverelbeta[4], raverelbeta[4];
    double phi_rtidal, gierszalpha;
    double tid_Rt, tid_phirt;  // tidal radius and its potential for the coming stripping pass
    double tid_alpha;          // gierszalpha (cmc_evolution_thr.c:550), fixed by GAMMA and N_STAR
    int tidal_done, tidal_iters;
    int err;
    int pad0;
    long long err_index;
    // sort bookkeeping
    long long n_bound;     // stars kept after the sort (r < SF_INFINITY)
    // set_velocities3 bookkeeping
    long long n_excess;    // stars whose predicted v^2 <= 0
    // potential bookkeeping: sequential points of the three recurrences, and
    // whether the last potential fell back to the one-thread loop
    long long phi_nsp[3];
    long long phi_fallback;
    // radius index (RIdx) of the current star order
    long long ridx_base;
    int ridx_shift, ridx_ok;
};

// Per-cluster constant description (built on the host, read-only on device).
struct Cluster {
    long long off;         // element offset of index 0 (sentinel) of this cluster
    long long cap;         // capacity in stars
    Scalars *sc;
    // parameters (.ini keys)
    long long p;           // AVEKERNEL
    double GAMMA, THETASEMAX;
    int PERTURB, RELAXATION, TIDALLY_STRIP_STARS, TIDAL_TREATMENT;
    long long n_try, apsides_max_iter;
    double apsides_precision, apsides_convergence;
    unsigned long long seed;
    int relax_fp32;
    int phi_sequential;    // 1: potential by the plain sequential loop (one thread)
    long long rec_off, rec_cap;  // this cluster's slice of the sequential-point records
    long long ridx_off;    // this cluster's radius index table (ridx_B + 1 entries)
    int ridx_B;
    int check_filters;     // verify every certified FP32 trial decision exactly (CMCG_ERR_FILTER)
};

// Device-resident fields (all concatenated over clusters).
struct Fields {
    double *r, *m, *phi, *inv_r;       // star_r, star_m, star_phi, 1/star_r
    double *vr, *vt, *E, *J;           // star[].vr, .vt, .E, .J
    double *vr_rel, *vt_rel;           // velocities after relaxation (star[].vr/.vt then)
    double *rnew, *vrnew, *vtnew;      // star[].rnew, .vrnew, .vtnew
    double *X, *Y, *r_peri, *r_apo;    // star[].X, .Y, .r_peri, .r_apo
    double *ec_pre;                    // vold^2 + (Uoldrold - Uoldrnew), see set_velocities3
    double *rOld;                      // star[].rOld after the sort
    double *sigma_r, *sigma;           // sigma_array.r, sigma_array.sigma
    float4 *rphif;                     // (r_k, Phi_k hi, Phi_k lo, 0) as floats: certified FP32 sign tests
    int *ridx;                         // radius index tables of all clusters (RIdx)
    long long *id;                     // star[].id
    // second buffers for the sort's gather (swapped on the host)
    double *r2, *m2, *ec_pre2;
    long long *id2;
};

// Block -> (cluster, tile) table entry for one tile size.
struct TileMap {
    const int2 *tiles;   // .x = cluster, .y = tile index within the cluster
    int ntiles;
};

// Deterministic cross-block reductions: each block writes its partials to a
// slot, the last block to arrive (atomic ticket) combines them in block order.
struct Partials {
    double *d;           // [ntiles][nd]
    unsigned int *ticket;// one counter per cluster
};

__device__ __forceinline__ void set_error(Scalars *sc, int code, long long idx)
{
    if (atomicCAS(&sc->err, 0, code) == 0) sc->err_index = idx;
}

// Every kernel checks the star counts it will index with against the
// cluster's capacity before touching memory (code 22 = CMCG_ERR_BOUNDS).
__device__ __forceinline__ bool counts_ok(const Cluster &C)
{
    const Scalars *sc = C.sc;
    const long long a = sc->N_MAX, b = sc->N_MAX_NEW;
    if (a < 0 || a > C.cap || b < 0 || b > C.cap) {
        set_error(C.sc, 22, a > C.cap || a < 0 ? a : b);
        return false;
    }
    return true;
}

// ---------------------------------------------------------------- Philox --
// Philox4x32-10 (Salmon et al., SC'11).  The same keying as the oracle:
// key = (seed lo, seed hi ^ tcount), counter = (id lo, id hi, site, n).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        if (i > 0) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        unsigned int hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        unsigned int hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

enum { SITE_Y = 1, SITE_PENC = 2, SITE_PSI = 3, SITE_TRIAL = 4, SITE_SIGN = 5, SITE_LTRIAL = 6 };

__device__ __forceinline__ uint4 draw_block(unsigned long long seed, long long tcount, int site,
                                            long long id, unsigned int n)
{
    uint2 key = make_uint2((unsigned int)seed, (unsigned int)(seed >> 32) ^ (unsigned int)tcount);
    unsigned long long uid = (unsigned long long)id;
    return philox4x32_10(make_uint4((unsigned int)uid, (unsigned int)(uid >> 32), (unsigned int)site, n), key);
}

// u32 -> [0,1) with the reference's 32-bit resolution (taus113-v2.c:186):
// u / 2^32, which is exact, assembled from its bits with integer instructions
// (the same double as (double)u / 4294967296.0, without the FP64 pipe).
__device__ __forceinline__ double u01(unsigned int u)
{
    if (u == 0u) return 0.0;
    const int lz = __clz(u);  // the leading 1 is bit 31 - lz: u 2^-32 = 2^(-1-lz) (1.f)
    const unsigned long long frac = (unsigned long long)(lz == 31 ? 0u : (u << (lz + 1))) << 20;
    return __longlong_as_double((long long)(((unsigned long long)(1022 - lz) << 52) | frac));
}

// ------------------------------------------------------- double-double --
// Error-free transformations (Knuth two-sum, FMA two-product) used to
// evaluate function_q with more precision than the reference's long double,
// so that the sign tests of its bisections agree.
struct dd {
    double hi, lo;
};
__device__ __forceinline__ dd two_sum(double a, double b)
{
    double s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    double err = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
    return {s, err};
}
__device__ __forceinline__ dd quick_two_sum(double a, double b)
{
    double s = __dadd_rn(a, b);
    return {s, __dsub_rn(b, __dsub_rn(s, a))};
}
__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo = __dadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __dadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_mul_d(dd a, double b)
{
    double p = __dmul_rn(a.hi, b);
    double e = __fma_rn(a.hi, b, -p);
    e = __fma_rn(a.lo, b, e);
    return quick_two_sum(p, e);
}
// a / b for doubles a, b, to double-double accuracy
__device__ __forceinline__ dd dd_div_dd(double a, double b)
{
    double q1 = __ddiv_rn(a, b);
    double r = __fma_rn(-q1, b, a);       // exact remainder a - q1*b
    double q2 = __ddiv_rn(r, b);
    return quick_two_sum(q1, q2);
}
// (long double)a / (long double)b where b is given as double-double
__device__ __forceinline__ dd dd_div_d_dd(double a, dd b)
{
    double q1 = __ddiv_rn(a, b.hi);
    // r = a - q1*b (to dd)
    double p = __dmul_rn(q1, b.hi);
    double pe = __fma_rn(q1, b.hi, -p);
    pe = __fma_rn(q1, b.lo, pe);
    double r = __dsub_rn(__dsub_rn(a, p), pe);
    double q2 = __ddiv_rn(r, b.hi);
    return quick_two_sum(q1, q2);
}

// ------------------------------------------------------ table lookups ---
// Orders positive doubles by their bit patterns (integer compare, no FP64 pipe).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
constexpr unsigned long long SIGN_BIT = 0x8000000000000000ull, INF_BITS = 0x7ff0000000000000ull;

// FP64 comparisons decided on the operands' bit patterns with integer
// instructions: on this GPU a DSETP occupies the FP64 pipe like an FMA.  Each
// returns exactly what the IEEE comparison returns, for signed zeros,
// infinities and NaNs too; c is a positive finite double.
__device__ __forceinline__ unsigned long long ubits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ bool ge0(double x)  // x >= 0.0
{
    const unsigned long long b = ubits(x);
    return b <= INF_BITS || b == SIGN_BIT;
}
__device__ __forceinline__ bool lt0(double x)  // x < 0.0
{
    const unsigned long long b = ubits(x);
    return b > SIGN_BIT && b <= (SIGN_BIT | INF_BITS);
}
__device__ __forceinline__ bool le0(double x)  // x <= 0.0
{
    const unsigned long long b = ubits(x);
    return b == 0 || (b >= SIGN_BIT && b <= (SIGN_BIT | INF_BITS));
}
__device__ __forceinline__ bool gt0(double x)  // x > 0.0
{
    const unsigned long long b = ubits(x);
    return b != 0 && b <= INF_BITS;
}
__device__ __forceinline__ bool eq0(double x) { return (ubits(x) & ~SIGN_BIT) == 0; }  // x == 0.0
__device__ __forceinline__ bool lt_pos(double x, double c)  // x < c
{
    const unsigned long long b = ubits(x);
    return b < SIGN_BIT ? b < ubits(c) : b <= (SIGN_BIT | INF_BITS);
}
__device__ __forceinline__ bool ge_pos(double x, double c)  // x >= c
{
    const unsigned long long b = ubits(x);
    return b >= ubits(c) && b <= INF_BITS;
}
// An ordered integer key of a double that is not a NaN: okey(x) < okey(y)
// exactly when x < y, and okey(-0.0) == okey(+0.0).
__device__ __forceinline__ long long okey(double x)
{
    const unsigned long long b = ubits(x), m = b & ~SIGN_BIT;
    return (b & SIGN_BIT) ? -(long long)m : (long long)m;
}
// The key a bound c is compared by in gt_key: a NaN bound gets a key no
// double reaches, since x > NaN is false.
__device__ __forceinline__ long long bound_key(double c)
{
    return (ubits(c) & ~SIGN_BIT) > INF_BITS ? 0x7fffffffffffffffll : okey(c);
}
__device__ __forceinline__ bool gt_key(double x, long long kc)  // x > c, with kc = bound_key(c)
{
    return (ubits(x) & ~SIGN_BIT) <= INF_BITS && okey(x) > kc;
}
__device__ __forceinline__ bool gt_pos(double x, double c)  // x > c
{
    const unsigned long long b = ubits(x);
    return b > ubits(c) && b <= INF_BITS;
}

// hi = (float)x and lo = (float)(x - (double)hi), both rounded to nearest
// even, from x's bits with integer instructions (FP64 conversions take the
// FP64 pipe).  hi keeps the top 24 of the 53 significand bits, rounded on the
// 29 below; x - hi is then D 2^(e-1075) exactly (|D| <= 2^28, e the biased
// exponent), and RN(D) scaled by a power of two is RN(x - hi).  The fast path
// takes 2^-74 <= |x| < 2^127, where hi and a nonzero lo are normal floats;
// other x go through the FP64 conversions.
__device__ __forceinline__ void f2_split(double x, float &hi, float &lo)
{
    const unsigned long long b = ubits(x);
    const int ed = (int)((b >> 52) & 0x7ffu);
    if (ed < 949 || ed > 1149) {
        hi = (float)x;
        lo = (float)(x - (double)hi);
        return;
    }
    const unsigned long long S = (b & 0x000fffffffffffffull) | (1ull << 52);
    unsigned long long H = S >> 29;
    const unsigned long long rem = S & ((1ull << 29) - 1);
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (H & 1ull))) ++H;  // H in [2^23, 2^24]
    const long long D = (long long)S - (long long)(H << 29);
    const unsigned int sgn = (unsigned int)(b >> 32) & 0x80000000u;
    // (e_f << 23) + (H - 2^23): a carry of H to 2^24 moves into the exponent
    hi = __uint_as_float(((unsigned int)(ed - 896) << 23) + (unsigned int)(H - (1ull << 23)) | sgn);
    const float scale = __uint_as_float((unsigned int)(ed - 1075 + 127) << 23);  // 2^(ed-1075), normal here
    const float l = __fmul_rn(__ll2float_rn(D), scale);
    lo = sgn ? -l : l;
}

// (float)x, rounded to nearest even (the hi part of f2_split).
__device__ __forceinline__ float d2f_rn(double x)
{
    float hi, lo;
    f2_split(x, hi, lo);
    return hi;
}

// (double)x, which is exact, assembled from x's bits with integer
// instructions for normal floats and zeros (the FP64 conversion takes the
// FP64 pipe); subnormals, infinities and NaN go through the conversion.
__device__ __forceinline__ double f2d_exact(float x)
{
    const unsigned int u = __float_as_uint(x);
    const unsigned int e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    if (e == 0u) {
        if ((u & 0x7fffffu) == 0u) return __longlong_as_double((long long)sgn);  // +-0
        return (double)x;
    }
    if (e == 0xffu) return (double)x;
    return __longlong_as_double(
        (long long)(sgn | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// FindZero_r, cmc_nr.c:62-82: largest k in [kmin,kmax] with r[k] < x (x > 0),
// for kmin < kmax (the only way the reference calls it).  The bisection
// halves a range of at most 2^63, so 64 rounds bound it.
__device__ __forceinline__ long long find_zero_r(const double *__restrict__ r, long long kmin, long long kmax,
                                                 double x)
{
    const long long xb = dbits(x);
    for (int it = 0; it < 64 && kmax != kmin; ++it) {
        long long ktry = (kmin + kmax + 1) >> 1;
        if (dbits(__ldg(r + ktry)) < xb)
            kmin = ktry;
        else
            kmax = ktry - 1;
    }
    return kmin;
}

// Bucketed index over the sorted radii: bucket(x) = (bits(x) - bits(r_1)) >> shift,
// clamped to B-1, and T[b] = the first star k in 1..N+1 whose radius lies in
// bucket b or above (T[B] = N+2).  Every star below T[b] has r_k < x and every
// star from T[b+1] on has r_k > x for x in bucket b, so the reference's search
// for x can start from [T[b]-1, T[b+1]-1] and gives the same index.
struct RIdx {
    const int *T;        // null: no index (radii not known to be in order)
    long long base;
    int shift, B;
};

__device__ __forceinline__ int ridx_bucket(const RIdx &ix, double x)
{
    const long long d = __double_as_longlong(x) - ix.base;
    if (d < 0) return 0;
    const long long b = d >> ix.shift;
    return b >= ix.B - 1 ? ix.B - 1 : (int)b;
}

// FindZero_r's answer for x >= r[1] (cmc_utils.c:140-146): the largest k in
// [1, N_MAX+1] with r[k] < x, through the radius index when there is one.
__device__ __forceinline__ long long potential_index(const double *__restrict__ r, long long N_MAX, double x,
                                                     const RIdx &ix)
{
    if (N_MAX == 1) return 1;
    if (ix.T) {
        const int b = ridx_bucket(ix, x);
        long long lo = __ldg(ix.T + b) - 1, hi = __ldg(ix.T + b + 1) - 1;
        if (lo < 1) lo = 1;
        if (hi > N_MAX + 1) hi = N_MAX + 1;
        return (hi <= lo) ? lo : find_zero_r(r, lo, hi, x);
    }
    return find_zero_r(r, 1, N_MAX + 1, x);
}

// The Henon interpolation of potential(r) in interval i (cmc_utils.c:147-163).
__device__ __forceinline__ double potential_in(const double *__restrict__ r, const double *__restrict__ phi,
                                               const double *__restrict__ inv_r, long long N_MAX, double x,
                                               long long i, int *ok, double ix = 0.0)
{
    if (i > N_MAX) {  // x beyond the r = SF_INFINITY sentinel: the reference's check fails too
        *ok = 0;
        return 0.0;
    }
    const double ri = __ldg(r + i), ri1 = __ldg(r + i + 1);
    if (ri > x || ri1 < x) {
        *ok = 0;
        return 0.0;
    }
    if (i == 0) return __ldg(phi + 1);
    const double pi = __ldg(phi + i), pi1 = __ldg(phi + i + 1);
    const double ii = __ldg(inv_r + i), ii1 = __ldg(inv_r + i + 1);
    if (ix == 0.0) ix = __drcp_rn(x);  // 1.0 / x, correctly rounded (or the caller's copy of it)
    return __dadd_rn(pi, __ddiv_rn(__dmul_rn(__dsub_rn(pi1, pi), __dsub_rn(ii, ix)), __dsub_rn(ii, ii1)));
}

// potential(r), cmc_utils.c:112-164 with SEARCH_GRID = 0.  inv_r[k] holds the
// correctly rounded 1.0/r[k], so the Henon interpolation performs exactly the
// reference's divisions with two of the three precomputed.
__device__ __forceinline__ double potential_at(const double *__restrict__ r, const double *__restrict__ phi,
                                               const double *__restrict__ inv_r, long long N_MAX, double x,
                                               int *ok, const RIdx &ix = RIdx{nullptr, 0, 0, 0})
{
    if (x == 0.0) return __ldg(phi);
    const double r1 = __ldg(r + 1);
    if (x < r1) {
        double p0 = __ldg(phi), p1 = __ldg(phi + 1);
        return __dsub_rn(p0, __ddiv_rn(__dmul_rn(__dsub_rn(p0, p1), r1), x));
    }
    return potential_in(r, phi, inv_r, N_MAX, x, potential_index(r, N_MAX, x, ix), ok);
}

// The radius index of cluster C, or none while it is stale.
__device__ __forceinline__ RIdx ridx_of(const Cluster &C, const Fields &f)
{
    const Scalars *sc = C.sc;
    if (!sc->ridx_ok || !f.ridx) return RIdx{nullptr, 0, 0, 0};
    return RIdx{f.ridx + C.ridx_off, sc->ridx_base, sc->ridx_shift, C.ridx_B};
}

// a / b rounded to nearest, given y = RN(1/b), in five FP64 operations instead
// of a division.  Markstein's theorem (P. Markstein, IBM J. Res. Dev. 34, 1990;
// restated as the quotient-correction theorem in Muller et al., Handbook of
// Floating-Point Arithmetic): if y is within half an ulp of 1/b and q within
// one ulp of a/b, then r = a - b q is exact (one FMA) and RN(q + r y) = RN(a/b).
// q0 = RN(a y) may lie up to 1.5 ulp from a/b; one correction brings it within
// half an ulp plus 2^-52 ulp, and the second correction is the theorem's step.
// Valid for normal operands whose quotient and remainders stay normal, which
// holds for the radii, masses, potentials and angular momenta it is used on.
__device__ __forceinline__ double div_rcp(double a, double b, double y)
{
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-q0, b, a), y, q0);
    return __fma_rn(__fma_rn(-q1, b, a), y, q1);
}

// MPI_PHI_S(rad, j), cmc.h:2175
__device__ __forceinline__ double phi_s(double rad, double rj, double mj, double invN)
{
    double t = (rad >= rj) ? __ddiv_rn(mj, rad) : __ddiv_rn(mj, rj);
    return __dmul_rn(t, invN);
}

// function_q, cmc_utils.c:1654-1662, which the reference evaluates in long
// double (SQR rounds J/r to double first, cmc.h:2030).  Evaluated here in
// double-double and rounded once to double.
__device__ __forceinline__ double function_q_dd(double r, double pot, double E, double J, double rj, double mj,
                                                double invN)
{
    const double q = __ddiv_rn(J, r);              // (double)(J/r)
    const double Jr = (q == 0.0) ? 0.0 : __dmul_rn(q, q);
    dd phis;
    if (r >= rj) {
        phis = dd_div_dd(mj, r);                    // m_j / r in extended precision
    } else {
        phis = {__ddiv_rn(mj, rj), 0.0};            // double division, then widened
    }
    phis = dd_mul_d(phis, invN);                    // * (1.0/N_STAR)
    dd t = dd_add({pot, 0.0}, phis);                // pot + phis
    dd u = dd_add({E, 0.0}, dd_neg(t));             // E - (pot + phis)
    u.hi *= 2.0;
    u.lo *= 2.0;
    dd res = dd_add(u, {-Jr, 0.0});                 // 2(E - ...) - Jr
    return __dadd_rn(res.hi, res.lo);
}

// Certified FP32 sign of function_q at a table point (r, Phi given as the
// round-to-nearest floats of the FP64 table).  Every input conversion,
// reciprocal, product and difference contributes at most a few units of 2^-24;
// summed, |Q_f32 - Q| <= 12.2u(|E|+|Phi|+|phis|) + 10.1u (J/r)^2 (u = 2^-24),
// and the threshold below is twice that.  Beyond it the FP32 sign is the exact
// sign, hence also the sign of the reference's long double evaluation.
// Returns +1, -1, or 0 when the caller must evaluate in double-double.
struct QF32 {
    float E, El, J, mjN, pj;  // E as a float pair (E ~ E + El), J, m_j/N_STAR, (m_j/r_j)/N_STAR as floats
    float Jl, mjNl, pjl;      // low parts of J, m_j/N_STAR, (m_j/r_j)/N_STAR (float-float stage)
    double rj;                // r_j: the self-potential branch is chosen in FP64
    double Ed, Jd, mjNd, pjd; // the same in FP64, for the second filter
};

// (r hi, Phi hi, Phi lo, r lo): r and Phi as float pairs hi + lo, each within
// 2^-48 of the double it stands for
__device__ __forceinline__ float4 rphi_entry(double r, double phi)
{
    float ph, pl, rh, rl;
    f2_split(phi, ph, pl);
    f2_split(r, rh, rl);
    return make_float4(rh, ph, pl, rl);
}

// E - Phi is formed in float-float (exact difference of the high parts plus
// the low parts), so its error is 2^-23 |E - Phi| + 2^-46 (|E| + |Phi|) rather
// than 2^-24 of each term.  With the reciprocal of the float radius (2^-23)
// the self-potential carries at most 2^-22, (J/r)^2 at most 2^-20.7, and the
// final combinations 2^-24 of their magnitudes:
//   |Q_f32 - Q| <= 2^-21 (|D| + phis + |A|) + 2^-20.5 (J/r)^2 + 2^-45 (|E| + |Phi|),
// D = E - Phi, A = D - phis.  The threshold below is over twice that.
__device__ __forceinline__ int fq_sign_f32(const QF32 &s, float4 rp, bool ge)
{
    const float ir = __frcp_rn(rp.x);
    const float phis = ge ? s.mjN * ir : s.pj;
    const float d = s.E - rp.y;
    const float bv = d - s.E;
    const float err = (s.E - (d - bv)) + (-rp.y - bv);  // Eh - Phi_hi = d + err exactly
    const float D = d + (err + (s.El - rp.z));
    const float A = D - phis;
    const float q = s.J * ir;
    const float B = q * q;
    // (J/r)^2 beyond the float range (the r = 1e-20 sentinel at k = 0) against a
    // finite 2(E - Phi - phis): Q is negative however either is rounded
    if (B == INFINITY && fabsf(A) < 1e30f) return -1;
    const float Q = 2.0f * A - B;
    const float bound = 0x1p-19f * (fabsf(D) + fabsf(phis) + fabsf(A) + B) + 0x1p-42f * (fabsf(s.E) + fabsf(rp.y));
    if (Q > bound) return 1;
    if (Q < -bound) return -1;
    return 0;
}

__device__ __forceinline__ float2 ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}

// Certified float-float sign of function_q at a table point: every operand an
// unevaluated float pair (within 2^-48 of its double), 1/r as y0 (1 + e) with
// y0 the float reciprocal and e = 1 - r y0 from FMAs, J/r and m_j/(N r) as
// compensated products, (J/r)^2 as a compensated square, the differences by
// two-sum (Knuth).  With u = 2^-24, charging every rounding and neglected
// term: 1/r to 9u^2, J/r to 17u^2, (J/r)^2 to 39u^2, the self-potential to
// 17u^2, E - Phi to 4u^2 (|E| + |Phi|); the two differences add at most
// 8u^2 (|E| + |Phi|) + 12u^2 phis + 6u^2 |A| + 4u^2 (J/r)^2.  In all
//   |Q_ff - Q| <= 20u^2 (|E|+|Phi|) + 52u^2 phis + 6u^2 |A| + 43u^2 (J/r)^2
// below 2^-42 of the magnitudes' sum; the reference's own roundings (J/r
// rounded to double: 2^-52 (J/r)^2; long double) add under 2^-51 of it.  The
// threshold is 2^-40 of the sum, plus 1e-30 against underflow.  Returns +1,
// -1, or 0 (undecided: within about 2^-40 of a root).
__device__ __forceinline__ int fq_sign_ff(const QF32 &s, float4 rp, bool ge)
{
    const float y0 = __frcp_rn(rp.x);
    const float e = __fmaf_rn(-rp.w, y0, __fmaf_rn(-rp.x, y0, 1.0f));
    const float il = __fmul_rn(y0, e);  // 1/r ~ y0 + il
    const float q = __fmul_rn(s.J, y0);
    const float ql = __fadd_rn(__fmaf_rn(s.J, y0, -q), __fadd_rn(__fmul_rn(s.J, il), __fmul_rn(s.Jl, y0)));
    const float b = __fmul_rn(q, q);
    const float bl = __fadd_rn(__fmaf_rn(q, q, -b), __fmul_rn(__fmul_rn(2.0f, q), ql));
    float ph = s.pj, pl = s.pjl;
    if (ge) {
        ph = __fmul_rn(s.mjN, y0);
        pl = __fadd_rn(__fmaf_rn(s.mjN, y0, -ph), __fadd_rn(__fmul_rn(s.mjN, il), __fmul_rn(s.mjNl, y0)));
    }
    const float2 d = ff_two_sum(s.E, -rp.y);
    const float dl = __fadd_rn(d.y, __fsub_rn(s.El, rp.z));
    const float2 a = ff_two_sum(d.x, -ph);
    const float al = __fadd_rn(a.y, __fsub_rn(dl, pl));
    const float2 qq = ff_two_sum(__fmul_rn(2.0f, a.x), -b);
    const float Q = __fadd_rn(qq.x, __fadd_rn(qq.y, __fsub_rn(__fmul_rn(2.0f, al), bl)));
    const float bound =
        __fadd_rn(__fmul_rn(0x1p-40f, fabsf(s.E) + fabsf(rp.y) + fabsf(ph) + fabsf(a.x) + b), 1e-30f);
    if (Q > bound) return 1;
    if (Q < -bound) return -1;
    return 0;
}

// Certified FP64 sign of function_q at table point k, from the stored
// correctly rounded 1/r_k (no division).  With u = 2^-53: J*inv_r differs from
// the reference's (double)(J/r) by at most 3.01u|J/r|, so the squares differ
// by at most 8.2u (J/r)^2; the self-potential from mjN*inv_r by at most
// 3.01u phis; the two subtractions and the final combination add at most
// 2u(|E|+|Phi|+|phis|) + u(2|A| + (J/r)^2).  Twice the sum, 16u of each
// magnitude, is the threshold.  Returns +1, -1, or 0 (undecided).
__device__ __forceinline__ int fq_sign_f64(const QF32 &s, double inv_rk, double phik, bool ge)
{
    const double phis = ge ? __dmul_rn(s.mjNd, inv_rk) : s.pjd;
    const double A = __dsub_rn(__dsub_rn(s.Ed, phik), phis);
    const double q = __dmul_rn(s.Jd, inv_rk);
    const double B = __dmul_rn(q, q);
    const double Q = __dsub_rn(__dmul_rn(2.0, A), B);
    const double bound = 0x1p-49 * (fabs(s.Ed) + fabs(phik) + fabs(phis) + fabs(A) + B);
    if (Q > bound) return 1;
    if (Q < -bound) return -1;
    return 0;
}

}  // namespace cmcg
