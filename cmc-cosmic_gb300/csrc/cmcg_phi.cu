// cmcg_phi.cu -- potential_calculate (cmc_utils.c:675-736) reproduced bit for
// bit from the approximate scan of cmcg_potential.cu.
//
// The reference evaluates three recurrences, each rounding once per step:
//   chain 1 (k = 1..N):  S_k = S_{k-1} + m_k                      S_0 = 0
//                        Mtotal = S_N madhoc + cenma_m madhoc
//   chain 2 (k = N..1):  M_{k-1} = M_k - q_k,  q_k = m_k / N_STAR   M_N = Mtotal
//   chain 3 (k = N..1):  Phi_k = Phi_{k+1} - t_k,
//                        t_k = M_k (1/r_k - 1/r_{k+1})            Phi_{N+1} = 0
// Each is s_j = fl(s_{j-1} + a_j) over known terms a_j.  While s_{j-1} and
// s_j both lie strictly inside one binade [2^E, 2^(E+1)), the sum rounds to
// the grid u = 2^(E-52), on which s_{j-1} already lies, so
//     s_j = s_{j-1} + rho_j u,    rho_j = round(a_j / u), an integer,
// unless a_j / u ends in exactly one half (a tie, decided by s_{j-1}).  So a
// chain is an integer prefix sum except at a few positions.  The carries
// of cmcg_potential.cu give every s_j to within a proven bound (tile_approx); a position whose before and
// after values are both farther than that bound from the edges of the same
// binade, and whose term is no tie, is "regular".  Every other position -- a
// binade change, a value within the bound of an edge, a tie, the first and
// the last position -- is a "sequential point": one thread replays those in
// order with the reference's FP64 addition, bridging each run of regular
// positions by one exact integer addition on the run's grid.  Every value is
// then  s_j = s_(last sequential point) + (rho summed over the run) u,
// assembled from bit fields without rounding.
//
// Passes over the potential's tiles (POT_T stars, chain order within a tile
// ascending k for chain 1 and descending k for chains 2 and 3):
//   k_phi_cls12  chains 1, 2: classify; per-tile run totals; the last block
//                of a cluster scans them over tiles
//   k_phi_rec12  chains 1, 2: record the sequential points; the last block
//                replays chain 1 (-> Mtotal, Rtidal), then chain 2
//   k_phi_cls3   chain 2 values -> t_k; chain 3: classify; last block scans
//   k_phi_rec3   chain 3: record; last block replays
//   k_phi_final  chain 3 values -> star_phi, the FP32 table, sentinels
// Each chain is classified once: the classifying pass keeps every position's
// rho, binade keys and sequential-point flag, and every thread's tile scans
// (store_cls), for the passes after it (load_cls).
//   k_phi_seq    the plain one-thread loop, run only for a cluster whose
//                replay was refused (radii out of order, non-finite input,
//                too many sequential points, a failed check) or that asked
//                for it (cmcg_params.phi_sequential)
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {

namespace {

constexpr unsigned long long MANT = (1ull << 52) - 1, HIDDEN = 1ull << 52;
constexpr int NW = POT_THREADS / 32;

struct AState {
    int key;    // sign and exponent bits (top 12 bits) of the approximate value
    bool safe;  // the sequential value provably lies strictly inside that binade
};

// ceil(margin / 2^(ex-1075)) -- the margin in grid units of binade ex --
// saturated at 2^64-1 when it reaches the binade's width.
__device__ __forceinline__ unsigned long long margin_units(double margin, unsigned ex)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(margin);
    unsigned em = (unsigned)(b >> 52) & 0x7ffu;
    unsigned long long mm = b & MANT;
    if (b >> 63) return ~0ull;  // a negative margin is a bug: refuse
    if (em == 0 && mm == 0) return 0;
    if (em == 0x7ffu) return ~0ull;
    if (em) mm |= HIDDEN;
    else em = 1;
    const int d = (int)em - (int)ex;
    if (d > 0) return ~0ull;
    if (d == 0) return mm;
    const int s = -d;
    if (s >= 64) return 1ull;
    return (mm + ((1ull << s) - 1)) >> s;
}

__device__ __forceinline__ AState astate(double x, double margin)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
    AState s;
    s.key = (int)(b >> 52);
    if (ex == 0 || ex >= 0x7feu) {  // zero, subnormal, the top binade, inf/NaN
        s.safe = false;
        return s;
    }
    const unsigned long long f = b & MANT, g = margin_units(margin, ex);
    s.safe = (f > g) && ((HIDDEN - f) > g);
    return s;
}

// rho = a / 2^(ex-1075) rounded to nearest.  False on a tie, on |a| >= 2^(ex-1023)
// (no sum of this size stays in the binade) and on a non-finite a.
__device__ __forceinline__ bool term_units(double a, unsigned ex, long long *rho)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    unsigned ea = (unsigned)(b >> 52) & 0x7ffu;
    unsigned long long ma = b & MANT;
    if (ea == 0x7ffu) return false;
    if (ea == 0 && ma == 0) {
        *rho = 0;
        return true;
    }
    if (ea) ma |= HIDDEN;
    else ea = 1;
    if (ea >= ex) return false;
    const unsigned sh = ex - ea;  // >= 1
    unsigned long long q = 0;
    if (sh <= 54) {
        q = ma >> sh;
        const unsigned long long rem = ma & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem == half) return false;
        q += rem > half ? 1ull : 0ull;
    }
    *rho = (b >> 63) ? -(long long)q : (long long)q;
    return true;
}

// Exact base + P * 2^(ex-1075) for base and result strictly inside binade
// `key` (sign and exponent bits); false if either is not.
__device__ __forceinline__ bool compose(double base, long long P, int key, double *out)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(base);
    if ((int)(b >> 52) != key) return false;
    const unsigned ex = (unsigned)key & 0x7ffu;
    if (ex == 0 || ex == 0x7ffu) return false;
    if (P > (1ll << 54) || P < -(1ll << 54)) return false;
    long long I = (long long)((b & MANT) | HIDDEN);
    const bool neg = (key & 0x800) != 0;
    if (neg) I = -I;
    I += P;
    if ((I < 0) != neg) return false;
    const unsigned long long A = (unsigned long long)(I < 0 ? -I : I);
    if (A <= HIDDEN || A >= (HIDDEN << 1)) return false;
    *out = __longlong_as_double((long long)(((unsigned long long)(unsigned)key << 52) | (A - HIDDEN)));
    return true;
}

// ---- segmented scan of (grid units, run length) with resets at sequential points
struct Seg {
    long long P;
    int c;
    int r;
};
__device__ __forceinline__ Seg seg_op(Seg x, Seg y) { return y.r ? y : Seg{x.P + y.P, x.c + y.c, x.r}; }

// Exclusive block scan (thread order); *total = the whole block's aggregate.
__device__ __forceinline__ Seg block_seg_excl(Seg v, Seg *s_w, Seg *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    Seg x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        Seg y;
        y.P = __shfl_up_sync(0xffffffffu, x.P, o);
        y.c = __shfl_up_sync(0xffffffffu, x.c, o);
        y.r = __shfl_up_sync(0xffffffffu, x.r, o);
        if (lane >= o) x = seg_op(y, x);
    }
    Seg ex;
    ex.P = __shfl_up_sync(0xffffffffu, x.P, 1);
    ex.c = __shfl_up_sync(0xffffffffu, x.c, 1);
    ex.r = __shfl_up_sync(0xffffffffu, x.r, 1);
    if (lane == 0) ex = Seg{0, 0, 0};
    __syncthreads();
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    Seg pre{0, 0, 0}, tot{0, 0, 0};
    for (int q = 0; q < NW; ++q) {
        if (q == w) pre = tot;
        tot = seg_op(tot, s_w[q]);
    }
    *total = tot;
    return seg_op(pre, ex);
}

__device__ __forceinline__ int block_int_excl(int v, int *s_w, int *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    int pre = 0, tot = 0;
    for (int q = 0; q < NW; ++q) {
        if (q == w) pre = tot;
        tot += s_w[q];
    }
    *total = tot;
    return pre + x - v;
}

// ---- the three chains seen from one tile
struct View {
    const double *m, *q, *t, *inv_r, *papx;  // cluster-relative, index k
    long long N;
    double marg1, marg2, c0, c1;
    // chains 1 and 2 (k_phi_cls12 only): the tile's approximate S_k and M_k by
    // position p = kst - k (tile_approx), and those of the tile below's first
    // position (p = POT_T)
    const double *sS, *sM;
    long long kst;
    double Sb, Mb;
};

__device__ __forceinline__ View make_view(const Cluster &C, const Fields &f, const PotBufs &pb, const PhiCtl &ctl)
{
    View v;
    const long long off = C.off;
    v.m = f.m + off;
    v.q = pb.q + off;
    v.t = pb.t + off;
    v.inv_r = f.inv_r + off;
    v.papx = pb.papx + off;
    v.sS = v.sM = nullptr;
    v.kst = 0;
    v.Sb = v.Mb = 0.0;
    v.N = C.sc->N_MAX;
    v.marg1 = ctl.marg1;
    v.marg2 = ctl.marg2;
    v.c0 = ctl.c0;
    v.c1 = ctl.c1;
    return v;
}

// star index of chain position p (0..POT_T-1) within the tile whose largest k is kstart
template <int CH>
__device__ __forceinline__ long long kpos(long long kstart, int p)
{
    return CH == 1 ? kstart - (POT_T - 1) + p : kstart - p;
}

// approximate value after the chain's step at star k, with its error bound
template <int CH>
__device__ __forceinline__ AState after_state(const View &v, long long k)
{
    if (CH == 1) {
        const long long p = v.kst - k;
        return astate(p < POT_T ? v.sS[p] : v.Sb, v.marg1);
    }
    if (CH == 2) {
        if (k <= 1) return AState{0, false};  // M_0 is never used
        const long long p = v.kst - (k - 1);
        return astate(p < POT_T ? v.sM[p] : v.Mb, v.marg2);
    }
    return astate(v.papx[k], __dadd_ru(v.c0, __dmul_ru(v.c1, v.inv_r[k])));
}

template <int CH>
__device__ __forceinline__ double term_at(const View &v, long long k)
{
    if (CH == 1) return v.m[k];
    if (CH == 2) return -v.q[k];
    return -v.t[k];
}

struct Items {
    long long k[POT_ITEMS];
    double a[POT_ITEMS];
    long long rho[POT_ITEMS];
    int key[POT_ITEMS], keyprev[POT_ITEMS];
    bool valid[POT_ITEMS], sp[POT_ITEMS];
};

struct TileSmem {
    int key[NW];
    int safe[NW];
    Seg seg[NW];
    int cnt[NW];
    int prev_key, prev_safe;
};

// Classify the tile's positions; it.a must hold the terms of valid positions.
template <int CH>
__device__ __forceinline__ void classify(const View &v, long long kstart, Items &it, TileSmem &sm)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    AState st[POT_ITEMS];
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = it.k[i];
        st[i] = it.valid[i] ? after_state<CH>(v, k) : AState{0, false};
    }
    // state after the position preceding item 0
    int pk = __shfl_up_sync(0xffffffffu, st[POT_ITEMS - 1].key, 1);
    int ps = __shfl_up_sync(0xffffffffu, (int)st[POT_ITEMS - 1].safe, 1);
    if (lane == 31) {
        sm.key[w] = st[POT_ITEMS - 1].key;
        sm.safe[w] = st[POT_ITEMS - 1].safe;
    }
    if (t == 0) {
        const long long kp = CH == 1 ? it.k[0] - 1 : it.k[0] + 1;
        AState s0{0, false};
        if (kp >= 1 && kp <= v.N) s0 = after_state<CH>(v, kp);
        sm.prev_key = s0.key;
        sm.prev_safe = s0.safe;
    }
    __syncthreads();
    if (lane == 0) {
        pk = w > 0 ? sm.key[w - 1] : sm.prev_key;
        ps = w > 0 ? sm.safe[w - 1] : sm.prev_safe;
    }
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const int kp = i == 0 ? pk : st[i - 1].key;
        const bool sp_ = i == 0 ? ps != 0 : st[i - 1].safe;
        const long long k = it.k[i];
        bool reg = it.valid[i] && k != 1 && k != v.N && sp_ && st[i].safe && kp == st[i].key;
        long long rho = 0;
        if (reg) reg = term_units(it.a[i], (unsigned)st[i].key & 0x7ffu, &rho);
        it.rho[i] = rho;
        it.key[i] = st[i].key;
        it.keyprev[i] = kp;
        it.sp[i] = it.valid[i] && !reg;
    }
    __syncthreads();  // sm.key/safe are reused by the caller's next classify
}

template <int CH>
__device__ __forceinline__ void load_positions(const View &v, long long kstart, Items &it)
{
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kpos<CH>(kstart, POT_ITEMS * threadIdx.x + i);
        it.k[i] = k;
        it.valid[i] = k >= 1 && k <= kstart;
    }
}

// Thread aggregate and block exclusive scans of the classified tile.
struct TileScan {
    Seg ex;      // run entering this thread's first item (tile-local)
    int spx;     // sequential points before this thread's first item (tile-local)
    Seg tot;     // the tile's aggregate
    int ntot;    // sequential points in the tile
};

__device__ __forceinline__ TileScan scan_tile(const Items &it, TileSmem &sm)
{
    Seg tv{0, 0, 0};
    int tsp = 0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        if (!it.valid[i]) continue;
        tv = seg_op(tv, it.sp[i] ? Seg{0, 0, 1} : Seg{it.rho[i], 1, 0});
        tsp += it.sp[i] ? 1 : 0;
    }
    TileScan s;
    s.ex = block_seg_excl(tv, sm.seg, &s.tot);
    s.spx = block_int_excl(tsp, sm.cnt, &s.ntot);
    return s;
}

// Keep the tile's classification of chain CH (slot 1 for chain 2, else 0)
// for the passes after this one.
template <int CH>
__device__ __forceinline__ void store_cls(const Items &it, const TileScan &s, const PhiBufs &ph, long long off)
{
    constexpr int slot = CH == 2 ? 1 : 0;
    long long *rho = ph.crho[slot] + off;
    unsigned int *meta = ph.cmeta[slot] + off;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        if (!it.valid[i]) continue;
        const long long k = it.k[i];
        rho[k] = it.rho[i];
        meta[k] = ((unsigned)it.key[i] & 0xfffu) | (((unsigned)it.keyprev[i] & 0xfffu) << 12) |
                  ((it.sp[i] ? 1u : 0u) << 24);
    }
    ph.cscan[slot][(size_t)blockIdx.x * POT_THREADS + threadIdx.x] = PhiScan{s.ex.P, s.ex.c, s.ex.r, s.spx, 0};
}

// The classification store_cls kept, in place of classify + scan_tile (the
// tile totals are not restored: only the classifying pass uses them).
// it.k, it.valid and it.a must be loaded.
template <int CH>
__device__ __forceinline__ TileScan load_cls(Items &it, const PhiBufs &ph, long long off)
{
    constexpr int slot = CH == 2 ? 1 : 0;
    const long long *rho = ph.crho[slot] + off;
    const unsigned int *meta = ph.cmeta[slot] + off;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        if (it.valid[i]) {
            const long long k = it.k[i];
            const unsigned mt = meta[k];
            it.rho[i] = rho[k];
            it.key[i] = (int)(mt & 0xfffu);
            it.keyprev[i] = (int)((mt >> 12) & 0xfffu);
            it.sp[i] = ((mt >> 24) & 1u) != 0;
        } else {
            it.rho[i] = 0;
            it.key[i] = it.keyprev[i] = 0;
            it.sp[i] = false;
        }
    }
    const PhiScan c = ph.cscan[slot][(size_t)blockIdx.x * POT_THREADS + threadIdx.x];
    TileScan s;
    s.ex = Seg{c.P, c.c, c.r};
    s.spx = c.spx;
    s.tot = Seg{0, 0, 0};
    s.ntot = 0;
    return s;
}

// Exact values before and after each valid item, from the replayed records.
// Returns false if a check fails (the cluster then falls back).
__device__ __forceinline__ bool tile_values(const Items &it, const TileScan &s, const ChainCarry &cy,
                                            const SPRec *R, long long nrec, double (&before)[POT_ITEMS],
                                            double (&after)[POT_ITEMS])
{
    Seg run = seg_op(Seg{cy.P, cy.cnt, 0}, s.ex);
    long long spi = (long long)cy.spoff + s.spx;
    bool ok = true;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        before[i] = after[i] = 0.0;
        if (!it.valid[i]) continue;
        if (it.sp[i]) {
            if (spi < 0 || spi >= nrec) {
                ok = false;
                continue;
            }
            before[i] = R[spi].sprev;
            after[i] = R[spi].snew;
            ++spi;
            run = Seg{0, 0, 1};
        } else {
            run = seg_op(run, Seg{it.rho[i], 1, 0});
            if (spi < 1 || spi > nrec) {
                ok = false;
                continue;
            }
            const double base = R[spi - 1].snew;
            ok &= compose(base, run.P, it.key[i], &after[i]);
            ok &= compose(base, run.P - it.rho[i], it.key[i], &before[i]);
        }
    }
    return ok;
}

// Record this tile's sequential points.
__device__ __forceinline__ void tile_records(const Items &it, const TileScan &s, const ChainCarry &cy, SPRec *R,
                                             long long nrec)
{
    Seg run = seg_op(Seg{cy.P, cy.cnt, 0}, s.ex);
    long long spi = (long long)cy.spoff + s.spx;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        if (!it.valid[i]) continue;
        if (it.sp[i]) {
            if (spi >= 0 && spi < nrec) {
                SPRec &r = R[spi];
                r.k = it.k[i];
                r.a = it.a[i];
                r.Pprev = run.P;
                r.keyprev = it.keyprev[i];
                r.cntprev = run.c;
            }
            ++spi;
            run = Seg{0, 0, 1};
        } else {
            run = seg_op(run, Seg{it.rho[i], 1, 0});
        }
    }
}

// Last block of a cluster: exclusive scan of the tiles' aggregates in chain
// order (reversed tile order for chain 1).  Returns the number of sequential
// points of the chain (all threads).
template <bool REV>
__device__ long long scan_tiles(const ChainAgg *agg, ChainCarry *carry, int first, int ntiles, TileSmem &sm)
{
    const int t = threadIdx.x;
    const int per = (ntiles + POT_THREADS - 1) / POT_THREADS;
    const int lo = min(ntiles, t * per), hi = min(ntiles, lo + per);
    Seg v{0, 0, 0};
    int n = 0;
    for (int cy = lo; cy < hi; ++cy) {
        const int y = REV ? ntiles - 1 - cy : cy;
        const ChainAgg *a = agg + first + y;
        const int ns = __ldcg(&a->nsp);
        v = seg_op(v, Seg{__ldcg(&a->P), __ldcg(&a->cnt), ns > 0 ? 1 : 0});
        n += ns;
    }
    Seg tot;
    int ntot;
    Seg ex = block_seg_excl(v, sm.seg, &tot);
    int nex = block_int_excl(n, sm.cnt, &ntot);
    for (int cy = lo; cy < hi; ++cy) {
        const int y = REV ? ntiles - 1 - cy : cy;
        const ChainAgg *a = agg + first + y;
        carry[first + y] = ChainCarry{ex.P, ex.c, nex};
        const int ns = __ldcg(&a->nsp);
        ex = seg_op(ex, Seg{__ldcg(&a->P), __ldcg(&a->cnt), ns > 0 ? 1 : 0});
        nex += ns;
    }
    return ntot;
}

// Last block of a cluster: replay the sequential points of one chain in
// order, starting from the exact value s0.  Returns the value after the last
// point (all threads); sets *bad on a failed check.
struct WalkSmem {
    double a[PHI_WALK_BATCH], sprev[PHI_WALK_BATCH], snew[PHI_WALK_BATCH];
    long long P[PHI_WALK_BATCH];
    int key[PHI_WALK_BATCH], cnt[PHI_WALK_BATCH];
    double cur;
    int bad;
};

__device__ double replay(SPRec *R, long long n, double s0, WalkSmem &ws, int *bad)
{
    const int t = threadIdx.x;
    __syncthreads();
    if (t == 0) {
        ws.cur = s0;
        ws.bad = 0;
    }
    for (long long b0 = 0; b0 < n; b0 += PHI_WALK_BATCH) {
        const int m = (int)min((long long)PHI_WALK_BATCH, n - b0);
        __syncthreads();
        for (int i = t; i < m; i += POT_THREADS) {
            const SPRec *r = R + b0 + i;
            ws.a[i] = __ldcg(&r->a);
            ws.P[i] = __ldcg(&r->Pprev);
            ws.key[i] = __ldcg(&r->keyprev);
            ws.cnt[i] = __ldcg(&r->cntprev);
        }
        __syncthreads();
        if (t == 0) {
            double cur = ws.cur;
            int b = ws.bad;
            for (int i = 0; i < m; ++i) {
                double sp = cur;
                if (ws.cnt[i] > 0 && !compose(cur, ws.P[i], ws.key[i], &sp)) {
                    b = 1;
                    sp = cur;
                }
                cur = __dadd_rn(sp, ws.a[i]);
                ws.sprev[i] = sp;
                ws.snew[i] = cur;
            }
            ws.cur = cur;
            ws.bad = b;
        }
        __syncthreads();
        for (int i = t; i < m; i += POT_THREADS) {
            R[b0 + i].sprev = ws.sprev[i];
            R[b0 + i].snew = ws.snew[i];
        }
    }
    __syncthreads();
    if (t == 0 && ws.bad) *bad = 1;
    const double out = ws.cur;
    __syncthreads();
    return out;
}

__device__ __forceinline__ int ctl_failed(const PhiCtl &ctl) { return *(volatile const int *)&ctl.fail; }

}  // namespace

// The approximate running values of chains 1 and 2 over one tile, and Phi_k
// (chain 3's) into pb.papx, from the carries entering the tile (k_pot_carry):
//   S_k, the forward mass sum through star k, and M_k, the enclosed mass the
//   backward loop multiplies at star k, into sS and sM by position p = kstart - k;
//   Phi_k for k_phi_cls3 and the Phi bound of k_phi_rec12.
// Thread t holds k = kstart - 4t - i; every value is the carry plus a block
// scan of the tile's terms (pot_block_excl_prefix), so the first position of
// a tile -- whose value the tile above also needs, as its boundary -- is the
// carry alone: S = Sm - SmIn, M = Mtot - Qin (tile_first_values).
__device__ __forceinline__ void tile_approx(const Cluster &C, const Fields &f, const PotBufs &pb, const PhiCtl &ctl,
                                            long long N, long long kstart, const double *cr, double *sS, double *sM,
                                            double *s_w, double *s_lastinv)
{
    const long long off = C.off;
    const double *r = f.r + off, *inv_r = f.inv_r + off, *m = f.m + off;
    const double Mtot = ctl.Mapx, Sm = ctl.Sm;
    const double Qin = cr[0], Din = cr[1], SmIn = cr[2];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double q[POT_ITEMS], inv[POT_ITEMS], mm[POT_ITEMS];
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kstart - POT_ITEMS * t - i;
        q[i] = (k >= 1) ? pb.q[off + k] : 0.0;
        inv[i] = (k >= 1) ? inv_r[k] : 0.0;
        mm[i] = (k >= 1) ? m[k] : 0.0;
    }
    double up = __shfl_up_sync(0xffffffffu, inv[POT_ITEMS - 1], 1);
    if (lane == 31) s_lastinv[w] = inv[POT_ITEMS - 1];
    __syncthreads();
    if (lane == 0) up = (w > 0) ? s_lastinv[w - 1] : pot_r_next_inv(r, kstart, N);
    double tq = 0.0, tmm = 0.0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        tq += q[i];
        tmm += mm[i];
    }
    const double qex = pot_block_excl_prefix<POT_THREADS>(tq, s_w);
    const double mex = pot_block_excl_prefix<POT_THREADS>(tmm, s_w);
    double dk[POT_ITEMS], run = qex, runm = mex, td = 0.0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kstart - POT_ITEMS * t - i;
        const double innext = (i == 0) ? up : inv[i - 1];
        const double Mk = (Mtot - Qin) - run;  // mprev when the reference reaches k
        dk[i] = (k >= 1) ? Mk * (inv[i] - innext) : 0.0;
        sM[POT_ITEMS * t + i] = Mk;
        sS[POT_ITEMS * t + i] = Sm - (SmIn + runm);
        run += q[i];
        runm += mm[i];
        td += dk[i];
    }
    const double dex = pot_block_excl_prefix<POT_THREADS>(td, s_w);
    double acc = Din + dex;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kstart - POT_ITEMS * t - i;
        acc += dk[i];
        if (k >= 1) pb.papx[off + k] = -acc;
    }
    __syncthreads();  // sS, sM complete
}

// S and M at a tile's first position (k = its kstart): the carries alone, as
// tile_approx forms them there (its exclusive prefixes are +0 at thread 0).
__device__ __forceinline__ void tile_first_values(const PhiCtl &ctl, const double *cr, double *S, double *M)
{
    *M = (ctl.Mapx - cr[0]) - 0.0;
    *S = ctl.Sm - (cr[2] + 0.0);
}

// ------------------------------------------------------------ kernels ----

__global__ void __launch_bounds__(POT_THREADS, 4) k_phi_cls12(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            PotBufs pb, PhiBufs ph, unsigned int *tickets)
{
    __shared__ TileSmem sm;
    __shared__ int s_last;
    __shared__ double s_S[POT_T], s_M[POT_T];
    __shared__ double s_w[POT_THREADS / 32], s_lastinv[POT_THREADS / 32];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    PhiCtl &ctl = ph.ctl[ct.x];
    const long long N = C.sc->N_MAX;
    const long long kstart = N - (long long)ct.y * POT_T;
    if (!ctl_failed(ctl) && kstart >= 1) {
        tile_approx(C, f, pb, ctl, N, kstart, pb.carry + (size_t)blockIdx.x * POT_CARRY, s_S, s_M, s_w, s_lastinv);
        View v = make_view(C, f, pb, ctl);
        v.sS = s_S;
        v.sM = s_M;
        v.kst = kstart;
        if (kstart - POT_T >= 1)  // the tile below (the next one of the cluster) starts at kstart - POT_T
            tile_first_values(ctl, pb.carry + (size_t)(blockIdx.x + 1) * POT_CARRY, &v.Sb, &v.Mb);
        Items it;
        load_positions<1>(v, kstart, it);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) it.a[i] = it.valid[i] ? term_at<1>(v, it.k[i]) : 0.0;
        classify<1>(v, kstart, it, sm);
        TileScan s = scan_tile(it, sm);
        if (threadIdx.x == 0) ph.agg[0][blockIdx.x] = ChainAgg{s.tot.P, s.tot.c, s.ntot};
        store_cls<1>(it, s, ph, C.off);
        load_positions<2>(v, kstart, it);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) it.a[i] = it.valid[i] ? term_at<2>(v, it.k[i]) : 0.0;
        classify<2>(v, kstart, it, sm);
        s = scan_tile(it, sm);
        if (threadIdx.x == 0) ph.agg[1][blockIdx.x] = ChainAgg{s.tot.P, s.tot.c, s.ntot};
        store_cls<2>(it, s, ph, C.off);
    } else if (threadIdx.x == 0) {
        ph.agg[0][blockIdx.x] = ChainAgg{0, 0, 0};
        ph.agg[1][blockIdx.x] = ChainAgg{0, 0, 0};
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        if (ctl_failed(ctl)) return;
        const int first = tm.first[ct.x], nt = tm.count[ct.x];
        const long long n1 = scan_tiles<true>(ph.agg[0], ph.carry[0], first, nt, sm);
        const long long n2 = scan_tiles<false>(ph.agg[1], ph.carry[1], first, nt, sm);
        if (threadIdx.x == 0) {
            ctl.nsp[0] = n1;
            ctl.nsp[1] = n2;
            if (n1 > C.rec_cap || n2 > C.rec_cap) ctl.fail = 1;
        }
    }
}

__global__ void __launch_bounds__(POT_THREADS) k_phi_rec12(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            PotBufs pb, PhiBufs ph, unsigned int *tickets)
{
    __shared__ WalkSmem ws;
    __shared__ int s_last;
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    PhiCtl &ctl = ph.ctl[ct.x];
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX;
    const long long kstart = N - (long long)ct.y * POT_T;
    SPRec *R1 = ph.rec[0] + C.rec_off, *R2 = ph.rec[1] + C.rec_off;
    if (!ctl_failed(ctl) && kstart >= 1) {
        const View v = make_view(C, f, pb, ctl);
        Items it;
        load_positions<1>(v, kstart, it);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) it.a[i] = it.valid[i] ? term_at<1>(v, it.k[i]) : 0.0;
        TileScan s = load_cls<1>(it, ph, C.off);
        tile_records(it, s, ph.carry[0][blockIdx.x], R1, ctl.nsp[0]);
        load_positions<2>(v, kstart, it);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) it.a[i] = it.valid[i] ? term_at<2>(v, it.k[i]) : 0.0;
        s = load_cls<2>(it, ph, C.off);
        tile_records(it, s, ph.carry[1][blockIdx.x], R2, ctl.nsp[1]);
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        if (ctl_failed(ctl)) return;
        int bad = 0;
        // chain 1 -> Mtotal and Rtidal (cmc_utils.c:693-697)
        const double S = replay(R1, ctl.nsp[0], 0.0, ws, &bad);
        const double madhoc = sc->madhoc;
        const double Mtotal = __dadd_rn(__dmul_rn(S, madhoc), __dmul_rn(sc->cenma_m, madhoc));
        replay(R2, ctl.nsp[1], Mtotal, ws, &bad);
        if (threadIdx.x == 0) {
            if (bad || isnan(S)) ctl.fail = 1;
            sc->Mtotal = Mtotal;
            sc->Rtidal = __dmul_rn(sc->orbit_r, pow(Mtotal, 1.0 / 3.0));
            // chain 3 bound (the radii are in order, so sum_{j>=k} d_j <= 1/r_k (1 + u)):
            //   |Phi~_k - Phi_k| <= c1 / r_k + c0, with c1 covering the enclosed-mass
            //   error marg2 and the scan's error 4 G (Mb + sum q), c0 the drift
            //   (n+3) u Phib of the sequential sum, Phib >= every |Phi_k|.
            const View v = make_view(C, f, pb, ctl);
            const double G = ctl.G, u = 0x1p-53;
            const double c1 = 1.01 * (ctl.marg2 + 4.0 * G * (ctl.Mb + ctl.Qtot * (1.0 + 2.0 * G))) * (1.0 + 0x1p-50);
            const double Phib = (fabs(v.papx[1]) + c1 * v.inv_r[1]) * (1.0 + 0x1p-20);
            ctl.c1 = c1;
            ctl.c0 = 1.01 * ((double)N + 3.0) * u * Phib;
        }
    }
}

__global__ void __launch_bounds__(POT_THREADS) k_phi_cls3(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                           PotBufs pb, PhiBufs ph, unsigned int *tickets)
{
    __shared__ TileSmem sm;
    __shared__ int s_last;
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    PhiCtl &ctl = ph.ctl[ct.x];
    const long long N = C.sc->N_MAX, off = C.off;
    const long long kstart = N - (long long)ct.y * POT_T;
    if (!ctl_failed(ctl) && kstart >= 1) {
        const View v = make_view(C, f, pb, ctl);
        Items it;
        // chain 2 values: M_k is the value before star k (records and rho give them, no terms)
        load_positions<2>(v, kstart, it);
        TileScan s = load_cls<2>(it, ph, off);
        double Mbef[POT_ITEMS], Maft[POT_ITEMS];
        const bool ok = tile_values(it, s, ph.carry[1][blockIdx.x], ph.rec[1] + C.rec_off, ctl.nsp[1], Mbef, Maft);
        if (!ok) ctl.fail = 1;
        // t_k = M_k (1/r_k - 1/r_{k+1}) as the reference rounds it (cmc_utils.c:716)
        const double inv_inf = __drcp_rn(CMCG_SF_INFINITY);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) {
            const long long k = it.k[i];
            double tk = 0.0;
            if (it.valid[i]) {
                const double innext = (k == N) ? inv_inf : v.inv_r[k + 1];
                tk = __dmul_rn(Mbef[i], __dsub_rn(v.inv_r[k], innext));
                pb.t[off + k] = tk;
            }
            it.a[i] = -tk;
        }
        // chain 3: same positions, new terms
        classify<3>(v, kstart, it, sm);
        s = scan_tile(it, sm);
        if (threadIdx.x == 0) ph.agg[0][blockIdx.x] = ChainAgg{s.tot.P, s.tot.c, s.ntot};
        store_cls<3>(it, s, ph, off);
    } else if (threadIdx.x == 0) {
        ph.agg[0][blockIdx.x] = ChainAgg{0, 0, 0};
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        if (ctl_failed(ctl)) return;
        const long long n3 = scan_tiles<false>(ph.agg[0], ph.carry[0], tm.first[ct.x], tm.count[ct.x], sm);
        if (threadIdx.x == 0) {
            ctl.nsp[2] = n3;
            if (n3 > C.rec_cap) ctl.fail = 1;
        }
    }
}

__global__ void __launch_bounds__(POT_THREADS) k_phi_rec3(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                           PotBufs pb, PhiBufs ph, unsigned int *tickets)
{
    __shared__ WalkSmem ws;
    __shared__ int s_last;
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    PhiCtl &ctl = ph.ctl[ct.x];
    const long long N = C.sc->N_MAX;
    const long long kstart = N - (long long)ct.y * POT_T;
    SPRec *R3 = ph.rec[0] + C.rec_off;
    if (!ctl_failed(ctl) && kstart >= 1) {
        const View v = make_view(C, f, pb, ctl);
        Items it;
        load_positions<3>(v, kstart, it);
#pragma unroll
        for (int i = 0; i < POT_ITEMS; ++i) it.a[i] = it.valid[i] ? term_at<3>(v, it.k[i]) : 0.0;
        TileScan s = load_cls<3>(it, ph, C.off);
        tile_records(it, s, ph.carry[0][blockIdx.x], R3, ctl.nsp[2]);
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        if (ctl_failed(ctl)) return;
        int bad = 0;
        replay(R3, ctl.nsp[2], 0.0, ws, &bad);
        if (threadIdx.x == 0 && bad) ctl.fail = 1;
    }
}

__global__ void __launch_bounds__(POT_THREADS) k_phi_final(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            PotBufs pb, PhiBufs ph)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    PhiCtl &ctl = ph.ctl[ct.x];
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, off = C.off;
    const long long kstart = N - (long long)ct.y * POT_T;
    if (ctl_failed(ctl) || kstart < 1) return;
    const View v = make_view(C, f, pb, ctl);
    Items it;
    load_positions<3>(v, kstart, it);  // the values need no terms: records and rho give them
    TileScan s = load_cls<3>(it, ph, off);
    double Pb[POT_ITEMS], Pa[POT_ITEMS];
    const bool ok = tile_values(it, s, ph.carry[0][blockIdx.x], ph.rec[0] + C.rec_off, ctl.nsp[2], Pb, Pa);
    if (!ok) {
        ctl.fail = 1;
        return;
    }
    double *r = f.r + off, *phi = f.phi + off;
    float4 *rphif = f.rphif + off;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        if (!it.valid[i]) continue;
        const long long k = it.k[i];
        const double ph_k = Pa[i];
        phi[k] = ph_k;
        rphif[k] = rphi_entry(r[k], ph_k);
        if (k == 1) {
            // cmc_utils.c:727
            const double p0 = __dadd_rn(ph_k, __ddiv_rn(__dmul_rn(sc->cenma_m, sc->madhoc), r[1]));
            phi[0] = p0;
            rphif[0] = rphi_entry(r[0], p0);
        }
    }
    if (ct.y == 0 && threadIdx.x == 0) {
        r[N + 1] = CMCG_SF_INFINITY;
        phi[N + 1] = 0.0;
        f.inv_r[off + N + 1] = __drcp_rn(CMCG_SF_INFINITY);
        f.inv_r[off] = __drcp_rn(r[0]);
        rphif[N + 1] = rphi_entry(CMCG_SF_INFINITY, 0.0);
        sc->phi_nsp[0] = ctl.nsp[0];
        sc->phi_nsp[1] = ctl.nsp[1];
        sc->phi_nsp[2] = ctl.nsp[2];
        sc->phi_fallback = 0;
    }
}

// The reference's loop on one thread (cmc_utils.c:683-731), for a cluster
// whose replay was refused.  Radii at or beyond SF_INFINITY end the star list
// as they do there.
__global__ void k_phi_seq(const Cluster *__restrict__ cls, Fields f, PhiBufs ph, int nclusters)
{
    const int c = blockIdx.x;
    if (c >= nclusters || threadIdx.x != 0) return;
    const Cluster &C = cls[c];
    if (!counts_ok(C)) return;
    if (!ctl_failed(ph.ctl[c])) return;
    Scalars *sc = C.sc;
    const long long off = C.off;
    double *r = f.r + off, *m = f.m + off, *phi = f.phi + off, *inv_r = f.inv_r + off;
    float4 *rphif = f.rphif + off;
    long long k = 1;
    double mprev = 0.0;
    const long long NM = sc->N_MAX;
    while (k <= NM && r[k] < CMCG_SF_INFINITY) {
        mprev = __dadd_rn(mprev, m[k]);
        if (isnan(mprev)) {
            set_error(sc, CMCG_ERR_NAN_MASS, k);
            return;
        }
        ++k;
    }
    const long long N = k - 1;
    sc->N_MAX = N;
    const double madhoc = sc->madhoc;
    sc->Mtotal = __dadd_rn(__dmul_rn(mprev, madhoc), __dmul_rn(sc->cenma_m, madhoc));
    sc->Rtidal = __dmul_rn(sc->orbit_r, pow(sc->Mtotal, 1.0 / 3.0));
    r[N + 1] = CMCG_SF_INFINITY;
    phi[N + 1] = 0.0;
    inv_r[N + 1] = __drcp_rn(CMCG_SF_INFINITY);
    rphif[N + 1] = rphi_entry(CMCG_SF_INFINITY, 0.0);
    const double NSTAR = (double)sc->N_STAR;
    mprev = sc->Mtotal;
    for (k = N; k >= 1; --k) {
        inv_r[k] = __drcp_rn(r[k]);
        const double d = __dsub_rn(inv_r[k], inv_r[k + 1]);
        phi[k] = __dsub_rn(phi[k + 1], __dmul_rn(mprev, d));
        mprev = __dsub_rn(mprev, __ddiv_rn(m[k], NSTAR));
        rphif[k] = rphi_entry(r[k], phi[k]);
        if (isnan(phi[k])) {
            set_error(sc, CMCG_ERR_NAN_PHI, k);
            return;
        }
    }
    phi[0] = __dadd_rn(phi[1], __ddiv_rn(__dmul_rn(sc->cenma_m, madhoc), r[1]));
    inv_r[0] = __drcp_rn(r[0]);
    rphif[0] = rphi_entry(r[0], phi[0]);
    if (isnan(phi[0])) set_error(sc, CMCG_ERR_NAN_PHI, 0);
    sc->phi_nsp[0] = sc->phi_nsp[1] = sc->phi_nsp[2] = 0;
    sc->phi_fallback = 1;
}

// Radius index of the new star order (RIdx, cmcg_internal.cuh): one thread
// per bucket finds its first star by a lower-bound search on the radii's bit
// patterns.  Not built (queries then search the whole table) when the radii
// are out of order or not finite.
__global__ void __launch_bounds__(RIDX_THREADS) k_ridx_build(const Cluster *__restrict__ cls, Fields f, PhiBufs ph,
                                                             int nclusters)
{
    const int c = blockIdx.y;
    if (c >= nclusters) return;
    const Cluster &C = cls[c];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX;
    const int B = C.ridx_B;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (*(volatile int *)&ph.ctl[c].disorder || N < 2 || B < 2) {
        if (b == 0) sc->ridx_ok = 0;
        return;
    }
    const double *r = f.r + C.off;
    const long long base = __double_as_longlong(r[1]), dmax = __double_as_longlong(r[N]) - base;
    int s = 0;
    while (s < 62 && (dmax >> s) > (long long)(B - 2)) ++s;
    if (b == 0) {
        sc->ridx_base = base;
        sc->ridx_shift = s;
        sc->ridx_ok = 1;
    }
    if (b > B) return;
    int *T = f.ridx + C.ridx_off;
    if (b == B) {
        T[B] = (int)(N + 2);
        return;
    }
    const long long key = base + ((long long)b << s);
    long long lo = 1, hi = N + 1;  // r[N+1] = SF_INFINITY is above every key of bucket B-1's range
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (__double_as_longlong(r[mid]) < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    T[b] = (int)lo;
}

}  // namespace cmcg
