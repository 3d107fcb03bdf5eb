// cmcg_sort.cu -- stable LSD radix sort of the stars by radius, per cluster.
//
// Restates qsorts_new (cmc_utils.c:2232-2254) with the one-rank sample_sort
// (cmc_sort.c:375-420: local qsort by r, remove_stripped_stars 343-354) and
// post_sort_comm (cmc_utils.c:2259-2288), preceded by the transfer half of
// ComputeIntermediateEnergy (cmc_utils.c:381-390: r = rnew, vr = vrnew,
// vt = vtnew, rOld = old r).
//
// Keys are the IEEE bit patterns of rnew (positive doubles order like their
// bits), values the star's slot.  Each pass handles one 8-bit digit:
//   k_sort_hist    per-tile digit counts, stored digit-major per cluster
//   k_sort_scan    per (cluster, digit) exclusive scan over tiles
//   k_sort_scatter stable in-tile ranking (warp match + per-warp counters),
//                  staged through shared memory so runs of one digit leave
//                  the block as contiguous stores
// Tiles never straddle clusters, so one launch sorts every cluster of an
// ensemble independently.  Passes whose digit is identical for every key of a
// cluster (found from the key range) are skipped for that cluster.
// k_sort_gather then moves the payload (rnew, m, vrnew, vtnew, id, r, ec_pre)
// into radial order with 128-bit-aligned SoA loads and drops the escapers
// (r == SF_INFINITY), which sort last.
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {


// Key range and bound count (r < SF_INFINITY) per cluster.
__global__ void __launch_bounds__(SORT_THREADS) k_sort_prep(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            SortBufs sb, double *partials, unsigned int *tickets)
{
    __shared__ unsigned long long s_min[SORT_THREADS / 32], s_max[SORT_THREADS / 32];
    __shared__ long long s_cnt[SORT_THREADS / 32];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX_NEW;
    const unsigned long long inf_bits = (unsigned long long)__double_as_longlong(CMCG_SF_INFINITY);
    unsigned long long kmn = ~0ull, kmx = 0ull;
    long long cnt = 0;
    const long long base = 1 + (long long)ct.y * SORT_T;
    for (int i = threadIdx.x; i < SORT_T; i += SORT_THREADS) {
        const long long k = base + i;
        if (k > N) break;
        const unsigned long long b = (unsigned long long)__double_as_longlong(f.rnew[C.off + k]);
        if (b != inf_bits) {
            cnt++;
            kmn = min(kmn, b);
            kmx = max(kmx, b);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kmn = min(kmn, __shfl_down_sync(0xffffffffu, kmn, o));
        kmx = max(kmx, __shfl_down_sync(0xffffffffu, kmx, o));
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_min[w] = kmn;
        s_max[w] = kmx;
        s_cnt[w] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < SORT_THREADS / 32; ++q) {
            kmn = min(kmn, s_min[q]);
            kmx = max(kmx, s_max[q]);
            cnt += s_cnt[q];
        }
        double *slot = partials + (size_t)blockIdx.x * 3;
        slot[0] = __longlong_as_double((long long)kmn);
        slot[1] = __longlong_as_double((long long)kmx);
        slot[2] = (double)cnt;
        if (arrive_last(tickets + ct.x, tm.count[ct.x])) {
            unsigned long long a = ~0ull, b = 0ull;
            long long n = 0;
            const int b0 = tm.first[ct.x];
            for (int q = 0; q < tm.count[ct.x]; ++q) {
                const double *s = partials + (size_t)(b0 + q) * 3;
                a = min(a, (unsigned long long)__double_as_longlong(s[0]));
                b = max(b, (unsigned long long)__double_as_longlong(s[1]));
                n += (long long)s[2];
            }
            sc->n_bound = n;
            // escapers sort after every bound star: the key range must include them
            const bool esc = (n < N);
            if (esc) b = inf_bits;
            if (n == 0) a = b = inf_bits;
            sb.kmin[ct.x] = 0ull;
            sb.kmax[ct.x] = b;
            // digits where every key agrees need no pass: highest differing bit
            const unsigned long long diff = a ^ b;
            int bits = diff ? 64 - __clzll((long long)diff) : 0;
            sb.npass[ct.x] = (bits + 7) / 8;
        }
    }
}

static __device__ __forceinline__ unsigned long long load_key(const Cluster &C, const Fields &f, const SortBufs &sb,
                                                              int pass, int cur, long long pos /*0-based*/)
{
    if (pass == 0) return (unsigned long long)__double_as_longlong(f.rnew[C.off + 1 + pos]);
    return (cur ? sb.keys[1] : sb.keys[0])[C.off + pos];
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            SortBufs sb, int pass)
{
    __shared__ unsigned int h[SORT_THREADS / 32][RADIX];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    if (pass >= sb.npass[ct.x]) return;
    const long long N = C.sc->N_MAX_NEW;
    const int w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (SORT_THREADS / 32) * RADIX; i += SORT_THREADS) (&h[0][0])[i] = 0u;
    __syncthreads();
    const int cur = pass & 1;
    const long long base = (long long)ct.y * SORT_T;
    const int shift = 8 * pass;
    for (int i = threadIdx.x; i < SORT_T; i += SORT_THREADS) {
        const long long pos = base + i;
        if (pos >= N) break;
        const unsigned int d = (unsigned int)(load_key(C, f, sb, pass, cur, pos) >> shift) & (RADIX - 1);
        atomicAdd(&h[w][d], 1u);
    }
    __syncthreads();
    const int ntiles = tm.count[ct.x];
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
        unsigned int s = 0;
        for (int q = 0; q < SORT_THREADS / 32; ++q) s += h[q][d];
        sb.hist[sb.hist_off[ct.x] + (long long)d * ntiles + ct.y] = s;
    }
}

// One block per (cluster, digit): exclusive scan over the cluster's tiles.
__global__ void __launch_bounds__(256) k_sort_scan(Tiles tm, SortBufs sb, int pass, int nclusters)
{
    __shared__ unsigned int s_warp[8];
    __shared__ unsigned int s_carry;
    const int c = blockIdx.x / RADIX, d = blockIdx.x % RADIX;
    if (c >= nclusters || pass >= sb.npass[c]) return;
    const int ntiles = tm.count[c];
    unsigned int *h = sb.hist + sb.hist_off[c] + (long long)d * ntiles;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 256) {
        const int t = base + threadIdx.x;
        const unsigned int v = (t < ntiles) ? h[t] : 0u;
        unsigned int x = v;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[wid] = x;
        __syncthreads();
        unsigned int wb = 0;
        for (int q = 0; q < wid; ++q) wb += s_warp[q];
        const unsigned int carry = s_carry;
        if (t < ntiles) h[t] = carry + wb + x - v;  // exclusive
        __syncthreads();
        if (threadIdx.x == 255) s_carry = carry + wb + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) sb.digit_total[c * RADIX + d] = s_carry;
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                               SortBufs sb, int pass)
{
    __shared__ unsigned int wcnt[SORT_THREADS / 32][RADIX];  // per-warp digit counters -> prefixes
    __shared__ unsigned int dstart[RADIX];                     // in-tile digit start
    __shared__ unsigned int gbase[RADIX];                      // global digit start for this tile
    __shared__ unsigned long long sk[SORT_T];
    __shared__ unsigned int sv[SORT_T];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    if (pass >= sb.npass[ct.x]) return;
    const long long N = C.sc->N_MAX_NEW;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int cur = pass & 1, nxt = cur ^ 1;
    const int shift = 8 * pass;
    const long long base = (long long)ct.y * SORT_T;
    for (int i = threadIdx.x; i < (SORT_THREADS / 32) * RADIX; i += SORT_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();

    unsigned long long key[SORT_ITEMS];
    unsigned int val[SORT_ITEMS], dig[SORT_ITEMS], rank[SORT_ITEMS];
    bool valid[SORT_ITEMS];
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        // warp-striped: warp w owns [w*256, w*256+256), item it, lane l -> w*256 + it*32 + l
        const long long pos = base + w * (SORT_ITEMS * 32) + it * 32 + lane;
        valid[it] = pos < N;
        key[it] = valid[it] ? load_key(C, f, sb, pass, cur, pos) : 0ull;
        val[it] = valid[it] ? (pass == 0 ? (unsigned int)pos : (cur ? sb.vals[1] : sb.vals[0])[C.off + pos]) : 0u;
        dig[it] = (unsigned int)(key[it] >> shift) & (RADIX - 1);
    }
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        const unsigned int tag = valid[it] ? dig[it] : (0x10000u + lane);
        const unsigned int peers = __match_any_sync(0xffffffffu, tag);
        const unsigned int below = peers & ((1u << lane) - 1u);
        unsigned int b = 0;
        if (valid[it]) b = wcnt[w][dig[it]];
        __syncwarp();
        if (valid[it] && below == 0u) wcnt[w][dig[it]] = b + __popc(peers);
        __syncwarp();
        rank[it] = b + __popc(below);
    }
    __syncthreads();
    // per digit: exclusive prefix over warps, tile total
    for (int d = threadIdx.x; d < RADIX; d += SORT_THREADS) {
        unsigned int s = 0;
        for (int q = 0; q < SORT_THREADS / 32; ++q) {
            const unsigned int t = wcnt[q][d];
            wcnt[q][d] = s;
            s += t;
        }
        dstart[d] = s;  // tile count for now
    }
    __syncthreads();
    // exclusive scan of the tile counts over digits (256 threads, one digit each)
    {
        const int d = threadIdx.x;
        const unsigned int v = dstart[d];
        unsigned int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        __shared__ unsigned int s_w[SORT_THREADS / 32];
        if (lane == 31) s_w[w] = x;
        // global base of digit d for this tile: digits below d in the cluster + tiles before
        const int ntiles = tm.count[ct.x];
        unsigned int dbelow = 0;
        const unsigned int *tot = sb.digit_total + ct.x * RADIX;
        // exclusive prefix of the cluster's digit totals
        unsigned int tv = tot[d], tx = tv;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned int y = __shfl_up_sync(0xffffffffu, tx, o);
            if (lane >= o) tx += y;
        }
        __shared__ unsigned int s_t[SORT_THREADS / 32];
        if (lane == 31) s_t[w] = tx;
        __syncthreads();
        unsigned int wb = 0, tb = 0;
        for (int q = 0; q < w; ++q) {
            wb += s_w[q];
            tb += s_t[q];
        }
        dbelow = tb + tx - tv;
        const unsigned int excl = wb + x - v;
        __syncthreads();
        dstart[d] = excl;
        gbase[d] = dbelow + sb.hist[sb.hist_off[ct.x] + (long long)d * ntiles + ct.y];
    }
    __syncthreads();
    // stage in shared memory in (digit, stable rank) order
#pragma unroll
    for (int it = 0; it < SORT_ITEMS; ++it) {
        if (valid[it]) {
            const unsigned int p = dstart[dig[it]] + wcnt[w][dig[it]] + rank[it];
            sk[p] = key[it];
            sv[p] = val[it];
        }
    }
    __syncthreads();
    long long nt = N - base;
    if (nt > SORT_T) nt = SORT_T;
    unsigned long long *kout = nxt ? sb.keys[1] : sb.keys[0];
    unsigned int *vout = nxt ? sb.vals[1] : sb.vals[0];
    for (int i = threadIdx.x; i < nt; i += SORT_THREADS) {
        const unsigned long long k = sk[i];
        const unsigned int d = (unsigned int)(k >> shift) & (RADIX - 1);
        const long long dst = (long long)gbase[d] + (i - (long long)dstart[d]);
        if (dst < 0 || dst >= N) {  // inconsistent counts: record, never write out of range
            set_error(C.sc, CMCG_ERR_SPIN, dst);
            continue;
        }
        kout[C.off + dst] = k;
        vout[C.off + dst] = sv[i];
    }
}

// Payload gather into radial order (ComputeIntermediateEnergy transfer +
// post_sort_comm).  Writes the second buffers of r, m, id, ec_pre, which the
// host then swaps with the first.
__global__ void __launch_bounds__(256) k_sort_gather(const Cluster *__restrict__ cls, Tiles tm, Fields f, SortBufs sb)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long nb = sc->n_bound;
    const int np = sb.npass[ct.x];
    const long long i = (long long)ct.y * 256 + threadIdx.x;  // 0-based output position
    const long long off = C.off;
    if (nb < 0 || nb > sc->N_MAX_NEW) {
        if (i == 0) set_error(sc, CMCG_ERR_BOUNDS, nb);
        return;
    }
    if (i < nb) {
        const long long src = 1 + (np == 0 ? i : (long long)((np & 1) ? sb.vals[1] : sb.vals[0])[off + i]);
        if (src < 1 || src > sc->N_MAX_NEW) {
            set_error(sc, CMCG_ERR_BOUNDS, src);
            return;
        }
        const long long gs = off + src, gd = off + 1 + i;
        f.r2[gd] = f.rnew[gs];
        f.m2[gd] = f.m[gs];
        f.vr[gd] = f.vrnew[gs];
        f.vt[gd] = f.vtnew[gs];
        f.id2[gd] = f.id[gs];
        f.rOld[gd] = f.r[gs];
        f.ec_pre2[gd] = f.ec_pre[gs];
    }
    if (i == 0) {
        // the second buffers become the live arrays: carry the sentinels over
        // (star_r[0] = ZERO, star_m[0] = 0; star_r[N+1] is reset by the potential)
        f.r2[off] = CMCG_ZERO;
        f.m2[off] = 0.0;
        f.id2[off] = 0;
        f.ec_pre2[off] = 0.0;
        f.r2[off + nb + 1] = CMCG_SF_INFINITY;
        f.m2[off + nb + 1] = 0.0;
    }
}

// New N_MAX after the gather (cmc_sort.c:343-354, cmc_utils.c:2246); a kernel of
// its own so no gather block ever sees the count change under it.
__global__ void k_sort_commit(const Cluster *__restrict__ cls, int nclusters)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nclusters) return;
    Scalars *sc = cls[c].sc;
    if (sc->n_bound < 0 || sc->n_bound > sc->N_MAX_NEW) {
        set_error(sc, CMCG_ERR_BOUNDS, sc->n_bound);
        return;
    }
    sc->N_MAX = sc->n_bound;
    sc->N_MAX_NEW = sc->n_bound;
}

}  // namespace cmcg
