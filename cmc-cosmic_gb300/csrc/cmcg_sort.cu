// cmcg_sort.cu -- stable LSD radix sort of the stars by radius, per cluster.
//
// Restates qsorts_new (cmc_utils.c:2232-2254) with the one-rank sample_sort
// (cmc_sort.c:375-420: local qsort by r, remove_stripped_stars 343-354) and
// post_sort_comm (cmc_utils.c:2259-2288), preceded by the transfer half of
// ComputeIntermediateEnergy (cmc_utils.c:381-390: r = rnew, vr = vrnew,
// vt = vtnew, rOld = old r).
//
// Keys are the IEEE bit patterns of rnew (positive doubles order like their
// bits) less the cluster's smallest, with every escaper (rnew = SF_INFINITY)
// at the first key of the 24-bit prefix after the largest bound key's;
// values the star's slot.  The digit passes sort the keys' top 24 bits (3
// passes); keys that share them then form runs in input order, which are put
// in full-key order as the payload moves (runs are a star or two at the
// densities of these clusters; the escapers' run is equal keys, already in
// order).
//   k_sort_prep      the key range and kept count per cluster; clears the
//                    sort's counters
//   k_sort_ghist     every 8-bit digit's histogram in one read of the keys
//   k_sort_onesweep  one kernel per digit pass over tiles of 4096 (default),
//                    2048 or 1024 keys: stable in-tile ranking (warp match +
//                    per-warp counters), tile offsets by decoupled look-back,
//                    staging through shared memory so runs of one digit leave
//                    the block as contiguous stores
// Tiles never straddle clusters, so one launch sorts every cluster of an
// ensemble independently.
// The radii (pass 0, the histograms, the key range) and the keys and values of
// the later passes are read with 128-bit loads: double2 pairs of radii,
// ulonglong2 pairs of keys and uint4 quads of values, staged through shared
// memory into the warp-striped order the ranking uses.
// k_sort_gather then moves the payload (rnew, m, vrnew, vtnew, id, r, ec_pre)
// into radial order, one 8-byte gather per field and star, and drops the
// escapers (r == SF_INFINITY), which sort last.  Each of its threads places
// its star within the star's run by the rank of (key, position) in it; runs
// longer than FIX_SHORT go to k_sort_fix_long, which sorts them and moves their
// payload.  (The allocation-free sort, which has no payload, sorts the runs
// in place with k_sort_fix and k_sort_fix_long instead.)
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
    // the sort's counters start at zero: the digit passes' tile counters, and
    // each cluster's digit totals and long-run count (k_sort_ghist, the gather)
    if (blockIdx.x == 0 && threadIdx.x < SORT_MAX_PASSES) sb.tile_next[threadIdx.x] = 0u;
    if (ct.y == 0) {
        for (int i = threadIdx.x; i < SORT_MAX_PASSES * RADIX; i += SORT_THREADS)
            sb.ghist[(size_t)ct.x * SORT_MAX_PASSES * RADIX + i] = 0ull;
        if (threadIdx.x == 0) sb.nlong[ct.x] = 0u;
    }
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX_NEW;
    const unsigned long long inf_bits = (unsigned long long)__double_as_longlong(CMCG_SF_INFINITY);
    unsigned long long kmn = ~0ull, kmx = 0ull;
    long long cnt = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(sb.epoch, 1u);  // this sort's look-back epoch
    // stars k = k0 + 1 .. k0 + SORT_T (1-based), with 128-bit loads: the
    // aligned pair at C.off + k0 + 2t holds stars k0 + 2t and k0 + 2t + 1
    const long long k0 = (long long)ct.y * SORT_T;
    const double *src = f.rnew + C.off + k0;
    for (int t = threadIdx.x; t <= SORT_T / 2; t += SORT_THREADS) {
        const long long k = k0 + 2 * (long long)t;  // the pair's first star
        if (k > N) break;
        const double2 v = *reinterpret_cast<const double2 *>(src + 2 * t);
        const unsigned long long b0 = (unsigned long long)__double_as_longlong(v.x);
        const unsigned long long b1 = (unsigned long long)__double_as_longlong(v.y);
        if (t > 0 && b0 != inf_bits) {
            cnt++;
            kmn = min(kmn, b0);
            kmx = max(kmx, b0);
        }
        if (k + 1 <= N && t < SORT_T / 2 && b1 != inf_bits) {
            cnt++;
            kmn = min(kmn, b1);
            kmx = max(kmx, b1);
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
    __shared__ int s_last;
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
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        // every thread folds a strided share of the tiles (loads bypass L1), then the warps combine
        unsigned long long a = ~0ull, b = 0ull;
        long long n = 0;
        const int b0 = tm.first[ct.x], nt = tm.count[ct.x];
        for (int q = threadIdx.x; q < nt; q += SORT_THREADS) {
            const double *sp = partials + (size_t)(b0 + q) * 3;
            a = min(a, (unsigned long long)__double_as_longlong(__ldcg(sp)));
            b = max(b, (unsigned long long)__double_as_longlong(__ldcg(sp + 1)));
            n += (long long)__ldcg(sp + 2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = min(a, __shfl_down_sync(0xffffffffu, a, o));
            b = max(b, __shfl_down_sync(0xffffffffu, b, o));
            n += __shfl_down_sync(0xffffffffu, n, o);
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) {
            s_min[w] = a;
            s_max[w] = b;
            s_cnt[w] = n;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int q = 1; q < SORT_THREADS / 32; ++q) {
                a = min(a, s_min[q]);
                b = max(b, s_max[q]);
                n += s_cnt[q];
            }
            sc->n_bound = n;
            // sort keys: a bound star's bit pattern minus the smallest one; the
            // digit passes sort the top SORT_PREFIX_BITS bits of the range
            // (bits below the shift are left to the run placement).  Escapers all take
            // the first key of the prefix after the largest bound key's: they
            // sort after every bound star as a run of equal keys of their own,
            // which the stable passes leave in input order.
            unsigned long long top = 0ull;
            int sh = 0;
            if (n == 0) {
                a = inf_bits;  // every key the same: nothing to sort
            } else {
                const unsigned long long R = b - a;
                const int bitsR = R ? 64 - __clzll((long long)R) : 0;
                sh = bitsR > SORT_PREFIX_BITS ? bitsR - SORT_PREFIX_BITS : 0;
                top = R;
                if (n < N) {
                    for (;;) {  // at most one more bit of range: settles in two turns
                        top = ((R >> sh) + 1ull) << sh;
                        if (64 - __clzll((long long)top) - sh <= SORT_PREFIX_BITS) break;
                        ++sh;
                    }
                }
            }
            sb.kmin[ct.x] = a;
            sb.kmax[ct.x] = top;
            const int bits = top ? 64 - __clzll((long long)top) : 0;
            sb.shift[ct.x] = sh;
            sb.npass[ct.x] = (bits - sh + 7) / 8;
        }
    }
}

// The sort key of a radius (k_sort_prep): bits - kmin, escapers the key kmax.
static __device__ __forceinline__ unsigned long long radius_key(double r, unsigned long long kmin,
                                                                unsigned long long kesc)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(r);
    return b == (unsigned long long)__double_as_longlong(CMCG_SF_INFINITY) ? kesc : b - kmin;
}

// All digit histograms of the cluster's keys in one read (they do not depend
// on the order the passes put the keys in): per-block shared counters, then
// one global add per (pass, digit).
__global__ void __launch_bounds__(SORT_THREADS) k_sort_ghist(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                             SortBufs sb)
{
    __shared__ unsigned int h[SORT_MAX_PASSES][RADIX];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const int np = sb.npass[ct.x];
    if (np == 0) return;
    const long long N = C.sc->N_MAX_NEW;
    const unsigned long long kmin = sb.kmin[ct.x], kesc = sb.kmax[ct.x];
    const int sh = sb.shift[ct.x];
    for (int i = threadIdx.x; i < SORT_MAX_PASSES * RADIX; i += SORT_THREADS) (&h[0][0])[i] = 0u;
    __syncthreads();
    const long long base = (long long)ct.y * SORT_T, ntile = N - base;
    // 128-bit loads: the aligned pair at src + 2t holds items 2t - 1 and 2t
    const double *src = f.rnew + C.off + base;
    for (int t = threadIdx.x; t <= SORT_T / 2; t += SORT_THREADS) {
        const long long i0 = 2 * (long long)t - 1;
        if (i0 >= ntile) break;
        const double2 v = *reinterpret_cast<const double2 *>(src + 2 * t);
        if (i0 >= 0) {
            const unsigned long long k = radius_key(v.x, kmin, kesc);
            for (int p = 0; p < np; ++p) atomicAdd(&h[p][(unsigned int)(k >> (sh + 8 * p)) & (RADIX - 1)], 1u);
        }
        if (i0 + 1 < ntile && i0 + 1 < SORT_T) {
            const unsigned long long k = radius_key(v.y, kmin, kesc);
            for (int p = 0; p < np; ++p) atomicAdd(&h[p][(unsigned int)(k >> (sh + 8 * p)) & (RADIX - 1)], 1u);
        }
    }
    __syncthreads();
    unsigned long long *g = sb.ghist + (size_t)ct.x * SORT_MAX_PASSES * RADIX;
    for (int i = threadIdx.x; i < np * RADIX; i += SORT_THREADS) {
        const unsigned int v = (&h[0][0])[i];
        if (v) atomicAdd(g + i, (unsigned long long)v);
    }
}

// Tile status word of the decoupled look-back: the pass's epoch (sort count x 8
// + pass) in the top 30 bits, a flag (1 = this tile's count, 2 = inclusive
// prefix through this tile) in the next two, the count below.  Words of
// earlier passes and sorts carry another epoch and read as not ready, so the
// words are never cleared (graph replays included).
constexpr unsigned long long ST_AGG = 1ull << 32, ST_INC = 2ull << 32, ST_VAL = 0xffffffffull;
constexpr int LOOKBACK = 8;  // predecessor tiles read per round trip of the look-back
__device__ __forceinline__ unsigned long long st_tag(unsigned int epoch, int pass)
{
    return ((unsigned long long)((epoch * SORT_MAX_PASSES + (unsigned)pass) & 0x3fffffffu)) << 34;
}

// One digit pass (onesweep): tiles take their order from an atomic counter,
// rank their keys stably in shared memory, publish per-digit counts and
// obtain the counts of the tiles before them in the cluster by decoupled
// look-back (Merrill & Garland's single-pass scan, as in Adinets & Merrill's
// onesweep radix sort), then write their keys in runs of one digit.  A tile
// only waits on tiles that took a smaller index, which have started; every
// wait is bounded and records CMCG_ERR_SPIN if it gives up.
template <int ITEMS>
__global__ void __launch_bounds__(OS_THREADS, 2) k_sort_onesweep(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                              SortBufs sb, int pass)
{
    constexpr int NWARP = OS_THREADS / 32, T = OS_THREADS * ITEMS;  // T keys per tile
    __shared__ unsigned int wcnt[NWARP][RADIX];  // per-warp digit counters -> prefixes
    __shared__ unsigned int dstart[RADIX];       // in-tile digit start
    __shared__ unsigned long long gbase[RADIX];  // global digit start for this tile
    // the tile's keys and values (dynamic: T x 12 bytes, 48 KB at 4096 keys)
    extern __shared__ __align__(16) unsigned char os_dyn[];
    unsigned long long *sk = reinterpret_cast<unsigned long long *>(os_dyn);
    unsigned int *sv = reinterpret_cast<unsigned int *>(os_dyn + sizeof(unsigned long long) * T);
    __shared__ unsigned int s_w[RADIX / 32];
    __shared__ unsigned long long s_t[RADIX / 32];
    __shared__ int s_b;
    if (threadIdx.x == 0) s_b = (int)atomicAdd(sb.tile_next + pass, 1u);
    __syncthreads();
    const int b = s_b;
    if (b >= tm.ntiles) return;
    const int2 ct = tm.tiles[b];
    const Cluster &C = cls[ct.x];
    // every tile of a cluster takes the same early exit, so no tile waits on one that left
    if (!counts_ok(C)) return;
    if (pass >= sb.npass[ct.x]) return;
    const long long N = C.sc->N_MAX_NEW;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int cur = pass & 1, nxt = cur ^ 1;
    const int shift = sb.shift[ct.x] + 8 * pass;
    const long long base = (long long)ct.y * T;
    for (int i = threadIdx.x; i < NWARP * RADIX; i += OS_THREADS) (&wcnt[0][0])[i] = 0u;
    __syncthreads();

    // The tile's keys and values into shared memory with 128-bit loads (the
    // output staging buffers are free until the ranking is done), then each
    // thread takes its warp-striped items from there.  Slices start on
    // 256-byte boundaries and are padded to 32 elements, so every vector load
    // is aligned and stays inside the cluster's slice.
    const long long ntile = N - base;  // items of this tile (<= 0: none)
    if (pass == 0) {
        // radii are 1-based: item i is rnew[C.off + 1 + base + i]; the aligned
        // pair at src + 2t holds items 2t - 1 and 2t
        const double *src = f.rnew + C.off + base;
        const unsigned long long kmin = sb.kmin[ct.x], kesc = sb.kmax[ct.x];
        for (int t = threadIdx.x; t <= T / 2; t += OS_THREADS) {
            const long long i0 = 2 * (long long)t - 1;
            if (i0 >= ntile) break;
            const double2 v = *reinterpret_cast<const double2 *>(src + 2 * t);
            if (i0 >= 0) sk[i0] = radius_key(v.x, kmin, kesc);
            if (i0 + 1 < ntile && i0 + 1 < T) sk[i0 + 1] = radius_key(v.y, kmin, kesc);
        }
    } else {
        const unsigned long long *ks = (cur ? sb.keys[1] : sb.keys[0]) + C.off + base;
        const unsigned int *vs = (cur ? sb.vals[1] : sb.vals[0]) + C.off + base;
        for (int t = threadIdx.x; t < T / 4; t += OS_THREADS) {
            const long long i0 = 4 * (long long)t;
            if (i0 >= ntile) break;
            if (i0 + 3 < ntile) {
                *reinterpret_cast<ulonglong2 *>(sk + i0) = *reinterpret_cast<const ulonglong2 *>(ks + i0);
                *reinterpret_cast<ulonglong2 *>(sk + i0 + 2) = *reinterpret_cast<const ulonglong2 *>(ks + i0 + 2);
                *reinterpret_cast<uint4 *>(sv + i0) = *reinterpret_cast<const uint4 *>(vs + i0);
            } else {
                for (long long q = i0; q < ntile; ++q) {
                    sk[q] = ks[q];
                    sv[q] = vs[q];
                }
            }
        }
    }
    __syncthreads();
    unsigned long long key[ITEMS];
    unsigned int val[ITEMS], dig[ITEMS], rank[ITEMS];
    bool valid[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
        // warp-striped: warp w owns [w*ITEMS*32, (w+1)*ITEMS*32), item it, lane l -> w*ITEMS*32 + it*32 + l
        const int i = w * (ITEMS * 32) + it * 32 + lane;
        valid[it] = i < ntile;
        key[it] = valid[it] ? sk[i] : 0ull;
        val[it] = valid[it] ? (pass == 0 ? (unsigned int)(base + i) : sv[i]) : 0u;
        dig[it] = (unsigned int)(key[it] >> shift) & (RADIX - 1);
    }
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
        const unsigned int tag = valid[it] ? dig[it] : (0x10000u + lane);
        const unsigned int peers = __match_any_sync(0xffffffffu, tag);
        const unsigned int below = peers & ((1u << lane) - 1u);
        unsigned int bb = 0;
        if (valid[it]) bb = wcnt[w][dig[it]];
        __syncwarp();
        if (valid[it] && below == 0u) wcnt[w][dig[it]] = bb + __popc(peers);
        __syncwarp();
        rank[it] = bb + __popc(below);
    }
    __syncthreads();
    // threads 0..RADIX-1 own one digit each: prefix over warps, publish, look back
    const int d = threadIdx.x;
    unsigned long long prefix = 0, tot = 0;
    unsigned int cnt = 0;
    if (d < RADIX) {
        for (int q = 0; q < NWARP; ++q) {
            const unsigned int t = wcnt[q][d];
            wcnt[q][d] = cnt;
            cnt += t;
        }
        const unsigned long long tag = st_tag(*(volatile unsigned int *)sb.epoch, pass);
        unsigned long long *st = sb.status + (size_t)b * RADIX;
        atomicExch(st + d, tag | (ct.y == 0 ? ST_INC : ST_AGG) | cnt);
        if (ct.y > 0) {
            // walk back to the nearest inclusive prefix, summing aggregates on
            // the way; LOOKBACK predecessors are read at once, so a long run
            // of aggregates costs one round trip per LOOKBACK tiles
            const int jfirst = b - ct.y;  // the cluster's first tile publishes inclusive
            int j = b - 1;
            long long spins = 0;
            bool found = false;
            while (!found) {
                unsigned long long v[LOOKBACK];
#pragma unroll
                for (int q = 0; q < LOOKBACK; ++q)
                    v[q] = (j - q >= jfirst) ? *(volatile unsigned long long *)(sb.status + (size_t)(j - q) * RADIX + d)
                                             : 0ull;
                int used = 0;
#pragma unroll
                for (int q = 0; q < LOOKBACK; ++q) {
                    if (found || used < q || j - q < jfirst) continue;
                    if ((v[q] & ~(ST_INC | ST_AGG | ST_VAL)) != tag || !(v[q] & (ST_INC | ST_AGG))) continue;
                    prefix += v[q] & ST_VAL;
                    if (v[q] & ST_INC) found = true;
                    else used = q + 1;  // an aggregate: go on to the next older tile
                }
                if (found) break;
                j -= used;
                if (used == 0 && ++spins > CMCG_SPIN_LIMIT) {
                    set_error(C.sc, CMCG_ERR_SPIN, j);
                    break;
                }
            }
            atomicExch(st + d, tag | ST_INC | (prefix + cnt));
        }
        tot = sb.ghist[((size_t)ct.x * SORT_MAX_PASSES + pass) * RADIX + d];
    }
    // exclusive scans over digits (warps 0..RADIX/32-1 are the digit owners):
    // the tile's counts -> in-tile digit starts; the cluster's totals -> global starts
    unsigned int x = cnt;
    unsigned long long tx = tot;
    if (d < RADIX) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
            const unsigned long long ty = __shfl_up_sync(0xffffffffu, tx, o);
            if (lane >= o) {
                x += y;
                tx += ty;
            }
        }
        if (lane == 31) {
            s_w[w] = x;
            s_t[w] = tx;
        }
    }
    __syncthreads();
    if (d < RADIX) {
        unsigned int wb = 0;
        unsigned long long tb = 0;
        for (int q = 0; q < w; ++q) {
            wb += s_w[q];
            tb += s_t[q];
        }
        dstart[d] = wb + x - cnt;
        gbase[d] = tb + tx - tot + prefix;
    }
    __syncthreads();
    // stage in shared memory in (digit, stable rank) order
#pragma unroll
    for (int it = 0; it < ITEMS; ++it) {
        if (valid[it]) {
            const unsigned int pidx = dstart[dig[it]] + wcnt[w][dig[it]] + rank[it];
            sk[pidx] = key[it];
            sv[pidx] = val[it];
        }
    }
    __syncthreads();
    long long nt = N - base;
    if (nt > T) nt = T;
    unsigned long long *kout = nxt ? sb.keys[1] : sb.keys[0];
    unsigned int *vout = nxt ? sb.vals[1] : sb.vals[0];
    for (int i = threadIdx.x; i < nt; i += OS_THREADS) {
        const unsigned long long k = sk[i];
        const unsigned int dd = (unsigned int)(k >> shift) & (RADIX - 1);
        const long long dst = (long long)gbase[dd] + (i - (long long)dstart[dd]);
        if (dst < 0 || dst >= N) {  // inconsistent counts: record, never write out of range
            set_error(C.sc, CMCG_ERR_SPIN, dst);
            continue;
        }
        kout[C.off + dst] = k;
        vout[C.off + dst] = sv[i];
    }
}

constexpr size_t os_dyn_bytes(int items)
{
    return (size_t)OS_THREADS * items * (sizeof(unsigned long long) + sizeof(unsigned int));
}

cudaError_t sort_onesweep_setup()
{
    // 4096-key tiles stage 48 KB of keys and values beside the static counters
    return cudaFuncSetAttribute(k_sort_onesweep<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)os_dyn_bytes(8));
}

void launch_sort_onesweep(int tile_keys, int ntiles, cudaStream_t s, const Cluster *cls, Tiles tm, Fields f,
                          SortBufs sb, int pass)
{
    if (tile_keys == OS_THREADS * 2)
        k_sort_onesweep<2><<<ntiles, OS_THREADS, os_dyn_bytes(2), s>>>(cls, tm, f, sb, pass);
    else if (tile_keys == OS_THREADS * 8)
        k_sort_onesweep<8><<<ntiles, OS_THREADS, os_dyn_bytes(8), s>>>(cls, tm, f, sb, pass);
    else
        k_sort_onesweep<4><<<ntiles, OS_THREADS, os_dyn_bytes(4), s>>>(cls, tm, f, sb, pass);
}

// After the digit passes, runs of keys sharing their sorted prefix are in
// input order; each is sorted here by its full key.  The thread at a run's
// start takes it: a run of one is done, a sorted run is done, runs up to
// FIX_SHORT are insertion-sorted (stable), longer runs are listed for
// k_sort_fix_long.
__global__ void __launch_bounds__(SORT_THREADS) k_sort_fix(const Cluster *__restrict__ cls, Tiles tm, SortBufs sb)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const int sh = sb.shift[ct.x];
    if (sh == 0) return;  // the passes sorted every bit
    const int np = sb.npass[ct.x];
    const long long N = C.sc->N_MAX_NEW;
    unsigned long long *K = ((np & 1) ? sb.keys[1] : sb.keys[0]) + C.off;
    unsigned int *V = ((np & 1) ? sb.vals[1] : sb.vals[0]) + C.off;
    // the escapers' run: equal keys, already in input order
    const unsigned long long pesc = C.sc->n_bound < N ? sb.kmax[ct.x] >> sh : ~0ull;
    for (int it = 0; it < SORT_T / SORT_THREADS; ++it) {
        const long long i = (long long)ct.y * SORT_T + it * SORT_THREADS + threadIdx.x;
        if (i >= N) break;
        const unsigned long long p = K[i] >> sh;
        if (i > 0 && (K[i - 1] >> sh) == p) continue;  // not a run start
        if (p == pesc) continue;
        long long j = i + 1;
        bool sorted = true;
        unsigned long long prev = K[i];
        while (j < N && j - i <= FIX_SHORT) {
            const unsigned long long kj = K[j];
            if ((kj >> sh) != p) break;
            if (kj < prev) sorted = false;
            prev = kj;
            ++j;
        }
        if (j - i > FIX_SHORT) {  // the run goes on past FIX_SHORT keys
            const unsigned int e = atomicAdd(sb.nlong + ct.x, 1u);
            sb.lstart[C.off / 32 + 64 * ct.x + e] = i;  // at most N / (FIX_SHORT + 1) runs fit
            continue;
        }
        if (sorted) continue;
        for (long long a = i + 1; a < j; ++a) {  // insertion sort: equal keys keep their order
            const unsigned long long ka = K[a];
            const unsigned int va = V[a];
            long long b = a - 1;
            while (b >= i && K[b] > ka) {
                K[b + 1] = K[b];
                V[b + 1] = V[b];
                --b;
            }
            K[b + 1] = ka;
            V[b + 1] = va;
        }
    }
}

// One star's payload from input slot v (0-based) to output position i
// (0-based) of the radial order (ComputeIntermediateEnergy transfer +
// post_sort_comm): the second buffers of r, m, id and ec_pre, which the host
// then swaps with the first.
__device__ __forceinline__ void move_star(const Cluster &C, const Fields &f, unsigned int v, long long i)
{
    const long long src = 1 + (long long)v;
    if (src > C.sc->N_MAX_NEW) {
        set_error(C.sc, CMCG_ERR_BOUNDS, src);
        return;
    }
    const long long gs = C.off + src, gd = C.off + 1 + i;
    f.r2[gd] = f.rnew[gs];
    f.m2[gd] = f.m[gs];
    f.vr[gd] = f.vrnew[gs];
    f.vt[gd] = f.vtnew[gs];
    f.id2[gd] = f.id[gs];
    f.rOld[gd] = f.r[gs];
    f.ec_pre2[gd] = f.ec_pre[gs];
}

// The output position of the key at sorted position i of n (keys 0..n-1 after
// the digit passes, which order the prefixes K >> sh): i itself when no
// neighbour shares its prefix; inside a run of keys sharing it, the run's
// start plus the rank of (key, position) among the run's members, which is
// the stable full-key order (members are in input order).  A run longer than
// FIX_SHORT returns -1; its first member lists it for k_sort_fix_long.
__device__ __forceinline__ long long run_place(const unsigned long long *K, long long i, long long n, int sh,
                                               unsigned int *nlong, long long *lists)
{
    const unsigned long long ki = K[i], p = ki >> sh;
    const bool up = i > 0 && (K[i - 1] >> sh) == p;
    const bool dn = i + 1 < n && (K[i + 1] >> sh) == p;
    if (!up && !dn) return i;
    long long s = i;  // walk back to the run's start, at most FIX_SHORT + 1 keys
#pragma unroll 1
    while (s > 0 && i - s <= FIX_SHORT && (K[s - 1] >> sh) == p) --s;
    long long e = i + 1;
#pragma unroll 1
    while (e < n && e - s <= FIX_SHORT && (K[e] >> sh) == p) ++e;
    if (e - s > FIX_SHORT) {
        if (!up) lists[atomicAdd(nlong, 1u)] = i;  // at most n / (FIX_SHORT + 1) runs fit
        return -1;
    }
    long long r = 0;
#pragma unroll 1
    for (long long j = s; j < e; ++j) {
        const unsigned long long kj = K[j];
        r += (kj < ki) || (kj == ki && j < i);
    }
    return s + r;
}

// (key, slot) pairs ordered by key, then by slot: the slots are the input
// positions, so this order is the stable one and no two pairs are equal.
__device__ __forceinline__ bool pair_less(unsigned long long ka, unsigned int va, unsigned long long kb,
                                          unsigned int vb)
{
    return ka < kb || (ka == kb && va < vb);
}

// New N_MAX after the gather (cmc_sort.c:343-354, cmc_utils.c:2246), once
// every block of the cluster is past it.
__device__ __forceinline__ void sort_commit(Scalars *sc)
{
    if (sc->n_bound < 0 || sc->n_bound > sc->N_MAX_NEW) {
        set_error(sc, CMCG_ERR_BOUNDS, sc->n_bound);
        return;
    }
    sc->N_MAX = sc->n_bound;
    sc->N_MAX_NEW = sc->n_bound;
}

// Runs longer than FIX_SHORT, each by one block (a cluster's tiles share its
// list): a bitonic network in the form whose first comparison of each merge
// pairs i with its mirror i ^ (k - 1), so every comparison is ascending and
// lengths need no padding.  Up to FIX_BLOCK keys in shared memory, longer
// runs in place in global memory.
// With gather, also each run's payload (the step's sort).
__device__ __forceinline__ void sort_long_runs(const Cluster &C, int2 ct, const Tiles &tm, const SortBufs &sb,
                                               const Fields &f, bool gather)
{
    __shared__ unsigned long long s_k[FIX_BLOCK];
    __shared__ unsigned int s_v[FIX_BLOCK];
    __shared__ long long s_len;
    const int sh = sb.shift[ct.x];
    const int np = sb.npass[ct.x];
    const long long N = C.sc->N_MAX_NEW;
    unsigned long long *K = ((np & 1) ? sb.keys[1] : sb.keys[0]) + C.off;
    unsigned int *V = ((np & 1) ? sb.vals[1] : sb.vals[0]) + C.off;
    const unsigned int nl = *(volatile unsigned int *)(sb.nlong + ct.x);
    for (unsigned int e = ct.y; e < nl; e += tm.count[ct.x]) {
        const long long s = sb.lstart[C.off / 32 + 64 * ct.x + e];
        if (threadIdx.x == 0) {
            const unsigned long long p = K[s] >> sh;
            long long j = s + 1;
            while (j < N && (K[j] >> sh) == p) ++j;
            s_len = j - s;
        }
        __syncthreads();
        const long long L = s_len;
        if (L <= FIX_BLOCK) {
            for (long long t = threadIdx.x; t < L; t += SORT_THREADS) {
                s_k[t] = K[s + t];
                s_v[t] = V[s + t];
            }
            __syncthreads();
            for (long long k = 2; k < 2 * L; k <<= 1) {
                for (long long jj = k >> 1; jj > 0; jj >>= 1) {
                    for (long long i = threadIdx.x; i < L; i += SORT_THREADS) {
                        const long long l = (jj == (k >> 1)) ? (i ^ (k - 1)) : (i ^ jj);
                        if (l > i && l < L && pair_less(s_k[l], s_v[l], s_k[i], s_v[i])) {
                            const unsigned long long tk = s_k[i];
                            const unsigned int tv = s_v[i];
                            s_k[i] = s_k[l];
                            s_v[i] = s_v[l];
                            s_k[l] = tk;
                            s_v[l] = tv;
                        }
                    }
                    __syncthreads();
                }
            }
            for (long long t = threadIdx.x; t < L; t += SORT_THREADS) {
                K[s + t] = s_k[t];
                V[s + t] = s_v[t];
                if (gather) move_star(C, f, s_v[t], s + t);
            }
        } else {
            unsigned long long *k0 = K + s;
            unsigned int *v0 = V + s;
            for (long long k = 2; k < 2 * L; k <<= 1) {
                for (long long jj = k >> 1; jj > 0; jj >>= 1) {
                    for (long long i = threadIdx.x; i < L; i += SORT_THREADS) {
                        const long long l = (jj == (k >> 1)) ? (i ^ (k - 1)) : (i ^ jj);
                        if (l > i && l < L && pair_less(k0[l], v0[l], k0[i], v0[i])) {
                            const unsigned long long tk = k0[i];
                            const unsigned int tv = v0[i];
                            k0[i] = k0[l];
                            v0[i] = v0[l];
                            k0[l] = tk;
                            v0[l] = tv;
                        }
                    }
                    __syncthreads();  // orders the block's global writes between stages
                }
            }
            if (gather)
                for (long long t = threadIdx.x; t < L; t += SORT_THREADS) move_star(C, f, v0[t], s + t);
        }
        __syncthreads();
    }
}

// The long runs, then (the step's sort, tickets given) the star-count commit.
__global__ void __launch_bounds__(SORT_THREADS) k_sort_fix_long(const Cluster *__restrict__ cls, Tiles tm,
                                                                SortBufs sb, Fields f, unsigned int *tickets)
{
    __shared__ int s_last;
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (counts_ok(C) && sb.shift[ct.x] != 0) sort_long_runs(C, ct, tm, sb, f, tickets != nullptr);
    // the step's sort: the cluster's last block commits the new star count
    if (tickets && block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last) && threadIdx.x == 0)
        sort_commit(C.sc);
}

// Payload gather into radial order (ComputeIntermediateEnergy transfer +
// post_sort_comm), each star placed within its run (run_place).  Writes the
// second buffers of r, m, id, ec_pre, which the host then swaps with the first.
template <int GT>
__global__ void __launch_bounds__(GT) k_sort_gather(const Cluster *__restrict__ cls, Tiles tm, Fields f, SortBufs sb)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long nb = sc->n_bound;
    const int np = sb.npass[ct.x];
    const long long i = (long long)ct.y * GT + threadIdx.x;  // 0-based sorted position
    const long long off = C.off;
    if (nb < 0 || nb > sc->N_MAX_NEW) {
        if (i == 0) set_error(sc, CMCG_ERR_BOUNDS, nb);
        return;
    }
    if (i < nb) {
        if (np == 0) {
            move_star(C, f, (unsigned int)i, i);
        } else {
            const int sel = np & 1;
            const unsigned int v = (sel ? sb.vals[1] : sb.vals[0])[off + i];
            const int sh = sb.shift[ct.x];
            // bound stars sort before the escapers' run, so their runs end by nb
            const long long dst = sh == 0 ? i
                                          : run_place((sel ? sb.keys[1] : sb.keys[0]) + off, i, nb, sh,
                                                      sb.nlong + ct.x, sb.lstart + off / 32 + 64 * ct.x);
            if (dst >= 0) move_star(C, f, v, dst);
        }
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

void launch_sort_gather(int block, int ntiles, cudaStream_t s, const Cluster *cls, Tiles tm, Fields f, SortBufs sb)
{
    if (block == 128)
        k_sort_gather<128><<<ntiles, 128, 0, s>>>(cls, tm, f, sb);
    else if (block == 1024)
        k_sort_gather<1024><<<ntiles, 1024, 0, s>>>(cls, tm, f, sb);
    else
        k_sort_gather<256><<<ntiles, 256, 0, s>>>(cls, tm, f, sb);
}

}  // namespace cmcg
