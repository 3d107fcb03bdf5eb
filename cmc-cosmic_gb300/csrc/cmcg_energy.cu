// cmcg_energy.cu -- step bookkeeping on the device.
//
// k_begin_step   cmc.c:246-257 (tallies of the previous step move to *_old);
//                a whole step does this in k_timestep's last block
// k_ec3 + k_ec3_fix   set_velocities3 (cmc_utils.c:254-349).  The per-star
//     prediction v_new^2 = vold^2 + (Uoldrold - Uoldrnew) + (Unewrold - Unewrnew)
//     and the velocity rescaling are independent per star (k_ec3).  Only the
//     "excess energy" carried from stars whose prediction is unphysical to the
//     stars after them is sequential; such stars are rare, so k_ec3 records
//     them in a list and k_ec3_fix replays exactly the reference's sequential
//     loop from each of them until the excess is used up.
// k_energy       compute_energy_new + ComputeEnergy (cmc_utils.c:2018-2028, 604-656)
// k_end_step     tcount++, Prev_Dt (cmc.c:294, 390); a whole step does this
//                in k_energy's last block
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {


static __device__ __forceinline__ double sqr(double x) { return x * x; }

__global__ void k_begin_step(const Cluster *__restrict__ cls, int nclusters)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nclusters) return;
    begin_step(cls[c]);
}

__global__ void k_end_step(const Cluster *__restrict__ cls, int nclusters)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nclusters) return;
    end_step(cls[c].sc);
}


__global__ void __launch_bounds__(EC3_T) k_ec3(const Cluster *__restrict__ cls, Tiles tm, Fields f, Ec3Bufs eb,
                                               double *const *hx)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long i = 1 + (long long)ct.y * EC3_T + threadIdx.x;
    const long long off = C.off, g = off + i;
    if (i > sc->N_MAX_NEW) return;
    const double invN = sc->madhoc;  // 1.0 / N_STAR (cmc_utils.c:1183)
    const double m = f.m[g], ri = f.r[g], rold = f.rOld[g];
    int pok = 1;
    // PHI_S (cmc.h:2175) by the stored 1/r_i, or by the 1/r_old the potential lookup forms anyway (div_rcp)
    const double iri = f.inv_r[g];
    const double phis_i = __dmul_rn(div_rcp(m, ri, iri), invN);
    double Unewrold;
    const double *rt = f.r + off, *pt = f.phi + off, *it = f.inv_r + off;
    if (gt0(rold) && ge_pos(rold, rt[1])) {  // rold > 0 && rold >= r_1 (r_1 > 0)
        const double iro = __drcp_rn(rold);
        Unewrold = potential_in(rt, pt, it, sc->N_MAX, rold, potential_index(rt, sc->N_MAX, rold, ridx_of(C, f)), &pok,
                                iro) +
                   (ge_pos(rold, ri) ? __dmul_rn(div_rcp(m, rold, iro), invN) : phis_i);
    } else {
        Unewrold = potential_at(rt, pt, it, sc->N_MAX, rold, &pok, ridx_of(C, f)) + phi_s(rold, ri, m, invN);
    }
    if (!pok) set_error(sc, CMCG_ERR_FINDZERO_R, i);
    const double Unewrnew = f.phi[g] + phis_i;
    const double q = 0.5;
    const double vnew2 = f.ec_pre[g] + 2.0 * q * (Unewrold - Unewrnew);
    double vr = f.vr[g], vt = f.vt[g];
    if (le0(vnew2)) {
        eb.a[g] = 0.5 * (sqr(vr) + sqr(vt) - vnew2) * m;
        const unsigned int slot = atomicAdd(eb.nlist + ct.x, 1u);
        if (slot < EXCESS_CAP) eb.list[(size_t)ct.x * EXCESS_CAP + slot] = i;
    } else {
        eb.a[g] = -1.0;
        // alpha = sqrt(vnew2 / v^2) (cmc_utils.c:291) as vnew2 rsqrt(vnew2 v^2): one
        // reciprocal square root instead of a division and a square root, within
        // 4 ulps of the reference's value
        const double v2 = sqr(vr) + sqr(vt);
        const double alpha = vnew2 * rsqrt(vnew2 * v2);
        vr *= alpha;
        vt *= alpha;
        f.vr[g] = vr;
        f.vt[g] = vt;
    }
    if (hx) {  // the caller's copy; k_ec3_fix rewrites the stars it changes
        hx[4 * ct.x][i - 1] = vr;
        hx[4 * ct.x + 1][i - 1] = vt;
        // J = r vt as compute_energy_new forms it (cmc_utils.c:604-617), sent
        // here so that it crosses the host link while this kernel runs
        hx[4 * ct.x + 3][i - 1] = ri * vt;
    }
}

// One segment of set_velocities3's loop (cmc_utils.c:270-307): entering
// listed star i0 with excess E (that star's own addition included), each
// following star up to `end` (the next listed star, or N_MAX_NEW + 1) gives
// up min(0.8 KE, excess) while the excess is positive.  Returns the excess
// left on reaching `end`, 0 once it is used up.  WRITE applies the changes.
template <bool WRITE>
static __device__ double ec3_walk(const Fields &f, long long off, long long i0, long long end, double E,
                                  double *hvr = nullptr, double *hvt = nullptr, double *hJ = nullptr)
{
    const double E_dump_factor = 0.8;
    for (long long i = i0 + 1; i < end && E > 0; ++i) {
        const long long g = off + i;
        const double m = f.m[g], vr = f.vr[g], vt = f.vt[g];
        const double v2 = sqr(vr) + sqr(vt);
        const double E_dump_capacity = E_dump_factor * 0.5 * m * v2;
        const double E_dump = (E_dump_capacity <= E) ? E_dump_capacity : E;
        if (WRITE) {
            const double exc_ratio = sqrt((v2 - 2 * E_dump / m) / v2);
            f.vr[g] = vr * exc_ratio;
            f.vt[g] = vt * exc_ratio;
            if (hvr) {
                hvr[i - 1] = vr * exc_ratio;
                hvt[i - 1] = vt * exc_ratio;
                hJ[i - 1] = f.r[g] * (vt * exc_ratio);
            }
        }
        E -= E_dump;
    }
    return E;
}

// One block per cluster.  The listed stars (unphysical predictions, which add
// excess) are put in radial order with a shared-memory bitonic sort; they cut
// the sequential loop into segments that start at a listed star and end
// before the next one.  The only thing one segment passes to the next is the
// excess still left at its end, which is almost always zero, so:
//   1. every segment is walked in parallel as if nothing were carried into it,
//      recording what it would carry out;
//   2. one thread carries the excess through the segments in order, walking
//      again only the segments that really receive some;
//   3. every segment is walked in parallel with the excess it really receives,
//      and writes.
// Each segment performs the reference's operations in the reference's order,
// so the result is the sequential loop's.  Beyond the list's capacity the
// whole sequential loop is replayed by one thread, reading windows of
// FIX_WINDOW consecutive stars that the block stages in shared memory.
__global__ void __launch_bounds__(EC3_FIX_THREADS) k_ec3_fix(const Cluster *__restrict__ cls, Fields f, Ec3Bufs eb,
                                                             int nclusters, double *const *hx)
{
    __shared__ __align__(16) int L[EXCESS_CAP];  // star indices (below 2^31: counts_ok bounds them by the capacity)
    __shared__ long long s_i;
    __shared__ double s_exc;
    __shared__ int s_done;
    const int c = blockIdx.x;
    if (c >= nclusters) return;
    const Cluster &C = cls[c];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long off = C.off, N = sc->N_MAX_NEW;
    double *hvr = hx ? hx[4 * c] : nullptr, *hvt = hx ? hx[4 * c + 1] : nullptr, *hJ = hx ? hx[4 * c + 3] : nullptr;
    const unsigned int n = eb.nlist[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        eb.nlist[c] = 0u;
        sc->n_excess = n;
    }
    if (n == 0) return;
    if (n <= EXCESS_CAP) {
        unsigned int P = 1;
        while (P < n) P <<= 1;
        const long long *G = eb.list + (size_t)c * EXCESS_CAP;
        for (unsigned int i = threadIdx.x; i < P; i += blockDim.x) L[i] = (i < n) ? (int)G[i] : INT_MAX;
        __syncthreads();
        for (unsigned int k = 2; k <= P; k <<= 1) {
            for (unsigned int jj = k >> 1; jj > 0; jj >>= 1) {
                for (unsigned int i = threadIdx.x; i < P; i += blockDim.x) {
                    const unsigned int l = i ^ jj;
                    if (l > i) {
                        const bool up = (i & k) == 0;
                        const int a = L[i], b = L[l];
                        if ((a > b) == up) {
                            L[i] = b;
                            L[l] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        double *carry = eb.carry + (size_t)c * EXCESS_CAP;
        const int nn = (int)n;
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            const long long i0 = L[t], end = (t + 1 < nn) ? L[t + 1] : N + 1;
            carry[t] = ec3_walk<false>(f, off, i0, end, eb.a[off + i0]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double cin = 0.0;  // excess entering segment t
            for (int t = 0; t < nn; ++t) {
                double cout = carry[t];
                if (cin > 0.0) {
                    const long long i0 = L[t], end = (t + 1 < nn) ? L[t + 1] : N + 1;
                    cout = ec3_walk<false>(f, off, i0, end, cin + eb.a[off + i0]);
                }
                carry[t] = cin;
                cin = cout;
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nn; t += blockDim.x) {
            const long long i0 = L[t], end = (t + 1 < nn) ? L[t + 1] : N + 1;
            ec3_walk<true>(f, off, i0, end, carry[t] + eb.a[off + i0], hvr, hvt, hJ);  // 0 + a = a when nothing is carried
        }
        return;
    }
    // overflow: the whole loop, one thread, staged windows
    double *wa = reinterpret_cast<double *>(L);  // 4 x FIX_WINDOW doubles fit in L's 16 KB
    double *wm = wa + FIX_WINDOW, *wvr = wm + FIX_WINDOW, *wvt = wvr + FIX_WINDOW;
    if (threadIdx.x == 0) {
        s_exc = 0.0;
        s_i = 1;
        s_done = 0;
    }
    __syncthreads();
    const double E_dump_factor = 0.8;
    // every window advances the walk by FIX_WINDOW stars
    for (long long guard = 0; guard <= N + 1; ++guard) {
        const long long i0 = s_i;
        if (s_done || i0 > N || i0 < 1) break;
        for (int k = threadIdx.x; k < FIX_WINDOW; k += blockDim.x) {
            const long long gi = i0 + k;
            if (gi <= N) {
                const long long g = off + gi;
                wa[k] = eb.a[g];
                wm[k] = f.m[g];
                wvr[k] = f.vr[g];
                wvt[k] = f.vt[g];
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double Eexcess = s_exc;
            long long i = i0;
            for (; i <= N && i < i0 + FIX_WINDOW; ++i) {
                const int k = (int)(i - i0);
                const double ai = wa[k];
                if (ai >= 0.0) {
                    Eexcess += ai;
                } else if (Eexcess > 0) {
                    const double m = wm[k];
                    double vr = wvr[k], vt = wvt[k];
                    const double v2 = sqr(vr) + sqr(vt);
                    const double E_dump_capacity = E_dump_factor * 0.5 * m * v2;
                    const double E_dump = (E_dump_capacity <= Eexcess) ? E_dump_capacity : Eexcess;
                    const double exc_ratio = sqrt((v2 - 2 * E_dump / m) / v2);
                    vr *= exc_ratio;
                    vt *= exc_ratio;
                    f.vr[off + i] = vr;
                    f.vt[off + i] = vt;
                    if (hvr) {
                        hvr[i - 1] = vr;
                        hvt[i - 1] = vt;
                        hJ[i - 1] = f.r[off + i] * vt;
                    }
                    Eexcess -= E_dump;
                }
            }
            s_exc = Eexcess;
            s_i = i;
            s_done = i > N;
        }
        __syncthreads();
    }
    // on one rank the remainder is dropped (cmc_utils.c:313-348)
}

// Eight stars per thread: the per-star FP64 work is the reference's
// expressions; the sums take one addition per star before the block tree.
__global__ void __launch_bounds__(EN_THREADS) k_energy(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                       double *partials, unsigned int *tickets, double *const *hx,
                                                       int end)
{
    __shared__ double red[EN_THREADS / 32];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, off = C.off;
    const double madhoc = sc->madhoc;
    // the central mass's share of PE, the same for every star (cmc_utils.c:633)
    const double pc = f.phi[off] * sc->cenma_m * madhoc / (double)N;
    // KE = sum 0.5 v^2 m madhoc and PE = sum (phi m madhoc + pc) (cmc_utils.c:623-633)
    // with the constant factors taken out of the sums: sum v^2 m and sum phi m
    // per star, 0.5 madhoc, madhoc and the stars' count times pc at the end
    // (two FP64 operations a star fewer for each; the sums are tree sums anyway)
    double K = 0.0, P = 0.0;
    int cnt = 0;
    // the caller's E (J went there from energy conservation, with the final vt)
    double *hE = hx ? hx[4 * ct.x + 2] : nullptr;
#pragma unroll 4
    for (int it = 0; it < EN_T / EN_THREADS; ++it) {
        const long long i = 1 + (long long)ct.y * EN_T + it * EN_THREADS + threadIdx.x;
        if (i > N) break;
        const long long g = off + i;
        const double vr = f.vr[g], vt = f.vt[g], ph = f.phi[g], m = f.m[g];
        const double v2 = sqr(vr) + sqr(vt);
        const double E = ph + 0.5 * v2, J = f.r[g] * vt;
        f.E[g] = E;
        f.J[g] = J;
        if (hE) hE[i - 1] = E;  // the caller's copy
        K += v2 * m;
        P += ph * m;
        ++cnt;
    }
    __shared__ double s_KP[EN_THREADS / 32][2];
    double KP[2] = {K, P};
    block_sums<EN_THREADS>(KP, s_KP);
    __shared__ int s_cnt[EN_THREADS / 32];
    const int bc = __reduce_add_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0) s_cnt[threadIdx.x >> 5] = bc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int n = 0;
        for (int q = 0; q < EN_THREADS / 32; ++q) n += s_cnt[q];
        KP[0] = 0.5 * madhoc * KP[0];
        KP[1] = madhoc * KP[1] + pc * (double)n;
    }
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        double *slot = partials + (size_t)blockIdx.x * 2;
        slot[0] = KP[0];
        slot[1] = KP[1];
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        const double sK = reduce_partials_sum<EN_THREADS>(partials, tm.first[ct.x], tm.count[ct.x], 2, 0, red);
        const double sP = reduce_partials_sum<EN_THREADS>(partials, tm.first[ct.x], tm.count[ct.x], 2, 1, red);
        if (threadIdx.x == 0) {
            double aK = sK, aP = sP;
            // compute_energy_new, cmc_utils.c:2020-2025
            sc->Eescaped += sc->Eescaped_old;
            sc->Jescaped += sc->Jescaped_old;
            sc->Etidal += sc->Etidal_old;
            aP *= 0.5;
            sc->KE = aK;
            sc->PE = aP;
            double tot = aK + aP + 0.0 + 0.0;
            tot += sc->cenma_E + sc->Eescaped + 0.0 + 0.0;
            sc->Etot = tot;
            if (end) end_step(sc);  // a whole step's last kernel: k_end_step's work
        }
    }
}

}  // namespace cmcg
