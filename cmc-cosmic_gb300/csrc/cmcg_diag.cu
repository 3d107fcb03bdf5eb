// cmcg_diag.cu -- the per-step quantities of dyn.dat and lagrad.dat.
//
// The reference computes, every step, from the sorted stars:
//   central_calculate (cmc_utils.c:1239-1345): the index just beyond the
//     half-mass radius, Casertano & Hut (1985) local densities rho_j over the
//     J = 6 neighbours of every star out to it, and density-weighted averages
//     (core density, rms velocity, core radius, rc_nb, mean mass);
//   clusdyn_calculate (cmc_utils.c:1613-1624): the half-mass radius;
//   comp_mass_percent (cmc_utils.c:872-968): for each mass fraction, the first
//     star at which the forward mass sum exceeds it (at most one fraction per
//     star), with the running kinetic sums there.
// Here, over the cluster's 1024-star tiles:
//   k_diag_sum      per-tile sums of the five running columns
//   k_diag_carry    their exclusive scan over tiles (one block)
//   k_diag_prefix   per-star running sums
//   k_diag_find     the half-mass star and each fraction's first crossing, by
//                   binary search over them (one block)
//   k_diag_central  rho_j and the weighted sums out to the half-mass index;
//                   its last block finishes: averages, the one-fraction-per-
//                   star rule, the values at each assigned star
// The per-star terms are the reference's expressions; the sums are taken by
// tiles and trees, so they agree with the reference's sequential loops to a
// few ulps of their magnitude, and the crossing stars agree unless a
// fraction lies within that of a running sum.
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {

namespace {

constexpr int DG_THREADS = POT_THREADS, DG_ITEMS = POT_ITEMS, DG_T = POT_T;

__device__ __forceinline__ double sqr(double x) { return x * x; }
__device__ __forceinline__ double cub(double x) { return x * x * x; }

// the five running terms of star k (comp_mass_percent, cmc_utils.c:905-908, 931)
__device__ __forceinline__ void star_terms(const Fields &f, long long g, double NSTAR, double madhoc,
                                           double t[DIAG_COLS])
{
    const double m = f.m[g], vr = f.vr[g], vt = f.vt[g];
    t[0] = div_rcp(m, NSTAR, madhoc);  // star_m[k] / clus.N_STAR
    t[1] = 0.5 * m * madhoc * vr * vr;
    t[2] = 0.5 * m * madhoc * vt * vt;
    t[3] = vr * vr;
    t[4] = vt * vt;
}

// exclusive prefix of each thread's value over the block (warp shuffles, then warps in order)
template <int K>
__device__ __forceinline__ void block_excl(double (&v)[K], double (*s_w)[K])
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double x[K];
#pragma unroll
    for (int c = 0; c < K; ++c) x[c] = v[c];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int c = 0; c < K; ++c) {
            const double y = __shfl_up_sync(0xffffffffu, x[c], o);
            if (lane >= o) x[c] += y;
        }
    }
    __syncthreads();
    if (lane == 31) {
#pragma unroll
        for (int c = 0; c < K; ++c) s_w[w][c] = x[c];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < K; ++c) {
        double b = 0.0;
        for (int q = 0; q < w; ++q) b += s_w[q][c];
        v[c] = b + x[c] - v[c];
    }
}

}  // namespace

__global__ void __launch_bounds__(DG_THREADS) k_diag_sum(const Cluster *__restrict__ cls, Tiles tm, Fields f, int b0,
                                                          double *partials)
{
    __shared__ double s_S[DG_THREADS / 32][DIAG_COLS];
    const int b = b0 + blockIdx.x;
    const int2 ct = tm.tiles[b];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const Scalars *sc = C.sc;
    const long long N = sc->N_MAX;
    const double NSTAR = (double)sc->N_STAR, madhoc = sc->madhoc;
    double S[DIAG_COLS] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < DG_ITEMS; ++i) {
        const long long k = 1 + (long long)ct.y * DG_T + DG_ITEMS * threadIdx.x + i;
        if (k <= N) {
            double t[DIAG_COLS];
            star_terms(f, C.off + k, NSTAR, madhoc, t);
#pragma unroll
            for (int c = 0; c < DIAG_COLS; ++c) S[c] += t[c];
        }
    }
    block_sums<DG_THREADS>(S, s_S);
    if (threadIdx.x == 0)
        for (int c = 0; c < DIAG_COLS; ++c) partials[(size_t)b * (DIAG_COLS + DIAG_CCOLS) + c] = S[c];
}

// One block: the tiles' sums become the sums of the tiles before each, in order.
__global__ void __launch_bounds__(DG_THREADS) k_diag_carry(const Cluster *__restrict__ cls, Tiles tm, int c, int b0,
                                                            int nt, double *partials)
{
    __shared__ double s_w[DG_THREADS / 32][DIAG_COLS];
    if (!counts_ok(cls[c])) return;
    constexpr int W = DIAG_COLS + DIAG_CCOLS;
    const int per = (nt + DG_THREADS - 1) / DG_THREADS;
    const int t0 = threadIdx.x * per, t1 = min(nt, t0 + per);
    double v[DIAG_COLS] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t = t0; t < t1; ++t)
        for (int q = 0; q < DIAG_COLS; ++q) v[q] += partials[(size_t)(b0 + t) * W + q];
    block_excl<DIAG_COLS>(v, s_w);
    for (int t = t0; t < t1; ++t) {
        for (int q = 0; q < DIAG_COLS; ++q) {
            double *p = partials + (size_t)(b0 + t) * W + q;
            const double x = *p;
            *p = v[q];
            v[q] += x;
        }
    }
}

__global__ void __launch_bounds__(DG_THREADS) k_diag_prefix(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                             int b0, const double *partials, DiagScratch ds)
{
    __shared__ double s_w[DG_THREADS / 32][DIAG_COLS];
    const int b = b0 + blockIdx.x;
    const int2 ct = tm.tiles[b];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const Scalars *sc = C.sc;
    const long long N = sc->N_MAX, off = C.off;
    const double NSTAR = (double)sc->N_STAR, madhoc = sc->madhoc;
    double t[DG_ITEMS][DIAG_COLS], v[DIAG_COLS] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < DG_ITEMS; ++i) {
        const long long k = 1 + (long long)ct.y * DG_T + DG_ITEMS * threadIdx.x + i;
        if (k <= N) {
            star_terms(f, off + k, NSTAR, madhoc, t[i]);
        } else {
#pragma unroll
            for (int c = 0; c < DIAG_COLS; ++c) t[i][c] = 0.0;
        }
#pragma unroll
        for (int c = 0; c < DIAG_COLS; ++c) v[c] += t[i][c];
    }
    block_excl<DIAG_COLS>(v, s_w);
    const double *cr = partials + (size_t)b * (DIAG_COLS + DIAG_CCOLS);
    double run[DIAG_COLS];
#pragma unroll
    for (int c = 0; c < DIAG_COLS; ++c) run[c] = cr[c] + v[c];
#pragma unroll
    for (int i = 0; i < DG_ITEMS; ++i) {
        const long long k = 1 + (long long)ct.y * DG_T + DG_ITEMS * threadIdx.x + i;
        if (k > N) break;
#pragma unroll
        for (int c = 0; c < DIAG_COLS; ++c) {
            run[c] += t[i][c];
            ds.col[c][off + k] = run[c];
        }
    }
}

// One block: the half-mass star (the first whose mass sum reaches half the
// mass: clusdyn_calculate's and central_calculate's loops) and, for each
// fraction, the first star whose sum from the central mass exceeds it
// (comp_mass_percent), by binary search over the stored running sums.
__global__ void __launch_bounds__(DG_THREADS) k_diag_find(const Cluster *__restrict__ cls, Fields f, int c,
                                                           DiagScratch ds, DiagDev *dd)
{
    const Cluster &C = cls[c];
    if (!counts_ok(C)) return;
    const Scalars *sc = C.sc;
    const long long N = sc->N_MAX;
    const double *F = ds.col[0] + C.off;
    const double Mtotal = sc->Mtotal;
    const double mprev0 = dd->bh_include ? sc->cenma_m * sc->madhoc : 0.0;
    const int q = (int)threadIdx.x - 1;  // thread 0: half mass; thread q + 1: fraction q
    if (q >= dd->n_pc) return;
    long long lo = 1, hi = N + 1;  // first k in [1, N] passing, N + 1 if none
    if (q < 0) {
        const double half = 0.5 * Mtotal;
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if (F[mid] >= half)
                hi = mid;
            else
                lo = mid + 1;
        }
        dd->jhalf = lo <= N ? lo : 0;
    } else {
        const double T = dd->pc[q] * Mtotal;
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if (mprev0 + F[mid] > T)
                hi = mid;
            else
                lo = mid + 1;
        }
        dd->first[q] = lo <= N ? lo : 0;
    }
}

__global__ void __launch_bounds__(DG_THREADS) k_diag_central(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                              int c, int b0, int nt, double *partials,
                                                              unsigned int *tickets, DiagScratch ds, DiagDev *dd)
{
    __shared__ double s_S[DG_THREADS / 32][DIAG_CCOLS];
    __shared__ int s_last;
    constexpr int W = DIAG_COLS + DIAG_CCOLS;
    const int b = b0 + blockIdx.x;
    const int2 ct = tm.tiles[b];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, off = C.off;
    const double madhoc = sc->madhoc;
    const double *r = f.r + off, *m = f.m + off;
    const long long J = 6;
    const long long nave = dd->jhalf + 1;  // the reference's loop index after it stops
    double S[DIAG_CCOLS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (dd->jhalf > 0 && nave < sc->N_STAR - 6 && nave + J <= N + 1) {
#pragma unroll
        for (int it = 0; it < DG_ITEMS; ++it) {
            const long long i = 1 + (long long)ct.y * DG_T + DG_ITEMS * threadIdx.x + it;
            if (i > nave) break;
            // rho_j, Eq. II.2 of Casertano & Hut (cmc_utils.c:1262-1272)
            const long long jmin = (i - J / 2 > 1) ? i - J / 2 : 1, jmax = jmin + J;
            double mrho = 0.0;
            for (long long j = jmin + 1; j <= jmax - 1; j++) mrho += m[j] * madhoc;
            const double Vrj = 4.0 / 3.0 * CMCG_PI * (cub(r[jmax]) - cub(r[jmin]));
            const double rhoj = mrho / Vrj;
            const double vr = f.vr[off + i], vt = f.vt[off + i];
            S[0] += rhoj;                          // rhojsum
            S[1] += sqr(rhoj);                     // rhoj2sum and central.rho
            S[2] += rhoj * (sqr(vr) + sqr(vt));    // central.v_rms
            S[3] += rhoj * r[i];                   // central.rc
            S[4] += sqr(rhoj * r[i]);              // rc_nb
            S[5] += rhoj * m[i] * madhoc;          // central.m_ave
        }
    }
    block_sums<DG_THREADS>(S, s_S);
    if (threadIdx.x == 0)
        for (int q = 0; q < DIAG_CCOLS; ++q) partials[(size_t)b * W + DIAG_COLS + q] = S[q];
    if (!block_arrive_last(tickets + c, nt, &s_last)) return;
    // last block: the tiles' sums in order
    double A[DIAG_CCOLS] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int t = threadIdx.x; t < nt; t += DG_THREADS)
        for (int q = 0; q < DIAG_CCOLS; ++q) A[q] += __ldcg(partials + (size_t)(b0 + t) * W + DIAG_COLS + q);
    __syncthreads();
    block_sums<DG_THREADS>(A, s_S);
    if (threadIdx.x != 0) return;
    if (dd->jhalf <= 0 || sc->N_STAR <= 2 * J || nave >= sc->N_STAR - 6 || nave + J > N + 1) {
        dd->status = CMCG_ERR_STATE;  // cmc_utils.c:1254: the reference exits here
        return;
    }
    dd->nave = nave;
    dd->rh = r[nave];  // clusdyn_calculate: star_r[k] after its loop stops
    double rho = A[1] / A[0];
    rho *= 4.0 / 5.0;
    rho *= 2.0;
    const double v_rms = sqrt(A[2] / A[0]), rc = A[3] / A[0], rc_nb = sqrt(A[4] / A[1]), m_ave = A[5] / A[0];
    dd->rho = rho;
    dd->v_rms = v_rms;
    dd->rc = rc;
    dd->rc_nb = rc_nb;
    dd->m_ave = m_ave;
    dd->n = rho / m_ave;
    dd->rc_spitzer = sqrt(3.0 * sqr(v_rms) / (4.0 * CMCG_PI * rho));
    dd->N_core = 4.0 / 3.0 * CMCG_PI * cub(rc) * (dd->n / 2.0);
    dd->N_core_nb = 4.0 / 3.0 * CMCG_PI * cub(rc_nb) * (dd->n / 2.0);
    dd->Trc = 0.065 * cub(v_rms) / (rho * m_ave);
    // comp_mass_percent: fractions the central mass already exceeds take
    // MINIMUM_R; then each fraction at the first star past it, at most one
    // fraction per star
    const double Mtotal = sc->Mtotal;
    const double mprev0 = dd->bh_include ? sc->cenma_m * madhoc : 0.0;
    int mc = 0;
    if (dd->bh_include)
        while (mc < dd->n_pc && mprev0 / Mtotal > dd->pc[mc]) dd->mass_r[mc++] = dd->minimum_r;
    long long kprev = 0;
    for (; mc < dd->n_pc; ++mc) {
        long long k = dd->first[mc];
        if (k <= 0) break;  // the sum never passes this fraction
        if (k <= kprev) k = kprev + 1;
        if (k > N) break;
        const double mprev = mprev0 + ds.col[0][off + k];
        dd->mass_r[mc] = r[k];
        dd->ave_mass_r[mc] = mprev / Mtotal / k * 1.0;  // initial_total_mass = 1 (cmc_utils.c:1904)
        dd->no_star_r[mc] = (double)k;
        dd->densities_r[mc] = mprev / (4.0 / 3.0 * CMCG_PI * pow(r[k], 3));
        dd->ke_rad_r[mc] = ds.col[1][off + k];
        dd->ke_tan_r[mc] = ds.col[2][off + k];
        dd->v2_rad_r[mc] = ds.col[3][off + k];
        dd->v2_tan_r[mc] = ds.col[4][off + k];
        kprev = k;
    }
    dd->n_set = mc;
    dd->status = 0;  // staged as CMCG_ERR_STATE by the host: a finish that never ran reads as an error
}

}  // namespace cmcg
