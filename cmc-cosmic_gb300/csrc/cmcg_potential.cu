// cmcg_potential.cu -- potential_calculate (cmc_utils.c:675-736), first pass:
// approximate values of its three running quantities, from a parallel scan.
// cmcg_phi.cu turns them into the reference's exact FP64 results.
//
// The reference walks k = N..1 with
//     Phi_k = Phi_{k+1} - M_k (1/r_k - 1/r_{k+1}),   M_{k-1} = M_k - m_k/N_STAR,
// starting from M_N = Mtotal.  Written as sums:
//     M_k   = Mtotal - sum_{j>k} q_j,                 q_j = m_j / N_STAR
//     Phi_k = -sum_{j>=k} M_j d_j,                    d_j = 1/r_j - 1/r_{j+1}
// Tiles of 1024 stars are taken from the outside in.  A tile's effect on the
// running (Q, D) = (sum q, sum M d) is linear in the Q entering it, so each
// tile is summarised by (q_T, Delta_T, C_T) = (sum q, sum d, sum Qin_p d_p)
// with the associative combine (outer A, inner B) ->
//     (q_A + q_B, Delta_A + Delta_B, C_A + C_B + q_A Delta_B),
// and the D entering a tile is Mtotal * Delta_before - C_before.
//   k_pot_agg    per tile: q_j, 1/r_j (stored), the triple, sum m_j, and a
//                flag for input the exact replay does not take (radii out of
//                order, non-finite or negative values)
//   k_pot_carry  per cluster: approximate Mtotal, the bounds the replay
//                classifies with, scan of the triples over tiles
//   (k_phi_cls12, cmcg_phi.cu, then forms each tile's approximate forward
//   mass sums, M_k and Phi_k from these carries before classifying them)
#include "cmcg_kernels.cuh"

namespace cmcg {


__global__ void __launch_bounds__(POT_THREADS) k_pot_agg(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                          PotBufs pb)
{
    __shared__ double s_w[POT_THREADS / 32];
    __shared__ double s_lastinv[POT_THREADS / 32];
    __shared__ double s_S[POT_THREADS / 32][4];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, off = C.off;
    const double NSTAR = (double)sc->N_STAR;
    const long long kstart = N - (long long)ct.y * POT_T;  // largest k of this tile
    const double *r = f.r + off, *m = f.m + off;
    double q[POT_ITEMS], inv[POT_ITEMS], mm[POT_ITEMS];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int bad = 0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kstart - POT_ITEMS * t - i;
        if (k >= 1) {
            mm[i] = m[k];
            const double rk = r[k];
            q[i] = div_rcp(mm[i], NSTAR, sc->madhoc);  // m_k / N_STAR (madhoc = RN(1/N_STAR))
            inv[i] = __drcp_rn(rk);
            pb.q[off + k] = q[i];
            f.inv_r[off + k] = inv[i];
            // !(m >= 0) || !(m < inf) || !(r > 0) || !(r < SF_INFINITY) || !(1/r < inf), decided on
            // the bit patterns with integer instructions (FP64 comparisons take the scarce FP64 pipe):
            // m is +-0 or positive finite, r lies strictly between 0 and SF_INFINITY, 1/r is finite
            const unsigned long long bm = dbits(mm[i]), br = dbits(rk), bi = dbits(inv[i]);
            if (!((bm < INF_BITS || bm == SIGN_BIT) && (long long)br > 0 && br < dbits(CMCG_SF_INFINITY) &&
                  bi < INF_BITS))
                bad = 1;
        } else {
            mm[i] = q[i] = inv[i] = 0.0;
        }
    }
    // inv of k+1 for item 0 comes from the previous thread's item 3
    double up = __shfl_up_sync(0xffffffffu, inv[POT_ITEMS - 1], 1);
    if (lane == 31) s_lastinv[w] = inv[POT_ITEMS - 1];
    __syncthreads();
    if (lane == 0) up = (w > 0) ? s_lastinv[w - 1] : pot_r_next_inv(r, kstart, N);
    double d[POT_ITEMS];
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        const long long k = kstart - POT_ITEMS * t - i;
        const double innext = (i == 0) ? up : inv[i - 1];
        d[i] = (k >= 1) ? inv[i] - innext : 0.0;
        // radii out of order: !(d >= 0), i.e. d neither +-0 nor positive (infinity included)
        const unsigned long long bd = dbits(d[i]);
        if (k >= 1 && !((bd & ~SIGN_BIT) == 0 || bd <= INF_BITS)) bad = 1;
    }
    bad = __syncthreads_or(bad);
    // exclusive prefix of q in processing order -> C = sum Qexcl * d
    double tq = 0.0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) tq += q[i];
    const double qex = pot_block_excl_prefix<POT_THREADS>(tq, s_w);
    double run = qex, tc = 0.0, td = 0.0, tm_ = 0.0;
#pragma unroll
    for (int i = 0; i < POT_ITEMS; ++i) {
        tc += run * d[i];
        run += q[i];
        td += d[i];
        tm_ += mm[i];
    }
    double S[4] = {tq, td, tc, tm_};
    block_sums<POT_THREADS>(S, s_S);
    if (t == 0) {
        double *a = pb.agg + (size_t)blockIdx.x * POT_AGG;
        a[0] = S[0];
        a[1] = S[1];
        a[2] = S[2];
        a[3] = S[3];
        a[4] = bad ? 1.0 : 0.0;
    }
}

// One block per cluster: approximate Mtotal, the replay's error bounds and
// the carries entering each tile.
//
// Bounds (u = 2^-53 the unit roundoff, n = N, G = (tiles + 4096) 2^-52, which
// exceeds twice the error factor gamma of every summation depth these scans
// use):
//   chain 1, S_k = S_{k-1} + m_k: the sequential value drifts from the exact
//     sum by at most (n+2) u Am (each step rounds by at most u |S| <= u Am,
//     Am >= sum m); the scan's value S~_k errs by at most 2 G Am.
//   Mtotal = S_N madhoc + cenma madhoc: |exact - approximate| <= dM0.
//   chain 2, M_{k-1} = M_k - q_k, start Mtotal: drift (n+2) u Mb with
//     Mb >= every |M_k|, start error dM0, scan error 2 G (Mb + sum q).
// Each bound carries a factor 1.01 over the sum of its terms.
__global__ void __launch_bounds__(POT_THREADS) k_pot_carry(const Cluster *__restrict__ cls, Tiles tm, PotBufs pb,
                                                            PhiBufs ph, int nclusters)
{
    __shared__ double s_a[POT_THREADS][4];
    __shared__ double s_tot[4];
    const int c = blockIdx.x;
    if (c >= nclusters) return;
    const Cluster &C = cls[c];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const int ntiles = tm.count[c], b0 = tm.first[c];
    const long long N = sc->N_MAX;
    const int t = threadIdx.x;
    const int per = (ntiles + POT_THREADS - 1) / POT_THREADS;
    const int lo = t * per, hi = min(ntiles, lo + per);
    // chunk aggregate (outer tiles first) and mass sum
    double q = 0.0, D = 0.0, Cc = 0.0, sm = 0.0;
    int bad = 0;
    for (int i = lo; i < hi; ++i) {
        const double *a = pb.agg + (size_t)(b0 + i) * POT_AGG;
        Cc = Cc + a[2] + q * a[1];
        q += a[0];
        D += a[1];
        sm += a[3];
        bad |= a[4] != 0.0;
    }
    s_a[t][0] = q;
    s_a[t][1] = D;
    s_a[t][2] = Cc;
    s_a[t][3] = sm;
    bad = __syncthreads_or(bad);
    PhiCtl &ctl = ph.ctl[c];
    // exclusive scan of the chunk aggregates over threads: the triple combine
    // (outer A, inner B) -> (q_A + q_B, D_A + D_B, C_A + C_B + q_A D_B) is
    // associative, so a warp-shuffle scan and a pass over the warp totals do it
    {
        const int lane = t & 31, wid = t >> 5;
        double xq = q, xD = D, xC = Cc, xm = sm;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double yq = __shfl_up_sync(0xffffffffu, xq, o), yD = __shfl_up_sync(0xffffffffu, xD, o);
            const double yC = __shfl_up_sync(0xffffffffu, xC, o), ym = __shfl_up_sync(0xffffffffu, xm, o);
            if (lane >= o) {
                xC = yC + xC + yq * xD;
                xq = yq + xq;
                xD = yD + xD;
                xm = ym + xm;
            }
        }
        __shared__ double s_wt[POT_THREADS / 32][4];
        if (lane == 31) {
            s_wt[wid][0] = xq;
            s_wt[wid][1] = xD;
            s_wt[wid][2] = xC;
            s_wt[wid][3] = xm;
        }
        __syncthreads();
        double pq = 0.0, pD = 0.0, pC = 0.0, pm = 0.0;  // warps before this one
        for (int u = 0; u < wid; ++u) {
            pC = pC + s_wt[u][2] + pq * s_wt[u][1];
            pq += s_wt[u][0];
            pD += s_wt[u][1];
            pm += s_wt[u][3];
        }
        // exclusive: the earlier warps, then the lanes before this one (previous lane's inclusive)
        double eq_ = __shfl_up_sync(0xffffffffu, xq, 1), eD_ = __shfl_up_sync(0xffffffffu, xD, 1);
        double eC_ = __shfl_up_sync(0xffffffffu, xC, 1), em_ = __shfl_up_sync(0xffffffffu, xm, 1);
        if (lane == 0) eq_ = eD_ = eC_ = em_ = 0.0;
        __syncthreads();
        s_a[t][0] = pq + eq_;
        s_a[t][1] = pD + eD_;
        s_a[t][2] = pC + eC_ + pq * eD_;
        s_a[t][3] = pm + em_;
        if (t == POT_THREADS - 1) {
            s_tot[0] = pq + xq;
            s_tot[1] = pD + xD;
            s_tot[2] = pC + xC + pq * xD;
            s_tot[3] = pm + xm;
        }
    }
    __syncthreads();
    if (t == 0) {
        const double eq = s_tot[0], eD = s_tot[1], em = s_tot[3];
        const double u = 0x1p-53, n = (double)N;
        const double G = ((double)ntiles + 4096.0) * 0x1p-52;
        const double madhoc = sc->madhoc, cm = __dmul_rn(sc->cenma_m, madhoc);
        const double Mapx = __dadd_rn(__dmul_rn(em, madhoc), cm);
        const double Am = em * (1.0 + 2.0 * G);
        const double marg1 = 1.01 * ((n + 2.0) * u * Am + 2.0 * G * Am);
        const double dM0 = 1.01 * marg1 * madhoc + 0x1p-50 * (fabs(Mapx) + fabs(cm));
        const double Mb = (fabs(Mapx) + dM0) * (1.0 + 0x1p-40);
        const double Qb = eq * (1.0 + 2.0 * G);
        ctl.Sm = em;
        ctl.Qtot = eq;
        ctl.Dtot = eD;
        ctl.Mapx = Mapx;
        ctl.Mb = Mb;
        ctl.G = G;
        ctl.marg1 = marg1;
        ctl.marg2 = 1.01 * ((n + 2.0) * u * Mb + dM0 + 2.0 * G * (Mb + Qb));
        ctl.c0 = ctl.c1 = 0.0;
        ctl.fail = (bad || C.phi_sequential) ? 1 : 0;
        ctl.disorder = bad ? 1 : 0;
        ctl.nsp[0] = ctl.nsp[1] = ctl.nsp[2] = 0;
    }
    __syncthreads();
    const double Mtot = ctl.Mapx;
    double eq = s_a[t][0], eD = s_a[t][1], eC = s_a[t][2], em = s_a[t][3];
    for (int i = lo; i < hi; ++i) {
        const double *a = pb.agg + (size_t)(b0 + i) * POT_AGG;
        double *cr = pb.carry + (size_t)(b0 + i) * POT_CARRY;
        cr[0] = eq;
        cr[1] = Mtot * eD - eC;
        cr[2] = em;
        eC = eC + a[2] + eq * a[1];
        eq += a[0];
        eD += a[1];
        em += a[3];
    }
}

}  // namespace cmcg
