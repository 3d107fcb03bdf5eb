// cmcg_relax.cu -- time step and the fused relaxation kernel.
//
// k_timestep restates simul_relax_new (cmc_dynamics_helper.c:2526-2579) and
// calc_timestep (cmc_utils.c:2132-2148): the per-star terms are formed by all
// threads, then one thread per 2p-star window adds them in the reference's
// order, so Dt is bit-identical.
//
// k_relax restates dynamics_apply (cmc_dynamics.c:17-542, relaxation branch
// 427-497) with calc_encounter_dyns, calc_n_local and set_star_EJ
// (cmc_dynamics_helper.c:768-882) and calc_sigma_r (2821-2986) in one pass:
// a block owns 256 consecutive stars (128 neighbour pairs (2k-1, 2k) in the
// reference's 1-based numbering), stages m*v^2 and m of its stars plus a p-star
// halo in shared memory to form the sliding-window sigma, then relaxes its
// pairs.  Velocities after relaxation go to separate arrays so that no block
// ever reads a neighbour's updated velocities in its sigma halo.
#include "cmcg_fftrig.cuh"
#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {


static __device__ __forceinline__ double sqr(double x) { return x * x; }
static __device__ __forceinline__ double cub(double x) { return x * x * x; }

// r_max^3 - r_min^3 over the 2p neighbours of star k (calc_n_local's window,
// cmc_dynamics_helper.c:768-786)
static __device__ __forceinline__ double window_dr3(const double *__restrict__ r, long long k, long long p,
                                                    long long N_LIMIT)
{
    long long kmin = k - p, kmax = k + p;
    if (kmin < 0) {
        kmin = 0;
        kmax = 2 * p + 1;
    } else if (kmax > N_LIMIT) {
        kmax = N_LIMIT;
        kmin = N_LIMIT - 2 * p - 1;
    }
    return cub(r[kmax]) - cub(r[kmin]);
}

// calc_n_local, cmc_dynamics_helper.c:768-786
static __device__ __forceinline__ double n_local_at(const double *__restrict__ r, long long k, long long p,
                                                    long long N_LIMIT)
{
    return (2.0 * ((double)p)) * 3.0 / (4.0 * CMCG_PI * window_dr3(r, k, p, N_LIMIT));
}

// ------------------------------------------------------------ time step --
// A block owns the windows (2p stars each, centres si = 1 + p + 2 p w) whose
// centre lies in its 1024-star tile.  All threads form the per-star terms
// m/N (vr^2 + vt^2), m/N and (m/N)^2 of those windows' stars into shared
// memory; then one thread per window adds its terms in the reference's
// order, so every sum, and Dt, is bit-identical.
__global__ void __launch_bounds__(TS_THREADS) k_timestep(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                         double *partials, unsigned int *tickets, int begin)
{
    constexpr int LMAX = TS_T + 2 * PMAX;  // stars of the windows centred in one tile
    __shared__ double s_mv[LMAX], s_mm[LMAX], s_m2[LMAX];
    __shared__ double red[TS_THREADS / 32];
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, p = C.p;
    const double madhoc = sc->madhoc;
    const double *r = f.r + C.off, *m = f.m + C.off, *vr = f.vr + C.off, *vt = f.vt + C.off;
    double dtmin = INFINITY;
    if (C.RELAXATION && N >= 2 * p + 2) {
        // windows w with s_lo <= si < min(s_hi, N + 1 - p)
        const long long s_lo = 1 + (long long)ct.y * TS_T, s_hi = s_lo + TS_T;
        const long long lim = s_hi < N + 1 - p ? s_hi : N + 1 - p;
        const long long w0 = (s_lo - 1 - p <= 0) ? 0 : (s_lo - 1 - p + 2 * p - 1) / (2 * p);
        const long long w1 = (lim - 1 - p <= 0) ? -1 : (lim - 1 - p + 2 * p - 1) / (2 * p) - 1;
        const long long k0 = 1 + 2 * p * w0;  // first star of window w0
        const int L = w1 >= w0 ? (int)(2 * p * (w1 - w0 + 1)) : 0;
        for (int i = threadIdx.x; i < L; i += TS_THREADS) {
            const long long k = k0 + i;
            const double tmp = m[k] * madhoc;
            s_mv[i] = tmp * (sqr(vr[k]) + sqr(vt[k]));
            s_mm[i] = tmp;
            s_m2[i] = sqr(tmp);
        }
        __syncthreads();
        for (long long w = w0 + threadIdx.x; w <= w1; w += TS_THREADS) {
            const long long si = 1 + p + 2 * p * w;
            const int b = (int)(2 * p * (w - w0));
            double Mv2ave = 0.0, Mave = 0.0, M2ave = 0.0;
            for (int q = 0; q < 2 * p; ++q) {
                Mv2ave += s_mv[b + q];
                Mave += s_mm[b + q];
                M2ave += s_m2[b + q];
            }
            Mv2ave /= (double)(2 * p);
            Mave /= (double)(2 * p);
            M2ave /= (double)(2 * p);
            const double sigma = sqrt(Mv2ave / Mave);
            const double W = 4.0 * sigma / sqrt(3.0 * CMCG_PI);
            const double nl = n_local_at(r, si, p, N);
            const double dt = sqr(2.0 * C.THETASEMAX / CMCG_PI) * (CMCG_PI / 32.0) * cub(W) /
                              (((double)sc->N_STAR) * nl * (4.0 * M2ave));
            dtmin = fmin(dtmin, dt);
        }
    }
    // exact min over blocks (min is order independent)
    __shared__ int s_last;
    const double bmin = -block_max<TS_THREADS>(-dtmin, red);
    // min over blocks as the negated max of negated block minima (order independent)
    if (threadIdx.x == 0) partials[blockIdx.x] = -bmin;
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        const double Dtmin = -reduce_partials_max<TS_THREADS>(partials, tm.first[ct.x], tm.count[ct.x], 1, 0, red);
        if (threadIdx.x == 0) {
            // a whole step's first kernel: k_begin_step's work, before the
            // tallies below read it (no block reads what it changes)
            if (begin) begin_step(C);
            double Dt = C.RELAXATION ? Dtmin : INFINITY;
            // GetTimeStep, cmc_evolution_thr.c:420: all other time scales are infinite
            if (isinf(Dt)) Dt = 0.001;
            // calc_timestep, cmc_utils.c:2138-2144
            if ((sc->TidalMassLoss_old - sc->OldTidalMassLoss) > 0.01) {
                Dt = sc->Prev_Dt * 0.8;
            } else if (Dt > 1.1 * sc->Prev_Dt && sc->Prev_Dt > 0 &&
                       (sc->TidalMassLoss - sc->OldTidalMassLoss) > 0.02) {
                Dt = sc->Prev_Dt * 1.1;
            }
            sc->Dt = Dt;
            sc->TotalTime += Dt;
        }
    }
}

// ------------------------------------------------------------ relaxation --
template <bool FP32, bool TRIG32 = false>
static __device__ __forceinline__ void relax_body(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                  double *partials, unsigned int *tickets, double dt_override)
{
    __shared__ double s_w[RELAX_T + 3 * PMAX + 8];
    __shared__ double s_m[RELAX_T + 3 * PMAX + 8];
    __shared__ double s_tot[2][RELAX_THREADS / 32];
    __shared__ double red[RELAX_THREADS / 32];

    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    Scalars *sc = C.sc;
    const long long N = sc->N_MAX, p = C.p;
    const double madhoc = sc->madhoc, NSTAR = (double)sc->N_STAR;
    const double dt = dt_override >= 0.0 ? dt_override : sc->Dt;
    const long long tcount = sc->tcount;
    const long long off = C.off;
    const double *__restrict__ r = f.r + off, *__restrict__ m = f.m + off, *__restrict__ phi = f.phi + off;
    const double *__restrict__ vr = f.vr + off, *__restrict__ vt = f.vt + off;
    const long long *__restrict__ id = f.id + off;
    const long long t0 = 1 + (long long)ct.y * RELAX_T;
    const int tid = threadIdx.x;

    // ---- sliding-window sigma (calc_sigma_r): prefix sums over the staged range
    // the reference's windows assume at least 2p+2 stars; below that they index
    // outside the star array, so such a cluster is left unrelaxed
    const bool live = (t0 <= N) && (N >= 2 * p + 2);
    long long lo_load = 1, hi_load = 0;
    if (live) {
        lo_load = t0 - p;
        if (N - 2 * p + 1 < lo_load) lo_load = N - 2 * p + 1;
        if (lo_load < 1) lo_load = 1;
        hi_load = t0 + RELAX_T - 1 + p - 1;
        if (hi_load < 2 * p) hi_load = 2 * p;
        if (hi_load > N) hi_load = N;
    }
    const int L = (int)(hi_load - lo_load + 1);
    const int chunk = (L + RELAX_THREADS - 1) / RELAX_THREADS;
    // FP64 window sums, or with FP32 kinematics float sums of float copies (made
    // with integer instructions, d2f_rn: the FP64 pipe is this kernel's bound)
    using acc_t = typename std::conditional<FP32, float, double>::type;
    acc_t *s_wa = reinterpret_cast<acc_t *>(s_w), *s_ma = reinterpret_cast<acc_t *>(s_m);
    const float madhoc_f = d2f_rn(madhoc);
    acc_t accw = 0, accm = 0;
    for (int i = tid * chunk; i < L && i < (tid + 1) * chunk; ++i) {
        const long long k = lo_load + i;
        if constexpr (FP32) {
            const float vrk = d2f_rn(vr[k]), vtk = d2f_rn(vt[k]);
            const float mm = d2f_rn(m[k]) * madhoc_f;
            accw += mm * (vrk * vrk + vtk * vtk);
            accm += mm;
        } else {
            const double vrk = vr[k], vtk = vt[k];
            const double mm = m[k] * madhoc;
            const double w = mm * (sqr(vrk) + sqr(vtk));
            accw += w;
            accm += mm;
        }
        s_wa[i] = accw;
        s_ma[i] = accm;
    }
    // exclusive scan of the per-thread totals
    {
        acc_t xw = accw, xm = accm;
        const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            acc_t yw = __shfl_up_sync(0xffffffffu, xw, o), ym = __shfl_up_sync(0xffffffffu, xm, o);
            if (lane >= o) {
                xw += yw;
                xm += ym;
            }
        }
        acc_t(*s_tota)[RELAX_THREADS / 32] = reinterpret_cast<acc_t(*)[RELAX_THREADS / 32]>(s_tot);
        if (lane == 31) {
            s_tota[0][wid] = xw;
            s_tota[1][wid] = xm;
        }
        __syncthreads();
        acc_t bw = 0, bm = 0;
        for (int q = 0; q < wid; ++q) {
            bw += s_tota[0][q];
            bm += s_tota[1][q];
        }
        const acc_t ew = bw + xw - accw, em = bm + xm - accm;  // exclusive offsets
        for (int i = tid * chunk; i < L && i < (tid + 1) * chunk; ++i) {
            s_wa[i] += ew;
            s_ma[i] += em;
        }
    }
    __syncthreads();

    double part[RELAX_NPART];
#pragma unroll
    for (int i = 0; i < RELAX_NPART; ++i) part[i] = 0.0;
    int relaxed = 0;  // this thread's pair was relaxed (Nrel, part[0]: counted without the FP64 pipe)

    if (live) {
        double *sig_r = f.sigma_r + off, *sig = f.sigma + off;
        for (int h = 0; h < 2; ++h) {
            const long long si = t0 + 2 * tid + h;
            if (si > N) break;
            long long lo = si - p, hi = lo + (2 * p - 1);
            if (lo < 1) {
                lo = 1;
                hi = 2 * p;
            } else if (hi > N) {
                hi = N;
                lo = hi - (2 * p - 1);
            }
            const int a = (int)(lo - lo_load) - 1, b = (int)(hi - lo_load);
            const acc_t Mv2 = s_wa[b] - (a >= 0 ? s_wa[a] : acc_t(0));
            const acc_t Mm = s_ma[b] - (a >= 0 ? s_ma[a] : acc_t(0));
            sig_r[si] = r[si];
            // sqrt(Mv2 / Mm) (calc_sigma_r, cmc_dynamics_helper.c:2977) as Mv2 rsqrt(Mv2 Mm): one
            // reciprocal square root for a division and a square root, within 3 ulps
            if constexpr (FP32)
                sig[si] = f2d_exact(Mv2 * rsqrtf(Mv2 * Mm));
            else
                sig[si] = Mv2 * rsqrt(Mv2 * Mm);
        }
    }

    // ---- neighbour pairs (k, k+1), k = t0 + 2 tid
    const long long k = t0 + 2 * tid, kp = k + 1;
    double *vr_o = f.vr_rel + off, *vt_o = f.vt_rel + off;
    if (k <= N) {
        if (!C.PERTURB || !(k <= N - N % 2 - 1) || N < 2 * p + 2) {
            // unpaired last star (odd N) or no perturbation: velocities unchanged
            vr_o[k] = vr[k];
            vt_o[k] = vt[k];
            if (kp <= N) {
                vr_o[kp] = vr[kp];
                vt_o[kp] = vt[kp];
            }
        } else {
            const double vtk = vt[k], vrk = vr[k], vtkp = vt[kp], vrkp = vr[kp];
            const double mass_k = m[k], mass_kp = m[kp];
            const long long idk = id[k];
            // calc_encounter_dyns, cmc_dynamics_helper.c:831-871
            const unsigned int wy = draw_block(C.seed, tcount, SITE_Y, idk, 0u).x;
            const double Y = u01(wy);
            f.Y[off + k] = Y;
            f.Y[off + kp] = Y;
            double vr_k, vt_k, vr_kp, vt_kp;
            bool ok = true;
            if constexpr (!FP32) {
                double v1 = vtk, v2 = 0.0, v3 = vrk, vp1, vp2, vp3 = vrkp, w1, w2, w3, W;
                {
                    double sa, ca;
                    if (TRIG32) {
                        sincos_2pi_draw(wy, &sa, &ca);  // sin and cos of Y 2 pi on the FP32 pipe (cmcg_fftrig.cuh)
                    } else {
                        const double ang = Y * 2.0 * CMCG_PI;
                        sincos(ang, &sa, &ca);
                    }
                    vp1 = vtkp * ca;
                    vp2 = vtkp * sa;
                    w1 = vp1 - v1;
                    w2 = vp2 - v2;
                    w3 = vp3 - v3;
                    W = sqrt(sqr(w1) + sqr(w2) + sqr(w3));
                }
                if (eq0(W)) {
                    set_error(sc, CMCG_ERR_W_ZERO, k);
                    ok = false;
                }
                // the three quotients by m_k + m_kp share one correctly rounded reciprocal (div_rcp)
                const double msum = mass_k + mass_kp, imsum = __drcp_rn(msum);
                // S = 0: single-single with SS_COLLISION off, so P_enc = 0 and the
                // encounter draw (cmc_dynamics.c:406) can never succeed.
                double beta = 0.0;
                if (ok && C.RELAXATION) {
                    // beta = (pi/2) sqrt(dt / Trel12) with Trel12 = (pi/32) W^3 / (N_STAR n_local
                    // ((m_k + m_k') madhoc)^2) and n_local = 6p / (4 pi (r_max^3 - r_min^3))
                    // (cmc_dynamics_helper.c:768-786, 831-871): the three quotients as one, within a
                    // few ulps of the reference's beta
                    const double num = dt * NSTAR * (192.0 * (double)p) * sqr(msum * madhoc);
                    const double den = (4.0 * CMCG_PI * CMCG_PI) * window_dr3(r, k, p, N) * cub(W);
                    beta = (CMCG_PI / 2.0) * sqrt(num / den);
                    const double relbeta[4] = {CMCG_PI / 2.0, CMCG_PI / 4.0, CMCG_PI / 8.0, CMCG_PI / 16.0};
                    relaxed = 1;
                    if (gt_pos(beta, relbeta[3])) {  // the smallest threshold: ratio and centre formed once per pair
                        const double qratio = fmax(mass_k, mass_kp) / fmin(mass_k, mass_kp);
                        const double rcm = div_rcp(m[k] * r[k] + m[kp] * r[kp], msum, imsum);
    #pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            if (gt_pos(beta, relbeta[i])) {
                                part[1 + i] += 1.0;
                                part[5 + i] += qratio;
                                part[9 + i] += (mass_k + mass_kp) / 2.0;
                                part[13 + i] += rcm;
                            }
                        }
                    }
                    if (gt_pos(beta, CMCG_PI / 2.0)) beta = CMCG_PI / 2.0;
                    const unsigned int wpsi = draw_block(C.seed, tcount, SITE_PSI, idk, 0u).x;
                    {
                        const double wp = sqrt(sqr(w1) + sqr(w2));
                        if (eq0(wp)) {
                            set_error(sc, CMCG_ERR_WP_ZERO, k);
                            ok = false;
                        } else {
                            const double iwp = __drcp_rn(wp);  // the four quotients by wp (div_rcp)
                            const double a1 = div_rcp(-w2 * W, wp, iwp), a2 = div_rcp(w1 * W, wp, iwp), a3 = 0.0;
                            const double b1 = div_rcp(-w1 * w3, wp, iwp), b2 = div_rcp(-w2 * w3, wp, iwp), b3 = wp;
                            double sb, cb, sp, cp;
                            if (TRIG32) {
                                sincos_beta(beta, &sb, &cb);     // cmcg_fftrig.cuh
                                sincos_2pi_draw(wpsi, &sp, &cp);  // psi = u01 * 2 pi
                            } else {
                                const double psi = u01(wpsi) * 2 * CMCG_PI;
                                sincos(beta, &sb, &cb);
                                sincos(psi, &sp, &cp);
                            }
                            const double wn1 = w1 * cb + a1 * sb * cp + b1 * sb * sp;
                            const double wn2 = w2 * cb + a2 * sb * cp + b2 * sb * sp;
                            const double wn3 = w3 * cb + a3 * sb * cp + b3 * sb * sp;
                            const double fk = div_rcp(mass_kp, msum, imsum), fkp = div_rcp(mass_k, msum, imsum);
                            const double vn1 = v1 - fk * (wn1 - w1), vn2 = v2 - fk * (wn2 - w2), vn3 = v3 - fk * (wn3 - w3);
                            const double pn1 = vp1 + fkp * (wn1 - w1), pn2 = vp2 + fkp * (wn2 - w2), pn3 = vp3 + fkp * (wn3 - w3);
                            vr_k = vn3;
                            vt_k = sqrt(sqr(vn1) + sqr(vn2));
                            vr_kp = pn3;
                            vt_kp = sqrt(sqr(pn1) + sqr(pn2));
                        }
                    }
                    if (ok) {
                        vr_o[k] = vr_k;
                        vt_o[k] = vt_k;
                        vr_o[kp] = vr_kp;
                        vt_o[kp] = vt_kp;
                        // set_star_EJ, cmc_dynamics_helper.c:878-882 (FP64 energies)
                        f.E[off + k] = phi[k] + 0.5 * (sqr(vr_k) + sqr(vt_k));
                        f.J[off + k] = r[k] * vt_k;
                        f.E[off + kp] = phi[kp] + 0.5 * (sqr(vr_kp) + sqr(vt_kp));
                        f.J[off + kp] = r[kp] * vt_kp;
                    }
                }
            } else {
                // FP32 kinematics with FP64 energies: the velocities as floats made with
                // integer instructions (d2f_rn), W, beta and the deflection in float; the
                // FP64 pipe keeps only the window's r^3 difference (which cancels), the
                // rare statistics branch and the energies
                const float fvtk = d2f_rn(vtk), fvrk = d2f_rn(vrk), fvtkp = d2f_rn(vtkp), fvrkp = d2f_rn(vrkp);
                float sa, ca;
                sincosf(__uint2float_rn(wy) * 0x1p-32f * 2.0f * (float)CMCG_PI, &sa, &ca);  // (float)Y 2 pi
                const float fvp1 = fvtkp * ca, fvp2 = fvtkp * sa;
                const float fw1 = fvp1 - fvtk, fw2 = fvp2, fw3 = fvrkp - fvrk;
                const float fW = sqrtf(fw1 * fw1 + fw2 * fw2 + fw3 * fw3);
                if (fW == 0.0f) {
                    set_error(sc, CMCG_ERR_W_ZERO, k);
                    ok = false;
                }
                if (ok && C.RELAXATION) {
                    // beta as in the FP64 path (one quotient), in float
                    const float fmk = d2f_rn(mass_k), fmkp = d2f_rn(mass_kp), msum_f = fmk + fmkp;
                    const float mmf = msum_f * madhoc_f;
                    const float num = d2f_rn(dt) * d2f_rn(NSTAR) * (192.0f * (float)p) * (mmf * mmf);
                    const float den =
                        (4.0f * (float)CMCG_PI * (float)CMCG_PI) * d2f_rn(window_dr3(r, k, p, N)) * (fW * fW * fW);
                    float beta = ((float)CMCG_PI / 2.0f) * sqrtf(num / den);
                    const float relbeta[4] = {(float)(CMCG_PI / 2.0), (float)(CMCG_PI / 4.0), (float)(CMCG_PI / 8.0),
                                              (float)(CMCG_PI / 16.0)};
                    relaxed = 1;
                    if (beta > relbeta[3]) {  // the smallest threshold: ratio and centre formed once per pair
                        const double msum = mass_k + mass_kp;
                        const double qratio = fmax(mass_k, mass_kp) / fmin(mass_k, mass_kp);
                        const double rcm = (m[k] * r[k] + m[kp] * r[kp]) / msum;
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            if (beta > relbeta[i]) {
                                part[1 + i] += 1.0;
                                part[5 + i] += qratio;
                                part[9 + i] += msum / 2.0;
                                part[13 + i] += rcm;
                            }
                        }
                    }
                    if (beta > relbeta[0]) beta = relbeta[0];
                    const unsigned int wpsi = draw_block(C.seed, tcount, SITE_PSI, idk, 0u).x;
                    const float wp = sqrtf(fw1 * fw1 + fw2 * fw2);
                    if (wp == 0.0f) {
                        set_error(sc, CMCG_ERR_WP_ZERO, k);
                        ok = false;
                    } else {
                        const float iwp = 1.0f / wp;
                        const float a1 = -fw2 * fW * iwp, a2 = fw1 * fW * iwp;
                        const float b1 = -fw1 * fw3 * iwp, b2 = -fw2 * fw3 * iwp, b3 = wp;
                        float sb, cb, sp, cp;
                        sincosf(beta, &sb, &cb);
                        sincosf(__uint2float_rn(wpsi) * 0x1p-32f * 2.0f * (float)CMCG_PI, &sp, &cp);  // psi
                        const float d1 = fw1 * (cb - 1.0f) + a1 * sb * cp + b1 * sb * sp;
                        const float d2 = fw2 * (cb - 1.0f) + a2 * sb * cp + b2 * sb * sp;
                        const float d3 = fw3 * (cb - 1.0f) + b3 * sb * sp;
                        const float fk = fmkp / msum_f, fkp = 1.0f - fk;
                        const float vn1 = fvtk - fk * d1, vn2 = -fk * d2, vn3 = fvrk - fk * d3;
                        const float pn1 = fvp1 + fkp * d1, pn2 = fvp2 + fkp * d2, pn3 = fvrkp + fkp * d3;
                        vr_k = f2d_exact(vn3);
                        vt_k = f2d_exact(sqrtf(vn1 * vn1 + vn2 * vn2));
                        vr_kp = f2d_exact(pn3);
                        vt_kp = f2d_exact(sqrtf(pn1 * pn1 + pn2 * pn2));
                    }
                    if (ok) {
                        vr_o[k] = vr_k;
                        vt_o[k] = vt_k;
                        vr_o[kp] = vr_kp;
                        vt_o[kp] = vt_kp;
                        // set_star_EJ, cmc_dynamics_helper.c:878-882 (FP64 energies)
                        f.E[off + k] = phi[k] + 0.5 * (sqr(vr_k) + sqr(vt_k));
                        f.J[off + k] = r[k] * vt_k;
                        f.E[off + kp] = phi[kp] + 0.5 * (sqr(vr_kp) + sqr(vt_kp));
                        f.J[off + kp] = r[kp] * vt_kp;
                    }
                }
            }
            if (!ok || !C.RELAXATION) {
                vr_o[k] = vrk;
                vt_o[k] = vtk;
                vr_o[kp] = vrkp;
                vt_o[kp] = vtkp;
            }
        }
    }

    // ---- statistics (cmc_dynamics.c:430-440), deterministic block order
    __shared__ int s_last;
    __shared__ double s_part[RELAX_THREADS / 32][RELAX_NPART];
    const int nrel = __syncthreads_count(relaxed);  // one pair per thread
    block_sums<RELAX_THREADS>(part, s_part);  // most columns are zero over most warps
    if (tid == 0) {
        double *slot = partials + (size_t)blockIdx.x * RELAX_NPART;
        part[0] = (double)nrel;
        for (int i = 0; i < RELAX_NPART; ++i) slot[i] = part[i];
    }
    if (block_arrive_last(tickets + ct.x, tm.count[ct.x], &s_last)) {
        double acc[RELAX_NPART];
        for (int i = 0; i < RELAX_NPART; ++i)
            acc[i] = reduce_partials_sum<RELAX_THREADS>(partials, tm.first[ct.x], tm.count[ct.x], RELAX_NPART, i, red);
        if (tid == 0) {
            sc->Nrel = (long long)acc[0];
            for (int i = 0; i < 4; ++i) {
                sc->Nrelbeta[i] = (long long)acc[1 + i];
                sc->qaverelbeta[i] = acc[5 + i];
                sc->maverelbeta[i] = acc[9 + i];
                sc->raverelbeta[i] = acc[13 + i];
            }
        }
    }
}

__global__ void __launch_bounds__(RELAX_THREADS, 5) k_relax64(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                           double *partials, unsigned int *tickets, double dt)
{
    relax_body<false>(cls, tm, f, partials, tickets, dt);
}

// Four blocks per SM (room for 128 registers): an autotuner candidate.
__global__ void __launch_bounds__(RELAX_THREADS, 4) k_relax64_lb4(const Cluster *__restrict__ cls, Tiles tm,
                                                               Fields f, double *partials, unsigned int *tickets,
                                                               double dt)
{
    relax_body<false>(cls, tm, f, partials, tickets, dt);
}

__global__ void __launch_bounds__(RELAX_THREADS, 5) k_relax64t(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                            double *partials, unsigned int *tickets, double dt)
{
    relax_body<false, true>(cls, tm, f, partials, tickets, dt);
}

// FP32 kinematics: with little FP64 work left, six blocks per SM (80 registers,
// ~56 bytes of spills) ran the 10^7-star relaxation in 1.33 ms, against 1.38
// at five and 1.48 at four (121 registers unbounded).
__global__ void __launch_bounds__(RELAX_THREADS, 6) k_relax32(const Cluster *__restrict__ cls, Tiles tm, Fields f,
                                                           double *partials, unsigned int *tickets, double dt)
{
    relax_body<true>(cls, tm, f, partials, tickets, dt);
}

// The relaxation's sines and cosines at given arguments (cmcg_trig_check).
__global__ void k_trig_check(const unsigned int *w, long long n, const double *beta, long long nb, double *out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) sincos_2pi_draw(w[i], &out[2 * i], &out[2 * i + 1]);
    if (i < nb) sincos_beta(beta[i], &out[2 * n + 2 * i], &out[2 * n + 2 * i + 1]);
}

}  // namespace cmcg

extern "C" int cmcg_trig_check(const unsigned int *w, long n, const double *beta, long nb, double *out)
{
    using namespace cmcg;
    if (n < 0 || nb < 0 || (n > 0 && !w) || (nb > 0 && !beta) || ((n > 0 || nb > 0) && !out)) return CMCG_ERR_ARG;
    for (long i = 0; i < nb; ++i)
        if (!(beta[i] >= 0.0 && beta[i] <= 1.57079632679489661923)) return CMCG_ERR_ARG;
    if (n == 0 && nb == 0) return CMCG_OK;
    unsigned int *dw = nullptr;
    double *db = nullptr, *dout = nullptr;
    const size_t no = 2 * (size_t)(n + nb) * sizeof(double);
    int rc = CMCG_OK;
    if (cudaMalloc(&dw, (size_t)(n > 0 ? n : 1) * sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&db, (size_t)(nb > 0 ? nb : 1) * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dout, no) != cudaSuccess)
        rc = CMCG_ERR_NOMEM;
    if (rc == CMCG_OK && n > 0 && cudaMemcpy(dw, w, (size_t)n * sizeof(unsigned int), cudaMemcpyHostToDevice))
        rc = CMCG_ERR_CUDA;
    if (rc == CMCG_OK && nb > 0 && cudaMemcpy(db, beta, (size_t)nb * sizeof(double), cudaMemcpyHostToDevice))
        rc = CMCG_ERR_CUDA;
    if (rc == CMCG_OK) {
        const long long m = n > nb ? n : nb;
        k_trig_check<<<(unsigned)((m + 255) / 256), 256>>>(dw, n, db, nb, dout);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, no, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = CMCG_ERR_CUDA;
    }
    cudaFree(dw);
    cudaFree(db);
    cudaFree(dout);
    if (rc == CMCG_ERR_NOMEM) cudaGetLastError();
    return rc;
}
