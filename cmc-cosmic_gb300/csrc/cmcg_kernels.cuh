// cmcg_kernels.cuh -- kernel entry points and their scratch buffers.
#pragma once
#include "cmcg_common.cuh"

namespace cmcg {

// ---- tile sizes (stars per block) of the launch families
constexpr int RELAX_T = 256, RELAX_THREADS = 128, PMAX = 64, RELAX_NPART = 17;
constexpr int TS_T = 1024, TS_THREADS = 128;  // time step: the potential's 1024-star tiles
constexpr int ORB_T = 128, ORB_NPART = 5;
constexpr int TID_T = 2048, TID_THREADS = 256, TID_NPART = 4;
constexpr int SORT_THREADS = 256, SORT_ITEMS = 8, SORT_T = SORT_THREADS * SORT_ITEMS, RADIX = 256;
constexpr int OS_THREADS = 512;  // onesweep digit pass: 4 keys per thread, 32 warps per SM
constexpr int POT_THREADS = 256, POT_ITEMS = 4, POT_T = POT_THREADS * POT_ITEMS;
static_assert(TS_T == POT_T, "the time step runs on the potential's tile table");
constexpr int EC3_T = 256, EN_T = 2048, EN_THREADS = 256;
constexpr int EXCESS_CAP = 4096;      // listed unphysical predictions per cluster (else full replay)
constexpr int EC3_FIX_THREADS = 512;
constexpr int FIX_WINDOW = 512;       // stars staged per window of the excess-energy replay
// The digit passes sort the top SORT_PREFIX_BITS bits of the keys; each run of
// keys sharing them is then put in full-key order: by the payload gather
// (k_sort_gather, the step's sort) or by k_sort_fix (the allocation-free sort),
// runs longer than FIX_SHORT by k_sort_fix_long.
constexpr int SORT_PREFIX_BITS = 24, SORT_MAX_PASSES = SORT_PREFIX_BITS / 8;
constexpr int FIX_SHORT = 32;   // runs up to this length are sorted by one thread
constexpr int FIX_BLOCK = 2048; // longer runs up to this length in shared memory, the rest in place
constexpr int TIDAL_PASSES = 32;  // bound on the stripping iteration (it settles in a few)

struct SortBufs {
    unsigned long long *keys[2];
    unsigned int *vals[2];
    unsigned long long *ghist;   // per cluster: [SORT_MAX_PASSES][RADIX] digit totals
    unsigned long long *status;  // per tile: [RADIX] look-back words (epoch | flag | count)
    unsigned int *tile_next;     // [SORT_MAX_PASSES] tile counters, zeroed by k_sort_prep
    unsigned int *epoch;         // sorts so far (advanced by k_sort_prep): tags the status words
    int *npass;                  // per cluster: passes needed
    int *shift;                  // per cluster: bits below the sorted prefix (0: the passes sort every bit)
    unsigned int *nlong;         // per cluster: runs longer than FIX_SHORT, zeroed by k_sort_prep
    long long *lstart;           // their first positions: cluster c from off[c] / 32 + 64 c
    unsigned long long *kmin, *kmax;
};

struct PotBufs {
    double *q;      // m_k / N_STAR per star
    double *agg;    // per tile: q, Delta, C, sum m, disorder flag (POT_AGG doubles)
    double *carry;  // per tile: Q, D and forward mass entering the tile (POT_CARRY doubles)
    // approximate running values of the three recurrences of potential_calculate
    double *sapx;   // forward mass sum after star k
    double *mapx;   // M_k, the enclosed mass the backward loop uses at star k
    double *papx;   // Phi_k
    double *t;      // exact M_k (1/r_k - 1/r_{k+1}) per star
};
constexpr int POT_AGG = 5, POT_CARRY = 3;

// 1/r of the star just outside a potential tile whose largest index is kstart
// (r[N+1] = SF_INFINITY).  A tile map sized for the capacity has tiles lying
// wholly below star 1 once N has shrunk (kstart < 1); they hold no stars and
// must not read r at all.
__device__ __forceinline__ double pot_r_next_inv(const double *r, long long kstart, long long N)
{
    if (kstart < 1 || kstart > N) return 0.0;
    return __drcp_rn(kstart == N ? CMCG_SF_INFINITY : r[kstart + 1]);
}

// Exclusive block prefix of one double per thread (thread order), as the
// potential's scans take it: warp shuffles, then the warps' totals in order.
template <int NT>
__device__ __forceinline__ double pot_block_excl_prefix(double tsum, double *s_w)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double x = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    double b = 0.0;
    for (int q = 0; q < w; ++q) b += s_w[q];
    return b + x - tsum;  // exclusive prefix of this thread
}

// ---- exact replay of the sequential potential recurrences (cmcg_phi.cu)
// A "sequential point" is a position whose rounding cannot be proven to stay
// on one binade grid; the other positions add an integer number of grid units.
struct ChainAgg {        // per tile, in the chain's order
    long long P;         // grid units summed since the tile's last sequential point
    int cnt;             // positions in that run
    int nsp;             // sequential points in the tile
};
struct ChainCarry {      // per tile: the run entering it and its first record index
    long long P;
    int cnt;
    int spoff;
};
struct SPRec {           // one sequential point
    long long k;         // star index
    double a;            // the term added at this position
    long long Pprev;     // grid units of the run ending just before it
    int keyprev;         // sign and exponent bits of that run's binade
    int cntprev;         // length of that run (0: the previous position is a sequential point)
    double sprev, snew;  // exact values before and after (filled by the replay)
};
struct PhiCtl {          // per cluster
    double Sm, Qtot, Dtot, Mapx;   // approximate totals: sum m, sum q, sum d, Mtotal
    double Mb, G;                  // bound on every |M_k|; scan error factor
    double marg1, marg2;           // bounds on |approximate - sequential| of chains 1, 2
    double c0, c1;                 // chain 3 bound: c0 + c1 / r_k
    int fail;                      // 1: replay impossible or refused, recompute sequentially
    int disorder;                  // radii out of order or non-finite input (no radius index)
    long long nsp[3];
};
struct PhiScan {         // per thread of a tile: its tile-local exclusive scans (TileScan)
    long long P;         // grid units of the run entering its first item
    int c, r;            // that run's length, and whether it starts at a sequential point
    int spx;             // sequential points before its first item
    int pad;
};
// A chain's classification, written by the pass that classifies it and read
// by the passes after it: per star, rho and (key | keyprev << 12 | sp << 24);
// per thread, its tile scans.  Slot 1 holds chain 2, slot 0 chain 1 and then
// chain 3 (chain 1's last reader runs before chain 3 is classified).
struct PhiBufs {
    ChainAgg *agg[2];
    ChainCarry *carry[2];
    SPRec *rec[2];
    PhiCtl *ctl;
    long long *crho[2];
    unsigned int *cmeta[2];
    PhiScan *cscan[2];
};
constexpr int PHI_WALK_BATCH = 512;

struct Ec3Bufs {
    double *a;           // per star: excess added by an unphysical prediction (or -1)
    long long *list;     // per cluster: [EXCESS_CAP] indices
    unsigned int *nlist; // per cluster
    double *carry;       // per cluster: [EXCESS_CAP] excess entering each listed star's segment
};

__global__ void k_timestep(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                           int begin);
// FP64 kinematics (parity with the reference) and FP32 kinematics with FP64 energies
__global__ void k_relax64(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                          double dt_override);
__global__ void k_relax32(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                          double dt_override);
// FP64 kinematics with the sines and cosines on the FP32 pipe (cmcg_params.relax_trig32)
__global__ void k_relax64t(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                           double dt_override);
__global__ void k_relax64_lb4(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                              double dt_override);
// Stars whose Q(j) <= 0 and the first index with Q > 0 found for each (k_posq_scan)
struct PosQ {
    int *slot;            // per star: PQ_POSITIVE (Q(j) > 0), a list entry, or PQ_SCAN_HERE
    unsigned int *count;  // list length this step
    int *cl;              // list: cluster,
    long long *j, *res;   //       star index, first index with Q > 0
};
constexpr int PQ_POSITIVE = -1, PQ_SCAN_HERE = -2, PQ_CAP = 1024;
__global__ void k_orbit_pre(const Cluster *cls, Tiles tm, Fields f, PosQ pq);
__global__ void k_posq_scan(const Cluster *cls, Fields f, PosQ pq);
__global__ void k_orbit(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets, PosQ pq);
__global__ void k_orbit_lb4(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets, PosQ pq);

// ---- learned proposal of the orbit sampler (cmcg_mlp.cu, cmcg_orbit.cu)
// An MLP 8 -> 64 -> 64 -> 33 (ReLU; BF16 weights and activations, FP32
// accumulation on the tensor cores) maps a star's orbit features to a
// 32-bin piecewise-constant density in the sampling variable X (a monotone
// piecewise-linear CDF) and to P, the predicted acceptance probability of the
// plain sampler's trial.  The sampler draws X from that density and accepts
// it against the true clipped density min(g(s), F) under the envelope
// kappa * F * P * q(X); a trial where the envelope fails sends the star back
// to the plain sampler.
constexpr int MLP_IN = 8, MLP_H = 64, MLP_OUT = 33, MLP_BINS = 32;
constexpr int MLP_T = 128;                 // rows (stars or samples) per tile = threads per CTA
constexpr int MLP_K1 = 16;                 // layer-1 K: the 8 features, zero-padded
constexpr int MLP_N3 = 48;                 // layer-3 N: the 33 outputs, zero-padded
constexpr int MLP_NG = 80, MLP_NG1 = 16;   // weight-gradient N: inputs, a column of ones (bias), padding
// master parameters (FP32): W1[64][8], b1[64], W2[64][64], b2[64], W3[33][64], b3[33]
constexpr int P_W1 = 0, P_B1 = P_W1 + MLP_H * MLP_IN, P_W2 = P_B1 + MLP_H, P_B2 = P_W2 + MLP_H * MLP_H,
              P_W3 = P_B2 + MLP_H, P_B3 = P_W3 + MLP_OUT * MLP_H, MLP_NPARAM = P_B3 + MLP_OUT;
constexpr int MLP_PSTRIDE = 6912;          // floats per training partial: gradients, then the two loss sums
static_assert(MLP_NPARAM + 2 <= MLP_PSTRIDE, "partial layout");
// packed operand image (bytes): the B operands of the forward pass, the
// biases (FP32), then the transposed weights of the backward pass
constexpr int IMG_W1 = 0, IMG_W2 = IMG_W1 + MLP_H * MLP_K1 * 2, IMG_W3 = IMG_W2 + MLP_H * MLP_H * 2,
              IMG_BIAS = IMG_W3 + MLP_N3 * MLP_H * 2, IMG_INFER = IMG_BIAS + 768, IMG_W3T = IMG_INFER,
              IMG_W2T = IMG_W3T + MLP_H * MLP_N3 * 2, IMG_TOTAL = IMG_W2T + MLP_H * MLP_H * 2;
static_assert(IMG_INFER % 128 == 0 && IMG_TOTAL % 128 == 0, "bulk copies of 16-byte multiples");
constexpr float MLP_FLOOR = 1.0f / 64.0f;  // share of the uniform density mixed into every proposal
constexpr int MLP_TRAIN_GRID_MAX = 152;    // partial slots of the training kernel

struct MlpNet {
    float *w, *m, *v;     // master parameters and Adam moments
    unsigned char *img;   // packed operand image (IMG_TOTAL bytes)
    float *partials;      // [grid][MLP_PSTRIDE]
    int *status;          // a bounded wait that gave up (CMCG_ERR_SPIN)
};
struct MlpData {
    const uint4 *feat;    // 8 BF16 features per sample
    const int *bin;       // bin of the accepted X (floor(32 X))
    const int *ntrial;    // trials the plain sampler used (>= 1)
    long long n;
    int ordered;          // 1: batch position p is sample p (gradient checks)
};
enum { LEARN_OFF = 0, LEARN_ON = 1, LEARN_COLLECT = 2 };
constexpr int LSTAT_TRIALS = 0, LSTAT_ACCEPT = 1, LSTAT_FAIL = 2, LSTAT_STARS = 3, LSTAT_PLAIN_TRIALS = 4,
              LSTAT_PLAIN_STARS = 5, LSTAT_N = 8;
struct Learn {
    uint4 *feat;              // per star slot: the 8 BF16 features (zero where no position is sampled)
    double *F;                // per star slot: the plain envelope F (> 0: the star samples a position)
    float *prop;              // [32][stride]: C_1 .. C_31 of the proposal's CDF, then P
    int *ntrial;              // per star slot: accepted trial, plain k > 0 or proposal -k
    unsigned long long *stats;  // LSTAT_* counters of the last step
    const int *mlp_status;    // the network's status word (a failed inference)
    long long stride;
    double kappa;             // envelope factor
    int mode;                 // LEARN_ON: proposal first; LEARN_COLLECT: plain trials only
};
__global__ void k_mlp_pack(MlpNet net);
__global__ void k_mlp_infer(MlpNet net, const uint4 *feat, long long nrows, float *prop, long long stride,
                            float *z_out);
__global__ void k_mlp_train(MlpNet net, MlpData data, int batch, unsigned long long seed, int step);
__global__ void k_mlp_adam(MlpNet net, int nparts, float lr, int t, int mode, float *out);
constexpr int MLP_INFER_SMEM = IMG_INFER + MLP_T * MLP_K1 * 2 + MLP_T * MLP_H * 2 + 64;
constexpr int MLP_TRAIN_SMEM = IMG_TOTAL + MLP_T * MLP_K1 * 2 + MLP_NG1 * MLP_T * 2 + 2 * MLP_T * MLP_H * 2 +
                               2 * MLP_NG * MLP_T * 2 + 2 * MLP_T * MLP_T * 2 + 192;
__global__ void k_orbit_aps(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets, PosQ pq,
                            Learn L);
__global__ void k_orbit_learn(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                              PosQ pq, Learn L);
// persistent forms of k_orbit / k_orbit_lb4: tiles taken from *next (zeroed before the launch)
__global__ void k_orbit_pers(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets, PosQ pq,
                             unsigned int *next);
__global__ void k_orbit_pers_lb4(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                                 PosQ pq, unsigned int *next);
__global__ void k_orbit_learn_lb4(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                                  PosQ pq, Learn L);

// ---- launch variants the autotuner chooses between (bit-identical results)
enum { V_ORBIT, V_RELAX, V_LEARN, V_MLP_GRID, V_SORT_TILE, V_GATHER_TILE, V_COUNT };
__global__ void k_tidal(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *bar, int nclusters);
__global__ void k_sort_prep(const Cluster *cls, Tiles tm, Fields f, SortBufs sb, double *partials,
                            unsigned int *tickets);
__global__ void k_sort_ghist(const Cluster *cls, Tiles tm, Fields f, SortBufs sb);
// One digit pass over tiles of `tile_keys` keys (1024, 2048 or 4096: the
// autotuner's candidates; tm is the matching tile table).  The 4096-key form
// stages 48 KB of dynamic shared memory, which sort_onesweep_setup allows
// (once per process, before any launch).  Host launchers of
// the templated kernels, defined beside them (a template kernel's launch stub
// is local to the file that instantiates it).
void launch_sort_onesweep(int tile_keys, int ntiles, cudaStream_t s, const Cluster *cls, Tiles tm, Fields f,
                          SortBufs sb, int pass);
cudaError_t sort_onesweep_setup();
__global__ void k_sort_fix(const Cluster *cls, Tiles tm, SortBufs sb);
// With tickets (the step's sort, after k_sort_gather): also moves the payload
// of the runs it sorts, and the last block of each cluster commits its new
// star count.  Without (the allocation-free sort): keys and values only.
__global__ void k_sort_fix_long(const Cluster *cls, Tiles tm, SortBufs sb, Fields f, unsigned int *tickets);
// The payload gather, `block` stars per block (128, 256 or 1024, on the
// matching tile table); it places the runs of up to FIX_SHORT keys and lists
// the longer ones for k_sort_fix_long.
void launch_sort_gather(int block, int ntiles, cudaStream_t s, const Cluster *cls, Tiles tm, Fields f, SortBufs sb);
__global__ void k_pot_agg(const Cluster *cls, Tiles tm, Fields f, PotBufs pb);
__global__ void k_pot_carry(const Cluster *cls, Tiles tm, PotBufs pb, PhiBufs ph, int nclusters);
__global__ void k_phi_cls12(const Cluster *cls, Tiles tm, Fields f, PotBufs pb, PhiBufs ph, unsigned int *tickets);
__global__ void k_phi_rec12(const Cluster *cls, Tiles tm, Fields f, PotBufs pb, PhiBufs ph, unsigned int *tickets);
__global__ void k_phi_cls3(const Cluster *cls, Tiles tm, Fields f, PotBufs pb, PhiBufs ph, unsigned int *tickets);
__global__ void k_phi_rec3(const Cluster *cls, Tiles tm, Fields f, PotBufs pb, PhiBufs ph, unsigned int *tickets);
__global__ void k_phi_final(const Cluster *cls, Tiles tm, Fields f, PotBufs pb, PhiBufs ph);
__global__ void k_phi_seq(const Cluster *cls, Fields f, PhiBufs ph, int nclusters);
__global__ void k_ridx_build(const Cluster *cls, Fields f, PhiBufs ph, int nclusters);
constexpr int RIDX_THREADS = 256;
__global__ void k_begin_step(const Cluster *cls, int nclusters);
__global__ void k_end_step(const Cluster *cls, int nclusters);
// Their work for one cluster (cmc.c:246-257; cmc.c:294, 390); a whole step
// does them in the last block of its first kernel (k_timestep, begin = 1)
// and of its last (k_energy, end = 1).
__device__ __forceinline__ void begin_step(const Cluster &C)
{
    Scalars *sc = C.sc;
    sc->Eescaped_old = sc->Eescaped;
    sc->Jescaped_old = sc->Jescaped;
    sc->TidalMassLoss_old = sc->TidalMassLoss;
    sc->Etidal_old = sc->Etidal;
    sc->Eescaped = 0.0;
    sc->Jescaped = 0.0;
    sc->TidalMassLoss = 0.0;
    sc->Etidal = 0.0;
    sc->N_MAX_NEW = sc->N_MAX;
    sc->tidal_done = C.TIDALLY_STRIP_STARS ? 0 : 1;
    sc->tidal_iters = 0;
}

__device__ __forceinline__ void end_step(Scalars *sc)
{
    sc->Prev_Dt = sc->Dt;
    sc->tcount += 1;
}

// hx: nullptr, or (host exchange) every cluster's pinned host arrays, which
// these kernels write as well as the fields: for cluster c, hx[4c] = vr,
// hx[4c+1] = vt, hx[4c+3] = J = r vt (k_ec3, k_ec3_fix), hx[4c+2] = E
// (k_energy), star i at element i - 1.
__global__ void k_ec3(const Cluster *cls, Tiles tm, Fields f, Ec3Bufs eb, double *const *hx);
__global__ void k_ec3_fix(const Cluster *cls, Fields f, Ec3Bufs eb, int nclusters, double *const *hx);
__global__ void k_energy(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                         double *const *hx, int end);
__global__ void k_potential_query(const Cluster *cls, Fields f, int c, double x, double *out);

// ---- step diagnostics of dyn.dat and lagrad.dat (cmcg_diag.cu)
constexpr int DIAG_PC_MAX = 64, DIAG_COLS = 5, DIAG_CCOLS = 6;
struct DiagDev {
    // inputs
    int n_pc, bh_include;
    double minimum_r;
    double pc[DIAG_PC_MAX];
    // found by k_diag_find
    long long first[DIAG_PC_MAX];  // first star whose mass sum exceeds each fraction (0: none)
    long long jhalf;               // first star whose mass sum reaches half the mass (0: none)
    // results
    int status;                    // 0, or the reason the reference would stop
    long long nave;
    double rh, rho, v_rms, rc, rc_nb, m_ave, n, rc_spitzer, N_core, N_core_nb, Trc;
    int n_set;                     // fractions assigned (the rest were not reached)
    double mass_r[DIAG_PC_MAX], ave_mass_r[DIAG_PC_MAX], no_star_r[DIAG_PC_MAX], densities_r[DIAG_PC_MAX];
    double ke_rad_r[DIAG_PC_MAX], ke_tan_r[DIAG_PC_MAX], v2_rad_r[DIAG_PC_MAX], v2_tan_r[DIAG_PC_MAX];
};
// per-star running sums the diagnostics keep between their passes (the
// potential's and the sort's scratch arrays, which every step rewrites)
struct DiagScratch {
    double *col[DIAG_COLS];
};
__global__ void k_diag_sum(const Cluster *cls, Tiles tm, Fields f, int b0, double *partials);
__global__ void k_diag_carry(const Cluster *cls, Tiles tm, int c, int b0, int nt, double *partials);
__global__ void k_diag_prefix(const Cluster *cls, Tiles tm, Fields f, int b0, const double *partials,
                              DiagScratch ds);
__global__ void k_diag_find(const Cluster *cls, Fields f, int c, DiagScratch ds, DiagDev *dd);
__global__ void k_diag_central(const Cluster *cls, Tiles tm, Fields f, int c, int b0, int nt, double *partials,
                               unsigned int *tickets, DiagScratch ds, DiagDev *dd);

}  // namespace cmcg
