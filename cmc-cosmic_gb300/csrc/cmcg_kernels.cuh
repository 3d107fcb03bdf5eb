// cmcg_kernels.cuh -- kernel entry points and their scratch buffers.
#pragma once
#include "cmcg_common.cuh"

namespace cmcg {

// ---- tile sizes (stars per block) of the launch families
constexpr int RELAX_T = 256, RELAX_THREADS = 128, PMAX = 64, RELAX_NPART = 17;
constexpr int TS_T = 5120;
constexpr int ORB_T = 128, ORB_NPART = 5;
constexpr int TID_T = 2048, TID_THREADS = 256, TID_NPART = 4;
constexpr int SORT_THREADS = 256, SORT_ITEMS = 8, SORT_T = SORT_THREADS * SORT_ITEMS, RADIX = 256;
constexpr int GATHER_T = 256;
constexpr int POT_THREADS = 256, POT_ITEMS = 4, POT_T = POT_THREADS * POT_ITEMS;
constexpr int EC3_T = 256, EN_T = 256;
constexpr int EXCESS_CAP = 4096;      // listed unphysical predictions per cluster (else full replay)
constexpr int EC3_FIX_THREADS = 512;
constexpr int SORT_MAX_PASSES = 8;
constexpr int TIDAL_PASSES = 32;  // passes after the cluster settles exit at once

struct SortBufs {
    unsigned long long *keys[2];
    unsigned int *vals[2];
    unsigned int *hist;          // per cluster: [RADIX][ntiles_c] at hist_off[c]
    unsigned int *digit_total;   // [nclusters][RADIX]
    long long *hist_off;         // per cluster offset into hist
    int *npass;                  // per cluster: passes needed
    unsigned long long *kmin, *kmax;
};

struct PotBufs {
    double *q;      // m_k / N_STAR per star
    double *agg;    // per tile: q, Delta, C, sum m
    double *carry;  // per tile: Q_after, D_after
};

struct Ec3Bufs {
    double *a;           // per star: excess added by an unphysical prediction (or -1)
    long long *list;     // per cluster: [EXCESS_CAP] indices
    unsigned int *nlist; // per cluster
};

__global__ void k_timestep(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets);
// FP64 kinematics (parity with the reference) and FP32 kinematics with FP64 energies
__global__ void k_relax64(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                          double dt_override);
__global__ void k_relax32(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets,
                          double dt_override);
__global__ void k_orbit(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets);
__global__ void k_tidal(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets);
__global__ void k_tidal_check(const Cluster *cls, int nclusters);
__global__ void k_sort_prep(const Cluster *cls, Tiles tm, Fields f, SortBufs sb, double *partials,
                            unsigned int *tickets);
__global__ void k_sort_hist(const Cluster *cls, Tiles tm, Fields f, SortBufs sb, int pass);
__global__ void k_sort_scan(Tiles tm, SortBufs sb, int pass, int nclusters);
__global__ void k_sort_scatter(const Cluster *cls, Tiles tm, Fields f, SortBufs sb, int pass);
__global__ void k_sort_gather(const Cluster *cls, Tiles tm, Fields f, SortBufs sb);
__global__ void k_sort_commit(const Cluster *cls, int nclusters);
__global__ void k_pot_agg(const Cluster *cls, Tiles tm, Fields f, PotBufs pb);
__global__ void k_pot_carry(const Cluster *cls, Tiles tm, PotBufs pb, int nclusters);
__global__ void k_pot_apply(const Cluster *cls, Tiles tm, Fields f, PotBufs pb);
__global__ void k_begin_step(const Cluster *cls, int nclusters);
__global__ void k_end_step(const Cluster *cls, int nclusters);
__global__ void k_ec3(const Cluster *cls, Tiles tm, Fields f, Ec3Bufs eb);
__global__ void k_ec3_fix(const Cluster *cls, Fields f, Ec3Bufs eb, int nclusters);
__global__ void k_energy(const Cluster *cls, Tiles tm, Fields f, double *partials, unsigned int *tickets);
__global__ void k_potential_query(const Cluster *cls, Fields f, int c, double x, double *out);

}  // namespace cmcg
