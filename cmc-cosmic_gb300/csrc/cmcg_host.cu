// cmcg_host.cu -- the C ABI of include/cmcgpu.h: context, device memory,
// launch geometry, the step sequence and CUDA-graph capture.
//
// Memory: one arena per context (a single cudaMalloc at creation), carved into
// the structure-of-arrays fields, the sort/scan scratch and the per-tile
// partial sums.  Nothing is allocated while stepping.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

using namespace cmcg;

namespace {

struct TileTable {
    int2 *d_tiles = nullptr;
    int *d_first = nullptr, *d_count = nullptr;
    int ntiles = 0;
    std::vector<int> first, count;
    Tiles view() const { return Tiles{d_tiles, d_first, d_count, ntiles}; }
};

// The step in parts, cut where the host exchange overlaps copies with
// kernels: the time step (which reads r, m, vr, vt only); relaxation to the
// sort (which swaps the field pointers); potential and energy conservation
// (r, m, id are final); energies (vr, vt are final).  The host exchange runs
// part HX_SORT as two: HX_XRELAX marks E, J and relaxes while the caller's E
// and J are still on their way; HX_XSORT merges them in, then orbits to the
// sort.  With the caller's arrays reachable from the device it runs parts 2
// and 3 as one, HX_XTAIL, whose kernels also write vr, vt (energy
// conservation) and E, J (energies) into those arrays.
constexpr int HX_PARTS = 4, HX_SORT = 1, HX_XRELAX = 4, HX_XSORT = 5, HX_XTAIL = 6, HX_ALL = 7;

enum Family { F_BEGIN, F_TIMESTEP, F_RELAX, F_ORBIT, F_TIDAL, F_SORT, F_POT, F_EC3, F_ENERGY, F_END, F_MLP, F_COUNT };
const char *kFamilyNames[F_COUNT] = {"begin", "timestep", "relax", "orbit", "tidal",
                                     "sort",  "potential", "ec3", "energy", "end", "mlp"};

// Autotuner candidates: per tunable launch, its variants and the kernel family timed.
const int kMlpGrid[4] = {4, 2, 3, 6};  // persistent CTAs per SM of the network's inference
struct Tunable {
    const char *name;
    int family;
    int nvar;
    const char *variant[4];
};
const Tunable kTunables[V_COUNT] = {
    {"orbit", F_ORBIT, 4, {"5 blocks/SM", "4 blocks/SM", "5 blocks/SM persistent", "4 blocks/SM persistent"}},
    {"relax", F_RELAX, 2, {"5 blocks/SM", "4 blocks/SM"}},
    {"orbit_learn", F_ORBIT, 2, {"5 blocks/SM", "4 blocks/SM"}},
    {"mlp_grid", F_MLP, 4, {"4 CTAs/SM", "2 CTAs/SM", "3 CTAs/SM", "6 CTAs/SM"}},
    {"sort_tile", F_SORT, 3, {"4096 keys/tile", "2048 keys/tile", "1024 keys/tile"}},
    {"gather_tile", F_SORT, 3, {"256 stars/block", "128 stars/block", "1024 stars/block"}},
};

struct ProfRec {
    int fam;
    cudaEvent_t a, b;
};

// One segment of a batched host exchange (k_xfer): n 8-byte words from src to dst.
struct XferSeg {
    unsigned long long *dst;
    const unsigned long long *src;
    long long n;   // 8-byte words
    long long c0;  // first chunk of the segment in its batch
};
constexpr int XFER_THREADS = 256, XFER_UNROLL = 4, XFER_CHUNK = XFER_THREADS * XFER_UNROLL;
constexpr int XFER_PER_CLUSTER = 4;  // upload segments per cluster: r, m, vr, vt
// The exchange's table, in one block (host and device alike) that goes up in
// one copy: the upload segments; every cluster's host arrays that kernels
// write (vr, vt, E, J: the hx argument of k_ec3, k_ec3_fix, k_energy); every
// cluster's star count.
static size_t xfer_table_bytes(int ncl)
{
    return (size_t)XFER_PER_CLUSTER * ncl * sizeof(XferSeg) + (size_t)4 * ncl * sizeof(double *) +
           (size_t)ncl * sizeof(long long);
}

}  // namespace

struct cmcg_ctx {
    int ncl = 0;
    cudaStream_t stream = nullptr;
    std::vector<long long> cap, off;
    long long total = 0;
    std::vector<cmcg_params> params;
    std::vector<Cluster> h_cls;
    Cluster *d_cls = nullptr;
    Scalars *d_sc = nullptr;
    Fields f{};
    double *partials = nullptr;
    unsigned int *tickets = nullptr;
    unsigned int *gbar = nullptr;  // grid barrier of the cooperative tidal kernel
    unsigned int *orbit_next = nullptr;  // tile counter of the persistent orbit kernels
    int tidal_grid = 1;
    PosQ pq{};
    int posq_grid = 1;
    SortBufs sb{};
    PotBufs pb{};
    PhiBufs ph{};
    long long rec_total = 0;
    long long ridx_total = 0;
    int ridx_Bmax = 0;
    Ec3Bufs eb{};
    double *d_query = nullptr;
    DiagDev *d_diag = nullptr;
    TileTable t128, t256, t1024, t2048, t4096;  // t4096: the 4096-key digit passes
    void *arena = nullptr;
    size_t arena_bytes = 0;
    int relax_fp32 = 0, relax_trig32 = 0;
    int nsm = 1;
    // learned proposal: the network (always), the per-star buffers (on first use)
    MlpNet net{};
    void *net_mem = nullptr;
    int adam_t = 0;             // Adam steps taken since the parameters were set
    int learn_mode = LEARN_OFF;
    double learn_kappa = 1.2;
    Learn lrn{};
    void *lrn_mem = nullptr;
    // launch variants (autotuner; every variant gives bit-identical results)
    int var[V_COUNT] = {};
    // part graphs of a step (HX_* above), per pointer parity at their start:
    // single steps and the host exchange (cmcg_step_host), whose copies run on
    // a second stream and overlap the parts
    cudaGraphExec_t hx[HX_ALL][2] = {};
    long hx_launches[HX_ALL][2] = {};
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_sorted = nullptr, ev_copied = nullptr, ev_in = nullptr, ev_ec3 = nullptr, ev_ej = nullptr;
    long long *d_nout = nullptr;  // per cluster: stars after the step
    // batched host exchange: segment tables (pinned host copy, device copy)
    // and per-cluster counts, XFER_PER_CLUSTER segments per cluster
    XferSeg *h_xfer = nullptr, *d_xfer = nullptr;
    double **h_hx = nullptr, **d_hx = nullptr;
    long long *h_xn = nullptr, *d_xn = nullptr;
    // graphs
    // The sort swaps the field pointers every step, so a captured two-step
    // graph is tied to the pointer parity it was captured at: one per parity.
    bool use_graph = false, graph_ready[2] = {false, false};
    int parity = 0;
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    long launches = 0, launches_last = 0, graph_launches[2] = {0, 0};
    // profiling
    bool profile = false;
    std::vector<ProfRec> prof;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_next = 0;
    double fam_ms[F_COUNT] = {0};
    long fam_n[F_COUNT] = {0};
    int cur_fam = -1;
    cudaEvent_t cur_a = nullptr;
};

#define CK(x)                                                                                    \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) {                                                                 \
            fprintf(stderr, "cmcgpu: %s failed: %s (%s:%d)\n", #x, cudaGetErrorString(e_), __FILE__, \
                    __LINE__);                                                                   \
            return CMCG_ERR_CUDA;                                                                \
        }                                                                                        \
    } while (0)

static cudaEvent_t take_event(cmcg_ctx *c)
{
    if (c->ev_next >= c->ev_pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->ev_pool.push_back(e);
    }
    return c->ev_pool[c->ev_next++];
}

static void fam_begin(cmcg_ctx *c, int fam)
{
    if (!c->profile) return;
    c->cur_fam = fam;
    c->cur_a = take_event(c);
    cudaEventRecord(c->cur_a, c->stream);
}

static void fam_end(cmcg_ctx *c)
{
    if (!c->profile || c->cur_fam < 0) return;
    cudaEvent_t b = take_event(c);
    cudaEventRecord(b, c->stream);
    c->prof.push_back(ProfRec{c->cur_fam, c->cur_a, b});
    c->cur_fam = -1;
}

static int build_table(TileTable &t, const std::vector<long long> &cap, int T, std::vector<int2> &host)
{
    const int n = (int)cap.size();
    t.first.assign(n, 0);
    t.count.assign(n, 0);
    host.clear();
    for (int c = 0; c < n; ++c) {
        long long k = (cap[c] + T - 1) / T;
        if (k < 1) k = 1;
        t.first[c] = (int)host.size();
        t.count[c] = (int)k;
        for (long long i = 0; i < k; ++i) host.push_back(make_int2(c, (int)i));
    }
    t.ntiles = (int)host.size();
    return 0;
}

namespace {
struct Carver {
    char *base;
    size_t used = 0;
    template <class T>
    T *take(size_t n)
    {
        used = (used + 255) & ~(size_t)255;
        T *p = base ? (T *)(base + used) : nullptr;
        used += n * sizeof(T);
        return p;
    }
};
}  // namespace

static int carve_all(cmcg_ctx *c, char *base, std::vector<int2> *tabs, size_t *bytes)
{
    Carver cv{base};
    const size_t tot = (size_t)c->total;
    Fields &f = c->f;
    double **dfields[] = {&f.r,     &f.m,     &f.phi,    &f.inv_r, &f.vr,     &f.vt,     &f.E,      &f.J,
                          &f.vr_rel, &f.vt_rel, &f.rnew, &f.vrnew, &f.vtnew,  &f.X,      &f.Y,      &f.r_peri,
                          &f.r_apo, &f.ec_pre, &f.rOld, &f.sigma_r, &f.sigma, &f.r2,     &f.m2,     &f.ec_pre2};
    for (double **p : dfields) *p = cv.take<double>(tot);
    f.id = cv.take<long long>(tot);
    f.id2 = cv.take<long long>(tot);
    f.rphif = cv.take<float4>(tot);
    c->sb.keys[0] = cv.take<unsigned long long>(tot);
    c->sb.keys[1] = cv.take<unsigned long long>(tot);
    c->sb.vals[0] = cv.take<unsigned int>(tot);
    c->sb.vals[1] = cv.take<unsigned int>(tot);
    c->sb.ghist = cv.take<unsigned long long>((size_t)c->ncl * SORT_MAX_PASSES * RADIX);
    // look-back words for the digit pass's smaller tiles (1024 keys), the
    // most tiles either tile size has
    c->sb.status = cv.take<unsigned long long>((size_t)std::max(c->t1024.ntiles, c->t2048.ntiles) * RADIX);
    c->sb.tile_next = cv.take<unsigned int>(SORT_MAX_PASSES);
    c->orbit_next = cv.take<unsigned int>(1);
    c->d_xfer = (XferSeg *)cv.take<char>(xfer_table_bytes(c->ncl));
    c->d_hx = c->d_xfer ? (double **)(c->d_xfer + (size_t)XFER_PER_CLUSTER * c->ncl) : nullptr;
    c->d_xn = c->d_xfer ? (long long *)(c->d_hx + (size_t)4 * c->ncl) : nullptr;
    c->sb.epoch = cv.take<unsigned int>(1);
    c->sb.npass = cv.take<int>(c->ncl);
    c->sb.shift = cv.take<int>(c->ncl);
    c->sb.nlong = cv.take<unsigned int>(c->ncl);
    c->sb.lstart = cv.take<long long>((size_t)(tot / 32 + 64 * (c->ncl + 1)));  // cluster c from off[c] / 32 + 64 c
    c->sb.kmin = cv.take<unsigned long long>(c->ncl);
    c->sb.kmax = cv.take<unsigned long long>(c->ncl);
    c->pb.q = cv.take<double>(tot);
    c->pb.agg = cv.take<double>((size_t)c->t1024.ntiles * POT_AGG);
    c->pb.carry = cv.take<double>((size_t)c->t1024.ntiles * POT_CARRY);
    c->pb.sapx = cv.take<double>(tot);
    c->pb.mapx = cv.take<double>(tot);
    c->pb.papx = cv.take<double>(tot);
    c->pb.t = cv.take<double>(tot);
    for (int i = 0; i < 2; ++i) {
        c->ph.agg[i] = cv.take<ChainAgg>(c->t1024.ntiles);
        c->ph.carry[i] = cv.take<ChainCarry>(c->t1024.ntiles);
        c->ph.rec[i] = cv.take<SPRec>((size_t)c->rec_total);
        c->ph.crho[i] = cv.take<long long>(tot);
        c->ph.cmeta[i] = cv.take<unsigned int>(tot);
        c->ph.cscan[i] = cv.take<PhiScan>((size_t)c->t1024.ntiles * POT_THREADS);
    }
    c->ph.ctl = cv.take<PhiCtl>(c->ncl);
    f.ridx = cv.take<int>((size_t)c->ridx_total);
    c->eb.a = cv.take<double>(tot);
    c->eb.list = cv.take<long long>((size_t)c->ncl * EXCESS_CAP);
    c->eb.nlist = cv.take<unsigned int>(c->ncl);
    c->eb.carry = cv.take<double>((size_t)c->ncl * EXCESS_CAP);
    size_t np = 0;
    np = std::max(np, (size_t)c->t256.ntiles * RELAX_NPART);
    np = std::max(np, (size_t)c->t128.ntiles * ORB_NPART);
    np = std::max(np, (size_t)c->t2048.ntiles * 4);
    np = std::max(np, (size_t)c->t256.ntiles * 2);
    np = std::max(np, (size_t)c->t1024.ntiles * 1);
    c->partials = cv.take<double>(np);
    c->tickets = cv.take<unsigned int>(c->ncl);
    c->gbar = cv.take<unsigned int>(2);
    c->pq.slot = cv.take<int>(tot);
    c->pq.count = cv.take<unsigned int>(1);
    c->pq.cl = cv.take<int>(PQ_CAP);
    c->pq.j = cv.take<long long>(PQ_CAP);
    c->pq.res = cv.take<long long>(PQ_CAP);
    c->d_sc = cv.take<Scalars>(c->ncl);
    c->d_cls = cv.take<Cluster>(c->ncl);
    c->d_query = cv.take<double>(2);
    c->d_diag = cv.take<DiagDev>(1);
    TileTable *tts[5] = {&c->t128, &c->t256, &c->t1024, &c->t2048, &c->t4096};
    for (int i = 0; i < 5; ++i) {
        tts[i]->d_tiles = cv.take<int2>(tabs[i].size());
        tts[i]->d_first = cv.take<int>(c->ncl);
        tts[i]->d_count = cv.take<int>(c->ncl);
    }
    *bytes = cv.used + 256;
    return 0;
}

// The network's parameters, Adam moments, packed image and training partials.
static int alloc_net(cmcg_ctx *c)
{
    Carver cv{nullptr};
    for (int pass = 0; pass < 2; ++pass) {
        cv.used = 0;
        MlpNet &n = c->net;
        n.w = cv.take<float>(MLP_NPARAM);
        n.m = cv.take<float>(MLP_NPARAM);
        n.v = cv.take<float>(MLP_NPARAM);
        n.img = cv.take<unsigned char>(IMG_TOTAL);
        n.partials = cv.take<float>((size_t)MLP_TRAIN_GRID_MAX * MLP_PSTRIDE);
        n.status = cv.take<int>(1);
        if (pass == 0) {
            if (cudaMalloc(&c->net_mem, cv.used + 256) != cudaSuccess) {
                cudaGetLastError();
                return CMCG_ERR_NOMEM;
            }
            CK(cudaMemsetAsync(c->net_mem, 0, cv.used + 256, c->stream));
            cv.base = (char *)c->net_mem;
        }
    }
    CK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_TRAIN_SMEM));
    CK(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_INFER_SMEM));
    return CMCG_OK;
}

// Per-star buffers of the learned proposal, allocated when it is first enabled.
static int ensure_learn(cmcg_ctx *c)
{
    if (c->lrn_mem) return CMCG_OK;
    const size_t tot = (size_t)c->total;
    Carver cv{nullptr};
    for (int pass = 0; pass < 2; ++pass) {
        cv.used = 0;
        Learn &L = c->lrn;
        L.feat = cv.take<uint4>(tot);
        L.F = cv.take<double>(tot);
        L.prop = cv.take<float>(tot * MLP_BINS);
        L.ntrial = cv.take<int>(tot);
        L.stats = cv.take<unsigned long long>(LSTAT_N);
        L.stride = (long long)tot;
        L.mlp_status = c->net.status;
        if (pass == 0) {
            if (cudaMalloc(&c->lrn_mem, cv.used + 256) != cudaSuccess) {
                cudaGetLastError();
                fprintf(stderr, "cmcgpu: cannot allocate %zu bytes for the learned proposal\n", cv.used);
                return CMCG_ERR_NOMEM;
            }
            CK(cudaMemsetAsync(c->lrn_mem, 0, cv.used + 256, c->stream));
            cv.base = (char *)c->lrn_mem;
        }
    }
    return CMCG_OK;
}

extern "C" {

void cmcg_default_params(cmcg_params *p)
{
    memset(p, 0, sizeof(*p));
    p->N_STAR = 0;
    p->AVEKERNEL = 20;
    p->GAMMA = 0.1;
    p->THETASEMAX = 1.412;
    p->PERTURB = 1;
    p->RELAXATION = 1;
    p->TIDALLY_STRIP_STARS = 1;
    p->TIDAL_TREATMENT = 1;
    p->orbit_r = 1.0e6;
    p->cenma_m = 0.0;
    p->apsides_max_iter = 100;
    p->apsides_precision = 1.0e-11;
    p->apsides_convergence = 5.0e-13;
    p->n_try = 50000;
    p->seed = 0;
    p->relax_fp32 = 0;
    p->relax_trig32 = 0;
    p->phi_sequential = 0;
    p->check_filters = 0;
}

// Sequential points of the potential replay a cluster may record (per chain):
// a few per binade crossed in practice; beyond this the cluster's potential
// is computed by the one-thread loop.
static long long phi_rec_cap(long long cap) { return 4096 + cap / 16; }

// Buckets of the radius index: about 16 stars each, 2^10 to 2^20.
static int ridx_buckets(long long cap)
{
    int B = 1024;
    while (B < (1 << 20) && (long long)B * 16 < cap) B <<= 1;
    return B;
}

int cmcg_create(cmcg_ctx **out, int nclusters, const long *capacity, const cmcg_params *params)
{
    if (!out || nclusters < 1 || !capacity || !params) return CMCG_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        fprintf(stderr, "cmcgpu: no CUDA device available; this library has no CPU fallback\n");
        return CMCG_ERR_CUDA;
    }
    for (int k = 0; k < nclusters; ++k) {
        if (capacity[k] < 1 || capacity[k] > (1L << 31) - 64) return CMCG_ERR_ARG;  // 32-bit star indices
        if (params[k].AVEKERNEL < 1 || params[k].AVEKERNEL > PMAX) return CMCG_ERR_ARG;
        if (params[k].relax_fp32 != params[0].relax_fp32) return CMCG_ERR_ARG;
        if (params[k].relax_trig32 != params[0].relax_trig32) return CMCG_ERR_ARG;
    }
    cmcg_ctx *c = new cmcg_ctx();
    c->ncl = nclusters;
    c->relax_fp32 = params[0].relax_fp32;
    c->relax_trig32 = params[0].relax_trig32;
    c->params.assign(params, params + nclusters);
    c->cap.resize(nclusters);
    c->off.resize(nclusters);
    long long tot = 0;
    for (int k = 0; k < nclusters; ++k) {
        c->cap[k] = capacity[k];
        c->off[k] = tot;
        long long stride = ((capacity[k] + 2 + 31) / 32) * 32;
        tot += stride;
    }
    c->total = tot;
    for (int k = 0; k < nclusters; ++k) {
        c->rec_total += phi_rec_cap(capacity[k]);
        c->ridx_total += ridx_buckets(capacity[k]) + 1;
        c->ridx_Bmax = std::max(c->ridx_Bmax, ridx_buckets(capacity[k]));
    }
    std::vector<int2> tabs[5];
    build_table(c->t128, c->cap, ORB_T, tabs[0]);
    build_table(c->t256, c->cap, RELAX_T, tabs[1]);
    build_table(c->t1024, c->cap, POT_T, tabs[2]);
    build_table(c->t2048, c->cap, SORT_T, tabs[3]);
    build_table(c->t4096, c->cap, 4096, tabs[4]);
    size_t bytes = 0;
    carve_all(c, nullptr, tabs, &bytes);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->arena, bytes) != cudaSuccess) {
        fprintf(stderr, "cmcgpu: cannot allocate %zu bytes of device memory\n", bytes);
        cudaGetLastError();
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return CMCG_ERR_NOMEM;
    }
    c->arena_bytes = bytes;
    carve_all(c, (char *)c->arena, tabs, &bytes);
    CK(cudaMemsetAsync(c->arena, 0, c->arena_bytes, c->stream));
    // cluster descriptors and tile tables
    c->h_cls.resize(nclusters);
    long long rec_off = 0, ridx_off = 0;
    for (int k = 0; k < nclusters; ++k) {
        Cluster &C = c->h_cls[k];
        const cmcg_params &p = params[k];
        memset(&C, 0, sizeof(C));
        C.off = c->off[k];
        C.cap = c->cap[k];
        C.sc = c->d_sc + k;
        C.p = p.AVEKERNEL;
        C.GAMMA = p.GAMMA;
        C.THETASEMAX = p.THETASEMAX;
        C.PERTURB = p.PERTURB;
        C.RELAXATION = p.RELAXATION;
        C.TIDALLY_STRIP_STARS = p.TIDALLY_STRIP_STARS;
        C.TIDAL_TREATMENT = p.TIDAL_TREATMENT;
        C.n_try = p.n_try;
        C.apsides_max_iter = p.apsides_max_iter;
        C.apsides_precision = p.apsides_precision;
        C.apsides_convergence = p.apsides_convergence;
        C.seed = p.seed;
        C.relax_fp32 = p.relax_fp32;
        C.phi_sequential = p.phi_sequential;
        C.check_filters = p.check_filters;
        C.rec_off = rec_off;
        C.rec_cap = phi_rec_cap(c->cap[k]);
        rec_off += C.rec_cap;
        C.ridx_off = ridx_off;
        C.ridx_B = ridx_buckets(c->cap[k]);
        ridx_off += C.ridx_B + 1;
    }
    CK(cudaMemcpyAsync(c->d_cls, c->h_cls.data(), nclusters * sizeof(Cluster), cudaMemcpyHostToDevice, c->stream));
    TileTable *tts[5] = {&c->t128, &c->t256, &c->t1024, &c->t2048, &c->t4096};
    for (int i = 0; i < 5; ++i) {
        CK(cudaMemcpyAsync(tts[i]->d_tiles, tabs[i].data(), tabs[i].size() * sizeof(int2), cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(tts[i]->d_first, tts[i]->first.data(), nclusters * sizeof(int), cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(tts[i]->d_count, tts[i]->count.data(), nclusters * sizeof(int), cudaMemcpyHostToDevice,
                           c->stream));
    }
    // grid of the cooperative tidal kernel: all co-resident blocks, at most one per tile
    int dev = 0, nsm = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(sort_onesweep_setup());
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tidal, TID_THREADS, 0));
    c->tidal_grid = std::max(1, std::min(c->t2048.ntiles, nsm * std::max(per_sm, 1)));
    c->posq_grid = 2 * nsm;
    c->nsm = nsm;
    {
        const int rc = alloc_net(c);
        if (rc) {
            cmcg_destroy(c);
            return rc;
        }
    }
    if (cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_sorted, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_ec3, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_ej, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&c->d_nout, (size_t)nclusters * sizeof(long long)) != cudaSuccess ||
        cudaHostAlloc((void **)&c->h_xfer, xfer_table_bytes(nclusters), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        cmcg_destroy(c);
        return CMCG_ERR_CUDA;
    }
    c->h_hx = (double **)(c->h_xfer + (size_t)XFER_PER_CLUSTER * nclusters);
    c->h_xn = (long long *)(c->h_hx + (size_t)4 * nclusters);
    CK(cudaStreamSynchronize(c->stream));
    *out = c;
    return CMCG_OK;
}

int cmcg_destroy(cmcg_ctx *c)
{
    if (!c) return CMCG_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int p = 0; p < 2; ++p) {
        if (c->gexec[p]) cudaGraphExecDestroy(c->gexec[p]);
        if (c->graph[p]) cudaGraphDestroy(c->graph[p]);
    }
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->arena) cudaFree(c->arena);
    if (c->net_mem) cudaFree(c->net_mem);
    if (c->lrn_mem) cudaFree(c->lrn_mem);
    for (int a = 0; a < HX_ALL; ++a)
        for (int p = 0; p < 2; ++p)
            if (c->hx[a][p]) cudaGraphExecDestroy(c->hx[a][p]);
    if (c->copy) cudaStreamDestroy(c->copy);
    for (cudaEvent_t e : {c->ev_sorted, c->ev_copied, c->ev_in, c->ev_ec3, c->ev_ej})
        if (e) cudaEventDestroy(e);
    if (c->d_nout) cudaFree(c->d_nout);
    if (c->h_xfer) cudaFreeHost(c->h_xfer);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return CMCG_OK;
}

int cmcg_load(cmcg_ctx *c, int k, long N, const double *r, const double *m, const double *vr, const double *vt,
              const int64_t *id)
{
    if (!c || k < 0 || k >= c->ncl || !r || !m || !vr || !vt) return CMCG_ERR_ARG;
    if (N < 2 * c->params[k].AVEKERNEL + 2) return CMCG_ERR_ARG;
    if (N > c->cap[k]) return CMCG_ERR_CAPACITY;
    const long long o = c->off[k];
    const cmcg_params &p = c->params[k];
    const long long NSTAR = p.N_STAR > 0 ? p.N_STAR : N;
    std::vector<double> tmp((size_t)N + 2);
    std::vector<long long> ids((size_t)N + 2, 0);
    // star_m: mass in N-body units times N_STAR (cmc_fits.c:99,123)
    tmp[0] = 0.0;
    for (long i = 0; i < N; ++i) tmp[i + 1] = m[i] * ((double)NSTAR);
    tmp[N + 1] = 0.0;
    CK(cudaMemcpy(c->f.m + o, tmp.data(), (N + 2) * sizeof(double), cudaMemcpyHostToDevice));
    tmp[0] = CMCG_ZERO;
    for (long i = 0; i < N; ++i) tmp[i + 1] = r[i];
    tmp[N + 1] = CMCG_SF_INFINITY;
    CK(cudaMemcpy(c->f.r + o, tmp.data(), (N + 2) * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemset(c->f.vr + o, 0, (N + 2) * sizeof(double)));
    CK(cudaMemset(c->f.vt + o, 0, (N + 2) * sizeof(double)));
    CK(cudaMemcpy(c->f.vr + o + 1, vr, N * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->f.vt + o + 1, vt, N * sizeof(double), cudaMemcpyHostToDevice));
    for (long i = 0; i < N; ++i) ids[i + 1] = id ? (long long)id[i] : (long long)(i + 1);
    CK(cudaMemcpy(c->f.id + o, ids.data(), (N + 2) * sizeof(long long), cudaMemcpyHostToDevice));
    Scalars s;
    memset(&s, 0, sizeof(s));
    s.N_MAX = N;
    s.N_MAX_NEW = N;
    s.N_STAR = NSTAR;
    s.tcount = 1;
    s.Mtotal = 1.0;
    s.orbit_r = p.orbit_r;
    s.madhoc = 1.0 / ((double)NSTAR);
    s.cenma_m = p.cenma_m;
    // constant over the run; formed on the host with the C library's pow and
    // log, as the reference forms it (cmc_evolution_thr.c:550)
    s.tid_alpha = 1.5 - 3.0 * pow(log(p.GAMMA * ((double)NSTAR)) / ((double)NSTAR), 0.25);
    CK(cudaMemcpy(c->d_sc + k, &s, sizeof(Scalars), cudaMemcpyHostToDevice));
    return CMCG_OK;
}

// Tables derived from star_r and star_phi (1/r and the FP32 copy), rebuilt
// after the host overwrites either array.
__global__ void k_refresh_tables(const Cluster *cls, Fields f, int k, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n + 1) return;
    const long long g = cls[k].off + i;
    const double r = f.r[g];
    f.inv_r[g] = __drcp_rn(r);
    f.rphif[g] = rphi_entry(r, f.phi[g]);
    if (i == 0) cls[k].sc->ridx_ok = 0;  // radii may have changed: search the whole table until rebuilt
}

// New star count after a host upload (the sentinel r[N+1] is copied separately).
__global__ void k_set_count(const Cluster *cls, int k, long long N)
{
    Scalars *sc = cls[k].sc;
    sc->N_MAX = N;
    sc->N_MAX_NEW = N;
    sc->ridx_ok = 0;
}

// Host exchange by kernel.  The four inputs the time step reads, for every
// cluster, go up in one launch that moves 8-byte words from the caller's
// pinned host arrays (addressed from the device through unified addressing)
// into the context's fields, in place of one cudaMemcpyAsync per array.  On
// this GPU a kernel reads and writes pinned host memory over NVLink-C2C as
// fast as the copy engines do (~200 GB/s each way); the launch replaces the
// per-copy set-up, which adds up over an ensemble's many small arrays.  The
// segments sit in order of their first chunk.
// (XferSeg and the chunk sizes: beside cmcg_ctx above)

__global__ void __launch_bounds__(XFER_THREADS) k_xfer(const XferSeg *__restrict__ seg, int nseg, long long nchunk)
{
    for (long long c = blockIdx.x; c < nchunk; c += gridDim.x) {
        int lo = 0, hi = nseg - 1;  // the last segment whose first chunk is <= c
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (seg[mid].c0 <= c)
                lo = mid;
            else
                hi = mid - 1;
        }
        const unsigned long long *src = seg[lo].src;
        unsigned long long *dst = seg[lo].dst;
        const long long n = seg[lo].n, i0 = (c - seg[lo].c0) * XFER_CHUNK + threadIdx.x;
        unsigned long long v[XFER_UNROLL];
#pragma unroll
        for (int u = 0; u < XFER_UNROLL; ++u) {
            const long long i = i0 + (long long)u * XFER_THREADS;
            if (i < n) v[u] = src[i];
        }
#pragma unroll
        for (int u = 0; u < XFER_UNROLL; ++u) {
            const long long i = i0 + (long long)u * XFER_THREADS;
            if (i < n) dst[i] = v[u];
        }
    }
}

// Every cluster's star count after the exchange's upload, and the sentinel
// star_r[N+1] = SF_INFINITY.
__global__ void k_set_counts(const Cluster *cls, Fields f, int nclusters, const long long *N)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nclusters) return;
    const long long n = N[k];
    if (n < 0 || n > cls[k].cap) return;  // the host checked; nothing outside the slice is written
    Scalars *sc = cls[k].sc;
    sc->N_MAX = n;
    sc->N_MAX_NEW = n;
    sc->ridx_ok = 0;
    f.r[cls[k].off + n + 1] = CMCG_SF_INFINITY;
}

// Host exchange: the caller's E and J travel into rnew and vrnew (which
// nothing reads before the orbits write them) while the relaxation runs.
// k_xchg_mark first fills E and J of stars 1..N with a bit pattern that the
// relaxation never writes (an all-ones NaN: the GPU's arithmetic returns the
// canonical NaN, sign bit clear); after the relaxation k_xchg_merge
// takes the staged pair wherever both still hold it.  Those are the stars the
// relaxation left alone, whose E and J put_stars would have set.
constexpr unsigned long long XCHG_MARK = ~0ull;
constexpr int XCHG_THREADS = 256;

__global__ void __launch_bounds__(XCHG_THREADS) k_xchg_mark(const Cluster *__restrict__ cls, Tiles tm, Fields f)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const long long N = C.sc->N_MAX, i0 = C.off + 1 + (long long)ct.y * POT_T;
    const long long n = N - (long long)ct.y * POT_T;  // stars of this tile with index <= N
    unsigned long long *E = (unsigned long long *)f.E, *J = (unsigned long long *)f.J;
    for (int q = threadIdx.x; q < POT_T && q < n; q += XCHG_THREADS) {
        E[i0 + q] = XCHG_MARK;
        J[i0 + q] = XCHG_MARK;
    }
}

__global__ void __launch_bounds__(XCHG_THREADS) k_xchg_merge(const Cluster *__restrict__ cls, Tiles tm, Fields f)
{
    const int2 ct = tm.tiles[blockIdx.x];
    const Cluster &C = cls[ct.x];
    if (!counts_ok(C)) return;
    const long long N = C.sc->N_MAX, i0 = C.off + 1 + (long long)ct.y * POT_T;
    const long long n = N - (long long)ct.y * POT_T;
    unsigned long long *E = (unsigned long long *)f.E, *J = (unsigned long long *)f.J;
    const unsigned long long *sE = (const unsigned long long *)f.rnew, *sJ = (const unsigned long long *)f.vrnew;
    for (int q = threadIdx.x; q < POT_T && q < n; q += XCHG_THREADS) {
        const long long g = i0 + q;
        if (E[g] == XCHG_MARK && J[g] == XCHG_MARK) {
            E[g] = sE[g];
            J[g] = sJ[g];
        }
    }
}

int cmcg_put_stars(cmcg_ctx *c, int k, long N, const double *r, const double *m, const double *vr, const double *vt,
                   const double *E, const double *J, const int64_t *id)
{
    if (!c || k < 0 || k >= c->ncl || !r || !m || !vr || !vt || !E || !J || !id) return CMCG_ERR_ARG;
    if (N > c->cap[k]) return CMCG_ERR_CAPACITY;
    if (N < 2 * c->params[k].AVEKERNEL + 2) return CMCG_ERR_ARG;
    const long long o = c->off[k] + 1;
    const size_t b = (size_t)N * sizeof(double);
    CK(cudaMemcpyAsync(c->f.r + o, r, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.m + o, m, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.vr + o, vr, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.vt + o, vt, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.E + o, E, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.J + o, J, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->f.id + o, id, (size_t)N * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
    static const double sentinel = CMCG_SF_INFINITY;
    CK(cudaMemcpyAsync(c->f.r + o + N, &sentinel, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_set_count<<<1, 1, 0, c->stream>>>(c->d_cls, k, (long long)N);
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

long cmcg_get_stars(cmcg_ctx *c, int k, long cap, double *r, double *m, double *vr, double *vt, double *E, double *J,
                    int64_t *id)
{
    if (!c || k < 0 || k >= c->ncl) return CMCG_ERR_ARG;
    long long N = 0;
    if (cudaMemcpyAsync(&N, &c->d_sc[k].N_MAX_NEW, sizeof(long long), cudaMemcpyDeviceToHost, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return CMCG_ERR_CUDA;
    if (N > cap) return CMCG_ERR_CAPACITY;
    const long long o = c->off[k] + 1;
    const size_t b = (size_t)N * sizeof(double);
    struct {
        double *dst;
        const double *src;
    } t[] = {{r, c->f.r}, {m, c->f.m}, {vr, c->f.vr}, {vt, c->f.vt}, {E, c->f.E}, {J, c->f.J}};
    for (auto &x : t)
        if (x.dst && cudaMemcpyAsync(x.dst, x.src + o, b, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
            return CMCG_ERR_CUDA;
    if (id && cudaMemcpyAsync(id, c->f.id + o, (size_t)N * sizeof(long long), cudaMemcpyDeviceToHost, c->stream) !=
                  cudaSuccess)
        return CMCG_ERR_CUDA;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return CMCG_ERR_CUDA;
    return (long)N;
}

}  // extern "C"

// ------------------------------------------------------------ launches ---
static int L_pot(cmcg_ctx *c)
{
    fam_begin(c, F_POT);
    const Tiles tv = c->t1024.view();
    const int nt = c->t1024.ntiles;
    k_pot_agg<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb);
    k_pot_carry<<<c->ncl, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->pb, c->ph, c->ncl);
    k_phi_cls12<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb, c->ph, c->tickets);
    k_phi_rec12<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb, c->ph, c->tickets);
    k_phi_cls3<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb, c->ph, c->tickets);
    k_phi_rec3<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb, c->ph, c->tickets);
    k_phi_final<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, c->pb, c->ph);
    k_phi_seq<<<c->ncl, 32, 0, c->stream>>>(c->d_cls, c->f, c->ph, c->ncl);
    k_ridx_build<<<dim3((unsigned)((c->ridx_Bmax + RIDX_THREADS) / RIDX_THREADS), (unsigned)c->ncl), RIDX_THREADS, 0,
                   c->stream>>>(c->d_cls, c->f, c->ph, c->ncl);
    fam_end(c);
    c->launches += 9;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

// end: the step's last kernel, which also does k_end_step's work
static int L_energy(cmcg_ctx *c, double *const *hx = nullptr, bool end = false)
{
    fam_begin(c, F_ENERGY);
    k_energy<<<c->t2048.ntiles, EN_THREADS, 0, c->stream>>>(c->d_cls, c->t2048.view(), c->f, c->partials,
                                                             c->tickets, hx, end ? 1 : 0);
    fam_end(c);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_begin(cmcg_ctx *c)
{
    fam_begin(c, F_BEGIN);
    k_begin_step<<<(c->ncl + 127) / 128, 128, 0, c->stream>>>(c->d_cls, c->ncl);
    fam_end(c);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_end(cmcg_ctx *c)
{
    fam_begin(c, F_END);
    k_end_step<<<(c->ncl + 127) / 128, 128, 0, c->stream>>>(c->d_cls, c->ncl);
    fam_end(c);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

// begin: the step's first kernel, which also does k_begin_step's work
static int L_timestep(cmcg_ctx *c, bool begin = false)
{
    fam_begin(c, F_TIMESTEP);
    k_timestep<<<c->t1024.ntiles, TS_THREADS, 0, c->stream>>>(c->d_cls, c->t1024.view(), c->f, c->partials, c->tickets,
                                                             begin ? 1 : 0);
    fam_end(c);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_relax(cmcg_ctx *c, double dt)
{
    fam_begin(c, F_RELAX);
    if (c->relax_fp32)
        k_relax32<<<c->t256.ntiles, RELAX_THREADS, 0, c->stream>>>(c->d_cls, c->t256.view(), c->f, c->partials,
                                                                    c->tickets, dt);
    else if (c->relax_trig32)
        k_relax64t<<<c->t256.ntiles, RELAX_THREADS, 0, c->stream>>>(c->d_cls, c->t256.view(), c->f, c->partials,
                                                                     c->tickets, dt);
    else
        (c->var[V_RELAX] ? k_relax64_lb4 : k_relax64)<<<c->t256.ntiles, RELAX_THREADS, 0, c->stream>>>(
            c->d_cls, c->t256.view(), c->f, c->partials, c->tickets, dt);
    fam_end(c);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_xchg(cmcg_ctx *c, bool merge)
{
    (merge ? k_xchg_merge : k_xchg_mark)<<<c->t1024.ntiles, XCHG_THREADS, 0, c->stream>>>(c->d_cls, c->t1024.view(),
                                                                                        c->f);
    c->launches += 1;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_orbit(cmcg_ctx *c)
{
    fam_begin(c, F_ORBIT);
    CK(cudaMemsetAsync(c->pq.count, 0, sizeof(unsigned int), c->stream));
    k_orbit_pre<<<c->t128.ntiles, ORB_T, 0, c->stream>>>(c->d_cls, c->t128.view(), c->f, c->pq);
    k_posq_scan<<<c->posq_grid, 256, 0, c->stream>>>(c->d_cls, c->f, c->pq);
    if (c->learn_mode == LEARN_OFF) {
        const int ov = c->var[V_ORBIT];
        if (ov < 2) {  // one block per tile, 5 or 4 blocks per SM
            (ov ? k_orbit_lb4 : k_orbit)<<<c->t128.ntiles, ORB_T, 0, c->stream>>>(
                c->d_cls, c->t128.view(), c->f, c->partials, c->tickets, c->pq);
        } else {  // persistent: as many blocks as the SMs hold, tiles taken from a counter
            const int per_sm = ov == 2 ? 5 : 4;
            const int grid = (int)std::min<long long>(c->t128.ntiles, (long long)per_sm * c->nsm);
            CK(cudaMemsetAsync(c->orbit_next, 0, sizeof(unsigned int), c->stream));
            (ov == 2 ? k_orbit_pers : k_orbit_pers_lb4)<<<grid, ORB_T, 0, c->stream>>>(
                c->d_cls, c->t128.view(), c->f, c->partials, c->tickets, c->pq, c->orbit_next);
        }
        c->launches += 3;
    } else {
        // apsides and features; the network on every star slot; the sampling
        Learn L = c->lrn;
        L.mode = c->learn_mode;
        L.kappa = c->learn_kappa;
        CK(cudaMemsetAsync(L.stats, 0, LSTAT_N * sizeof(unsigned long long), c->stream));
        k_orbit_aps<<<c->t128.ntiles, ORB_T, 0, c->stream>>>(c->d_cls, c->t128.view(), c->f, c->partials,
                                                             c->tickets, c->pq, L);
        if (c->learn_mode == LEARN_ON) {
            fam_end(c);
            fam_begin(c, F_MLP);
            const long long ntl = (c->total + MLP_T - 1) / MLP_T;
            const int grid = (int)std::min<long long>(ntl, (long long)kMlpGrid[c->var[V_MLP_GRID]] * c->nsm);
            k_mlp_infer<<<grid, MLP_T, MLP_INFER_SMEM, c->stream>>>(c->net, L.feat, c->total, L.prop, L.stride,
                                                                    nullptr);
            c->launches += 1;
            fam_end(c);
            fam_begin(c, F_ORBIT);
        }
        (c->var[V_LEARN] ? k_orbit_learn_lb4 : k_orbit_learn)<<<c->t128.ntiles, ORB_T, 0, c->stream>>>(
            c->d_cls, c->t128.view(), c->f, c->partials, c->tickets, c->pq, L);
        c->launches += 4;
    }
    fam_end(c);
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

// One cooperative launch: every block of the grid is resident at once, as the
// kernel's grid barrier requires (the launch fails rather than run otherwise).
static int L_tidal(cmcg_ctx *c)
{
    fam_begin(c, F_TIDAL);
    Tiles tv = c->t2048.view();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)c->tidal_grid);
    cfg.blockDim = dim3(TID_THREADS);
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // arrivals start at zero even after a barrier that timed out; the
    // generation word is left alone
    CK(cudaMemsetAsync(c->gbar, 0, sizeof(unsigned int), c->stream));
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_tidal, (const Cluster *)c->d_cls, tv, c->f, c->partials,
                                             c->gbar, c->ncl);
    fam_end(c);
    c->launches += 1;
    if (e != cudaSuccess) {
        fprintf(stderr, "cmcgpu: tidal stripping launch failed: %s\n", cudaGetErrorString(e));
        return CMCG_ERR_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static void swap_sorted(cmcg_ctx *c)
{
    std::swap(c->f.r, c->f.r2);
    std::swap(c->f.m, c->f.m2);
    std::swap(c->f.id, c->f.id2);
    std::swap(c->f.ec_pre, c->f.ec_pre2);
    c->parity ^= 1;
}

static int L_sort(cmcg_ctx *c)
{
    fam_begin(c, F_SORT);
    k_sort_prep<<<c->t2048.ntiles, SORT_THREADS, 0, c->stream>>>(c->d_cls, c->t2048.view(), c->f, c->sb,
                                                                   c->partials, c->tickets);
    k_sort_ghist<<<c->t2048.ntiles, SORT_THREADS, 0, c->stream>>>(c->d_cls, c->t2048.view(), c->f, c->sb);
    // digit passes over 4096-, 2048- or 1024-key tiles (autotuner)
    const int sv = c->var[V_SORT_TILE];
    const TileTable &ost = sv == 1 ? c->t2048 : sv == 2 ? c->t1024 : c->t4096;
    for (int p = 0; p < SORT_MAX_PASSES; ++p)
        launch_sort_onesweep(sv == 1 ? 2048 : sv == 2 ? 1024 : 4096, ost.ntiles, c->stream, c->d_cls, ost.view(), c->f,
                             c->sb, p);
    // the payload gather, placing runs of up to FIX_SHORT keys, 256, 128 or
    // 1024 stars per block (autotuner); then the longer runs
    {
        const int gv = c->var[V_GATHER_TILE];
        const TileTable &gt = gv == 1 ? c->t128 : gv == 2 ? c->t1024 : c->t256;
        launch_sort_gather(gv == 1 ? 128 : gv == 2 ? 1024 : 256, gt.ntiles, c->stream, c->d_cls, gt.view(), c->f, c->sb);
    }
    // the long runs spread over the cluster's 4096-key tiles: at 10^8 stars, with
    // ~6 stars to a 24-bit prefix, runs longer than FIX_SHORT number in the
    // thousands (one block per cluster took 9 s a step there)
    k_sort_fix_long<<<c->t4096.ntiles, SORT_THREADS, 0, c->stream>>>(c->d_cls, c->t4096.view(), c->sb, c->f,
                                                                      c->tickets);
    fam_end(c);
    c->launches += 4 + SORT_MAX_PASSES;
    swap_sorted(c);
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

static int L_ec3(cmcg_ctx *c, double *const *hx = nullptr)
{
    fam_begin(c, F_EC3);
    k_ec3<<<c->t256.ntiles, EC3_T, 0, c->stream>>>(c->d_cls, c->t256.view(), c->f, c->eb, hx);
    k_ec3_fix<<<c->ncl, EC3_FIX_THREADS, 0, c->stream>>>(c->d_cls, c->f, c->eb, c->ncl, hx);
    fam_end(c);
    c->launches += 2;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

#define RUN(x)                \
    do {                      \
        int rc_ = (x);        \
        if (rc_) return rc_;  \
    } while (0)

static int issue_part(cmcg_ctx *c, int part)
{
    switch (part) {
    case 0:
        RUN(L_timestep(c, true));
        break;
    case 1:
        RUN(L_relax(c, -1.0));
        RUN(L_orbit(c));
        RUN(L_tidal(c));
        RUN(L_sort(c));
        break;
    case 2:
        RUN(L_pot(c));
        RUN(L_ec3(c));
        break;
    case HX_XRELAX:
        RUN(L_xchg(c, false));
        RUN(L_relax(c, -1.0));
        break;
    case HX_XSORT:
        RUN(L_xchg(c, true));
        RUN(L_orbit(c));
        RUN(L_tidal(c));
        RUN(L_sort(c));
        break;
    case HX_XTAIL:
        RUN(L_pot(c));
        RUN(L_ec3(c, c->d_hx));
        RUN(L_energy(c, c->d_hx, true));
        break;
    default:
        RUN(L_energy(c, nullptr, true));
    }
    return CMCG_OK;
}

static int issue_step(cmcg_ctx *c)
{
    for (int part = 0; part < HX_PARTS; ++part) RUN(issue_part(c, part));
    return CMCG_OK;
}

__global__ void k_gather_counts(const Cluster *cls, int nclusters, long long *out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nclusters) out[k] = cls[k].sc->N_MAX_NEW;
}

// Runs part `part` of a step from a graph captured at the current parity
// (capturing it first).  Parts HX_SORT and HX_XSORT end with the sort's
// pointer swap, which the host mirrors after the launch.
static int run_part_graph(cmcg_ctx *c, int part)
{
    const int p = c->parity;
    if (!c->hx[part][p]) {
        const bool prof = c->profile;
        c->profile = false;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const long l0 = c->launches;
        const int rc = issue_part(c, part);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        c->profile = prof;
        c->hx_launches[part][p] = c->launches - l0;
        c->launches = l0;
        const bool sorts = part == HX_SORT || part == HX_XSORT;
        if (sorts && c->parity != p) swap_sorted(c);  // the capture ran no kernel: undo the swap
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return CMCG_ERR_CUDA;
        const cudaError_t ei = cudaGraphInstantiate(&c->hx[part][p], g, 0);
        cudaGraphDestroy(g);
        CK(ei);
    }
    CK(cudaGraphLaunch(c->hx[part][p], c->stream));
    c->launches += c->hx_launches[part][p];
    if (part == HX_SORT || part == HX_XSORT) swap_sorted(c);
    return CMCG_OK;
}

extern "C" {

int cmcg_initialize(cmcg_ctx *c)
{
    if (!c) return CMCG_ERR_ARG;
    RUN(L_pot(c));
    RUN(L_energy(c));
    CK(cudaStreamSynchronize(c->stream));
    std::vector<Scalars> s(c->ncl);
    CK(cudaMemcpy(s.data(), c->d_sc, c->ncl * sizeof(Scalars), cudaMemcpyDeviceToHost));
    for (auto &x : s) x.Etot_ini = x.Etot;
    CK(cudaMemcpy(c->d_sc, s.data(), c->ncl * sizeof(Scalars), cudaMemcpyHostToDevice));
    return CMCG_OK;
}

int cmcg_begin_step(cmcg_ctx *c) { return c ? L_begin(c) : CMCG_ERR_ARG; }
int cmcg_calc_timestep(cmcg_ctx *c) { return c ? L_timestep(c) : CMCG_ERR_ARG; }
int cmcg_dynamics_apply(cmcg_ctx *c, double dt) { return c ? L_relax(c, dt) : CMCG_ERR_ARG; }
int cmcg_new_orbits_calculate(cmcg_ctx *c) { return c ? L_orbit(c) : CMCG_ERR_ARG; }
int cmcg_tidally_strip_stars(cmcg_ctx *c) { return c ? L_tidal(c) : CMCG_ERR_ARG; }
int cmcg_qsorts_new(cmcg_ctx *c) { return c ? L_sort(c) : CMCG_ERR_ARG; }
int cmcg_calc_potential(cmcg_ctx *c) { return c ? L_pot(c) : CMCG_ERR_ARG; }
int cmcg_energy_conservation3(cmcg_ctx *c) { return c ? L_ec3(c) : CMCG_ERR_ARG; }
int cmcg_compute_energy(cmcg_ctx *c) { return c ? L_energy(c) : CMCG_ERR_ARG; }
int cmcg_end_step(cmcg_ctx *c) { return c ? L_end(c) : CMCG_ERR_ARG; }

int cmcg_use_graph(cmcg_ctx *c, int enable)
{
    if (!c) return CMCG_ERR_ARG;
    c->use_graph = enable != 0;
    return CMCG_OK;
}

static int capture_pair(cmcg_ctx *c)
{
    const bool prof = c->profile;
    c->profile = false;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const long l0 = c->launches;
    int rc = issue_step(c);
    if (!rc) rc = issue_step(c);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->profile = prof;
    const int p = c->parity;  // two swaps: back at the parity captured at
    c->graph_launches[p] = c->launches - l0;  // kernel nodes in the two-step graph
    c->launches = l0;
    if (rc) return rc;
    if (e != cudaSuccess) return CMCG_ERR_CUDA;
    c->graph[p] = g;
    CK(cudaGraphInstantiate(&c->gexec[p], g, 0));
    c->graph_ready[p] = true;
    return CMCG_OK;
}

int cmcg_step(cmcg_ctx *c) { return cmcg_run(c, 1); }

int cmcg_run(cmcg_ctx *c, int nsteps)
{
    if (!c || nsteps < 0) return CMCG_ERR_ARG;
    const long l0 = c->launches;
    int done = 0;
    if (c->use_graph && !c->profile && nsteps >= 2) {
        const int p = c->parity;
        if (!c->graph_ready[p]) RUN(capture_pair(c));
        // one graph holds two steps, which bring the pointer parity back to p
        while (nsteps - done >= 2) {
            CK(cudaGraphLaunch(c->gexec[p], c->stream));
            c->launches += c->graph_launches[p];
            done += 2;
        }
    }
    // single steps (and an odd last step) from the four part graphs
    const bool parts = c->use_graph && !c->profile;
    for (; done < nsteps; ++done) {
        if (parts) {
            for (int part = 0; part < HX_PARTS; ++part) RUN(run_part_graph(c, part));
        } else {
            RUN(issue_step(c));
        }
    }
    c->launches_last = c->launches - l0;
    return CMCG_OK;
}

int cmcg_synchronize(cmcg_ctx *c)
{
    if (!c) return CMCG_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    return CMCG_OK;
}

long cmcg_launch_count(cmcg_ctx *c) { return c ? c->launches_last : -1; }

void *cmcg_stream(cmcg_ctx *c) { return c ? (void *)c->stream : nullptr; }

int cmcg_profile(cmcg_ctx *c, int enable)
{
    if (!c) return CMCG_ERR_ARG;
    c->profile = enable != 0;
    return CMCG_OK;
}

int cmcg_kernel_time(cmcg_ctx *c, const char *family, double *ms_total, long *launches)
{
    if (!c || !family) return CMCG_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    for (const ProfRec &p : c->prof) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        c->fam_ms[p.fam] += ms;
        c->fam_n[p.fam] += 1;
    }
    c->prof.clear();
    c->ev_next = 0;
    if (!strcmp(family, "reset")) {
        for (int i = 0; i < F_COUNT; ++i) {
            c->fam_ms[i] = 0.0;
            c->fam_n[i] = 0;
        }
        return CMCG_OK;
    }
    for (int i = 0; i < F_COUNT; ++i) {
        if (!strcmp(family, kFamilyNames[i])) {
            if (ms_total) *ms_total = c->fam_ms[i];
            if (launches) *launches = c->fam_n[i];
            return CMCG_OK;
        }
    }
    return CMCG_ERR_ARG;
}

int cmcg_diagnostics(cmcg_ctx *c, int k, const double *mass_pc, int n_pc, int bh_include, double minimum_r,
                     cmcg_diag *out)
{
    if (!c || k < 0 || k >= c->ncl || !out || n_pc < 0 || n_pc > CMCG_MASS_PC_MAX || (n_pc > 0 && !mass_pc))
        return CMCG_ERR_ARG;
    static_assert(CMCG_MASS_PC_MAX == DIAG_PC_MAX, "one limit on the mass fractions");
    for (int i = 0; i < n_pc; ++i)
        if (!(mass_pc[i] >= 0.0) || (i > 0 && !(mass_pc[i] >= mass_pc[i - 1]))) return CMCG_ERR_ARG;
    DiagDev h;
    memset(&h, 0, sizeof(h));
    h.n_pc = n_pc;
    h.bh_include = bh_include ? 1 : 0;
    h.minimum_r = minimum_r;
    h.status = CMCG_ERR_STATE;  // cleared by the last block of k_diag_central
    for (int i = 0; i < n_pc; ++i) h.pc[i] = mass_pc[i];
    CK(cudaMemcpyAsync(c->d_diag, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    const Tiles tv = c->t1024.view();
    const int b0 = c->t1024.first[k], nt = c->t1024.count[k];
    DiagScratch ds;
    ds.col[0] = c->pb.sapx;
    ds.col[1] = c->pb.mapx;
    ds.col[2] = c->pb.papx;
    ds.col[3] = c->pb.t;
    ds.col[4] = reinterpret_cast<double *>(c->sb.keys[0]);
    k_diag_sum<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, b0, c->partials);
    k_diag_carry<<<1, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, k, b0, nt, c->partials);
    k_diag_prefix<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, b0, c->partials, ds);
    k_diag_find<<<1, POT_THREADS, 0, c->stream>>>(c->d_cls, c->f, k, ds, c->d_diag);
    k_diag_central<<<nt, POT_THREADS, 0, c->stream>>>(c->d_cls, tv, c->f, k, b0, nt, c->partials, c->tickets, ds,
                                                      c->d_diag);
    CK(cudaGetLastError());
    Scalars sc;
    CK(cudaMemcpyAsync(&h, c->d_diag, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&sc, c->d_sc + k, sizeof(sc), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    memset(out, 0, sizeof(*out));
    out->TotalTime = sc.TotalTime;
    out->Dt = sc.Dt;
    out->tcount = (long)sc.tcount;
    out->N_MAX = (long)sc.N_MAX;
    out->Mtotal = sc.Mtotal;
    out->Etot = sc.Etot;
    out->KE = sc.KE;
    out->PE = sc.PE;
    out->E_cenma = sc.cenma_E;
    out->Eescaped = sc.Eescaped;
    out->Eoops = sc.Eoops;
    out->max_r = sc.max_r;
    out->nave = (long)h.nave;
    out->rh = h.rh;
    out->rho_0 = h.rho;
    out->v0_rms = h.v_rms;
    out->core_radius = h.rc;
    out->rc_nb = h.rc_nb;
    out->m_ave = h.m_ave;
    out->n_central = h.n;
    out->rc_spitzer = h.rc_spitzer;
    out->N_core = h.N_core;
    out->N_core_nb = h.N_core_nb;
    out->Trc = h.Trc;
    out->n_pc = n_pc;
    out->n_set = h.n_set;
    for (int i = 0; i < n_pc; ++i) {
        out->mass_pc[i] = mass_pc[i];
        out->mass_r[i] = h.mass_r[i];
        out->ave_mass_r[i] = h.ave_mass_r[i];
        out->no_star_r[i] = h.no_star_r[i];
        out->densities_r[i] = h.densities_r[i];
        out->ke_rad_r[i] = h.ke_rad_r[i];
        out->ke_tan_r[i] = h.ke_tan_r[i];
        out->v2_rad_r[i] = h.v2_rad_r[i];
        out->v2_tan_r[i] = h.v2_tan_r[i];
    }
    return h.status ? h.status : CMCG_OK;
}

// snprintf into buf at *len; false once the buffer is full
static bool append(char *buf, long cap, long *len, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    const int n = vsnprintf(buf + *len, (size_t)(cap - *len), fmt, ap);
    va_end(ap);
    if (n < 0 || *len + n >= cap) return false;
    *len += n;
    return true;
}

long cmcg_format_dyn_line(const cmcg_diag *a, const cmcg_diag *d, char *buf, long cap)
{
    if (!a || !d || !buf || cap < 1) return -1;
    long len = 0;
    buf[0] = 0;
    // PrintFileOutput, cmc_io.c:320-323; without binaries and stellar evolution
    // Etotal.Eint, Etotal.Eb, Ebescaped, Eintescaped, DMse and DMrejuv are 0
    const double z = 0.0;
    if (!append(buf, cap, &len,
                "%.8g %.8g %ld %ld %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g "
                "%.8g %.8g %.8g %.8g %.8g %.8g %.8g %.8g\n",
                d->TotalTime, d->Dt, d->tcount, d->N_MAX, d->Mtotal, -2.0 * d->KE / d->PE, a->N_core,
                a->core_radius, d->max_r, d->Etot, d->KE, d->PE, z, z, d->E_cenma, d->Eescaped, z, z, d->Eoops,
                d->Etot + d->Eoops, d->rh, a->rho_0, a->rc_spitzer, a->v0_rms, a->rc_nb, z, z, a->N_core_nb))
        return -1;
    return len;
}

long cmcg_format_lagrad_line(const cmcg_diag *d, char *buf, long cap)
{
    if (!d || !buf || cap < 1) return -1;
    long len = 0;
    buf[0] = 0;
    if (!append(buf, cap, &len, "%.9e ", d->TotalTime)) return -1;
    for (int i = 0; i < d->n_pc; ++i)
        if (!append(buf, cap, &len, "%e ", d->mass_r[i])) return -1;
    if (!append(buf, cap, &len, "\n")) return -1;
    return len;
}

long cmcg_format_dyn_header(char *buf, long cap)
{
    if (!buf || cap < 1) return -1;
    long len = 0;
    buf[0] = 0;
    // cmc_io.c:2346-2347
    if (!append(buf, cap, &len, "# Dynamical information [code units]\n") ||
        !append(buf, cap, &len,
                "#1:t #2:Dt #3:tcount #4:N #5:M #6:VR #7:N_c #8:r_c #9:r_max #10:Etot #11:KE #12:PE "
                "#13:Etot_int #14:Etot_bin #15:E_cenma #16:Eesc #17:Ebesc #18:Eintesc #19:Eoops #20:Etot+Eoops "
                "#21:r_h #22:rho_0 #23:rc_spitzer #24:v0_rms #25:rc_nb #26.DMse(MSUN) #27.DMrejuv(MSUN) "
                "#28.N_c_nb\n"))
        return -1;
    return len;
}

long cmcg_format_lagrad_header(const double *mass_pc, int n_pc, char *buf, long cap)
{
    if (!buf || cap < 1 || n_pc < 0 || (n_pc > 0 && !mass_pc)) return -1;
    long len = 0;
    buf[0] = 0;
    // cmc_io.c:2294, 2306, 2319, 2332
    if (!append(buf, cap, &len, "# Lagrange radii [code units]\n") || !append(buf, cap, &len, "#1:t"))
        return -1;
    for (long i = 0; i < n_pc; ++i)
        if (!append(buf, cap, &len, " %ld:r(%g)", i + 2, mass_pc[i])) return -1;
    if (!append(buf, cap, &len, "\n")) return -1;
    return len;
}

int cmcg_potential(cmcg_ctx *c, int k, double r, double *out)
{
    if (!c || k < 0 || k >= c->ncl || !out) return CMCG_ERR_ARG;
    k_potential_query<<<1, 1, 0, c->stream>>>(c->d_cls, c->f, k, r, c->d_query);
    double h[2];
    CK(cudaMemcpyAsync(h, c->d_query, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *out = h[0];
    return h[1] != 0.0 ? CMCG_ERR_FINDZERO_R : CMCG_OK;
}

}  // extern "C"

// ------------------------------------------------------------ field access
static double *star_field(cmcg_ctx *c, const char *name, bool *global)
{
    *global = false;
    Fields &f = c->f;
    struct {
        const char *n;
        double *p;
        bool g;
    } tab[] = {{"r", f.r, false},         {"m", f.m, false},           {"vr", f.vr, false},
               {"vt", f.vt, false},       {"E", f.E, false},           {"J", f.J, false},
               {"vr_rel", f.vr_rel, false}, {"vt_rel", f.vt_rel, false}, {"rnew", f.rnew, false},
               {"vrnew", f.vrnew, false}, {"vtnew", f.vtnew, false},   {"X", f.X, false},
               {"Y", f.Y, false},         {"r_peri", f.r_peri, false}, {"r_apo", f.r_apo, false},
               {"rOld", f.rOld, false},   {"ec_pre", f.ec_pre, false}, {"phi", f.phi, false},
               {"star_r", f.r, true},     {"star_m", f.m, true},       {"star_phi", f.phi, true},
               {"sigma_r", f.sigma_r, true}, {"sigma", f.sigma, true}, {"inv_r", f.inv_r, true}};
    for (auto &t : tab)
        if (!strcmp(name, t.n)) {
            *global = t.g;
            return t.p;
        }
    return nullptr;
}

static int read_scalars(cmcg_ctx *c, int k, Scalars *s)
{
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(s, c->d_sc + k, sizeof(Scalars), cudaMemcpyDeviceToHost));
    return CMCG_OK;
}

extern "C" {

long cmcg_nstars(cmcg_ctx *c, int k)
{
    if (!c || k < 0 || k >= c->ncl) return -1;
    Scalars s;
    if (read_scalars(c, k, &s)) return -1;
    return (long)s.N_MAX_NEW;
}

long cmcg_get_field(cmcg_ctx *c, int k, const char *name, double *out, long cap)
{
    if (!c || k < 0 || k >= c->ncl || !name || !out) return -1;
    bool g;
    double *p = star_field(c, name, &g);
    if (!p) return -1;
    Scalars s;
    if (read_scalars(c, k, &s)) return -1;
    long n = g ? (long)s.N_MAX + 2 : (long)s.N_MAX_NEW;
    if (n > cap) n = cap;
    const long long o = c->off[k] + (g ? 0 : 1);
    if (cudaMemcpy(out, p + o, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return n;
}

long cmcg_set_field(cmcg_ctx *c, int k, const char *name, const double *in, long n)
{
    if (!c || k < 0 || k >= c->ncl || !name || !in) return -1;
    bool g;
    double *p = star_field(c, name, &g);
    if (!p) return -1;
    if (n > c->cap[k] + (g ? 2 : 0)) n = c->cap[k] + (g ? 2 : 0);
    const long long o = c->off[k] + (g ? 0 : 1);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return -1;
    if (cudaMemcpy(p + o, in, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return -1;
    if (g && (p == c->f.r || p == c->f.phi)) {
        const long long nn = n - 2;  // global arrays span 0..N+1
        k_refresh_tables<<<(unsigned)((nn + 2 + 255) / 256), 256, 0, c->stream>>>(c->d_cls, c->f, k, nn);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return -1;
    }
    return n;
}

long cmcg_get_ids(cmcg_ctx *c, int k, int64_t *out, long cap)
{
    if (!c || k < 0 || k >= c->ncl || !out) return -1;
    Scalars s;
    if (read_scalars(c, k, &s)) return -1;
    long n = (long)s.N_MAX_NEW;
    if (n > cap) n = cap;
    if (cudaMemcpy(out, c->f.id + c->off[k] + 1, n * sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return n;
}

#define SCALAR_TABLE(X)                                                                                    \
    X(Mtotal) X(Rtidal) X(orbit_r) X(madhoc) X(cenma_m) X(cenma_E) X(Dt) X(Prev_Dt) X(TotalTime) X(max_r)    \
        X(TidalMassLoss) X(TidalMassLoss_old) X(OldTidalMassLoss) X(DTidalMassLoss) X(Eescaped) X(Jescaped) \
            X(Etidal) X(Eoops) X(Eescaped_old) X(Jescaped_old) X(Etidal_old) X(Etot) X(KE) X(PE) X(Etot_ini) \
                X(phi_rtidal)

int cmcg_get_scalar(cmcg_ctx *c, int k, const char *name, double *out)
{
    if (!c || k < 0 || k >= c->ncl || !name || !out) return CMCG_ERR_ARG;
    Scalars s;
    RUN(read_scalars(c, k, &s));
#define X(n)                  \
    if (!strcmp(name, #n)) {  \
        *out = (double)s.n;   \
        return CMCG_OK;       \
    }
    SCALAR_TABLE(X)
#undef X
    struct {
        const char *n;
        double v;
    } ints[] = {{"N_MAX", (double)s.N_MAX},         {"N_MAX_NEW", (double)s.N_MAX_NEW},
                {"N_STAR", (double)s.N_STAR},       {"tcount", (double)s.tcount},
                {"Nrel", (double)s.Nrel},           {"Nrelbeta0", (double)s.Nrelbeta[0]},
                {"Nrelbeta1", (double)s.Nrelbeta[1]}, {"Nrelbeta2", (double)s.Nrelbeta[2]},
                {"Nrelbeta3", (double)s.Nrelbeta[3]}, {"n_excess", (double)s.n_excess},
                {"tidal_iters", (double)s.tidal_iters}, {"err", (double)s.err},
                {"qaverelbeta0", s.qaverelbeta[0]}, {"maverelbeta0", s.maverelbeta[0]},
                {"raverelbeta0", s.raverelbeta[0]},
                {"phi_nsp1", (double)s.phi_nsp[0]}, {"phi_nsp2", (double)s.phi_nsp[1]},
                {"phi_nsp3", (double)s.phi_nsp[2]}, {"phi_fallback", (double)s.phi_fallback}};
    for (auto &t : ints)
        if (!strcmp(name, t.n)) {
            *out = t.v;
            return CMCG_OK;
        }
    return CMCG_ERR_ARG;
}

int cmcg_set_scalar(cmcg_ctx *c, int k, const char *name, double v)
{
    if (!c || k < 0 || k >= c->ncl || !name) return CMCG_ERR_ARG;
    Scalars s;
    RUN(read_scalars(c, k, &s));
    bool hit = false;
#define X(n)                  \
    if (!strcmp(name, #n)) {  \
        s.n = v;              \
        hit = true;           \
    }
    SCALAR_TABLE(X)
#undef X
    if (!strcmp(name, "tcount")) {
        s.tcount = (long long)v;
        hit = true;
    }
    if (!hit) return CMCG_ERR_ARG;
    CK(cudaMemcpy(c->d_sc + k, &s, sizeof(Scalars), cudaMemcpyHostToDevice));
    return CMCG_OK;
}

int cmcg_last_error(cmcg_ctx *c, int *cluster, long *index)
{
    if (!c) return CMCG_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        fprintf(stderr, "cmcgpu: stream error: %s\n", cudaGetErrorString(e));
        return CMCG_ERR_CUDA;
    }
    std::vector<Scalars> s(c->ncl);
    CK(cudaMemcpy(s.data(), c->d_sc, c->ncl * sizeof(Scalars), cudaMemcpyDeviceToHost));
    for (int k = 0; k < c->ncl; ++k) {
        if (s[k].err) {
            const int code = s[k].err;
            if (cluster) *cluster = k;
            if (index) *index = (long)s[k].err_index;
            s[k].err = 0;
            s[k].err_index = 0;
            CK(cudaMemcpy(c->d_sc + k, &s[k], sizeof(Scalars), cudaMemcpyHostToDevice));
            return code;
        }
    }
    return CMCG_OK;
}

// Host copy of the device's counter-based draw (same keying as the kernels).
double cmcg_draw(uint64_t seed, long tcount, int site, int64_t id, uint32_t n, int word)
{
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32) ^ (uint32_t)tcount;
    uint64_t uid = (uint64_t)id;
    uint32_t c0 = (uint32_t)uid, c1 = (uint32_t)(uid >> 32), c2 = (uint32_t)site, c3 = n;
    for (int i = 0; i < 10; ++i) {
        if (i > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0;
        c1 = (uint32_t)p1;
        c2 = n2;
        c3 = (uint32_t)p0;
    }
    const uint32_t w[4] = {c0, c1, c2, c3};
    return w[word & 3] / 4294967296.0;
}

// ---------------------------------------------------- learned proposal --
static uint16_t f2bf(float x)  // round to nearest even (finite inputs)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float bf2f(uint16_t h)
{
    const uint32_t u = (uint32_t)h << 16;
    float x;
    memcpy(&x, &u, 4);
    return x;
}
static void drop_graphs(cmcg_ctx *c)
{
    for (int p = 0; p < 2; ++p) {
        if (c->gexec[p]) cudaGraphExecDestroy(c->gexec[p]);
        if (c->graph[p]) cudaGraphDestroy(c->graph[p]);
        c->gexec[p] = nullptr;
        c->graph[p] = nullptr;
        c->graph_ready[p] = false;
        for (int a = 0; a < HX_ALL; ++a) {
            if (c->hx[a][p]) cudaGraphExecDestroy(c->hx[a][p]);
            c->hx[a][p] = nullptr;
        }
    }
}
static int net_status(cmcg_ctx *c)
{
    int st = 0;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(&st, c->net.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        const int z = 0;
        CK(cudaMemcpy(c->net.status, &z, sizeof(int), cudaMemcpyHostToDevice));
        return st;
    }
    return CMCG_OK;
}
// Device buffers of a training or inference set (features as BF16).
struct MlpSet {
    void *mem = nullptr;
    uint4 *feat = nullptr;
    int *bin = nullptr, *ntrial = nullptr;
    ~MlpSet()
    {
        if (mem) cudaFree(mem);
    }
};
static int upload_set(cmcg_ctx *c, MlpSet &S, const float *feat, const int *bin, const int *ntrial, long n,
                      size_t extra, void **extra_ptr)
{
    const size_t fb = ((size_t)n * 16 + 255) & ~(size_t)255, ib = ((size_t)n * 4 + 255) & ~(size_t)255;
    if (cudaMalloc(&S.mem, fb + 2 * ib + extra) != cudaSuccess) {
        cudaGetLastError();
        return CMCG_ERR_NOMEM;
    }
    S.feat = (uint4 *)S.mem;
    S.bin = (int *)((char *)S.mem + fb);
    S.ntrial = (int *)((char *)S.mem + fb + ib);
    if (extra_ptr) *extra_ptr = (char *)S.mem + fb + 2 * ib;
    std::vector<uint16_t> h((size_t)n * MLP_IN);
    for (size_t i = 0; i < h.size(); ++i) h[i] = f2bf(feat[i]);
    CK(cudaMemcpy(S.feat, h.data(), h.size() * 2, cudaMemcpyHostToDevice));
    if (bin) CK(cudaMemcpy(S.bin, bin, (size_t)n * 4, cudaMemcpyHostToDevice));
    if (ntrial) CK(cudaMemcpy(S.ntrial, ntrial, (size_t)n * 4, cudaMemcpyHostToDevice));
    return CMCG_OK;
}

int cmcg_set_learned(cmcg_ctx *c, int mode, double kappa)
{
    if (!c || mode < LEARN_OFF || mode > LEARN_COLLECT || !(kappa > 0.0)) return CMCG_ERR_ARG;
    if (mode != LEARN_OFF) RUN(ensure_learn(c));
    if (mode != c->learn_mode || kappa != c->learn_kappa) drop_graphs(c);  // another launch sequence
    c->learn_mode = mode;
    c->learn_kappa = kappa;
    return CMCG_OK;
}

int cmcg_mlp_set_params(cmcg_ctx *c, const float *params)
{
    if (!c || !params) return CMCG_ERR_ARG;
    CK(cudaMemcpy(c->net.w, params, MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemset(c->net.m, 0, MLP_NPARAM * sizeof(float)));
    CK(cudaMemset(c->net.v, 0, MLP_NPARAM * sizeof(float)));
    c->adam_t = 0;
    k_mlp_pack<<<8, 256, 0, c->stream>>>(c->net);
    CK(cudaGetLastError());
    return net_status(c);
}

int cmcg_mlp_get_params(cmcg_ctx *c, float *params)
{
    if (!c || !params) return CMCG_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(params, c->net.w, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return CMCG_OK;
}

// Uniform initialisation, +-sqrt(6 / fan_in) (+-0.1 sqrt(6 / fan_in) for the
// output layer, so the first proposals are near uniform); zero biases.
int cmcg_mlp_init(cmcg_ctx *c, uint64_t seed)
{
    if (!c) return CMCG_ERR_ARG;
    std::vector<float> w(MLP_NPARAM, 0.0f);
    uint64_t z = seed;
    auto next = [&z]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int at, int n, double a) {
        for (int i = 0; i < n; ++i) w[at + i] = (float)((2.0 * next() - 1.0) * a);
    };
    fill(P_W1, MLP_H * MLP_IN, sqrt(6.0 / MLP_IN));
    fill(P_W2, MLP_H * MLP_H, sqrt(6.0 / MLP_H));
    fill(P_W3, MLP_OUT * MLP_H, 0.1 * sqrt(6.0 / MLP_H));
    return cmcg_mlp_set_params(c, w.data());
}

int cmcg_mlp_forward(cmcg_ctx *c, const float *feat, long n, float *z_out, float *prop_out)
{
    if (!c || !feat || n < 1) return CMCG_ERR_ARG;
    MlpSet S;
    void *extra = nullptr;
    const size_t zb = ((size_t)n * MLP_OUT * 4 + 255) & ~(size_t)255;
    RUN(upload_set(c, S, feat, nullptr, nullptr, n, zb + (size_t)n * MLP_BINS * 4, &extra));
    float *dz = (float *)extra, *dp = (float *)((char *)extra + zb);
    const long long ntl = (n + MLP_T - 1) / MLP_T;
    const int grid = (int)std::min<long long>(ntl, 4LL * c->nsm);
    k_mlp_infer<<<grid, MLP_T, MLP_INFER_SMEM, c->stream>>>(c->net, S.feat, n, dp, n, z_out ? dz : nullptr);
    CK(cudaGetLastError());
    RUN(net_status(c));
    if (z_out) CK(cudaMemcpy(z_out, dz, (size_t)n * MLP_OUT * 4, cudaMemcpyDeviceToHost));
    if (prop_out) {
        std::vector<float> h((size_t)n * MLP_BINS);
        CK(cudaMemcpy(h.data(), dp, h.size() * 4, cudaMemcpyDeviceToHost));
        for (long i = 0; i < n; ++i)
            for (int b = 0; b < MLP_BINS; ++b) prop_out[(size_t)i * MLP_BINS + b] = h[(size_t)b * n + i];
    }
    return CMCG_OK;
}

static int train_pass(cmcg_ctx *c, const MlpSet &S, long n, int batch, uint64_t seed, int step, int ordered,
                      int *grid_out)
{
    const int ntl = (batch + MLP_T - 1) / MLP_T;
    const int grid = std::max(1, std::min(ntl, std::min(c->nsm, MLP_TRAIN_GRID_MAX)));
    MlpData d{S.feat, S.bin, S.ntrial, (long long)n, ordered};
    k_mlp_train<<<grid, MLP_T, MLP_TRAIN_SMEM, c->stream>>>(c->net, d, batch, seed, step);
    *grid_out = grid;
    return cudaGetLastError() == cudaSuccess ? CMCG_OK : CMCG_ERR_CUDA;
}

int cmcg_mlp_gradient(cmcg_ctx *c, const float *feat, const int *bin, const int *ntrial, long n, float *grad)
{
    if (!c || !feat || !bin || !ntrial || !grad || n < 1 || n > (1L << 30)) return CMCG_ERR_ARG;
    MlpSet S;
    void *extra = nullptr;
    RUN(upload_set(c, S, feat, bin, ntrial, n, (MLP_NPARAM + 2) * sizeof(float), &extra));
    int grid = 0;
    RUN(train_pass(c, S, n, (int)n, 0, 0, 1, &grid));
    k_mlp_adam<<<1, 1024, 0, c->stream>>>(c->net, grid, 0.0f, 1, 1, (float *)extra);
    CK(cudaGetLastError());
    RUN(net_status(c));
    CK(cudaMemcpy(grad, extra, (MLP_NPARAM + 2) * sizeof(float), cudaMemcpyDeviceToHost));
    return CMCG_OK;
}

int cmcg_mlp_train(cmcg_ctx *c, const float *feat, const int *bin, const int *ntrial, long n, int steps, int batch,
                   double lr, uint64_t seed, float *loss)
{
    if (!c || !feat || !bin || !ntrial || n < 1 || steps < 0 || batch < 1 || !(lr >= 0.0)) return CMCG_ERR_ARG;
    MlpSet S;
    void *extra = nullptr;
    RUN(upload_set(c, S, feat, bin, ntrial, n, (size_t)std::max(steps, 1) * 2 * sizeof(float), &extra));
    float *dl = (float *)extra;
    for (int s = 0; s < steps; ++s) {
        int grid = 0;
        RUN(train_pass(c, S, n, batch, seed, c->adam_t, 0, &grid));
        c->adam_t += 1;
        k_mlp_adam<<<1, 1024, 0, c->stream>>>(c->net, grid, (float)lr, c->adam_t, 0, dl + 2 * s);
        CK(cudaGetLastError());
    }
    RUN(net_status(c));
    if (loss && steps > 0) CK(cudaMemcpy(loss, dl, (size_t)steps * 2 * sizeof(float), cudaMemcpyDeviceToHost));
    return CMCG_OK;
}

long cmcg_learned_samples(cmcg_ctx *c, int k, float *feat, double *X, int *ntrial, long cap)
{
    if (!c || k < 0 || k >= c->ncl || !c->lrn_mem || cap < 0) return CMCG_ERR_ARG;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return CMCG_ERR_CUDA;
    const long long o = c->off[k], n = c->cap[k] + 2;
    std::vector<double> F(n), Xd(n), rn(n);
    std::vector<uint4> fe(n);
    std::vector<int> nt(n);
    if (cudaMemcpy(F.data(), c->lrn.F + o, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(Xd.data(), c->f.X + o, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(rn.data(), c->f.rnew + o, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(fe.data(), c->lrn.feat + o, n * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(nt.data(), c->lrn.ntrial + o, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return CMCG_ERR_CUDA;
    long cnt = 0;
    for (long long j = 1; j < n; ++j) {
        if (!(F[j] > 0.0) || rn[j] == CMCG_SF_INFINITY || nt[j] == 0) continue;
        if (cnt < cap) {
            const uint16_t *h = (const uint16_t *)&fe[j];
            if (feat)
                for (int i = 0; i < MLP_IN; ++i) feat[(size_t)cnt * MLP_IN + i] = bf2f(h[i]);
            if (X) X[cnt] = Xd[j];
            if (ntrial) ntrial[cnt] = nt[j];
        }
        ++cnt;
    }
    return cnt;
}

int cmcg_learned_stats(cmcg_ctx *c, uint64_t *out)
{
    if (!c || !out) return CMCG_ERR_ARG;
    if (!c->lrn_mem) {
        memset(out, 0, LSTAT_N * sizeof(uint64_t));
        return CMCG_OK;
    }
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(out, c->lrn.stats, LSTAT_N * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    return CMCG_OK;
}

// ------------------------------------------------------------ autotuner --
int cmcg_set_variant(cmcg_ctx *c, const char *name, int v)
{
    if (!c || !name) return CMCG_ERR_ARG;
    for (int t = 0; t < V_COUNT; ++t) {
        if (strcmp(name, kTunables[t].name)) continue;
        if (v < 0 || v >= kTunables[t].nvar) return CMCG_ERR_ARG;
        if (c->var[t] != v) drop_graphs(c);  // another launch sequence
        c->var[t] = v;
        return CMCG_OK;
    }
    return CMCG_ERR_ARG;
}

int cmcg_get_variant(cmcg_ctx *c, const char *name)
{
    if (!c || !name) return CMCG_ERR_ARG;
    for (int t = 0; t < V_COUNT; ++t)
        if (!strcmp(name, kTunables[t].name)) return c->var[t];
    return CMCG_ERR_ARG;
}

// Times every variant of the launches the current configuration uses, over
// `steps` whole steps each (after one untimed step), with CUDA events around
// the tuned kernel family, and keeps the fastest.  The steps are real steps
// of the run: the variants give bit-identical results.
int cmcg_autotune(cmcg_ctx *c, int steps, char *report, long report_len)
{
    if (!c || steps < 1) return CMCG_ERR_ARG;
    std::string rep;
    const bool prof0 = c->profile;
    for (int t = 0; t < V_COUNT; ++t) {
        const bool used = (t == V_ORBIT && c->learn_mode == LEARN_OFF) || (t == V_RELAX && !c->relax_fp32 && !c->relax_trig32) ||
                          (t == V_LEARN && c->learn_mode != LEARN_OFF) ||
                          (t == V_MLP_GRID && c->learn_mode == LEARN_ON) || t == V_SORT_TILE ||
                          t == V_GATHER_TILE;
        if (!used) continue;
        const Tunable &T = kTunables[t];
        int best = c->var[t];
        double best_ms = 1e300;
        char buf[160];
        snprintf(buf, sizeof buf, "%s:", T.name);
        rep += buf;
        for (int v = 0; v < T.nvar; ++v) {
            c->var[t] = v;
            c->profile = false;
            RUN(issue_step(c));
            c->profile = true;
            RUN(cmcg_kernel_time(c, "reset", nullptr, nullptr));
            for (int k = 0; k < steps; ++k) RUN(issue_step(c));
            double ms = 0.0;
            long n = 0;
            RUN(cmcg_kernel_time(c, kFamilyNames[T.family], &ms, &n));
            ms /= steps;
            snprintf(buf, sizeof buf, " %s %.4f ms", T.variant[v], ms);
            rep += buf;
            if (ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        c->var[t] = best;
        snprintf(buf, sizeof buf, " -> %s; ", T.variant[best]);
        rep += buf;
    }
    c->profile = prof0;
    drop_graphs(c);
    RUN(cmcg_kernel_time(c, "reset", nullptr, nullptr));
    if (report && report_len > 0) snprintf(report, (size_t)report_len, "%s", rep.c_str());
    return CMCG_OK;
}

// ------------------------------------------------------- host exchange --
// One step on host star arrays: the fields go in, the step runs, the fields
// come back, with copies overlapping kernels where the data allow:
//   r, m, vr, vt go up first; the time step runs while id, E, J follow on the
//   copy stream (relaxation, which writes E and J, waits for them);
//   r, m, id are final after the sort and come back during the potential
//   and energy conservation; vr, vt after energy conservation, during the
//   energies; E, J last.
// Each part is replayed from its own graph when graphs are enabled.

// The device address of a caller's host array when a kernel can reach it
// (pinned or registered host memory, or device or managed memory), else
// nullptr: pageable memory goes by the copy engines.
static const void *device_view(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return a.devicePointer;
    return nullptr;
}

// The step on host arrays that kernels can reach (pinned or registered host
// memory, or device memory).  The uploads of r, m, vr, vt, which precede the
// time step with nothing else to run, go by one k_xfer launch over every
// cluster.  The results that are final only at the step's end are written
// into the caller's arrays by the kernels that compute them: vr, vt and
// J = r vt by energy conservation, E by the energies (part HX_XTAIL), so that
// they cross the host link while those kernels run.  The transfers that
// overlap other kernels stay on the copy engines, one cudaMemcpyAsync per
// array (id up during the time step, E and J staged during the relaxation,
// r, m, id down during the potential): a copy kernel beside a kernel that
// fills the SMs waits for free slots, a copy engine does not.  Sets
// *pageable, and does nothing, when some caller array is not reachable from
// the device: the caller then takes the copy path for every transfer.
static int step_host_batched(cmcg_ctx *c, const cmcg_stars *in, cmcg_stars *out, bool graphs, long l0,
                             bool *pageable)
{
    *pageable = false;
    const int ncl = c->ncl;
    XferSeg *t = c->h_xfer;
    long long nchunk = 0;
    int nseg = 0;
    auto add = [&](void *dst, const void *src, long long n) {
        XferSeg &e = t[nseg++];
        e.dst = (unsigned long long *)dst;
        e.src = (const unsigned long long *)src;
        e.n = n;
        e.c0 = nchunk;
        nchunk += (n + XFER_CHUNK - 1) / XFER_CHUNK;
    };
    for (int k = 0; k < ncl; ++k) {
        const void *src[4] = {in[k].r, in[k].m, in[k].vr, in[k].vt};
        const void *dst[4] = {out[k].vr, out[k].vt, out[k].E, out[k].J};
        const void *ds[4], *dd[4];
        for (int q = 0; q < 4; ++q) {
            ds[q] = device_view(src[q]);
            dd[q] = device_view(dst[q]);
            if (!ds[q] || !dd[q]) {
                *pageable = true;
                return CMCG_OK;
            }
        }
        const long long o = c->off[k] + 1, N = in[k].N;
        double *fields[4] = {c->f.r, c->f.m, c->f.vr, c->f.vt};
        for (int q = 0; q < 4; ++q) add(fields[q] + o, ds[q], N);
        for (int q = 0; q < 4; ++q) c->h_hx[4 * k + q] = (double *)dd[q];
        c->h_xn[k] = N;
    }
    auto part = [&](int p) { return graphs ? run_part_graph(c, p) : issue_part(c, p); };
    // the caller's arrays may be host or device memory here: the copies below
    // take their direction from unified addressing (cudaMemcpyDefault)
    // the table goes up first (one copy); everything after is ordered behind it
    CK(cudaMemcpyAsync(c->d_xfer, c->h_xfer, xfer_table_bytes(ncl), cudaMemcpyHostToDevice, c->stream));
    if (nchunk > 0) {
        const long long grid = std::min<long long>(nchunk, 2LL * c->nsm);  // nothing runs beside it
        k_xfer<<<(unsigned)grid, XFER_THREADS, 0, c->stream>>>(c->d_xfer, nseg, nchunk);
        c->launches += 1;
    }
    k_set_counts<<<(ncl + 127) / 128, 128, 0, c->stream>>>(c->d_cls, c->f, ncl, c->d_xn);
    c->launches += 1;
    CK(cudaEventRecord(c->ev_in, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev_in, 0));  // the copy stream's uploads follow the counts
    for (int k = 0; k < ncl; ++k)
        CK(cudaMemcpyAsync(c->f.id + c->off[k] + 1, in[k].id, (size_t)in[k].N * sizeof(long long),
                           cudaMemcpyDefault, c->copy));
    CK(cudaEventRecord(c->ev_in, c->copy));
    for (int k = 0; k < ncl; ++k) {
        const long long o = c->off[k] + 1;
        const size_t bytes = (size_t)in[k].N * sizeof(double);
        CK(cudaMemcpyAsync(c->f.rnew + o, in[k].E, bytes, cudaMemcpyDefault, c->copy));   // E, staged
        CK(cudaMemcpyAsync(c->f.vrnew + o, in[k].J, bytes, cudaMemcpyDefault, c->copy));  // J, staged
    }
    CK(cudaEventRecord(c->ev_ej, c->copy));
    RUN(part(0));
    CK(cudaStreamWaitEvent(c->stream, c->ev_in, 0));
    RUN(part(HX_XRELAX));
    CK(cudaStreamWaitEvent(c->stream, c->ev_ej, 0));
    RUN(part(HX_XSORT));
    CK(cudaEventRecord(c->ev_sorted, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev_sorted, 0));
    // a cluster never grows in a step: N given in bounds the stars after it
    for (int k = 0; k < ncl; ++k) {
        const long long o = c->off[k] + 1;
        const size_t bytes = (size_t)in[k].N * sizeof(double);
        CK(cudaMemcpyAsync(out[k].r, c->f.r + o, bytes, cudaMemcpyDefault, c->copy));
        CK(cudaMemcpyAsync(out[k].m, c->f.m + o, bytes, cudaMemcpyDefault, c->copy));
        CK(cudaMemcpyAsync(out[k].id, c->f.id + o, (size_t)in[k].N * sizeof(long long), cudaMemcpyDefault,
                           c->copy));
    }
    CK(cudaEventRecord(c->ev_copied, c->copy));
    RUN(part(HX_XTAIL));
    k_gather_counts<<<(ncl + 127) / 128, 128, 0, c->stream>>>(c->d_cls, ncl, c->d_nout);
    c->launches += 1;
    CK(cudaGetLastError());
    std::vector<long long> n(ncl);
    CK(cudaMemcpyAsync(n.data(), c->d_nout, (size_t)ncl * sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamWaitEvent(c->stream, c->ev_copied, 0));  // the next call's uploads follow the read-back
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < ncl; ++k) out[k].N = (long)n[k];
    c->launches_last = c->launches - l0;
    return CMCG_OK;
}

static int step_host_run(cmcg_ctx *c, const cmcg_stars *in, cmcg_stars *out)
{
    const bool graphs = c->use_graph && !c->profile;
    const long l0 = c->launches;
    {
        bool pageable = false;
        const int rc = step_host_batched(c, in, out, graphs, l0, &pageable);
        if (rc || !pageable) return rc;
    }
    auto part = [&](int p) { return graphs ? run_part_graph(c, p) : issue_part(c, p); };
    auto up = [&](double *dst, const double *src, long n, cudaStream_t s) {
        return cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    };
    auto down = [&](double *dst, const double *src, long n, cudaStream_t s) {
        return cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s);
    };
    static const double sentinel = CMCG_SF_INFINITY;
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        const long N = in[k].N;
        CK(up(c->f.r + o, in[k].r, N, c->stream));
        CK(up(c->f.m + o, in[k].m, N, c->stream));
        CK(up(c->f.vr + o, in[k].vr, N, c->stream));
        CK(up(c->f.vt + o, in[k].vt, N, c->stream));
        CK(cudaMemcpyAsync(c->f.r + o + N, &sentinel, sizeof(double), cudaMemcpyHostToDevice, c->stream));
        k_set_count<<<1, 1, 0, c->stream>>>(c->d_cls, k, (long long)N);
        c->launches += 1;
    }
    CK(cudaEventRecord(c->ev_in, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev_in, 0));  // the copy stream's uploads follow the counts
    // id (the relaxation's draws) during the time step; E and J, staged,
    // during the relaxation
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        CK(cudaMemcpyAsync(c->f.id + o, in[k].id, (size_t)in[k].N * sizeof(long long), cudaMemcpyHostToDevice,
                           c->copy));
    }
    CK(cudaEventRecord(c->ev_in, c->copy));
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        CK(up(c->f.rnew + o, in[k].E, in[k].N, c->copy));
        CK(up(c->f.vrnew + o, in[k].J, in[k].N, c->copy));
    }
    CK(cudaEventRecord(c->ev_ej, c->copy));
    RUN(part(0));
    CK(cudaStreamWaitEvent(c->stream, c->ev_in, 0));
    RUN(part(HX_XRELAX));
    CK(cudaStreamWaitEvent(c->stream, c->ev_ej, 0));
    RUN(part(HX_XSORT));
    CK(cudaEventRecord(c->ev_sorted, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev_sorted, 0));
    // a cluster never grows in a step: N given in bounds the stars after it
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        const long N = in[k].N;
        CK(down(out[k].r, c->f.r + o, N, c->copy));
        CK(down(out[k].m, c->f.m + o, N, c->copy));
        CK(cudaMemcpyAsync(out[k].id, c->f.id + o, (size_t)N * sizeof(long long), cudaMemcpyDeviceToHost,
                           c->copy));
    }
    RUN(part(2));
    CK(cudaEventRecord(c->ev_ec3, c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev_ec3, 0));
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        CK(down(out[k].vr, c->f.vr + o, in[k].N, c->copy));
        CK(down(out[k].vt, c->f.vt + o, in[k].N, c->copy));
    }
    CK(cudaEventRecord(c->ev_copied, c->copy));
    RUN(part(3));
    k_gather_counts<<<(c->ncl + 127) / 128, 128, 0, c->stream>>>(c->d_cls, c->ncl, c->d_nout);
    c->launches += 1;
    CK(cudaGetLastError());
    for (int k = 0; k < c->ncl; ++k) {
        const long long o = c->off[k] + 1;
        CK(down(out[k].E, c->f.E + o, in[k].N, c->stream));
        CK(down(out[k].J, c->f.J + o, in[k].N, c->stream));
    }
    std::vector<long long> n(c->ncl);
    CK(cudaMemcpyAsync(n.data(), c->d_nout, (size_t)c->ncl * sizeof(long long), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamWaitEvent(c->stream, c->ev_copied, 0));  // the next call's uploads follow the read-back
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < c->ncl; ++k) out[k].N = (long)n[k];
    c->launches_last = c->launches - l0;
    return CMCG_OK;
}

int cmcg_step_host(cmcg_ctx *c, const cmcg_stars *in, cmcg_stars *out)
{
    if (!c || !in || !out) return CMCG_ERR_ARG;
    for (int k = 0; k < c->ncl; ++k) {
        const cmcg_stars &a = in[k], &b = out[k];
        if (!a.r || !a.m || !a.vr || !a.vt || !a.E || !a.J || !a.id) return CMCG_ERR_ARG;
        if (!b.r || !b.m || !b.vr || !b.vt || !b.E || !b.J || !b.id || b.cap < a.N) return CMCG_ERR_ARG;
        if (a.N > c->cap[k]) return CMCG_ERR_CAPACITY;
        if (a.N < 2 * c->params[k].AVEKERNEL + 2) return CMCG_ERR_ARG;
    }
    const int rc = step_host_run(c, in, out);
    if (rc) {  // copies from or to the caller's arrays may still be in flight: they end before the return
        cudaStreamSynchronize(c->copy);
        cudaStreamSynchronize(c->stream);
    }
    return rc;
}

}  // extern "C"
