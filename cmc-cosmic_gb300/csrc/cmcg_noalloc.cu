// cmcg_noalloc.cu -- radius sort that allocates nothing.
//
// Some callers cannot allocate device memory once they are running: a host
// code that embeds this library in a process whose GPU memory is owned by
// another runtime (a framework allocator that reserved the device up front),
// or a long run on a shared GPU that must not risk a failed allocation in the
// middle of a simulation.  cmcg_sort_radii_noalloc gives them the stable
// radius sort of qsorts_new without any allocation: its working memory is a
// file-scope __device__ array of fixed size, so the caller passes only the
// input radii and the output permutation.
//
// The array is held by every GPU that loads the library until the process
// exits (about 34 MB for the 2^20-star maximum).  Its device address is looked
// up on every call, with the caller's device current; the first call on a
// device also loads the module there, so make that first call before any
// stream capture.  All calls share the one array and it keeps the previous
// call's contents: the parts that must start from zero are cleared on every
// call, and calls that overlap on the GPU (on different streams, or from
// different host threads) race on it.
//
// Errors the sort kernels record on the device (a bounded wait that gave up,
// inconsistent counts) are read back only by the synchronizing form of the
// call (n_bound given); the asynchronous form returns after queueing its work
// and reports only what the host can see.
#include <cstdio>

#include "cmcg_kernels.cuh"
#include "cmcgpu.h"

namespace cmcg {

constexpr long long NA_MAX = CMCG_NOALLOC_MAX_STARS;
constexpr long long NA_TILES = (NA_MAX + SORT_T - 1) / SORT_T;

// byte layout of the scratch array (every part 256-byte aligned)
constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t NA_R = 0;                                                          // radii, 1-based
constexpr size_t NA_K0 = na_align(NA_R + sizeof(double) * (NA_MAX + 2));
constexpr size_t NA_K1 = na_align(NA_K0 + sizeof(unsigned long long) * NA_MAX);
constexpr size_t NA_V0 = na_align(NA_K1 + sizeof(unsigned long long) * NA_MAX);
constexpr size_t NA_V1 = na_align(NA_V0 + sizeof(unsigned int) * NA_MAX);
constexpr size_t NA_STATUS = na_align(NA_V1 + sizeof(unsigned int) * NA_MAX);      // look-back words
constexpr size_t NA_GHIST = na_align(NA_STATUS + sizeof(unsigned long long) * RADIX * NA_TILES);
constexpr size_t NA_MISC = na_align(NA_GHIST + sizeof(unsigned long long) * SORT_MAX_PASSES * RADIX);
// NA_MISC: epoch (+0), npass (+8), kmin (+16), kmax (+24), shift (+32), long-run count (+40),
// tile counters (+48)
constexpr size_t NA_LRUN = na_align(NA_MISC + 48 + sizeof(unsigned int) * SORT_MAX_PASSES);  // long-run starts
constexpr size_t NA_PART = na_align(NA_LRUN + sizeof(long long) * (NA_MAX / 32 + 64));
constexpr size_t NA_TICK = na_align(NA_PART + sizeof(double) * 3 * NA_TILES);
constexpr size_t NA_SC = na_align(NA_TICK + sizeof(unsigned int));
constexpr size_t NA_CL = na_align(NA_SC + sizeof(Scalars));
constexpr size_t NA_TILE = na_align(NA_CL + sizeof(Cluster));
constexpr size_t NA_FC = na_align(NA_TILE + sizeof(int2) * NA_TILES);             // first, count
constexpr size_t NA_BYTES = na_align(NA_FC + 2 * sizeof(int));

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Describe one cluster of n keys to the shared sort kernels.
__global__ void k_na_setup(unsigned char *base, long long n, int ntiles)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int2 *tiles = (int2 *)(base + NA_TILE);
    if (i < ntiles) tiles[i] = make_int2(0, i);
    if (i == 0) {
        Scalars *sc = (Scalars *)(base + NA_SC);
        Cluster *cl = (Cluster *)(base + NA_CL);
        int *fc = (int *)(base + NA_FC);
        sc->N_MAX = n;
        sc->N_MAX_NEW = n;
        sc->err = 0;
        sc->err_index = 0;
        cl->off = 0;
        cl->cap = NA_MAX;
        cl->sc = sc;
        fc[0] = 0;
        fc[1] = ntiles;
        *(unsigned int *)(base + NA_TICK) = 0u;
    }
}

// Output: perm[i] = 0-based input position of the i-th smallest radius.
__global__ void k_na_perm(unsigned char *base, long long n, unsigned int *perm)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int np = *(const int *)(base + NA_MISC + 8);
    const unsigned int *v = (np & 1) ? (const unsigned int *)(base + NA_V1) : (const unsigned int *)(base + NA_V0);
    perm[i] = (np == 0) ? (unsigned int)i : v[i];
}

}  // namespace cmcg

using namespace cmcg;

extern "C" int cmcg_sort_radii_noalloc(const double *d_r, long n, uint32_t *d_perm, long *n_bound, void *stream)
{
    if (!d_r || !d_perm || n < 1) return CMCG_ERR_ARG;
    if (n > NA_MAX) {
        fprintf(stderr, "cmcg_sort_radii_noalloc: %ld stars exceed the fixed maximum of %lld\n", n, NA_MAX);
        return CMCG_ERR_CAPACITY;
    }
    // the array's address on the current device, looked up on every call: a
    // cached address would go stale if the device's context were reset
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess || !addr) {
        fprintf(stderr, "cmcg_sort_radii_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
        return CMCG_ERR_CUDA;
    }
    unsigned char *base = (unsigned char *)addr;
    cudaStream_t s = (cudaStream_t)stream;
    const int ntiles = (int)((n + SORT_T - 1) / SORT_T);
    // radii into slots 1..n (the sort kernels read the reference's 1-based layout)
    if (cudaMemcpyAsync(base + NA_R + sizeof(double), d_r, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice,
                        s) != cudaSuccess)
        return CMCG_ERR_CUDA;
    k_na_setup<<<(ntiles + 255) / 256, 256, 0, s>>>(base, n, ntiles);
    Fields f{};
    f.rnew = (double *)(base + NA_R);
    SortBufs sb{};
    sb.keys[0] = (unsigned long long *)(base + NA_K0);
    sb.keys[1] = (unsigned long long *)(base + NA_K1);
    sb.vals[0] = (unsigned int *)(base + NA_V0);
    sb.vals[1] = (unsigned int *)(base + NA_V1);
    sb.status = (unsigned long long *)(base + NA_STATUS);
    sb.ghist = (unsigned long long *)(base + NA_GHIST);
    sb.epoch = (unsigned int *)(base + NA_MISC);
    sb.npass = (int *)(base + NA_MISC + 8);
    sb.shift = (int *)(base + NA_MISC + 32);
    sb.nlong = (unsigned int *)(base + NA_MISC + 40);
    sb.lstart = (long long *)(base + NA_LRUN);
    sb.tile_next = (unsigned int *)(base + NA_MISC + 48);
    sb.kmin = (unsigned long long *)(base + NA_MISC + 16);
    sb.kmax = (unsigned long long *)(base + NA_MISC + 24);
    const Cluster *cls = (const Cluster *)(base + NA_CL);
    Tiles tm{(const int2 *)(base + NA_TILE), (const int *)(base + NA_FC), (const int *)(base + NA_FC) + 1, ntiles};
    double *partials = (double *)(base + NA_PART);
    unsigned int *tickets = (unsigned int *)(base + NA_TICK);
    // k_sort_prep zeroes the digit totals, tile counters and long-run count
    k_sort_prep<<<ntiles, SORT_THREADS, 0, s>>>(cls, tm, f, sb, partials, tickets);
    k_sort_ghist<<<ntiles, SORT_THREADS, 0, s>>>(cls, tm, f, sb);
    for (int p = 0; p < SORT_MAX_PASSES; ++p) launch_sort_onesweep(SORT_T, ntiles, s, cls, tm, f, sb, p);
    k_sort_fix<<<ntiles, SORT_THREADS, 0, s>>>(cls, tm, sb);
    k_sort_fix_long<<<ntiles, SORT_THREADS, 0, s>>>(cls, tm, sb, f, nullptr);
    k_na_perm<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(base, n, d_perm);
    if (cudaGetLastError() != cudaSuccess) return CMCG_ERR_CUDA;
    if (n_bound) {
        // the synchronizing form: the kept count and the kernels' status word
        Scalars sc;
        if (cudaMemcpyAsync(&sc, base + NA_SC, sizeof(sc), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return CMCG_ERR_CUDA;
        if (sc.err) {
            fprintf(stderr, "cmcg_sort_radii_noalloc: device error %d at %lld\n", sc.err, sc.err_index);
            return sc.err;
        }
        *n_bound = (long)sc.n_bound;
    }
    return CMCG_OK;
}
