// cmcg_common.cuh -- launch geometry and deterministic block reductions.
#pragma once
#include "cmcg_internal.cuh"

namespace cmcg {

// Table of tiles for one tile size: tiles[b] = (cluster, tile-in-cluster);
// first[c], count[c] give cluster c's contiguous range of table entries.
struct Tiles {
    const int2 *tiles;
    const int *first;
    const int *count;
    int ntiles;
};

template <int NT>
__device__ __forceinline__ double block_sum(double v, double *smem /* >= NT/32 */)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) smem[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NT / 32; ++i) s = __dadd_rn(s, smem[i]);
    }
    return s;  // valid in thread 0
}

template <int NT>
__device__ __forceinline__ double block_max(double v, double *smem)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) smem[w] = v;
    __syncthreads();
    double s = -INFINITY;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NT / 32; ++i) s = fmax(s, smem[i]);
    }
    return s;
}

// K sums over the block in one pass, valid in thread 0's v[].  Each warp
// reduces a column by shuffles only when one of its lanes holds a nonzero
// value (a column that is zero over the warp contributes exactly 0), then
// thread 0 adds the warps in a fixed order: the same tree as block_sum, with
// two barriers for all K columns instead of two per column.
template <int NT, int K>
__device__ __forceinline__ void block_sums(double (&v)[K], double (*smem)[K] /* [NT/32][K], not shared with others */)
{
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        double x = v[i];
        // x != 0.0 (NaN included), decided on the bits: an FP64 comparison
        // would take the FP64 pipe once per column and thread
        if (__any_sync(0xffffffffu, ((unsigned long long)__double_as_longlong(x) << 1) != 0ull)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = __dadd_rn(x, __shfl_down_sync(0xffffffffu, x, o));
        }
        if (l == 0) smem[w][i] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < K; ++i) {
            double s = 0.0;
            for (int q = 0; q < NT / 32; ++q) s = __dadd_rn(s, smem[q][i]);
            v[i] = s;
        }
    }
}

// Maximum of non-negative doubles (valid in thread 0), compared as their bit
// patterns, which order like the values: integer instructions only.
template <int NT>
__device__ __forceinline__ double block_max_nonneg(double v, long long *smem /* >= NT/32, not shared */)
{
    long long b = __double_as_longlong(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_down_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = 1; i < NT / 32; ++i) b = max(b, smem[i]);
    return __longlong_as_double(b);
}

template <int NT>
__device__ __forceinline__ long long block_sum_ll(long long v, long long *smem)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) smem[w] = v;
    __syncthreads();
    long long s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NT / 32; ++i) s += smem[i];
    }
    return s;
}

// Last-block-done protocol.  Thread 0 of every block calls this after writing
// its partials; it returns true in exactly one block per cluster (the last to
// arrive), which may then read all of that cluster's partials.
__device__ __forceinline__ bool arrive_last(unsigned int *ticket, int count)
{
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    if (t == (unsigned int)(count - 1)) {
        __threadfence();
        *ticket = 0u;  // reset for the next launch
        return true;
    }
    return false;
}

// Whole-block form: every thread calls it after thread 0 has written the
// block's partials; returns the same answer in all threads of the block.
__device__ __forceinline__ bool block_arrive_last(unsigned int *ticket, int count, int *s_flag)
{
    __threadfence();  // every thread's writes before the ticket, not only thread 0's
    __syncthreads();
    if (threadIdx.x == 0) *s_flag = arrive_last(ticket, count) ? 1 : 0;
    __syncthreads();
    return *s_flag != 0;
}

// In the last block: sum of column `col` of a cluster's [count][width]
// partials, all threads striding over tiles in a fixed order, then a fixed
// tree (deterministic).  Loads bypass L1: the partials come from other SMs.
template <int NT>
__device__ __forceinline__ double reduce_partials_sum(const double *partials, int b0, int count, int width, int col,
                                                      double *red)
{
    double v = 0.0;
    for (int b = threadIdx.x; b < count; b += NT) v += __ldcg(partials + (size_t)(b0 + b) * width + col);
    return block_sum<NT>(v, red);
}

template <int NT>
__device__ __forceinline__ double reduce_partials_max(const double *partials, int b0, int count, int width, int col,
                                                      double *red)
{
    double v = -INFINITY;
    for (int b = threadIdx.x; b < count; b += NT) v = fmax(v, __ldcg(partials + (size_t)(b0 + b) * width + col));
    return block_max<NT>(v, red);
}

}  // namespace cmcg
