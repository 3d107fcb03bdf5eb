// cmcg_mlp.cu -- the learned proposal's network on the fifth-generation tensor
// cores: inference for every star of a step, and the training step (forward,
// loss, backward and weight gradients) with an Adam update.
//
// Every matrix product is a tcgen05.mma of kind::f16 (BF16 operands in shared
// memory, FP32 accumulator in TMEM) issued by one thread of the CTA; the
// other threads stage operands and run the epilogues, each owning one row
// (star or sample) of the 128-row tile, which is also the TMEM lane the
// accumulator row lives in.  The packed weight image reaches shared memory
// in one bulk (TMA) copy.
//
// Forward:  h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), z = W3 h2 + b3.
// Outputs:  q_b = (1 - f) softmax(z_0..31)_b + f / 32 (f = MLP_FLOOR), stored
//           as the CDF C_1..C_31; P = sigmoid(z_32).
// Loss per sample with accepted bin b and plain trial count k:
//           -log softmax(z)_b - (k - 1) log(1 - P) - log P
// (the bins' negative log-likelihood, and the geometric likelihood of k
// trials at acceptance probability P), averaged over the batch.
// Weight gradients are products over the batch (K = samples): dW = dH^T X,
// with a column of ones appended to X giving the bias gradient in the same
// product.
#include <cuda_bf16.h>
#include "cmcg_kernels.cuh"
#include "cmcg_tc.cuh"
#include "cmcgpu.h"

namespace cmcg {
using namespace tc;

static __device__ __forceinline__ uint32_t bf2(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}
static __device__ __forceinline__ uint4 pack8(const float *v)
{
    return make_uint4(bf2(v[0], v[1]), bf2(v[2], v[3]), bf2(v[4], v[5]), bf2(v[6], v[7]));
}
static __device__ __forceinline__ void st_bf16(unsigned char *base, uint32_t off, float v)
{
    *reinterpret_cast<__nv_bfloat16 *>(base + off) = __float2bfloat16_rn(v);
}
static __device__ __forceinline__ void unpack8(uint4 u, float *v)
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = __uint_as_float(w[i] << 16);
        v[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

// The packed image from the master parameters (every thread of the launch takes a share).
static __device__ void pack_image(const float *__restrict__ w, unsigned char *__restrict__ img, int t, int nt)
{
    for (int e = t; e < MLP_H * MLP_K1; e += nt) {
        const int n = e / MLP_K1, k = e % MLP_K1;
        st_bf16(img + IMG_W1, kmaj(n, k, MLP_K1), k < MLP_IN ? w[P_W1 + n * MLP_IN + k] : 0.0f);
    }
    for (int e = t; e < MLP_H * MLP_H; e += nt) {
        const int n = e / MLP_H, k = e % MLP_H;
        st_bf16(img + IMG_W2, kmaj(n, k, MLP_H), w[P_W2 + n * MLP_H + k]);
        // W2^T: row = layer-1 unit, K = layer-2 unit
        st_bf16(img + IMG_W2T, kmaj(n, k, MLP_H), w[P_W2 + k * MLP_H + n]);
    }
    for (int e = t; e < MLP_N3 * MLP_H; e += nt) {
        const int n = e / MLP_H, k = e % MLP_H;
        st_bf16(img + IMG_W3, kmaj(n, k, MLP_H), n < MLP_OUT ? w[P_W3 + n * MLP_H + k] : 0.0f);
    }
    for (int e = t; e < MLP_H * MLP_N3; e += nt) {
        const int n = e / MLP_N3, k = e % MLP_N3;  // W3^T: row = layer-2 unit, K = output
        st_bf16(img + IMG_W3T, kmaj(n, k, MLP_N3), k < MLP_OUT ? w[P_W3 + k * MLP_H + n] : 0.0f);
    }
    float *bias = reinterpret_cast<float *>(img + IMG_BIAS);
    for (int e = t; e < MLP_H; e += nt) {
        bias[e] = w[P_B1 + e];
        bias[MLP_H + e] = w[P_B2 + e];
    }
    for (int e = t; e < MLP_N3; e += nt) bias[2 * MLP_H + e] = e < MLP_OUT ? w[P_B3 + e] : 0.0f;
}

__global__ void k_mlp_pack(MlpNet net)
{
    pack_image(net.w, net.img, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// relu(accumulator + bias) of this thread's row, 64 columns, as BF16 into the
// K-major A operand `dst` (row `row`, K = 64); bit i of mask[i / 32] tells
// whether unit i was active.  Optionally also into column `row` of the
// transposed operand `dstT` (rows = units, K = 128 samples).
static __device__ __forceinline__ void hidden_epilogue(uint32_t tl, const float *b, unsigned char *dst, int row,
                                                       unsigned char *dstT, uint32_t (&mask)[2])
{
    mask[0] = mask[1] = 0u;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float v[16];
        tmem_ld16(tl + 16 * c, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float x = v[i] + b[16 * c + i];
            if (x > 0.0f) mask[c >> 1] |= 1u << ((16 * c + i) & 31);
            v[i] = fmaxf(x, 0.0f);
        }
        *reinterpret_cast<uint4 *>(dst + kmaj(row, 16 * c, MLP_H)) = pack8(v);
        *reinterpret_cast<uint4 *>(dst + kmaj(row, 16 * c + 8, MLP_H)) = pack8(v + 8);
        if (dstT) {
#pragma unroll
            for (int i = 0; i < 16; ++i) st_bf16(dstT, kmaj(16 * c + i, row, MLP_T), v[i]);
        }
    }
}

// z (33 logits) -> the 31 CDF knots C_1..C_31 and P
static __device__ __forceinline__ void proposal(const float *z, float *out)
{
    float mx = z[0];
#pragma unroll
    for (int i = 1; i < MLP_BINS; ++i) mx = fmaxf(mx, z[i]);
    float e[MLP_BINS], S = 0.0f;
#pragma unroll
    for (int i = 0; i < MLP_BINS; ++i) {
        e[i] = expf(z[i] - mx);
        S += e[i];
    }
    const float a = (1.0f - MLP_FLOOR) / S, u = MLP_FLOOR / MLP_BINS;
    float c = 0.0f;
#pragma unroll
    for (int i = 0; i < MLP_BINS - 1; ++i) {
        c += e[i] * a + u;
        out[i] = c;
    }
    out[MLP_BINS - 1] = 1.0f / (1.0f + expf(-z[MLP_BINS]));
}

// ------------------------------------------------------------ inference --
// Persistent: each CTA loads the image once and walks 128-row tiles.  Row r
// takes features feat[r] and writes prop[b * stride + r] (b = 0..31), and its
// 33 logits to z_out[33 r ..] when z_out is given.
constexpr int INF_A0 = IMG_INFER, INF_H = INF_A0 + MLP_T * MLP_K1 * 2, INF_BAR = INF_H + MLP_T * MLP_H * 2;
static_assert(INF_BAR + 64 == MLP_INFER_SMEM, "inference shared-memory layout");

__global__ void __launch_bounds__(MLP_T) k_mlp_infer(MlpNet net, const uint4 *__restrict__ feat, long long nrows,
                                                     float *__restrict__ prop, long long stride,
                                                     float *__restrict__ z_out)
{
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *img = smem, *A0 = smem + INF_A0, *H = smem + INF_H;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + INF_BAR);  // [0] image copy, [1] MMAs
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(smem + INF_BAR + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long ntiles = (nrows + MLP_T - 1) / MLP_T;
    if ((long long)blockIdx.x >= ntiles) return;  // whole block, before any allocation
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        fence_async_smem();
    }
    if (warp == 0) {
        tmem_alloc(s_tmem, 64);
        tmem_relinquish();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *s_tmem;
    if (tid == 0) {
        mbar_arrive_expect_tx(&bar[0], IMG_INFER);
        bulk_g2s(img, net.img, IMG_INFER, &bar[0]);
    }
    int ok = __syncthreads_and(mbar_wait(&bar[0], 0, WAIT_LIMIT));
    const float *b1 = reinterpret_cast<const float *>(img + IMG_BIAS), *b2 = b1 + MLP_H, *b3 = b1 + 2 * MLP_H;
    const uint32_t aA0 = smem_addr(A0), aH = smem_addr(H);
    const uint32_t aW1 = smem_addr(img + IMG_W1), aW2 = smem_addr(img + IMG_W2), aW3 = smem_addr(img + IMG_W3);
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's TMEM lanes
    uint32_t phase = 0, mask[2];
    for (long long tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        const long long row = tile * MLP_T + tid;
        const uint4 x = row < nrows ? feat[row] : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4 *>(A0 + kmaj(tid, 0, MLP_K1)) = x;
        *reinterpret_cast<uint4 *>(A0 + kmaj(tid, 8, MLP_K1)) = make_uint4(0u, 0u, 0u, 0u);
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            mma_bf16(tmem, kmaj_desc(aA0, MLP_K1, 0), kmaj_desc(aW1, MLP_K1, 0), idesc_bf16(128, MLP_H), 0u);
            mma_commit(&bar[1]);
        }
        ok = __syncthreads_and(mbar_wait(&bar[1], phase, WAIT_LIMIT));
        phase ^= 1u;
        if (!ok) break;
        fence_after();
        hidden_epilogue(tl, b1, H, tid, nullptr, mask);
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int k = 0; k < MLP_H / 16; ++k)
                mma_bf16(tmem, kmaj_desc(aH, MLP_H, k), kmaj_desc(aW2, MLP_H, k), idesc_bf16(128, MLP_H), k > 0);
            mma_commit(&bar[1]);
        }
        ok = __syncthreads_and(mbar_wait(&bar[1], phase, WAIT_LIMIT));
        phase ^= 1u;
        if (!ok) break;
        fence_after();
        hidden_epilogue(tl, b2, H, tid, nullptr, mask);
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int k = 0; k < MLP_H / 16; ++k)
                mma_bf16(tmem, kmaj_desc(aH, MLP_H, k), kmaj_desc(aW3, MLP_H, k), idesc_bf16(128, MLP_N3), k > 0);
            mma_commit(&bar[1]);
        }
        ok = __syncthreads_and(mbar_wait(&bar[1], phase, WAIT_LIMIT));
        phase ^= 1u;
        if (!ok) break;
        fence_after();
        float z[MLP_N3];
        tmem_ld16(tl, *reinterpret_cast<float(*)[16]>(z));
        tmem_ld16(tl + 16, *reinterpret_cast<float(*)[16]>(z + 16));
        tmem_ld16(tl + 32, *reinterpret_cast<float(*)[16]>(z + 32));
#pragma unroll
        for (int i = 0; i < MLP_OUT; ++i) z[i] += b3[i];
        if (row < nrows) {
            if (z_out)
                for (int i = 0; i < MLP_OUT; ++i) z_out[row * MLP_OUT + i] = z[i];
            float out[MLP_BINS];
            proposal(z, out);
#pragma unroll
            for (int b = 0; b < MLP_BINS; ++b) prop[b * stride + row] = out[b];
        }
        fence_before();  // the TMEM reads above precede the next tile's MMA
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, 64);
    if (!ok && tid == 0) atomicExch(net.status, CMCG_ERR_SPIN);
}

// ------------------------------------------------------------- training --
constexpr int TR_A0 = IMG_TOTAL, TR_XT = TR_A0 + MLP_T * MLP_K1 * 2, TR_R1 = TR_XT + MLP_NG1 * MLP_T * 2,
              TR_R2 = TR_R1 + MLP_T * MLP_H * 2, TR_H1T = TR_R2 + MLP_T * MLP_H * 2,
              TR_H2T = TR_H1T + MLP_NG * MLP_T * 2, TR_T1 = TR_H2T + MLP_NG * MLP_T * 2,
              TR_T2 = TR_T1 + MLP_T * MLP_T * 2, TR_BAR = TR_T2 + MLP_T * MLP_T * 2;
static_assert(TR_BAR + 192 == MLP_TRAIN_SMEM, "training shared-memory layout");
// TMEM columns: the layer accumulator, then the three weight-gradient
// accumulators, each on a 128-column boundary (one CTA per SM: its shared
// memory allows no second, so all 512 columns are free)
constexpr uint32_t TM_ACT = 0, TM_G3 = 128, TM_G2 = 256, TM_G1 = 384, TM_COLS = 512;
static_assert(TM_G3 >= MLP_H && TM_G2 >= TM_G3 + MLP_NG && TM_G1 >= TM_G2 + MLP_NG && TM_G1 + MLP_NG1 <= TM_COLS,
              "TMEM columns");

static __device__ __forceinline__ long long sample_index(unsigned long long seed, int step, int pos, long long n)
{
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (((unsigned long long)(unsigned)step << 32) + pos + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (long long)(z % (unsigned long long)n);
}

// softplus(x) = log(1 + e^x), without overflow
static __device__ __forceinline__ float softplus(float x) { return fmaxf(x, 0.0f) + log1pf(expf(-fabsf(x))); }

// One training pass over `batch` samples (drawn by sample_index, or in order):
// each CTA walks 128-sample tiles, keeps its weight gradients in TMEM, and
// writes them with its loss sums to its partial slot.  Shared memory holds
// the image, the tile's operands in both orientations, and the transposed
// gradients (rows beyond the real units stay zero).
__global__ void __launch_bounds__(MLP_T, 1) k_mlp_train(MlpNet net, MlpData data, int batch,
                                                         unsigned long long seed, int step)
{
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *img = smem, *A0 = smem + TR_A0, *XT = smem + TR_XT, *R1 = smem + TR_R1, *R2 = smem + TR_R2;
    unsigned char *H1T = smem + TR_H1T, *H2T = smem + TR_H2T, *T1 = smem + TR_T1, *T2 = smem + TR_T2;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + TR_BAR);
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(smem + TR_BAR + 16);
    float *s_red = reinterpret_cast<float *>(smem + TR_BAR + 64);  // [4 warps][2]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntiles = (batch + MLP_T - 1) / MLP_T;
    // rows 64..127 of the transposed gradients stay zero (M = 128, 64 real rows)
    for (int i = tid; i < MLP_T * MLP_T * 2 / 2 / 16; i += MLP_T) {
        reinterpret_cast<uint4 *>(T1 + MLP_T * MLP_T)[i] = make_uint4(0u, 0u, 0u, 0u);
        reinterpret_cast<uint4 *>(T2 + MLP_T * MLP_T)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        fence_async_smem();
    }
    if (warp == 0) {
        tmem_alloc(s_tmem, TM_COLS);
        tmem_relinquish();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *s_tmem;
    if (tid == 0) {
        mbar_arrive_expect_tx(&bar[0], IMG_TOTAL);
        bulk_g2s(img, net.img, IMG_TOTAL, &bar[0]);
    }
    int ok = __syncthreads_and(mbar_wait(&bar[0], 0, WAIT_LIMIT));
    const float *b1 = reinterpret_cast<const float *>(img + IMG_BIAS), *b2 = b1 + MLP_H, *b3 = b1 + 2 * MLP_H;
    const uint32_t aA0 = smem_addr(A0), aXT = smem_addr(XT), aR1 = smem_addr(R1), aR2 = smem_addr(R2);
    const uint32_t aH1T = smem_addr(H1T), aH2T = smem_addr(H2T), aT1 = smem_addr(T1), aT2 = smem_addr(T2);
    const uint32_t aW1 = smem_addr(img + IMG_W1), aW2 = smem_addr(img + IMG_W2), aW3 = smem_addr(img + IMG_W3);
    const uint32_t aW3T = smem_addr(img + IMG_W3T), aW2T = smem_addr(img + IMG_W2T);
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0, m1[2], m2[2];
    float nll_sum = 0.0f, geo_sum = 0.0f;
    int ntl = 0;
#define MLP_WAIT()                                                        \
    ok = __syncthreads_and(mbar_wait(&bar[1], phase, WAIT_LIMIT));        \
    phase ^= 1u;                                                          \
    if (!ok) break;                                                       \
    fence_after()
#define MLP_ISSUE_BEGIN() \
    fence_async_smem();   \
    fence_before();       \
    __syncthreads();      \
    if (tid == 0) {       \
        fence_after();
#define MLP_ISSUE_END()       \
    mma_commit(&bar[1]);      \
    }
    for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++ntl) {
        const int pos = tile * MLP_T + tid;
        const bool valid = pos < batch;
        uint4 x = make_uint4(0u, 0u, 0u, 0u);
        int bin = 0, kt = 1;
        if (valid) {
            const long long s = data.ordered ? (long long)pos : sample_index(seed, step, pos, data.n);
            x = data.feat[s];
            bin = min(max(data.bin[s], 0), MLP_BINS - 1);
            kt = max(data.ntrial[s], 1);
        }
        const float w = valid ? 1.0f / (float)batch : 0.0f;
        *reinterpret_cast<uint4 *>(A0 + kmaj(tid, 0, MLP_K1)) = x;
        *reinterpret_cast<uint4 *>(A0 + kmaj(tid, 8, MLP_K1)) = make_uint4(0u, 0u, 0u, 0u);
        {
            float xf[8];
            unpack8(x, xf);
#pragma unroll
            for (int i = 0; i < MLP_NG1; ++i)
                st_bf16(XT, kmaj(i, tid, MLP_T), i < MLP_IN ? xf[i] : (i == MLP_IN ? 1.0f : 0.0f));
        }
        // layer 1
        MLP_ISSUE_BEGIN();
        mma_bf16(tmem + TM_ACT, kmaj_desc(aA0, MLP_K1, 0), kmaj_desc(aW1, MLP_K1, 0), idesc_bf16(128, MLP_H), 0u);
        MLP_ISSUE_END();
        MLP_WAIT();
        hidden_epilogue(tl + TM_ACT, b1, R1, tid, H1T, m1);
#pragma unroll
        for (int i = MLP_H; i < MLP_NG; ++i) st_bf16(H1T, kmaj(i, tid, MLP_T), i == MLP_H ? 1.0f : 0.0f);
        // layer 2
        MLP_ISSUE_BEGIN();
#pragma unroll
        for (int k = 0; k < MLP_H / 16; ++k)
            mma_bf16(tmem + TM_ACT, kmaj_desc(aR1, MLP_H, k), kmaj_desc(aW2, MLP_H, k), idesc_bf16(128, MLP_H), k > 0);
        MLP_ISSUE_END();
        MLP_WAIT();
        hidden_epilogue(tl + TM_ACT, b2, R2, tid, H2T, m2);
#pragma unroll
        for (int i = MLP_H; i < MLP_NG; ++i) st_bf16(H2T, kmaj(i, tid, MLP_T), i == MLP_H ? 1.0f : 0.0f);
        // layer 3
        MLP_ISSUE_BEGIN();
#pragma unroll
        for (int k = 0; k < MLP_H / 16; ++k)
            mma_bf16(tmem + TM_ACT, kmaj_desc(aR2, MLP_H, k), kmaj_desc(aW3, MLP_H, k), idesc_bf16(128, MLP_N3), k > 0);
        MLP_ISSUE_END();
        MLP_WAIT();
        {
            float z[MLP_N3];
            tmem_ld16(tl + TM_ACT, *reinterpret_cast<float(*)[16]>(z));
            tmem_ld16(tl + TM_ACT + 16, *reinterpret_cast<float(*)[16]>(z + 16));
            tmem_ld16(tl + TM_ACT + 32, *reinterpret_cast<float(*)[16]>(z + 32));
#pragma unroll
            for (int i = 0; i < MLP_OUT; ++i) z[i] += b3[i];
            float mx = z[0];
#pragma unroll
            for (int i = 1; i < MLP_BINS; ++i) mx = fmaxf(mx, z[i]);
            float S = 0.0f;
#pragma unroll
            for (int i = 0; i < MLP_BINS; ++i) S += expf(z[i] - mx);
            const float lse = mx + logf(S);
            float zbin = 0.0f;
            float dz[MLP_N3];
#pragma unroll
            for (int i = 0; i < MLP_BINS; ++i) {
                if (i == bin) zbin = z[i];
                dz[i] = (expf(z[i] - lse) - (i == bin ? 1.0f : 0.0f)) * w;
            }
            const float zp = z[MLP_BINS], P = 1.0f / (1.0f + expf(-zp));
            // -log P = softplus(-zp), -log(1 - P) = softplus(zp)
            nll_sum += w * (lse - zbin);
            geo_sum += w * ((float)(kt - 1) * softplus(zp) + softplus(-zp));
            dz[MLP_BINS] = ((float)kt * P - 1.0f) * w;
#pragma unroll
            for (int i = MLP_OUT; i < MLP_N3; ++i) dz[i] = 0.0f;
            // dZ as the A operand (row = sample, K = 48) into R1 (free: layer 2 is done)
#pragma unroll
            for (int c = 0; c < MLP_N3 / 8; ++c)
                *reinterpret_cast<uint4 *>(R1 + kmaj(tid, 8 * c, MLP_N3)) = pack8(dz + 8 * c);
            // dZ^T (rows = outputs, K = samples) into T1, rows 33..63 zero
#pragma unroll
            for (int o = 0; o < MLP_H; ++o) st_bf16(T1, kmaj(o, tid, MLP_T), o < MLP_N3 ? dz[o] : 0.0f);
        }
        // dH2 = dZ W3 (B = W3^T, K = 48);  dW3 += dZ^T [H2 | 1]
        MLP_ISSUE_BEGIN();
#pragma unroll
        for (int k = 0; k < MLP_N3 / 16; ++k)
            mma_bf16(tmem + TM_ACT, kmaj_desc(aR1, MLP_N3, k), kmaj_desc(aW3T, MLP_N3, k), idesc_bf16(128, MLP_H),
                     k > 0);
#pragma unroll
        for (int k = 0; k < MLP_T / 16; ++k)
            mma_bf16(tmem + TM_G3, kmaj_desc(aT1, MLP_T, k), kmaj_desc(aH2T, MLP_T, k), idesc_bf16(128, MLP_NG),
                     (ntl > 0 || k > 0) ? 1u : 0u);
        MLP_ISSUE_END();
        MLP_WAIT();
        // dH2 masked by layer 2's activity -> R2 (row = sample) and T2 (rows = units)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            tmem_ld16(tl + TM_ACT + 16 * c, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int u = 16 * c + i;
                if (!((m2[u >> 5] >> (u & 31)) & 1u)) v[i] = 0.0f;
                st_bf16(T2, kmaj(u, tid, MLP_T), v[i]);
            }
            *reinterpret_cast<uint4 *>(R2 + kmaj(tid, 16 * c, MLP_H)) = pack8(v);
            *reinterpret_cast<uint4 *>(R2 + kmaj(tid, 16 * c + 8, MLP_H)) = pack8(v + 8);
        }
        // dH1 = dH2' W2 (B = W2^T);  dW2 += dH2'^T [H1 | 1]
        MLP_ISSUE_BEGIN();
#pragma unroll
        for (int k = 0; k < MLP_H / 16; ++k)
            mma_bf16(tmem + TM_ACT, kmaj_desc(aR2, MLP_H, k), kmaj_desc(aW2T, MLP_H, k), idesc_bf16(128, MLP_H),
                     k > 0);
#pragma unroll
        for (int k = 0; k < MLP_T / 16; ++k)
            mma_bf16(tmem + TM_G2, kmaj_desc(aT2, MLP_T, k), kmaj_desc(aH1T, MLP_T, k), idesc_bf16(128, MLP_NG),
                     (ntl > 0 || k > 0) ? 1u : 0u);
        MLP_ISSUE_END();
        MLP_WAIT();
        // dH1 masked by layer 1's activity -> T1 (rows = units; dZ^T is consumed)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[16];
            tmem_ld16(tl + TM_ACT + 16 * c, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int u = 16 * c + i;
                st_bf16(T1, kmaj(u, tid, MLP_T), ((m1[u >> 5] >> (u & 31)) & 1u) ? v[i] : 0.0f);
            }
        }
        // dW1 += dH1'^T [X | 1]
        MLP_ISSUE_BEGIN();
#pragma unroll
        for (int k = 0; k < MLP_T / 16; ++k)
            mma_bf16(tmem + TM_G1, kmaj_desc(aT1, MLP_T, k), kmaj_desc(aXT, MLP_T, k), idesc_bf16(128, MLP_NG1),
                     (ntl > 0 || k > 0) ? 1u : 0u);
        MLP_ISSUE_END();
        MLP_WAIT();
        fence_before();
    }
#undef MLP_WAIT
#undef MLP_ISSUE_BEGIN
#undef MLP_ISSUE_END
    float *part = net.partials + (size_t)blockIdx.x * MLP_PSTRIDE;
    if (ok) {
        if (ntl == 0) {
            for (int p = tid; p < MLP_NPARAM; p += MLP_T) part[p] = 0.0f;
        } else if (warp < 2) {  // gradient rows 0..63 live in the first 64 lanes
            const int row = tid;
            float v[16];
#pragma unroll
            for (int c = 0; c < MLP_NG / 16; ++c) {
                tmem_ld16(tl + TM_G3 + 16 * c, v);
                if (row < MLP_OUT) {
                    for (int i = 0; i < 16; ++i) {
                        const int col = 16 * c + i;
                        if (col < MLP_H) part[P_W3 + row * MLP_H + col] = v[i];
                        else if (col == MLP_H) part[P_B3 + row] = v[i];
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < MLP_NG / 16; ++c) {
                tmem_ld16(tl + TM_G2 + 16 * c, v);
                for (int i = 0; i < 16; ++i) {
                    const int col = 16 * c + i;
                    if (col < MLP_H) part[P_W2 + row * MLP_H + col] = v[i];
                    else if (col == MLP_H) part[P_B2 + row] = v[i];
                }
            }
            tmem_ld16(tl + TM_G1, v);
            for (int i = 0; i < MLP_IN; ++i) part[P_W1 + row * MLP_IN + i] = v[i];
            part[P_B1 + row] = v[MLP_IN];
        }
        // loss sums over the block, in a fixed order
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nll_sum += __shfl_down_sync(0xffffffffu, nll_sum, o);
            geo_sum += __shfl_down_sync(0xffffffffu, geo_sum, o);
        }
        if (lane == 0) {
            s_red[2 * warp] = nll_sum;
            s_red[2 * warp + 1] = geo_sum;
        }
        __syncthreads();
        if (tid == 0) {
            float a = 0.0f, b = 0.0f;
            for (int q = 0; q < MLP_T / 32; ++q) {
                a += s_red[2 * q];
                b += s_red[2 * q + 1];
            }
            part[MLP_NPARAM] = a;
            part[MLP_NPARAM + 1] = b;
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_dealloc(tmem, TM_COLS);
    if (!ok && tid == 0) atomicExch(net.status, CMCG_ERR_SPIN);
}

// Sum of the training partials in slot order (deterministic); mode 0 takes an
// Adam step (beta1 0.9, beta2 0.999, eps 1e-8, step t >= 1), writes the two
// mean losses to out[0..1] (when out is given) and repacks the image; mode 1
// only writes the summed gradient and the losses to out[0 .. MLP_NPARAM + 1].
__global__ void __launch_bounds__(1024) k_mlp_adam(MlpNet net, int nparts, float lr, int t, int mode, float *out)
{
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(beta1, (float)t), c2 = 1.0f - powf(beta2, (float)t);
    for (int p = threadIdx.x; p < MLP_NPARAM + 2; p += blockDim.x) {
        float g = 0.0f;
        for (int c = 0; c < nparts; ++c) g += net.partials[(size_t)c * MLP_PSTRIDE + p];
        if (mode == 1) {
            out[p] = g;
        } else if (p >= MLP_NPARAM) {
            if (out) out[p - MLP_NPARAM] = g;
        } else {
            const float m = beta1 * net.m[p] + (1.0f - beta1) * g;
            const float v = beta2 * net.v[p] + (1.0f - beta2) * g * g;
            net.m[p] = m;
            net.v[p] = v;
            net.w[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
        }
    }
    if (mode == 1) return;
    __syncthreads();
    pack_image(net.w, net.img, threadIdx.x, blockDim.x);
}

}  // namespace cmcg
