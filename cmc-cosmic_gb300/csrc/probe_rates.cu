// probe_rates.cu -- throughput of the arithmetic pipes this step leans on:
// FP64 FMA, divide and sqrt, FP32 FMA, INT64 compare/add.  Fixed independent
// chains per thread over 8 blocks per SM; CUDA-event timed after a warm-up.
// Built and run by `python bench.py --probe-rates`.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void k_dfma(double *out, int iters) {
    double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    }
    if (a0 + a1 + a2 + a3 == 12345.0) out[0] = a0;
}
__global__ void k_ffma(float *out, int iters) {
    float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
        a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
    }
    if (a0 + a1 + a2 + a3 == 12345.0f) out[0] = a0;
}
__global__ void k_ddiv(double *out, int iters) {
    double a0 = threadIdx.x + 1.5, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    for (int i = 0; i < iters; ++i) {
        a0 = 1.0 / a0 + 1.0; a1 = 1.0 / a1 + 1.0; a2 = 1.0 / a2 + 1.0; a3 = 1.0 / a3 + 1.0;
    }
    if (a0 + a1 + a2 + a3 == 12345.0) out[0] = a0;
}
__global__ void k_dsqrt(double *out, int iters) {
    double a0 = threadIdx.x + 1.5, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    for (int i = 0; i < iters; ++i) {
        a0 = sqrt(a0) + 1.0; a1 = sqrt(a1) + 1.0; a2 = sqrt(a2) + 1.0; a3 = sqrt(a3) + 1.0;
    }
    if (a0 + a1 + a2 + a3 == 12345.0) out[0] = a0;
}
__global__ void k_i64(long long *out, int iters) {
    long long a0 = threadIdx.x, a1 = a0 + 7, a2 = a0 + 13, a3 = a0 + 17;
    const long long t = 1LL << 40;
    for (int i = 0; i < iters; ++i) {
        a0 = (a0 < t) ? a0 + 3 : a0 - 5; a1 = (a1 < t) ? a1 + 3 : a1 - 5;
        a2 = (a2 < t) ? a2 + 3 : a2 - 5; a3 = (a3 < t) ? a3 + 3 : a3 - 5;
    }
    if (a0 + a1 + a2 + a3 == 12345) out[0] = a0;
}

template <class F>
float timeit(F f) {
    cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
    f(); cudaDeviceSynchronize();
    cudaEventRecord(a); f(); cudaEventRecord(b); cudaEventSynchronize(b);
    float ms; cudaEventElapsedTime(&ms, a, b); return ms;
}

int main() {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    int blocks = sms * 8, threads = 256, it = 4096;
    double *d; float *f; long long *l;
    cudaMalloc(&d, 8); cudaMalloc(&f, 8); cudaMalloc(&l, 8);
    double nthr = (double)blocks * threads;
    float ms;
    ms = timeit([&] { k_dfma<<<blocks, threads>>>(d, it); });
    printf("DFMA : %.3f ms  %.2f TFLOP/s\n", ms, nthr * it * 4 * 2 / ms / 1e9);
    ms = timeit([&] { k_ffma<<<blocks, threads>>>(f, it); });
    printf("FFMA : %.3f ms  %.2f TFLOP/s\n", ms, nthr * it * 4 * 2 / ms / 1e9);
    ms = timeit([&] { k_ddiv<<<blocks, threads>>>(d, it / 8); });
    printf("DDIV : %.3f ms  %.2f Gdiv/s\n", ms, nthr * (it / 8) * 4 / ms / 1e6);
    ms = timeit([&] { k_dsqrt<<<blocks, threads>>>(d, it / 8); });
    printf("DSQRT: %.3f ms  %.2f Gsqrt/s\n", ms, nthr * (it / 8) * 4 / ms / 1e6);
    ms = timeit([&] { k_i64<<<blocks, threads>>>(l, it); });
    printf("I64  : %.3f ms  %.2f Gop/s\n", ms, nthr * it * 4 / ms / 1e6);
    printf("err: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 0;
}
