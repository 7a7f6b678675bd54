// m2_peaks.cu -- integer-multiply roofline denominator.
//
// The squaring chain is exact modular arithmetic on the integer pipes; its
// compute roofline counts 32x32->64-bit products (PTX mul.wide.u32 /
// mad.wide.u32).  This kernel measures their peak rate on the running GPU:
// eight independent mad.wide.u32 chains per thread, enough warps per SM to
// hide the dependent-issue latency.
#include "m2_kernels.cuh"

namespace m2k {

namespace {
constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) k_wide_mul_rate(unsigned long long* sink, unsigned int iters, unsigned int seed) {
    unsigned long long acc[CHAINS];
    unsigned int a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) { a[k] = seed + threadIdx.x * CHAINS + k; acc[k] = k; }
    const unsigned int b = seed ^ 0x9E3779B9u;
    for (unsigned int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k)
            asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc[k]) : "r"(a[k]), "r"(b));
    }
    unsigned long long s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s ^= acc[k];
    if (s == 0x1234567ull) sink[blockIdx.x] = s;   // keeps the chains live
}
}  // namespace

double measure_wide_mul_rate(int device) {
    if (cudaSetDevice(device) != cudaSuccess) return 0.0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    const unsigned int iters = 8192;
    unsigned long long* sink = nullptr;
    if (cudaMalloc(&sink, sizeof(unsigned long long) * blocks) != cudaSuccess) return 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_wide_mul_rate<<<blocks, threads>>>(sink, 256, 1u);   // warm-up
    float best = 1e30f;
    for (int r = 0; r < 3; ++r) {
        cudaEventRecord(e0);
        k_wide_mul_rate<<<blocks, threads>>>(sink, iters, 7u + r);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess || best <= 0.f) return 0.0;
    const double products = (double)blocks * threads * iters * CHAINS;
    return products / (best * 1e-3);
}

}  // namespace m2k
