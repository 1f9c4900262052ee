// Integer roofline probe (measurement only, built into its own library
// liblcg_probe.so, not into the alignment engine): the sustained rate of the
// operation the Sankoff recursion is made of, an int32 add followed by a max
// (max(x + y, z)), on every SM. Each thread runs independent dependency chains so the probe is
// throughput-, not latency-bound. One add+max counts as 2 integer ops, the
// unit of the DP's operation count (10 per cell, 2 per arc-pair candidate).
#include <cuda_runtime.h>
#include <stdint.h>

namespace lcg {

constexpr int PEAK_CHAINS = 8;

template <bool DPX>
__global__ void int_peak_kernel(const int *__restrict__ seed, int iters, int *__restrict__ out) {
    int x[PEAK_CHAINS];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int inc = seed[0] + (t & 7), floor_v = seed[1];
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = seed[2 + c] + t;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < PEAK_CHAINS; ++c) {
            if (DPX) x[c] = __viaddmax_s32(x[c], inc, floor_v + c);
            else x[c] = max(x[c] + inc, floor_v + c);
        }
    }
    int s = 0;
#pragma unroll
    for (int c = 0; c < PEAK_CHAINS; ++c) s ^= x[c];
    if (s == 0x7fffffff) out[t] = s;  // keeps the chains alive
}

// Returns the measured rate in G int32 ops/s (2 per add+max).
cudaError_t measure_int_peak(int sms, bool dpx, cudaStream_t st, double *gops) {
    int *d = nullptr;
    const int threads = 256, blocks = sms * 8;
    const int iters = 1 << 14;
    cudaError_t e = cudaMalloc(&d, sizeof(int) * (16 + (size_t)threads * blocks));
    if (e != cudaSuccess) return e;
    int h[16] = {-3, -1000000, 1, 2, 3, 4, 5, 6, 7, 8};
    cudaMemcpyAsync(d, h, sizeof h, cudaMemcpyHostToDevice, st);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(a, st);
        if (dpx) int_peak_kernel<true><<<blocks, threads, 0, st>>>(d, iters, d + 16);
        else int_peak_kernel<false><<<blocks, threads, 0, st>>>(d, iters, d + 16);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    double ops = 2.0 * PEAK_CHAINS * (double)iters * threads * blocks;
    *gops = ops / (best * 1e-3) / 1e9;
    return e;
}

}  // namespace lcg

// Measured int32 add+max rate of CUDA device `device` in G ops/s, with plain
// add/max instructions (dpx = 0) or the fused __viaddmax_s32 (dpx = 1).
// Returns 0 on success, else the cudaError_t of the failing call.
extern "C" int lcg_probe_int_peak(int device, int dpx, double *gops) {
    if (!gops) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return (int)e;
    e = lcg::measure_int_peak(sms, dpx != 0, (cudaStream_t)0, gops);
    return (int)e;
}
