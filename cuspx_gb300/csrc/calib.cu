// calib.cu -- integer-ALU peak microbenchmark (the roofline denominator).
//
// The hash cores are bound by 32-bit integer issue: funnel-shift rotates
// (SHF), three-input logic (LOP3) and three-input adds (IADD3).  This kernel
// issues that mix -- per step 3 SHF + 1 LOP3 + 1 IADD3, the shape of one
// SHA-256 Sigma plus its add -- on eight independent chains per thread so
// latency is hidden, at full occupancy on every SM.  ops/s = threads x
// iterations x ops per iteration / elapsed.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cuspx.h"

namespace {

constexpr int kChains = 8;
constexpr int kOpsPerStep = 5;  // 3 SHF + LOP3 + IADD3

__global__ void k_int_mix(uint32_t *out, int iters, uint32_t seed) {
    uint32_t x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = seed * (threadIdx.x + 1) + c * 0x9e3779b9u + blockIdx.x;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            uint32_t v = x[c];
            uint32_t s = __funnelshift_r(v, v, 6) ^ __funnelshift_r(v, v, 11) ^ __funnelshift_r(v, v, 25);
            x[c] = v + s + 0x428a2f98u + c;
        }
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) acc ^= x[c];
    if (acc == 0x12345678u) out[0] = acc;  // keeps the chains live
}

}  // namespace

extern "C" int cuspx_int_peak(int device, int iters, double *ops_per_s, float *ms_out) {
    if (!ops_per_s) return CUSPX_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return CUSPX_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = sms * 8;
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, 4) != cudaSuccess) return CUSPX_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_int_mix<<<blocks, threads>>>(out, iters / 4 + 1, 1u);  // warm-up
    cudaEventRecord(e0);
    k_int_mix<<<blocks, threads>>>(out, iters, 1u);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return CUSPX_ECUDA;
    const double ops = (double)blocks * threads * iters * kChains * kOpsPerStep;
    *ops_per_s = ops / (ms * 1e-3);
    if (ms_out) *ms_out = ms;
    return CUSPX_OK;
}
