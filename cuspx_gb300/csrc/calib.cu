// calib.cu -- integer peak microbenchmarks (the roofline denominators).
//
// The hash cores are bound by 32-bit integer issue: funnel-shift rotates
// (SHF), three-input logic (LOP3) and three-input adds (IADD3) on the ALU
// pipe.  Mix 0 issues that shape alone -- per step 3 SHF + 1 LOP3 + 1 IADD3,
// one SHA-256 Sigma plus its add -- which is also the Keccak-f shape (no
// adds move off the ALU there).  Mix 1 is a SHA-256 round as the hash core
// issues it: Sigma (3 SHF + LOP3), Ch (LOP3), a four-input add (2 IADD3) and
// one add as IMAD on the FMA pipe (a * c_one + b with an opaque constant-bank
// one), 7 ALU : 1 FMA like the compression's 1208 : 176.  Both run eight
// independent chains per thread so latency is hidden, at full occupancy on
// every SM.  ops/s = threads x iterations x chains x ops per step / elapsed.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cuspx.h"
#include "spx_hash.cuh"

namespace {

constexpr int kChains = 8;
__constant__ uint32_t c_calib_one = 1u;

template <int MIX>
__global__ void k_int_mix(uint32_t *out, int iters, uint32_t seed) {
    uint32_t x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = seed * (threadIdx.x + 1) + c * 0x9e3779b9u + blockIdx.x;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            uint32_t v = x[c];
            uint32_t s = __funnelshift_r(v, v, 6) ^ __funnelshift_r(v, v, 11) ^ __funnelshift_r(v, v, 25);
            if (MIX == 0) {
                x[c] = v + s + 0x428a2f98u + c;
            } else {
                uint32_t y = x[(c + 1) % kChains], z = x[(c + 2) % kChains];
                uint32_t t = v + s + ((v & y) ^ (~v & z)) + 0x428a2f98u;
                x[c] = t * c_calib_one + (0x71374491u + c);
            }
        }
    }
    uint32_t acc = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) acc ^= x[c];
    if (acc == 0x12345678u) out[0] = acc;  // keeps the chains live
}

// Each thread runs `iters` SHA-256 compressions in a dependent chain (every
// block is built from the previous state), like one lane of a verify task:
// with one warp per SM this is the latency of a compression, with more it
// shows how many warps an SM needs before the ALU pipe, not the round's
// dependency chain, sets the rate.
__global__ void k_cmp_chain(uint32_t *out, int iters, uint32_t seed) {
    uint32_t st[8], w[16];
#pragma unroll
    for (int i = 0; i < 8; i++) st[i] = seed * (threadIdx.x + 1) + i * 0x9e3779b9u + blockIdx.x;
#pragma unroll
    for (int i = 0; i < 16; i++) w[i] = seed ^ (i * 0x7f4a7c15u) ^ threadIdx.x;
    for (int it = 0; it < iters; it++) {
        uint32_t m[16];
#pragma unroll
        for (int i = 0; i < 16; i++) m[i] = w[i] ^ st[i & 7];
        cuspx::sha256_compress(st, m);
    }
    uint32_t acc = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) acc ^= st[i];
    if (acc == 0x12345678u) out[0] = acc;  // keeps the chain live
}

}  // namespace

extern "C" int cuspx_cmp_rate(int device, int warps_per_sm, int iters, double *cmp_per_s, double *ns_per_cmp) {
    if (!cmp_per_s || iters <= 0 || warps_per_sm < 1 || warps_per_sm > 32) return CUSPX_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return CUSPX_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // one block per SM, so every SM holds exactly warps_per_sm warps
    const int threads = 32 * warps_per_sm, blocks = sms;
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, 4) != cudaSuccess) return CUSPX_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_cmp_chain<<<blocks, threads>>>(out, iters / 8 + 1, 1u);  // warm-up
    cudaEventRecord(e0);
    k_cmp_chain<<<blocks, threads>>>(out, iters, 1u);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return CUSPX_ECUDA;
    *cmp_per_s = (double)blocks * threads * iters / (ms * 1e-3);
    if (ns_per_cmp) *ns_per_cmp = ms * 1e6 / iters;
    return CUSPX_OK;
}

extern "C" int cuspx_int_peak_mix(int device, int iters, int mix, double *ops_per_s, float *ms_out) {
    if (!ops_per_s || iters <= 0 || (mix != 0 && mix != 1)) return CUSPX_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return CUSPX_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = sms * 8;
    void (*kern)(uint32_t *, int, uint32_t) = mix ? k_int_mix<1> : k_int_mix<0>;
    const int ops_per_step = mix ? 8 : 5;
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, 4) != cudaSuccess) return CUSPX_ECUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    kern<<<blocks, threads>>>(out, iters / 4 + 1, 1u);  // warm-up
    cudaEventRecord(e0);
    kern<<<blocks, threads>>>(out, iters, 1u);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return CUSPX_ECUDA;
    const double ops = (double)blocks * threads * iters * kChains * ops_per_step;
    *ops_per_s = ops / (ms * 1e-3);
    if (ms_out) *ms_out = ms;
    return CUSPX_OK;
}

extern "C" int cuspx_int_peak(int device, int iters, double *ops_per_s, float *ms_out) {
    return cuspx_int_peak_mix(device, iters, 0, ops_per_s, ms_out);
}
