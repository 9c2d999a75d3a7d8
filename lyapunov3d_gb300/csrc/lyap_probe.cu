// lyap_probe.cu -- pipe-rate probes: the measured denominators of the
// lambda kernels' roofline.  The lambda loop is bound by the FP32 pipe
// (FMUL/FFMA) or by the MUFU pipe (lg2.approx), not by memory, so its peak
// is "FP32 ops per second" or "lg2 per second" of this GPU at its present
// clock.  Each probe thread runs 8 independent dependency chains so that
// latency is hidden and the pipe, not the chain, limits the rate.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_device.cuh"
#include "lyap_internal.h"

namespace lyapgb {

constexpr int PROBE_CHAINS = 8;

__global__ void __launch_bounds__(256) probe_ffma(uint32_t iters, float *sink)
{
    float a[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) a[k] = 0.5f + 0.01f * (float)(threadIdx.x + k);
    const float m = 0.999f, c = 1e-4f;
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int k = 0; k < PROBE_CHAINS; k++) a[k] = __fmaf_rn(a[k], m, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) s += a[k];
    if (s == 12345.678f) sink[0] = s;   // keeps the chains live
}

__global__ void __launch_bounds__(256) probe_lg2(uint32_t iters, float *sink)
{
    float a[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) a[k] = 1.5f + 0.01f * (float)(threadIdx.x + k);
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int k = 0; k < PROBE_CHAINS; k++) a[k] = lg2_approx(a[k]) + 1.5f;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) s += a[k];
    if (s == 12345.678f) sink[0] = s;
}

// packed pairs: fma.rn.f32x2 rounds each half as fma.rn.f32 does
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t pack2(float lo, float hi)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__global__ void __launch_bounds__(256) probe_ffma2(uint32_t iters, float *sink)
{
    uint64_t a[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++)
        a[k] = pack2(0.5f + 0.01f * (float)(threadIdx.x + k), 0.25f + 0.01f * (float)(threadIdx.x + k));
    const uint64_t m = pack2(0.999f, 0.999f), c = pack2(1e-4f, 1e-4f);
    for (uint32_t i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
#pragma unroll
            for (int k = 0; k < PROBE_CHAINS; k++) a[k] = ffma2(a[k], m, c);
        }
    }
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) s ^= a[k];
    if (s == 0x1234567ull) sink[0] = 1.0f;
}

}  // namespace lyapgb

using namespace lyapgb;

// kind 0: FFMA (ops counted = FFMA instructions x 32 lanes);
// kind 1: lg2.approx (+ one FADD each, counted as lg2 only);
// kind 2: packed FFMA2 (fma.rn.f32x2; ops counted = 2 FMAs per lane per instruction).
// *ops receives the number of operations the launch performs.
extern "C" int lyap_pipe_probe(uint32_t kind, uint32_t iters, float *d_sink, double *ops, void *stream)
{
    if (!d_sink || !ops || kind > 2 || iters == 0)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_pipe_probe: bad arguments");
    const int sms = device_sm_count();
    if (sms <= 0) return cuda_error(cudaErrorNoDevice, "lyap_pipe_probe");
    const uint32_t blocks = (uint32_t)sms * 8, threads = 256;
    if (kind == 0)
        probe_ffma<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, d_sink);
    else if (kind == 1)
        probe_lg2<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, d_sink);
    else
        probe_ffma2<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, d_sink);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "lyap_pipe_probe: launch");
    *ops = (double)blocks * threads * iters * 16.0 * PROBE_CHAINS * (kind == 2 ? 2.0 : 1.0);
    return LYAP_OK;
}
