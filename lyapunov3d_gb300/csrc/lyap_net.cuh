// lyap_net.cuh -- the learned proposal's network on the device: Fourier
// features, GELU, BF16 operand tiles and the tensor-core matrix products.
//
// Network (lyap_gb300.h, LyapNet): u = (P - lo) / (hi - lo) in [0,1]^3;
// 48 features sin(pi 2^k u_j), cos(pi 2^k u_j) (k = 0..7, j = 0..2, index
// 2*(3k+j) + {0, 1}); h1 = gelu(W1 f + b1), h2 = gelu(W2 h1 + b2) (64 each);
// lambda = w3 . h2 + b3.  Both matrix products run on the tensor cores as
// tcgen05.mma kind::f16 with BF16 operands and FP32 accumulators in TMEM, for
// tiles of 128 points (one point per thread and per TMEM lane).
#pragma once

#include <stdint.h>

#include "lyap_gb300.h"
#include "lyap_tc.cuh"

namespace lyapgb {
namespace net {

constexpr uint32_t NF = LYAP_NET_FEATURES, NH = LYAP_NET_HIDDEN, TILE = 128;
constexpr uint32_t OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
                   OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
static_assert(NPARAM == LYAP_NET_PARAMS, "parameter layout");

// polls of an mbarrier before a tensor-core wait counts as failed (about
// 0.1-0.5 s; a product of these sizes completes within microseconds)
constexpr uint32_t WAIT_POLLS = 1u << 24;

__device__ __forceinline__ unsigned short to_bf16(float x)
{
    unsigned short h;
    asm("cvt.rn.bf16.f32 %0, %1;" : "=h"(h) : "f"(x));
    return h;
}
__device__ __forceinline__ float bf16_round(float x) { return __uint_as_float((uint32_t)to_bf16(x) << 16); }
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// GELU, tanh form: x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
constexpr float GELU_K0 = 0.7978845608028654f, GELU_K1 = 0.044715f;
__device__ __forceinline__ float gelu(float x, float &th)
{
    th = tanh_approx(GELU_K0 * fmaf(GELU_K1 * x * x, x, x));
    return 0.5f * x * (1.0f + th);
}
__device__ __forceinline__ float gelu_grad(float x, float th)
{
    return 0.5f * (1.0f + th) + 0.5f * x * (1.0f - th * th) * GELU_K0 * fmaf(3.0f * GELU_K1, x * x, 1.0f);
}

// The 48 features: one sincospi per axis, then the double-angle recurrence
// sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a).
__device__ __forceinline__ void features(float u0, float u1, float u2, float (&f)[NF])
{
    const float u[3] = {u0, u1, u2};
#pragma unroll
    for (int j = 0; j < 3; j++) {
        float s, c;
        sincospif(u[j], &s, &c);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            f[2 * (3 * k + j)] = s;
            f[2 * (3 * k + j) + 1] = c;
            const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
}

// Row `row` (K values, rounded to BF16) of a K-major tile with R rows.
template <int K>
__device__ __forceinline__ void store_row(uint8_t *tile, uint32_t R, uint32_t row, const float *v)
{
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 8) {
        uint4 q;
        q.x = pack_bf16x2(v[k0 + 0], v[k0 + 1]);
        q.y = pack_bf16x2(v[k0 + 2], v[k0 + 3]);
        q.z = pack_bf16x2(v[k0 + 4], v[k0 + 5]);
        q.w = pack_bf16x2(v[k0 + 6], v[k0 + 7]);
        *reinterpret_cast<uint4 *>(tile + tc::kmajor_offset(row, (uint32_t)k0, R)) = q;
    }
}
__device__ __forceinline__ void store_elem(uint8_t *tile, uint32_t R, uint32_t r, uint32_t k, float v)
{
    *reinterpret_cast<unsigned short *>(tile + tc::kmajor_offset(r, k, R)) = to_bf16(v);
}

// A weight matrix W[N][K] (row-major FP32) as the B operand of x W^T: an
// N-row K-major BF16 tile; transposed: the K-row tile of W^T (element
// (k, n) = W[n][k]), the B operand of d W.
__device__ __forceinline__ void load_weight(uint8_t *tile, const float *__restrict__ W, uint32_t N, uint32_t K,
                                            bool transposed)
{
    for (uint32_t e = threadIdx.x; e < N * K; e += blockDim.x) {
        const uint32_t n = e / K, k = e % K;
        const float w = __ldg(W + e);
        if (transposed) store_elem(tile, K, k, n, w);
        else store_elem(tile, N, n, k, w);
    }
}

// D[tmem] = A (128 x K) . B (N x K)^T, K a multiple of 16; one thread issues.
__device__ __forceinline__ void mma_tile(uint32_t d_tmem, const uint8_t *A, const uint8_t *B, uint32_t RB,
                                         uint32_t K, uint32_t N)
{
    const uint32_t a = tc::smem_addr(A), b = tc::smem_addr(B);
    const uint32_t lboA = (TILE / 8) * 128, lboB = (RB / 8) * 128;
    const uint32_t idesc = tc::idesc_bf16_f32(TILE, N);
    for (uint32_t s = 0; s < K / 16; s++)
        tc::mma_bf16(d_tmem, tc::smem_desc(a + s * 2 * lboA, lboA, 128), tc::smem_desc(b + s * 2 * lboB, lboB, 128),
                     idesc, s > 0 ? 1u : 0u);
}

// Hand the tiles written by all threads to the tensor core: thread 0 issues
// `issue` (a sequence of mma_tile) and commits onto mbar; every thread waits
// for the products.  Returns false (on every thread) if the wait ran out.
template <class Issue>
__device__ __forceinline__ bool run_mma(uint64_t *mbar, uint32_t &phase, Issue issue)
{
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        issue();
        tc::mma_commit(mbar);
    }
    const bool ok = tc::mbar_wait(mbar, phase, WAIT_POLLS);
    phase ^= 1u;
    tc::fence_after_sync();
    return __syncthreads_and(ok) != 0;
}

// 32 FP32 columns starting at `col` of this thread's TMEM lane
__device__ __forceinline__ void tmem_row32(uint32_t tmem, uint32_t col, float (&v)[32])
{
    const uint32_t warp = threadIdx.x >> 5;
    tc::tmem_ld32(tmem + ((warp * 32u) << 16) + col, v);
}

}  // namespace net
}  // namespace lyapgb
