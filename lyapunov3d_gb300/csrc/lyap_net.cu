// lyap_net.cu -- the learned proposal: training of the lambda-predicting MLP
// on the GPU, its forward pass at arbitrary points, and the proposal grid a
// render reads (a lower bound of the net's lambda per cell, built once per
// net and cached).  No reference counterpart: the reference marches every
// sample (kernel.cu:326-363).
//
// Kernels (all tiles of 128 points, one per thread and per TMEM lane):
//  * make_samples  -- training set: seeded points uniform in the box, lambda
//    by the plain FP32 method (RuntimeLambda<MODE_PLAIN>, the drop-in's own
//    lyap4d), clamped;
//  * train_tile    -- forward and backward of one batch tile: four
//    tcgen05.mma products (f.W1^T, h1.W2^T, dz2.W2, and both weight
//    gradients at once as [dz2^T; dz1^T] . [h1^T; f^T]^T, M = 128, N = 112,
//    K = the tile's 128 points), partial gradients per CTA;
//  * adam_step     -- sums the CTAs' partials in a fixed order (training is
//    deterministic) and applies Adam with a cosine learning rate;
//  * forward_tiles -- the forward pass at the corners of the proposal grid,
//    at the held-out samples, and for lyap_net_eval;
//  * grid_cells / grid_dilate -- per cell of the proposal grid the minimum
//    of the net at its 8 corners (any NaN: -inf), optionally the minimum
//    over the 27 cells around it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "lyap_internal.h"
#include "lyap_kernels.cuh"
#include "lyap_net.cuh"

namespace lyapgb {
namespace net {

// ------------------------------------------------ shared-memory layouts
// The tiles sit so that every operand read, under either reading of the
// descriptors' two byte offsets, stays inside the CTA's allocation.
struct FwdLayout {
    static constexpr uint32_t A1 = 0;                     // 128 x 48 features
    static constexpr uint32_t A2 = A1 + TILE * NF * 2;    // 128 x 64 h1
    static constexpr uint32_t W1 = A2 + TILE * NH * 2;    // 64 x 48
    static constexpr uint32_t W2 = W1 + NH * NF * 2;      // 64 x 64
    static constexpr uint32_t PAR = W2 + NH * NH * 2;     // b1[64] b2[64] w3[64] b3 (FP32)
    static constexpr uint32_t MBAR = PAR + 1024;
    static constexpr uint32_t TSLOT = MBAR + 8;
    static constexpr uint32_t END = TSLOT + 8;
    // 56 KiB keeps at most four CTAs on an SM: 4 x 128 TMEM columns = all 512
    static constexpr uint32_t BYTES = 56 * 1024;
    static constexpr uint32_t TMEM_COLS = 128;
};
static_assert(FwdLayout::END <= FwdLayout::BYTES, "forward layout");

struct TrainLayout {
    static constexpr uint32_t RS = 67;                    // reduction row stride (floats)
    static constexpr uint32_t A1 = 0;                     // 128 x 48 features
    static constexpr uint32_t A2 = A1 + TILE * NF * 2;    // 128 x 64 h1
    static constexpr uint32_t W1 = A2 + TILE * NH * 2;    // 64 x 48
    static constexpr uint32_t W2 = W1 + NH * NF * 2;      // 64 x 64
    static constexpr uint32_t W2T = W2 + NH * NH * 2;     // 64 x 64, transposed
    static constexpr uint32_t DZ2 = W2T + NH * NH * 2;    // 128 x 64 dz2
    static constexpr uint32_t AG = DZ2 + TILE * NH * 2;   // 128 x 128: [dz2^T; dz1^T] over the tile's points
    static constexpr uint32_t BG = AG + 128 * TILE * 2;   // 112 x 128: [h1^T; f^T]
    static constexpr uint32_t RED = BG + 112 * TILE * 2;  // 128 x RS floats
    static constexpr uint32_t PAR = RED + TILE * RS * 4;
    static constexpr uint32_t MBAR = PAR + 1024;
    static constexpr uint32_t TSLOT = MBAR + 8;
    static constexpr uint32_t END = TSLOT + 8;
    static constexpr uint32_t BYTES = (END + 1023) & ~1023u;   // > 114 KiB: one CTA per SM
    static constexpr uint32_t TMEM_COLS = 512;
    // TMEM columns of the four products
    static constexpr uint32_t D1 = 0, D2 = 64, D3 = 128, DG = 256;
};
static_assert(TrainLayout::BYTES <= 227 * 1024, "train layout");
static_assert(TrainLayout::BYTES > 114 * 1024, "one train CTA per SM");

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// small parameters into shared memory: b1, b2, BF16-rounded w3, b3
__device__ __forceinline__ void load_small(float *par, const float *__restrict__ params)
{
    const uint32_t t = threadIdx.x;
    if (t < NH) {
        par[t] = params[OFF_B1 + t];
        par[NH + t] = params[OFF_B2 + t];
        par[2 * NH + t] = bf16_round(params[OFF_W3 + t]);
    }
    if (t == 0) par[3 * NH] = params[OFF_B3];
}

// ------------------------------------------------------------ training set
__global__ void __launch_bounds__(256) make_samples(const int32_t *seq, uint32_t period, LyapParams prm,
                                                     float3 lo, float3 ext, uint64_t seed, uint32_t n, float tlo,
                                                     float thi, float4 *__restrict__ out)
{
    const RuntimeLambda<MODE_PLAIN> lam(seq, period, prm);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t it = 0; it < rounds; it++) {
        const uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const uint64_t key = seed + 3ull * (i < n ? i : 0u);
        const float u0 = (float)(mix64(key) >> 40) * 0x1p-24f;
        const float u1 = (float)(mix64(key + 1) >> 40) * 0x1p-24f;
        const float u2 = (float)(mix64(key + 2) >> 40) * 0x1p-24f;
        bool sk, fb;
        const float l = lam(lo.x + ext.x * u0, lo.y + ext.y * u1, lo.z + ext.z * u2, sk, fb);
        const float t = (l != l) ? tlo : fminf(fmaxf(l, tlo), thi);
        if (i < n) out[i] = make_float4(u0, u1, u2, t);
    }
}

// points (device xyz) and targets into the training-set format, in the net's box
__global__ void __launch_bounds__(256) to_samples(const float *__restrict__ xyz, const float *__restrict__ target,
                                                   uint32_t n, float3 lo, float3 inv, float4 *__restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = make_float4((xyz[3 * i] - lo.x) * inv.x, (xyz[3 * i + 1] - lo.y) * inv.y,
                             (xyz[3 * i + 2] - lo.z) * inv.z, target ? target[i] : 0.0f);
}

// --------------------------------------------------------- train one tile
struct TrainArgs {
    const float *params;     // FP32 masters
    const float4 *data;      // (u0, u1, u2, target)
    uint32_t n_data;
    uint32_t random;         // 1: sample with replacement (hash of seed, step, slot); 0: slot = index
    uint64_t seed;
    const uint32_t *step;    // device step counter (random)
    float *partial;          // per CTA NPARAM gradient sums + the loss
    float inv_batch;         // 1 / (gridDim.x * 128)
    unsigned long long *stats;
};

__global__ void __launch_bounds__(128, 1) train_tile(const TrainArgs a)
{
    using L = TrainLayout;
    extern __shared__ __align__(1024) uint8_t sm[];
    const uint32_t tid = threadIdx.x;
    float *par = reinterpret_cast<float *>(sm + L::PAR);
    float *red = reinterpret_cast<float *>(sm + L::RED);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + L::MBAR);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + L::TSLOT);

    load_weight(sm + L::W1, a.params + OFF_W1, NH, NF, false);
    load_weight(sm + L::W2, a.params + OFF_W2, NH, NH, false);
    load_weight(sm + L::W2T, a.params + OFF_W2, NH, NH, true);
    load_small(par, a.params);
    if (tid == 0) {
        tc::mbar_init(mbar, 1);
        tc::mbar_fence_init();
    }
    if (tid < 32) {
        tc::tmem_alloc(tslot, L::TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;

    const uint32_t slot = blockIdx.x * TILE + tid;
    uint32_t idx = slot;
    if (a.random) idx = (uint32_t)(mix64(a.seed + ((uint64_t)(*a.step) << 32) + slot) % a.n_data);
    const float4 d = a.data[idx];
    {
        float f[NF];
        features(d.x, d.y, d.z, f);
        store_row<NF>(sm + L::A1, TILE, tid, f);
#pragma unroll
        for (uint32_t c = 0; c < NF; c++) store_elem(sm + L::BG, 112, NH + c, tid, f[c]);
    }
    bool ok = run_mma(mbar, phase, [&] { mma_tile(tmem + L::D1, sm + L::A1, sm + L::W1, NH, NF, NH); });

    if (ok) {
        float h1[NH];
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            float v[32];
            tmem_row32(tmem, L::D1 + half * 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) {
                float th;
                h1[half * 32 + i] = gelu(v[i] + par[half * 32 + i], th);
            }
        }
        store_row<NH>(sm + L::A2, TILE, tid, h1);
#pragma unroll
        for (uint32_t c = 0; c < NH; c++) store_elem(sm + L::BG, 112, c, tid, h1[c]);
        ok = run_mma(mbar, phase, [&] { mma_tile(tmem + L::D2, sm + L::A2, sm + L::W2, NH, NH, NH); });
    }

    // output, loss, and the output layer's gradients
    float *part = a.partial + (size_t)blockIdx.x * (NPARAM + 1);
    if (ok) {
        float out = par[3 * NH];
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            float v[32];
            tmem_row32(tmem, L::D2 + half * 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) {
                float th;
                out += gelu(v[i] + par[NH + half * 32 + i], th) * par[2 * NH + half * 32 + i];
            }
        }
        const float err = out - d.w;
        const float g = 2.0f * err * a.inv_batch;
        float dz2[NH];
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            float v[32];
            tmem_row32(tmem, L::D2 + half * 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) {
                const uint32_t c = half * 32 + i;
                const float z = v[i] + par[NH + c];
                float th;
                const float h = gelu(z, th);
                red[tid * L::RS + c] = g * h;
                dz2[c] = g * par[2 * NH + c] * gelu_grad(z, th);
            }
        }
        red[tid * L::RS + 64] = g;
        red[tid * L::RS + 65] = err * err * a.inv_batch;
        store_row<NH>(sm + L::DZ2, TILE, tid, dz2);
#pragma unroll
        for (uint32_t c = 0; c < NH; c++) store_elem(sm + L::AG, TILE, c, tid, dz2[c]);
        __syncthreads();
        if (tid < 66) {
            float s = 0.0f;
            for (uint32_t r = 0; r < TILE; r++) s += red[r * L::RS + tid];
            part[tid < 64 ? OFF_W3 + tid : (tid == 64 ? OFF_B3 : NPARAM)] = s;
        }
        __syncthreads();
#pragma unroll
        for (uint32_t c = 0; c < NH; c++) red[tid * L::RS + c] = dz2[c];
        __syncthreads();
        if (tid < NH) {
            float s = 0.0f;
            for (uint32_t r = 0; r < TILE; r++) s += red[r * L::RS + tid];
            part[OFF_B2 + tid] = s;
        }
        __syncthreads();
        // dh1 = dz2 . W2
        ok = run_mma(mbar, phase, [&] { mma_tile(tmem + L::D3, sm + L::DZ2, sm + L::W2T, NH, NH, NH); });
    }
    if (ok) {
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            float vd[32], vz[32];
            tmem_row32(tmem, L::D3 + half * 32, vd);
            tmem_row32(tmem, L::D1 + half * 32, vz);
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) {
                const uint32_t c = half * 32 + i;
                const float z = vz[i] + par[c];
                float th;
                (void)gelu(z, th);
                const float dz1 = vd[i] * gelu_grad(z, th);
                store_elem(sm + L::AG, TILE, NH + c, tid, dz1);
                red[tid * L::RS + c] = dz1;
            }
        }
        __syncthreads();
        if (tid < NH) {
            float s = 0.0f;
            for (uint32_t r = 0; r < TILE; r++) s += red[r * L::RS + tid];
            part[OFF_B1 + tid] = s;
        }
        // both weight gradients: rows 0..63 x columns 0..63 = dW2, rows 64..127 x columns 64..111 = dW1
        ok = run_mma(mbar, phase, [&] { mma_tile(tmem + L::DG, sm + L::AG, sm + L::BG, 112, TILE, 112); });
    }
    if (ok) {
        if (tid < NH) {
#pragma unroll
            for (uint32_t half = 0; half < 2; half++) {
                float v[32];
                tmem_row32(tmem, L::DG + half * 32, v);
#pragma unroll
                for (uint32_t i = 0; i < 32; i++) part[OFF_W2 + tid * NH + half * 32 + i] = v[i];
            }
        } else {
            float v[32], w[16];
            tmem_row32(tmem, L::DG + 64, v);
            tc::tmem_ld16(tmem + (((tid >> 5) * 32u) << 16) + L::DG + 96, w);
            float *row = part + OFF_W1 + (tid - NH) * NF;
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) row[i] = v[i];
#pragma unroll
            for (uint32_t i = 0; i < 16; i++) row[32 + i] = w[i];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, L::TMEM_COLS);
    }
    if (!ok && tid == 0 && a.stats) atomicAdd(a.stats + LYAP_STAT_NET_TIMEOUTS, 1ull);
}

// ------------------------------------------------------------------ Adam
// ctr[0] = step, ctr[1] = ticket; the last block to finish advances the step.
__global__ void __launch_bounds__(256) adam_step(float *__restrict__ params, float *__restrict__ m,
                                                  float *__restrict__ v, const float *__restrict__ partial,
                                                  uint32_t nparts, uint32_t *ctr, uint32_t total, float lr,
                                                  float *__restrict__ loss_hist)
{
    const uint32_t step = *reinterpret_cast<volatile uint32_t *>(ctr);
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p <= NPARAM) {
        float g = 0.0f;
        for (uint32_t c = 0; c < nparts; c++) g += partial[(size_t)c * (NPARAM + 1) + p];
        if (p == NPARAM) {
            if (loss_hist) loss_hist[step] = g;
        } else {
            const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
            const float mm = b1 * m[p] + (1.0f - b1) * g;
            const float vv = b2 * v[p] + (1.0f - b2) * g * g;
            m[p] = mm;
            v[p] = vv;
            const float t = (float)(step + 1);
            const float mhat = mm / (1.0f - powf(b1, t));
            const float vhat = vv / (1.0f - powf(b2, t));
            const float lr_t = lr * 0.5f * (1.0f + cospif((float)step / (float)total));
            params[p] -= lr_t * mhat / (sqrtf(vhat) + eps);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(ctr + 1, 1u);
        if (t == gridDim.x - 1) {
            ctr[1] = 0u;
            __threadfence();
            atomicAdd(ctr, 1u);
        }
    }
}

// fixed-order sum of the CTAs' partials (lyap_net_grad)
__global__ void __launch_bounds__(256) sum_partials(const float *__restrict__ partial, uint32_t nparts,
                                                     float *__restrict__ grad, float *__restrict__ loss)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > NPARAM) return;
    float g = 0.0f;
    for (uint32_t c = 0; c < nparts; c++) g += partial[(size_t)c * (NPARAM + 1) + p];
    if (p < NPARAM) grad[p] = g;
    else if (loss) *loss = g;
}

// --------------------------------------------------------- forward tiles
template <class Src>
__global__ void __launch_bounds__(128) forward_tiles(const float *__restrict__ params, const Src src,
                                                      unsigned long long *stats)
{
    using L = FwdLayout;
    extern __shared__ __align__(1024) uint8_t sm[];
    const uint32_t tid = threadIdx.x;
    float *par = reinterpret_cast<float *>(sm + L::PAR);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + L::MBAR);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + L::TSLOT);

    const uint64_t ntiles = src.tiles();
    if ((uint64_t)blockIdx.x >= ntiles) return;   // whole CTA: nothing allocated yet
    load_weight(sm + L::W1, params + OFF_W1, NH, NF, false);
    load_weight(sm + L::W2, params + OFF_W2, NH, NH, false);
    load_small(par, params);
    if (tid == 0) {
        tc::mbar_init(mbar, 1);
        tc::mbar_fence_init();
    }
    if (tid < 32) {
        tc::tmem_alloc(tslot, L::TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;
    bool ok = true;
    uint32_t points = 0;

    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t p = tile * TILE + tid;
        float u0, u1, u2;
        const bool valid = src.point(p, u0, u1, u2);
        points += valid ? 1u : 0u;
        {
            float f[NF];
            features(u0, u1, u2, f);
            store_row<NF>(sm + L::A1, TILE, tid, f);
        }
        ok = run_mma(mbar, phase, [&] { mma_tile(tmem, sm + L::A1, sm + L::W1, NH, NF, NH); });
        if (!ok) break;
        {
            float h1[NH];
#pragma unroll
            for (uint32_t half = 0; half < 2; half++) {
                float v[32];
                tmem_row32(tmem, half * 32, v);
#pragma unroll
                for (uint32_t i = 0; i < 32; i++) {
                    float th;
                    h1[half * 32 + i] = gelu(v[i] + par[half * 32 + i], th);
                }
            }
            store_row<NH>(sm + L::A2, TILE, tid, h1);
        }
        ok = run_mma(mbar, phase, [&] { mma_tile(tmem + NH, sm + L::A2, sm + L::W2, NH, NH, NH); });
        if (!ok) break;
        float out = par[3 * NH];
#pragma unroll
        for (uint32_t half = 0; half < 2; half++) {
            float v[32];
            tmem_row32(tmem, NH + half * 32, v);
#pragma unroll
            for (uint32_t i = 0; i < 32; i++) {
                float th;
                out += gelu(v[i] + par[NH + half * 32 + i], th) * par[2 * NH + half * 32 + i];
            }
        }
        src.result(p, valid, out);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, L::TMEM_COLS);
    }
    if (stats) {
        const uint32_t s = __reduce_add_sync(FULL, points);
        if ((tid & 31u) == 0 && s && Src::POINT_STAT >= 0) atomicAdd(stats + Src::POINT_STAT, (unsigned long long)s);
        if (!ok && tid == 0) atomicAdd(stats + LYAP_STAT_NET_TIMEOUTS, 1ull);
    }
}

// lyap_net_eval: points from device xyz
struct EvalSrc {
    static constexpr int POINT_STAT = -1;
    const float *xyz;
    float *out;
    uint64_t n;
    float lo[3], inv[3];
    __device__ uint64_t tiles() const { return (n + TILE - 1) / TILE; }
    __device__ bool point(uint64_t p, float &u0, float &u1, float &u2) const
    {
        u0 = u1 = u2 = 0.5f;
        if (p >= n) return false;
        u0 = (xyz[3 * p] - lo[0]) * inv[0];
        u1 = (xyz[3 * p + 1] - lo[1]) * inv[1];
        u2 = (xyz[3 * p + 2] - lo[2]) * inv[2];
        return true;
    }
    __device__ void result(uint64_t p, bool valid, float o) const
    {
        if (valid) out[p] = o;
    }
};

// the training set's held-out part (u already in [0,1]^3)
struct SampleSrc {
    static constexpr int POINT_STAT = -1;
    const float4 *data;
    float *out;
    uint64_t n;
    __device__ uint64_t tiles() const { return (n + TILE - 1) / TILE; }
    __device__ bool point(uint64_t p, float &u0, float &u1, float &u2) const
    {
        u0 = u1 = u2 = 0.5f;
        if (p >= n) return false;
        const float4 d = data[p];
        u0 = d.x;
        u1 = d.y;
        u2 = d.z;
        return true;
    }
    __device__ void result(uint64_t p, bool valid, float o) const
    {
        if (valid) out[p] = o;
    }
};

// ---------------------------------------------------------- proposal grid
// the corners of an n^3 grid over the net's box: (n + 1)^3 points, x fastest
struct GridSrc {
    static constexpr int POINT_STAT = LYAP_STAT_PROPOSAL_POINTS;
    float *out;
    uint32_t m;   // corners per axis (n + 1)
    uint64_t total;
    __device__ uint64_t tiles() const { return (total + TILE - 1) / TILE; }
    __device__ bool point(uint64_t p, float &u0, float &u1, float &u2) const
    {
        u0 = u1 = u2 = 0.5f;
        if (p >= total) return false;
        const uint64_t mm = (uint64_t)m * m;
        const uint32_t k = (uint32_t)(p / mm);
        const uint32_t j = (uint32_t)((p - (uint64_t)k * mm) / m);
        const uint32_t i = (uint32_t)(p - (uint64_t)k * mm - (uint64_t)j * m);
        const float inv = 1.0f / (float)(m - 1);
        u0 = (float)i * inv;
        u1 = (float)j * inv;
        u2 = (float)k * inv;
        return true;
    }
    __device__ void result(uint64_t p, bool valid, float o) const
    {
        if (valid) out[p] = o;
    }
};

// cell (i, j, k) of n^3 = min of the net at its 8 corners; a NaN corner
// makes the cell -inf (never skipped)
__global__ void __launch_bounds__(256) grid_cells(const float *__restrict__ corner, float *__restrict__ cell,
                                                  uint32_t n)
{
    const uint64_t total = (uint64_t)n * n * n;
    const uint64_t m = n + 1;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < total;
         c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t nn = (uint64_t)n * n;
        const uint64_t k = c / nn, j = (c - k * nn) / n, i = c - k * nn - j * n;
        float v = __int_as_float(0x7f800000);
#pragma unroll
        for (int d = 0; d < 8; d++) {
            const float x = corner[((k + (d >> 2)) * m + (j + ((d >> 1) & 1))) * m + (i + (d & 1))];
            v = (x == x) ? fminf(v, x) : __int_as_float(0xff800000);
        }
        cell[c] = v;
    }
}

// the proposal's bits for one threshold: bit c set when cell[c] >= tau
__global__ void __launch_bounds__(256) grid_bits(const float *__restrict__ cell, uint32_t *__restrict__ bits,
                                                 uint64_t ncell, float tau)
{
    const uint64_t nword = (ncell + 31) / 32;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nword;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = 0;
        for (uint32_t j = 0; j < 32; j++) {
            const uint64_t c = w * 32 + j;
            if (c < ncell && cell[c] >= tau) b |= 1u << j;
        }
        bits[w] = b;
    }
}

// the minimum over the (up to) 27 cells around each cell
__global__ void __launch_bounds__(256) grid_dilate(const float *__restrict__ in, float *__restrict__ out, uint32_t n)
{
    const uint64_t total = (uint64_t)n * n * n;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < total;
         c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t nn = (uint64_t)n * n;
        const int k = (int)(c / nn), j = (int)((c - (uint64_t)k * nn) / n), i = (int)(c - (uint64_t)k * nn - (uint64_t)j * n);
        float v = __int_as_float(0x7f800000);
        for (int dk = -1; dk <= 1; dk++)
            for (int dj = -1; dj <= 1; dj++)
                for (int di = -1; di <= 1; di++) {
                    const int kk = k + dk, jj = j + dj, ii = i + di;
                    if (kk < 0 || jj < 0 || ii < 0 || kk >= (int)n || jj >= (int)n || ii >= (int)n) continue;
                    v = fminf(v, in[((uint64_t)kk * n + jj) * n + ii]);
                }
        out[c] = v;
    }
}

static bool g_attr_done[64];

static cudaError_t set_smem_attrs()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64 && g_attr_done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TrainLayout::BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(forward_tiles<EvalSrc>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)FwdLayout::BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(forward_tiles<SampleSrc>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)FwdLayout::BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(forward_tiles<GridSrc>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)FwdLayout::BYTES);
    if (e == cudaSuccess && dev >= 0 && dev < 64) g_attr_done[dev] = true;
    return e;
}

static uint32_t fwd_grid(uint64_t tiles)
{
    const uint64_t cap = (uint64_t)device_sm_count() * 4;
    return (uint32_t)(tiles < cap ? (tiles ? tiles : 1) : cap);
}

}  // namespace net

// ------------------------------------------------ proposal grid (lyap_render)
// FNV-1a 64 (LyapNet.hash, and the grid cache's key)
uint64_t fnv64(const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

namespace {

// built grids, per (device, hash of the net's bytes, cells per axis,
// dilation); kept for the life of the process (kGridsKeep at most, the least
// recently used dropped).  The hash is computed here, not read from
// LyapNet.hash, which callers that fill the struct themselves may not set.
struct GridEntry {
    float *grid = nullptr;
    uint64_t order = 0;
};
std::mutex g_grid_mu;
std::map<std::tuple<int, uint64_t, uint32_t, uint32_t>, GridEntry> g_grids;
uint64_t g_grid_order = 0;
constexpr size_t kGridsKeep = 8;
// the bits of a grid for one threshold (tau's bit pattern in the key)
std::map<std::tuple<int, uint64_t, uint32_t, uint32_t, uint32_t>, GridEntry> g_bits;

template <class Map>
void drop_oldest(Map &m)
{
    if (m.size() < kGridsKeep) return;
    auto old = m.begin();
    for (auto jt = m.begin(); jt != m.end(); ++jt)
        if (jt->second.order < old->second.order) old = jt;
    cudaFree(old->second.grid);   // synchronises the device: no launch still reads it
    m.erase(old);
}

}  // namespace

static cudaError_t proposal_grid_locked(const LyapNet &netw, uint64_t hash, uint32_t n, uint32_t dilate,
                                       const float **grid, unsigned long long *stats, cudaStream_t s);

cudaError_t proposal_grid(const LyapNet &netw, uint32_t n, uint32_t dilate, const float **grid,
                          unsigned long long *stats, cudaStream_t s)
{
    std::lock_guard<std::mutex> lock(g_grid_mu);
    return proposal_grid_locked(netw, fnv64(&netw, offsetof(LyapNet, hash)), n, dilate, grid, stats, s);
}

cudaError_t proposal_bits(const LyapNet &netw, uint32_t n, uint32_t dilate, float tau, const uint32_t **bits,
                          unsigned long long *stats, cudaStream_t s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    uint32_t tau_bits;
    memcpy(&tau_bits, &tau, sizeof(tau_bits));
    const uint64_t hash = fnv64(&netw, offsetof(LyapNet, hash));
    const auto key = std::make_tuple(dev, hash, n, dilate, tau_bits);
    std::lock_guard<std::mutex> lock(g_grid_mu);
    auto it = g_bits.find(key);
    if (it != g_bits.end()) {
        it->second.order = ++g_grid_order;
        *bits = reinterpret_cast<const uint32_t *>(it->second.grid);
        return cudaSuccess;
    }
    const float *grid = nullptr;
    if ((e = proposal_grid_locked(netw, hash, n, dilate, &grid, stats, s)) != cudaSuccess) return e;
    const uint64_t ncell = (uint64_t)n * n * n, nword = (ncell + 31) / 32;
    uint32_t *out = nullptr;
    if ((e = cudaMalloc((void **)&out, nword * sizeof(uint32_t))) != cudaSuccess) return e;
    net::grid_bits<<<(uint32_t)device_sm_count() * 4u, 256, 0, s>>>(grid, out, ncell, tau);
    e = cudaGetLastError();
    // complete before any stream may read it from the cache
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(out);
        return e;
    }
    drop_oldest(g_bits);
    GridEntry ent;
    ent.grid = reinterpret_cast<float *>(out);
    ent.order = ++g_grid_order;
    g_bits[key] = ent;
    *bits = out;
    return cudaSuccess;
}

static cudaError_t proposal_grid_locked(const LyapNet &netw, uint64_t hash, uint32_t n, uint32_t dilate,
                                       const float **grid, unsigned long long *stats, cudaStream_t s)
{
    using namespace net;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(dev, hash, n, dilate);
    auto it = g_grids.find(key);
    if (it != g_grids.end()) {
        it->second.order = ++g_grid_order;
        *grid = it->second.grid;
        return cudaSuccess;
    }
    if ((e = set_smem_attrs()) != cudaSuccess) return e;
    const uint64_t m = (uint64_t)n + 1, ncorner = m * m * m, ncell = (uint64_t)n * n * n;
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    // scratch: the net's parameters, the corner values, and (with dilation) the undilated cells
    const size_t bytes = up(NPARAM * sizeof(float)) + up(ncorner * sizeof(float)) +
                         (dilate ? up(ncell * sizeof(float)) : 0);
    char *tmp = nullptr;
    float *out = nullptr;
    if ((e = cudaMalloc((void **)&out, ncell * sizeof(float))) != cudaSuccess) return e;
    if ((e = scratch_alloc((void **)&tmp, bytes, s)) != cudaSuccess) {
        cudaFree(out);
        return e;
    }
    float *d_params = reinterpret_cast<float *>(tmp);
    float *corner = reinterpret_cast<float *>(tmp + up(NPARAM * sizeof(float)));
    float *undilated = dilate ? reinterpret_cast<float *>(tmp + up(NPARAM * sizeof(float)) +
                                                          up(ncorner * sizeof(float)))
                              : out;
    e = cudaMemcpyAsync(d_params, netw.params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        GridSrc src;
        src.out = corner;
        src.m = (uint32_t)m;
        src.total = ncorner;
        forward_tiles<GridSrc><<<fwd_grid((ncorner + TILE - 1) / TILE), TILE, FwdLayout::BYTES, s>>>(d_params, src,
                                                                                                     stats);
        e = cudaGetLastError();
    }
    const uint32_t blocks = (uint32_t)device_sm_count() * 8u;
    if (e == cudaSuccess) {
        grid_cells<<<blocks, 256, 0, s>>>(corner, undilated, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && dilate) {
        grid_dilate<<<blocks, 256, 0, s>>>(undilated, out, n);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(tmp, s);
    // complete before any stream may read it from the cache
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(out);
        return e;
    }
    drop_oldest(g_grids);
    GridEntry ent;
    ent.grid = out;
    ent.order = ++g_grid_order;
    g_grids[key] = ent;
    *grid = out;
    return cudaSuccess;
}

}  // namespace lyapgb

// ============================================================ C entry points
using namespace lyapgb;
using namespace lyapgb::net;

namespace {

uint32_t fnv32_add(uint32_t h, const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 16777619u;
    }
    return h;
}

void net_rehash(LyapNet *net) { net->hash = fnv64(net, offsetof(LyapNet, hash)); }

int check_net(const LyapNet *net, const char *fn)
{
    if (!net) return set_error(LYAP_ERR_INVALID_ARG, "%s: null net", fn);
    if (net->magic != LYAP_NET_MAGIC || net->version != LYAP_NET_VERSION)
        return set_error(LYAP_ERR_INVALID_ARG, "%s: not a LyapNet (magic %08x, version %u)", fn, net->magic,
                         net->version);
    for (int k = 0; k < 3; k++)
        if (!(net->hi[k] > net->lo[k]))
            return set_error(LYAP_ERR_INVALID_ARG, "%s: empty input box on axis %d", fn, k);
    return LYAP_OK;
}

// He-normal initial weights, zero biases (SplitMix64 + Box-Muller)
void init_params(float *p, uint64_t seed)
{
    uint64_t state = seed ^ 0x4C59504E45540000ull;
    auto uni = [&]() {
        state += 0x9E3779B97F4A7C15ull;
        return ((double)(mix64(state) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() {
        const double u = uni(), v = uni();
        return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
    };
    std::memset(p, 0, NPARAM * sizeof(float));
    for (uint32_t i = 0; i < NH * NF; i++) p[OFF_W1 + i] = (float)(normal() * std::sqrt(2.0 / NF));
    for (uint32_t i = 0; i < NH * NH; i++) p[OFF_W2 + i] = (float)(normal() * std::sqrt(2.0 / NH));
    for (uint32_t i = 0; i < NH; i++) p[OFF_W3 + i] = (float)(normal() * std::sqrt(1.0 / NH));
}

struct DeviceBuffers {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit DeviceBuffers(cudaStream_t st) : s(st) {}
    cudaError_t alloc(void **p, size_t bytes)
    {
        cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, s);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    ~DeviceBuffers()
    {
        for (void *p : ptrs) cudaFreeAsync(p, s);
    }
};

}  // namespace

extern "C" int lyap_net_train(const LyapParams *prm, const int32_t *seq, size_t seq_len,
                              const LyapNetTrainOptions *opt, LyapNet *net, void *stream)
{
    const char *fn = "lyap_net_train";
    if (!prm || !seq || !net) return set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    if (seq_len < 2 || seq_len > LYAP_MAX_SEQ_LEN)
        return set_error(LYAP_ERR_SEQUENCE, "%s: seq_len %zu outside [2, %d]", fn, seq_len, LYAP_MAX_SEQ_LEN);
    for (size_t i = 0; i + 1 < seq_len; i++)
        if (seq[i] < 0 || seq[i] > 3) return set_error(LYAP_ERR_SEQUENCE, "%s: symbol %d at %zu", fn, seq[i], i);
    if (seq[seq_len - 1] != -1) return set_error(LYAP_ERR_SEQUENCE, "%s: sequence is not -1 terminated", fn);
    LyapNetTrainOptions o;
    std::memset(&o, 0, sizeof(o));
    if (opt) {
        if (opt->size != sizeof(LyapNetTrainOptions))
            return set_error(LYAP_ERR_INVALID_ARG, "%s: LyapNetTrainOptions.size is %u, expected %zu", fn, opt->size,
                             sizeof(LyapNetTrainOptions));
        o = *opt;
    }
    const uint32_t n = o.n_samples ? o.n_samples : (1u << 20);
    const uint32_t nval = o.n_val ? o.n_val : (1u << 16);
    const uint32_t batch = o.batch ? o.batch : 4096u;
    const uint32_t steps = o.steps ? o.steps : 8192u;
    const float lr = o.lr != 0.0f ? o.lr : 3e-3f;
    const float tlo = (o.target_lo == 0.0f && o.target_hi == 0.0f) ? -3.0f : o.target_lo;
    const float thi = (o.target_lo == 0.0f && o.target_hi == 0.0f) ? 1.0f : o.target_hi;
    if (batch % TILE || batch > 32768u) return set_error(LYAP_ERR_INVALID_ARG, "%s: batch %u", fn, batch);
    if (n > (1u << 28) || nval > (1u << 24)) return set_error(LYAP_ERR_INVALID_ARG, "%s: too many samples", fn);
    if (!(lr > 0.0f) || !(thi > tlo)) return set_error(LYAP_ERR_INVALID_ARG, "%s: bad lr or target range", fn);
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        lo[k] = o.box_lo ? o.box_lo[k] : prm->lMin;
        hi[k] = o.box_hi ? o.box_hi[k] : prm->lMax;
        if (!(hi[k] > lo[k])) return set_error(LYAP_ERR_INVALID_ARG, "%s: empty box on axis %d", fn, k);
    }
    if (device_sm_count() <= 0) return cuda_error(cudaErrorNoDevice, fn);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = set_smem_attrs();
    if (e != cudaSuccess) return cuda_error(e, fn);

    const uint32_t nct = batch / TILE;
    std::vector<float> h_params(NPARAM);
    init_params(h_params.data(), o.seed);
    int rc = LYAP_OK;
    {
        DeviceBuffers B(s);
        int32_t *d_seq = nullptr;
        float4 *d_data = nullptr;
        float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_partial = nullptr, *d_loss = nullptr,
              *d_val = nullptr;
        uint32_t *d_ctr = nullptr;
        unsigned long long *d_stats = nullptr;
        if ((e = B.alloc((void **)&d_seq, seq_len * sizeof(int32_t))) == cudaSuccess &&
            (e = B.alloc((void **)&d_data, (size_t)(n + nval) * sizeof(float4))) == cudaSuccess &&
            (e = B.alloc((void **)&d_params, NPARAM * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_m, NPARAM * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_v, NPARAM * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_partial, (size_t)nct * (NPARAM + 1) * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_loss, (size_t)steps * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_val, (size_t)nval * sizeof(float))) == cudaSuccess &&
            (e = B.alloc((void **)&d_ctr, 2 * sizeof(uint32_t))) == cudaSuccess &&
            (e = B.alloc((void **)&d_stats, LYAP_STAT_COUNT * sizeof(unsigned long long))) == cudaSuccess) {
            e = cudaMemcpyAsync(d_seq, seq, seq_len * sizeof(int32_t), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_params, h_params.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(d_m, 0, NPARAM * sizeof(float), s);
            if (e == cudaSuccess) e = cudaMemsetAsync(d_v, 0, NPARAM * sizeof(float), s);
            if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, 2 * sizeof(uint32_t), s);
            if (e == cudaSuccess) e = cudaMemsetAsync(d_stats, 0, LYAP_STAT_COUNT * sizeof(unsigned long long), s);
        }
        if (e == cudaSuccess) {
            const int sms = device_sm_count();
            make_samples<<<(uint32_t)sms * 8, 256, 0, s>>>(d_seq, (uint32_t)(seq_len - 1), *prm,
                                                           make_float3(lo[0], lo[1], lo[2]),
                                                           make_float3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]),
                                                           o.seed * 0x9E3779B97F4A7C15ull + 1u, n + nval, tlo, thi,
                                                           d_data);
            e = cudaGetLastError();
            TrainArgs a;
            a.params = d_params;
            a.data = d_data;
            a.n_data = n;
            a.random = 1;
            a.seed = mix64(o.seed + 0x7261696Eull);
            a.step = d_ctr;
            a.partial = d_partial;
            a.inv_batch = 1.0f / (float)batch;
            a.stats = d_stats;
            const uint32_t agrid = (NPARAM + 1 + 255) / 256;
            for (uint32_t st = 0; st < steps && e == cudaSuccess; st++) {
                train_tile<<<nct, TILE, TrainLayout::BYTES, s>>>(a);
                adam_step<<<agrid, 256, 0, s>>>(d_params, d_m, d_v, d_partial, nct, d_ctr, steps, lr, d_loss);
                if ((st & 511u) == 511u || st == 0) {
                    // stop early if a tensor-core wait ran out (each later step would wait as long)
                    unsigned long long to = 0;
                    e = cudaMemcpyAsync(&to, d_stats + LYAP_STAT_NET_TIMEOUTS, sizeof(to), cudaMemcpyDeviceToHost, s);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                    if (e == cudaSuccess && to) break;
                }
            }
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) {
                SampleSrc src;
                src.data = d_data + n;
                src.out = d_val;
                src.n = nval;
                forward_tiles<SampleSrc><<<fwd_grid((nval + TILE - 1) / TILE), TILE, FwdLayout::BYTES, s>>>(
                    d_params, src, d_stats);
                e = cudaGetLastError();
            }
        }
        std::vector<float> h_loss(steps), h_val(nval);
        std::vector<float4> h_tgt(nval);
        unsigned long long h_stats[LYAP_STAT_COUNT] = {};
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_params.data(), d_params, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_loss.data(), d_loss, steps * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_val.data(), d_val, nval * sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_tgt.data(), d_data + n, nval * sizeof(float4), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_stats, d_stats, sizeof(h_stats), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = cuda_error(e, fn);
        } else if (h_stats[LYAP_STAT_NET_TIMEOUTS]) {
            rc = set_error(LYAP_ERR_CUDA, "%s: %llu tensor-core waits timed out", fn, h_stats[LYAP_STAT_NET_TIMEOUTS]);
        } else {
            std::memset(net, 0, sizeof(*net));
            net->magic = LYAP_NET_MAGIC;
            net->version = LYAP_NET_VERSION;
            for (int k = 0; k < 3; k++) {
                net->lo[k] = lo[k];
                net->hi[k] = hi[k];
            }
            std::memcpy(net->params, h_params.data(), NPARAM * sizeof(float));
            const uint32_t tail = steps < 100u ? steps : 100u;
            double tl = 0.0;
            for (uint32_t i = steps - tail; i < steps; i++) tl += h_loss[i];
            net->train_mse = (float)(tl / tail);
            double vl = 0.0;
            for (uint32_t i = 0; i < nval; i++) {
                const double d = (double)h_val[i] - (double)h_tgt[i].w;
                vl += d * d;
            }
            net->val_mse = (float)(vl / nval);
            net->steps = steps;
            net->batch = batch;
            net->n_samples = n;
            uint32_t h = 2166136261u;
            h = fnv32_add(h, seq, seq_len * sizeof(int32_t));
            h = fnv32_add(h, &prm->settle, sizeof(prm->settle));
            h = fnv32_add(h, &prm->accum, sizeof(prm->accum));
            h = fnv32_add(h, &prm->d, sizeof(prm->d));
            net->seq_hash = h;
            net_rehash(net);
            if (o.h_loss) std::memcpy(o.h_loss, h_loss.data(), steps * sizeof(float));
        }
    }
    return rc;
}

extern "C" int lyap_net_grid(const LyapNet *netw, uint32_t n, uint32_t dilate, float *d_out, void *stream)
{
    const char *fn = "lyap_net_grid";
    int rc = check_net(netw, fn);
    if (rc) return rc;
    if (!d_out) return set_error(LYAP_ERR_INVALID_ARG, "%s: null output", fn);
    if (n == 0) n = LYAP_PROPOSAL_GRID_DEFAULT;
    if (n < 2 || n > 512) return set_error(LYAP_ERR_INVALID_ARG, "%s: %u cells per axis outside 2..512", fn, n);
    if (dilate > 1) return set_error(LYAP_ERR_INVALID_ARG, "%s: dilate must be 0 or 1", fn);
    if (device_sm_count() <= 0) return cuda_error(cudaErrorNoDevice, fn);
    cudaStream_t s = (cudaStream_t)stream;
    const float *grid = nullptr;
    cudaError_t e = proposal_grid(*netw, n, dilate, &grid, nullptr, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_out, grid, (size_t)n * n * n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, fn);
}

extern "C" int lyap_net_eval(const LyapNet *netw, const float *d_xyz, size_t n, float *d_out, void *stream)
{
    const char *fn = "lyap_net_eval";
    int rc = check_net(netw, fn);
    if (rc) return rc;
    if (!d_xyz || !d_out) return set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    if (n == 0) return LYAP_OK;
    if (device_sm_count() <= 0) return cuda_error(cudaErrorNoDevice, fn);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = set_smem_attrs();
    float *d_params = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_params, NPARAM * sizeof(float), s);
    if (e != cudaSuccess) return cuda_error(e, fn);
    e = cudaMemcpyAsync(d_params, netw->params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        EvalSrc src;
        src.xyz = d_xyz;
        src.out = d_out;
        src.n = n;
        for (int k = 0; k < 3; k++) {
            src.lo[k] = netw->lo[k];
            src.inv[k] = 1.0f / (netw->hi[k] - netw->lo[k]);
        }
        forward_tiles<EvalSrc><<<fwd_grid((n + TILE - 1) / TILE), TILE, FwdLayout::BYTES, s>>>(d_params, src,
                                                                                               nullptr);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(d_params, s);
    if (e != cudaSuccess) return cuda_error(e, fn);
    if (e2 != cudaSuccess) return cuda_error(e2, fn);
    return LYAP_OK;
}

extern "C" int lyap_net_grad(const LyapNet *netw, const float *d_xyz, const float *d_target, size_t n, float *d_grad,
                             float *d_loss, void *stream)
{
    const char *fn = "lyap_net_grad";
    int rc = check_net(netw, fn);
    if (rc) return rc;
    if (!d_xyz || !d_target || !d_grad) return set_error(LYAP_ERR_INVALID_ARG, "%s: null pointer", fn);
    if (n == 0 || n % TILE || n > 32768)
        return set_error(LYAP_ERR_INVALID_ARG, "%s: n = %zu is not a multiple of 128 in [128, 32768]", fn, n);
    if (device_sm_count() <= 0) return cuda_error(cudaErrorNoDevice, fn);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = set_smem_attrs();
    if (e != cudaSuccess) return cuda_error(e, fn);
    const uint32_t nct = (uint32_t)(n / TILE);
    DeviceBuffers B(s);
    float *d_params = nullptr, *d_partial = nullptr;
    float4 *d_data = nullptr;
    if ((e = B.alloc((void **)&d_params, NPARAM * sizeof(float))) == cudaSuccess &&
        (e = B.alloc((void **)&d_partial, (size_t)nct * (NPARAM + 1) * sizeof(float))) == cudaSuccess &&
        (e = B.alloc((void **)&d_data, n * sizeof(float4))) == cudaSuccess)
        e = cudaMemcpyAsync(d_params, netw->params, NPARAM * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        float3 lo = make_float3(netw->lo[0], netw->lo[1], netw->lo[2]);
        float3 inv = make_float3(1.0f / (netw->hi[0] - netw->lo[0]), 1.0f / (netw->hi[1] - netw->lo[1]),
                                 1.0f / (netw->hi[2] - netw->lo[2]));
        to_samples<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(d_xyz, d_target, (uint32_t)n, lo, inv, d_data);
        TrainArgs a;
        std::memset(&a, 0, sizeof(a));
        a.params = d_params;
        a.data = d_data;
        a.n_data = (uint32_t)n;
        a.random = 0;
        a.partial = d_partial;
        a.inv_batch = 1.0f / (float)n;
        train_tile<<<nct, TILE, TrainLayout::BYTES, s>>>(a);
        sum_partials<<<(NPARAM + 1 + 255) / 256, 256, 0, s>>>(d_partial, nct, d_grad, d_loss);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, fn);
}

extern "C" int lyap_net_save(const LyapNet *netw, const char *path)
{
    int rc = check_net(netw, "lyap_net_save");
    if (rc) return rc;
    if (!path) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_save: null path");
    LyapNet copy = *netw;
    net_rehash(&copy);
    FILE *f = std::fopen(path, "wb");
    if (!f) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_save: cannot open %s", path);
    const size_t w = std::fwrite(&copy, sizeof(copy), 1, f);
    const int c = std::fclose(f);
    if (w != 1 || c != 0) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_save: write to %s failed", path);
    return LYAP_OK;
}

extern "C" int lyap_net_load(LyapNet *netw, const char *path)
{
    if (!netw || !path) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_load: null pointer");
    FILE *f = std::fopen(path, "rb");
    if (!f) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_load: cannot open %s", path);
    LyapNet tmp;
    const size_t r = std::fread(&tmp, sizeof(tmp), 1, f);
    const int extra = std::fgetc(f);
    std::fclose(f);
    if (r != 1 || extra != EOF) return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_load: %s is not %zu bytes", path, sizeof(tmp));
    int rc = check_net(&tmp, "lyap_net_load");
    if (rc) return rc;
    if (fnv64(&tmp, offsetof(LyapNet, hash)) != tmp.hash)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_net_load: %s: hash mismatch", path);
    *netw = tmp;
    return LYAP_OK;
}
