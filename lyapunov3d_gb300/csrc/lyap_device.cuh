// lyap_device.cuh -- device-side building blocks of the hot path (sm_103a).
//
//  * per-ray arithmetic (ray setup, box slab test, march / hone / normal
//    state machine, shading) that rounds every operation exactly as the
//    reference's host build does (kernel.cu:25-486): this translation unit
//    is compiled with -fmad=false, IEEE division and square root, and uses
//    double precision wherever a double literal in the reference promotes
//    the expression.  Ray positions and step decisions are therefore
//    bit-identical to the oracle's whenever the lambda values agree;
//  * the lambda evaluators (kernel.cu:108-154), the only hot loop:
//      MODE_PLAIN   -- one lg2.approx per accumulated step (the drop-in);
//      MODE_PRODUCT -- running FP32 product of |r(1-2x)| renormalised by
//                      exponent extraction every 8 steps, one lg2 at the end.
//    Both iterate the orbit identically: t = r*x; x = fma(-t, x, t);
//    d = fma(-2r, x, r).  The sequence symbol at every step is warp-uniform,
//    so for periods up to 16 the loop is unrolled over whole periods with
//    the four candidate values of r held in registers.
#pragma once

#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif
#include <stdint.h>

#include "lyap_gb300.h"
#include "lyap_jobs.h"

namespace lyapgb {

constexpr uint32_t MODE_PLAIN = 0;
constexpr uint32_t MODE_PRODUCT = 1;

constexpr uint32_t HONE_CAP = 256;          // honing samples per ray
constexpr uint32_t MARCH_MAX = 4194304u;    // march samples per ray
constexpr float LN2F = 0.693147180559945309417232121458f;

// statistics slots (LYAP_STAT_* in lyap_gb300.h)
constexpr int ST_SAMPLES = 0, ST_SKIPPED = 1, ST_MARCH = 2, ST_HONE = 3, ST_NORMAL = 4,
              ST_HITS = 5, ST_RAYS = 6, ST_FALLBACK = 7;

// Exact float classification without library calls (identical under nvcc and NVRTC).
__device__ __forceinline__ bool f_isnan(float v) { return v != v; }
__device__ __forceinline__ bool f_isfinite(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }

// ---------------------------------------------------------------- vectors
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3(const LyapVec &v) { return V3{v.x, v.y, v.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
// dot in the reference's order: (x*x' + y*y') + z*z'
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// vec3.hpp:127-154: zero below 1e-12, unchanged when |v|^2 == 1, else v/|v|
__device__ __forceinline__ V3 normalized(V3 a)
{
    float mag2 = a.x * a.x + a.y * a.y + a.z * a.z;
    if ((double)mag2 < 1e-12) return v3(0.f, 0.f, 0.f);
    if (mag2 == 1.0f || ((double)mag2 > (1.0 - 1e-12) && (double)mag2 < (1.0 + 1e-12))) return a;
    return a / sqrtf(mag2);
}

struct C4 {
    float x, y, z, w;
};
__device__ __forceinline__ C4 c4(const LyapColor &c) { return C4{c.x, c.y, c.z, c.w}; }
__device__ __forceinline__ C4 operator+(C4 a, C4 b) { return C4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
__device__ __forceinline__ C4 operator*(C4 a, float s) { return C4{a.x * s, a.y * s, a.z * s, a.w * s}; }

// VEC3::clamp(T) (vec3.hpp:190): value-preserving, the compare is in double
__device__ __forceinline__ float clamp01(float v) { return (double)v < 0.0 ? 0.0f : ((double)v > 1.0 ? 1.0f : v); }

__device__ __forceinline__ float lg2_approx(float x)
{
    float y;
    asm("lg2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// --------------------------------------------------------------- sequence
// Everything the lambda loop needs about the forcing sequence, uniform per
// warp.  `wS` packs the symbols of period positions 0..L-1 (2 bits each),
// `wA` those of positions S..S+L-1 (mod L), where accumulation starts.
struct SeqInfo {
    const int32_t *seq;   // -1 terminated, device memory
    uint32_t L;           // period (entries before the terminator)
    uint32_t S, A;        // settle / accumulate iteration counts
    uint32_t wS, wA;      // packed symbols when L <= 16
    uint32_t oA;          // S mod L
    float d;              // value of symbol D
};

__device__ __forceinline__ SeqInfo seq_setup(const int32_t *seq, uint32_t L, const LyapParams &prm)
{
    SeqInfo si;
    si.seq = seq;
    si.L = L;
    si.S = prm.settle;
    si.A = prm.accum;
    si.d = prm.d;
    si.oA = prm.settle % L;
    si.wS = si.wA = 0;
    if (L <= 16) {
        uint32_t k = si.oA;
        for (uint32_t j = 0; j < L; j++) {
            si.wS |= ((uint32_t)seq[j] & 3u) << (2 * j);
            si.wA |= ((uint32_t)seq[k] & 3u) << (2 * j);
            k = (k + 1 == L) ? 0 : k + 1;
        }
    }
    return si;
}

// abcd[sym] (kernel.cu:110-114), as selects on a uniform symbol
__device__ __forceinline__ float pick(uint32_t sym, float x, float y, float z, float d)
{
    float lo = (sym & 1u) ? y : x;
    float hi = (sym & 1u) ? d : z;
    return (sym & 2u) ? hi : lo;
}

// ---------------------------------------------------------------- lambda
// One settle step and one accumulate step of the map (kernel.cu:135,143-146).
__device__ __forceinline__ float map_step(float r, float v)
{
    float t = r * v;
    return __fmaf_rn(-t, v, t);
}

// The product form multiplies the factors d of B consecutive accumulation
// steps (a block) into a running product that restarts every block at
// m * 2^(E-127), m in [1, 2): the block's float exponent goes into an integer
// and the mantissa carries on.  B = 24 when the period's unrolled body
// (max(16, lcm(L, 8)) steps) is a multiple of 24, else 16 when it is a
// multiple of 16, else 8, so that blocks end at fixed places of the body.
// |d| = |r (1 - 2v)| <= r <= 4 on an orbit in [0, 1], so a block stays below
// 2^(E-126) * 4^B < 2^127 with E = 227, 221, 205 (2^100, 2^94, 2^78) for
// B = 8, 16, 24; a product that was subnormal after some step ends below
// 2^-126 * 4^(B-1) = 2^(2B-128), biased exponent 2B - 1.  Scaling by powers
// of 2 is exact, so while no block leaves [2^(2B-128), 2^127) the mantissas,
// exponents and lambda are those of a product restarted at 1 -- the same for
// every B.  The form is defined by B = 8: a sample whose blocks of 16 or 24
// left the range is taken again with blocks of 8 (if a block of 24 stays in
// range, each of its blocks of 8 ends above 2^100 * 2^-159 / 4^16 = 2^-91,
// in range too, so nothing else changes), and a sample out of range with
// blocks of 8 goes to the plain form (below).
__host__ __device__ constexpr uint32_t lcm8(uint32_t L)
{
    return (L % 8u == 0u) ? L : (L % 4u == 0u) ? 2u * L : (L % 2u == 0u) ? 4u * L : 8u * L;
}
__host__ __device__ constexpr uint32_t product_block(uint32_t L)
{
    return (lcm8(L) < 16u ? 16u : lcm8(L)) % 24u == 0u ? 24u : (lcm8(L) < 16u ? 16u : lcm8(L)) % 16u == 0u ? 16u : 8u;
}
__host__ __device__ constexpr uint32_t product_exp(uint32_t B) { return B == 24u ? 205u : B == 16u ? 221u : 227u; }
__host__ __device__ constexpr uint32_t product_lo(uint32_t B) { return 2u * B - 1u; }   // lowest valid block end
__device__ __forceinline__ float product_start(uint32_t B) { return __uint_as_float(product_exp(B) << 23); }

// The plain form's lambda is NaN exactly when its sum of lg2|d| is not
// finite (kernel.cu returns NaN for a non-finite sum), i.e. when some factor
// d is 0, infinite or NaN: a finite sum of at most 2^32 terms of magnitude
// below 2^8 cannot overflow.  Two cases of an out-of-range product are known
// to be such samples without redoing them:
//  - the orbit ended non-finite (r > 4 -- a sample just outside the box, as
//    normal estimation and the last march step take -- lets v leave [0, 1],
//    after which it runs to -inf): the last factor was +inf or NaN;
//  - B = 8, the worst block ended at exactly 0 or subnormal ((biased
//    exponent - 15) = ZERO_BLOCK unsigned) and every r is at least 1/4: for a
//    float v != 1/2, |1 - 2v| >= 2^-24, so eight non-zero factors take a block
//    from 2^100 at most down to 2^100 * 2^-208 -- it had a factor 0.
constexpr uint32_t ZERO_BLOCK = 0u - 15u;
__device__ __forceinline__ bool product_is_nan(uint32_t B, uint32_t mx, float s_end, float x, float y, float z,
                                               float d)
{
    return !f_isfinite(s_end) || (B == 8u && mx == ZERO_BLOCK &&
                                  fminf(fminf(fabsf(x), fabsf(y)), fminf(fabsf(z), fabsf(d))) >= 0.25f);
}

// a block out of range: (biased exponent - lo) above 253 - lo as an unsigned
__device__ __forceinline__ bool product_bad(uint32_t B, uint32_t mx) { return mx > 253u - product_lo(B); }

// the renormalised product's mantissa in [1, 2), for the sample's one log2
__device__ __forceinline__ float product_mantissa(float p)
{
    return __uint_as_float((__float_as_uint(p) & 0x007fffffu) | 0x3f800000u);
}

// The product form's accumulated step on the negated state s = -v, with the
// signed product (|p| is the scalar form's p; renormalisation drops the
// sign): mt = r*s = -(r*v); s' = mt*s + mt = -(t - t*v); d = (2r)*s' + r =
// r - 2r*v'; p' = p*d.  Round-to-nearest is symmetric, so every quantity is
// the plain statement's value or its exact negation -- and no instruction
// beyond the four FP32 operations is needed (no abs, no negation).
__device__ __forceinline__ void product_step(float r, float tr, float &s, float &p)
{
    const float mt = r * s;
    s = __fmaf_rn(mt, s, mt);
    p = p * __fmaf_rn(tr, s, r);
}

// block end with the range check folded into one unsigned maximum: the
// largest (biased exponent - lo) over all blocks decides (product_bad)
__device__ __forceinline__ void renorm_max(uint32_t B, float &p, int32_t &e, uint32_t &mx)
{
    const uint32_t bits = __float_as_uint(p);
    const uint32_t ef = (bits >> 23) & 0xffu;
    mx = max(mx, ef - product_lo(B));
    e += (int32_t)ef;
    p = __uint_as_float((bits & 0x007fffffu) | (product_exp(B) << 23));
}

__host__ __device__ constexpr int ctz_lcm8(int L) { return (L % 8 == 0) ? L : (L % 4 == 0) ? 2 * L : (L % 2 == 0) ? 4 * L : 8 * L; }
template <int L>
struct Unroll {
    static constexpr int U = ctz_lcm8(L) < 16 ? 16 : ctz_lcm8(L);   // multiple of L and of 8
};

template <uint32_t MODE>
__device__ __noinline__ float lambda_generic(float x, float y, float z, const SeqInfo &si, bool &skipped,
                                             bool &fallback, uint32_t block = 0);

// lambda for a period L <= 16: whole blocks of U = lcm(L, 8) steps run fully
// unrolled with r in registers; the < U remaining steps run rolled, taking
// their symbol from the packed word.  Returns lambda; `skipped` = the settle
// landed exactly on 0.5 (or NaN) so nothing was accumulated (kernel.cu:138);
// `fallback` = the product form had to redo the sample in the plain form.
template <uint32_t MODE, int L>
__device__ __forceinline__ float lambda_fixed(float x, float y, float z, const SeqInfo &si, bool &skipped,
                                              bool &fallback)
{
    constexpr int U = Unroll<L>::U;
    const float d = si.d;
    float rS[L], rA[L], mA[L];
#pragma unroll
    for (int j = 0; j < L; j++) {
        rS[j] = pick((si.wS >> (2 * j)) & 3u, x, y, z, d);
        rA[j] = pick((si.wA >> (2 * j)) & 3u, x, y, z, d);
        mA[j] = -2.0f * rA[j];
    }
    float v = 0.5f;
    const uint32_t S = si.S, A = si.A;
    {
        const uint32_t nb = S / U, rem = S - nb * U;
        for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
            for (int j = 0; j < U; j++) v = map_step(rS[j % L], v);
        }
        uint32_t k = 0;
        for (uint32_t j = 0; j < rem; j++) {
            v = map_step(pick((si.wS >> (2 * k)) & 3u, x, y, z, d), v);
            k = (k + 1 == (uint32_t)L) ? 0 : k + 1;
        }
    }
    skipped = !(v < 0.5f || v > 0.5f);
    fallback = false;
    float l2 = 0.0f;
    if (!skipped) {
        const uint32_t nb = A / U, rem = A - nb * U;
        if (MODE == MODE_PLAIN) {
            for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
                for (int j = 0; j < U; j++) {
                    v = map_step(rA[j % L], v);
                    float dd = __fmaf_rn(mA[j % L], v, rA[j % L]);
                    l2 += lg2_approx(fabsf(dd));
                }
            }
            uint32_t k = 0;
            for (uint32_t j = 0; j < rem; j++) {
                const float r = pick((si.wA >> (2 * k)) & 3u, x, y, z, d);
                k = (k + 1 == (uint32_t)L) ? 0 : k + 1;
                v = map_step(r, v);
                float dd = __fmaf_rn(-2.0f * r, v, r);
                l2 += lg2_approx(fabsf(dd));
            }
        } else {
            constexpr uint32_t B = product_block(L);
            static_assert(U % B == 0, "blocks end inside the unrolled body");
            float p = product_start(B), sv = -v;
            int32_t e = 0;
            uint32_t mx = 0;
            for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
                for (int j = 0; j < U; j++) {
                    product_step(rA[j % L], -mA[j % L], sv, p);
                    if (j % B == B - 1) renorm_max(B, p, e, mx);
                }
            }
            uint32_t k = 0, kb = 0;
            for (uint32_t j = 0; j < rem; j++) {
                const float r = pick((si.wA >> (2 * k)) & 3u, x, y, z, d);
                k = (k + 1 == (uint32_t)L) ? 0 : k + 1;
                product_step(r, 2.0f * r, sv, p);
                if (++kb == B) {
                    kb = 0;
                    renorm_max(B, p, e, mx);
                }
            }
            renorm_max(B, p, e, mx);
            const bool bad = product_bad(B, mx);
            // e holds the sum of biased exponents, one bias of product_exp(B) per renorm
            const uint32_t nrenorm = A / B + 1;
            l2 = (float)(e - (int32_t)(product_exp(B) * nrenorm)) + lg2_approx(product_mantissa(p));
            if (bad && product_is_nan(B, mx, sv, x, y, z, d)) return __int_as_float(0x7fffffff);
            if (bad && B != 8u) {
                // blocks of 16 / 24 left the range: take the sample with blocks of 8 (out of line)
                bool sk, fb;
                fallback = true;
                return lambda_generic<MODE_PRODUCT>(x, y, z, si, sk, fb, 8u);
            }
            if (bad) {
                // an intermediate product may have been subnormal: redo in the plain
                // form (the rolled evaluator: same operations, kept out of line)
                fallback = true;
                bool sk, fb;
                return lambda_generic<MODE_PLAIN>(x, y, z, si, sk, fb);
            }
        }
    }
    if (!f_isfinite(l2)) return __int_as_float(0x7fffffff);
    return (l2 * LN2F) / (float)A;
}

// lambda for any period: the symbol is loaded each step (uniform, L1-resident).
// block = 0: the period's block length; 8: the defining one (a redo)
template <uint32_t MODE>
__device__ __noinline__ float lambda_generic(float x, float y, float z, const SeqInfo &si, bool &skipped,
                                             bool &fallback, uint32_t block)
{
    const float d = si.d;
    const int32_t *seq = si.seq;
    const uint32_t L = si.L;
    float v = 0.5f;
    uint32_t k = 0;
    for (uint32_t n = 0; n < si.S; n++) {
        float r = pick((uint32_t)seq[k] & 3u, x, y, z, d);
        k = (k + 1 == L) ? 0 : k + 1;
        v = map_step(r, v);
    }
    skipped = !(v < 0.5f || v > 0.5f);
    fallback = false;
    float l2 = 0.0f;
    if (!skipped) {
        const uint32_t kA = k;
        const float vA = v;
        const uint32_t B = block ? block : product_block(L);
        float p = product_start(B);
        int32_t e = 0;
        uint32_t mx = 0, kb = 0;
        for (uint32_t n = 0; n < si.A; n++) {
            float r = pick((uint32_t)seq[k] & 3u, x, y, z, d);
            k = (k + 1 == L) ? 0 : k + 1;
            v = map_step(r, v);
            float dd = __fmaf_rn(-2.0f * r, v, r);
            if (MODE == MODE_PLAIN) {
                l2 += lg2_approx(fabsf(dd));
            } else {
                p = p * fabsf(dd);
                if (++kb == B) {
                    kb = 0;
                    renorm_max(B, p, e, mx);
                }
            }
        }
        if (MODE == MODE_PRODUCT) {
            renorm_max(B, p, e, mx);
            const uint32_t nrenorm = si.A / B + 1;
            l2 = (float)(e - (int32_t)(product_exp(B) * nrenorm)) + lg2_approx(product_mantissa(p));
            if (product_bad(B, mx) && product_is_nan(B, mx, v, x, y, z, d)) return __int_as_float(0x7fffffff);
            if (product_bad(B, mx) && B != 8u) {
                // blocks of 16 / 24 left the range: take the sample with blocks of 8
                bool sk, fb;
                fallback = true;
                return lambda_generic<MODE_PRODUCT>(x, y, z, si, sk, fb, 8u);
            }
            if (product_bad(B, mx)) {
                fallback = true;
                l2 = 0.0f;
                v = vA;
                k = kA;
                for (uint32_t n = 0; n < si.A; n++) {
                    float r = pick((uint32_t)seq[k] & 3u, x, y, z, d);
                    k = (k + 1 == L) ? 0 : k + 1;
                    v = map_step(r, v);
                    float dd = __fmaf_rn(-2.0f * r, v, r);
                    l2 += lg2_approx(fabsf(dd));
                }
            }
        }
    }
    if (!f_isfinite(l2)) return __int_as_float(0x7fffffff);
    return (l2 * LN2F) / (float)si.A;
}

template <uint32_t MODE>
__device__ __forceinline__ float eval_lambda(float x, float y, float z, const SeqInfo &si, bool &skipped,
                                             bool &fallback)
{
    switch (si.L) {
#define LYAP_CASE(n) \
    case n: return lambda_fixed<MODE, n>(x, y, z, si, skipped, fallback);
        LYAP_CASE(1) LYAP_CASE(2) LYAP_CASE(3) LYAP_CASE(4) LYAP_CASE(5) LYAP_CASE(6) LYAP_CASE(7) LYAP_CASE(8)
        LYAP_CASE(9) LYAP_CASE(10) LYAP_CASE(11) LYAP_CASE(12) LYAP_CASE(13) LYAP_CASE(14) LYAP_CASE(15)
        LYAP_CASE(16)
#undef LYAP_CASE
    default: return lambda_generic<MODE>(x, y, z, si, skipped, fallback);
    }
}

// ------------------------------------------- lambda, sequence known at compile time
// A period of up to 64 symbols packed 2 bits each into two 64-bit template
// constants.  When the loop below is unrolled, at(j) folds to a constant, so
// picking r for a step is a register choice, not an instruction: the loop
// keeps only x, y, z, d, their -2 multiples and the orbit state live, which
// leaves room for K independent samples per thread (K dependency chains
// interleaved to hide the 8-cycle FMUL->FFMA latency of one chain).
template <int L_, uint64_t W0, uint64_t W1>
struct CSeq {
    static constexpr int L = L_;
    __device__ static constexpr uint32_t at(int j)
    {
        return (uint32_t)(((j < 32) ? (W0 >> (2 * j)) : (W1 >> (2 * (j - 32)))) & 3u);
    }
    __device__ static __forceinline__ uint32_t at_rt(uint32_t j)
    {
        return (uint32_t)(((j < 32u) ? (W0 >> (2u * j)) : (W1 >> (2u * (j - 32u)))) & 3u);
    }
};

template <int L>
struct UnrollC {
    static constexpr int U = (L <= 16) ? Unroll<L>::U : ((L % 8 == 0) ? L : ctz_lcm8(L) <= 256 ? ctz_lcm8(L) : L);
    static constexpr bool aligned8 = (U % 8) == 0;   // renormalisation points fall on j % 8 == 7
};

// ---------------------------------------------------- packed FP32 pairs
// fma.rn.f32x2 / mul.rn.f32x2 round each half exactly as fma.rn.f32 /
// mul.rn.f32 do; one instruction carries two samples' operations, which
// halves the issue slots of the FP32 work (the FP32 pipe rate is unchanged).
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b)
{
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

template <class SS, class SA>
__device__ __forceinline__ void lambda_const_x2(const float (&px)[2], const float (&py)[2], const float (&pz)[2],
                                                float d, uint32_t S, uint32_t A, float (&out)[2],
                                                uint32_t &skipped, uint32_t &fallback);
// the product form's rare redo of a sample in the plain form, kept out of
// line so that its unrolled loops stay out of the kernels' hot code
template <class SS, class SA>
__device__ __noinline__ float lambda_const_plain_redo(float x, float y, float z, float d, uint32_t S, uint32_t A);
// the product form's redo of a sample with the defining blocks of 8, out of line
template <class SS, class SA>
__device__ __noinline__ float lambda_const_block8_redo(float x, float y, float z, float d, uint32_t S, uint32_t A,
                                                       uint32_t &fallback);

// K samples (px[k], py[k], pz[k]) with the settle symbols SS and the
// accumulation symbols SA (SS rotated by settle mod L).  Same arithmetic as
// lambda_fixed, sample by sample.  skipped / fallback: bit k set for sample k.
template <uint32_t MODE, int K, class SS, class SA, uint32_t BF = 0>
__device__ __forceinline__ void lambda_const(const float (&px)[K], const float (&py)[K], const float (&pz)[K],
                                             float d, uint32_t S, uint32_t A, float (&out)[K],
                                             uint32_t &skipped, uint32_t &fallback)
{
    if constexpr (MODE == MODE_PRODUCT && K == 2) {
        lambda_const_x2<SS, SA>(px, py, pz, d, S, A, out, skipped, fallback);
        return;
    }
    constexpr int L = SS::L;
    constexpr int U = UnrollC<L>::U;
    static_assert(UnrollC<L>::aligned8 || MODE == MODE_PLAIN, "product form needs U % 8 == 0");
    const float md = -2.0f * d;
    float mx[K], my[K], mz[K], v[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        mx[k] = -2.0f * px[k];
        my[k] = -2.0f * py[k];
        mz[k] = -2.0f * pz[k];
        v[k] = 0.5f;
    }
    {
        const uint32_t nb = S / U, rem = S - nb * U;
        for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
            for (int j = 0; j < U; j++) {
#pragma unroll
                for (int k = 0; k < K; k++) v[k] = map_step(pick(SS::at(j % L), px[k], py[k], pz[k], d), v[k]);
            }
        }
        uint32_t jj = 0;
        for (uint32_t j = 0; j < rem; j++) {
            const uint32_t sym = SS::at_rt(jj);
            jj = (jj + 1 == (uint32_t)L) ? 0 : jj + 1;
#pragma unroll
            for (int k = 0; k < K; k++) v[k] = map_step(pick(sym, px[k], py[k], pz[k], d), v[k]);
        }
    }
    skipped = 0;
    fallback = 0;
#pragma unroll
    for (int k = 0; k < K; k++)
        if (!(v[k] < 0.5f || v[k] > 0.5f)) skipped |= 1u << k;
    float l2[K];
    uint32_t redo8 = 0;   // samples to take again with blocks of 8
    const uint32_t nb = A / U, rem = A - nb * U;
    if (MODE == MODE_PLAIN) {
#pragma unroll
        for (int k = 0; k < K; k++) l2[k] = 0.0f;
        for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
            for (int j = 0; j < U; j++) {
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const uint32_t sym = SA::at(j % L);
                    const float r = pick(sym, px[k], py[k], pz[k], d);
                    const float m = pick(sym, mx[k], my[k], mz[k], md);
                    v[k] = map_step(r, v[k]);
                    l2[k] += lg2_approx(fabsf(__fmaf_rn(m, v[k], r)));
                }
            }
        }
        uint32_t jj = 0;
        for (uint32_t j = 0; j < rem; j++) {
            const uint32_t sym = SA::at_rt(jj);
            jj = (jj + 1 == (uint32_t)L) ? 0 : jj + 1;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float r = pick(sym, px[k], py[k], pz[k], d);
                const float m = pick(sym, mx[k], my[k], mz[k], md);
                v[k] = map_step(r, v[k]);
                l2[k] += lg2_approx(fabsf(__fmaf_rn(m, v[k], r)));
            }
        }
    } else {
        constexpr uint32_t B = BF ? BF : product_block(L);
        static_assert(U % B == 0, "blocks end inside the unrolled body");
        float p[K], sv[K];
        int32_t e[K];
        uint32_t emx[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            p[k] = product_start(B);
            sv[k] = -v[k];
            e[k] = 0;
            emx[k] = 0;
        }
        for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
            for (int j = 0; j < U; j++) {
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const uint32_t sym = SA::at(j % L);
                    const float r = pick(sym, px[k], py[k], pz[k], d);
                    const float m = pick(sym, mx[k], my[k], mz[k], md);
                    product_step(r, -m, sv[k], p[k]);
                    if (j % B == B - 1) renorm_max(B, p[k], e[k], emx[k]);
                }
            }
        }
        uint32_t jj = 0, kb = 0;
        for (uint32_t j = 0; j < rem; j++) {
            const uint32_t sym = SA::at_rt(jj);
            jj = (jj + 1 == (uint32_t)L) ? 0 : jj + 1;
            const bool end = ++kb == B;
            if (end) kb = 0;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float r = pick(sym, px[k], py[k], pz[k], d);
                const float m = pick(sym, mx[k], my[k], mz[k], md);
                product_step(r, -m, sv[k], p[k]);
                if (end) renorm_max(B, p[k], e[k], emx[k]);
            }
        }
        const int32_t bias = (int32_t)(product_exp(B) * (A / B + 1));
#pragma unroll
        for (int k = 0; k < K; k++) {
            renorm_max(B, p[k], e[k], emx[k]);
            l2[k] = (float)(e[k] - bias) + lg2_approx(product_mantissa(p[k]));
            if (product_bad(B, emx[k]) && !((skipped >> k) & 1u)) {
                if (product_is_nan(B, emx[k], sv[k], px[k], py[k], pz[k], d))
                    l2[k] = __int_as_float(0x7fffffff);
                else if (B != 8u)
                    redo8 |= 1u << k;
                else
                    fallback |= 1u << k;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        float lk = ((skipped >> k) & 1u) ? 0.0f : l2[k];
        out[k] = f_isfinite(lk) ? (lk * LN2F) / (float)A : __int_as_float(0x7fffffff);
    }
    if (MODE == MODE_PRODUCT && fallback) {
        // an intermediate product may have been subnormal: redo those samples in the plain form
#pragma unroll
        for (int k = 0; k < K; k++) {
            if ((fallback >> k) & 1u) {
                out[k] = lambda_const_plain_redo<SS, SA>(px[k], py[k], pz[k], d, S, A);
            }
        }
    }
    if (MODE == MODE_PRODUCT && redo8) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            if ((redo8 >> k) & 1u) {
                uint32_t fb = 0;
                out[k] = lambda_const_block8_redo<SS, SA>(px[k], py[k], pz[k], d, S, A, fb);
            }
        }
        fallback |= redo8;
    }
}

template <class SS, class SA>
__device__ __noinline__ float lambda_const_plain_redo(float x, float y, float z, float d, uint32_t S, uint32_t A)
{
    const float qx[1] = {x}, qy[1] = {y}, qz[1] = {z};
    float o[1];
    uint32_t sk, fb;
    lambda_const<MODE_PLAIN, 1, SS, SA>(qx, qy, qz, d, S, A, o, sk, fb);
    return o[0];
}

template <class SS, class SA>
__device__ __noinline__ float lambda_const_block8_redo(float x, float y, float z, float d, uint32_t S, uint32_t A,
                                                       uint32_t &fallback)
{
    const float qx[1] = {x}, qy[1] = {y}, qz[1] = {z};
    float o[1];
    uint32_t sk;
    lambda_const<MODE_PRODUCT, 1, SS, SA, 8u>(qx, qy, qz, d, S, A, o, sk, fallback);
    return o[0];
}

// The product form for two samples at once on packed FP32 pairs.  The
// state is kept negated, s = -v, so that every operation is a plain packed
// mul / fma with the scalar form's rounding:
//   mt = r*s        = -(r*v)                   (the scalar t, negated)
//   s' = mt*s + mt  = -(t - t*v)               (the scalar fma(-t, v, t), negated)
//   d  = (2r)*s' + r = r - 2r*v'               (the scalar fma(-2r, v', r))
//   p' = p*d                                    (|p'| = the scalar p*|d|)
// Round-to-nearest is symmetric, so each quantity is the scalar one or its
// exact negation; renorm discards the sign of p.
template <class SS, class SA>
__device__ __forceinline__ void lambda_const_x2(const float (&px)[2], const float (&py)[2], const float (&pz)[2],
                                                float d, uint32_t S, uint32_t A, float (&out)[2],
                                                uint32_t &skipped, uint32_t &fallback)
{
    constexpr int L = SS::L;
    constexpr int U = UnrollC<L>::U;
    static_assert(UnrollC<L>::aligned8, "product form needs U % 8 == 0");
    const uint64_t R[4] = {f2_pack(px[0], px[1]), f2_pack(py[0], py[1]), f2_pack(pz[0], pz[1]), f2_pack(d, d)};
    const uint64_t TR[4] = {f2_pack(2.0f * px[0], 2.0f * px[1]), f2_pack(2.0f * py[0], 2.0f * py[1]),
                            f2_pack(2.0f * pz[0], 2.0f * pz[1]), f2_pack(2.0f * d, 2.0f * d)};
    uint64_t s = f2_pack(-0.5f, -0.5f);
    {
        const uint32_t nb = S / U, rem = S - nb * U;
        for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
            for (int j = 0; j < U; j++) {
                const uint64_t mt = f2_mul(R[SS::at(j % L)], s);
                s = f2_fma(mt, s, mt);
            }
        }
        uint32_t jj = 0;
        for (uint32_t j = 0; j < rem; j++) {
            const uint32_t sym = SS::at_rt(jj);
            jj = (jj + 1 == (uint32_t)L) ? 0 : jj + 1;
            const uint64_t r = (sym & 2u) ? ((sym & 1u) ? R[3] : R[2]) : ((sym & 1u) ? R[1] : R[0]);
            const uint64_t mt = f2_mul(r, s);
            s = f2_fma(mt, s, mt);
        }
    }
    skipped = 0;
    fallback = 0;
    {
        float s0, s1;
        f2_unpack(s, s0, s1);
        const float v0 = -s0, v1 = -s1;
        if (!(v0 < 0.5f || v0 > 0.5f)) skipped |= 1u;
        if (!(v1 < 0.5f || v1 > 0.5f)) skipped |= 2u;
    }
    constexpr uint32_t B = product_block(L);
    static_assert(U % B == 0, "blocks end inside the unrolled body");
    uint64_t p = f2_pack(product_start(B), product_start(B));
    int32_t e0 = 0, e1 = 0;
    uint32_t mx0 = 0, mx1 = 0;
    auto renorm2 = [&]() {
        float a, b;
        f2_unpack(p, a, b);
        renorm_max(B, a, e0, mx0);
        renorm_max(B, b, e1, mx1);
        p = f2_pack(a, b);
    };
    const uint32_t nb = A / U, rem = A - nb * U;
    for (uint32_t b = 0; b < nb; b++) {
#pragma unroll
        for (int j = 0; j < U; j++) {
            const uint32_t sym = SA::at(j % L);
            const uint64_t mt = f2_mul(R[sym], s);
            s = f2_fma(mt, s, mt);
            p = f2_mul(p, f2_fma(TR[sym], s, R[sym]));
            if (j % B == B - 1) renorm2();
        }
    }
    uint32_t jj = 0, kb = 0;
    for (uint32_t j = 0; j < rem; j++) {
        const uint32_t sym = SA::at_rt(jj);
        jj = (jj + 1 == (uint32_t)L) ? 0 : jj + 1;
        const uint64_t r = (sym & 2u) ? ((sym & 1u) ? R[3] : R[2]) : ((sym & 1u) ? R[1] : R[0]);
        const uint64_t tr = (sym & 2u) ? ((sym & 1u) ? TR[3] : TR[2]) : ((sym & 1u) ? TR[1] : TR[0]);
        const uint64_t mt = f2_mul(r, s);
        s = f2_fma(mt, s, mt);
        p = f2_mul(p, f2_fma(tr, s, r));
        if (++kb == B) {
            kb = 0;
            renorm2();
        }
    }
    renorm2();
    float p0, p1;
    f2_unpack(p, p0, p1);
    const int32_t bias = (int32_t)(product_exp(B) * (A / B + 1));
    float l2[2] = {(float)(e0 - bias) + lg2_approx(product_mantissa(p0)),
                   (float)(e1 - bias) + lg2_approx(product_mantissa(p1))};
    float s_end0, s_end1;
    f2_unpack(s, s_end0, s_end1);
    uint32_t redo8 = 0;   // samples to take again with blocks of 8
    if (product_bad(B, mx0) && !(skipped & 1u)) {
        if (product_is_nan(B, mx0, s_end0, px[0], py[0], pz[0], d))
            l2[0] = __int_as_float(0x7fffffff);
        else if (B != 8u)
            redo8 |= 1u;
        else
            fallback |= 1u;
    }
    if (product_bad(B, mx1) && !(skipped & 2u)) {
        if (product_is_nan(B, mx1, s_end1, px[1], py[1], pz[1], d))
            l2[1] = __int_as_float(0x7fffffff);
        else if (B != 8u)
            redo8 |= 2u;
        else
            fallback |= 2u;
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float lk = ((skipped >> k) & 1u) ? 0.0f : l2[k];
        out[k] = f_isfinite(lk) ? (lk * LN2F) / (float)A : __int_as_float(0x7fffffff);
    }
    if (fallback) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if ((fallback >> k) & 1u) {
                out[k] = lambda_const_plain_redo<SS, SA>(px[k], py[k], pz[k], d, S, A);
            }
        }
    }
    if (redo8) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if ((redo8 >> k) & 1u) {
                uint32_t fb = 0;
                out[k] = lambda_const_block8_redo<SS, SA>(px[k], py[k], pz[k], d, S, A, fb);
            }
        }
        fallback |= redo8;
    }
}

// ------------------------------------------------------- lambda in double
// The FP64 evaluator used by the precision form's bisection and by
// lyap_lambda_points: the reference's DOUBLE_REALS arithmetic for the orbit
// (v = r*v*(1-v) and d = r - 2r*v, each product and difference rounded once
// in double, kernel.cu:135,143-144 with Real = double), so the orbit is
// bit-identical to the FP64 oracle's; the logarithms are accumulated as a
// running double product renormalised by exponent extraction every 16 steps
// with one log2 per sample (a block ending outside [2^-900, 2^900], or a
// zero factor, redoes the sample with one log per step).  Agrees with the
// per-step-log oracle to ~1e-13 relative.
__device__ __forceinline__ double pick_d(uint32_t sym, double x, double y, double z, double d)
{
    double lo = (sym & 1u) ? y : x;
    double hi = (sym & 1u) ? d : z;
    return (sym & 2u) ? hi : lo;
}

static __device__ __noinline__ double lambda_f64_core(double x, double y, double z, double d, const int32_t *seq,
                                                      uint32_t L, uint32_t S, uint32_t A)
{
    struct {
        uint32_t S, A;
    } si = {S, A};
    double v = 0.5;
    uint32_t k = 0;
    for (uint32_t n = 0; n < si.S; n++) {
        const double r = pick_d((uint32_t)seq[k] & 3u, x, y, z, d);
        k = (k + 1 == L) ? 0 : k + 1;
        v = r * v * (1.0 - v);
    }
    if (!((v - 0.5 <= -1e-8) || (v - 0.5 >= 1e-8))) return 0.0 / (double)si.A;
    const uint32_t kA = k;
    const double vA = v;
    double p = 1.0;
    int64_t e = 0;
    bool bad = false;
    for (uint32_t n = 0; n < si.A; n++) {
        const double r = pick_d((uint32_t)seq[k] & 3u, x, y, z, d);
        k = (k + 1 == L) ? 0 : k + 1;
        v = r * v * (1.0 - v);
        double dd = r - 2.0 * r * v;
        p = p * fabs(dd);
        if ((n & 15u) == 15u || n + 1 == si.A) {
            const uint64_t bits = (uint64_t)__double_as_longlong(p);
            const int64_t ef = (int64_t)((bits >> 52) & 0x7ffu);
            if (ef < 123 || ef > 1923) bad = true;   // outside [2^-900, 2^900], zero, inf or NaN
            e += ef - 1023;
            p = __longlong_as_double((long long)((bits & 0x000fffffffffffffull) | 0x3ff0000000000000ull));
        }
    }
    double l;
    if (bad) {
        // one log per step, as the oracle does, from the start of accumulation
        v = vA;
        k = kA;
        l = 0.0;
        for (uint32_t n = 0; n < si.A; n++) {
            const double r = pick_d((uint32_t)seq[k] & 3u, x, y, z, d);
            k = (k + 1 == L) ? 0 : k + 1;
            v = r * v * (1.0 - v);
            double dd = r - 2.0 * r * v;
            if (dd < 0) dd = -dd;
            l += log(dd);
            if ((((uint64_t)__double_as_longlong(l) >> 52) & 0x7ffu) == 0x7ffu)
                return __longlong_as_double(0x7ff8000000000000ll);
        }
    } else {
        l = ((double)e + log2(p)) * 0.693147180559945309417232121458176568;
    }
    return l / (double)si.A;
}

// lambda in double at a float parameter d (the float-params callers)
static __device__ __forceinline__ double lambda_f64(double x, double y, double z, const SeqInfo &si)
{
    return lambda_f64_core(x, y, z, (double)si.d, si.seq, si.L, si.S, si.A);
}

// --------------------------------------------------------------- the ray
enum : uint32_t { PH_MARCH0 = 0, PH_MARCH = 1, PH_HONE = 2, PH_NORM0 = 3 };

struct Ray {
    V3 P, V, QdV, N;
    float t, t1, dt, Fdt, Ndt, a, c, l;
    float Qdt, Qt0, Qt1, minQdt, mag, lprev;
    float tprev;   // t of the previous march sample (the bracket's far end)
    uint32_t phase, nm, nh, cap;
    uint32_t ns;     // march samples the learned proposal skipped (counted in nm, never evaluated)
    bool near, sign;
    // learned proposal only (ray_advance<true>): pst packs the run of
    // skipped positions the pending march sample confirms (bits 0-5: the
    // sample is that many steps past P, where the ray waits until the run is
    // confirmed), a rewind counter (bits 6-13: samples taken ahead for this
    // ray are stale once it changes) and the samples rewinds discarded (bits
    // 14-31); positions are evaluated exactly while nm < pnoskip
    uint32_t pst, pnoskip;
};

struct CamRays {   // the per-frame camera quantities raymarch reads
    V3 C, S0, SDX, SDY;
    float M;
};

__device__ __forceinline__ CamRays cam_rays(const LyapCam &cam)
{
    return CamRays{v3(cam.C), v3(cam.S0), v3(cam.SDX), v3(cam.SDY), cam.M};
}

// Ray setup and box clipping (kernel.cu:160-315): the direction, where the
// ray enters and leaves the box [lMin, lMax]^3, its step and its sample cap.
// Returns false when the ray misses the box (raymarch returns 1 before any
// sample).
__device__ __forceinline__ bool ray_geometry(const CamRays &cam, const LyapParams &prm, uint32_t sx, uint32_t sy,
                                             RayEntry &e)
{
    V3 V = (cam.S0 + cam.SDX * (float)sx) + cam.SDY * (float)sy;
    V = normalized(V);
    V = V / cam.M;
    const double LMIN = (double)prm.lMin, LMAX = (double)prm.lMax;
    const float INF = __int_as_float(0x7f800000), QNAN = __int_as_float(0x7fffffff);
    float ts[6];
    ts[0] = (V.x != 0.0f) ? (float)((LMIN - (double)cam.C.x) / (double)V.x) : INF;
    ts[1] = (V.x != 0.0f) ? (float)((LMAX - (double)cam.C.x) / (double)V.x) : INF;
    ts[2] = (V.y != 0.0f) ? (float)((LMIN - (double)cam.C.y) / (double)V.y) : INF;
    ts[3] = (V.y != 0.0f) ? (float)((LMAX - (double)cam.C.y) / (double)V.y) : INF;
    ts[4] = (V.z != 0.0f) ? (float)((LMIN - (double)cam.C.z) / (double)V.z) : INF;
    ts[5] = (V.z != 0.0f) ? (float)((LMAX - (double)cam.C.z) / (double)V.z) : INF;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        if (ts[k] != INF) {
            V3 P = cam.C + V * ts[k];
            float u = (k < 2) ? P.y : P.x;
            float w = (k < 4) ? P.z : P.y;
            if ((double)u < LMIN || (double)u > LMAX || (double)w < LMIN || (double)w > LMAX) ts[k] = QNAN;
        }
    }
    int i0 = -1, i1 = -1;
    float t0 = 3.40282347e+38f, t1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        if (f_isfinite(ts[k])) {
            if (i0 == -1 || ts[k] < t0) { t0 = ts[k]; i0 = k; }
            if (i1 == -1 || ts[k] > t1) { t1 = ts[k]; i1 = k; }
        }
    }
    if (i0 == -1 && i1 == -1) return false;
    if (i1 == -1 || i0 == i1) {
        t1 = t0;
        t0 = 0.0f;
    }
    if (t0 < 0.0f) t0 = 0.0f;

    float Fdt;
    if (prm.stepMethod == 1)
        Fdt = (t1 - t0) / prm.depth;
    else
        Fdt = sqrtf(V.x * V.x + V.y * V.y + V.z * V.z) / prm.depth;
    const float Ndt = Fdt / prm.nearMultiplier;
    float dmin = Fdt < Ndt ? Fdt : Ndt;
    double capd = ceil((double)(t1 - t0) / (double)dmin * 1.001) + 16.0;
    e.t0 = t0;
    e.t1 = t1;
    e.cap = (capd > 0.0 && capd < (double)MARCH_MAX) ? (uint32_t)capd : MARCH_MAX;
    e.vx = V.x;
    e.vy = V.y;
    e.vz = V.z;
    e.Fdt = Fdt;
    return true;
}

// The ray's march state at its first sample, from its setup.
__device__ __forceinline__ void ray_start(Ray &r, V3 C, const RayEntry &e, const LyapParams &prm)
{
    const V3 V = v3(e.vx, e.vy, e.vz);
    r.pst = r.pnoskip = 0;
    r.V = V;
    r.t = e.t0;
    r.t1 = e.t1;
    r.P = C + V * e.t0;
    r.a = 0.0f;
    r.c = 0.0f;
    r.Fdt = e.Fdt;
    r.dt = e.Fdt;
    r.Ndt = e.Fdt / prm.nearMultiplier;
    r.near = false;
    r.cap = e.cap;
    r.nm = 0;
    r.nh = 0;
    r.ns = 0;
    r.phase = PH_MARCH0;
    r.l = 0.0f;
    r.tprev = e.t0;
}

// Ray setup and start in one (kernel.cu:160-315).  Returns false when the
// ray misses the box.
__device__ __forceinline__ bool ray_init(Ray &r, const CamRays &cam, const LyapParams &prm, uint32_t sx, uint32_t sy)
{
    r.pst = r.pnoskip = 0;
    RayEntry e;
    if (!ray_geometry(cam, prm, sx, sy, e)) return false;
    ray_start(r, cam.C, e, prm);
    return true;
}

// ---------------------------------------------------- the learned proposal
__device__ __forceinline__ uint32_t prop_run(const Ray &r) { return r.pst & 63u; }
__device__ __forceinline__ uint32_t prop_gen(const Ray &r) { return (r.pst >> 6) & 255u; }
__device__ __forceinline__ uint32_t prop_rewound(const Ray &r) { return r.pst >> 14; }

// The proposal's bits in shared memory (the render's dynamic shared memory,
// filled at its start when PropGrid.smem_words > 0).
extern __shared__ uint32_t lyap_prop_smem[];

// Is the march position P in a cell whose bit is set (the net's lower bound
// at least the skip threshold)?  Positions outside the grid never are.  pg
// is the kernel parameter's copy (__grid_constant__): its fields are read
// from the constant bank and hold no registers across the lambda loop.
__device__ __forceinline__ bool prop_skippable(const PropGrid &pg, V3 P)
{
    const float nf = (float)pg.n;
    const float fx = (P.x - pg.lo[0]) * pg.scale[0];
    const float fy = (P.y - pg.lo[1]) * pg.scale[1];
    const float fz = (P.z - pg.lo[2]) * pg.scale[2];
    if (!(fx >= 0.0f && fx < nf && fy >= 0.0f && fy < nf && fz >= 0.0f && fz < nf)) return false;
    const uint32_t c = ((uint32_t)fz * pg.n + (uint32_t)fy) * pg.n + (uint32_t)fx;   // each index < n
    const uint32_t w = pg.smem_words ? lyap_prop_smem[c >> 5] : __ldg(pg.bits + (c >> 5));
    return (w >> (c & 31u)) & 1u;
}

// k march steps from P, as ray_advance takes them (fixed step length)
__device__ __forceinline__ V3 prop_steps(V3 P, V3 V, float dt, uint32_t k)
{
    for (uint32_t j = 0; j < k; j++) P = P + V * dt;
    return P;
}

// After a march step (the ray at its next position P, index nm + 1): the
// run of skippable positions that starts there -- at most pg.run, never the
// last position before t1 or the sample cap.  The ray stays at P; its
// pending sample is the position after the run, which confirms it
// (ray_advance<true>), and ray_sample_point<true> finds it by taking the
// run's steps exactly as the march would, so every later position is
// bit-identical to the exact march's.
__device__ __forceinline__ void prop_form_run(Ray &r, const PropGrid &pg)
{
    if (r.nm < r.pnoskip) return;
    uint32_t k = 0;
    V3 Q = r.P;
    float tq = r.t;
    while (k < pg.run && r.nm + k + 1 < r.cap && prop_skippable(pg, Q)) {
        const float tn = tq + r.dt;
        if (tn > r.t1) break;   // Q is the last position in the box: it confirms
        tq = tn;
        Q = Q + r.V * r.dt;
        k++;
    }
    r.pst = (r.pst & ~63u) | k;
}

// The march position `offset` evaluated samples after the pending one (run
// `run` steps past P, index nm + run + 1), assuming every sample until then
// is above the threshold and confirms its run: the positions
// ray_advance<true> and prop_form_run visit.  valid = false once the ray
// would have left the box or reached the cap.
__device__ __forceinline__ V3 prop_march_ahead(V3 P, V3 V, float dt, float t, float t1, uint32_t nm, uint32_t cap,
                                               uint32_t noskip, uint32_t run, const PropGrid &pg, uint32_t offset,
                                               bool &valid)
{
    valid = true;
    for (uint32_t j = 0; j < run; j++) {
        t = t + dt;
        P = P + V * dt;
    }
    nm += run;
    for (uint32_t j = 0; j < offset; j++) {
        nm += 1;
        if (nm >= cap) {
            valid = false;
            return P;
        }
        t = t + dt;
        P = P + V * dt;
        if (t > t1) {
            valid = false;
            return P;
        }
        if (nm >= noskip) {
            uint32_t k = 0;
            while (k < pg.run && nm + k + 1 < cap && prop_skippable(pg, P)) {
                const float tn = t + dt;
                if (tn > t1) break;
                t = tn;
                P = P + V * dt;
                k++;
            }
            nm += k;
        }
    }
    return P;
}

// Where the next lambda sample of this ray is taken.  PROP: a pending
// sample that confirms a run of the learned proposal lies the run's steps
// past P.
template <bool PROP = false>
__device__ __forceinline__ V3 ray_sample_point(const Ray &r)
{
    V3 Q = r.P;
    if constexpr (PROP) {
        if (r.phase <= PH_MARCH) return prop_steps(Q, r.V, r.dt, prop_run(r));
    }
    if (r.phase >= PH_NORM0) {
        const uint32_t k = r.phase - PH_NORM0;   // kernel.cu:457-463
        const float m = r.mag;
        if (k == 0) Q.x = Q.x - m;
        else if (k == 1) Q.x = Q.x + m;
        else if (k == 2) Q.y = Q.y - m;
        else if (k == 3) Q.y = Q.y + m;
        else if (k == 4) Q.z = Q.z - m;
        else Q.z = Q.z + m;
    }
    return Q;
}

// RAY_BRACKET: the march crossed the surface and the caller asked for the
// crossing bracket [tprev, t] instead of honing (the precision form bisects it
// in FP64 afterwards).
enum : int { RAY_CONTINUE = 0, RAY_HIT = 1, RAY_MISS = 2, RAY_BRACKET = 3 };

// The normal's normalisation at a ray's end (vec3.hpp:127-154), out of line:
// it runs once per hit, and kept out of ray_advance's inlined copies it
// leaves the instruction cache to the code every sample round runs.
static __device__ __noinline__ V3 normalized_cold(V3 a) { return normalized(a); }

// Feed one lambda sample to the ray (kernel.cu:318-473); the ray either asks
// for its next sample (RAY_CONTINUE) or ends.  PROP: the learned proposal's
// skipping (prop_form_run) after every march step, and the confirmation of
// every skipped run by the sample after it: a confirming lambda at or below
// pg.tau (the threshold the skip was made for) sends the ray back to the
// run's first position, from where every position up to the confirming one
// is evaluated exactly -- so a surface is lost only if it enters and leaves
// the ray inside one run of positions the net called empty.
template <bool PROP = false>
__device__ __forceinline__ int ray_advance(Ray &r, float lam, const LyapParams &prm, bool bracket = false,
                                           const PropGrid *pg = nullptr)
{
    const float opaque = prm.opaqueThreshold;
    bool to_normal = false;
    if (r.phase >= PH_NORM0) {
        const uint32_t k = r.phase - PH_NORM0;
        if ((k & 1u) == 0) {
            r.lprev = lam;
        } else {
            const float diff = lam - r.lprev;   // ls[2i+1] - ls[2i]
            if (k == 1) r.N.x = diff;
            else if (k == 3) r.N.y = diff;
            else r.N.z = diff;
        }
        if (k == 5) {
            r.N = normalized_cold(r.N);
            return RAY_HIT;
        }
        r.phase += 1;
        return RAY_CONTINUE;
    }
    if (r.phase == PH_HONE) {
        r.nh += 1;
        r.l = lam;
        if (lam == opaque) {
            to_normal = true;
        } else {
            const bool osign = r.sign;
            r.sign = !(lam < opaque);
            if (r.sign != osign) {
                r.Qdt = r.Qdt * -0.5f;
                r.QdV = r.QdV * -0.5f;
            }
        }
    } else {
        if constexpr (PROP) {
            const uint32_t k = prop_run(r);
            if (k) {
                if (!(lam > pg->tau)) {
                    // not clearly empty (NaN included): the ray, still at the
                    // run's first position, evaluates every position through
                    // this one exactly
                    r.pnoskip = r.nm + k + 1;
                    // run 0, rewind counter + 1 (mod 256), discarded samples + 1
                    r.pst = (((r.pst >> 14) + 1u) << 14) | (((prop_gen(r) + 1u) & 255u) << 6);
                    return RAY_CONTINUE;
                }
                // confirmed: the run's steps, as the exact march takes them;
                // the sample is the march sample at the position after them
                for (uint32_t j = 0; j < k; j++) {
                    r.tprev = r.t;
                    r.t = r.t + r.dt;
                    r.P = r.P + r.V * r.dt;
                }
                r.nm += k;
                r.ns += k;
                r.pst &= ~63u;
            }
        }
        r.nm += 1;
        r.l = lam;
        if (r.phase == PH_MARCH) {
            if (lam > prm.chaosThreshold) r.c = r.c + lam;
            else if (lam > opaque) r.a = r.a + lam;
            if (lam <= prm.nearThreshold && !r.near) {
                r.near = true;
                r.dt = r.Ndt;
            } else if (lam > prm.nearThreshold && r.near) {
                r.near = false;
                r.dt = r.Fdt;
            }
        }
        if (r.l > opaque) {
            // march on (kernel.cu:326-363)
            if (r.nm >= r.cap) return RAY_MISS;
            float step = r.dt;
            if (prm.jitter != 0.0f) {   // the reference compares in double; same outcome for a float
                float jit = r.l - truncf(r.l);
                if (jit < 0.0f)
                    jit = (float)(1.0 - (double)(jit * prm.jitter));
                else
                    jit = (float)(1.0 + (double)(jit * prm.jitter));
                if (f_isfinite(jit)) step = r.dt * jit;
            }
            r.tprev = r.t;
            r.t = r.t + step;
            r.P = r.P + r.V * step;
            if (r.t > r.t1) return RAY_MISS;
            r.phase = PH_MARCH;
            if constexpr (PROP) prop_form_run(r, *pg);
            return RAY_CONTINUE;
        }
        if (r.t > r.t1) return RAY_MISS;
        if (bracket) return RAY_BRACKET;
        // start honing (kernel.cu:402-416)
        r.sign = false;
        r.Qdt = r.dt * -0.5f;
        r.QdV = r.V * r.Qdt;
        r.Qt1 = r.t;
        r.Qt0 = r.t - r.dt;
        r.minQdt = r.dt / prm.refine;
    }
    if (!to_normal) {
        // honing condition (kernel.cu:420)
        if (r.t <= r.Qt1 && r.t >= r.Qt0 && (r.Qdt <= -r.minQdt || r.Qdt >= r.minQdt) && r.nh < HONE_CAP) {
            const float tn = r.t + r.Qdt;
            const V3 Pn = r.P + r.QdV;
            if (r.phase == PH_HONE && tn == r.t && Pn.x == r.P.x && Pn.y == r.P.y && Pn.z == r.P.z) {
                // a step below half an ulp of t and of P (a ray grazing the box,
                // whose step is tiny): every remaining hone step samples this
                // same point again -- the same lambda, the same sign, no change
                // but the count -- until the cap, so the cap is taken at once
                r.nh = HONE_CAP;
            } else {
                r.t = tn;
                r.P = Pn;
                r.phase = PH_HONE;
                return RAY_CONTINUE;
            }
        }
    }
    // normal from six central differences (kernel.cu:456)
    r.mag = r.dt * prm.gradient;
    r.phase = PH_NORM0;
    return RAY_CONTINUE;
}

// --------------------------------------------------------------- shading
__device__ __forceinline__ unsigned char to_byte(float ch)
{
    const double v = 255.0 * (double)ch;   // color.hpp:171-174, saturated (H6)
    if (!(v > 0.0)) return 0;
    if (v >= 255.0) return 255;
    return (unsigned char)v;
}

// shade (kernel.cu:25-106) for one point with the reference's spot lights.
__device__ __forceinline__ C4 shade_spot(const LyapPoint &pt, V3 camC, const LyapLight *lights, uint32_t n)
{
    C4 color{0.f, 0.f, 0.f, 0.f};
    if (f_isnan(pt.a)) return color;
    const V3 P = v3(pt.P), N = v3(pt.N);
    const float c = pt.c;
    for (uint32_t li = 0; li < n; li++) {
        const LyapLight &L = lights[li];
        C4 phong;
        V3 camV = camC - P;
        V3 lightV = v3(L.C) - P;
        float lightD2 = lightV.x * lightV.x + lightV.y * lightV.y + lightV.z * lightV.z;
        lightV = normalized(lightV);
        float i = dot(lightV, N);
        float j = dot(lightV, v3(L.V));
        j = -j;
        if (j > L.lightOuterCone) {
            i = clamp01(i);
            C4 diffuse = c4(L.diffuseColor) * (i * L.diffusePower);
            V3 halfV = normalized(camV + lightV);
            i = clamp01(dot(N, halfV));
            i = powf(i, L.specularHardness);
            C4 specular = c4(L.specularColor) * (i * L.specularPower);
            phong = (specular + diffuse) * (L.lightRange / lightD2);
            if (j < L.lightInnerCone) phong = phong * ((j - L.lightOuterCone) / (L.lightInnerCone - L.lightOuterCone));
            phong = phong + c4(L.ambient);
        } else {
            phong = c4(L.ambient);
        }
        if ((double)c > 0.0) phong = phong + c4(L.chaosColor) * (float)(0.1125 / (double)logf(c));
        color = color + phong;
    }
    return color;
}

// Directional Lambert light (an extension: the reference has spot lights
// only): ambient + diffuseColor * diffusePower * clamp(N . -V_light), plus
// the reference's chaos tint.
__device__ __forceinline__ C4 shade_directional(const LyapPoint &pt, const LyapLight *lights, uint32_t n)
{
    C4 color{0.f, 0.f, 0.f, 0.f};
    if (f_isnan(pt.a)) return color;
    const V3 N = v3(pt.N);
    for (uint32_t li = 0; li < n; li++) {
        const LyapLight &L = lights[li];
        const V3 toLight = v3(0.f, 0.f, 0.f) - v3(L.V);
        const float i = clamp01(dot(N, toLight));
        C4 phong = c4(L.diffuseColor) * (i * L.diffusePower) + c4(L.ambient);
        if ((double)pt.c > 0.0) phong = phong + c4(L.chaosColor) * (float)(0.1125 / (double)logf(pt.c));
        color = color + phong;
    }
    return color;
}

}  // namespace lyapgb
