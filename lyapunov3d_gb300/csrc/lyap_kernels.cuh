// lyap_kernels.cuh -- the raymarch and volume kernels as templates over the
// lambda evaluator.  Compiled twice: into the library by nvcc with
// RuntimeLambda (any sequence, read from device memory), and at run time by
// NVRTC with ConstLambda (the caller's sequence baked in as template
// constants, lyap_jit.cpp).
//
// render_persistent (kernel_calc_render, kernel.cu:500).  Every lambda
// sample of a ray costs the same (settle + accum map iterations), but rays
// need 0 to ~depth*nearMultiplier samples.  A thread-per-pixel kernel (the
// reference's) keeps a warp busy until its longest ray ends.  Here each
// lane of a persistent warp owns one ray at a time; after every sample the
// lanes whose ray ended write their pixel and take the next pixel from a
// global queue, so all 32 lanes evaluate a sample in every round until the
// queue is empty.  The lambda loop is uniform across the warp.
//
// volume_sweep (kernel_calc_volume, kernel.cu:518).  Every voxel costs the
// same; each warp takes 32*K consecutive voxels, K per lane, evaluated as K
// interleaved dependency chains, and stores them with coalesced streaming
// 128-byte stores (st.global.cs: written once, never read back here).
#pragma once

#include "lyap_device.cuh"
#include "lyap_jobs.h"

#ifndef LYAP_RENDER_THREADS
#define LYAP_RENDER_THREADS 128
#endif
// per lambda form: threads per block of the persistent render (its
// end-of-frame hand-over works within a block)
#ifndef LYAP_RENDER_THREADS_PRODUCT
#define LYAP_RENDER_THREADS_PRODUCT LYAP_RENDER_THREADS
#endif
#ifndef LYAP_RENDER_THREADS_PLAIN
#define LYAP_RENDER_THREADS_PLAIN LYAP_RENDER_THREADS
#endif
// the batch kernel's blocks (its warps switch requests, they hand nothing over)
#ifndef LYAP_BATCH_THREADS
#define LYAP_BATCH_THREADS 128
#endif
#ifndef LYAP_RENDER_MIN_BLOCKS
#define LYAP_RENDER_MIN_BLOCKS 4
#endif
// per lambda form: paired rounds (two samples per lane, sample_round_pair)
// and the resident blocks per SM the render is compiled for
#ifndef LYAP_RENDER_PAIRS_PRODUCT
#define LYAP_RENDER_PAIRS_PRODUCT 0
#endif
#ifndef LYAP_RENDER_PAIRS_PLAIN
#define LYAP_RENDER_PAIRS_PLAIN 0
#endif
#ifndef LYAP_RENDER_MIN_BLOCKS_PRODUCT
#define LYAP_RENDER_MIN_BLOCKS_PRODUCT LYAP_RENDER_MIN_BLOCKS
#endif
#ifndef LYAP_RENDER_MIN_BLOCKS_PLAIN
#define LYAP_RENDER_MIN_BLOCKS_PLAIN LYAP_RENDER_MIN_BLOCKS
#endif
#ifndef LYAP_VOLUME_THREADS
#define LYAP_VOLUME_THREADS 256
#endif
#ifndef LYAP_VOLUME_MIN_BLOCKS
#define LYAP_VOLUME_MIN_BLOCKS 2
#endif

namespace lyapgb {

constexpr uint32_t FULL = 0xffffffffu;

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------------ lambda evaluators
// Any sequence: period and symbols read from device memory per warp.
template <uint32_t MODE>
struct RuntimeLambda {
    static constexpr uint32_t mode = MODE;
    SeqInfo si;
    __device__ __forceinline__ RuntimeLambda(const int32_t *seq, uint32_t period, const LyapParams &prm)
        : si(seq_setup(seq, period, prm)) {}
    __device__ __forceinline__ float operator()(float x, float y, float z, bool &skipped, bool &fallback) const
    {
        return eval_lambda<MODE>(x, y, z, si, skipped, fallback);
    }
    template <int K>
    __device__ __forceinline__ void eval(const float (&x)[K], const float (&y)[K], const float (&z)[K],
                                         float (&out)[K], uint32_t &skipped, uint32_t &fallback) const
    {
        skipped = fallback = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            bool sk, fb;
            out[k] = eval_lambda<MODE>(x[k], y[k], z[k], si, sk, fb);
            skipped |= (sk ? 1u : 0u) << k;
            fallback |= (fb ? 1u : 0u) << k;
        }
    }
};

// The sequence fixed at compile time: SS = symbols of period positions
// 0..L-1, SA = the same rotated to where accumulation starts (OA = settle
// mod L).  The constructor checks the device sequence and the settle count
// against the constants; on any mismatch it evaluates with the runtime path
// instead, so a stale specialisation can cost speed but never correctness.
template <uint32_t MODE, uint32_t OA, class SS, class SA>
struct ConstLambda {
    static constexpr uint32_t mode = MODE;
    SeqInfo si;
    bool match;
    __device__ __forceinline__ ConstLambda(const int32_t *seq, uint32_t period, const LyapParams &prm)
    {
        si.seq = seq;
        si.L = period;
        si.S = prm.settle;
        si.A = prm.accum;
        si.d = prm.d;
        si.oA = prm.settle % (period ? period : 1u);
        si.wS = si.wA = 0;
        bool ok = (period == (uint32_t)SS::L) && (prm.settle % (uint32_t)SS::L == OA);
        if (ok) {
            for (uint32_t j = 0; j < period; j++) ok = ok && ((uint32_t)seq[j] == SS::at_rt(j));
        }
        match = ok;
    }
    __device__ __forceinline__ float operator()(float x, float y, float z, bool &skipped, bool &fallback) const
    {
        if (match) {
            const float px[1] = {x}, py[1] = {y}, pz[1] = {z};
            float o[1];
            uint32_t sk, fb;
            lambda_const<MODE, 1, SS, SA>(px, py, pz, si.d, si.S, si.A, o, sk, fb);
            skipped = sk != 0;
            fallback = fb != 0;
            return o[0];
        }
        return lambda_generic<MODE>(x, y, z, si, skipped, fallback);
    }
    template <int K>
    __device__ __forceinline__ void eval(const float (&x)[K], const float (&y)[K], const float (&z)[K],
                                         float (&out)[K], uint32_t &skipped, uint32_t &fallback) const
    {
        if (match) {
            lambda_const<MODE, K, SS, SA>(x, y, z, si.d, si.S, si.A, out, skipped, fallback);
            return;
        }
        skipped = fallback = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            bool sk, fb;
            out[k] = lambda_generic<MODE>(x[k], y[k], z[k], si, sk, fb);
            skipped |= (sk ? 1u : 0u) << k;
            fallback |= (fb ? 1u : 0u) << k;
        }
    }
};

// -------------------------------------------------------------- outputs
struct LaneStats {
    uint32_t samples, skipped, march, hone, normal, hits, rays, fallback, spec, spec_used;
    uint32_t rounds, lane_rounds;   // per warp, kept by every lane alike
    uint32_t prop_skip;             // march samples skipped on the learned proposal's word
    uint32_t prop_rej;              // samples a rewind of the proposal discarded
    uint32_t handed;                // rays handed to another warp at the end of a frame
};

// position of the n-th (0-based) set bit of mask; mask has more than n bits
// set.  A binary search on population counts: five fixed steps, where
// clearing the lowest bit n times took up to 31 dependent steps.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t mask, uint32_t n)
{
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t w = 16; w; w >>= 1) {
        const uint32_t c = (uint32_t)__popc(mask & ((1u << w) - 1u));
        if (n >= c) {
            n -= c;
            mask >>= w;
            pos += w;
        }
    }
    return pos;
}

// Helper results of one sample round, per warp: the helper of rank k among
// the lanes without a ray posts its lambda values and skip / fallback bits
// in slot k; the owner of the ray reads its helpers' slots in order.  The
// persistent render runs 1-D blocks of LYAP_RENDER_THREADS_PRODUCT /
// _PLAIN threads, the batch kernel of LYAP_BATCH_THREADS (their launch
// bounds); the reference-shaped kernel_calc_render runs 2-D blocks of up to
// 256 threads (its round: BLOCK2D).
constexpr uint32_t ROUND_THREADS_MAX =
    LYAP_RENDER_THREADS_PRODUCT > LYAP_RENDER_THREADS_PLAIN ? LYAP_RENDER_THREADS_PRODUCT : LYAP_RENDER_THREADS_PLAIN;
constexpr uint32_t ROUND_WARPS = (ROUND_THREADS_MAX > LYAP_BATCH_THREADS ? ROUND_THREADS_MAX : LYAP_BATCH_THREADS) / 32;
constexpr uint32_t ROUND_WARPS_2D = 256 / 32;

// The thread's lane and warp in its block: 1-D blocks by threadIdx.x, any
// block (BLOCK2D) by its linear index, of which warps are runs of 32.
template <bool BLOCK2D>
__device__ __forceinline__ void lane_warp(uint32_t &lane, uint32_t &warp)
{
    const uint32_t tid =
        BLOCK2D ? threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z) : threadIdx.x;
    lane = tid & 31u;
    warp = tid >> 5;
}

__device__ __forceinline__ void store_point(LyapPoint *dst, const Ray &r, bool hit)
{
    float *f = reinterpret_cast<float *>(dst);
    if (hit) {
        f[0] = r.P.x; f[1] = r.P.y; f[2] = r.P.z;
        f[3] = r.N.x; f[4] = r.N.y; f[5] = r.N.z;
        f[6] = r.a; f[7] = r.c; f[8] = r.l;
    } else {
        // a miss: all-NaN bytes (the reference leaves the point unwritten)
        const float nanf_ = __int_as_float(-1);
#pragma unroll
        for (int k = 0; k < 9; k++) f[k] = nanf_;
    }
}

// The colour of a hit (shade, kernel.cu:25-106) as RGBA8.  Out of line and
// by value: it runs once per ray, and kept out of the sample rounds' code it
// leaves the instruction cache to the code that runs every round.
static __device__ __noinline__ uint32_t shade_pixel(V3 P, V3 N, float a, float c, float l, V3 camC,
                                                    const LyapLight *lights, uint32_t n_lights, uint32_t light_model)
{
    LyapPoint pt;
    pt.P = LyapVec{P.x, P.y, P.z};
    pt.N = LyapVec{N.x, N.y, N.z};
    pt.a = a;
    pt.c = c;
    pt.l = l;
    C4 col = (light_model == LYAP_LIGHT_DIRECTIONAL) ? shade_directional(pt, lights, n_lights)
                                                     : shade_spot(pt, camC, lights, n_lights);
    return (uint32_t)to_byte(col.x) | ((uint32_t)to_byte(col.y) << 8) | ((uint32_t)to_byte(col.z) << 16) |
           ((uint32_t)to_byte(col.w) << 24);
}

// Write one finished pixel: point, colour, optional per-pixel sample counts.
__device__ __forceinline__ void finish_pixel(RGBA *rgba, LyapPoint *points, uint32_t *counts, uint32_t ind,
                                             const Ray &r, bool hit, V3 camC, const LyapLight *lights,
                                             uint32_t n_lights, uint32_t light_model, LaneStats &st)
{
    store_point(points + ind, r, hit);
    const uint32_t px = hit ? shade_pixel(r.P, r.N, r.a, r.c, r.l, camC, lights, n_lights, light_model) : 0u;
    reinterpret_cast<uint32_t *>(rgba)[ind] = px;
    if (counts) {
        counts[3 * (size_t)ind + 0] = r.nm - r.ns;
        counts[3 * (size_t)ind + 1] = r.nh;
        counts[3 * (size_t)ind + 2] = hit ? 6u : 0u;
    }
    st.march += r.nm - r.ns;
    st.prop_skip += r.ns;
    st.prop_rej += prop_rewound(r);
    st.hone += r.nh;
    st.normal += hit ? 6u : 0u;
    st.hits += hit ? 1u : 0u;
    st.rays += 1;
}

__device__ __forceinline__ void flush_stats(unsigned long long *stats, const LaneStats &st, uint32_t mask)
{
    if (!stats) return;
    const uint32_t v[10] = {st.samples, st.skipped, st.march, st.hone, st.normal,
                            st.hits, st.rays, st.fallback, st.spec, st.spec_used};
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1;
#pragma unroll
    for (int k = 0; k < 10; k++) {
        const uint32_t s = __reduce_add_sync(mask, v[k]);
        if (lane == leader && s) atomicAdd(stats + k, (unsigned long long)s);
    }
    const uint32_t ps = __reduce_add_sync(mask, st.prop_skip);
    if (lane == leader && ps) atomicAdd(stats + LYAP_STAT_PROPOSAL_SKIPPED, (unsigned long long)ps);
    const uint32_t pr = __reduce_add_sync(mask, st.prop_rej);
    if (lane == leader && pr) atomicAdd(stats + LYAP_STAT_PROPOSAL_REWOUND, (unsigned long long)pr);
    const uint32_t ho = __reduce_add_sync(mask, st.handed);
    if (lane == leader && ho) atomicAdd(stats + LYAP_STAT_TAIL_HANDOVERS, (unsigned long long)ho);
    if (lane == leader && st.rounds) {
        atomicAdd(stats + LYAP_STAT_ROUNDS, (unsigned long long)st.rounds);
        atomicAdd(stats + LYAP_STAT_LANE_ROUNDS, (unsigned long long)st.lane_rounds);
        atomicMax(stats + LYAP_STAT_MAX_ROUNDS, (unsigned long long)st.rounds);
    }
}

// ----------------------------------------------------------------- render
// Hone rays with at least HONE_AHEAD steps behind them are sampled ahead
// too: honing almost always ends within 10 steps, but a ray whose hone step
// is below an ulp of t (a grazing ray) walks the cap of 256 steps one sample
// per round -- the last work of many frames.  Its next positions are known
// as long as the sign of lambda does not flip (a flip halves the step).
constexpr uint32_t HONE_AHEAD = 12;

__device__ __forceinline__ bool known_ahead(const Ray &r, bool fixed_step)
{
    return (fixed_step && r.phase <= PH_MARCH) || (r.phase >= PH_NORM0 && r.phase < PH_NORM0 + 5) ||
           (r.phase == PH_HONE && r.nh >= HONE_AHEAD);
}

// What a lane needs of another lane's ray to take samples ahead for it.
struct AheadState {
    V3 P, V, QdV;
    float dt, mag, t, t1;
    uint32_t phase, nm, cap, noskip, run;
};

__device__ __forceinline__ AheadState ahead_state(const Ray &r)
{
    return AheadState{r.P, r.V, r.QdV, r.dt, r.mag, r.t, r.t1, r.phase, r.nm, r.cap, r.pnoskip, prop_run(r)};
}

// lane `src`'s AheadState (the march bookkeeping only with a proposal)
template <bool PROP>
__device__ __forceinline__ AheadState shfl_ahead(const AheadState &a, uint32_t src)
{
    AheadState o;
    o.P.x = __shfl_sync(FULL, a.P.x, src);
    o.P.y = __shfl_sync(FULL, a.P.y, src);
    o.P.z = __shfl_sync(FULL, a.P.z, src);
    o.V.x = __shfl_sync(FULL, a.V.x, src);
    o.V.y = __shfl_sync(FULL, a.V.y, src);
    o.V.z = __shfl_sync(FULL, a.V.z, src);
    o.QdV.x = __shfl_sync(FULL, a.QdV.x, src);
    o.QdV.y = __shfl_sync(FULL, a.QdV.y, src);
    o.QdV.z = __shfl_sync(FULL, a.QdV.z, src);
    o.dt = __shfl_sync(FULL, a.dt, src);
    o.mag = __shfl_sync(FULL, a.mag, src);
    o.phase = __shfl_sync(FULL, a.phase, src);
    if constexpr (PROP) {
        o.t = __shfl_sync(FULL, a.t, src);
        o.t1 = __shfl_sync(FULL, a.t1, src);
        o.nm = __shfl_sync(FULL, a.nm, src);
        o.cap = __shfl_sync(FULL, a.cap, src);
        o.noskip = __shfl_sync(FULL, a.noskip, src);
        o.run = __shfl_sync(FULL, a.run, src);
    }
    return o;
}

// The sample `offset` positions ahead of the one at P: march steps and hone
// steps added one by one as ray_advance adds them (a hone step assumes no
// flip; the owner drops the result once its step changed), normal samples
// by index.  `valid` is false past the last normal sample.
__device__ __forceinline__ V3 sample_ahead(V3 P, V3 V, float dt, float mag, V3 QdV, uint32_t phase, uint32_t offset,
                                           bool &valid)
{
    valid = true;
    if (phase <= PH_MARCH) {
        for (uint32_t j = 0; j < offset; j++) P = P + V * dt;
        return P;
    }
    if (phase == PH_HONE) {
        for (uint32_t j = 0; j < offset; j++) P = P + QdV;
        return P;
    }
    const uint32_t k = phase - PH_NORM0 + offset;
    valid = k <= 5u;
    Ray tmp;
    tmp.P = P;
    tmp.mag = mag;
    tmp.phase = PH_NORM0 + (k > 5u ? 5u : k);
    return ray_sample_point(tmp);
}

// sample_ahead for the ray described by `a`.  PROP: the march positions skip
// the proposal's runs as the ray will (prop_march_ahead).
template <bool PROP>
__device__ __forceinline__ V3 sample_ahead(const AheadState &a, const PropGrid &pg, uint32_t offset, bool &valid)
{
    if constexpr (PROP) {
        if (a.phase <= PH_MARCH)
            return prop_march_ahead(a.P, a.V, a.dt, a.t, a.t1, a.nm, a.cap, a.noskip, a.run, pg, offset, valid);
    }
    return sample_ahead(a.P, a.V, a.dt, a.mag, a.QdV, a.phase, offset, valid);
}

// is the ray still where a sample taken ahead in phase `kind` at the round's
// start (hone step qdt0) continues it?
// gen0: the ray's proposal rewind count at the round's start (a rewind sends
// the march back, and the samples taken ahead no longer continue it).
__device__ __forceinline__ bool still_ahead(const Ray &r, uint32_t kind, float qdt0, uint32_t gen0)
{
    return kind == 1u ? (r.phase == PH_MARCH && prop_gen(r) == gen0)
                      : kind == 2u ? r.phase >= PH_NORM0 : (kind == 3u && r.phase == PH_HONE && r.Qdt == qdt0);
}

__device__ __forceinline__ uint32_t sample_kind(const Ray &r)
{
    return r.phase <= PH_MARCH ? 1u : r.phase >= PH_NORM0 ? 2u : 3u;
}

// One round of the render loop for a warp: every lane evaluates one lambda
// sample -- its own ray's next one, or, when the lane has no ray and
// speculation is allowed, a sample ahead on a ray still running in the warp --
// and the rays consume their results.  Returns the lane's ray outcome
// (RAY_CONTINUE while it needs more samples).
//
// Speculation in the tail.  Once the queue is empty, lanes without a ray
// evaluate, for the rays still running in this warp, the samples those rays
// will ask for next.  That is only possible where the next positions do not
// depend on the lambdas still to come: march steps when the step length is
// fixed (no jitter, near multiplier 1; with a proposal, the runs it skips
// are a function of the position and so known too), and the six normal
// samples.  Helper lane (owner, j) takes the owner's j-th sample ahead; the
// owner feeds the results to its state machine in order and drops the rest
// once the ray leaves that phase (or a proposal run is rewound).
template <bool PROP, class Lam, bool BLOCK2D = false>
__device__ __forceinline__ int sample_round(Ray &r, const bool active, const uint32_t amask, const Lam &lam,
                                            const LyapParams &prm, const bool spec_ok, const bool bracket_mode,
                                            const PropGrid &pg, LaneStats &st)
{
    uint32_t lane, warp;
    lane_warp<BLOCK2D>(lane, warp);
    __shared__ float slot_l[BLOCK2D ? ROUND_WARPS_2D : ROUND_WARPS][32];
    __shared__ uint32_t slot_b[BLOCK2D ? ROUND_WARPS_2D : ROUND_WARPS][32];
    uint32_t emask = 0, imask = 0, ne = 0, ni = 0, maxj = 0;
    bool helper = false;
    uint32_t owner = lane, offset = 0, rank = 0;
    if (spec_ok && amask != FULL) {
        const bool elig = active && known_ahead(r, true);
        emask = __ballot_sync(FULL, elig);
        ne = __popc(emask);
        if (ne) {
            imask = ~amask;
            ni = __popc(imask);
            maxj = (ni + ne - 1) / ne;
            if (!active) {
                rank = __popc(imask & ((1u << lane) - 1u));
                owner = nth_set_bit(emask, rank % ne);
                offset = 1 + rank / ne;
                helper = true;
            }
        }
    }
    V3 Q = active ? ray_sample_point<PROP>(r) : v3(3.0f, 3.0f, 3.0f);
    if (ne) {
        // every lane reads its owner's state (its own, for non-helpers)
        const AheadState o = shfl_ahead<PROP>(ahead_state(r), owner);
        if (helper) {
            bool v;
            Q = sample_ahead<PROP>(o, pg, offset, v);
            st.spec += 1;
        }
    }

    // one lambda sample for every lane (idle lanes evaluate a dummy point)
    st.rounds += 1;
    st.lane_rounds += __popc(amask) + (ne ? (ni < maxj * ne ? ni : maxj * ne) : 0u);
    bool skipped, fallback;
    const float lam_v = lam(Q.x, Q.y, Q.z, skipped, fallback);
    uint32_t bits = (skipped ? 1u : 0u) | (fallback ? 2u : 0u);
    if (ne) {
        __syncwarp();   // the owners' reads of the previous round are done
        if (helper) {
            slot_l[warp][rank] = lam_v;
            slot_b[warp][rank] = bits;
        }
        __syncwarp();
    }
    int res = RAY_CONTINUE;
    if (active) {
        const uint32_t kind = sample_kind(r);   // 1: march, 2: normal, 3: hone
        const float qdt0 = r.Qdt;
        const uint32_t gen0 = prop_gen(r);
        // this ray's helpers: ranks idx, idx + ne, ... below ni, one sample each
        uint32_t idx = 0, nh = 0;
        if (ne && ((emask >> lane) & 1u)) {
            idx = __popc(emask & ((1u << lane) - 1u));
            nh = idx < ni ? (ni - idx + ne - 1) / ne : 0u;
        }
        float l = lam_v;
        // the own sample, then the helpers' in order while the ray continues
        // in the phase they were taken for
        for (uint32_t j = 0;; j++) {
            st.samples += 1;
            st.skipped += bits & 1u;
            st.fallback += (bits >> 1) & 1u;
            st.spec_used += j ? 1u : 0u;
            res = ray_advance<PROP>(r, l, prm, bracket_mode, &pg);
            if (res != RAY_CONTINUE || j >= nh || !still_ahead(r, kind, qdt0, gen0)) break;
            l = slot_l[warp][j * ne + idx];
            bits = slot_b[warp][j * ne + idx];
        }
    }
    return res;
}

// The owner's consumption of a round's samples while its ray marches with a
// fixed step (no proposal): samples 0 and 1 are its own pair, then two per
// helper pair k, in slot k * ne + idx.  ray_advance would take them one by
// one; here the lane keeps only what depends on the order -- the sample
// count, the a / c sums, the near flag, t and the cap and box-exit checks --
// and takes each sample's position from where it was evaluated (the helpers
// stepped P exactly as the march steps it).  The sample at which the march
// stops (at or below the opaque threshold, or NaN) goes through ray_advance
// itself, on the ray as it stands there.  Same ray state, same statistics.
__device__ __forceinline__ int consume_march(Ray &r, float l0, float l1, uint32_t bits, V3 Q1, uint32_t nh,
                                             uint32_t ne, uint32_t idx, const float2 *slot_l,
                                             const uint32_t *slot_b, const float4 *slot_p,
                                             const LyapParams &prm, bool bracket_mode, LaneStats &st)
{
    const float opaque = prm.opaqueThreshold, chaos = prm.chaosThreshold, near_t = prm.nearThreshold;
    float a = r.a, c = r.c, t = r.t, tprev = r.tprev, lam_prev = r.l;
    uint32_t nm = r.nm, phase = r.phase;
    bool near = r.near;
    V3 Pa = r.P, Pb = Q1;   // positions of the current pair's two samples
    float la = l0, lb = l1;
    uint32_t bb = bits;
    auto store = [&](V3 P) {
        r.a = a;
        r.c = c;
        r.t = t;
        r.tprev = tprev;
        r.l = lam_prev;
        r.nm = nm;
        r.phase = phase;
        r.near = near;
        r.dt = near ? r.Ndt : r.Fdt;
        r.P = P;
    };
    for (uint32_t j = 0;; j++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float lam = h ? lb : la;
            const V3 P = h ? Pb : Pa;
            st.samples += 1;
            st.skipped += (bb >> h) & 1u;
            st.fallback += (bb >> (2 + h)) & 1u;
            st.spec_used += j ? 1u : 0u;
            if (!(lam > opaque)) {
                // the march stops here: the whole step on the ray as it stands
                store(P);
                return ray_advance<false>(r, lam, prm, bracket_mode, nullptr);
            }
            nm += 1;
            lam_prev = lam;
            if (phase == PH_MARCH) {
                if (lam > chaos) c = c + lam;
                else a = a + lam;
                near = lam <= near_t;
            }
            if (nm >= r.cap) {
                store(P);
                return RAY_MISS;
            }
            const float step = near ? r.Ndt : r.Fdt;
            tprev = t;
            t = t + step;
            if (t > r.t1) {
                store(P + r.V * step);
                return RAY_MISS;
            }
            phase = PH_MARCH;
            if (h == 1 && j >= nh) {
                store(P + r.V * step);
                return RAY_CONTINUE;
            }
        }
        const uint32_t slot = j * ne + idx;
        const float2 v = slot_l[slot];
        la = v.x;
        lb = v.y;
        bb = slot_b[slot];
        const float4 pa = slot_p[2 * slot], pb = slot_p[2 * slot + 1];
        Pa = v3(pa.x, pa.y, pa.z);
        Pb = v3(pb.x, pb.y, pb.z);
    }
}

// Paired rounds (RenderTuning::pairs): every lane evaluates two lambda samples
// per round as one packed evaluation (Lam::eval<2>; the product form runs both
// on FP32 pairs, fma.rn.f32x2).  Slot 0 is what sample_round evaluates; slot 1
// is the same ray's next sample when its position is already known -- the
// next march position when the step length is fixed (with a proposal: after
// the run it skips there), or the next normal sample -- else a dummy.  Lanes
// without a ray take the next samples of running rays two at a time: helper
// (owner, j) evaluates the owner's samples 2j and 2j+1 ahead.  The rays
// consume the results in order, exactly as sample_round does one by one.
template <bool PROP, class Lam>
__device__ __forceinline__ int sample_round_pair(Ray &r, const bool active, const uint32_t amask, const Lam &lam,
                                                 const LyapParams &prm, const bool fixed_step, const bool spec_ok,
                                                 const bool bracket_mode, const PropGrid &pg, LaneStats &st)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __shared__ float2 slot_l[ROUND_WARPS][32];
    __shared__ uint32_t slot_b[ROUND_WARPS][32];
    __shared__ float4 slot_p[PROP ? 1 : ROUND_WARPS][PROP ? 1 : 64];   // the helpers' sample positions
    // can this ray's next positions be known before its current sample's lambda?
    const bool ahead = active && known_ahead(r, fixed_step);
    // the ray's own second slot also takes its next hone step, assuming the
    // sign of lambda does not flip (a coin toss while honing converges); the
    // slot would otherwise evaluate a dummy, and the result is dropped when
    // the step changed.  Helpers keep to the samples known_ahead allows.
    const bool ahead_self = ahead || (active && r.phase == PH_HONE);
    uint32_t emask = 0, imask = 0, ne = 0, ni = 0, maxj = 0;
    bool helper = false;
    uint32_t owner = lane, offset = 0, rank = 0;
    if (spec_ok && amask != FULL) {
        emask = __ballot_sync(FULL, ahead);
        ne = __popc(emask);
        if (ne) {
            imask = ~amask;
            ni = __popc(imask);
            maxj = (ni + ne - 1) / ne;
            if (!active) {
                rank = __popc(imask & ((1u << lane) - 1u));
                owner = nth_set_bit(emask, rank % ne);
                offset = 2 + 2 * (rank / ne);
                helper = true;
            }
        }
    }
    V3 Q0 = active ? ray_sample_point<PROP>(r) : v3(3.0f, 3.0f, 3.0f);
    V3 Q1 = v3(3.0f, 3.0f, 3.0f);
    if (ahead_self) {
        bool v;
        Q1 = sample_ahead<PROP>(ahead_state(r), pg, 1u, v);
    }
    if (ne) {
        const AheadState o = shfl_ahead<PROP>(ahead_state(r), owner);
        if (helper) {
            bool v0, v1;
            Q0 = sample_ahead<PROP>(o, pg, offset, v0);
            Q1 = sample_ahead<PROP>(o, pg, offset + 1u, v1);
            st.spec += (v0 ? 1u : 0u) + (v1 ? 1u : 0u);
        }
    }

    st.rounds += 1;
    st.lane_rounds += __popc(amask) + (ne ? (ni < maxj * ne ? ni : maxj * ne) : 0u);
    const float qx[2] = {Q0.x, Q1.x}, qy[2] = {Q0.y, Q1.y}, qz[2] = {Q0.z, Q1.z};
    float lv[2];
    uint32_t skb, fbb;
    lam.template eval<2>(qx, qy, qz, lv, skb, fbb);
    uint32_t bits = skb | (fbb << 2);
    if (ne) {
        __syncwarp();   // the owners' reads of the previous round are done
        if (helper) {
            slot_l[warp][rank] = make_float2(lv[0], lv[1]);
            slot_b[warp][rank] = bits;
            if constexpr (!PROP) {
                slot_p[warp][2 * rank] = make_float4(Q0.x, Q0.y, Q0.z, 0.0f);
                slot_p[warp][2 * rank + 1] = make_float4(Q1.x, Q1.y, Q1.z, 0.0f);
            }
        }
        __syncwarp();
    }
    int res = RAY_CONTINUE;
    if (active) {
        const uint32_t kind = sample_kind(r);   // 1: march, 2: normal, 3: hone
        const float qdt0 = r.Qdt;
        const uint32_t gen0 = prop_gen(r);
        // this ray's helpers: ranks idx, idx + ne, ... below ni, two samples each
        uint32_t idx = 0, nh = 0;
        if (ne && ahead) {
            idx = __popc(emask & ((1u << lane) - 1u));
            nh = idx < ni ? (ni - idx + ne - 1) / ne : 0u;
        }
        if constexpr (!PROP) {
            // a fixed-step march: the lean consumption (ahead_self holds)
            if (kind == 1u && fixed_step)
                return consume_march(r, lv[0], lv[1], bits, Q1, nh, ne, idx, slot_l[warp], slot_b[warp],
                                     slot_p[warp], prm, bracket_mode, st);
        }
        float l0 = lv[0], l1 = lv[1];
        // the own pair (its second sample only when taken ahead), then the
        // helpers' pairs in order while the ray continues in the phase they
        // were taken for
        for (uint32_t j = 0;; j++) {
            st.samples += 1;
            st.skipped += bits & 1u;
            st.fallback += (bits >> 2) & 1u;
            st.spec_used += j ? 1u : 0u;
            res = ray_advance<PROP>(r, l0, prm, bracket_mode, &pg);
            if (res != RAY_CONTINUE || !ahead_self || !still_ahead(r, kind, qdt0, gen0)) break;
            st.samples += 1;
            st.skipped += (bits >> 1) & 1u;
            st.fallback += (bits >> 3) & 1u;
            st.spec_used += j ? 1u : 0u;
            res = ray_advance<PROP>(r, l1, prm, bracket_mode, &pg);
            if (res != RAY_CONTINUE || j >= nh || !still_ahead(r, kind, qdt0, gen0)) break;
            const float2 v = slot_l[warp][j * ne + idx];
            l0 = v.x;
            l1 = v.y;
            bits = slot_b[warp][j * ne + idx];
        }
    }
    return res;
}

// Queue position qi -> entry.  A ray's cost is set by where it meets the
// surface, and neighbouring rays cost alike: in scanline order the last
// entries handed out -- the rays still running when the queue drains -- are
// one band of the image.  With LYAP_FLAG_SPREAD_ORDER a stride near 0.618 n,
// coprime with the queue length n, spreads every 32 consecutive positions
// over the whole image.  Every entry is still taken exactly once.
__host__ __device__ inline uint32_t coprime_stride(uint32_t n)
{
    if (n < 3u) return 0u;
    uint32_t s = (uint32_t)((double)n * 0.6180339887498949 + 0.5);
    for (;; s++) {
        uint32_t a = n, b = s;
        while (b) {
            const uint32_t t = a % b;
            a = b;
            b = t;
        }
        if (a == 1u) return s;
    }
}

__device__ __forceinline__ uint32_t queue_entry(uint32_t qi, uint32_t n, uint32_t stride)
{
    return stride ? (uint32_t)(((uint64_t)qi * stride) % n) : qi;
}

// ---------------------------------------------------- the end of a frame
// After the pixel queue drains, warps leave as their rays end, and the few
// long rays left run on fewer and fewer warps.  Within a block, a warp left
// without rays asks for one, and a warp still holding two or more running
// rays hands its longest over through a one-ray mailbox in shared memory;
// the receiving warp runs it with 31 idle lanes sampling ahead for it.  The
// whole ray state moves, so the ray continues exactly as it would have.
// Only the warps of one block take part (always co-resident); no warp ever
// waits for another's work, and the receivers' polling is bounded.
struct TailBox {
    Ray r;
    uint32_t pix;
    int state;   // TAIL_EMPTY, TAIL_WRITING, TAIL_FULL, TAIL_TAKING
    int waiting, live, closed;   // warps asking / warps not yet gone / no more hand-overs
};
constexpr int TAIL_EMPTY = 0, TAIL_WRITING = 1, TAIL_FULL = 2, TAIL_TAKING = 3;
constexpr uint32_t TAIL_POLLS = 1u << 20;        // a receiver's polls before it stops asking
constexpr uint32_t TAIL_MIN_STEPS = 16u;         // rays with fewer march steps left stay put

__device__ __forceinline__ int tail_load(const int *p) { return *(volatile const int *)p; }

// A ray's march steps left (0 outside the march): what a hand-over is worth.
__device__ __forceinline__ uint32_t tail_steps_left(const Ray &r)
{
    if (r.phase > PH_MARCH || !(r.dt > 0.0f)) return 0u;
    const float k = (r.t1 - r.t) / r.dt;
    return k >= 1.0e6f ? 1000000u : (k > 0.0f ? (uint32_t)k : 0u);
}

// A warp without rays (the queue drained): wait for a handed-over ray.
// Returns true with the ray in lane 0's r / pix; false when no warp of the
// block can hand one over any more (the warp then leaves).
__device__ __forceinline__ bool tail_receive(TailBox &box, Ray &r, uint32_t &pix)
{
    const uint32_t lane = threadIdx.x & 31u;
    int got = 0;
    if (lane == 0) {
        atomicAdd(&box.waiting, 1);
        for (uint32_t it = 0; it < TAIL_POLLS; it++) {
            if (atomicCAS(&box.state, TAIL_FULL, TAIL_TAKING) == TAIL_FULL) {
                got = 1;
                break;
            }
            // every warp still here is asking: nobody holds a ray to hand over
            if (tail_load(&box.waiting) >= tail_load(&box.live)) break;
            __nanosleep(256);
        }
        if (!got && tail_load(&box.waiting) < tail_load(&box.live)) {
            // polls ran out: stop hand-overs, and take one already under way
            atomicExch(&box.closed, 1);
            __threadfence_block();
            for (uint32_t it = 0; it < 65536u && tail_load(&box.state) == TAIL_WRITING; it++) __nanosleep(64);
            if (atomicCAS(&box.state, TAIL_FULL, TAIL_TAKING) == TAIL_FULL) got = 1;
        }
        if (got) {
            __threadfence_block();
            r = box.r;
            pix = box.pix;
            __threadfence_block();
            atomicExch(&box.state, TAIL_EMPTY);
        } else {
            atomicSub(&box.live, 1);   // leaving
        }
        atomicSub(&box.waiting, 1);
    }
    return __shfl_sync(FULL, got, 0) != 0;
}

// A warp in the tail with two or more running rays: hand the longest over
// when a warp of the block is asking.  Returns true on the lane whose ray left.
__device__ __forceinline__ bool tail_offer(TailBox &box, const Ray &r, uint32_t pix, bool active)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t amask = __ballot_sync(FULL, active);
    if (__popc(amask) < 2) return false;
    if (tail_load(&box.waiting) <= 0 || tail_load(&box.closed) || tail_load(&box.state) != TAIL_EMPTY) return false;
    const uint32_t key = active ? tail_steps_left(r) : 0u;
    const uint32_t best = __reduce_max_sync(FULL, key);
    if (best < TAIL_MIN_STEPS) return false;
    const uint32_t donor = __ffs(__ballot_sync(FULL, key == best)) - 1;
    int gave = 0;
    if (lane == donor && atomicCAS(&box.state, TAIL_EMPTY, TAIL_WRITING) == TAIL_EMPTY) {
        if (tail_load(&box.closed)) {
            atomicExch(&box.state, TAIL_EMPTY);
        } else {
            box.r = r;
            box.pix = pix;
            __threadfence_block();
            atomicExch(&box.state, TAIL_FULL);
            gave = 1;
        }
    }
    return gave != 0;
}

template <class Lam>
struct RenderTuning {
    static constexpr bool product = Lam::mode == MODE_PRODUCT;
    static constexpr bool pairs = product ? LYAP_RENDER_PAIRS_PRODUCT != 0 : LYAP_RENDER_PAIRS_PLAIN != 0;
    static constexpr int min_blocks = product ? LYAP_RENDER_MIN_BLOCKS_PRODUCT : LYAP_RENDER_MIN_BLOCKS_PLAIN;
    static constexpr int threads = product ? LYAP_RENDER_THREADS_PRODUCT : LYAP_RENDER_THREADS_PLAIN;
    // the batch kernel, in blocks of LYAP_BATCH_THREADS: the same registers per thread
    static constexpr int batch_min_blocks =
        (min_blocks * threads + LYAP_BATCH_THREADS - 1) / LYAP_BATCH_THREADS;
};

// PROP: the learned proposal's grid (job.prop) decides which march
// positions are skipped; the host launches this instantiation only with a
// grid and a fixed step length (jitter 0, near multiplier 1).
template <class Lam, bool PROP = false>
__global__ void __launch_bounds__(RenderTuning<Lam>::threads, RenderTuning<Lam>::min_blocks)
    render_persistent(const __grid_constant__ RenderJob job, uint32_t *__restrict__ work_counter,
                      unsigned long long *__restrict__ stats)
{
    const uint32_t lane = threadIdx.x & 31u;
    // the queue: the listed rays that meet the box, or every pixel
    const uint32_t nq = job.list ? *job.list_count : job.width * job.height;
    const uint32_t stride = (job.flags & LYAP_FLAG_SPREAD_ORDER) ? coprime_stride(nq) : 0u;
    const Lam lam(job.seq, job.seq_period, job.prm);
    const CamRays cr = cam_rays(job.cam);
    // march positions are known ahead only with a fixed step length
    const bool fixed_step = (job.prm.jitter == 0.0f) && (job.prm.nearMultiplier == 1.0f);
    const bool spec_ok = fixed_step && !(job.flags & LYAP_FLAG_NO_SPECULATION);
    const bool bracket_mode = (job.flags & LYAP_FLAG_BISECT_F64) != 0u;
    const PropGrid &pg = job.prop;   // the parameter itself: constant-bank reads
    if constexpr (PROP) {
        // the proposal's bits in shared memory when they fit (the launch sized it)
        if (pg.smem_words) {
            for (uint32_t i = threadIdx.x; i < pg.smem_words; i += blockDim.x) lyap_prop_smem[i] = __ldg(pg.bits + i);
            __syncthreads();
        }
    }
    LaneStats st = {};
    Ray r;
    r.phase = PH_MARCH0;
    uint32_t pix = 0;
    bool active = false, drained = false, drain_seen = false;
    if (stats && lane == 0) atomicMax(stats + LYAP_STAT_T_START, ~global_ns());
    __shared__ TailBox tail_box;
    const bool tail_balance = !(job.flags & LYAP_FLAG_NO_TAIL_BALANCE);
    if (threadIdx.x == 0) {
        tail_box.state = TAIL_EMPTY;
        tail_box.waiting = 0;
        tail_box.live = (int)(blockDim.x >> 5);
        tail_box.closed = 0;
    }
    __syncthreads();

    for (;;) {
        // refill the lanes whose ray has ended
        for (;;) {
            const bool need = !active && !drained;
            const uint32_t mask = __ballot_sync(FULL, need);
            if (mask == 0) break;
            const uint32_t leader = __ffs(mask) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work_counter, (uint32_t)__popc(mask));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const uint32_t qi = base + __popc(mask & ((1u << lane) - 1u));
                if (qi >= nq) {
                    drained = true;
                } else {
                    const uint32_t e = queue_entry(qi, nq, stride);
                    if (job.list) {
                        // a listed ray meets the box; its setup comes with it
                        const RayEntry en = job.list[e];
                        pix = en.pix;
                        ray_start(r, cr.C, en, job.prm);
                        active = true;
                    } else {
                        pix = e;
                        if (ray_init(r, cr, job.prm, e % job.width, e / job.width)) {
                            active = true;
                        } else {
                            r.nm = r.nh = r.ns = 0;
                            finish_pixel(job.rgba, job.points, job.counts, e, r, false, cr.C, job.lights,
                                         job.n_lights, job.light_model, st);
                        }
                    }
                }
            }
        }
        if (!drain_seen && __any_sync(FULL, drained)) {
            drain_seen = true;
            if (stats && lane == 0) atomicMax(stats + LYAP_STAT_T_DRAIN, ~global_ns());
        }
        // in the tail, hand the warp's longest ray to a warp of the block that asks
        if (tail_balance && drain_seen && tail_offer(tail_box, r, pix, active)) {
            active = false;
            st.handed += 1;
        }
        const uint32_t amask = __ballot_sync(FULL, active);
        if (amask == 0) {
            // the queue has drained for every lane: take over a ray of another warp, or leave
            if (tail_balance && tail_receive(tail_box, r, pix)) {
                active = lane == 0;
                continue;
            }
            break;
        }

        int res;
        if constexpr (RenderTuning<Lam>::pairs)
            res = sample_round_pair<PROP>(r, active, amask, lam, job.prm, fixed_step, spec_ok, bracket_mode, pg, st);
        else
            res = sample_round<PROP>(r, active, amask, lam, job.prm, spec_ok, bracket_mode, pg, st);
        if (active && res == RAY_BRACKET) {
            // precision form: hand the crossing to the FP64 bisection pass
            job.bracket[2 * (size_t)pix + 0] = r.tprev;
            job.bracket[2 * (size_t)pix + 1] = r.t;
            const uint32_t slot = atomicAdd(job.hits, 1u);
            job.hits[1 + slot] = pix;
            Ray keep = r;
            keep.N = v3(0.f, 0.f, 0.f);
            store_point(job.points + pix, keep, true);
            reinterpret_cast<uint32_t *>(job.rgba)[pix] = 0u;
            if (job.counts) {
                job.counts[3 * (size_t)pix + 0] = r.nm - r.ns;
                job.counts[3 * (size_t)pix + 1] = 0u;
                job.counts[3 * (size_t)pix + 2] = 0u;
            }
            st.march += r.nm - r.ns;
            st.prop_skip += r.ns;
            st.prop_rej += prop_rewound(r);
            st.rays += 1;
            active = false;
        } else if (active && res != RAY_CONTINUE) {
            finish_pixel(job.rgba, job.points, job.counts, pix, r, res == RAY_HIT, cr.C, job.lights, job.n_lights,
                         job.light_model, st);
            active = false;
        }
    }
    flush_stats(stats, st, FULL);
    if (stats && lane == 0) atomicMax(stats + LYAP_STAT_T_END, global_ns());
}

// ----------------------------------------------------------------- batch
struct BatchTables {
    const RenderJob *jobs;
    const uint32_t *chunk_job;    // per chunk: request index
    const uint32_t *chunk_tile;   // per chunk: first tile within the request
    uint32_t n_chunks;
    uint32_t tile_w, tile_h, tiles_per_chunk;
};

// Many requests in one launch (lyap_batch.cu): persistent warps take chunks
// of tiles from a global counter; a warp renders one request at a time (its
// lambda loop must be uniform), so it continues with the next chunk while
// that belongs to the same request and otherwise lets its rays run out --
// idle lanes speculate for the rays still running -- before switching.  Lam
// is RuntimeLambda (any sequences; the library's kernel) or, for the
// requests of one sequence group of the batch, ConstLambda compiled for that
// sequence at run time, which runs paired rounds as the single-frame render
// does.
template <class Lam>
__global__ void __launch_bounds__(LYAP_BATCH_THREADS, RenderTuning<Lam>::batch_min_blocks)
    render_batch(const __grid_constant__ BatchTables tb, uint32_t *__restrict__ chunk_counter,
                 unsigned long long *__restrict__ stats)
{
    if (tb.n_chunks == 0) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t tile_px = tb.tile_w * tb.tile_h;
    const uint32_t slots_per_chunk = tb.tiles_per_chunk * tile_px;
    LaneStats st = {};

    // the warp's request (uniform)
    uint32_t cur = tb.chunk_job[0];
    const RenderJob *J = tb.jobs + cur;
    Lam lam(J->seq, J->seq_period, J->prm);
    LyapParams prm = J->prm;
    CamRays cr = cam_rays(J->cam);
    uint32_t W = J->width, H = J->height, tiles_x = (W + tb.tile_w - 1) / tb.tile_w;
    uint32_t n_tiles = tiles_x * ((H + tb.tile_h - 1) / tb.tile_h);
    bool spec_ok = (prm.jitter == 0.0f) && (prm.nearMultiplier == 1.0f) && !(J->flags & LYAP_FLAG_NO_SPECULATION);
    bool have_job = false;
    uint32_t tile0 = 0, slot_next = 0, slot_end = 0;
    uint32_t pending = 0xffffffffu;   // a claimed chunk of another request
    bool no_more = false;

    Ray r;
    r.phase = PH_MARCH0;
    uint32_t pix = 0;
    bool active = false;

    for (;;) {
        // refill idle lanes from the current chunk, claiming chunks of the same request
        for (;;) {
            const bool need = !active && have_job;
            const uint32_t mask = __ballot_sync(FULL, need);
            if (mask == 0) break;
            if (slot_next >= slot_end) {
                if (no_more || pending != 0xffffffffu) break;
                uint32_t c = 0;
                if (lane == 0) c = atomicAdd(chunk_counter, 1u);
                c = __shfl_sync(FULL, c, 0);
                if (c >= tb.n_chunks) {
                    no_more = true;
                    break;
                }
                if (tb.chunk_job[c] != cur) {
                    pending = c;   // switch once this request's rays have run out
                    break;
                }
                tile0 = tb.chunk_tile[c];
                slot_next = 0;
                slot_end = slots_per_chunk;
            }
            const uint32_t s = slot_next + __popc(mask & ((1u << lane) - 1u));
            slot_next += __popc(mask);
            if (need && s < slot_end) {
                const uint32_t tile = tile0 + s / tile_px, within = s % tile_px;
                const uint32_t x = (tile % tiles_x) * tb.tile_w + within % tb.tile_w;
                const uint32_t y = (tile / tiles_x) * tb.tile_h + within / tb.tile_w;
                if (tile < n_tiles && x < W && y < H) {
                    pix = x + y * W;
                    if (ray_init(r, cr, prm, x, y)) {
                        active = true;
                    } else {
                        r.nm = r.nh = r.ns = 0;
                        finish_pixel(J->rgba, J->points, J->counts, pix, r, false, cr.C, J->lights, J->n_lights,
                                     J->light_model, st);
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(FULL, active);
        if (amask == 0) {
            // every ray of this warp has ended: move to the pending request, or claim one
            uint32_t c = pending;
            if (c == 0xffffffffu) {
                if (no_more) break;
                if (lane == 0) c = atomicAdd(chunk_counter, 1u);
                c = __shfl_sync(FULL, c, 0);
                if (c >= tb.n_chunks) break;
            }
            pending = 0xffffffffu;
            cur = tb.chunk_job[c];
            J = tb.jobs + cur;
            lam = Lam(J->seq, J->seq_period, J->prm);
            prm = J->prm;
            cr = cam_rays(J->cam);
            W = J->width;
            H = J->height;
            tiles_x = (W + tb.tile_w - 1) / tb.tile_w;
            n_tiles = tiles_x * ((H + tb.tile_h - 1) / tb.tile_h);
            spec_ok = (prm.jitter == 0.0f) && (prm.nearMultiplier == 1.0f) && !(J->flags & LYAP_FLAG_NO_SPECULATION);
            have_job = true;
            tile0 = tb.chunk_tile[c];
            slot_next = 0;
            slot_end = slots_per_chunk;
            continue;
        }
        int res;
        if constexpr (RenderTuning<Lam>::pairs) {
            const bool fixed_step = (prm.jitter == 0.0f) && (prm.nearMultiplier == 1.0f);
            res = sample_round_pair<false>(r, active, amask, lam, prm, fixed_step, spec_ok, false, PropGrid{}, st);
        } else {
            res = sample_round<false>(r, active, amask, lam, prm, spec_ok, false, PropGrid{}, st);
        }
        if (active && res != RAY_CONTINUE) {
            finish_pixel(J->rgba, J->points, J->counts, pix, r, res == RAY_HIT, cr.C, J->lights, J->n_lights,
                         J->light_model, st);
            active = false;
        }
    }
    flush_stats(stats, st, FULL);
}


// ----------------------------------------------------------------- volume
__device__ __forceinline__ float voxel_coord(float lo, float hi, uint32_t i, uint32_t n)
{
    return lo + ((hi - lo) * (float)i) / (float)n;
}

template <class Lam, int K>
__global__ void __launch_bounds__(LYAP_VOLUME_THREADS, LYAP_VOLUME_MIN_BLOCKS)
    volume_sweep(const __grid_constant__ VolumeJob job, unsigned long long *__restrict__ stats)
{
    const Lam lam(job.seq, job.seq_period, job.prm);
    const uint64_t nxy = (uint64_t)job.nx * job.ny;
    const uint64_t total = nxy * job.nz;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nwork = (total + 32u * K - 1) / (32u * K);
    const uint64_t wstride = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    uint32_t skipped_n = 0, fallback_n = 0, samples = 0;
    for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwork; w += wstride) {
        float px[K], py[K], pz[K], out[K];
        uint64_t idx[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            uint64_t i = w * (32u * K) + 32u * k + lane;
            idx[k] = i;
            if (i >= total) i = total - 1;
            const uint32_t z = (uint32_t)(i / nxy);
            const uint64_t rxy = i - (uint64_t)z * nxy;
            const uint32_t y = (uint32_t)(rxy / job.nx);
            const uint32_t x = (uint32_t)(rxy - (uint64_t)y * job.nx);
            px[k] = voxel_coord(job.lo[0], job.hi[0], x, job.nx);
            py[k] = voxel_coord(job.lo[1], job.hi[1], y, job.ny);
            pz[k] = voxel_coord(job.lo[2], job.hi[2], z, job.nz);
        }
        uint32_t sk, fb;
        lam.template eval<K>(px, py, pz, out, sk, fb);
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (idx[k] < total) {
                __stcs(job.out + idx[k], out[k]);
                samples += 1;
                skipped_n += (sk >> k) & 1u;
                fallback_n += (fb >> k) & 1u;
            }
        }
    }
    if (stats) {
        const uint32_t mask = __activemask();
        const uint32_t s0 = __reduce_add_sync(mask, samples);
        const uint32_t s1 = __reduce_add_sync(mask, skipped_n);
        const uint32_t s7 = __reduce_add_sync(mask, fallback_n);
        if (lane == (uint32_t)(__ffs(mask) - 1)) {
            if (s0) atomicAdd(stats + ST_SAMPLES, (unsigned long long)s0);
            if (s1) atomicAdd(stats + ST_SKIPPED, (unsigned long long)s1);
            if (s7) atomicAdd(stats + ST_FALLBACK, (unsigned long long)s7);
        }
    }
}

}  // namespace lyapgb
