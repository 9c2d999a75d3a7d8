/*
 * lyap_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * lyapunov3d hot path: the per-ray Lyapunov raymarch (kernel_calc_render,
 * kernel.cu:500) and the dense lambda volume sweep (kernel_calc_volume,
 * kernel.cu:518), plus the host scene helpers the reference runs before a
 * launch (scene.hpp:11-15).
 *
 * Structs are binary-identical to the reference's structs.hpp:26-80 with
 * Real = float (sizes 224 / 56 / 36 / 4 bytes); the *D variants are the
 * DOUBLE_REALS layouts (structs.hpp:10-13; 384 / 104 / 72 bytes).  The
 * struct names (_LyapCamLight, LyapParams, LyapPoint, RGBA) are the
 * reference's, so C++ code that launches kernel_calc_render through
 * lyap_kernel.hpp links against this library under the reference's mangled
 * names.
 *
 * Conventions of every entry point:
 *  - returns LYAP_OK (0) or a negative LYAP_ERR_* code; never exits the
 *    process (the reference's helper_cuda checks and scene.cu:98-100 call
 *    exit); lyap_last_error_string() describes the last failure of the
 *    calling thread;
 *  - "d_" pointers are device memory owned by the caller;
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream); device entry points are asynchronous on it unless the name
 *    says _host.
 */
#ifndef LYAP_GB300_H
#define LYAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LYAP_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define LYAP_OK                 0
#define LYAP_ERR_INVALID_ARG   (-1)  /* null pointer, zero/oversized size  */
#define LYAP_ERR_SEQUENCE      (-2)  /* bad sequence letter / length       */
#define LYAP_ERR_CUDA          (-3)  /* a CUDA runtime call failed         */
#define LYAP_ERR_NO_DEVICE     (-4)  /* no usable sm_103 device            */
#define LYAP_ERR_OUT_OF_MEMORY (-5)
#define LYAP_ERR_CAPACITY      (-6)  /* output buffer too small            */
#define LYAP_ERR_JIT           (-7)  /* run-time specialisation required
                                        (LYAP_FLAG_REQUIRE_JIT) but unavailable */

/* Longest expanded sequence (entries, including the -1 terminator). */
#define LYAP_MAX_SEQ_LEN 4096
/* MAX_LIGHTS, params.hpp:21 */
#define LYAP_MAX_LIGHTS 16

/* ---- ABI types (structs.hpp:20-80, Real = float) ----------------------- */
#if defined(__GNUC__) || defined(__clang__) || defined(__CUDACC__)
#define LYAP_ALIGN16 __attribute__((aligned(16)))
#else
#define LYAP_ALIGN16
#endif

typedef struct { float x, y, z; } LyapVec;                     /* float3 */
typedef struct LYAP_ALIGN16 { float x, y, z, w; } LyapQuat;     /* float4 */
typedef struct LYAP_ALIGN16 { float x, y, z, w; } LyapColor;    /* float4 r,g,b,a */

/* structs.hpp:26-51: one type serves as camera and as light. */
typedef struct _LyapCamLight {
    LyapVec C;                 /* position */
    LyapQuat Q;                /* orientation */
    float M;                   /* screen half-width at unit distance */
    LyapVec V;                 /* forward axis, Q*(0,0,1) */
    LyapVec S0;                /* screen corner ray, Q*(-M,-M,1) */
    LyapVec SDX;               /* per-pixel x step, Q*(2M/renderWidth,0,0) */
    LyapVec SDY;               /* per-pixel y step, Q*(0,2M/renderHeight,0) */
    uint32_t textureWidth;
    uint32_t textureHeight;
    uint32_t renderWidth;
    uint32_t renderHeight;
    uint32_t renderDenominator;
    float lightInnerCone, lightOuterCone;
    float lightRange;
    LyapColor ambient;
    LyapColor diffuseColor;
    float diffusePower;
    LyapColor specularColor;
    float specularPower;
    float specularHardness;
    LyapColor chaosColor;
} LyapLight;
typedef struct _LyapCamLight LyapCam;

/* structs.hpp:53-68 */
typedef struct {
    float d;                   /* value of symbol D */
    uint32_t settle;           /* iterations before accumulation */
    uint32_t accum;            /* accumulated iterations */
    uint32_t stepMethod;       /* 1: depth steps per box chord; else |V|/depth */
    float nearThreshold;
    float nearMultiplier;
    float opaqueThreshold;     /* march stops at lambda <= this */
    float chaosThreshold;
    float depth;
    float jitter;
    float refine;
    float gradient;
    float lMin;                /* parameter box [lMin, lMax]^3 (honoured here) */
    float lMax;
} LyapParams;

/* structs.hpp:70-76 */
typedef struct {
    LyapVec P;                 /* hit point */
    LyapVec N;                 /* unit normal (central differences) */
    float a;                   /* lambda accumulated between opaque and chaos */
    float c;                   /* lambda accumulated above chaos */
    float l;                   /* lambda at the hit point */
} LyapPoint;

/* structs.hpp:78-80 */
typedef struct { unsigned char r, g, b, a; } RGBA;

/* ---- DOUBLE_REALS layouts (structs.hpp:10-13) -------------------------- */
typedef struct { double x, y, z; } LyapVecD;                     /* double3 */
typedef struct LYAP_ALIGN16 { double x, y, z, w; } LyapQuatD;    /* double4 */
typedef struct LYAP_ALIGN16 { double x, y, z, w; } LyapColorD;

typedef struct _LyapCamLightD {
    LyapVecD C;
    LyapQuatD Q;
    double M;
    LyapVecD V, S0, SDX, SDY;
    uint32_t textureWidth, textureHeight, renderWidth, renderHeight;
    uint32_t renderDenominator;
    double lightInnerCone, lightOuterCone;
    double lightRange;
    LyapColorD ambient;
    LyapColorD diffuseColor;
    double diffusePower;
    LyapColorD specularColor;
    double specularPower;
    double specularHardness;
    LyapColorD chaosColor;
} LyapLightD;
typedef struct _LyapCamLightD LyapCamD;

typedef struct {
    double d;
    uint32_t settle, accum, stepMethod;
    double nearThreshold, nearMultiplier, opaqueThreshold, chaosThreshold;
    double depth, jitter, refine, gradient, lMin, lMax;
} LyapParamsD;

typedef struct {
    LyapVecD P, N;
    double a, c, l;
} LyapPointD;

#ifndef __CUDACC_RTC__   /* offsetof checks run in host compiles */
/* Layout checks against the reference's structs (sizes and offsets as the
 * reference's own build lays them out with CUDA's vector types). */
#if defined(__cplusplus)
#define LYAP_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define LYAP_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif
LYAP_STATIC_ASSERT(sizeof(LyapCam) == 224, "LyapCam size");
LYAP_STATIC_ASSERT(offsetof(LyapCam, Q) == 16, "LyapCam.Q");
LYAP_STATIC_ASSERT(offsetof(LyapCam, SDY) == 72, "LyapCam.SDY");
LYAP_STATIC_ASSERT(offsetof(LyapCam, lightRange) == 112, "LyapCam.lightRange");
LYAP_STATIC_ASSERT(offsetof(LyapCam, ambient) == 128, "LyapCam.ambient");
LYAP_STATIC_ASSERT(offsetof(LyapCam, specularColor) == 176, "LyapCam.specularColor");
LYAP_STATIC_ASSERT(offsetof(LyapCam, chaosColor) == 208, "LyapCam.chaosColor");
LYAP_STATIC_ASSERT(sizeof(LyapParams) == 56, "LyapParams size");
LYAP_STATIC_ASSERT(offsetof(LyapParams, lMax) == 52, "LyapParams.lMax");
LYAP_STATIC_ASSERT(sizeof(LyapPoint) == 36, "LyapPoint size");
LYAP_STATIC_ASSERT(sizeof(RGBA) == 4, "RGBA size");
LYAP_STATIC_ASSERT(sizeof(LyapCamD) == 384, "LyapCamD size");
LYAP_STATIC_ASSERT(offsetof(LyapCamD, lightInnerCone) == 192, "LyapCamD.lightInnerCone");
LYAP_STATIC_ASSERT(offsetof(LyapCamD, chaosColor) == 352, "LyapCamD.chaosColor");
LYAP_STATIC_ASSERT(sizeof(LyapParamsD) == 104, "LyapParamsD size");
LYAP_STATIC_ASSERT(offsetof(LyapParamsD, nearThreshold) == 24, "LyapParamsD.nearThreshold");
LYAP_STATIC_ASSERT(sizeof(LyapPointD) == 72, "LyapPointD size");
#endif /* !__CUDACC_RTC__ */

/* ---- extensions (kept out of the reference structs) -------------------- */
#define LYAP_VERSION_STRING "0.1.0"
#define LYAP_MAX_PIXELS  (1ull << 31)    /* per frame */
#define LYAP_MAX_VOXELS  (1ull << 36)    /* per volume (256 GiB of float) */

/* How lambda is accumulated.  Both iterate the orbit identically
 * (t = r*x; x = fma(-t, x, t); d = fma(-2r, x, r)). */
#define LYAP_VARIANT_PLAIN   0u  /* sum of log2|d| per step (the drop-in)    */
#define LYAP_VARIANT_PRODUCT 1u  /* running product of |d|, renormalised by
                                    exponent extraction every 8 steps, one
                                    log2 at the end                          */

#define LYAP_LIGHT_SPOT        0u /* the reference's shade() (kernel.cu:25)  */
#define LYAP_LIGHT_DIRECTIONAL 1u /* Lambert: ambient + diffuse*clamp(N.-V)  */

/* Slots of the optional statistics array (LyapRenderExt / LyapVolumeExt
 * d_stats, LYAP_STAT_COUNT x uint64, accumulated with atomics; the caller
 * zeroes it).  Speculative samples that a ray does not use are not counted
 * in SAMPLES.
 * Logistic-map iterations performed = SAMPLES*(settle+accum) - SKIPPED*accum. */
#define LYAP_STAT_SAMPLES  0  /* lambda evaluations                          */
#define LYAP_STAT_SKIPPED  1  /* evaluations whose settle landed on x = 0.5  */
#define LYAP_STAT_MARCH    2  /* render: march samples                       */
#define LYAP_STAT_HONE     3  /* render: honing samples                      */
#define LYAP_STAT_NORMAL   4  /* render: normal samples                      */
#define LYAP_STAT_HITS     5  /* render: rays that hit                       */
#define LYAP_STAT_RAYS     6  /* render: rays finished                       */
#define LYAP_STAT_FALLBACK 7  /* product evaluations taken again: with blocks
                                 of 8 steps after longer blocks left the
                                 range, or in the plain form               */
#define LYAP_STAT_SPEC     8  /* render: samples taken ahead by idle lanes   */
#define LYAP_STAT_SPEC_USED 9 /* render: of those, samples the rays used      */
#define LYAP_STAT_ROUNDS   10 /* render: warp rounds (one lambda sample each) */
#define LYAP_STAT_LANE_ROUNDS 11 /* render: lanes sampling, summed over rounds */
#define LYAP_STAT_MAX_ROUNDS 12  /* render: most rounds of any warp (max)     */
#define LYAP_STAT_PROPOSAL_SKIPPED 13 /* render: march samples the learned
                                          proposal skipped (not evaluated) */
#define LYAP_STAT_PROPOSAL_POINTS 14  /* render: points the proposal net evaluated
                                          (grid corners, when this call built
                                          the net's grid; 0 when it was cached) */
#define LYAP_STAT_NET_TIMEOUTS 15     /* tensor-core waits that ran out; the
                                          tiles concerned skip nothing */
/* render timing (%globaltimer, ns): START and DRAIN hold the bitwise NOT of
 * the earliest warp start / the earliest moment a warp found the pixel queue
 * empty (kept with atomicMax on ~t, so a zeroed array works); END the latest
 * warp end.  (END - ~DRAIN) / (END - ~START) is the share of the launch spent
 * finishing rays already started. */
#define LYAP_STAT_T_START  16
#define LYAP_STAT_T_DRAIN  17
#define LYAP_STAT_T_END    18
#define LYAP_STAT_PROPOSAL_REWOUND 19 /* render: confirming samples at or below the
                                          proposal's threshold, each of which sent
                                          its ray back to the start of the skipped
                                          run (evaluated, then discarded) */
#define LYAP_STAT_TAIL_HANDOVERS 20   /* render: rays a warp handed to another warp of
                                          its block after the pixel queue drained */
#define LYAP_STAT_COUNT    21

/* LyapRenderExt / LyapVolumeExt flags.  Given the host copy of the sequence
 * (h_seq), the library compiles the kernels for that sequence at run time
 * (NVRTC, cached per sequence for the process; identical results, fewer
 * registers, faster); without NVRTC or for periods above 32 it uses its
 * precompiled kernels. */
#define LYAP_FLAG_NO_JIT      1u  /* always use the precompiled kernels       */
#define LYAP_FLAG_REQUIRE_JIT 2u  /* fail (LYAP_ERR_JIT) instead of falling back */
#define LYAP_FLAG_NO_SPECULATION 4u /* render: idle lanes do not take samples
                                       ahead for running rays (same results) */
#define LYAP_FLAG_NO_TAIL_BALANCE 32u /* render: after the pixel queue
                                         drains, warps of a block do not hand
                                         their longest rays to warps left
                                         without one (same results) */
#define LYAP_FLAG_SPREAD_ORDER 16u /* render: the pixel queue spreads
                                      consecutive pixels over the image
                                      instead of scanline order (same
                                      results; frame time within +-10%) */
#define LYAP_FLAG_BISECT_F64  8u  /* render, precision form: instead of the
                                     reference's honing, bisect each ray's
                                     crossing [last sample above, first at or
                                     below the opaque threshold] bisect_halvings
                                     times (default 20) with lambda in double;
                                     the point's l is then the double lambda at
                                     the stored (float) point */

typedef struct {
    uint32_t size;               /* = sizeof(LyapRenderExt) */
    uint32_t variant;            /* LYAP_VARIANT_* (default PLAIN) */
    uint32_t light_model;        /* LYAP_LIGHT_* (default SPOT) */
    uint32_t flags;              /* LYAP_FLAG_* */
    uint32_t *d_counts;          /* optional device array, 3 per pixel:
                                    march, honing, normal samples */
    unsigned long long *d_stats; /* optional device array, LYAP_STAT_COUNT */
    uint32_t blocks_per_sm;      /* launch shape, 0 = automatic */
    uint32_t threads_per_block;  /* multiple of 32, <= 128; 0 = automatic */
    const int32_t *h_seq;        /* optional host copy of d_seq (seq_len entries) */
    uint32_t bisect_halvings;    /* LYAP_FLAG_BISECT_F64: halvings (0 = 20) */
    uint32_t pad_;
    /* learned proposal (no reference counterpart): with a trained net
     * (lyap_net_train), the library evaluates the net once at the corners
     * of a proposal_grid^3 grid over the net's box and keeps, per cell, the
     * minimum (with proposal_dilate, the minimum over the 27 cells around);
     * the grid is cached per device and net, so only the first call with a
     * net pays for it (and synchronises its stream once).  The march then
     * skips march positions whose cell holds a value >=
     * opaqueThreshold + proposal_margin, at most proposal_segment - 1 in a
     * row, and evaluates the position after every such run exactly: at or
     * below that threshold the ray goes back to the run's first position and
     * evaluates every position up to it.  So every hit is exact, and a
     * surface is missed only where it enters and leaves the ray within one
     * run the net called empty.  Skipped positions add nothing to the point's
     * a and c sums.  Needs jitter 0 and nearMultiplier 1.  Callers built
     * against the shorter struct (size = offsetof(LyapRenderExt, proposal))
     * keep working. */
    const struct LyapNet *proposal; /* host struct, or NULL */
    float proposal_margin;       /* >= 0 */
    uint32_t proposal_segment;   /* longest skipped run + 1, 1..64 (0 = 8) */
    uint32_t proposal_dilate;    /* 0 or 1 */
    uint32_t proposal_grid;      /* cells per axis, 2..512 (0 = LYAP_PROPOSAL_GRID_DEFAULT) */
} LyapRenderExt;
#define LYAP_PROPOSAL_GRID_DEFAULT 64u
/* grids of up to this many bytes of bits (n^3 / 8; 64^3 = 32 KB) are read
 * from shared memory during the march, larger ones from global memory */
#define LYAP_PROPOSAL_SMEM_MAX 49152u

typedef struct {
    uint32_t size;               /* = sizeof(LyapVolumeExt) */
    uint32_t variant;            /* LYAP_VARIANT_* */
    unsigned long long *d_stats; /* optional, LYAP_STAT_COUNT */
    uint32_t blocks_per_sm;      /* 0 = automatic */
    uint32_t threads_per_block;  /* multiple of 32, <= 256; 0 = automatic */
    uint32_t flags;              /* LYAP_FLAG_* */
    uint32_t pad_;
    const int32_t *h_seq;        /* optional host copy of d_seq */
} LyapVolumeExt;

/* ---- learned proposal (no reference counterpart) ------------------------
 * A Fourier-feature MLP over the parameter box predicts lambda, so that the
 * march can skip segments the net calls empty (LyapRenderExt.proposal):
 *   u = (P - lo) / (hi - lo);  f = 48 features sin(pi 2^k u_j), cos(pi 2^k u_j)
 *   (k = 0..7, j = 0..2, feature 2*(3k+j) the sine, 2*(3k+j)+1 the cosine);
 *   h1 = gelu(W1 f + b1), h2 = gelu(W2 h1 + b2) (64 each), lambda = w3.h2 + b3;
 *   gelu(x) = x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
 * The two matrix products run on the tensor cores with BF16 operands (f, W1,
 * h1, W2 rounded to nearest-even BF16) and FP32 accumulation; w3 is rounded
 * to BF16 as well, biases and h2 stay FP32.  params holds the FP32 master
 * values: w1[64][48] (row = output), b1[64], w2[64][64], b2[64], w3[64], b3. */
#define LYAP_NET_MAGIC    0x4E50594Cu  /* "LYPN" */
#define LYAP_NET_VERSION  1u
#define LYAP_NET_FEATURES 48
#define LYAP_NET_HIDDEN   64
#define LYAP_NET_PARAMS   7361
typedef struct LyapNet {
    uint32_t magic;              /* LYAP_NET_MAGIC */
    uint32_t version;            /* LYAP_NET_VERSION */
    float lo[3], hi[3];          /* input box */
    float params[LYAP_NET_PARAMS];
    float train_mse;             /* mean batch loss over the last 100 steps */
    float val_mse;               /* on the held-out samples */
    uint32_t steps, batch, n_samples;
    uint32_t seq_hash;           /* FNV-1a 32 of the sequence, settle, accum and d it was trained for */
    uint64_t hash;               /* FNV-1a 64 of every byte before it */
} LyapNet;

/* Training set-up (lyap_net_train); zero fields take the defaults. */
typedef struct {
    uint32_t size;               /* = sizeof(LyapNetTrainOptions) */
    uint32_t n_samples;          /* training samples (0 = 1 << 20) */
    uint32_t n_val;              /* held-out samples (0 = 1 << 16) */
    uint32_t batch;              /* samples per step, multiple of 128, <= 32768 (0 = 4096) */
    uint32_t steps;              /* Adam steps (0 = 8192) */
    float lr;                    /* peak learning rate, cosine decay to 0 (0 = 3e-3) */
    float target_lo, target_hi;  /* lambda clamp; NaN counts as target_lo (both 0: -3, 1) */
    uint64_t seed;
    const float *box_lo;         /* host, 3 floats; NULL = (lMin, lMin, lMin) */
    const float *box_hi;         /* host, 3 floats; NULL = (lMax, lMax, lMax) */
    float *h_loss;               /* optional host array of `steps` floats: each step's batch loss */
} LyapNetTrainOptions;

#ifndef __CUDACC_RTC__   /* host entry points: not part of device-side compiles */
/* ---- entry points ------------------------------------------------------ */

int lyap_abi_version(void);
const char *lyap_version(void);
/* Message of the calling thread's last failure ("" if none). */
const char *lyap_last_error_string(void);
const char *lyap_status_string(int code);

/* scene_convert_sequence (scene.cu:69; declared scene.hpp:11).  Letters A-D
 * (any case) give symbols 0-3, a digit k repeats the previous letter k more
 * times (B before any letter), a -1 terminator is appended.  *len receives
 * the entry count including the -1.  A bad character gives
 * LYAP_ERR_SEQUENCE (the reference exits); a short buffer LYAP_ERR_CAPACITY. */
int lyap_seq_parse(const char *str, int32_t *out, size_t cap, size_t *len);

/* scene_cam_recalculate (scene.cu:31; scene.hpp:13): fills V, S0, SDX, SDY,
 * the render size (texture size / denominator) and the cones of `cam`;
 * tw/th/td of 0 keep the current values. */
int lyap_cam_recalculate(LyapCam *cam, uint32_t tw, uint32_t th, uint32_t td);

/* scene_lights_recalculate (scene.cu:20; scene.hpp:15): axis V and cones. */
int lyap_lights_recalculate(LyapLight *lights, size_t n);

/* kernel_calc_render (kernel.cu:500; launched at lyap_interactive.cu:711)
 * over a width x height image, pixel (x, y) at index x + y*width.  `cam`
 * and `prm` are host structs (by value in the reference); d_seq (seq_len
 * entries incl. the -1), d_lights, d_rgba and d_points are device memory.
 * A hit writes its LyapPoint; a miss writes an all-NaN point and RGBA 0.
 * Colour bytes saturate.  Every row is rendered.  Asynchronous on stream. */
int lyap_render(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points,
                uint32_t width, uint32_t height, const LyapRenderExt *ext, void *stream);

/* kernel_calc_volume (kernel.cu:518; launched at lyap_calculate.cu:72):
 * lambda at (lo + (hi-lo)*i/n) per axis, x fastest, into d_out[nx*ny*nz].
 * lo/hi (3 floats each) may be NULL for the reference's [0, 4).  */
int lyap_volume(float *d_out, uint32_t nx, uint32_t ny, uint32_t nz, const float *lo, const float *hi,
                const LyapParams *prm, const int32_t *d_seq, size_t seq_len, const LyapVolumeExt *ext,
                void *stream);

/* Host-buffer forms of the two above (the reference front-ends' whole
 * round trip: upload, launch, download; lyap_interactive.cu:696-741,
 * lyap_calculate.cu:58-91).  seq / lights are host arrays, outputs are host
 * memory (points may be NULL); returns after the stream is synchronised.
 * lyap_volume_host writes a page-locked output (cudaHostAlloc,
 * cudaHostRegister) in place from the kernel, without a staging copy;
 * other outputs go through device memory. */
int lyap_render_host(const LyapCam *cam, const LyapParams *prm, const int32_t *seq, size_t seq_len,
                     const LyapLight *lights, uint32_t n_lights, RGBA *rgba, LyapPoint *points,
                     uint32_t width, uint32_t height, const LyapRenderExt *ext, void *stream);
int lyap_volume_host(float *out, uint32_t nx, uint32_t ny, uint32_t nz, const float *lo, const float *hi,
                     const LyapParams *prm, const int32_t *seq, size_t seq_len, const LyapVolumeExt *ext,
                     void *stream);

/* The reference's own __global__ entry points (lyap_kernel.hpp) launched
 * with an explicit launch shape, for callers without <<<>>>: exactly
 * kernel_calc_render<<<(grid_x, grid_y), (block_x, block_y)>>>
 * (lyap_interactive.cu:711) and kernel_calc_volume<<<grid, block>>>
 * (lyap_calculate.cu:72), with their index and coordinate conventions
 * (image width / volume extents = grid * block).  Plain FP32.
 * kernel_calc_render takes blocks of at most 256 threads (the reference's
 * 16 x 16); larger ones are LYAP_ERR_INVALID_ARG here (a <<<>>> launch of
 * them fails to launch). */
int lyap_kernel_calc_render(uint32_t grid_x, uint32_t grid_y, uint32_t block_x, uint32_t block_y,
                            RGBA *d_rgba, LyapPoint *d_points, const LyapCam *cam, const LyapParams *prm,
                            int32_t *d_seq, LyapLight *d_lights, uint32_t n_lights, void *stream);
int lyap_kernel_calc_volume(const uint32_t grid[3], const uint32_t block[3], float *d_exps,
                            const LyapParams *prm, int32_t *d_seq, void *stream);

/* ---- batches: many renders in one launch -------------------------------
 * No reference counterpart beyond kernel_calc_render itself: the reference
 * renders one frame per launch (lyap_interactive.cu:711) and sweeps by
 * re-running the program (scale.pl).  A batch holds requests of any image
 * size, parameters, sequence (period <= LYAP_MAX_SEQ_LEN - 1) and light set;
 * lyap_batch_create checks them, orders their tiles longest-job-first,
 * optionally times candidate launch shapes on a sample of the batch (tile
 * 32x1 / 8x4 / 16x16, 1 or 4 tiles per claim, 3 or 4 blocks per SM) and
 * captures one CUDA graph that lyap_batch_run replays on any stream.  Each
 * request's outputs are exactly what lyap_render gives for it. */
typedef struct {
    LyapCam cam;                  /* recalculated camera */
    LyapParams prm;
    const int32_t *d_seq;         /* device, seq_len entries incl. the -1 */
    const LyapLight *d_lights;    /* device, recalculated */
    RGBA *d_rgba;                 /* device, width*height */
    LyapPoint *d_points;          /* device, width*height */
    uint32_t *d_counts;           /* optional, 3 per pixel */
    uint32_t seq_len, n_lights, width, height;
    uint32_t light_model;         /* LYAP_LIGHT_* */
    uint32_t flags;               /* LYAP_FLAG_NO_SPECULATION */
} LyapRequest;

typedef struct {
    uint32_t size;                /* = sizeof(LyapBatchOptions) */
    uint32_t variant;             /* LYAP_VARIANT_* for every request */
    uint32_t autotune;            /* 1: time the candidate launch shapes */
    uint32_t tile_w, tile_h, tiles_per_chunk, blocks_per_sm;   /* used when autotune = 0 */
    uint32_t flags;               /* LYAP_FLAG_NO_JIT: every request on the library's
                                     kernel, none compiled for its sequence */
    unsigned long long *d_stats;  /* optional device LYAP_STAT_COUNT array */
    uint32_t jit_groups;          /* at most this many sequence groups get a kernel
                                     compiled for them (0: LYAP_BATCH_JIT_GROUPS_DEFAULT;
                                     at most LYAP_BATCH_JIT_GROUPS_MAX).  A caller built
                                     without this field passes size =
                                     offsetof(LyapBatchOptions, jit_groups). */
} LyapBatchOptions;

/* Requests with the same sequence (and settle count mod its period) form a
 * group; the batch kernel is compiled at run time (NVRTC, parallel host
 * threads, cached for the process) for the heaviest groups that carry at
 * least 1/1000 of the batch's estimated cost, and each such group runs as a
 * launch of its own in the batch's graph; the other requests run the
 * library's kernel.  A batch of one sequence is one specialised launch. */
#define LYAP_BATCH_JIT_GROUPS_DEFAULT 255u
#define LYAP_BATCH_JIT_GROUPS_MAX 255u

typedef struct {
    uint32_t size, requests, chunks;
    uint32_t tile_w, tile_h, tiles_per_chunk, blocks_per_sm, threads_per_block;
    uint32_t candidates;
    uint32_t specialised;         /* requests run by kernels compiled for their
                                     sequence at run time (all of them for a batch of
                                     one sequence; 0 with LYAP_FLAG_NO_JIT) */
    float tuned_ms[16];           /* time of each candidate on the sample */
} LyapBatchInfo;

typedef struct LyapBatch LyapBatch;

int lyap_batch_create(const LyapRequest *reqs, uint32_t n, const LyapBatchOptions *opt, LyapBatch **out);
int lyap_batch_run(LyapBatch *batch, void *stream);
int lyap_batch_info(const LyapBatch *batch, LyapBatchInfo *info);
int lyap_batch_destroy(LyapBatch *batch);

/* lyap4d (kernel.cu:108-154) at n arbitrary points: d_xyz holds x, y, z per
 * point (device, 3*n floats), symbol D takes prm->d; d_out receives n
 * lambdas in the form `form` (LYAP_VARIANT_PLAIN, LYAP_VARIANT_PRODUCT, or
 * LYAP_FORM_F64: the double-precision evaluator of the precision form's
 * bisection, whose orbit is the reference's DOUBLE_REALS arithmetic).
 * d_out is float[n], or double[n] for LYAP_FORM_F64. */
#define LYAP_FORM_F64 2u
int lyap_lambda_points(const float *d_xyz, size_t n, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                       uint32_t form, void *d_out, void *stream);

/* lyap_render without any device allocation.  It has no counterpart in the
 * reference (whose front-ends cudaMalloc everything up front).  For callers
 * that cannot allocate per call: devices or drivers without stream-ordered
 * memory pools (where lyap_render's stream-ordered allocation of its
 * scratch -- the queue counter and the list of rays that meet the box --
 * fails), applications that own all device memory and forbid
 * library allocations, loops that must not risk a failing or blocking
 * allocation mid-frame.  Same arguments and the same images as lyap_render
 * with the precompiled kernels: it always launches those (it ignores
 * ext->h_seq, and LYAP_FLAG_REQUIRE_JIT returns LYAP_ERR_INVALID_ARG), and it
 * refuses the learned proposal and LYAP_FLAG_BISECT_F64, which need
 * per-pixel scratch.  The caller still passes all inputs and outputs.  The
 * scratch is a static
 * device array of LYAP_NOALLOC_SCRATCH_BYTES per device (held until the
 * library is unloaded), of which a call uses 4 bytes, zeroed on `stream`
 * before the launch; images are limited to LYAP_MAX_PIXELS (larger sizes
 * return LYAP_ERR_INVALID_ARG).  All calls share that array: calls whose
 * work overlaps on the GPU race and corrupt each other's images, so
 * serialise them.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current and keeps it for
 * the life of the process; make that first call before any stream capture,
 * and do not call this entry point on a device after cudaDeviceReset there
 * (the kept address then belongs to the destroyed context). */
#define LYAP_NOALLOC_SCRATCH_BYTES 256
int lyap_render_noalloc(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                        const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points,
                        uint32_t width, uint32_t height, const LyapRenderExt *ext, void *stream);

/* State of the run-time specialisation (no reference counterpart): writes a
 * one-line description (NVRTC loaded or why not, compiles, launches, cached
 * sequences, the last compile errors) into buf; returns 1 if NVRTC loaded. */
int lyap_jit_info(char *buf, size_t cap);

/* Measurement support (no reference counterpart): a pipe-rate probe whose
 * launch the caller times.  kind 0 = dependent-chain-free FFMA, kind 1 =
 * lg2.approx, kind 2 = packed FFMA2 (fma.rn.f32x2, two FMAs per lane);
 * *ops receives the operations performed.  The rate is the denominator of
 * the lambda kernels' FP32 / MUFU roofline. */
int lyap_pipe_probe(uint32_t kind, uint32_t iters, float *d_sink, double *ops, void *stream);

/* ---- DOUBLE_REALS render mode ------------------------------------------ */
/* The reference built with -DDOUBLE_REALS (structs.hpp:10-14, Real =
 * double): scene_cam_recalculate / scene_lights_recalculate on the double
 * structs (bit-identical to that build's host code), and kernel_calc_render
 * with every Real in double on the GPU (lambda's log sum as a renormalised
 * double product, within ~1e-13 relative of one log per step).  d_counts
 * (optional, 3 per pixel) receives march / honing / normal samples;
 * light_model is LYAP_LIGHT_*.  FP64 is this GPU's slow path: the mode is
 * for precision work.  Asynchronous on stream. */
int lyap_cam_recalculate_d(LyapCamD *cam, uint32_t tw, uint32_t th, uint32_t td);
int lyap_lights_recalculate_d(LyapLightD *lights, size_t n);
int lyap_render_d(const LyapCamD *cam, const LyapParamsD *prm, const int32_t *d_seq, size_t seq_len,
                  const LyapLightD *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPointD *d_points, uint32_t width,
                  uint32_t height, uint32_t light_model, uint32_t *d_counts, void *stream);

/* ---- preset, animation path and output files (host only) -------------- */
/* params_init (params.cu:21-114): the reference's preset parameters, camera
 * (before scene_cam_recalculate), light(s), sequence string ("BCABA") and
 * default image size (3840x2160), bit-identical to its host build.  Every
 * output pointer may be NULL; lights needs light_cap >= 1 (one light is
 * written, *n_lights = 1).  The _d form is the DOUBLE_REALS build. */
int lyap_params_init(LyapParams *prm, LyapCam *cam, LyapLight *lights, uint32_t light_cap, uint32_t *n_lights,
                     char *seq, size_t seq_cap, uint32_t *width, uint32_t *height);
int lyap_params_init_d(LyapParamsD *prm, LyapCamD *cam, LyapLightD *lights, uint32_t light_cap,
                       uint32_t *n_lights, char *seq, size_t seq_cap, uint32_t *width, uint32_t *height);
/* easeInOutQuart of the animation driver (scale.pl:5-11; a quadratic ease). */
double lyap_ease_in_out_quart(double t, double b, double c, double d);
/* The camera params.cu's startcalc block computes for interpolation value i
 * (scale.pl:30-46 substitutes the eased value for params.cu's 1): C and Q
 * only, other fields untouched.  i is first rounded to 15 significant
 * digits, as the driver prints it into the source. */
int lyap_anim_camera(double i, LyapCam *cam);
int lyap_anim_camera_d(double i, LyapCamD *cam);
/* save_ppm (lyap_interactive.cu:570-612): "P3\n<w> <h>\n255\n", then
 * "%3d %3d %3d " per pixel in memory order, then "\n"; binary != 0 writes
 * P6 instead (an extension).  rgba is host memory. */
int lyap_write_ppm(const char *path, const RGBA *rgba, uint32_t width, uint32_t height, int binary);
/* save_points (lyap_interactive.cu:617-652): the LyapPoint array's bytes. */
int lyap_write_points(const char *path, const LyapPoint *points, size_t n);
/* lyap_calculate.cu:84-86 (exps.raw): the float volume's bytes, x fastest. */
int lyap_write_exps(const char *path, const float *values, size_t n);
/* The reference's output file name (lyap_interactive.cu:576-604):
 * "<kind>_<stamp>_<w>x<h>_<seq>_cx=.._cy=.._cz=.._step=.._D=.._i=<settle>,
 * <accum>_d=<depth>_j=.._r=<refine>_ot=.._time=<h>h<mm>m<ss>s.<ext>", kind
 * "Render" or "Points", cut to 254 characters as the reference's buffers do. */
int lyap_output_name(char *buf, size_t cap, const char *kind, long stamp, uint32_t width, uint32_t height,
                     const char *seq, const LyapCam *cam, const LyapParams *prm, uint32_t elapsed_s, const char *ext);

/* ---- learned proposal entry points (no reference counterpart) ----------- */
/* Trains `net` on the GPU: n_samples + n_val points uniform in the box,
 * lambda at each by the plain FP32 method for this sequence and parameters
 * (the drop-in's own lyap4d), clamped; then `steps` Adam steps of mean
 * squared error on random batches, each a forward and backward pass on the
 * tensor cores.  seq is a host array (seq_len entries incl. the -1).
 * Deterministic for a given seed.  Returns after the stream is synchronised. */
int lyap_net_train(const LyapParams *prm, const int32_t *seq, size_t seq_len, const LyapNetTrainOptions *opt,
                   LyapNet *net, void *stream);
/* The learned proposal's grid as lyap_render reads it: n^3 cells (x
 * fastest) over the net's box, each the minimum of the net at the cell's 8
 * corners (a NaN corner gives -inf), with dilate the minimum over the 27
 * cells around it, into d_out[n^3] (device).  n = 0 takes
 * LYAP_PROPOSAL_GRID_DEFAULT; 2..512.  Builds the grid on `stream` and caches
 * it (as lyap_render does) if it is not cached yet. */
int lyap_net_grid(const LyapNet *net, uint32_t n, uint32_t dilate, float *d_out, void *stream);
/* The net at n points (d_xyz: 3 floats per point, device) into d_out[n]
 * (device), on the tensor cores.  Asynchronous. */
int lyap_net_eval(const LyapNet *net, const float *d_xyz, size_t n, float *d_out, void *stream);
/* Gradient of the loss (1/n) sum_i (net(x_i) - t_i)^2 with respect to
 * params, by the training kernels (forward and backward on the tensor
 * cores): d_grad receives LYAP_NET_PARAMS floats, d_loss (may be NULL) the
 * loss.  n is a multiple of 128, at most 32768.  Asynchronous. */
int lyap_net_grad(const LyapNet *net, const float *d_xyz, const float *d_target, size_t n, float *d_grad,
                  float *d_loss, void *stream);
/* The net as a file (the struct's bytes) and back; load checks magic,
 * version and hash. */
int lyap_net_save(const LyapNet *net, const char *path);
int lyap_net_load(LyapNet *net, const char *path);

#endif /* !__CUDACC_RTC__ */

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LYAP_GB300_H */
