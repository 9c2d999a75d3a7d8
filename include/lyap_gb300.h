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

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LYAP_GB300_H */
