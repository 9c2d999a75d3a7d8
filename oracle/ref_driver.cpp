/*
 * ref_driver.cpp -- extern "C" entry points over the reference's own code,
 * compiled as host C++ (see ref_shim.h and oracle/Makefile, target `ref`).
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement
 * (oracle/lyap_oracle.c) and to generate the golden fixtures under
 * tests/golden/.  It never ships and is never what a benchmark measures.
 *
 * Built twice: Real = float (the reference default) and Real = double
 * (-DDOUBLE_REALS=1, structs.hpp:10-18).  Structs cross this boundary as raw
 * bytes in the reference's own layout; the Python side describes them.
 *
 * The "launches" run the reference's __global__ functions on host threads:
 * for every (block, thread) of the grid the built-in coordinates are set and
 * kernel_calc_render (kernel.cu:500) / kernel_calc_volume (kernel.cu:518) is
 * called as an ordinary function.
 */
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <cstdlib>

#include "kernel.hpp"
#include "scene.hpp"
#include "params.hpp"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

/* Defined in kernel.cu; kernel.hpp declares the never-defined `raycast`
 * instead (kernel.hpp:15 vs kernel.cu:156). */
Int raymarch(LyapPoint *point, Uint sx, Uint sy, LyapCam cam, LyapParams prm, Int *seq);
Real pointcalc(Real a, Real b, Real c, LyapParams prm, Int *seq);
/* kernel.hpp:19 declares Real* but kernel.cu:518 defines float*. */
void kernel_calc_volume(float *exps, LyapParams prm, Int *seq);

#define OFF(T, f) ((long long)offsetof(T, f))

extern "C" {

int ref_real_bytes(void) { return (int)sizeof(Real); }

/* sizeof and field offsets of every ABI struct, in a fixed order:
 *   [0] sizeof(LyapCam) [1] alignof(LyapCam) then 22 LyapCam field offsets,
 *   [24] sizeof(LyapParams) then 14 offsets, [39] sizeof(LyapPoint) then 5
 *   offsets, [45] sizeof(RGBA). */
int ref_layout(long long *out, int cap)
{
    long long v[] = {
        (long long)sizeof(LyapCam), (long long)alignof(LyapCam),
        OFF(LyapCam, C), OFF(LyapCam, Q), OFF(LyapCam, M), OFF(LyapCam, V),
        OFF(LyapCam, S0), OFF(LyapCam, SDX), OFF(LyapCam, SDY),
        OFF(LyapCam, textureWidth), OFF(LyapCam, textureHeight),
        OFF(LyapCam, renderWidth), OFF(LyapCam, renderHeight),
        OFF(LyapCam, renderDenominator), OFF(LyapCam, lightInnerCone),
        OFF(LyapCam, lightOuterCone), OFF(LyapCam, lightRange),
        OFF(LyapCam, ambient), OFF(LyapCam, diffuseColor),
        OFF(LyapCam, diffusePower), OFF(LyapCam, specularColor),
        OFF(LyapCam, specularPower), OFF(LyapCam, specularHardness),
        OFF(LyapCam, chaosColor),
        (long long)sizeof(LyapParams),
        OFF(LyapParams, d), OFF(LyapParams, settle), OFF(LyapParams, accum),
        OFF(LyapParams, stepMethod), OFF(LyapParams, nearThreshold),
        OFF(LyapParams, nearMultiplier), OFF(LyapParams, opaqueThreshold),
        OFF(LyapParams, chaosThreshold), OFF(LyapParams, depth),
        OFF(LyapParams, jitter), OFF(LyapParams, refine),
        OFF(LyapParams, gradient), OFF(LyapParams, lMin), OFF(LyapParams, lMax),
        (long long)sizeof(LyapPoint),
        OFF(LyapPoint, P), OFF(LyapPoint, N), OFF(LyapPoint, a),
        OFF(LyapPoint, c), OFF(LyapPoint, l),
        (long long)sizeof(RGBA),
    };
    int n = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < n && i < cap; i++) out[i] = v[i];
    return n;
}

/* scene_convert_sequence (scene.cu:69); returns the length including the -1
 * terminator, copies at most `cap` entries. */
size_t ref_seq_parse(const char *s, int *out, size_t cap)
{
    Int *seq = nullptr;
    size_t n = scene_convert_sequence(&seq, (unsigned char *)s);
    for (size_t i = 0; i < n && i < cap; i++) out[i] = seq[i];
    free(seq);
    return n;
}

/* params_init (params.cu:21) and a copy of its globals. */
void ref_params_init(void *prm_out, void *cam_out, void *lights_out,
                     unsigned *nl, char *seq_out, size_t seq_cap,
                     unsigned *def_w, unsigned *def_h)
{
    params_init();
    memcpy(prm_out, &prm, sizeof(LyapParams));
    memcpy(cam_out, &cam, sizeof(LyapCam));
    memcpy(lights_out, lights, sizeof(LyapLight) * MAX_LIGHTS);
    *nl = num_lights;
    if (seq_cap) {
        strncpy(seq_out, (const char *)sequence, seq_cap - 1);
        seq_out[seq_cap - 1] = 0;
    }
    *def_w = default_imageWidth;
    *def_h = default_imageHeight;
}

void ref_cam_recalculate(void *cam_io, unsigned tw, unsigned th, unsigned td)
{
    scene_cam_recalculate((LyapCam *)cam_io, tw, th, td);
}

void ref_lights_recalculate(void *lights_io, size_t n)
{
    scene_lights_recalculate((LyapLight *)lights_io, n);
}

/* lyap4d (kernel.cu:108) at n points; pts holds (x, y, z, d) per point. */
void ref_lyap4d(const double *pts, size_t n, unsigned settle, unsigned accum,
                const int *seq, double *out)
{
    #pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; i++) {
        Vec P((Real)pts[4 * i + 0], (Real)pts[4 * i + 1], (Real)pts[4 * i + 2]);
        out[i] = (double)lyap4d(P, (Real)pts[4 * i + 3], settle, accum, seq);
    }
}

/* raymarch (kernel.cu:156) for one pixel; returns its 0 = hit / 1 = miss. */
int ref_raymarch(void *point_io, unsigned sx, unsigned sy, const void *cam,
                 const void *prm_in, const int *seq)
{
    return raymarch((LyapPoint *)point_io, sx, sy, *(const LyapCam *)cam,
                    *(const LyapParams *)prm_in, (Int *)seq);
}

/* shade (kernel.cu:25) + to_rgba (color.hpp:169) of one point. */
void ref_shade(const void *point, const void *cam, const void *lights_in,
               unsigned nl, double *color_out, unsigned char *rgba_out)
{
    Color c = shade(*(const LyapPoint *)point, *(const LyapCam *)cam,
                    (LyapLight *)lights_in, nl);
    color_out[0] = c.x; color_out[1] = c.y; color_out[2] = c.z; color_out[3] = c.w;
    c.to_rgba(rgba_out);
}

/* kernel_calc_render<<<(gw, gh), (bw, bh)>>> run on host threads. The caller
 * pre-fills `points` (the reference leaves a miss's point unwritten). */
void ref_render(void *rgba, void *points, const void *cam, const void *prm_in,
                const int *seq, const void *lights_in, unsigned nl,
                unsigned gw, unsigned gh, unsigned bw, unsigned bh)
{
    LyapCam c = *(const LyapCam *)cam;
    LyapParams p = *(const LyapParams *)prm_in;
    long long nblocks = (long long)gw * gh;
    #pragma omp parallel for schedule(dynamic, 1)
    for (long long b = 0; b < nblocks; b++) {
        gridDim = dim3(gw, gh, 1);
        blockDim = dim3(bw, bh, 1);
        blockIdx.x = (unsigned)(b % gw);
        blockIdx.y = (unsigned)(b / gw);
        blockIdx.z = 0;
        for (unsigned ty = 0; ty < bh; ty++)
            for (unsigned tx = 0; tx < bw; tx++) {
                threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = 0;
                kernel_calc_render((RGBA *)rgba, (LyapPoint *)points, c, p,
                                   (Int *)seq, (LyapLight *)lights_in, nl);
            }
    }
}

/* kernel_calc_volume<<<(n/bs)^3, (bs)^3>>> run on host threads. */
void ref_volume(float *out, const void *prm_in, const int *seq, unsigned n,
                unsigned bs)
{
    LyapParams p = *(const LyapParams *)prm_in;
    unsigned g = n / bs;
    long long nblocks = (long long)g * g * g;
    #pragma omp parallel for schedule(dynamic, 1)
    for (long long b = 0; b < nblocks; b++) {
        gridDim = dim3(g, g, g);
        blockDim = dim3(bs, bs, bs);
        blockIdx.x = (unsigned)(b % g);
        blockIdx.y = (unsigned)((b / g) % g);
        blockIdx.z = (unsigned)(b / ((long long)g * g));
        for (unsigned tz = 0; tz < bs; tz++)
            for (unsigned ty = 0; ty < bs; ty++)
                for (unsigned tx = 0; tx < bs; tx++) {
                    threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
                    kernel_calc_volume(out, p, (Int *)seq);
                }
    }
}

} /* extern "C" */
