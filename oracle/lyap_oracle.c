/*
 * lyap_oracle.c -- the ORACLE (test infrastructure only; see lyap_oracle.h).
 *
 * A plain-C restatement of the reference's hot path, written from its
 * behaviour: lyap4d (kernel.cu:108-154), raymarch (kernel.cu:156-486), shade
 * (kernel.cu:25-106), kernel_calc_render / kernel_calc_volume
 * (kernel.cu:488-532), scene_convert_sequence / scene_cam_recalculate /
 * scene_lights_recalculate (scene.cu:20-108).  Pinned bit-exact against the
 * reference's own code built as host C++ (oracle/Makefile target `ref`;
 * fixtures in tests/golden/).
 *
 * Besides the reference's arithmetic (ORC_REF) it emulates the product's
 * two FP32 lambda forms (ORC_PLAIN, ORC_PRODUCT) exactly except for the
 * logarithm: libm log2f here, the GPU's lg2.approx there.  The iterated
 * orbit does not depend on the logarithm, so those forms reproduce the
 * product's orbit bit for bit.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "lyap_oracle.h"

#define LN2F 0.693147180559945309417232121458f

int orc_abi_version(void) { return LYAP_ABI_VERSION; }

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n > 0 ? n : 0; }
int orc_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#ifdef _OPENMP
#define OMP_THREADS num_threads(orc_get_threads())
#else
#define OMP_THREADS
#endif

/* ---- scene_convert_sequence (scene.cu:69-108) --------------------------
 * Letters A-D (any case) append symbol 0-3 and become `last`; a digit k
 * appends k further copies of `last` (which starts as B = 1, scene.cu:78);
 * a -1 terminator follows.  The reference exits on any other character,
 * including '0' and an empty string (its do-while inspects the NUL); here
 * those return -2. */
int orc_seq_parse(const char *s, int32_t *out, size_t cap, size_t *len)
{
    if (!s || !out || !len) return LYAP_ERR_INVALID_ARG;
    size_t n = 0;
    int last = 1;
    const unsigned char *p = (const unsigned char *)s;
    do {
        unsigned ch = *p;
        int reps = 0, sym = -1;
        if (ch >= '1' && ch <= '9') reps = (int)(ch - '0');
        else if (ch == 'a' || ch == 'A') sym = 0;
        else if (ch == 'b' || ch == 'B') sym = 1;
        else if (ch == 'c' || ch == 'C') sym = 2;
        else if (ch == 'd' || ch == 'D') sym = 3;
        else return LYAP_ERR_SEQUENCE;
        if (sym >= 0) { last = sym; reps = 1; }
        for (int k = 0; k < reps; k++) {
            if (n + 1 >= cap) return LYAP_ERR_CAPACITY;
            out[n++] = last;
        }
    } while (*(++p));
    if (n + 1 > cap) return LYAP_ERR_CAPACITY;
    out[n++] = -1;
    *len = n;
    return LYAP_OK;
}

/* ---- lambda ------------------------------------------------------------ */

/* Reference host arithmetic (kernel.cu:108-154 with Real = float): the
 * literals 1.0 and 2.0 make the map's products double; logf per step; the
 * NaN return fires on the first non-finite partial sum. */
static float lyap_ref_f(float x, float y, float z, float d, uint32_t settle,
                        uint32_t accum, const int32_t *seq)
{
    float abcd[4] = {x, y, z, d};
    uint32_t seqi = 0, n;
    float r, v = 0.5, l = 0;
    for (n = 0; n < settle; n++) {
        r = abcd[seq[seqi++]];
        if (seq[seqi] == -1) seqi = 0;
        v = r * v * (1.0 - v);
    }
    if ((v - 0.5 <= -1e-8) || (v - 0.5 >= 1e-8)) {
        for (n = 0; n < accum; n++) {
            r = abcd[seq[seqi++]];
            if (seq[seqi] == -1) seqi = 0;
            v = r * v * (1.0 - v);
            r = r - 2.0 * r * v;
            if (r < 0) r = -r;
            l += logf(r);
            if (!isfinite(l)) return NAN;
        }
    }
    return l / (float)accum;
}

/* The product's plain FP32 form.  One step: t = r*x; x = fma(-t, x, t)
 * (= r x (1-x) rounded once); d = fma(-2r, x, r) (= r (1-2x) rounded once);
 * sum += log2|d|.  lambda = (sum * ln2) / accum; a non-finite sum gives NaN.
 * The settle result x skips accumulation exactly when x == 0.5 or NaN,
 * which is the reference's |x - 0.5| < 1e-8 test for a float x. */
static float lyap_plain_f(float x, float y, float z, float d, uint32_t settle,
                          uint32_t accum, const int32_t *seq)
{
    float abcd[4] = {x, y, z, d};
    uint32_t seqi = 0, n;
    float r, t, v = 0.5f, l2 = 0.0f;
    for (n = 0; n < settle; n++) {
        r = abcd[seq[seqi++]];
        if (seq[seqi] == -1) seqi = 0;
        t = r * v;
        v = fmaf(-t, v, t);
    }
    if (v < 0.5f || v > 0.5f) {
        for (n = 0; n < accum; n++) {
            r = abcd[seq[seqi++]];
            if (seq[seqi] == -1) seqi = 0;
            t = r * v;
            v = fmaf(-t, v, t);
            float dd = fmaf(-2.0f * r, v, r);
            l2 += log2f(fabsf(dd));
        }
    }
    if (!isfinite(l2)) return NAN;
    return (l2 * LN2F) / (float)accum;
}

/* The product's precision form: p *= |d| each step; after every 8th step
 * (and at the end) the float exponent of p is moved into the integer e and
 * p is reset into [1, 2).  If a block ends with p outside [2^-100, 2^100]
 * (or NaN), an intermediate product may have left the normal range, and the
 * whole sample is recomputed in the plain form. */
/* The product form: |d| multiplied up in blocks of 8 accumulation steps,
 * each block starting at m * 2^100 (m in [1, 2)); at each block end the
 * float exponent moves into an integer.  A block that ends outside
 * [2^-112, 2^127) redoes the sample in the plain form. */
static float lyap_product_f(float x, float y, float z, float d, uint32_t settle,
                            uint32_t accum, const int32_t *seq)
{
    float abcd[4] = {x, y, z, d};
    uint32_t seqi = 0, n;
    float r, t, v = 0.5f, p = 0x1p100f;
    int32_t e = 0;
    int bad = 0;
    for (n = 0; n < settle; n++) {
        r = abcd[seq[seqi++]];
        if (seq[seqi] == -1) seqi = 0;
        t = r * v;
        v = fmaf(-t, v, t);
    }
    if (v < 0.5f || v > 0.5f) {
        for (n = 0; n < accum; n++) {
            r = abcd[seq[seqi++]];
            if (seq[seqi] == -1) seqi = 0;
            t = r * v;
            v = fmaf(-t, v, t);
            float dd = fmaf(-2.0f * r, v, r);
            p = p * fabsf(dd);
            if ((n & 7u) == 7u || n + 1 == accum) {
                uint32_t bits;
                memcpy(&bits, &p, 4);
                int32_t ef = (int32_t)((bits >> 23) & 0xffu);
                if (ef < 15 || ef > 253) bad = 1;
                e += ef - 227;
                bits = (bits & 0x007fffffu) | (227u << 23);
                memcpy(&p, &bits, 4);
            }
        }
    }
    if (bad)
        return lyap_plain_f(x, y, z, d, settle, accum, seq);
    {   /* the mantissa in [1, 2) for the one log2 */
        uint32_t bits;
        memcpy(&bits, &p, 4);
        bits = (bits & 0x007fffffu) | 0x3f800000u;
        memcpy(&p, &bits, 4);
    }
    float l2 = (float)e + log2f(p);
    if (!isfinite(l2)) return NAN;
    return (l2 * LN2F) / (float)accum;
}

float orc_lyap4d(int mode, float x, float y, float z, float d,
                 uint32_t settle, uint32_t accum, const int32_t *seq)
{
    switch (mode) {
    case ORC_PLAIN: return lyap_plain_f(x, y, z, d, settle, accum, seq);
    case ORC_PRODUCT: return lyap_product_f(x, y, z, d, settle, accum, seq);
    default: return lyap_ref_f(x, y, z, d, settle, accum, seq);
    }
}

/* DOUBLE_REALS lyap4d: the same code with Real = double. */
double orc_lyap4d_d(double x, double y, double z, double d, uint32_t settle,
                    uint32_t accum, const int32_t *seq)
{
    double abcd[4] = {x, y, z, d};
    uint32_t seqi = 0, n;
    double r, v = 0.5, l = 0;
    for (n = 0; n < settle; n++) {
        r = abcd[seq[seqi++]];
        if (seq[seqi] == -1) seqi = 0;
        v = r * v * (1.0 - v);
    }
    if ((v - 0.5 <= -1e-8) || (v - 0.5 >= 1e-8)) {
        for (n = 0; n < accum; n++) {
            r = abcd[seq[seqi++]];
            if (seq[seqi] == -1) seqi = 0;
            v = r * v * (1.0 - v);
            r = r - 2.0 * r * v;
            if (r < 0) r = -r;
            l += log(r);
            if (!isfinite(l)) return NAN;
        }
    }
    return l / (double)accum;
}

void orc_lyap4d_batch(int mode, const double *pts, size_t n, uint32_t settle,
                      uint32_t accum, const int32_t *seq, double *out)
{
    #pragma omp parallel for schedule(dynamic, 64) OMP_THREADS
    for (long long i = 0; i < (long long)n; i++) {
        const double *q = pts + 4 * i;
        if (mode < 0)
            out[i] = orc_lyap4d_d(q[0], q[1], q[2], q[3], settle, accum, seq);
        else
            out[i] = (double)orc_lyap4d(mode, (float)q[0], (float)q[1], (float)q[2],
                                        (float)q[3], settle, accum, seq);
    }
}

/* The proposal grid lookup of the product's march (prop_skippable in
 * lyap_device.cuh), in float: cell = (P - lo) * scale, truncated. */
static int orc_prop_skippable(const OrcProposal *p, float x, float y, float z)
{
    const float nf = (float)p->n;
    const float fx = (x - p->lo[0]) * p->scale[0];
    const float fy = (y - p->lo[1]) * p->scale[1];
    const float fz = (z - p->lo[2]) * p->scale[2];
    if (!(fx >= 0.0f && fx < nf && fy >= 0.0f && fy < nf && fz >= 0.0f && fz < nf)) return 0;
    const uint32_t ix = (uint32_t)fx, iy = (uint32_t)fy, iz = (uint32_t)fz;
    return p->grid[((size_t)iz * p->n + iy) * p->n + ix] >= p->tau;
}

/* ---- the two instantiations of oracle_impl.h ---------------------------- */
#define R float
#define SFX(name) name##_f
#define RLOG logf
#define RSQRT sqrtf
#define VEC LyapVec
#define QUAT LyapQuat
#define COLOR LyapColor
#define CAM LyapCam
#define LIGHT LyapLight
#define PARAMS LyapParams
#define POINT LyapPoint
#define LAMBDA(P, d) orc_lyap4d(mode, (P).x, (P).y, (P).z, (d), prm->settle, prm->accum, seq)
#include "oracle_impl.h"
#undef R
#undef SFX
#undef RLOG
#undef RSQRT
#undef VEC
#undef QUAT
#undef COLOR
#undef CAM
#undef LIGHT
#undef PARAMS
#undef POINT
#undef LAMBDA
#undef VEC_EPSILON
#undef QUAT_EPSILON

#define R double
#define SFX(name) name##_d
#define RLOG log
#define RSQRT sqrt
#define VEC LyapVecD
#define QUAT LyapQuatD
#define COLOR LyapColorD
#define CAM LyapCamD
#define LIGHT LyapLightD
#define PARAMS LyapParamsD
#define POINT LyapPointD
#define LAMBDA(P, d) orc_lyap4d_d((P).x, (P).y, (P).z, (d), prm->settle, prm->accum, seq)
#include "oracle_impl.h"

void orc_cam_recalculate(LyapCam *cam, uint32_t tw, uint32_t th, uint32_t td)
{ orc_cam_recalculate_impl_f(cam, tw, th, td); }
void orc_lights_recalculate(LyapLight *lights, size_t n)
{ orc_lights_recalculate_impl_f(lights, n); }
void orc_cam_recalculate_d(LyapCamD *cam, uint32_t tw, uint32_t th, uint32_t td)
{ orc_cam_recalculate_impl_d(cam, tw, th, td); }
void orc_lights_recalculate_d(LyapLightD *lights, size_t n)
{ orc_lights_recalculate_impl_d(lights, n); }

int orc_raymarch(int mode, LyapPoint *pt, uint32_t sx, uint32_t sy,
                 const LyapCam *cam, const LyapParams *prm,
                 const int32_t *seq, uint32_t *counts)
{ return orc_raymarch_impl_f(mode, pt, sx, sy, cam, prm, seq, counts, NULL, NULL); }

int orc_raymarch_prop(int mode, LyapPoint *pt, uint32_t sx, uint32_t sy,
                      const LyapCam *cam, const LyapParams *prm,
                      const int32_t *seq, const OrcProposal *prop,
                      uint32_t *counts, uint32_t *pcounts)
{ return orc_raymarch_impl_f(mode, pt, sx, sy, cam, prm, seq, counts, prop, pcounts); }

int orc_raymarch_d(LyapPointD *pt, uint32_t sx, uint32_t sy,
                   const LyapCamD *cam, const LyapParamsD *prm,
                   const int32_t *seq, uint32_t *counts)
{ return orc_raymarch_impl_d(0, pt, sx, sy, cam, prm, seq, counts, NULL, NULL); }

/* ---- shade (kernel.cu:25-106) and the byte conversion ------------------- */

/* to_rgba (color.hpp:169-175) converts 255.0 * channel in double; out of
 * [0, 256) that is undefined in C++.  Here it saturates (H6); inside the
 * range it truncates exactly like the reference. */
static unsigned char to_byte(double ch)
{
    double v = 255.0 * ch;
    if (!(v > 0.0)) return 0;
    if (v >= 255.0) return 255;
    return (unsigned char)v;
}

void orc_shade(const LyapPoint *pt, const LyapCam *cam, const LyapLight *lights,
               uint32_t n_lights, float *color_out, RGBA *rgba)
{
    LyapColor color = c4_f(0, 0, 0, 0);
    if (isnan(pt->a)) {
        color.x = 0;
        color.w = 0;
    } else {
        for (uint32_t li = 0; li < n_lights; li++) {
            const LyapLight *L = &lights[li];
            LyapVec P = pt->P, N = pt->N;
            float c = pt->c;
            LyapColor diffuse, specular, phong;
            LyapVec camV = vsub_f(cam->C, P);
            LyapVec lightV = vsub_f(L->C, P);
            float lightD2 = vmag2_f(lightV);
            lightV = vnormalized_f(lightV);
            float i = vdot_f(lightV, N);
            float j = vdot_f(lightV, L->V);
            j = -j;
            if (j > L->lightOuterCone) {
                i = clamp01_f(i);
                diffuse = cscale_f(L->diffuseColor, i * L->diffusePower);
                LyapVec halfV = vadd_f(camV, lightV);
                halfV = vnormalized_f(halfV);
                i = clamp01_f(vdot_f(N, halfV));
                i = powf(i, L->specularHardness);
                specular = cscale_f(L->specularColor, i * L->specularPower);
                phong = cscale_f(cadd_f(specular, diffuse), L->lightRange / lightD2);
                if (j < L->lightInnerCone)
                    phong = cscale_f(phong, (j - L->lightOuterCone) / (L->lightInnerCone - L->lightOuterCone));
                phong = cadd_f(phong, L->ambient);
            } else {
                phong = L->ambient;
            }
            if (c > 0.0) {
                LyapColor chaos = cscale_f(L->chaosColor, (float)(0.1125 / logf(c)));
                phong = cadd_f(phong, chaos);
            }
            color = cadd_f(color, phong);
        }
    }
    if (color_out) {
        color_out[0] = color.x; color_out[1] = color.y;
        color_out[2] = color.z; color_out[3] = color.w;
    }
    if (rgba) {
        rgba->r = to_byte(color.x);
        rgba->g = to_byte(color.y);
        rgba->b = to_byte(color.z);
        rgba->a = to_byte(color.w);
    }
}

/* ---- kernel_calc_render (kernel.cu:500-516) ----------------------------- */
void orc_render_rows(int mode, RGBA *rgba, LyapPoint *points,
                     const LyapCam *cam, const LyapParams *prm,
                     const int32_t *seq, const LyapLight *lights,
                     uint32_t n_lights, uint32_t w, uint32_t y0, uint32_t y1,
                     uint32_t *counts)
{
    orc_render_rows_prop(mode, rgba, points, cam, prm, seq, lights, n_lights, w, y0, y1, NULL, counts, NULL);
}

void orc_render_rows_prop(int mode, RGBA *rgba, LyapPoint *points,
                          const LyapCam *cam, const LyapParams *prm,
                          const int32_t *seq, const LyapLight *lights,
                          uint32_t n_lights, uint32_t w, uint32_t y0, uint32_t y1,
                          const OrcProposal *prop, uint32_t *counts, uint32_t *pcounts)
{
    long long n = (long long)w * (long long)(y1 - y0);
    #pragma omp parallel for schedule(dynamic, 16) OMP_THREADS
    for (long long k = 0; k < n; k++) {
        uint32_t x = (uint32_t)(k % w), y = y0 + (uint32_t)(k / w);
        size_t ind = (size_t)x + (size_t)y * w;
        LyapPoint pt;
        uint32_t cnt[3], pc[2];
        if (orc_raymarch_impl_f(mode, &pt, x, y, cam, prm, seq, cnt, prop, pc) != 0)
            memset(&pt, 0xff, sizeof(pt));
        if (pcounts) {
            pcounts[2 * ind + 0] = pc[0];
            pcounts[2 * ind + 1] = pc[1];
        }
        points[ind] = pt;
        orc_shade(&pt, cam, lights, n_lights, NULL, &rgba[ind]);
        if (counts) {
            counts[3 * ind + 0] = cnt[0];
            counts[3 * ind + 1] = cnt[1];
            counts[3 * ind + 2] = cnt[2];
        }
    }
}

void orc_render(int mode, RGBA *rgba, LyapPoint *points, const LyapCam *cam,
                const LyapParams *prm, const int32_t *seq,
                const LyapLight *lights, uint32_t n_lights, uint32_t w,
                uint32_t h, uint32_t *counts)
{
    orc_render_rows(mode, rgba, points, cam, prm, seq, lights, n_lights, w, 0, h, counts);
}

/* ---- kernel_calc_volume (kernel.cu:488-498, 518-532) -------------------- */
static inline float vox_coord(const float *lo, const float *hi, int axis,
                              uint32_t i, uint32_t n)
{
    float l0 = lo ? lo[axis] : 0.0f, h0 = hi ? hi[axis] : 4.0f;
    return l0 + ((h0 - l0) * (float)i) / (float)n;
}

void orc_volume(int mode, float *out, uint32_t nx, uint32_t ny, uint32_t nz,
                const float *lo, const float *hi, const LyapParams *prm,
                const int32_t *seq)
{
    long long rows = (long long)ny * nz;
    #pragma omp parallel for schedule(dynamic, 1) OMP_THREADS
    for (long long rz = 0; rz < rows; rz++) {
        uint32_t y = (uint32_t)(rz % ny), z = (uint32_t)(rz / ny);
        float b = vox_coord(lo, hi, 1, y, ny), c = vox_coord(lo, hi, 2, z, nz);
        for (uint32_t x = 0; x < nx; x++) {
            float a = vox_coord(lo, hi, 0, x, nx);
            out[(size_t)x + ((size_t)y + (size_t)z * ny) * nx] =
                orc_lyap4d(mode, a, b, c, prm->d, prm->settle, prm->accum, seq);
        }
    }
}

void orc_volume_d(double *out, uint32_t nx, uint32_t ny, uint32_t nz,
                  const float *lo, const float *hi, const LyapParamsD *prm,
                  const int32_t *seq)
{
    long long rows = (long long)ny * nz;
    #pragma omp parallel for schedule(dynamic, 1) OMP_THREADS
    for (long long rz = 0; rz < rows; rz++) {
        uint32_t y = (uint32_t)(rz % ny), z = (uint32_t)(rz / ny);
        float b = vox_coord(lo, hi, 1, y, ny), c = vox_coord(lo, hi, 2, z, nz);
        for (uint32_t x = 0; x < nx; x++) {
            float a = vox_coord(lo, hi, 0, x, nx);
            out[(size_t)x + ((size_t)y + (size_t)z * ny) * nx] =
                orc_lyap4d_d(a, b, c, prm->d, prm->settle, prm->accum, seq);
        }
    }
}
