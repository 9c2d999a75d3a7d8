/*
 * lyap_oracle.h -- the ORACLE: a plain-C restatement of the reference's hot
 * path (kernel.cu, scene.cu, vec3.hpp, quat.hpp, color.hpp), used ONLY as the
 * checker by tests/, __graft_entry__.smoke() and the CPU-baseline legs of
 * bench.py.  The product (lyapunov3d_gb300/) never links or calls it.
 *
 * Parity pin: with lambda mode ORC_REF the restatement is bit-exact against
 * the reference compiled as host C++ (oracle/Makefile target `ref`), and the
 * *_d functions against its DOUBLE_REALS build; tests/golden/ holds the
 * fixtures that pin it and the script that made them.
 *
 * Where the product deliberately defines behaviour the reference leaves
 * undefined, the oracle implements the product's definition:
 *   H3  a miss writes a point of all-NaN bytes (0xFF) instead of leaving it
 *       unwritten; shade() of it gives RGBA 0,0,0,0;
 *   H4  every row of the image is computed (the reference's grid truncates);
 *   H5  the parameter box [lMin, lMax]^3 of LyapParams is honoured (the
 *       reference fixes [0, 4]; with lMin = 0, lMax = 4 the arithmetic is
 *       the reference's, in double as its 0.0 / 4.0 literals make it);
 *   H6  colour -> byte saturates to [0, 255] (NaN -> 0) instead of the
 *       reference's out-of-range conversion;
 *   --  loops are bounded: the march stops after
 *       ceil((t1 - t0) / min(Fdt, Ndt) * 1.001) + 16 samples (at most
 *       ORC_MARCH_MAX) and is then a miss; honing stops after ORC_HONE_CAP
 *       samples.  Neither bound is reached on any
 *       input where the reference itself terminates normally.
 */
#ifndef LYAP_ORACLE_H
#define LYAP_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "lyap_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* How lambda at a sample point is computed. */
enum {
    ORC_REF = 0,     /* reference host FP32 arithmetic (kernel.cu:108-154) with
                        its double promotions and libm logf */
    ORC_PLAIN = 1,   /* the product's plain FP32 arithmetic: fma orbit,
                        sum of log2 (libm log2f), times ln2 / accum */
    ORC_PRODUCT = 2  /* the product's precision form: running FP32 product of
                        |r(1-2x)| renormalised to [2^100, 2^101) by exponent
                        extraction every 8 steps, one log2 at the end */
};

#define ORC_HONE_CAP 256
#define ORC_MARCH_MAX 4194304u

int orc_abi_version(void);

/* scene.cu:69-108; returns 0, -2 on a bad letter / empty string, -6 when
 * `cap` is too small.  *len = entries written including the -1. */
int orc_seq_parse(const char *s, int32_t *out, size_t cap, size_t *len);

/* scene.cu:20-63 */
void orc_cam_recalculate(LyapCam *cam, uint32_t tw, uint32_t th, uint32_t td);
void orc_lights_recalculate(LyapLight *lights, size_t n);
void orc_cam_recalculate_d(LyapCamD *cam, uint32_t tw, uint32_t th, uint32_t td);
void orc_lights_recalculate_d(LyapLightD *lights, size_t n);

/* lambda at one point; seq is -1 terminated (kernel.cu:108-154). */
float orc_lyap4d(int mode, float x, float y, float z, float d,
                 uint32_t settle, uint32_t accum, const int32_t *seq);
double orc_lyap4d_d(double x, double y, double z, double d,
                    uint32_t settle, uint32_t accum, const int32_t *seq);

/* lambda at n points (x, y, z, d per point), OpenMP-parallel. mode < 0
 * selects the double-precision form. */
void orc_lyap4d_batch(int mode, const double *pts, size_t n, uint32_t settle,
                      uint32_t accum, const int32_t *seq, double *out);

/* kernel_calc_volume (kernel.cu:488-532) over an nx*ny*nz grid, x fastest,
 * coordinate lo + ((hi - lo) * i) / n per axis (lo/hi NULL: [0, 4)). */
void orc_volume(int mode, float *out, uint32_t nx, uint32_t ny, uint32_t nz,
                const float *lo, const float *hi, const LyapParams *prm,
                const int32_t *seq);
void orc_volume_d(double *out, uint32_t nx, uint32_t ny, uint32_t nz,
                  const float *lo, const float *hi, const LyapParamsD *prm,
                  const int32_t *seq);

/* raymarch (kernel.cu:156-486) for pixel (sx, sy).  Returns 0 on a hit,
 * 1 on a miss; writes *pt on a hit only (as the reference).  counts, if not
 * NULL, receives {march samples, honing samples, normal samples}. */
int orc_raymarch(int mode, LyapPoint *pt, uint32_t sx, uint32_t sy,
                 const LyapCam *cam, const LyapParams *prm,
                 const int32_t *seq, uint32_t *counts);
int orc_raymarch_d(LyapPointD *pt, uint32_t sx, uint32_t sy,
                   const LyapCamD *cam, const LyapParamsD *prm,
                   const int32_t *seq, uint32_t *counts);

/* shade (kernel.cu:25-106); color[4] = pre-quantisation colour. */
void orc_shade(const LyapPoint *pt, const LyapCam *cam, const LyapLight *lights,
               uint32_t n_lights, float *color, RGBA *rgba);

/* kernel_calc_render (kernel.cu:500-516) over a w*h image, index x + y*w;
 * misses get an all-NaN point.  counts (3 per pixel) may be NULL. */
void orc_render(int mode, RGBA *rgba, LyapPoint *points, const LyapCam *cam,
                const LyapParams *prm, const int32_t *seq,
                const LyapLight *lights, uint32_t n_lights, uint32_t w,
                uint32_t h, uint32_t *counts);
void orc_render_rows(int mode, RGBA *rgba, LyapPoint *points,
                     const LyapCam *cam, const LyapParams *prm,
                     const int32_t *seq, const LyapLight *lights,
                     uint32_t n_lights, uint32_t w, uint32_t y0, uint32_t y1,
                     uint32_t *counts);

/* The product's learned-proposal march (not the reference's: it has no
 * proposal), restated so that the GPU's proposal path has a checker: a
 * grid of n^3 cells (x fastest) over the box lo + [0, n / scale) with a
 * lower bound of the net's lambda per cell (lyap_net_grid writes it), the
 * skip / confirm threshold tau and the longest skipped run. */
typedef struct {
    const float *grid;
    uint32_t n, run;
    float lo[3], scale[3];
    float tau;
} OrcProposal;

/* orc_raymarch with the proposal; counts[0] = evaluated march samples,
 * pcounts[0..1] = skipped positions, rewound runs (either may be NULL). */
int orc_raymarch_prop(int mode, LyapPoint *pt, uint32_t sx, uint32_t sy,
                      const LyapCam *cam, const LyapParams *prm,
                      const int32_t *seq, const OrcProposal *prop,
                      uint32_t *counts, uint32_t *pcounts);
/* orc_render_rows with the proposal (prop NULL: orc_render_rows);
 * pcounts: 2 per pixel, may be NULL. */
void orc_render_rows_prop(int mode, RGBA *rgba, LyapPoint *points,
                          const LyapCam *cam, const LyapParams *prm,
                          const int32_t *seq, const LyapLight *lights,
                          uint32_t n_lights, uint32_t w, uint32_t y0, uint32_t y1,
                          const OrcProposal *prop, uint32_t *counts, uint32_t *pcounts);

/* Threads the OpenMP loops use (0 = runtime default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
