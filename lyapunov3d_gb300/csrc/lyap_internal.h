// lyap_internal.h -- host/device shared declarations of the library (not
// part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_gb300.h"

namespace lyapgb {

// One frame to render: everything kernel_calc_render receives (kernel.cu:500)
// plus the image size, the lambda form and optional outputs.
struct RenderJob {
    LyapCam cam;                 // already recalculated (scene_cam_recalculate)
    LyapParams prm;
    const int32_t *seq;          // device, -1 terminated
    const LyapLight *lights;     // device, n_lights entries (recalculated)
    RGBA *rgba;                  // device, width*height
    LyapPoint *points;           // device, width*height
    uint32_t *counts;            // device, 3 per pixel, or null
    uint32_t seq_period;         // entries before the terminator
    uint32_t n_lights;
    uint32_t width, height;
    uint32_t light_model;        // LYAP_LIGHT_SPOT | LYAP_LIGHT_DIRECTIONAL
    uint32_t pad_;
};

struct VolumeJob {
    float *out;                  // device, nx*ny*nz, x fastest
    const int32_t *seq;
    LyapParams prm;
    uint32_t seq_period;
    uint32_t nx, ny, nz;
    float lo[3], hi[3];
};

// kernels launchers (lyap_render.cu, lyap_volume.cu); return a cudaError_t
cudaError_t launch_render(const RenderJob &job, uint32_t mode, uint32_t *d_work_counter,
                          unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads,
                          cudaStream_t stream);
cudaError_t launch_volume(const VolumeJob &job, uint32_t mode, unsigned long long *d_stats,
                          uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream);

// per-device SM count (cached)
int device_sm_count();

// argument checks and job assembly shared by the render entry points (lyap_capi.cu)
int check_render_args(const LyapCam *cam, const LyapParams *prm, const void *seq, size_t seq_len,
                      const void *lights, uint32_t n_lights, const void *rgba, const void *points,
                      uint32_t width, uint32_t height, const LyapRenderExt *ext, const char *fn);
RenderJob make_job(const LyapCam *cam, const LyapParams *prm, const int32_t *d_seq, size_t seq_len,
                   const LyapLight *d_lights, uint32_t n_lights, RGBA *d_rgba, LyapPoint *d_points,
                   uint32_t width, uint32_t height, const LyapRenderExt *ext);

// error reporting (lyap_capi.cu)
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);

}  // namespace lyapgb
