// lyap_jobs.h -- the kernel parameter blocks (host and device, nvcc and NVRTC).
#pragma once

#include <stdint.h>

#include "lyap_gb300.h"

namespace lyapgb {

// One frame to render: everything kernel_calc_render receives (kernel.cu:500)
// plus the image size, the light model and optional outputs.
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
    uint32_t flags;              // LYAP_FLAG_* (LYAP_FLAG_NO_SPECULATION is read here)
};

struct VolumeJob {
    float *out;                  // device, nx*ny*nz, x fastest
    const int32_t *seq;
    LyapParams prm;
    uint32_t seq_period;
    uint32_t nx, ny, nz;
    float lo[3], hi[3];
};

}  // namespace lyapgb
