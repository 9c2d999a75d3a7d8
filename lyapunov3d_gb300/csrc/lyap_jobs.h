// lyap_jobs.h -- the kernel parameter blocks (host and device, nvcc and NVRTC).
#pragma once

#include <stdint.h>

#include "lyap_gb300.h"

namespace lyapgb {

// The learned proposal as the march reads it: one bit per cell of an n^3
// grid over the net's box, set when the cell's lower bound of the net's
// lambda is at least tau (opaque threshold + margin).  A march position in a
// set cell may be skipped, at most `run` positions in a row; the sample
// after every run is evaluated exactly and confirms it (prop_form_run and
// ray_advance, lyap_device.cuh).
struct PropGrid {
    const uint32_t *bits;        // device, n^3 bits, cell (x + (y + z n) n) = bit c % 32 of word c / 32; null = none
    uint32_t n;                  // cells per axis
    uint32_t run;                // longest run of skipped positions (segment length - 1)
    float lo[3], scale[3];       // cell coordinate = (P - lo) * scale
    float tau;                   // skip / confirm threshold
    uint32_t smem_words;         // > 0: the render copies the bits into shared memory first
};

// A ray that meets the box, as the render's pre-pass (ray_list) lists it:
// what ray_init derives for the march -- the direction, the box's entry and
// exit (the slab test's FP64 divisions), the step and the sample cap (an FP64
// division) -- so a lane of the render takes a new ray with two 16-byte loads
// instead of repeating that setup.
struct alignas(16) RayEntry {
    uint32_t pix;
    float t0, t1;
    uint32_t cap;
    float vx, vy, vz, Fdt;
};

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
    uint32_t flags;              // LYAP_FLAG_* (NO_SPECULATION and BISECT_F64 are read here)
    // LYAP_FLAG_BISECT_F64 only: the march stops at the crossing and records
    // it; a second pass bisects it in double (lyap_precise.cu)
    float *bracket;              // device, 2 per pixel: t of the last sample above, first at/below
    uint32_t *hits;              // device, [0] = count, then the pixel indices that crossed
    // learned proposal (render_persistent<Lam, true> only; grid null = none)
    PropGrid prop;
    // the rays that meet the box, listed by ray_list (null: the queue runs
    // over every pixel); the render's queue hands out list[i]
    const RayEntry *list;
    const uint32_t *list_count;  // device: entries in list
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
