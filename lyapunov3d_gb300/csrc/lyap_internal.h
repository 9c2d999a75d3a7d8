// lyap_internal.h -- host/device shared declarations of the library (not
// part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_gb300.h"
#include "lyap_jobs.h"

namespace lyapgb {

// kernels launchers (lyap_render.cu, lyap_volume.cu); return a cudaError_t
cudaError_t launch_render(const RenderJob &job, uint32_t mode, uint32_t *d_work_counter,
                          unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads,
                          cudaStream_t stream);
// the render's pre-pass: finishes the pixels whose ray misses the box and
// lists the others in `list` (length in *count, which must start at 0)
cudaError_t launch_ray_list(const RenderJob &job, RayEntry *list, uint32_t *count, unsigned long long *d_stats,
                            cudaStream_t stream);
cudaError_t launch_bisect(const RenderJob &job, uint32_t mode, uint32_t halvings, unsigned long long *d_stats,
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

// the learned proposal (lyap_net.cu): the net's grid of n^3 cells over its
// box (the minimum of the net at each cell's corners; with dilate the
// minimum over the 27 cells around), built on `stream` on first use and
// cached per device, net hash, n and dilation for the life of the process
cudaError_t proposal_grid(const LyapNet &net, uint32_t n, uint32_t dilate, const float **grid,
                          unsigned long long *stats, cudaStream_t stream);
// the march's form of it for one threshold: bit c set when cell c >= tau
// (PropGrid.bits), cached likewise per threshold
cudaError_t proposal_bits(const LyapNet &net, uint32_t n, uint32_t dilate, float tau, const uint32_t **bits,
                          unsigned long long *stats, cudaStream_t stream);
// shared memory the proposal's bits take in the render (0: they stay in global memory)
uint32_t proposal_smem_bytes(const RenderJob &job);
// LyapRenderExt.proposal when the struct has the field, else null (lyap_capi.cu)
const LyapNet *ext_proposal(const LyapRenderExt *ext);

// stream-ordered scratch from the library's memory pool of the current
// device (lyap_capi.cu); release with cudaFreeAsync
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t s);

// error reporting (lyap_capi.cu)
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);

}  // namespace lyapgb
