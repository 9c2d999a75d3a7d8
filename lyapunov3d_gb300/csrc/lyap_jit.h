// lyap_jit.h -- run-time specialisation of the kernels (lyap_jit.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "lyap_jobs.h"

// Launch shape of the specialised kernels: with the sequence compiled in,
// the plain render fits in 80 registers without spilling (3 blocks of 256
// threads per SM, against 4 of 128 for the precompiled kernel) and the volume
// sweep evaluates LYAP_JIT_VOLUME_K voxels per thread in 64 registers (4
// blocks of 256 threads per SM).  The end-of-frame hand-over of the render
// works within a block, so the paired product render runs one block of 512
// threads per SM (16 warps, up to 128 registers): 12.69-12.72 ms per 1080p
// frame against 13.00-13.07 with 2 blocks of 256 and about 13.15 with 4 of
// 128, the same warps per SM each time.
#define LYAP_JIT_MAX_PERIOD 32
#define LYAP_JIT_RENDER_MIN_BLOCKS 3
#define LYAP_JIT_RENDER_THREADS 256
// paired rounds (two samples per lane, packed FP32 pairs) in the specialised
// product-form render: 5-10 % faster 1080p frames than one sample per lane
// at 24 warps/SM; with 16 warps/SM (up to 128 registers) 1-4 % faster than
// with 20 or 24.  The plain form is MUFU-bound: packing gains it nothing and
// the lower occupancy costs it, so it keeps one sample per lane.
#define LYAP_JIT_RENDER_PAIRS_PRODUCT 1
#define LYAP_JIT_RENDER_PAIRS_PLAIN 0
#define LYAP_JIT_RENDER_MIN_BLOCKS_PAIRS 1
#define LYAP_JIT_RENDER_THREADS_PAIRS 512
#define LYAP_JIT_VOLUME_K 2
#define LYAP_JIT_VOLUME_MIN_BLOCKS 4
#define LYAP_VOLUME_THREADS_JIT 256

namespace lyapgb {

// Both return 1 when the specialised kernel was launched (its launch status
// in *launch_err) and 0 when the path is unavailable for this call (reason
// in *why); the caller then launches the precompiled kernel.
int jit_launch_render(const RenderJob &job, uint32_t mode, const int32_t *h_seq, uint32_t *d_work_counter,
                      unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream,
                      cudaError_t *launch_err, std::string *why);
int jit_launch_volume(const VolumeJob &job, uint32_t mode, const int32_t *h_seq, unsigned long long *d_stats,
                      uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream, cudaError_t *launch_err,
                      std::string *why);
// The batch kernel render_batch<ConstLambda<...>> for one sequence (period L,
// settle count `settle`) and lambda form: 1 with *kernel set, 0 with the
// reason in *why.
int jit_batch_kernel(const int32_t *h_seq, uint32_t L, uint32_t settle, uint32_t mode, cudaKernel_t *kernel,
                     std::string *why);

}  // namespace lyapgb
