// lyap_render.cu -- the raymarch renderer (kernel_calc_render, kernel.cu:500):
// the library's precompiled instantiation of render_persistent (any
// sequence, RuntimeLambda; lyap_kernels.cuh), its launcher, the reference's
// own __global__ entry point and its C-ABI launcher.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_internal.h"
#include "lyap_kernel.hpp"
#include "lyap_kernels.cuh"

namespace lyapgb {

int device_sm_count()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
        cached[dev] = n;
    }
    return cached[dev];
}

uint32_t proposal_smem_bytes(const RenderJob &job)
{
    return job.prop.bits ? job.prop.smem_words * 4u : 0u;
}

cudaError_t launch_render(const RenderJob &job, uint32_t mode, uint32_t *d_work_counter,
                          unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads,
                          cudaStream_t stream)
{
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    if (threads == 0) threads = LYAP_RENDER_THREADS;
    if (blocks_per_sm == 0) blocks_per_sm = LYAP_RENDER_MIN_BLOCKS;
    const uint32_t grid = (uint32_t)sms * blocks_per_sm;
    const bool prop = job.prop.bits != nullptr;   // the learned proposal's instantiation
    const uint32_t smem = proposal_smem_bytes(job);
    if (mode == MODE_PRODUCT) {
        if (prop)
            render_persistent<RuntimeLambda<MODE_PRODUCT>, true>
                <<<grid, threads, smem, stream>>>(job, d_work_counter, d_stats);
        else
            render_persistent<RuntimeLambda<MODE_PRODUCT>><<<grid, threads, 0, stream>>>(job, d_work_counter, d_stats);
    } else {
        if (prop)
            render_persistent<RuntimeLambda<MODE_PLAIN>, true>
                <<<grid, threads, smem, stream>>>(job, d_work_counter, d_stats);
        else
            render_persistent<RuntimeLambda<MODE_PLAIN>><<<grid, threads, 0, stream>>>(job, d_work_counter, d_stats);
    }
    return cudaGetLastError();
}

// The pre-pass of the render: every pixel's ray is set up once; a ray that
// misses the box is finished here (exactly as the render finishes one), a ray
// that meets it is appended to `list` (one atomic per block of 256 pixels,
// pixel order within a block).  The render's queue then walks the list only:
// handing out runs of missing rays one atomic at a time stalled every warp
// of a frame with a sky band at the end of its scanline order.
__global__ void __launch_bounds__(256) ray_list(const __grid_constant__ RenderJob job, RayEntry *__restrict__ list,
                                                uint32_t *__restrict__ count, unsigned long long *__restrict__ stats)
{
    __shared__ uint32_t warp_n[8], block_base;
    const uint32_t npix = job.width * job.height;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const CamRays cr = cam_rays(job.cam);
    LaneStats st = {};
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool cross = false;
    RayEntry en;
    if (i < npix) {
        Ray r;
        r.phase = PH_MARCH0;
        r.pst = 0;
        if (ray_geometry(cr, job.prm, i % job.width, i / job.width, en)) {
            cross = true;
            en.pix = i;
        } else {
            r.nm = r.nh = r.ns = 0;
            finish_pixel(job.rgba, job.points, job.counts, i, r, false, cr.C, job.lights, job.n_lights,
                         job.light_model, st);
        }
    }
    const uint32_t m = __ballot_sync(FULL, cross);
    if (lane == 0) warp_n[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); w++) tot += warp_n[w];
        block_base = tot ? atomicAdd(count, tot) : 0u;
    }
    __syncthreads();
    uint32_t off = block_base;
    for (uint32_t w = 0; w < warp; w++) off += warp_n[w];
    if (cross) list[off + __popc(m & ((1u << lane) - 1u))] = en;
    flush_stats(stats, st, FULL);
}

cudaError_t launch_ray_list(const RenderJob &job, RayEntry *list, uint32_t *count, unsigned long long *d_stats,
                            cudaStream_t stream)
{
    const uint64_t npix = (uint64_t)job.width * job.height;
    const uint32_t blocks = (uint32_t)((npix + 255) / 256);
    ray_list<<<blocks, 256, 0, stream>>>(job, list, count, d_stats);
    return cudaGetLastError();
}

}  // namespace lyapgb

using namespace lyapgb;

// kernel_calc_render (kernel.cu:500-516) with the reference's signature and
// launch shape: pixel (x, y) = (blockIdx*blockDim + threadIdx), index
// x + y * gridDim.x * blockDim.x, no bounds beyond the grid (as the
// reference).  The block's warps share the block's pixels through a
// shared-memory counter, so a warp stays full until its block runs dry;
// then, when the block is whole warps (the reference's 16 x 16 is eight)
// and the step length is fixed, lanes without a ray take samples ahead for
// the rays still running in their warp (sample_round, as the persistent
// render), so a block's longest ray no longer holds it one sample per round.
// Plain FP32 lambda; the sequence length is found from its -1 terminator.
// Blocks of at most 256 threads (the reference launches 16 x 16), two
// resident per SM: 128 registers, no spills.
LYAP_KERNEL_EXPORT __global__ void __launch_bounds__(256, 2)
    kernel_calc_render(RGBA *rgba, LyapPoint *points, LyapCam cam, LyapParams prm, int *seq, LyapLight *lights,
                       unsigned int num_lights)
{
    __shared__ uint32_t next;
    __shared__ uint32_t period;
    const uint32_t tid = threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y;
    if (tid == 0) {
        next = 0;
        uint32_t L = 0;
        while (L < LYAP_MAX_SEQ_LEN - 1 && seq[L] != -1) L++;
        period = L == 0 ? 1u : L;
    }
    __syncthreads();
    const uint32_t wmask = __activemask();
    const uint32_t lane = threadIdx.x & 31u;   // lanes of a block are consecutive in tid
    const uint32_t nitems = blockDim.x * blockDim.y;
    const uint32_t stride = gridDim.x * blockDim.x;
    const RuntimeLambda<MODE_PLAIN> lam(seq, period, prm);
    const CamRays cr = cam_rays(cam);
    LaneStats st = {};
    // sampling ahead needs whole warps (its ballots and shuffles span 32
    // lanes) and a slot table for each of the block's warps
    const uint32_t nthreads = blockDim.x * blockDim.y * blockDim.z;
    const bool whole_warps = (nthreads % 32u) == 0 && nthreads / 32u <= ROUND_WARPS_2D;
    const bool spec_ok = whole_warps && prm.jitter == 0.0f && prm.nearMultiplier == 1.0f;
    const PropGrid no_prop = {};
    Ray r;
    uint32_t ind = 0;
    bool active = false, drained = (threadIdx.z != 0);   // the reference's 2-D launch shape
    (void)lane;
    for (;;) {
        for (;;) {
            const bool need = !active && !drained;
            const uint32_t mask = __ballot_sync(wmask, need);
            if (mask == 0) break;
            const uint32_t lid = tid & 31u;
            const uint32_t leader = __ffs(mask) - 1;
            uint32_t base = 0;
            if (lid == leader) base = atomicAdd(&next, (uint32_t)__popc(mask));
            base = __shfl_sync(wmask, base, leader);
            if (need) {
                const uint32_t k = base + __popc(mask & ((1u << lid) - 1u));
                if (k >= nitems) {
                    drained = true;
                } else {
                    const uint32_t x = blockIdx.x * blockDim.x + (k % blockDim.x);
                    const uint32_t y = blockIdx.y * blockDim.y + (k / blockDim.x);
                    ind = x + y * stride;
                    if (ray_init(r, cr, prm, x, y)) {
                        active = true;
                    } else {
                        r.nm = r.nh = r.ns = 0;
                        finish_pixel(rgba, points, nullptr, ind, r, false, cr.C, lights, num_lights,
                                     LYAP_LIGHT_SPOT, st);
                    }
                }
            }
        }
        const uint32_t amask = __ballot_sync(wmask, active);
        if (amask == 0) break;
        int res;
        if (whole_warps) {
            res = sample_round<false, RuntimeLambda<MODE_PLAIN>, true>(r, active, amask, lam, prm, spec_ok, false,
                                                                       no_prop, st);
        } else {
            V3 Q = active ? ray_sample_point(r) : v3(3.0f, 3.0f, 3.0f);
            bool skipped, fallback;
            const float l = lam(Q.x, Q.y, Q.z, skipped, fallback);
            res = active ? ray_advance(r, l, prm) : RAY_CONTINUE;
        }
        if (active && res != RAY_CONTINUE) {
            finish_pixel(rgba, points, nullptr, ind, r, res == RAY_HIT, cr.C, lights, num_lights, LYAP_LIGHT_SPOT,
                         st);
            active = false;
        }
    }
}

// C-ABI launcher of kernel_calc_render with an explicit launch shape, for
// callers that cannot use <<<>>> (FFI); the reference launches it at
// lyap_interactive.cu:711 with grid (W/16, H/16) and blocks (16, 16).
extern "C" int lyap_kernel_calc_render(uint32_t grid_x, uint32_t grid_y, uint32_t block_x, uint32_t block_y,
                                       RGBA *d_rgba, LyapPoint *d_points, const LyapCam *cam,
                                       const LyapParams *prm, int32_t *d_seq, LyapLight *d_lights,
                                       uint32_t n_lights, void *stream)
{
    if (!cam || !prm || !d_seq || !d_rgba || !d_points || (n_lights && !d_lights))
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_render: null pointer");
    if (n_lights > LYAP_MAX_LIGHTS) return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_render: too many lights");
    if (!grid_x || !grid_y || !block_x || !block_y || (uint64_t)block_x * block_y > 256)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_render: bad launch shape (blocks of at most 256 "
                                               "threads)");
    kernel_calc_render<<<dim3(grid_x, grid_y), dim3(block_x, block_y), 0, (cudaStream_t)stream>>>(
        d_rgba, d_points, *cam, *prm, d_seq, d_lights, n_lights);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, "lyap_kernel_calc_render: launch");
}
