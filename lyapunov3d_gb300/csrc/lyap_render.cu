// lyap_render.cu -- the raymarch renderer (kernel_calc_render, kernel.cu:500).
//
// Work decomposition.  Every sample of a ray costs the same (settle + accum
// map iterations), but rays need from 0 to ~depth*nearMultiplier samples.
// A thread-per-pixel kernel (the reference's) keeps a warp busy until its
// longest ray ends.  Here each lane of a persistent warp owns one ray at a
// time; after every sample the lanes whose ray ended write their pixel and
// take the next pixel from a queue, so all 32 lanes evaluate a sample in
// every round until the queue is empty.  The lambda loop itself is uniform
// across the warp (same sequence, same iteration counts), which keeps the
// FP32 and MUFU pipes busy without divergence.
//
//  * render_persistent<MODE>: the C-ABI path (lyap_render): one global
//    pixel counter, grid = SMs x resident blocks;
//  * kernel_calc_render: the reference's __global__ entry point with its
//    launch shape; each block's pixels form the queue of that block's warps.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_device.cuh"
#include "lyap_internal.h"
#include "lyap_kernel.hpp"

namespace lyapgb {

constexpr uint32_t FULL = 0xffffffffu;

struct LaneStats {
    uint32_t samples, skipped, march, hone, normal, hits, rays, fallback;
};

__device__ __forceinline__ void store_point(LyapPoint *dst, const Ray &r, bool hit)
{
    float *f = reinterpret_cast<float *>(dst);
    if (hit) {
        f[0] = r.P.x; f[1] = r.P.y; f[2] = r.P.z;
        f[3] = r.N.x; f[4] = r.N.y; f[5] = r.N.z;
        f[6] = r.a; f[7] = r.c; f[8] = r.l;
    } else {
        // a miss: all-NaN bytes (the reference leaves the point unwritten)
        const float nanf_ = __int_as_float(-1);
#pragma unroll
        for (int k = 0; k < 9; k++) f[k] = nanf_;
    }
}

// Write one finished pixel: point, colour, optional per-pixel sample counts.
__device__ __forceinline__ void finish_pixel(RGBA *rgba, LyapPoint *points, uint32_t *counts, uint32_t ind,
                                             const Ray &r, bool hit, V3 camC, const LyapLight *lights,
                                             uint32_t n_lights, uint32_t light_model, LaneStats &st)
{
    store_point(points + ind, r, hit);
    uint32_t px = 0;
    if (hit) {
        LyapPoint pt;
        pt.P = LyapVec{r.P.x, r.P.y, r.P.z};
        pt.N = LyapVec{r.N.x, r.N.y, r.N.z};
        pt.a = r.a;
        pt.c = r.c;
        pt.l = r.l;
        C4 col = (light_model == LYAP_LIGHT_DIRECTIONAL) ? shade_directional(pt, lights, n_lights)
                                                         : shade_spot(pt, camC, lights, n_lights);
        px = (uint32_t)to_byte(col.x) | ((uint32_t)to_byte(col.y) << 8) | ((uint32_t)to_byte(col.z) << 16) |
             ((uint32_t)to_byte(col.w) << 24);
    }
    reinterpret_cast<uint32_t *>(rgba)[ind] = px;
    if (counts) {
        counts[3 * (size_t)ind + 0] = r.nm;
        counts[3 * (size_t)ind + 1] = r.nh;
        counts[3 * (size_t)ind + 2] = hit ? 6u : 0u;
    }
    st.march += r.nm;
    st.hone += r.nh;
    st.normal += hit ? 6u : 0u;
    st.hits += hit ? 1u : 0u;
    st.rays += 1;
}

__device__ __forceinline__ void flush_stats(unsigned long long *stats, LaneStats st, uint32_t mask)
{
    if (!stats) return;
    uint32_t v[8] = {st.samples, st.skipped, st.march, st.hone, st.normal, st.hits, st.rays, st.fallback};
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t s = __reduce_add_sync(mask, v[k]);
        if (lane == leader && s) atomicAdd(stats + k, (unsigned long long)s);
    }
}

// The C-ABI renderer: persistent warps, per-lane refill from a global queue.
template <uint32_t MODE>
__global__ void __launch_bounds__(128, 4) render_persistent(const __grid_constant__ RenderJob job,
                                                          uint32_t *__restrict__ work_counter,
                                                          unsigned long long *__restrict__ stats)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t npix = job.width * job.height;
    const SeqInfo si = seq_setup(job.seq, job.seq_period, job.prm);
    const CamRays cr = cam_rays(job.cam);
    LaneStats st = {};
    Ray r;
    uint32_t pix = 0;
    bool active = false, drained = false;

    for (;;) {
        // refill the lanes whose ray has ended
        for (;;) {
            const bool need = !active && !drained;
            const uint32_t mask = __ballot_sync(FULL, need);
            if (mask == 0) break;
            const uint32_t leader = __ffs(mask) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(work_counter, (uint32_t)__popc(mask));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const uint32_t my = base + __popc(mask & ((1u << lane) - 1u));
                if (my >= npix) {
                    drained = true;
                } else {
                    pix = my;
                    const uint32_t sx = my % job.width, sy = my / job.width;
                    if (ray_init(r, cr, job.prm, sx, sy)) {
                        active = true;
                    } else {
                        r.nm = r.nh = 0;
                        finish_pixel(job.rgba, job.points, job.counts, my, r, false, cr.C, job.lights,
                                     job.n_lights, job.light_model, st);
                    }
                }
            }
        }
        if (__ballot_sync(FULL, active) == 0) break;

        // one lambda sample for every lane (idle lanes evaluate a dummy point)
        V3 Q = active ? ray_sample_point(r) : v3(3.0f, 3.0f, 3.0f);
        bool skipped, fallback;
        const float lam = eval_lambda<MODE>(Q.x, Q.y, Q.z, si, skipped, fallback);
        if (active) {
            st.samples += 1;
            st.skipped += skipped ? 1u : 0u;
            st.fallback += fallback ? 1u : 0u;
            const int res = ray_advance(r, lam, job.prm);
            if (res != RAY_CONTINUE) {
                finish_pixel(job.rgba, job.points, job.counts, pix, r, res == RAY_HIT, cr.C, job.lights,
                             job.n_lights, job.light_model, st);
                active = false;
            }
        }
    }
    flush_stats(stats, st, FULL);
}

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

cudaError_t launch_render(const RenderJob &job, uint32_t mode, uint32_t *d_work_counter,
                          unsigned long long *d_stats, uint32_t blocks_per_sm, uint32_t threads,
                          cudaStream_t stream)
{
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    if (threads == 0) threads = 128;
    if (blocks_per_sm == 0) blocks_per_sm = 4;
    const uint32_t grid = (uint32_t)sms * blocks_per_sm;
    if (mode == MODE_PRODUCT)
        render_persistent<MODE_PRODUCT><<<grid, threads, 0, stream>>>(job, d_work_counter, d_stats);
    else
        render_persistent<MODE_PLAIN><<<grid, threads, 0, stream>>>(job, d_work_counter, d_stats);
    return cudaGetLastError();
}

}  // namespace lyapgb

using namespace lyapgb;

// kernel_calc_render (kernel.cu:500-516) with the reference's signature and
// launch shape: pixel (x, y) = (blockIdx*blockDim + threadIdx), index
// x + y * gridDim.x * blockDim.x, no bounds beyond the grid (as the
// reference).  The block's warps share the block's pixels through a
// shared-memory counter, so a warp stays full until its block runs dry.
// Plain FP32 lambda; the sequence length is found from its -1 terminator.
LYAP_KERNEL_EXPORT __global__ void kernel_calc_render(RGBA *rgba, LyapPoint *points, LyapCam cam, LyapParams prm, int *seq,
                                   LyapLight *lights, unsigned int num_lights)
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
    const SeqInfo si = seq_setup(seq, period, prm);
    const CamRays cr = cam_rays(cam);
    LaneStats st = {};
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
                        r.nm = r.nh = 0;
                        finish_pixel(rgba, points, nullptr, ind, r, false, cr.C, lights, num_lights,
                                     LYAP_LIGHT_SPOT, st);
                    }
                }
            }
        }
        if (__ballot_sync(wmask, active) == 0) break;
        V3 Q = active ? ray_sample_point(r) : v3(3.0f, 3.0f, 3.0f);
        bool skipped, fallback;
        const float lam = eval_lambda<MODE_PLAIN>(Q.x, Q.y, Q.z, si, skipped, fallback);
        if (active) {
            const int res = ray_advance(r, lam, prm);
            if (res != RAY_CONTINUE) {
                finish_pixel(rgba, points, nullptr, ind, r, res == RAY_HIT, cr.C, lights, num_lights,
                             LYAP_LIGHT_SPOT, st);
                active = false;
            }
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
    if (!grid_x || !grid_y || !block_x || !block_y || (uint64_t)block_x * block_y > 1024)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_render: bad launch shape");
    kernel_calc_render<<<dim3(grid_x, grid_y), dim3(block_x, block_y), 0, (cudaStream_t)stream>>>(
        d_rgba, d_points, *cam, *prm, d_seq, d_lights, n_lights);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, "lyap_kernel_calc_render: launch");
}
