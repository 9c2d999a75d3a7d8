// lyap_volume.cu -- the dense lambda volume sweep (kernel_calc_volume,
// kernel.cu:488-532; front-end lyap_calculate.cu:58-91).
//
// Every voxel costs the same settle + accum iterations, so there is no
// divergence to manage: a grid-stride loop over the x-fastest voxel index
// gives each warp 32 consecutive voxels and one coalesced 128-byte store.
// The store bypasses L1 and is marked evict-first (st.global.cs): the
// volume (512 MiB at 512^3) is written once and never read back here.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_device.cuh"
#include "lyap_internal.h"
#include "lyap_kernel.hpp"

namespace lyapgb {

__device__ __forceinline__ float voxel_coord(float lo, float hi, uint32_t i, uint32_t n)
{
    return lo + ((hi - lo) * (float)i) / (float)n;
}

template <uint32_t MODE>
__global__ void __launch_bounds__(256, 2) volume_sweep(const __grid_constant__ VolumeJob job,
                                                     unsigned long long *__restrict__ stats)
{
    const SeqInfo si = seq_setup(job.seq, job.seq_period, job.prm);
    const uint64_t nxy = (uint64_t)job.nx * job.ny;
    const uint64_t total = nxy * job.nz;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t skipped_n = 0, fallback_n = 0, samples = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const uint32_t z = (uint32_t)(i / nxy);
        const uint64_t rxy = i - (uint64_t)z * nxy;
        const uint32_t y = (uint32_t)(rxy / job.nx);
        const uint32_t x = (uint32_t)(rxy - (uint64_t)y * job.nx);
        const float a = voxel_coord(job.lo[0], job.hi[0], x, job.nx);
        const float b = voxel_coord(job.lo[1], job.hi[1], y, job.ny);
        const float c = voxel_coord(job.lo[2], job.hi[2], z, job.nz);
        bool skipped, fallback;
        const float lam = eval_lambda<MODE>(a, b, c, si, skipped, fallback);
        __stcs(job.out + i, lam);
        samples += 1;
        skipped_n += skipped ? 1u : 0u;
        fallback_n += fallback ? 1u : 0u;
    }
    if (stats) {
        const uint32_t mask = __activemask();
        const uint32_t s0 = __reduce_add_sync(mask, samples);
        const uint32_t s1 = __reduce_add_sync(mask, skipped_n);
        const uint32_t s7 = __reduce_add_sync(mask, fallback_n);
        if ((threadIdx.x & 31u) == (uint32_t)(__ffs(mask) - 1)) {
            if (s0) atomicAdd(stats + ST_SAMPLES, (unsigned long long)s0);
            if (s1) atomicAdd(stats + ST_SKIPPED, (unsigned long long)s1);
            if (s7) atomicAdd(stats + ST_FALLBACK, (unsigned long long)s7);
        }
    }
}

cudaError_t launch_volume(const VolumeJob &job, uint32_t mode, unsigned long long *d_stats,
                          uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream)
{
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    if (threads == 0) threads = 256;
    if (blocks_per_sm == 0) blocks_per_sm = 2;
    const uint64_t total = (uint64_t)job.nx * job.ny * job.nz;
    uint64_t grid = (uint64_t)sms * blocks_per_sm;
    const uint64_t need = (total + threads - 1) / threads;
    if (need < grid) grid = need;
    if (grid == 0) return cudaSuccess;
    if (mode == MODE_PRODUCT)
        volume_sweep<MODE_PRODUCT><<<(uint32_t)grid, threads, 0, stream>>>(job, d_stats);
    else
        volume_sweep<MODE_PLAIN><<<(uint32_t)grid, threads, 0, stream>>>(job, d_stats);
    return cudaGetLastError();
}

}  // namespace lyapgb

using namespace lyapgb;

// kernel_calc_volume (kernel.cu:518-532) with the reference's signature and
// launch shape: one voxel per thread, coordinate 4*i/N over [0, 4) per axis
// with N = gridDim*blockDim, stored at x + (y + z*Ny)*Nx.  Plain FP32.
LYAP_KERNEL_EXPORT __global__ void kernel_calc_volume(float *exps, LyapParams prm, int *seq)
{
    __shared__ uint32_t period;
    const uint32_t tid = threadIdx.x + threadIdx.y * blockDim.x + threadIdx.z * blockDim.x * blockDim.y;
    if (tid == 0) {
        uint32_t L = 0;
        while (L < LYAP_MAX_SEQ_LEN - 1 && seq[L] != -1) L++;
        period = L == 0 ? 1u : L;
    }
    __syncthreads();
    const SeqInfo si = seq_setup(seq, period, prm);
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    const uint32_t z = blockIdx.z * blockDim.z + threadIdx.z;
    const uint32_t Nx = gridDim.x * blockDim.x, Ny = gridDim.y * blockDim.y, Nz = gridDim.z * blockDim.z;
    const uint32_t ind = x + (y + z * Ny) * Nx;
    const float a = voxel_coord(0.0f, 4.0f, x, Nx);
    const float b = voxel_coord(0.0f, 4.0f, y, Ny);
    const float c = voxel_coord(0.0f, 4.0f, z, Nz);
    bool skipped, fallback;
    exps[ind] = eval_lambda<MODE_PLAIN>(a, b, c, si, skipped, fallback);
}

// C-ABI launcher of kernel_calc_volume with an explicit launch shape; the
// reference launches it at lyap_calculate.cu:72 with (N/8)^3 blocks of 8^3.
extern "C" int lyap_kernel_calc_volume(const uint32_t grid[3], const uint32_t block[3], float *d_exps,
                                       const LyapParams *prm, int32_t *d_seq, void *stream)
{
    if (!grid || !block || !d_exps || !prm || !d_seq)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_volume: null pointer");
    if (!grid[0] || !grid[1] || !grid[2] || !block[0] || !block[1] || !block[2] ||
        (uint64_t)block[0] * block[1] * block[2] > 1024)
        return set_error(LYAP_ERR_INVALID_ARG, "lyap_kernel_calc_volume: bad launch shape");
    kernel_calc_volume<<<dim3(grid[0], grid[1], grid[2]), dim3(block[0], block[1], block[2]), 0,
                         (cudaStream_t)stream>>>(d_exps, *prm, d_seq);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LYAP_OK : cuda_error(e, "lyap_kernel_calc_volume: launch");
}
