// lyap_volume.cu -- the dense lambda volume sweep (kernel_calc_volume,
// kernel.cu:488-532; front-end lyap_calculate.cu:58-91): the library's
// precompiled instantiation of volume_sweep (any sequence; lyap_kernels.cuh),
// its launcher, the reference's own __global__ entry point and its C-ABI
// launcher.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lyap_internal.h"
#include "lyap_kernel.hpp"
#include "lyap_kernels.cuh"

namespace lyapgb {

cudaError_t launch_volume(const VolumeJob &job, uint32_t mode, unsigned long long *d_stats,
                          uint32_t blocks_per_sm, uint32_t threads, cudaStream_t stream)
{
    const int sms = device_sm_count();
    if (sms <= 0) return cudaErrorNoDevice;
    if (threads == 0) threads = LYAP_VOLUME_THREADS;
    if (blocks_per_sm == 0) blocks_per_sm = LYAP_VOLUME_MIN_BLOCKS;
    const uint64_t total = (uint64_t)job.nx * job.ny * job.nz;
    uint64_t grid = (uint64_t)sms * blocks_per_sm;
    const uint64_t need = (total + threads - 1) / threads;
    if (need < grid) grid = need;
    if (grid == 0) return cudaSuccess;
    if (mode == MODE_PRODUCT)
        volume_sweep<RuntimeLambda<MODE_PRODUCT>, 1><<<(uint32_t)grid, threads, 0, stream>>>(job, d_stats);
    else
        volume_sweep<RuntimeLambda<MODE_PLAIN>, 1><<<(uint32_t)grid, threads, 0, stream>>>(job, d_stats);
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
