// lyap_kernel.hpp -- the reference's device entry points (kernel.hpp:17-19)
// for CUDA C++ callers that launch them directly, e.g. the reference's own
// front-ends (lyap_interactive.cu:711, lyap_calculate.cu:72):
//
//     kernel_calc_render<<<dim3(W/16, H/16), dim3(16, 16)>>>(rgba, points, cam, prm, seq, lights, n);
//     kernel_calc_volume<<<dim3(N/8, N/8, N/8), dim3(8, 8, 8)>>>(exps, prm, seq);
//
// Same names, parameter types and launch-shape semantics as kernel.cu:500
// and kernel.cu:518 (the struct names are the reference's, so the mangled
// symbols match and a reference object file links against this library in
// place of kernel.o).  Both compute lambda in the plain FP32 form.
// kernel.hpp also declares the __device__ helpers shade / lyap4d / raycast;
// they are internal here (no relocatable device code is exported).
#ifndef LYAP_KERNEL_HPP
#define LYAP_KERNEL_HPP

#include "lyap_gb300.h"

#if defined(__CUDACC__)
// The host launch stubs are exported from the shared library (nvcc gives
// __global__ stubs hidden visibility by default).
#define LYAP_KERNEL_EXPORT __attribute__((visibility("default")))

// kernel.cu:500 -- one pixel per thread position; points[x + y*W] and
// rgba[x + y*W] with W = gridDim.x*blockDim.x; a miss writes an all-NaN point.
// Blocks of at most 256 threads (the reference's launch is 16 x 16).
LYAP_KERNEL_EXPORT __global__ void kernel_calc_render(RGBA *rgba, LyapPoint *points, LyapCam cam, LyapParams prm, int *seq,
                                   LyapLight *lights, unsigned int num_lights);

// kernel.cu:518 -- lambda at (4x/Nx, 4y/Ny, 4z/Nz, prm.d), N = gridDim*blockDim
// per axis, stored at exps[x + (y + z*Ny)*Nx].
LYAP_KERNEL_EXPORT __global__ void kernel_calc_volume(float *exps, LyapParams prm, int *seq);
#endif

#endif
