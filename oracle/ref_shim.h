/*
 * ref_shim.h -- force-included (g++ -include) when the reference's own CUDA
 * sources (kernel.cu, scene.cu, params.cu) are compiled as host C++ into
 * oracle/_ref/.  TEST INFRASTRUCTURE ONLY: nothing in the product links it.
 *
 * It supplies what nvcc would: the CUDA vector types, empty __device__ /
 * __global__ / __host__ qualifiers (crt/host_defines.h does that for a
 * non-CUDA compiler), the built-in launch coordinates as per-host-thread
 * variables, and __umul24.  It also supplies <cstring>, which scene.cu uses
 * (strlen, scene.cu:73) without including, and brings std::isnan/isfinite
 * into the global namespace, where kernel.cu calls them unqualified
 * (kernel.cu:29,147,251,344).
 *
 * The reference calls exit(1) on a bad sequence letter (scene.cu:98-100);
 * callers of the reference build must only pass valid sequences.
 */
#ifndef LYAP_REF_SHIM_H
#define LYAP_REF_SHIM_H

#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <vector_types.h>

using std::isnan;
using std::isfinite;

/* kernel_calc_render / kernel_calc_volume read these (kernel.cu:502-504,520-525);
 * ref_driver.cpp sets them per host thread before each "thread" of a launch. */
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

static inline unsigned int __umul24(unsigned int a, unsigned int b)
{
    return (a & 0xffffffu) * (b & 0xffffffu);
}

#endif
