/******************************************************************************
ref_shim.h -- TEST INFRASTRUCTURE ONLY (oracle side, never product code).

Lets g++ compile the reference's unmodified CUDA headers (include/*.cuh of
weisluke/ccf) as plain host C++, so that the reference's own functions can be
run on the CPU as the checker for this project's GPU results.

What it does:
  * includes the CUDA runtime and curand headers first (curand's XORWOW
    generator has host code paths, so seeded star fields match the GPU);
  * defines the CUDA execution-space keywords away and maps the built-in
    index variables to host globals with gridDim = blockDim = 1, so every
    grid-stride loop of a reference kernel runs serially in index order;
  * supplies serial atomics and a no-op __syncthreads();
  * maps the three cudaDeviceProp fields that CUDA 13 removed (read only by
    the reference's show_device_info, include/util.cuh:282-286) onto fields
    that still exist, so the header compiles; that function is never called;
  * routes cudaMallocManaged to malloc and makes the error checks succeed,
    since this build never touches a GPU.
******************************************************************************/
#pragma once

#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cstdlib>

struct ShimDim3
{
	unsigned int x, y, z;
};

inline ShimDim3 shim_threadIdx = {0, 0, 0};
inline ShimDim3 shim_blockIdx = {0, 0, 0};
inline ShimDim3 shim_blockDim = {1, 1, 1};
inline ShimDim3 shim_gridDim = {1, 1, 1};

#undef threadIdx
#undef blockIdx
#undef blockDim
#undef gridDim
#define threadIdx shim_threadIdx
#define blockIdx shim_blockIdx
#define blockDim shim_blockDim
#define gridDim shim_gridDim

#undef __global__
#undef __device__
#undef __host__
#undef __shared__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __shared__
#define __forceinline__ inline

#define __syncthreads() ((void)0)

inline int atomicAdd(int* p, int v) { int old = *p; *p += v; return old; }
inline int atomicSub(int* p, int v) { int old = *p; *p -= v; return old; }
inline int atomicMin(int* p, int v) { int old = *p; if (v < *p) *p = v; return old; }
inline int atomicMax(int* p, int v) { int old = *p; if (v > *p) *p = v; return old; }
inline int atomicExch(int* p, int v) { int old = *p; *p = v; return old; }

/* fields removed from cudaDeviceProp in CUDA 13 (read only by show_device_info) */
#define clockRate major
#define memoryClockRate minor
#define singleToDoublePrecisionPerfRatio major

inline cudaError_t shim_malloc_managed(void** p, size_t n)
{
	*p = std::calloc(n, 1);
	return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
#define cudaMallocManaged(p, n) shim_malloc_managed((void**)(p), (n))
/* launch-shape helpers (include/util.cuh:200-269) are compiled but never called */
inline cudaError_t shim_get_device(int* d) { *d = 0; return cudaErrorNoDevice; }
inline cudaError_t shim_get_device_properties(cudaDeviceProp*, int) { return cudaErrorNoDevice; }
#define cudaGetDevice(d) shim_get_device(d)
#define cudaGetDeviceProperties(p, d) shim_get_device_properties((p), (d))
#define cudaGetLastError() (cudaSuccess)
#define cudaDeviceSynchronize() (cudaSuccess)
