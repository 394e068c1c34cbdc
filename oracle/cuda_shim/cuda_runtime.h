/* Host-only stand-in for <cuda_runtime.h>.
 *
 * Test infrastructure: it lets the reference's own CUDA C kernel sources be
 * compiled by g++ as ordinary host functions, so that the oracle can be pinned
 * against the reference's arithmetic without a GPU.  Nothing in the product
 * includes this file.
 *
 * A kernel compiled through this header is a plain function that reads the
 * thread-local threadIdx/blockIdx/blockDim/gridDim below; the launcher in
 * oracle/ref_harness.cpp sets them and calls the function once per emulated
 * thread.  Every kernel the harness runs is free of inter-thread
 * communication, so the serial order gives the same result as a GPU launch.
 */
#ifndef SFWI_CUDA_SHIM_RUNTIME_H
#define SFWI_CUDA_SHIM_RUNTIME_H

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>

#define __global__
#define __device__
#define __host__
/* The reference defines its stencil table `__constant__ float coeff2[6]` in a
 * header included by two translation units; internal linkage keeps one copy
 * per unit, as CUDA's whole-program compilation does. */
#define __constant__ static
#define __shared__ static
#define __forceinline__ inline
#define __restrict__

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3 { unsigned x, y, z; };
struct float2 { float x, y; };
struct double2 { double x, y; };

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

typedef void *cudaStream_t;
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };

inline void __syncthreads() {}

#endif
