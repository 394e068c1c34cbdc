/* Host-only stand-in for <curand_kernel.h>: type names only.  Test
 * infrastructure for compiling the reference's kernel sources with g++. */
#ifndef SFWI_CUDA_SHIM_CURAND_H
#define SFWI_CUDA_SHIM_CURAND_H
struct curandState { unsigned long long s; };
#endif
