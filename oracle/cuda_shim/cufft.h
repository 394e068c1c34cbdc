/* Host-only stand-in for <cufft.h>: type names only.  Test infrastructure for
 * compiling the reference's kernel sources with g++. */
#ifndef SFWI_CUDA_SHIM_CUFFT_H
#define SFWI_CUDA_SHIM_CUFFT_H
typedef int cufftHandle;
typedef int cufftResult;
#define CUFFT_SUCCESS 0
struct cufftDoubleComplex { double x, y; };
#endif
