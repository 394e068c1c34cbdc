/* Host-only stand-in for <cublas_v2.h>: type names only.  Test infrastructure
 * for compiling the reference's kernel sources with g++ (see cuda_runtime.h). */
#ifndef SFWI_CUDA_SHIM_CUBLAS_H
#define SFWI_CUDA_SHIM_CUBLAS_H
typedef void *cublasHandle_t;
typedef int cublasStatus_t;
#endif
