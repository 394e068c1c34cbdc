/* ref_harness.cpp — MPI-free CPU driver of the reference's own kernels.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  oracle/ref_build.py
 * compiles this file in ONE translation unit after the reference's kernel
 * sources (sfwi-stage{1,2}/born.cu and the kernels it cuts out of
 * sfwi-stage{1,2}/FD2DGPU.cu), all built as host C++ through oracle/cuda_shim.
 * The result, oracle/_ref/libsfwi_ref_s{1,2}.so, runs the reference's
 * arithmetic on the CPU so the restatement in sfwi_oracle.c can be pinned to
 * it.  Only the launch sequence (oracle/ref_sequence.inc, shared with the GPU
 * build in oracle/ref_gpu_harness.cpp) is written here; every cell update is
 * the reference's own code.
 *
 * The sequence restates IMAGE_SINGLESHOT:
 *   stage 1: sfwi-stage1/FD2DGPU.cu:4321-4695 (forward born_modeling mode 0,
 *            record_background_wave, residual syn-obs, adjoint direction +1)
 *   stage 2: sfwi-stage2/FD2DGPU.cu:3978-4570 (forward mode 1 with the Born
 *            source, record_scatter(it,true), residual (du-obs)+u0, adjoint
 *            direction -1, rho forced to 2000 by GPUcalculate_elastic_rho_C)
 * preceded by the caller's per-shot set-up (sfwi-stage1/main.cpp:585-625):
 * record_copytoGPU, bufferVpVsHtoD(delta_left+record_left_in_v), geometry.
 * Launch shapes are the reference's: Grid_Block 32x32 over the padded grid
 * (FD2DGPU.cu:57-60), imagesize over the interior (:1475-1478), 32-thread
 * rows over traces (:1371-1372), 32x32 over [ntr][nt] for the residual.
 * Stage 2 also reloads the scattered-field edge strips into b_vx/b_vz during
 * the backward loop (sfwi-stage2/FD2DGPU.cu:4420-4450); nothing downstream
 * reads them, so that copy is left out here.
 */
#ifndef SFWI_STAGE
#error "SFWI_STAGE must be 1 or 2"
#endif

#include <algorithm>
#include <vector>
#include <cstdint>
#include "sfwi_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace {

template <class F>
void launch(dim3 grid, dim3 block, F &&body) {
    const long nblocks = (long)grid.x * grid.y * grid.z;
#pragma omp parallel for schedule(static)
    for (long b = 0; b < nblocks; ++b) {
        gridDim = grid;
        blockDim = block;
        blockIdx.x = (unsigned)(b % grid.x);
        blockIdx.y = (unsigned)((b / grid.x) % grid.y);
        blockIdx.z = (unsigned)(b / ((long)grid.x * grid.y));
        for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    threadIdx.x = tx;
                    threadIdx.y = ty;
                    threadIdx.z = tz;
                    body();
                }
    }
}

// arrays of the emulated device (zero-filled, as the reference memsets them)
template <class T>
struct Arr {
    std::vector<T> v;
    explicit Arr(size_t n = 0) : v(n, T(0)) {}
    T *p() { return v.data(); }
    void upload(const T *h, size_t n) { std::copy(h, h + n, v.begin()); }
    std::vector<T> host() const { return v; }
};
typedef Arr<float> Dev;
typedef Arr<int> IDev;

} // namespace

extern "C" int sfwi_ref_stage(void) { return SFWI_STAGE; }

#define REF_LAUNCH(grid, block, kernel, ...) launch(grid, block, [&] { kernel(__VA_ARGS__); })
#ifdef _OPENMP
#define REF_SET_THREADS(n) \
    do {                   \
        if ((n) > 0) omp_set_num_threads(n); \
    } while (0)
#else
#define REF_SET_THREADS(n) (void)(n)
#endif

extern "C" int sfwi_ref_image_singleshot(const sfwi_oracle_shot *sp, const sfwi_oracle_io *io) {
#include "ref_sequence.inc"
}
