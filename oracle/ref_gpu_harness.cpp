/* ref_gpu_harness.cpp — the reference's own kernels, run on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the reference-GPU timing, never
 * the product).  oracle/ref_build.py compiles the reference's kernel sources
 * (sfwi-stage{1,2}/born.cu and the kernels it cuts out of FD2DGPU.cu) for
 * sm_103a with the reference's nvcc flags into oracle/_ref/ref_born_s{N}.cubin
 * and ref_fdk_s{N}.cubin, and lists every kernel's symbol and parameter kinds
 * in oracle/_ref/ref_kernels_s{N}.txt.  This file, compiled with the system
 * C++ compiler on the GPU machine (oracle/pyoracle.py:build_refgpu), loads
 * those modules and runs IMAGE_SINGLESHOT's launch sequence
 * (oracle/ref_sequence.inc, the same text the CPU build runs) with the
 * reference's launch shapes, so every cell update is the reference's CUDA
 * code on the GB300.  A launch is matched to the kernel overload whose
 * parameter kinds equal its arguments' kinds; a mismatch fails the call
 * before anything is launched.
 *
 * The kernels' indexing was checked on the CPU build under AddressSanitizer
 * at the test and benchmark shapes before any of them ran on a GPU.
 */
#ifndef SFWI_STAGE
#error "SFWI_STAGE must be 1 or 2"
#endif

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "sfwi_oracle.h"

namespace {

char g_err[1024] = "";
bool g_fail = false;

void set_error(const char *fmt, ...) {
    if (g_fail) return;  // keep the first error
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    g_fail = true;
}

struct Kernel {
    std::string kinds;
    CUfunction f;
};
std::multimap<std::string, Kernel> g_kernels;
bool g_loaded = false;

template <class T>
constexpr char kind_of() {
    if constexpr (std::is_pointer_v<T>) return 'p';
    else if constexpr (std::is_same_v<T, bool>) return 'b';
    else if constexpr (std::is_same_v<T, float>) return 'f';
    else if constexpr (std::is_same_v<T, double>) return 'd';
    else if constexpr (std::is_integral_v<T> && sizeof(T) == 4) return 'i';
    else if constexpr (std::is_integral_v<T> && sizeof(T) == 8) return 'l';
    else return '?';
}

template <class... A>
void launch_by_name(const char *name, dim3 grid, dim3 block, A... a) {
    if (g_fail) return;
    const std::string kinds = {kind_of<A>()...};
    auto range = g_kernels.equal_range(name);
    for (auto it = range.first; it != range.second; ++it) {
        if (it->second.kinds != kinds) continue;
        void *params[] = {static_cast<void *>(&a)...};
        const CUresult r = cuLaunchKernel(it->second.f, grid.x, grid.y, grid.z, block.x, block.y, block.z, 0, nullptr,
                                          params, nullptr);
        if (r != CUDA_SUCCESS) {
            const char *msg = "";
            cuGetErrorString(r, &msg);
            set_error("launch of %s: %s", name, msg);
        }
        return;
    }
    set_error("no kernel %s with parameter kinds %s", name, kinds.c_str());
}

// device arrays, zero-filled as the reference memsets them
template <class T>
struct Arr {
    T *d = nullptr;
    size_t n;
    explicit Arr(size_t n_) : n(n_) {
        if (!n || g_fail) return;
        if (cudaMalloc(&d, n * sizeof(T)) != cudaSuccess || cudaMemset(d, 0, n * sizeof(T)) != cudaSuccess) {
            set_error("device allocation of %zu bytes failed", n * sizeof(T));
            d = nullptr;
        }
    }
    ~Arr() {
        if (d) cudaFree(d);
    }
    Arr(const Arr &) = delete;
    Arr &operator=(const Arr &) = delete;
    T *p() { return d; }
    void upload(const T *h, size_t m) {
        if (g_fail || !d) return;
        if (cudaMemcpy(d, h, m * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) set_error("upload failed");
    }
    std::vector<T> host() const {
        std::vector<T> v(n, T(0));
        if (!g_fail && d && cudaMemcpy(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess)
            set_error("download failed");
        return v;
    }
};
typedef Arr<float> Dev;
typedef Arr<int> IDev;

#define REF_LAUNCH(grid, block, kernel, ...) launch_by_name(#kernel, grid, block, __VA_ARGS__)
#define REF_SET_THREADS(n) (void)(n)

int run_sequence(const sfwi_oracle_shot *sp, const sfwi_oracle_io *io) {
#include "ref_sequence.inc"
}

}  // namespace

extern "C" const char *sfwi_refgpu_error(void) { return g_err; }

extern "C" int sfwi_refgpu_stage(void) { return SFWI_STAGE; }

// load the stage's modules and kernel list from `dir` (oracle/_ref)
extern "C" int sfwi_refgpu_init(const char *dir) {
    if (g_loaded) return 0;
    g_fail = false;
    if (cudaFree(nullptr) != cudaSuccess) {  // creates the primary context
        set_error("no CUDA device");
        return -1;
    }
    const std::string base(dir);
    const std::string stage = std::to_string(SFWI_STAGE);
    CUmodule born = nullptr, fdk = nullptr;
    if (cuModuleLoad(&born, (base + "/ref_born_s" + stage + ".cubin").c_str()) != CUDA_SUCCESS ||
        cuModuleLoad(&fdk, (base + "/ref_fdk_s" + stage + ".cubin").c_str()) != CUDA_SUCCESS) {
        set_error("cannot load the reference's device modules from %s", dir);
        return -1;
    }
    std::ifstream lst(base + "/ref_kernels_s" + stage + ".txt");
    std::string line;
    while (std::getline(lst, line)) {
        std::istringstream ls(line);
        std::string name, module, sym, kinds;
        if (!(ls >> name >> module >> sym >> kinds)) continue;
        CUfunction f = nullptr;
        if (cuModuleGetFunction(&f, module == "born" ? born : fdk, sym.c_str()) != CUDA_SUCCESS) {
            set_error("kernel %s not found in the %s module", sym.c_str(), module.c_str());
            return -1;
        }
        g_kernels.emplace(name, Kernel{kinds, f});
    }
    if (g_kernels.empty()) {
        set_error("empty kernel list in %s", dir);
        return -1;
    }
    g_loaded = true;
    return 0;
}

extern "C" int sfwi_refgpu_image_singleshot(const sfwi_oracle_shot *sp, const sfwi_oracle_io *io) {
    if (!g_loaded) {
        std::snprintf(g_err, sizeof g_err, "sfwi_refgpu_init has not succeeded");
        return -10;
    }
    g_fail = false;
    g_err[0] = 0;
    const int rc = run_sequence(sp, io);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) set_error("device: %s", cudaGetErrorString(e));
    return g_fail ? -3 : rc;
}
