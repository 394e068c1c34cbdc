// compat_driver.cpp — a caller of include/FD2DGPU_compat.hpp written in the
// call order of the reference's stage drivers, for tests/test_compat.py.
//
// Gradient loop as in sfwi-stage1/main.cpp:534-635 (sfwi-stage2/main.cpp:
// 497-594): construct the engine, upload the model (and the stage-2
// perturbation), then per shot record_copytoGPU, bufferVpVsHtoD, the public
// fields, IMAGE_SINGLESHOT; then imagebuffer_resettozero.  Line search as in
// sfwi-stage1/main.cpp:1100-1186 (CALCULATE_ALPHA_parabola_mb per shot) or
// sfwi-stage2/main.cpp:770-850 (CALCULATE_ALPHA per shot).  The MPI task farm
// of the reference becomes a plain loop over the shots.
//
//   compat_driver <dir>
// reads <dir>/params.txt and raw little-endian arrays (float32; receiver
// coordinates int32), writes <dir>/out_grad_pp.bin, out_grad_ps.bin,
// out_illum.bin and <dir>/out.txt.  Exit status 3 and "error <code>: <message>"
// on stderr when a call throws.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "FD2DGPU_compat.hpp"

// the reference's drivers define normalize themselves (sfwi-stage1/main.cpp:24-32)
void normalize(float *matrix, int length, int tracenum) {
    float m = 0.f;
    for (int i = 0; i < length * tracenum; i++) m = matrix[i] > m ? matrix[i] : (-matrix[i] > m ? -matrix[i] : m);
    if (m > 0.f)
        for (int i = 0; i < length * tracenum; i++) matrix[i] /= m;
}

namespace {

template <class T>
std::vector<T> load(const std::string &path, size_t n) {
    std::vector<T> v(n);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

void save(const std::string &path, const std::vector<float> &v) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(float), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
}

struct Shot {
    int ntr, ngx_left, delta_left, record_left_in_v, isx, isz, igz;
    std::vector<float> rz, rx;
    std::vector<int> gc;
};

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: compat_driver <dir>\n");
        return 2;
    }
    const std::string dir = argv[1];
    FILE *pf = std::fopen((dir + "/params.txt").c_str(), "r");
    if (!pf) return 2;
    int stage, allnx, allnz, nxpml, nzpml, pml, nt, ntr_pre, nshots, rbc;
    float dx, dz, dt, step1, step2;
    if (std::fscanf(pf, "%d %d %d %d %d %d %d %d %f %f %f %d %d", &stage, &allnx, &allnz, &nxpml, &nzpml, &pml, &nt,
                    &ntr_pre, &dx, &dz, &dt, &rbc, &nshots) != 13)
        return 2;
    std::vector<Shot> shots(nshots);
    for (auto &s : shots)
        if (std::fscanf(pf, "%d %d %d %d %d %d %d", &s.ntr, &s.ngx_left, &s.delta_left, &s.record_left_in_v, &s.isx,
                        &s.isz, &s.igz) != 7)
            return 2;
    if (std::fscanf(pf, "%f %f", &step1, &step2) != 2) return 2;
    std::fclose(pf);
    const size_t n = (size_t)allnx * allnz;
    std::vector<float> sou = load<float>(dir + "/sou.bin", nt);
    std::vector<float> vp = load<float>(dir + "/vp.bin", n), vs = load<float>(dir + "/vs.bin", n);
    std::vector<float> rho = stage == 1 ? load<float>(dir + "/rho.bin", n) : std::vector<float>();
    std::vector<float> image_pp = stage == 2 ? load<float>(dir + "/dvp.bin", n) : std::vector<float>(n, 0.f);
    std::vector<float> image_ps = stage == 2 ? load<float>(dir + "/dvs.bin", n) : std::vector<float>(n, 0.f);
    std::vector<float> dir_pp = load<float>(dir + "/dir_pp.bin", n), dir_ps = load<float>(dir + "/dir_ps.bin", n);
    for (int k = 0; k < nshots; k++) {
        Shot &s = shots[k];
        s.rz = load<float>(dir + "/shot" + std::to_string(k) + "_z.bin", (size_t)s.ntr * nt);
        s.rx = load<float>(dir + "/shot" + std::to_string(k) + "_x.bin", (size_t)s.ntr * nt);
        s.gc = load<int>(dir + "/shot" + std::to_string(k) + "_gc.bin", s.ntr);
    }
    std::vector<float> pp_grad(n), ps_grad(n), illumination(n), b1(n), b2(n), b3(n), b4(n);
    char imagedir[] = ".";
    double misfit = 0.0, m0 = 0.0, m1 = 0.0, m2 = 0.0, fenzi = 0.0, fenmu = 0.0;
    float misfit_ot = 0.f, m0_ot = 0.f, m1_ot = 0.f, m2_ot = 0.f;
    const int iter = 0, iter_round1 = 1, maxiter = 1, myid = 1, ntt = 100;
    const bool cpu_mem = false;
    try {
        FD2DGPU_ELASTIC image2delastic(sou.data(), dx, dz, dt, nxpml, nzpml, allnx, allnz, 1, pml, nt, 4, ntr_pre);
        if (stage == 1)
            image2delastic.GPUbufferVPVS(vp.data(), vs.data(), rho.data());
        else
            image2delastic.GPUbufferVPVS(vp.data(), vs.data());
        image2delastic.GPUbufferM(image_pp.data(), image_ps.data());
        const int Dim = nxpml * nzpml;
        for (int k = 0; k < nshots; k++) {
            Shot &s = shots[k];
            image2delastic.ntr = s.ntr;
            image2delastic.record_copytoGPU(s.rz.data(), s.rx.data(), s.gc.data());
            image2delastic.bufferVpVsHtoD(s.delta_left + s.record_left_in_v);
            image2delastic.delta_left = s.delta_left;
            image2delastic.record_left_in_v = s.record_left_in_v;
            image2delastic.isx = s.isx;
            image2delastic.isz = s.isz;
            image2delastic.igz = s.igz;
            image2delastic.cmin = s.delta_left + s.record_left_in_v;
            image2delastic.ngx_left = s.ngx_left;
            if (stage == 1)
                IMAGE_SINGLESHOT(image2delastic, k + 1, Dim, myid, s.rz.data(), s.rx.data(), s.gc.data(), rbc != 0,
                                 cpu_mem, ntt, iter, iter_round1, maxiter, imagedir, image_pp.data(), image_ps.data(),
                                 pp_grad.data(), ps_grad.data(), misfit, &misfit_ot);
            else
                IMAGE_SINGLESHOT(image2delastic, k + 1, Dim, myid, s.rz.data(), s.rx.data(), s.gc.data(), rbc != 0,
                                 cpu_mem, ntt, iter, imagedir, image_pp.data(), image_ps.data(), pp_grad.data(),
                                 ps_grad.data(), misfit);
        }
        image2delastic.imagebuffer_resettozero(pp_grad.data(), ps_grad.data(), illumination.data(), b1.data(),
                                               b2.data(), b3.data(), b4.data());
        // line search over the same shots
        for (int k = 0; k < nshots; k++) {
            Shot &s = shots[k];
            image2delastic.ntr = s.ntr;
            image2delastic.record_copytoGPU(s.rz.data(), s.rx.data(), s.gc.data());
            image2delastic.bufferVpVsHtoD(s.delta_left + s.record_left_in_v);
            image2delastic.delta_left = s.delta_left;
            image2delastic.record_left_in_v = s.record_left_in_v;
            image2delastic.isx = s.isx;
            image2delastic.isz = s.isz;
            image2delastic.igz = s.igz;
            image2delastic.cmin = s.delta_left + s.record_left_in_v;
            image2delastic.ngx_left = s.ngx_left;
            if (stage == 1)
                CALCULATE_ALPHA_parabola_mb(image2delastic, k + 1, Dim, myid, s.rz.data(), s.rx.data(), s.gc.data(),
                                            rbc != 0, cpu_mem, ntt, iter, image_pp.data(), image_ps.data(),
                                            dir_pp.data(), dir_ps.data(), m0, m1, m2, step1, step2, &m0_ot, &m1_ot,
                                            &m2_ot);
            else
                CALCULATE_ALPHA(image2delastic, k + 1, Dim, myid, s.rz.data(), s.rx.data(), s.gc.data(), imagedir,
                                rbc != 0, cpu_mem, ntt, iter, image_pp.data(), image_ps.data(), dir_pp.data(),
                                dir_ps.data(), fenzi, fenmu);
        }
    } catch (const sfwi_compat::error &e) {
        std::fprintf(stderr, "error %d: %s\n", e.code(), e.what());
        return 3;
    }
    save(dir + "/out_grad_pp.bin", pp_grad);
    save(dir + "/out_grad_ps.bin", ps_grad);
    save(dir + "/out_illum.bin", illumination);
    FILE *o = std::fopen((dir + "/out.txt").c_str(), "w");
    if (!o) return 2;
    std::fprintf(o, "%.17g %.17g %.17g %.17g %.17g %.17g\n", misfit, m0, m1, m2, fenzi, fenmu);
    std::fclose(o);
    return 0;
}
