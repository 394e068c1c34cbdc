// sfwi_fwi.cpp — the stage-1 and stage-2 inversion drivers on one GPU.
//
//   sfwi_fwi <para_file> [--stage 1|2] [--iters N] [--misfit l2|ot|ot_power|ot_alltrace]
//            [--snapshots K f32|f16|bf16] [--source txx_tzz|vz] [--gradient-only] [--resume]
//
// The reference runs these as MPI programs (sfwi-stage1/main.cpp,
// sfwi-stage2/main.cpp): a master hands shots to one worker per GPU, each
// worker calls IMAGE_SINGLESHOT shot by shot, the gradients are reduced, and
// the master updates the model.  Here every shot of an iteration advances in
// the same kernel launches on one GPU (sfwi_enqueue_shot / sfwi_run), and the
// line search runs all shots and trial models in one batch as well.  The
// update arithmetic per iteration is the reference's:
//
// stage 1 (main.cpp:636-1290; the Hessian inner loop has max_inner = 0):
//   g = grad / illumination, zero above layer 26; beta_num = sum(grad . g);
//   beta = beta_num / beta_num(previous) (0 at the first iteration);
//   cg = g + beta cg_old; d = cg normalised by the largest |cg_pp|, |cg_ps|;
//   misfits at steps 0, 30, 150 along -d (CALCULATE_ALPHA_parabola_mb);
//   alpha = vertex of the parabola (cal_step2), clamped to [-100, 300];
//   vp -= alpha d_pp, vs -= alpha d_ps; layers above 26 take vp[0][0], vs[0][0].
// stage 2 (sfwi-stage2/main.cpp:600-890): the model perturbation (image)
//   starts at zero; below layer 26 cg = grad / illumination, above it grad =
//   cg = 0; beta_num = sum(grad^2 / illumination); cg += beta cg_old;
//   alpha = fenzi / fenmu (CALCULATE_ALPHA); image -= alpha cg.
// Output files (float32 [allnx][allnz]) carry the reference's names.
//
// Checkpoints: after each iteration the driver also writes state.bin, the
// whole state the next iteration starts from (the model or the model
// perturbation, the previous CG direction, the CG denominator and the first
// misfit).  With --resume it continues from that file, and every later file
// equals an uninterrupted run's bit for bit.  The reference's drivers can
// only restart from a dumped model, without the CG state.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/sfwi_gb300.h"
#include "sfwi_host.h"

namespace {

constexpr float kStep1 = 30.f, kStep2 = 150.f;

void die(const char *what) {
    std::fprintf(stderr, "sfwi_fwi: %s\n", what);
    std::exit(1);
}
void check(int rc, const char *what) {
    if (rc) {
        std::fprintf(stderr, "sfwi_fwi: %s: %s\n", what, sfwi_last_error());
        std::exit(1);
    }
}

std::vector<float> read_model(const char *path, size_t n) {
    std::vector<float> v(n);
    FILE *f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(float), n, f) != n) {
        std::fprintf(stderr, "sfwi_fwi: cannot read %zu floats from %s\n", n, path);
        std::exit(1);
    }
    std::fclose(f);
    return v;
}

void write_model(const std::string &dir, const char *name, int iter, int allnx, int allnz, const float *a) {
    char path[2048];
    std::snprintf(path, sizeof path, "%s/%s_%d_%d_%d.dat", dir.c_str(), name, iter, allnx, allnz);
    FILE *f = std::fopen(path, "wb");
    if (!f) die("cannot write an output file");
    std::fwrite(a, sizeof(float), (size_t)allnx * allnz, f);
    std::fclose(f);
}

// ricker_wave, sfwi-stage1/main.cpp:251-260 (PI a double literal, the
// exponent a float product)
std::vector<float> ricker(int nt, float dt, float fm) {
    const double PI = 3.14159265358979;
    const float Nk = (float)(PI * PI * fm * fm * dt * dt);
    const int t0 = (int)std::ceil(1.0 / (fm * dt));
    std::vector<float> w(nt);
    for (int t = 0; t < nt; t++)
        w[t] = (float)((1.0 - 2.0 * Nk * (t - t0) * (t - t0)) * std::exp(-Nk * (t - t0) * (t - t0)));
    return w;
}

struct Shot {
    sfwi_shot_desc d;
    std::vector<int> gc;
    std::vector<float> rz, rx;
};

// state.bin: a fixed header, then four float32 [allnx][allnz] arrays: the
// model (vp, vs; stage 1) or the perturbation (image_pp, image_ps; stage 2),
// then the previous CG direction (pp, ps)
struct StateHeader {
    char magic[8];
    int version, stage, next_iter, allnx, allnz, pad;
    double beta_fenmu, max_misfit;
};
constexpr char kStateMagic[8] = {'S', 'F', 'W', 'I', 'S', 'T', 'A', 'T'};

void write_state(const std::string &dir, const StateHeader &hdr, const std::vector<const float *> &arrays, size_t n) {
    const std::string tmp = dir + "/state.bin.tmp", path = dir + "/state.bin";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) die("cannot write the checkpoint");
    bool ok = std::fwrite(&hdr, sizeof hdr, 1, f) == 1;
    for (const float *a : arrays) ok = ok && std::fwrite(a, sizeof(float), n, f) == n;
    ok = std::fclose(f) == 0 && ok;
    // the old checkpoint stays whole until the new one is complete
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) die("cannot write the checkpoint");
}

bool read_state(const std::string &dir, StateHeader *hdr, const std::vector<float *> &arrays, size_t n) {
    FILE *f = std::fopen((dir + "/state.bin").c_str(), "rb");
    if (!f) return false;
    bool ok = std::fread(hdr, sizeof *hdr, 1, f) == 1 && std::memcmp(hdr->magic, kStateMagic, 8) == 0 &&
              hdr->version == 1;
    for (float *a : arrays) ok = ok && std::fread(a, sizeof(float), n, f) == n;
    std::fclose(f);
    return ok;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) die("usage: sfwi_fwi <para_file> [--stage 1|2] [--iters N] [--misfit l2|ot|...] "
                      "[--snapshots K f32|f16|bf16] [--source txx_tzz|vz] [--gradient-only]");
    int stage = 1, iters = -1, misfit_kind = SFWI_MISFIT_L2, snap_k = 0, snap_fmt = SFWI_SNAP_F16;
    int source = SFWI_SOURCE_TXX_TZZ;
    bool gradient_only = false, resume = false;
    for (int i = 2; i < argc; i++) {
        if (!std::strcmp(argv[i], "--stage") && i + 1 < argc)
            stage = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--iters") && i + 1 < argc)
            iters = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--misfit") && i + 1 < argc) {
            const char *m = argv[++i];
            misfit_kind = !std::strcmp(m, "ot")            ? SFWI_MISFIT_OT
                          : !std::strcmp(m, "ot_power")    ? SFWI_MISFIT_OT_POWER
                          : !std::strcmp(m, "ot_alltrace") ? SFWI_MISFIT_OT_ALLTRACE
                                                           : SFWI_MISFIT_L2;
        } else if (!std::strcmp(argv[i], "--snapshots") && i + 2 < argc) {
            snap_k = std::atoi(argv[++i]);
            const char *f = argv[++i];
            snap_fmt = !std::strcmp(f, "f32") ? SFWI_SNAP_F32 : !std::strcmp(f, "bf16") ? SFWI_SNAP_BF16 : SFWI_SNAP_F16;
        } else if (!std::strcmp(argv[i], "--source") && i + 1 < argc) {
            const char *k = argv[++i];
            if (!std::strcmp(k, "vz"))
                source = SFWI_SOURCE_VZ_FORCE;
            else if (!std::strcmp(k, "txx_tzz"))
                source = SFWI_SOURCE_TXX_TZZ;
            else
                die("--source must be txx_tzz or vz");
        } else if (!std::strcmp(argv[i], "--gradient-only"))
            gradient_only = true;
        else if (!std::strcmp(argv[i], "--resume"))
            resume = true;
        else
            die("unknown argument");
    }
    if (stage != 1 && stage != 2) die("--stage must be 1 or 2");
    sfwi_para par;
    if (sfwi_para_read(argv[1], &par)) die("cannot read the parameter file");
    const int maxiter = iters >= 0 ? iters : par.maxiter;
    const int allnx = par.allnx, allnz = par.allnz, pml = par.pml;
    const size_t n = (size_t)allnx * allnz;
    mkdir(par.outdir, 0755);

    // shots of the record files (index_shot, main.cpp:76-165)
    int nt = 0, nsh = 0;
    float dt = 0;
    if (sfwi_su_index(par.rec_z, &nt, &dt, nullptr, 0, &nsh) || nsh < 1) die("cannot index the z records");
    std::vector<sfwi_su_shot> table(nsh);
    check(sfwi_su_index(par.rec_z, &nt, &dt, table.data(), nsh, &nsh), "index");
    int all_left = table[0].cx_min;
    for (auto &t : table) all_left = std::min(all_left, t.cx_min);
    std::printf("shots %d, nt %d, dt %g s\n", nsh, nt, dt);

    // per-shot geometry (main.cpp:585-625) and records
    std::vector<Shot> shots;
    int max_nx = 0;
    for (auto &t : table) {
        if (t.no < par.minshot || t.no > par.maxshot) continue;
        Shot s;
        s.gc.resize(t.ntr);
        s.rz.resize((size_t)t.ntr * nt);
        s.rx.resize((size_t)t.ntr * nt);
        if (sfwi_su_read(par.rec_z, t.pos, t.ntr, nt, s.rz.data(), s.gc.data()) ||
            sfwi_su_read(par.rec_x, t.pos, t.ntr, nt, s.rx.data(), nullptr))
            die("cannot read a shot gather");
        const int nx = (int)(t.cx_max / par.dx + 0.5f) - (int)(t.cx_min / par.dx + 0.5f) + 1;
        max_nx = std::max(max_nx, nx);
        s.d.nx = nx;
        s.d.isx = pml + (int)((t.sx - t.cx_min) / par.dx);
        s.d.isz = pml + par.sy;
        s.d.igz = pml + par.gy;
        s.d.ngx_left = t.cx_min;
        s.d.delta_left = (int)((t.cx_min - all_left) / par.dx);
        s.d.record_left_in_v = 0;
        s.d.ntr = t.ntr;
        shots.push_back(std::move(s));
    }
    if (shots.empty()) die("no shot in [minshot, maxshot]");
    if (par.rbc) die("rbc = 1 (the random boundary) is not provided");
    for (auto &s : shots) {  // pointers into the vectors, which no longer move
        s.d.gc = s.gc.data();
        s.d.rec_z = s.rz.data();
        s.d.rec_x = s.rx.data();
    }

    // models: vp, vs from the parameter file; rho = 2000 (main.cpp:1472-1475)
    std::vector<float> vp = read_model(par.vp, n), vs = read_model(par.vs, n), rho(n, 2000.f);
    std::vector<float> sou = ricker(nt, dt, par.f0);
    sfwi_handle *h = nullptr;
    check(sfwi_create(&h, stage, sou.data(), par.dx, par.dz, dt, max_nx + 2 * pml, allnz + 2 * pml, allnx, allnz, 1,
                      pml, nt, 4, shots[0].d.ntr),
          "sfwi_create");
    check(sfwi_set_misfit(h, misfit_kind), "misfit");
    if (snap_k > 0) check(sfwi_set_snapshots(h, snap_k, snap_fmt), "snapshots");
    check(sfwi_set_source(h, source), "source");
    // the parameter file's cpu_mem keeps the edge strips in host memory in
    // chunks of iointerval steps, the chunk length the reference's driver
    // passes to IMAGE_SINGLESHOT as ntt (sfwi-stage1/main.cpp:631)
    if (par.cpu_mem) check(sfwi_set_cpu_mem(h, 1, par.iointerval), "cpu_mem");

    std::vector<float> grad_pp(n), grad_ps(n), illum(n), cg_pp(n), cg_ps(n), cg_pp_old(n, 0.f), cg_ps_old(n, 0.f);
    std::vector<float> image_pp(n, 0.f), image_ps(n, 0.f);  // stage 2: model perturbation
    double beta_fenmu = 0.0, max_misfit = 0.0;  // CG state across iterations
    const std::string out = par.outdir;
    auto enqueue_all = [&]() {
        for (auto &s : shots) check(sfwi_enqueue_shot(h, &s.d), "enqueue");
    };
    // the state an iteration leaves for the next: stage 1 updates the model,
    // stage 2 the perturbation; both carry the CG direction and denominator
    float *model_a = stage == 1 ? vp.data() : image_pp.data(), *model_b = stage == 1 ? vs.data() : image_ps.data();
    int first_iter = 0;
    if (resume) {
        StateHeader hdr{};
        if (!read_state(out, &hdr, {model_a, model_b, cg_pp_old.data(), cg_ps_old.data()}, n))
            die("--resume: no readable state.bin in the output directory");
        if (hdr.stage != stage || hdr.allnx != allnx || hdr.allnz != allnz)
            die("--resume: state.bin is of another stage or grid");
        first_iter = hdr.next_iter;
        beta_fenmu = hdr.beta_fenmu;
        max_misfit = hdr.max_misfit;
        std::printf("resuming at iteration %d\n", first_iter);
    }

    for (int iter = first_iter; iter < std::max(maxiter, gradient_only ? 1 : 0); iter++) {
        if (stage == 1) {
            check(sfwi_gpu_buffer_vpvs(h, vp.data(), vs.data(), rho.data()), "model");
        } else {
            check(sfwi_gpu_buffer_vpvs(h, vp.data(), vs.data(), nullptr), "model");
            check(sfwi_gpu_buffer_m(h, image_pp.data(), image_ps.data()), "perturbation");
        }
        double misfit = 0.0;
        enqueue_all();
        check(sfwi_run(h, &misfit, nullptr), "gradient pass");
        check(sfwi_imagebuffer_resettozero(h, grad_pp.data(), grad_ps.data(), illum.data(), nullptr, nullptr, nullptr,
                                           nullptr),
              "gradients");
        if (iter == 0) max_misfit = misfit;
        {
            FILE *f = std::fopen((out + "/misfit.txt").c_str(), "a");
            if (f) {
                std::fprintf(f, "i = %d,misfit = %4.3e,rms = %f\n", iter, misfit, misfit / max_misfit);
                std::fclose(f);
            }
        }
        std::printf("iter %d misfit %.6e\n", iter, misfit);
        if (gradient_only) {
            write_model(out, "sum_grad_pp", iter, allnx, allnz, grad_pp.data());
            write_model(out, "sum_grad_ps", iter, allnx, allnz, grad_ps.data());
            write_model(out, "sum_illum", iter, allnx, allnz, illum.data());
            break;
        }
        // preconditioning, the conjugate-gradient direction and the update
        // (the reference's arithmetic, in libsfwi_host: sfwi_host.h)
        if (stage == 1) {
            write_model(out, "sum_grad_pp", iter, allnx, allnz, grad_pp.data());
            write_model(out, "sum_grad_ps", iter, allnx, allnz, grad_ps.data());
            write_model(out, "sum_illum", iter, allnx, allnz, illum.data());
            std::vector<float> d_pp(n), d_ps(n);
            sfwi_stage1_direction(allnx, allnz, iter, grad_pp.data(), grad_ps.data(), illum.data(), cg_pp_old.data(),
                                  cg_ps_old.data(), &beta_fenmu, cg_pp.data(), cg_ps.data(), d_pp.data(), d_ps.data());
            write_model(out, "sum_cg_pp", iter, allnx, allnz, cg_pp.data());
            // line search along the normalised direction, all shots and the
            // three trial models in one batch
            double m3[3] = {0.0, 0.0, 0.0};
            enqueue_all();
            check(sfwi_line_search_parabola(h, d_pp.data(), d_ps.data(), kStep1, kStep2, m3, nullptr), "line search");
            const double alpha = sfwi_stage1_alpha(m3[0], m3[1], m3[2], kStep1, kStep2);
            {
                FILE *f = std::fopen((out + "/misfit.txt").c_str(), "a");
                if (f) {
                    std::fprintf(f, "i = %d,alpha = %5.3e\n", iter, alpha);
                    std::fclose(f);
                }
            }
            std::printf("iter %d line search misfits %.17g %.17g %.17g alpha %.17g\n", iter, m3[0], m3[1], m3[2],
                        alpha);
            sfwi_stage1_update(allnx, allnz, alpha, d_pp.data(), d_ps.data(), vp.data(), vs.data());
            write_model(out, "vel_p", iter, allnx, allnz, vp.data());
            write_model(out, "vel_s", iter, allnx, allnz, vs.data());
        } else {
            sfwi_stage2_direction(allnx, allnz, iter, grad_pp.data(), grad_ps.data(), illum.data(), cg_pp_old.data(),
                                  cg_ps_old.data(), &beta_fenmu, cg_pp.data(), cg_ps.data());
            // the gradients as the reference writes them, zeroed above the cut
            write_model(out, "sum_grad_pp", iter, allnx, allnz, grad_pp.data());
            write_model(out, "sum_grad_ps", iter, allnx, allnz, grad_ps.data());
            write_model(out, "sum_cggrad_pp", iter, allnx, allnz, cg_pp.data());
            write_model(out, "sum_cggrad_ps", iter, allnx, allnz, cg_ps.data());
            write_model(out, "sum_illum", iter, allnx, allnz, illum.data());
            double fenzi = 0.0, fenmu = 0.0;
            enqueue_all();
            check(sfwi_line_search_exact(h, image_pp.data(), image_ps.data(), cg_pp.data(), cg_ps.data(), &fenzi, &fenmu,
                                         nullptr),
                  "step length");
            const double alpha = sfwi_stage2_update(allnx, allnz, fenzi, fenmu, cg_pp.data(), cg_ps.data(),
                                                    image_pp.data(), image_ps.data());
            std::printf("iter %d fenzi %.17g fenmu %.17g alpha %.17g\n", iter, fenzi, fenmu, alpha);
            write_model(out, "sum_image_pp", iter, allnx, allnz, image_pp.data());
            write_model(out, "sum_image_ps", iter, allnx, allnz, image_ps.data());
        }
        StateHeader hdr{};
        std::memcpy(hdr.magic, kStateMagic, 8);
        hdr.version = 1;
        hdr.stage = stage;
        hdr.next_iter = iter + 1;
        hdr.allnx = allnx;
        hdr.allnz = allnz;
        hdr.beta_fenmu = beta_fenmu;
        hdr.max_misfit = max_misfit;
        write_state(out, hdr, {model_a, model_b, cg_pp_old.data(), cg_ps_old.data()}, n);
    }
    sfwi_destroy(h);
    return 0;
}
