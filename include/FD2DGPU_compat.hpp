/* FD2DGPU_compat.hpp — the class-shaped interface of SFWI's per-shot engine,
 * header-only, over the C ABI of sfwi_gb300.h.
 *
 * It stands in for the reference's FD2DGPU.cuh in a driver written against
 * it (sfwi-stage1/main.cpp, sfwi-stage2/main.cpp): the class FD2DGPU_ELASTIC
 * with the constructor, the public fields and the methods those drivers use,
 * and the free functions IMAGE_SINGLESHOT, CALCULATE_ALPHA_parabola_mb,
 * CALCULATE_ALPHA, OT, OT_power, OT_alltrace with the reference's signatures.
 * A driver includes this header in place of FD2DGPU.cuh and links
 * libsfwi_gb300.so; its calls keep their order and arguments.
 *
 * Differences a caller sees:
 *   - Errors.  The reference returns void and checks nothing.  Here a failed
 *     call throws sfwi_compat::error (a std::runtime_error carrying the
 *     SFWI_E* code and the library's message).
 *   - Stage.  Both reference programs name their engine FD2DGPU_ELASTIC, with
 *     different arithmetic (sfwi-stage1: background forward, adjoint
 *     direction +1; sfwi-stage2: Born forward, direction -1, density 2000).
 *     Define SFWI_COMPAT_STAGE to 1 or 2 before including this header to fix
 *     it; otherwise the first GPUbufferVPVS call decides, as the two drivers
 *     differ there: the three-argument form (vp, vs, rho) is stage 1's
 *     (sfwi-stage1/FD2DGPU.cuh:296), the two-argument form stage 2's
 *     (sfwi-stage2/FD2DGPU.cuh:297).  Any other call made first selects
 *     stage 1.
 *   - rbc (random boundary, cuRAND) is not provided: rbc = true throws.
 *     cpu_mem / ntt keep the edge strips in pinned host memory with a device
 *     ring of two ntt-step chunks (sfwi_set_cpu_mem), with the same values
 *     as strips kept on the device.
 *   - OT, OT_power and OT_alltrace are only declared in the reference
 *     (sfwi-stage1/FD2DGPU.cuh:23-25).  Here they are defined; the misfit
 *     depends on the sample interval, which their arguments do not carry, so
 *     they use the dt of the most recently constructed FD2DGPU_ELASTIC.
 *   - normalize and sign stay declarations, as in the reference: the drivers
 *     define normalize themselves (sfwi-stage1/main.cpp:24-32).
 */
#ifndef SFWI_FD2DGPU_COMPAT_HPP
#define SFWI_FD2DGPU_COMPAT_HPP

#include <cuda_runtime_api.h>  // cudaStream_t, as in the reference's record_copytoGPU

#include <stdexcept>
#include <string>

#include "sfwi_gb300.h"

#ifndef PI
#define PI 3.14159265358979  // FD2DGPU.cuh:7
#endif

namespace sfwi_compat {

class error : public std::runtime_error {
  public:
    error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

inline void check(int rc, const char *call) {
    if (rc != SFWI_OK) {
        const char *m = sfwi_last_error();
        throw error(rc, std::string(call) + ": " + (m ? m : "error"));
    }
}

// sample interval of the most recently constructed engine (for OT)
inline float &last_dt() {
    static float dt = 0.f;
    return dt;
}

}  // namespace sfwi_compat

// FD2DGPU_ELASTIC, sfwi-stage1/FD2DGPU.cuh:146-459 (sfwi-stage2/FD2DGPU.cuh:146-447):
// the members the stage drivers use.
class FD2DGPU_ELASTIC {
  public:
    // FD2DGPU.cuh:152-153; copies sou[nt]
    FD2DGPU_ELASTIC(const float *sou, const float dx1, const float dz1, const float dt1, const int nxpml1,
                    const int nzpml1, const int allnx1, const int allnz1, const int scale1, const int pml1,
                    const int nt1, const int nop1, int ntr1)
        : dx(dx1), dz(dz1), dt(dt1), nxpml(nxpml1), nzpml(nzpml1), allnx(allnx1), allnz(allnz1), scale(scale1),
          pml(pml1), nt(nt1), nop(nop1), ntr(ntr1), sou_(sou) {
        sfwi_compat::last_dt() = dt1;
#if defined(SFWI_COMPAT_STAGE)
        create(SFWI_COMPAT_STAGE);
#endif
    }
    ~FD2DGPU_ELASTIC() { sfwi_destroy(h_); }
    FD2DGPU_ELASTIC(const FD2DGPU_ELASTIC &) = delete;
    FD2DGPU_ELASTIC &operator=(const FD2DGPU_ELASTIC &) = delete;

    // sizes as the constructor received them
    const float dx, dz, dt;
    const int nxpml, nzpml, allnx, allnz, scale, pml, nt, nop;

    // public fields the drivers write before each shot (FD2DGPU.cuh:156-169,
    // :389-391; sfwi-stage1/main.cpp:619-625)
    int isx = 0, isz = 0;
    int igz = 0;
    float cmin = 0.f;
    int ntr;
    int delta_left = 0;
    int record_left_in_v = 0;
    int ngx_left = 0;

    // GPUbufferVPVS(vp_all, vs_all, rho_all), sfwi-stage1/FD2DGPU.cuh:296
    void GPUbufferVPVS(float *vp_all, float *vs_all, float *cpu_rho_all) {
        sfwi_compat::check(sfwi_gpu_buffer_vpvs(handle(1), vp_all, vs_all, cpu_rho_all), "GPUbufferVPVS");
    }
    // GPUbufferVPVS(vp_all, vs_all), sfwi-stage2/FD2DGPU.cuh:297 (density 2000)
    void GPUbufferVPVS(float *vp_all, float *vs_all) {
        sfwi_compat::check(sfwi_gpu_buffer_vpvs(handle(2), vp_all, vs_all, nullptr), "GPUbufferVPVS");
    }
    // GPUbufferM(pp, ps), FD2DGPU.cuh:237: the stage-2 model perturbation
    void GPUbufferM(float *pp, float *ps) {
        sfwi_compat::check(sfwi_gpu_buffer_m(handle(1), pp, ps), "GPUbufferM");
    }
    // bufferVpVsHtoD(ngx_min), FD2DGPU.cuh:297: window start of the next shot
    void bufferVpVsHtoD(const int ngx_min) {
        sfwi_compat::check(sfwi_buffer_vpvs_htod(handle(1), ngx_min), "bufferVpVsHtoD");
    }
    // record_copytoGPU(record_z, record_x, gc), FD2DGPU.cuh:387: observed
    // records [ntr][nt] of the next shot, with ntr the current field value.
    // The copy is synchronous whatever the stream, as in the reference.
    void record_copytoGPU(float *record, float *record_x, int *gc, cudaStream_t stream = 0) {
        (void)stream;
        push_geometry();
        sfwi_compat::check(sfwi_record_copy_to_gpu(h_, record, record_x, gc), "record_copytoGPU");
    }
    // imagebuffer_resettozero(...), FD2DGPU.cuh:248: copy the accumulated
    // gradients and illumination out, then zero them on the device
    void imagebuffer_resettozero(float *cpu_pp_grad, float *cpu_ps_grad, float *illuminaiton, float *b_cpu_pp_grad,
                                 float *b_cpu_ps_grad, float *b_cpu_pp_grad2, float *b_cpu_ps_grad2) {
        sfwi_compat::check(sfwi_imagebuffer_resettozero(handle(1), cpu_pp_grad, cpu_ps_grad, illuminaiton,
                                                        b_cpu_pp_grad, b_cpu_ps_grad, b_cpu_pp_grad2, b_cpu_ps_grad2),
                           "imagebuffer_resettozero");
    }

    // the C ABI handle behind this object, for the library's own calls
    // (batched shots, misfit choice, tile shapes); created on first use
    sfwi_handle *handle(int stage_if_new = 1) {
        if (!h_) create(stage_if_new);
        return h_;
    }
    // the public fields as the library's shot geometry
    void push_geometry() {
        sfwi_compat::check(sfwi_set_shot_geometry(handle(1), isx, isz, igz, ngx_left, delta_left, record_left_in_v, ntr),
                           "shot geometry");
    }

  private:
    void create(int stage) {
        sfwi_compat::check(
            sfwi_create(&h_, stage, sou_, dx, dz, dt, nxpml, nzpml, allnx, allnz, scale, pml, nt, nop, ntr),
            "FD2DGPU_ELASTIC");
    }
    const float *sou_;
    sfwi_handle *h_ = nullptr;
};

namespace sfwi_compat {
inline void no_random_boundary(bool rbc, const char *call) {
    if (rbc) throw error(SFWI_E_ARG, std::string(call) + ": the random boundary (rbc) is not provided");
}
}  // namespace sfwi_compat

// IMAGE_SINGLESHOT, sfwi-stage1/FD2DGPU.cuh:466-467: one shot-gradient of the
// shot described by the object's fields and its last record_copytoGPU.
// misfit += the shot's misfit; the gradients and the illumination accumulate
// on the device until imagebuffer_resettozero.  sxnum, nDim, myid, iter,
// cpu_mem and ntt keep the edge strips in host memory (sfwi_set_cpu_mem);
// iter_round1, maxiter, snapdir, image_pp/ps, the old gradients and
// misfit_ot take no part in the reference's live path and are not read.
inline void IMAGE_SINGLESHOT(FD2DGPU_ELASTIC &fdtdgpu, const int sxnum, const int nDim, const int myid, float *record,
                             float *record_x, int *gc, bool rbc, bool cpu_mem, int ntt, int iter, int iter_round1,
                             int maxiter, char *snapdir, float *image_pp, float *image_ps, float *cpu_pp_grad_old,
                             float *cpu_ps_grad_old, double &misfit, float *misfit_ot) {
    (void)sxnum, (void)nDim, (void)myid, (void)record, (void)record_x, (void)gc, (void)iter;
    (void)iter_round1, (void)maxiter, (void)snapdir, (void)image_pp, (void)image_ps, (void)cpu_pp_grad_old;
    (void)cpu_ps_grad_old, (void)misfit_ot;
    sfwi_compat::no_random_boundary(rbc, "IMAGE_SINGLESHOT");
    sfwi_compat::check(sfwi_set_cpu_mem(fdtdgpu.handle(), cpu_mem ? 1 : 0, ntt), "IMAGE_SINGLESHOT");
    fdtdgpu.push_geometry();
    sfwi_compat::check(sfwi_image_singleshot(fdtdgpu.handle(), &misfit), "IMAGE_SINGLESHOT");
}

// IMAGE_SINGLESHOT, sfwi-stage2/FD2DGPU.cuh:455-456: the stage-2 form (Born
// forward with the perturbation of GPUbufferM); misfit3 += the shot's misfit.
inline void IMAGE_SINGLESHOT(FD2DGPU_ELASTIC &fdtdgpu, const int sxnum, const int nDim, const int myid, float *record,
                             float *record_x, int *gc, bool rbc, bool cpu_mem, int ntt, int iter, char *snapdir,
                             float *image_pp, float *image_ps, float *cpu_pp_grad_old, float *cpu_ps_grad_old,
                             double &misfit3) {
    (void)sxnum, (void)nDim, (void)myid, (void)record, (void)record_x, (void)gc, (void)iter;
    (void)snapdir, (void)image_pp, (void)image_ps, (void)cpu_pp_grad_old, (void)cpu_ps_grad_old;
    sfwi_compat::no_random_boundary(rbc, "IMAGE_SINGLESHOT");
    sfwi_compat::check(sfwi_set_cpu_mem(fdtdgpu.handle(), cpu_mem ? 1 : 0, ntt), "IMAGE_SINGLESHOT");
    fdtdgpu.push_geometry();
    sfwi_compat::check(sfwi_image_singleshot(fdtdgpu.handle(), &misfit3), "IMAGE_SINGLESHOT");
}

// CALCULATE_ALPHA_parabola_mb, sfwi-stage1/FD2DGPU.cuh:471-472
// (FD2DGPU.cu:4819-5036): the L2 misfit of the current shot at the trial
// models vp - s*cpu_pp_grad_old, vs - s*cpu_ps_grad_old for s = 0, step_1,
// step_2, added to misfit_step0..2.  The window starts at column cmin, as
// the reference's bufferVpVsHtoD(cmin).  The *_ot outputs are left as they
// are (the reference's OT lines are commented out).
inline void CALCULATE_ALPHA_parabola_mb(FD2DGPU_ELASTIC &fdtdgpu, const int sxnum, const int nDim, const int myid,
                                        float *record, float *record_x, int *gc, bool rbc, bool cpu_mem, int ntt,
                                        int iter, float *image_pp, float *image_ps, float *cpu_pp_grad_old,
                                        float *cpu_ps_grad_old, double &misfit_step0, double &misfit_step1,
                                        double &misfit_step2, float step_1, float step_2, float *misfit_step0_ot,
                                        float *misfit_step1_ot, float *misfit_step2_ot) {
    (void)sxnum, (void)nDim, (void)myid, (void)record, (void)record_x, (void)gc, (void)cpu_mem, (void)ntt, (void)iter;
    (void)image_pp, (void)image_ps, (void)misfit_step0_ot, (void)misfit_step1_ot, (void)misfit_step2_ot;
    sfwi_compat::no_random_boundary(rbc, "CALCULATE_ALPHA_parabola_mb");
    fdtdgpu.bufferVpVsHtoD((int)fdtdgpu.cmin);
    fdtdgpu.push_geometry();
    sfwi_compat::check(sfwi_calculate_alpha_parabola_mb(fdtdgpu.handle(), cpu_pp_grad_old, cpu_ps_grad_old, step_1,
                                                        step_2, &misfit_step0, &misfit_step1, &misfit_step2),
                       "CALCULATE_ALPHA_parabola_mb");
}

// CALCULATE_ALPHA, sfwi-stage2/FD2DGPU.cuh:457 (FD2DGPU.cu:4576-4722): Born
// runs of the current shot with the perturbation image_pp/ps (residual r)
// and with the search direction cpu_pp_grad_old/cpu_ps_grad_old (scattered
// records q); fenzi += sum q.r, fenmu += sum q.q.
inline void CALCULATE_ALPHA(FD2DGPU_ELASTIC &fdtdgpu, const int sxnum, const int nDim, const int myid, float *record,
                            float *record_x, int *gc, char *snapdir, bool rbc, bool cpu_mem, int ntt, int iter,
                            float *image_pp, float *image_ps, float *cpu_pp_grad_old, float *cpu_ps_grad_old,
                            double &fenzi, double &fenmu) {
    (void)sxnum, (void)nDim, (void)myid, (void)record, (void)record_x, (void)gc, (void)snapdir, (void)cpu_mem;
    (void)ntt, (void)iter;
    sfwi_compat::no_random_boundary(rbc, "CALCULATE_ALPHA");
    fdtdgpu.bufferVpVsHtoD((int)fdtdgpu.cmin);
    fdtdgpu.push_geometry();
    sfwi_compat::check(sfwi_calculate_alpha(fdtdgpu.handle(), image_pp, image_ps, cpu_pp_grad_old, cpu_ps_grad_old,
                                            &fenzi, &fenmu),
                       "CALCULATE_ALPHA");
}

// OT / OT_power / OT_alltrace, sfwi-stage1/FD2DGPU.cuh:23-25 (declared only in
// the reference): 1D quadratic-Wasserstein misfit of [tracenum][length]
// gathers, misfit += W2, residual = (1/2) dW2/dcal; the sample interval is
// that of the most recently constructed FD2DGPU_ELASTIC.
inline void OT(float *record_obs_x, float *record_obs_z, float *record_cal_x, float *record_cal_z,
               float *record_residual_x, float *record_residual_z, int length, int tracenum, double &misfit) {
    sfwi_compat::check(sfwi_ot(record_obs_x, record_obs_z, record_cal_x, record_cal_z, record_residual_x,
                               record_residual_z, length, tracenum, sfwi_compat::last_dt(), &misfit),
                       "OT");
}
inline void OT_power(float *record_obs_x, float *record_obs_z, float *record_cal_x, float *record_cal_z,
                     float *record_residual_x, float *record_residual_z, int length, int tracenum, double &misfit) {
    sfwi_compat::check(sfwi_ot_power(record_obs_x, record_obs_z, record_cal_x, record_cal_z, record_residual_x,
                                     record_residual_z, length, tracenum, sfwi_compat::last_dt(), &misfit),
                       "OT_power");
}
inline void OT_alltrace(float *record_obs_x, float *record_obs_z, float *record_cal_x, float *record_cal_z,
                        float *record_residual_x, float *record_residual_z, int length, int tracenum, double &misfit) {
    sfwi_compat::check(sfwi_ot_alltrace(record_obs_x, record_obs_z, record_cal_x, record_cal_z, record_residual_x,
                                        record_residual_z, length, tracenum, sfwi_compat::last_dt(), &misfit),
                       "OT_alltrace");
}

// declared, not defined, as in FD2DGPU.cuh:21, :27 (the drivers define normalize)
int sign(float x);
void normalize(float *matrix, int length, int tracenum);

#endif
