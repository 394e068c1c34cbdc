/* sfwi_host.h — host-side pieces of the SFWI drivers: SU record I/O, shot
 * indexing, the para_stage parameter files and the model-update arithmetic.  Plain C++ (no CUDA), built
 * into sfwi_gb300/lib/libsfwi_host.so and linked by the sfwi_fwi driver.
 *
 * SU traces are a 240-byte header followed by ns float32 samples, in the
 * byte order of the machine that wrote them (the reference freads them into
 * its header struct, sfwi-stage1/segy.h).  The fields used here sit at the
 * standard SU offsets: sx at byte 72, gx at 80 (int32, coordinates in the
 * model's length unit), ns at 114 and dt at 116 (uint16, microseconds).
 */
#ifndef SFWI_HOST_H
#define SFWI_HOST_H

#ifdef __cplusplus
extern "C" {
#endif

/* one shot of an SU file, as index_shot tabulates it
 * (sfwi-stage1/main.cpp:76-165): traces of a shot are consecutive and share sx */
typedef struct {
    int no;        /* 1-based shot number */
    int ntr;       /* traces */
    int sx;        /* source coordinate */
    int cx_min;    /* smallest of sx and the receivers' gx */
    int cx_max;    /* largest of sx and the receivers' gx */
    long long pos; /* index of the shot's first trace in the file */
} sfwi_su_shot;

/* Index an SU file: *nt and *dt (seconds) from the first header; up to
 * max_shots entries into shots; *nshots the number found.  Returns 0, or -1
 * when the file cannot be read. */
int sfwi_su_index(const char *path, int *nt, float *dt, sfwi_su_shot *shots, int max_shots, int *nshots);

/* Read ntr traces of nt samples starting at trace `pos` (read_shot_gather_su,
 * main.cpp:195-219): samples into dat[ntr][nt], gx into gc[ntr].  Returns 0
 * or -1. */
int sfwi_su_read(const char *path, long long pos, int ntr, int nt, float *dat, int *gc);

/* Write (append when `append` is nonzero) ntr traces dat[ntr][nt] with
 * source coordinate sx and receiver coordinates gc, sample interval dt in
 * seconds.  Returns 0 or -1. */
int sfwi_su_write(const char *path, int append, int ntr, int nt, float dt, int sx, const int *gc, const float *dat);

/* para_stage1 / para_stage2 (read by main, sfwi-stage1/main.cpp:1322-1350):
 *   dx dz pml allnx allnz minshot maxshot
 *   vp-file  vs-file  rho-file
 *   record-z.su  record-x.su  output-directory
 *   f0 maxiter iter_round1
 *   sy gy
 *   light rbc cpu_mem iointerval */
typedef struct {
    float dx, dz;
    int pml, allnx, allnz, minshot, maxshot;
    char vp[1024], vs[1024], rho[1024];
    char rec_z[1024], rec_x[1024], outdir[1024];
    float f0;
    int maxiter, iter_round1;
    int sy, gy;
    int light, rbc, cpu_mem, iointerval;
} sfwi_para;

/* Returns 0, or -1 when the file is missing or a field cannot be read. */
int sfwi_para_read(const char *path, sfwi_para *out);

/* ---- model-update arithmetic of the inversion drivers ----
 * The steps rank 1 of the reference performs between the gradient reduction
 * and the model broadcast, on [allnx][allnz] float arrays, with the
 * reference's operand types (float products and quotients, double
 * accumulators and CG/line-search scalars).  cut_layer = 26 and the alpha
 * clamp [-100, 300] are the reference's constants.  State carried from one
 * iteration to the next (the previous CG direction and beta's denominator)
 * lives in the caller's cg_old arrays and *beta_fenmu. */
#define SFWI_CUT_LAYER 26

/* Stage 1 (sfwi-stage1/main.cpp:687-750, :832-841): g = grad / illumination,
 * zero for z < 26; beta_fenzi = sum(grad . g) (float terms, double sum);
 * beta = beta_fenzi / *beta_fenmu (0 at iter 0); cg = g + beta cg_old;
 * cg_old = cg; *beta_fenmu = beta_fenzi; d = cg divided by the largest |cg|
 * of both components (normalize_all, main.cpp:35-49).  cg and d may be
 * NULL when not wanted.  Returns beta. */
double sfwi_stage1_direction(int allnx, int allnz, int iter, const float *grad_pp, const float *grad_ps,
                             const float *illum, float *cg_old_pp, float *cg_old_ps, double *beta_fenmu, float *cg_pp,
                             float *cg_ps, float *d_pp, float *d_ps);
/* Stage 1 step length (cal_step2, main.cpp:64-73, and the clamp, :1228-1237):
 * the vertex of the parabola through the misfits at steps 0, step1, step2,
 * clamped to [-100, 300]. */
double sfwi_stage1_alpha(double misfit0, double misfit1, double misfit2, float step1, float step2);
/* Stage 1 model update (main.cpp:1247-1264): vp -= alpha d_pp, vs -= alpha
 * d_ps (double products, stored as float); then every cell with z < 26 takes
 * the updated vp[0][0], vs[0][0]. */
void sfwi_stage1_update(int allnx, int allnz, double alpha, const float *d_pp, const float *d_ps, float *vp, float *vs);

/* Stage 2 (sfwi-stage2/main.cpp:646-703): for z >= 26 cg = grad / illum, for
 * z < 26 grad = cg = 0 (grad is written); beta_fenzi = sum(grad^2/illum) over
 * both components; beta, cg += beta cg_old, cg_old = cg, *beta_fenmu as in
 * stage 1.  Returns beta. */
double sfwi_stage2_direction(int allnx, int allnz, int iter, float *grad_pp, float *grad_ps, const float *illum,
                             float *cg_old_pp, float *cg_old_ps, double *beta_fenmu, float *cg_pp, float *cg_ps);
/* Stage 2 update (main.cpp:865-875): alpha = fenzi / fenmu; image -= alpha cg.
 * Returns alpha. */
double sfwi_stage2_update(int allnx, int allnz, double fenzi, double fenmu, const float *cg_pp, const float *cg_ps,
                          float *image_pp, float *image_ps);

#ifdef __cplusplus
}
#endif
#endif
