// sfwi_host.cpp — SU record I/O, shot indexing, parameter files (see
// sfwi_host.h).
#include "sfwi_host.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr int kHeader = 240;
constexpr int kSx = 72, kGx = 80, kNs = 114, kDt = 116;

int32_t get_i32(const unsigned char *h, int off) {
    int32_t v;
    std::memcpy(&v, h + off, 4);
    return v;
}
uint16_t get_u16(const unsigned char *h, int off) {
    uint16_t v;
    std::memcpy(&v, h + off, 2);
    return v;
}
void put_i32(unsigned char *h, int off, int32_t v) { std::memcpy(h + off, &v, 4); }
void put_u16(unsigned char *h, int off, uint16_t v) { std::memcpy(h + off, &v, 2); }

struct File {
    FILE *f = nullptr;
    File(const char *p, const char *mode) : f(std::fopen(p, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

int sfwi_su_index(const char *path, int *nt, float *dt, sfwi_su_shot *shots, int max_shots, int *nshots) {
    File fp(path, "rb");
    if (!fp.f || !nt || !dt || !nshots) return -1;
    unsigned char h[kHeader];
    if (std::fread(h, kHeader, 1, fp.f) != 1) return -1;
    *nt = get_u16(h, kNs);
    *dt = get_u16(h, kDt) / 1000000.0f;
    if (*nt < 1) return -1;  // no samples: not a record file
    const long long trace_bytes = (long long)*nt * 4;
    // a file that is not a whole number of traces is truncated or corrupt
    if (std::fseek(fp.f, 0, SEEK_END) != 0) return -1;
    const long long size = std::ftell(fp.f);
    if (size < 0 || size % (kHeader + trace_bytes) != 0) return -1;
    std::fseek(fp.f, 0, SEEK_SET);
    int ns = 0;
    long long pos = 0;
    sfwi_su_shot cur{};
    bool open = false;
    while (std::fread(h, kHeader, 1, fp.f) == 1) {
        const int sx = get_i32(h, kSx), gx = get_i32(h, kGx);
        if (!open || sx != cur.sx) {
            if (open) {
                if (ns < max_shots) shots[ns] = cur;
                ns++;
            }
            cur = sfwi_su_shot{};
            cur.no = ns + 1;
            cur.sx = sx;
            cur.cx_min = INT_MAX;
            cur.cx_max = INT_MIN;
            cur.pos = pos;
            open = true;
        }
        cur.ntr++;
        cur.cx_min = std::min({cur.cx_min, sx, gx});
        cur.cx_max = std::max({cur.cx_max, sx, gx});
        pos++;
        if (std::fseek(fp.f, trace_bytes, SEEK_CUR) != 0) return -1;
    }
    if (open) {
        if (ns < max_shots) shots[ns] = cur;
        ns++;
    }
    *nshots = ns;
    return 0;
}

int sfwi_su_read(const char *path, long long pos, int ntr, int nt, float *dat, int *gc) {
    File fp(path, "rb");
    if (!fp.f || ntr < 0 || nt < 1) return -1;
    const long long trace_bytes = kHeader + (long long)nt * 4;
    if (std::fseek(fp.f, (long)(trace_bytes * pos), SEEK_SET) != 0) return -1;
    unsigned char h[kHeader];
    for (int i = 0; i < ntr; i++) {
        if (std::fread(h, kHeader, 1, fp.f) != 1) return -1;
        if (gc) gc[i] = get_i32(h, kGx);
        if (std::fread(dat + (size_t)i * nt, 4, nt, fp.f) != (size_t)nt) return -1;
    }
    return 0;
}

int sfwi_su_write(const char *path, int append, int ntr, int nt, float dt, int sx, const int *gc, const float *dat) {
    File fp(path, append ? "ab" : "wb");
    if (!fp.f || nt < 1 || nt > 65535) return -1;
    unsigned char h[kHeader];
    for (int i = 0; i < ntr; i++) {
        std::memset(h, 0, sizeof h);
        put_i32(h, kSx, sx);
        put_i32(h, kGx, gc[i]);
        put_u16(h, kNs, (uint16_t)nt);
        put_u16(h, kDt, (uint16_t)(dt * 1000000.0f + 0.5f));
        if (std::fwrite(h, kHeader, 1, fp.f) != 1) return -1;
        if (std::fwrite(dat + (size_t)i * nt, 4, nt, fp.f) != (size_t)nt) return -1;
    }
    return 0;
}

int sfwi_para_read(const char *path, sfwi_para *p) {
    File fp(path, "r");
    if (!fp.f || !p) return -1;
    std::memset(p, 0, sizeof *p);
    if (std::fscanf(fp.f, "%f %f %d %d %d %d %d", &p->dx, &p->dz, &p->pml, &p->allnx, &p->allnz, &p->minshot,
                    &p->maxshot) != 7)
        return -1;
    if (std::fscanf(fp.f, "%1023s %1023s %1023s", p->vp, p->vs, p->rho) != 3) return -1;
    if (std::fscanf(fp.f, "%1023s %1023s %1023s", p->rec_z, p->rec_x, p->outdir) != 3) return -1;
    if (std::fscanf(fp.f, "%f %d %d", &p->f0, &p->maxiter, &p->iter_round1) != 3) return -1;
    if (std::fscanf(fp.f, "%d %d", &p->sy, &p->gy) != 2) return -1;
    if (std::fscanf(fp.f, "%d %d %d %d", &p->light, &p->rbc, &p->cpu_mem, &p->iointerval) != 4) return -1;
    return 0;
}

// ---- model-update arithmetic (sfwi_host.h) ----
// Every float expression below keeps the reference's operand types: float
// products and quotients, promoted to double where the reference adds them to
// a double or multiplies them by one.  The library builds with
// -ffp-contract=off, so no product is fused into a sum on any machine.

// normalize_all, sfwi-stage1/main.cpp:35-49: both arrays divided by the
// largest |value| of the two (a float), as the reference does even when it is 0
static void normalize_pair(float *a, float *b, size_t n) {
    float m = 0.f;
    for (size_t i = 0; i < n; i++) m = std::fabs(a[i]) > m ? std::fabs(a[i]) : m;
    for (size_t i = 0; i < n; i++) m = std::fabs(b[i]) > m ? std::fabs(b[i]) : m;
    for (size_t i = 0; i < n; i++) {
        a[i] = a[i] / m;
        b[i] = b[i] / m;
    }
}

// cg = cg + beta cg_old (a double product, stored as float), then cg_old = cg
static void cg_recurrence(size_t n, double beta, float *cp, float *cs, float *cg_old_pp, float *cg_old_ps) {
    for (size_t k = 0; k < n; k++) {
        cp[k] = cp[k] + beta * cg_old_pp[k];
        cs[k] = cs[k] + beta * cg_old_ps[k];
    }
    std::memcpy(cg_old_pp, cp, n * sizeof(float));
    std::memcpy(cg_old_ps, cs, n * sizeof(float));
}

double sfwi_stage1_direction(int allnx, int allnz, int iter, const float *grad_pp, const float *grad_ps,
                             const float *illum, float *cg_old_pp, float *cg_old_ps, double *beta_fenmu, float *cg_pp,
                             float *cg_ps, float *d_pp, float *d_ps) {
    const size_t n = (size_t)allnx * allnz;
    std::vector<float> cp(n), cs(n);
    double beta_fenzi = 0.0;
    // sum_grad = grad / illumination (main.cpp:689-700), cut above layer 26
    // (:702-714), cg = sum_grad and beta_fenzi += grad . sum_grad (:717-724)
    for (int i = 0; i < allnx; i++)
        for (int j = 0; j < allnz; j++) {
            const size_t k = (size_t)i * allnz + j;
            float gp = grad_pp[k] / illum[k], gs = grad_ps[k] / illum[k];
            if (j < SFWI_CUT_LAYER) gp = gs = 0.f;
            cp[k] = gp;
            cs[k] = gs;
            beta_fenzi += grad_pp[k] * gp + grad_ps[k] * gs;
        }
    // beta (:729-735), the recurrence (:739-748), beta_fenmu (:750)
    const double beta = iter == 0 ? 0.0 : beta_fenzi / *beta_fenmu;
    cg_recurrence(n, beta, cp.data(), cs.data(), cg_old_pp, cg_old_ps);
    *beta_fenmu = beta_fenzi;
    if (cg_pp) std::memcpy(cg_pp, cp.data(), n * sizeof(float));
    if (cg_ps) std::memcpy(cg_ps, cs.data(), n * sizeof(float));
    // the line-search direction: cg normalised (:832-841; again at :1060-1063,
    // which leaves it unchanged: its largest |value| is then exactly 1)
    if (d_pp && d_ps) {
        normalize_pair(cp.data(), cs.data(), n);
        std::memcpy(d_pp, cp.data(), n * sizeof(float));
        std::memcpy(d_ps, cs.data(), n * sizeof(float));
    }
    return beta;
}

double sfwi_stage1_alpha(double misfit0, double misfit1, double misfit2, float step1, float step2) {
    // cal_step2, main.cpp:64-73 (float products of the steps, double sums)
    const double fenzi = (step1 * step1 - step2 * step2) * misfit0 + (step2 * step2) * misfit1 +
                         (-step1 * step1) * misfit2;
    const double fenmu = (step1 - step2) * misfit0 + (step2)*misfit1 + (-step1) * misfit2;
    double alpha = fenzi / fenmu / 2.0f;
    // main.cpp:1228-1237
    if (alpha > 300) alpha = 300;
    if (alpha < -100) alpha = -100;
    return alpha;
}

void sfwi_stage1_update(int allnx, int allnz, double alpha, const float *d_pp, const float *d_ps, float *vp,
                        float *vs) {
    const size_t n = (size_t)allnx * allnz;
    // main.cpp:1247-1253
    for (size_t k = 0; k < n; k++) {
        vp[k] = vp[k] - alpha * d_pp[k];
        vs[k] = vs[k] - alpha * d_ps[k];
    }
    // main.cpp:1257-1264: the layers above the cut take the corner value
    for (int i = 0; i < allnx; i++)
        for (int j = 0; j < allnz && j < SFWI_CUT_LAYER; j++) {
            vp[(size_t)i * allnz + j] = vp[0];
            vs[(size_t)i * allnz + j] = vs[0];
        }
}

double sfwi_stage2_direction(int allnx, int allnz, int iter, float *grad_pp, float *grad_ps, const float *illum,
                             float *cg_old_pp, float *cg_old_ps, double *beta_fenmu, float *cg_pp, float *cg_ps) {
    const size_t n = (size_t)allnx * allnz;
    double beta_fenzi = 0.0;
    // sfwi-stage2/main.cpp:646-671
    for (int i = 0; i < allnx; i++)
        for (int j = 0; j < allnz; j++) {
            const size_t k = (size_t)i * allnz + j;
            if (j >= SFWI_CUT_LAYER) {
                cg_pp[k] = grad_pp[k] / illum[k];
                cg_ps[k] = grad_ps[k] / illum[k];
            } else {
                grad_pp[k] = 0.f;
                grad_ps[k] = 0.f;
                cg_pp[k] = grad_pp[k];
                cg_ps[k] = grad_ps[k];
            }
            beta_fenzi += grad_pp[k] * grad_pp[k] / illum[k] + grad_ps[k] * grad_ps[k] / illum[k];
        }
    // :674-703
    const double beta = iter == 0 ? 0.0 : beta_fenzi / *beta_fenmu;
    cg_recurrence(n, beta, cg_pp, cg_ps, cg_old_pp, cg_old_ps);
    *beta_fenmu = beta_fenzi;
    return beta;
}

double sfwi_stage2_update(int allnx, int allnz, double fenzi, double fenmu, const float *cg_pp, const float *cg_ps,
                          float *image_pp, float *image_ps) {
    // sfwi-stage2/main.cpp:865-875
    const double alpha = fenzi / fenmu;
    const size_t n = (size_t)allnx * allnz;
    for (size_t k = 0; k < n; k++) {
        image_pp[k] = (image_pp[k] - alpha * cg_pp[k]);
        image_ps[k] = (image_ps[k] - alpha * cg_ps[k]);
    }
    return alpha;
}

}  // extern "C"
