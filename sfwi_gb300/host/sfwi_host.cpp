// sfwi_host.cpp — SU record I/O, shot indexing, parameter files (see
// sfwi_host.h).
#include "sfwi_host.h"

#include <algorithm>
#include <climits>
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

}  // extern "C"
