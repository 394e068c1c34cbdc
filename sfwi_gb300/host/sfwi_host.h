/* sfwi_host.h — host-side pieces of the SFWI drivers: SU record I/O, shot
 * indexing and the para_stage parameter files.  Plain C++ (no CUDA), built
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

#ifdef __cplusplus
}
#endif
#endif
