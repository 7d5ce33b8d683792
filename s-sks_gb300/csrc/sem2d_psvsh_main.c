/*
 * sem2d_psvsh_gb300 — drop-in replacement of the reference program
 * `sem2d_psvsh par=run.par` (semsyn/src/sem2d_psvsh.c:82-521) on one GB300.
 *
 * Same command line (getpar words), same input files, same outputs: with
 * plot_trace=1 it writes seis.u, seis.w and seis.v in the working directory,
 * nst records of ntrace float32 each (kirrecord_zhl, :2116-2160).  Extra
 * words choose the arithmetic, the device and, instead of the greenfile /
 * shgreenfile records, boundary records generated on the device:
 *   sks_precision=fp64|fp32c   (default fp64)
 *   sks_device=N               (default 0)
 *   sks_plane_wave=vs,p,f0[,sv_amp[,sh_amp]]
 *                              a plane SV/SH wave in the bottom medium
 *                              (sks_set_boundary_plane_wave; amplitudes 1, 0)
 *   sks_stack=FILE sks_wave=p,f0[,p_amp[,sv_amp[,sh_amp]]]
 *                              a plane wave through the layers listed in FILE,
 *                              one "vp vs rho thickness" line per medium from
 *                              the box's bottom medium down to the half-space
 *                              (sks_set_boundary_layered_wave; amplitudes 0, 1, 0)
 * Invoked as `sem2d_gb300` (or with psv_only=1) it behaves as the P-SV solver
 * semsyn/src/sem2d.c, which reads no SH boundary file.
 * Errors print a message and exit with status 1 instead of the reference's
 * exit(-1/-2/-3).
 */
#include "sks.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* up to n comma-separated numbers; returns how many were read, -1 on junk */
static int numbers(const char *s, double *v, int n)
{
    int k = 0;
    while (k < n && *s) {
        char *end;
        v[k] = strtod(s, &end);
        if (end == s) return -1;
        k++;
        if (*end == ',') s = end + 1;
        else if (*end == 0) s = end;
        else return -1;
    }
    return *s ? -1 : k;
}

/* the stack file: "vp vs rho thickness" per line, '#' comments */
static int read_stack(const char *path, sks_stack_layer_t **out, int *n)
{
    FILE *f = fopen(path, "r");
    char line[512];
    int cap = 8;
    sks_stack_layer_t *L;
    if (!f) return -1;
    L = (sks_stack_layer_t *)malloc(sizeof(*L) * cap);
    *n = 0;
    while (L && fgets(line, sizeof line, f)) {
        double v[4] = {0, 0, 0, 0};
        int k;
        char *h = strchr(line, '#');
        if (h) *h = 0;
        k = sscanf(line, "%lf %lf %lf %lf", v, v + 1, v + 2, v + 3);
        if (k <= 0) continue;
        if (k < 3) { free(L); fclose(f); return -2; }
        if (*n == cap) {
            sks_stack_layer_t *g = (sks_stack_layer_t *)realloc(L, sizeof(*L) * (cap *= 2));
            if (!g) { free(L); fclose(f); return -1; }
            L = g;
        }
        L[*n].vp = v[0]; L[*n].vs = v[1]; L[*n].rho = v[2]; L[*n].thickness = v[3];
        (*n)++;
    }
    fclose(f);
    if (!L) return -1;
    *out = L;
    return 0;
}

int main(int argc, char **argv)
{
    int precision = SKS_FP64, device = 0, i, rc, chunk = 1000, step = 0;
    const char **args = (const char **)calloc((size_t)argc + 2, sizeof(char *));
    int nargs = 0;
    sks_solver *s = NULL;
    sks_info_t info;
    const char *pw_word = NULL, *stack_word = NULL, *wave_word = NULL;
    double pw[5] = {0, 0, 0, 1.0, 0.0}, wv[5] = {0, 0, 0.0, 1.0, 0.0};
    sks_stack_layer_t *stack = NULL;
    int nstack = 0;
    FILE *fu = NULL, *fw = NULL, *fv = NULL;
    float *su, *sv, *sw;
    const char *prog = strrchr(argv[0], '/');
    prog = prog ? prog + 1 : argv[0];
    args[nargs++] = argv[0];
    for (i = 1; i < argc; i++) {
        if (!strncmp(argv[i], "sks_precision=", 14)) {
            precision = (!strcmp(argv[i] + 14, "fp32c") || !strcmp(argv[i] + 14, "1")) ? SKS_FP32C : SKS_FP64;
            continue;
        }
        if (!strncmp(argv[i], "sks_device=", 11)) { device = atoi(argv[i] + 11); continue; }
        if (!strncmp(argv[i], "sks_plane_wave=", 15)) { pw_word = argv[i] + 15; continue; }
        if (!strncmp(argv[i], "sks_stack=", 10)) { stack_word = argv[i] + 10; continue; }
        if (!strncmp(argv[i], "sks_wave=", 9)) { wave_word = argv[i] + 9; continue; }
        args[nargs++] = argv[i];
    }
    if (pw_word && (stack_word || wave_word)) {
        fprintf(stderr, "%s: sks_plane_wave and sks_stack/sks_wave exclude each other\n", prog);
        return 1;
    }
    if (pw_word && numbers(pw_word, pw, 5) < 3) {
        fprintf(stderr, "%s: sks_plane_wave=vs,p,f0[,sv_amp[,sh_amp]]: cannot read \"%s\"\n", prog, pw_word);
        return 1;
    }
    if (!stack_word != !wave_word) {
        fprintf(stderr, "%s: sks_stack=FILE and sks_wave=p,f0[,...] go together\n", prog);
        return 1;
    }
    if (wave_word && numbers(wave_word, wv, 5) < 2) {
        fprintf(stderr, "%s: sks_wave=p,f0[,p_amp[,sv_amp[,sh_amp]]]: cannot read \"%s\"\n", prog, wave_word);
        return 1;
    }
    if (stack_word) {
        const int r = read_stack(stack_word, &stack, &nstack);
        if (r || nstack < 2) {
            fprintf(stderr, "%s: %s: %s\n", prog, stack_word,
                    r == -1 ? "cannot read the stack file" : "needs \"vp vs rho thickness\" lines, 2 media at least");
            return 1;
        }
    }
    if (!strncmp(prog, "sem2d_gb300", 11)) args[nargs++] = "psv_only=1";
    rc = sks_open_par(nargs, args, precision, device, &s);
    if (rc) { fprintf(stderr, "%s: %s\n", prog, sks_last_error()); return 1; }
    sks_get_info(s, &info);
    printf("%s: nx=%d nz=%d eh=%.6f h=%.6f nst=%d inject=%d ntrace=%d materials=%d %s %s\n", prog,
           info.nx, info.nz, info.eh, info.h, info.nst, info.nt_inject, info.ntrace, info.nmat,
           info.anisotropic ? "anisotropic" : "isotropic", precision == SKS_FP64 ? "fp64" : "fp32c");
    if (pw_word) {
        const sks_plane_wave_t p = {pw[0], pw[1], pw[2], pw[3], pw[4]};
        rc = sks_set_boundary_plane_wave(s, &p);
    } else if (stack) {
        const sks_layered_wave_t w = {wv[0], wv[1], wv[2], wv[3], wv[4]};
        rc = sks_set_boundary_layered_wave(s, stack, nstack, &w);
        free(stack);
    } else {
        rc = sks_load_boundary_files(s);
    }
    if (rc) { fprintf(stderr, "%s: %s\n", prog, sks_last_error()); sks_destroy(s); return 1; }
    su = (float *)malloc(sizeof(float) * (size_t)chunk * (info.ntrace + 1));
    sv = (float *)malloc(sizeof(float) * (size_t)chunk * (info.ntrace + 1));
    sw = (float *)malloc(sizeof(float) * (size_t)chunk * (info.ntrace + 1));
    if (info.ntrace > 0) {
        fu = fopen("seis.u", "wb"); fw = fopen("seis.w", "wb"); fv = fopen("seis.v", "wb");
        if (!fu || !fw || !fv) { fprintf(stderr, "%s: cannot open seis.* for writing\n", prog); return 1; }
    }
    while (step < info.nst) {
        int n = sks_run(s, chunk, su, sv, sw);
        if (n < 0) { fprintf(stderr, "%s: %s\n", prog, sks_last_error()); sks_destroy(s); return 1; }
        if (n == 0) break;
        if (info.ntrace > 0) {
            int k;
            for (k = 0; k < n; k++) {   /* per step: u, then w, then v (kirrecord_zhl order) */
                fwrite(su + (size_t)k * info.ntrace, sizeof(float), info.ntrace, fu);
                fwrite(sw + (size_t)k * info.ntrace, sizeof(float), info.ntrace, fw);
                fwrite(sv + (size_t)k * info.ntrace, sizeof(float), info.ntrace, fv);
            }
        }
        step += n;
    }
    if (fu) { fclose(fu); fclose(fw); fclose(fv); }
    {
        /* snapshots as the reference's snapshot() writes them (sem2d.c:1667-1683) */
        int32_t dims[2] = {0, 0};
        float *buf;
        int k;
        sks_snapshot(s, 0, NULL, dims);
        buf = (float *)malloc(sizeof(float) * 2 * ((size_t)dims[0] * dims[1] + 1));
        for (k = 0; k < 26 && buf; k++) {
            char name[16];
            FILE *f;
            int ix, iz;
            if (sks_snapshot(s, k, buf, dims) < 0) continue;
            snprintf(name, sizeof name, "out%d", k + 1);
            if (!(f = fopen(name, "wt"))) { fprintf(stderr, "%s: cannot open %s\n", prog, name); return 1; }
            for (ix = 0; ix < dims[0]; ix++)
                for (iz = 0; iz < dims[1]; iz++) {
                    const float *q = buf + ((size_t)ix * dims[1] + iz) * 2;
                    fprintf(f, "%d %d %e %e\n", 2 * ix, 2 * iz, q[0], q[1]);
                }
            fclose(f);
        }
        free(buf);
    }
    printf("%s: SEM calculation finished, %d steps\n", prog, step);
    free(su); free(sv); free(sw); free(args);
    sks_destroy(s);
    return 0;
}
