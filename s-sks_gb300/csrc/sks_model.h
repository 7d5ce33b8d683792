/*
 * Host-side model of one SEM solve: everything the reference's main()
 * computes before its time loop (semsyn/src/sem2d_psvsh.c:82-416), in FP64,
 * laid out for the device.  Internal to the library.
 */
#ifndef SKS_MODEL_H
#define SKS_MODEL_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKS_MAX_N 6
/* snapshots the reference writes with plot_snap=1: out1..out26 at steps
 * startsnap + k*incresnap (sem2d_psvsh.c:483-510) */
#define SKS_NSNAP 26
#define SKS_MAT_STRIDE 16   /* 15 stiffness entries + rho per material */

typedef struct {
    /* par words (sem2d_psvsh.c:154-205) */
    int flat, nt, nex, nst, nfil, hpn, absorb, readpars, neh, atten, xtrace;
    int get_rec, plot_trace, idxplot, msource, semmodel_full, psv_only;
    int plot_snap, snap_start, snap_incre;   /* snapshots (sem2d_psvsh.c:149-150,202-204) */
    /* boundary taper with atten > 0 (sem2d_psvsh.c:95-98,176-178,236-240):
     * nh_att = neh*hpn factors exp(alpha n), alpha = log10(ass)/(nh log10(2.73)),
     * as the reference's floats and in FP64 */
    double ass;
    float ass_f;
    int nh_att;
    float *taper_f;
    double *taper_d;
    double dp, eh_par, sdt, xbeg, zbeg;
    float dp_f, eh_par_f, sdt_f, xbeg_f, zbeg_f;
    char greenfile[512], shgreenfile[512], raymodel[512], semmodel[512], rec_file[512];

    /* mesh (discret, sem2d_psvsh.c:534-606) */
    int nez, nx, nz;
    double eh, h;            /* FP64 element size / GLL spacing          */
    float eh_f, h_f;         /* the reference's float values (decisions) */

    /* materials: table of distinct materials + per-point index.
     * Row layout (16 doubles): the symmetric 5x5 block of the Voigt
     * stiffness on the strain list (e11, e12, e13, e23, e33) stored upper
     * triangle row by row: C11 C16 C15 C14 C13 | C66 C56 C46 C36 | C55 C45
     * C35 | C44 C34 | C33, then rho.  These are the only entries the 2-D
     * stress (d/dy = 0) touches (Stress_ij, sem2d_psvsh.c:1345-1380). */
    int nmat, mat_cap;
    double *mat;
    uint16_t *mat_id;        /* nx*nz, row-major, iz = 0 at the bottom   */
    int anisotropic;

    /* GLL tables (lagrange.c) and uniform Jacobian (sem2d_psvsh.c:279-300) */
    double gllp[SKS_MAX_N + 1], gllw[SKS_MAX_N + 1];
    double dlagP[(SKS_MAX_N + 1) * (SKS_MAX_N + 1)];  /* [j*(N+1)+i] = l'_i(xi_j) */
    double Je, JeI, Jb;

    /* lumped mass and Stacey matrix, per point, reference summation order */
    double *mass;            /* nx*nz */
    double *ab;              /* 3*nx*nz, zero off the absorbing edges */

    /* receivers: flat offsets iz*nx+ix (nx*nz addresses a point that
     * stays zero, as the reference's extra array element does) */
    int ntrace;
    int64_t *rec_off;

    /* boundary-trace schedule (interpl.c:16-91 with the shared ring of
     * sem2d_psvsh.c:430-431): for steps [0, nt_sem) four taps per family,
     * a record index (-1: a slot never filled, reads 0) and an FP64 weight */
    int nt_sem, mtotal, shtotal;
    int nrec_psv, nrec_sh;
    int32_t *tap_psv, *tap_sh;
    double *w_psv, *w_sh;
} sks_model;

/* status codes match include/sks.h; internal to the library */
__attribute__((visibility("hidden")))
int  sks_model_from_par(sks_model *m, int argc, const char *const *argv, char *err, size_t errlen);
__attribute__((visibility("hidden")))
void sks_model_free(sks_model *m);
/* 1 when a material row (the 15 stiffness entries, then rho) has the
 * isotropic pattern exactly: zero coupling entries, C11 = C33, C44 = C55 = C66 */
__attribute__((visibility("hidden")))
int sks_material_is_isotropic(const double *r);
__attribute__((visibility("hidden")))
int  sks_mesh_spacing(const char *raymodel, int flat, int nfil, float eh_par, int hpn, int *nez, float *eh_f,
                      float *h_f, char *err, size_t errlen);
__attribute__((visibility("hidden")))
int  sks_par_lookup(int argc, const char *const *argv, int n, const char *const *names, char **values, char *err,
                    size_t errlen);

/* Stacey boundary-point index (-1 off the absorbing edges): left column,
 * bottom row, right column, then top-row points 1..3N (sem2d_psvsh.c:1834-1892) */
static inline int64_t sks_stacey_index(int ix, int iz, int nx, int nz, int N)
{
    if (ix == 0) return iz;
    if (iz == 0) return (int64_t)nz + ix;
    if (ix == nx - 1) return (int64_t)nz + nx + iz;
    if (iz == nz - 1 && ix >= 1 && ix <= 3 * N) return 2 * (int64_t)nz + nx + ix;
    return -1;
}
static inline int64_t sks_stacey_count(int nx, int nz, int N) { return 2 * (int64_t)nz + nx + 3 * N + 1; }

#ifdef __cplusplus
}
#endif
#endif
