/*
 * ORACLE — test infrastructure, not product code.
 *
 * CPU restatement of the semsyn SEM time-stepping path of the reference
 * solver `sem2d_psvsh` (semsyn/src/sem2d_psvsh.c) together with the set-up it
 * needs (par file, ray model, SEM model, GLL tables, mass, Stacey matrix,
 * receivers, GRT boundary-trace interpolation).  Only tests/, the smoke entry
 * and the CPU-baseline leg of bench.py may use it, and only as the checker.
 *
 * One source, two builds:
 *   -DORACLE_REAL=float   reproduces the reference's own float arithmetic,
 *                         including every float->double promotion of its C
 *                         expressions, so its seismograms equal the reference
 *                         binary's bit for bit (this is how the restatement is
 *                         pinned to the reference; built with
 *                         -ffp-contract=off so no FMA is formed);
 *   -DORACLE_REAL=double  the FP64 oracle: identical control flow, every real
 *                         quantity in double.
 * Control decisions with integer results (element count, layer row cuts,
 * receiver indices, number of injection steps, which boundary record is read
 * at which step) are taken with the reference's float arithmetic in both
 * builds, so both builds mesh and schedule exactly as the reference does.
 *
 * Extensions beyond the reference (used identically by the product):
 *   semmodel_full=1  each SEM-model layer line carries all 21 Voigt constants
 *                    (c11 c12 c13 c14 c15 c16 c22 c23 c24 c25 c26 c33 c34 c35
 *                    c36 c44 c45 c46 c55 c56 c66) then rho, so a tilted
 *                    symmetry axis can be represented (the reference keeps 13,
 *                    sem2d_psvsh.c:1528-1563);
 *   psv_only=1       no SH boundary file, SH traces are zero (the P-SV solver
 *                    semsyn/src/sem2d.c differs from sem2d_psvsh.c only there).
 * Undefined behaviour of the reference is given a definite meaning here:
 *   - the GRT guard reads g[-1] and g[mtotal] at the array ends
 *     (sem2d_psvsh.c:433-443); they are taken as 0;
 *   - lip() leaves its result unset for x equal to the last control point
 *     (sem2d_psvsh.c:831-846); the last segment is used;
 *   - a leading "ratio" SEM layer multiplies an uninitialised struct
 *     (sem2d_psvsh.c:758-763); it starts from zeros;
 *   - absorb=0 leaves the Stacey matrix unallocated while Absorbs() still
 *     runs (sem2d_psvsh.c:316-329,1027); it is taken as zero.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real;
#define IS_FLOAT (sizeof(real) == sizeof(float))

#define ORC_OK 0
#define ORC_ERR (-1)

static char orc_errbuf[512];
static int fail(const char *msg, const char *arg)
{
    snprintf(orc_errbuf, sizeof orc_errbuf, "%s%s%s", msg, arg ? ": " : "", arg ? arg : "");
    return ORC_ERR;
}
const char *oracle_last_error(void) { return orc_errbuf; }

/* ------------------------------------------------------------------------
 * Par-file arguments (Caltech getpar semantics, semsyn/src/getpar/lib/getpar.c
 * :101-190 setpar, :326-430 getpar, :510-548 par files): name=value words on
 * the command line, par=FILE splices a file of such words (# starts a
 * comment), and the LAST occurrence of a name wins.
 * ---------------------------------------------------------------------- */
typedef struct { char name[64]; char value[256]; } ParEntry;
typedef struct { ParEntry *e; int n, cap; } ParList;

static void par_add(ParList *pl, const char *name, const char *value)
{
    if (pl->n == pl->cap) {
        pl->cap = pl->cap ? 2 * pl->cap : 64;
        pl->e = (ParEntry *)realloc(pl->e, pl->cap * sizeof(ParEntry));
    }
    snprintf(pl->e[pl->n].name, 64, "%s", name);
    snprintf(pl->e[pl->n].value, 256, "%s", value);
    pl->n++;
}

static int par_file(ParList *pl, const char *fname, int level)
{
    char line[1024];
    FILE *f;
    if (level > 4) return fail("par files nested too deeply", fname);
    f = fopen(fname, "r");
    if (!f) return fail("cannot open par file", fname);
    while (fgets(line, sizeof line, f)) {
        char *p = line;
        for (;;) {
            char name[64], value[256];
            int n = 0, v = 0;
            char q1, q2;
            while (*p == ' ' || *p == '\t') p++;
            if (*p == '\0' || *p == '\n' || *p == '#') break;
            while (*p && *p != '=' && *p != ' ' && *p != '\t' && *p != '\n') {
                if (n < 63) name[n++] = *p;
                p++;
            }
            name[n] = '\0';
            if (*p == '=') p++;
            if (*p == '"' || *p == '\'') { q1 = q2 = *p++; } else { q1 = ' '; q2 = '\t'; }
            while (*p && *p != q1 && *p != q2 && *p != '\n') {
                if (v < 255) value[v++] = *p;
                p++;
            }
            value[v] = '\0';
            if (*p == '"' || *p == '\'') p++;
            par_add(pl, name, value);
            if (strcmp(name, "par") == 0 && par_file(pl, value, level + 1)) { fclose(f); return ORC_ERR; }
        }
    }
    fclose(f);
    return ORC_OK;
}

static int par_parse(ParList *pl, int argc, char **argv)
{
    int i;
    for (i = 1; i < argc; i++) {
        const char *a = argv[i];
        char name[64];
        int n = 0;
        while (*a == ' ' || *a == '\t') a++;
        while (*a && *a != '=') { if (n < 63) name[n++] = *a; a++; }
        name[n] = '\0';
        if (*a == '=') a++;
        par_add(pl, name, a);
        if (strcmp(name, "par") == 0 && par_file(pl, a, 1)) return ORC_ERR;
    }
    return ORC_OK;
}

static const char *par_get(const ParList *pl, const char *name)
{
    int i;
    for (i = pl->n - 1; i >= 0; i--)
        if (strcmp(pl->e[i].name, name) == 0) return pl->e[i].value;
    return NULL;
}

/* ------------------------------------------------------------------------
 * Solver state.  Real quantities have type `real`; *_f shadows hold the
 * reference's float values used for control decisions.
 * ---------------------------------------------------------------------- */
typedef struct { real u[3]; } Vec3;
typedef struct { real c[3][3][3][3]; real rho; } Cmat;

typedef struct {
    /* par */
    int flat, nt, nex, nst, nfil, hpn, absorb, readpars, neh, atten, xtrace;
    int get_rec, plot_trace, idxplot, msource, semmodel_full, psv_only;
    real dp, eh, xmin, sdt, xbeg, zbeg;
    float dp_f, eh_f, sdt_f, xbeg_f, zbeg_f;
    char greenfile[256], shgreenfile[256], raymodel[256], semmodel[256], rec_file[256];
    /* mesh */
    int nez, nx, nz;
    real h; float h_f;
    Cmat *mesh;
    /* GLL */
    real gllp[8], gllw[8], dlagP[64], dlagP_JeI[64], dlagP_Gllw[64];
    real Uni_Je, Uni_JeI, Uni_Jb;
    real *Mass, *Mass_dt2;
    Vec3 *Ab;
    /* receivers */
    int ntrace;
    long *rec_off;
    /* boundary traces */
    int mtotal, shtotal, nt_sem;
    float rdt_f; real rdt;
    real *grtuw, *grtuw0, *grtv, *grtv0;
    float *sy, *sy_sh;          /* [mtotal][4], [shtotal][4] as the file gives them */
    int ns[4];
    FILE *gf, *shf;
    /* wavefield */
    Vec3 *u, *u0, *u1, *K;
    /* snapshots (plot_snap, sem2d_psvsh.c:483-510): every second point of
     * (u[0], u[1]) at steps ist + k*incre, k < NSNAP */
    int plot_snap, ist, incre, nxs, nzs;
    float *snaps;               /* [NSNAP][nxs][nzs][2] */
    int snap_taken[32];
    /* boundary taper (atten > 0): nh = neh*hpn factors, ass at the edge */
    int nh_att;
    float ass_f; real ass;
    real *taper;
} Oracle;

#define NSNAP 26

/* ---------------- ray model (semsyn/src/readmodel.c:43-109) ------------- */
typedef struct {
    int jo, nb, lfinal;
    real *cc, *ss, *dd, *tth;      /* real-typed values */
    float *cc_f, *ss_f, *dd_f, *tth_f;  /* reference float values */
    int nrec;
} RayModel;

static double flatten_f(int layer, const float *tth)
{   /* readmodel.c:155-166 */
    int i;
    double thickness = 0.0;
    for (i = 0; i < layer; i++) thickness += tth[i];
    thickness += 0.5 * tth[layer];
    return 6371.0 / (6371.0 - thickness);
}
static double flatten_r(int layer, const real *tth)
{
    int i;
    double thickness = 0.0;
    for (i = 0; i < layer; i++) thickness += tth[i];
    thickness += 0.5 * tth[layer];
    return 6371.0 / (6371.0 - thickness);
}

static int read_raymodel(RayModel *rm, const char *fname, int flat)
{
    FILE *f = fopen(fname, "r");
    int j, n, k, nen0 = 0;
    if (!f) return fail("cannot open ray model", fname);
    if (fscanf(f, "%d %d", &rm->jo, &rm->nb) != 2 || rm->jo <= 0) { fclose(f); return fail("bad ray model header", fname); }
    rm->cc = (real *)calloc(rm->jo + 1, sizeof(real)); rm->ss = (real *)calloc(rm->jo + 1, sizeof(real));
    rm->dd = (real *)calloc(rm->jo + 1, sizeof(real)); rm->tth = (real *)calloc(rm->jo + 1, sizeof(real));
    rm->cc_f = (float *)calloc(rm->jo + 1, sizeof(float)); rm->ss_f = (float *)calloc(rm->jo + 1, sizeof(float));
    rm->dd_f = (float *)calloc(rm->jo + 1, sizeof(float)); rm->tth_f = (float *)calloc(rm->jo + 1, sizeof(float));
    for (j = 0; j < rm->jo; j++) {
        char t[4][64];
        if (fscanf(f, "%63s %63s %63s %63s", t[0], t[1], t[2], t[3]) != 4) { fclose(f); return fail("short ray model", fname); }
        rm->cc_f[j] = strtof(t[0], NULL); rm->ss_f[j] = strtof(t[1], NULL);
        rm->dd_f[j] = strtof(t[2], NULL); rm->tth_f[j] = strtof(t[3], NULL);
        if (IS_FLOAT) {
            rm->cc[j] = rm->cc_f[j]; rm->ss[j] = rm->ss_f[j]; rm->dd[j] = rm->dd_f[j]; rm->tth[j] = rm->tth_f[j];
        } else {
            rm->cc[j] = strtod(t[0], NULL); rm->ss[j] = strtod(t[1], NULL);
            rm->dd[j] = strtod(t[2], NULL); rm->tth[j] = strtod(t[3], NULL);
        }
    }
    if (flat == 0) {
        double *qf = (double *)malloc(rm->jo * sizeof(double)), *qr = (double *)malloc(rm->jo * sizeof(double));
        for (j = 0; j < rm->jo; j++) { qf[j] = flatten_f(j, rm->tth_f); qr[j] = flatten_r(j, rm->tth); }
        for (j = 0; j < rm->jo; j++) {
            rm->cc_f[j] = (float)(rm->cc_f[j] * qf[j]); rm->ss_f[j] = (float)(rm->ss_f[j] * qf[j]);
            rm->dd_f[j] = (float)(rm->dd_f[j] * qf[j]); rm->tth_f[j] = (float)(rm->tth_f[j] * qf[j]);
            rm->cc[j] = (real)(rm->cc[j] * qr[j]); rm->ss[j] = (real)(rm->ss[j] * qr[j]);
            rm->dd[j] = (real)(rm->dd[j] * qr[j]); rm->tth[j] = (real)(rm->tth[j] * qr[j]);
        }
        free(qf); free(qr);
    }
    /* the first ray's layer list gives nrec = na[nen[0]-2] (sem2d_psvsh.c:591) */
    if (fscanf(f, "%d", &rm->lfinal) != 1 || rm->lfinal < 1) { fclose(f); return fail("ray model has no rays", fname); }
    rm->nrec = -1;
    for (n = 0; n < rm->lfinal; n++) {
        int nen, v, cnt;
        if (fscanf(f, "%d", &nen) != 1 || nen < 2) { fclose(f); return fail("bad ray in ray model", fname); }
        if (n == 0) nen0 = nen;
        for (k = 0; k < nen; k++) {
            if (fscanf(f, "%d", &v) != 1) { fclose(f); return fail("short ray in ray model", fname); }
            if (n == 0 && k == nen0 - 2) rm->nrec = v;
        }
        if (fscanf(f, "%d", &cnt) != 1) { fclose(f); return fail("short ray in ray model", fname); }
        for (k = 0; k < nen; k++)
            if (fscanf(f, "%d", &v) != 1) { fclose(f); return fail("short ray in ray model", fname); }
    }
    fclose(f);
    if (rm->nrec < 1 || rm->nrec > rm->jo) return fail("ray model nrec out of range", fname);
    return ORC_OK;
}

/* ---------------- Voigt helpers (sem2d_psvsh.c:1528-1595) --------------- */
static int voigt(int i, int j)
{   /* 0..5 = 11 22 33 23 13 12 */
    if (i == j) return i;
    if ((i == 1 && j == 2) || (i == 2 && j == 1)) return 3;
    if ((i == 0 && j == 2) || (i == 2 && j == 0)) return 4;
    return 5;
}

/* full symmetric 6x6 (Voigt, 0-based) -> c_ijkl */
static void fill_cijkl(Cmat *m, const real C[6][6], real rho)
{
    int i, j, k, l;
    for (i = 0; i < 3; i++) for (j = 0; j < 3; j++) for (k = 0; k < 3; k++) for (l = 0; l < 3; l++)
        m->c[i][j][k][l] = C[voigt(i, j)][voigt(k, l)];
    m->rho = rho;
}

/* the 13 constants the reference keeps (Cijkl_3D) + rho */
typedef struct { real c11, c12, c13, c16, c22, c23, c26, c33, c36, c44, c45, c55, c66, rho; real full[21]; int is_full; } Layer13;

static void layer_to_6x6(const Layer13 *a, real C[6][6])
{
    int i, j;
    for (i = 0; i < 6; i++) for (j = 0; j < 6; j++) C[i][j] = 0;
    if (a->is_full) {
        int k = 0;
        for (i = 0; i < 6; i++) for (j = i; j < 6; j++) { C[i][j] = C[j][i] = a->full[k]; k++; }
        return;
    }
    C[0][0] = a->c11; C[0][1] = C[1][0] = a->c12; C[0][2] = C[2][0] = a->c13; C[0][5] = C[5][0] = a->c16;
    C[1][1] = a->c22; C[1][2] = C[2][1] = a->c23; C[1][5] = C[5][1] = a->c26;
    C[2][2] = a->c33; C[2][5] = C[5][2] = a->c36;
    C[3][3] = a->c44; C[3][4] = C[4][3] = a->c45; C[4][4] = a->c55; C[5][5] = a->c66;
}

/* lip(): piecewise-linear interface height (sem2d_psvsh.c:831-846), float */
static int lip_f(const float *an, const float *bn, int np, float x, float *out)
{
    int i;
    float dep = 0.f;
    if (x < an[0] || x > an[np - 1]) return ORC_ERR;
    if (np == 1) { *out = bn[0]; return ORC_OK; }
    dep = bn[np - 1];
    for (i = 0; i < np - 1; i++)
        if (x >= an[i] && x < an[i + 1]) {
            float s = (bn[i + 1] - bn[i]) / (an[i + 1] - an[i]);
            dep = bn[i] + s * (x - an[i]);
        }
    *out = dep;
    return ORC_OK;
}

/* discret(): mesh size and per-point material (sem2d_psvsh.c:534-828) */
static int discret(Oracle *o)
{
    RayModel rm;
    int i, j, k, nrec, nlay1, nlay2, nlaynum, inlay, iz1, iz2;
    float thickness_f = 0.f, thk2_f = 0.f;
    real thickness = 0;
    memset(&rm, 0, sizeof rm);
    if (read_raymodel(&rm, o->raymodel, o->flat)) return ORC_ERR;
    nrec = rm.nrec;
    if (o->nfil > nrec) {
        for (i = nrec; i < o->nfil; i++) { thickness_f += rm.tth_f[i]; thickness += rm.tth[i]; }
    } else {
        for (i = o->nfil - 1; i < nrec - 1; i++) { thickness_f += rm.tth_f[i]; thickness += rm.tth[i]; }
    }
    o->nez = (int)((thickness_f - 1.e-3) / o->eh_f);
    if (o->nez < 1) return fail("model thickness gives no element rows", NULL);
    o->eh_f = (float)((thickness_f - 1.e-3) / o->nez);
    o->eh = (real)((thickness - 1.e-3) / o->nez);
    o->nx = o->nex * o->hpn + 1;
    o->nz = o->nez * o->hpn + 1;
    o->h_f = o->eh_f / o->hpn;
    o->h = o->eh / o->hpn;
    o->mesh = (Cmat *)calloc((size_t)o->nx * o->nz, sizeof(Cmat));
    if (!o->mesh) return fail("cannot allocate mesh", NULL);

    /* 1-D model by grid rows, bottom to top */
    nlay1 = (o->nfil > nrec) ? nrec : nrec - 2;
    nlay2 = (o->nfil > nrec) ? o->nfil + 200 : o->nfil - 200;
    if (nlay2 < 0) nlay2 = 0;
    nlaynum = nlay2 - nlay1;
    if (nlaynum < 0) nlaynum = -nlaynum;
    nlaynum += 1;
    inlay = (o->nfil > nrec) ? 1 : -1;
    iz1 = 0;
    for (k = 0; k < nlaynum; k++) {
        Layer13 a;
        real C[6][6];
        Cmat tc;
        float ivp_f, ivs_f;
        real t_c11, t_c44, t_c13, ivp, ivs, iden;
        i = nlay1 + k * inlay;
        if (i < 0 || i >= rm.jo) break;
        thk2_f += rm.tth_f[i];
        iz2 = (int)((thk2_f + 1.e-3) / o->h_f) + 1;
        if (iz2 > o->nz - 1) iz2 = o->nz - 1;
        if (iz2 < iz1) break;
        (void)ivp_f; (void)ivs_f;
        ivp = rm.cc[i] * rm.cc[i]; ivs = rm.ss[i] * rm.ss[i]; iden = rm.dd[i];
        t_c11 = ivp * iden; t_c44 = ivs * iden;
        t_c13 = (real)(t_c11 - 2.0 * t_c44);
        memset(&a, 0, sizeof a);
        a.c11 = t_c11; a.c12 = t_c13; a.c13 = t_c13; a.c16 = 0;
        a.c22 = t_c11; a.c23 = t_c13; a.c26 = 0; a.c33 = t_c11; a.c36 = 0;
        a.c44 = t_c44; a.c45 = 0; a.c55 = t_c44; a.c66 = t_c44;
        layer_to_6x6(&a, C);
        fill_cijkl(&tc, C, iden);
        for (j = iz1; j <= iz2; j++) {
            int ix;
            for (ix = 0; ix < o->nx; ix++) o->mesh[(size_t)j * o->nx + ix] = tc;
        }
        iz1 = iz2 + 1;
        if (iz2 == o->nz - 1) break;
    }

    /* SEM model overrides, per grid column (sem2d_psvsh.c:703-799) */
    if (o->readpars == 1) {
        FILE *f = fopen(o->semmodel, "r");
        int nll, firstlayer = 0, ix;
        Layer13 *L;
        int *np, *ratio;
        float **an, **bn;
        Layer13 ap;
        if (!f) return fail("cannot open SEM model", o->semmodel);
        if (fscanf(f, "%d", &nll) != 1) { fclose(f); return fail("bad SEM model header", o->semmodel); }
        if (nll < 0) { firstlayer = 1; nll = -nll; }
        if (nll == 0) { fclose(f); return fail("SEM model has no layers", o->semmodel); }
        L = (Layer13 *)calloc(nll, sizeof(Layer13));
        np = (int *)calloc(nll, sizeof(int)); ratio = (int *)calloc(nll, sizeof(int));
        an = (float **)calloc(nll, sizeof(float *)); bn = (float **)calloc(nll, sizeof(float *));
        for (j = 0; j < nll; j++) {
            char t[32][64];
            int nv = o->semmodel_full ? 22 : 14, q;
            if (fscanf(f, "%d", &np[j]) != 1) { fclose(f); return fail("short SEM model", o->semmodel); }
            for (q = 0; q < nv; q++)
                if (fscanf(f, "%63s", t[q]) != 1) { fclose(f); return fail("short SEM model", o->semmodel); }
#define RV(s) (IS_FLOAT ? (real)strtof((s), NULL) : (real)strtod((s), NULL))
            if (o->semmodel_full) {
                for (q = 0; q < 21; q++) L[j].full[q] = RV(t[q]);
                L[j].rho = RV(t[21]);
                L[j].is_full = 1;
            } else {
                L[j].c11 = RV(t[0]); L[j].c12 = RV(t[1]); L[j].c13 = RV(t[2]); L[j].c16 = RV(t[3]);
                L[j].c22 = RV(t[4]); L[j].c23 = RV(t[5]); L[j].c26 = RV(t[6]); L[j].c33 = RV(t[7]);
                L[j].c36 = RV(t[8]); L[j].c44 = RV(t[9]); L[j].c45 = RV(t[10]); L[j].c55 = RV(t[11]);
                L[j].c66 = RV(t[12]); L[j].rho = RV(t[13]);
            }
#undef RV
            if (np[j] < 0) { ratio[j] = 1; np[j] = -np[j]; }
            if (np[j] < 1 || np[j] > 1000) { fclose(f); return fail("SEM model control-point count out of range", o->semmodel); }
            an[j] = (float *)calloc(np[j], sizeof(float)); bn[j] = (float *)calloc(np[j], sizeof(float));
            for (i = 0; i < np[j]; i++) if (fscanf(f, "%f", &an[j][i]) != 1) { fclose(f); return fail("short SEM model", o->semmodel); }
            for (i = 0; i < np[j]; i++) if (fscanf(f, "%f", &bn[j][i]) != 1) { fclose(f); return fail("short SEM model", o->semmodel); }
        }
        fclose(f);
        memset(&ap, 0, sizeof ap);
        for (ix = 0; ix < o->nx; ix++) {
            float x = ix * o->h_f, dep;
            iz1 = 0;
            if (firstlayer == 1) {
                if (lip_f(an[0], bn[0], np[0], x, &dep)) return fail("SEM model out of range", o->semmodel);
                iz1 = (int)((dep + 1.e-3) / o->h_f);
            }
            if (iz1 < 0) iz1 = 0;
            for (j = firstlayer; j < nll; j++) {
                real C[6][6];
                Cmat tc;
                int iz;
                if (lip_f(an[j], bn[j], np[j], x, &dep)) return fail("SEM model out of range", o->semmodel);
                iz2 = (int)((dep + 1.e-3) / o->h_f);
                if (iz2 > o->nz - 1) iz2 = o->nz - 1;
                if (ratio[j] == 1) {
                    if (L[j].is_full) {
                        int q;
                        for (q = 0; q < 21; q++) ap.full[q] *= L[j].full[q];
                        ap.is_full = 1;
                    } else {
                        ap.c11 *= L[j].c11; ap.c12 *= L[j].c12; ap.c13 *= L[j].c13; ap.c16 *= L[j].c16;
                        ap.c22 *= L[j].c22; ap.c23 *= L[j].c23; ap.c26 *= L[j].c26; ap.c33 *= L[j].c33;
                        ap.c36 *= L[j].c36; ap.c44 *= L[j].c44; ap.c45 *= L[j].c45; ap.c55 *= L[j].c55;
                        ap.c66 *= L[j].c66;
                    }
                    ap.rho *= L[j].rho;
                } else {
                    ap = L[j];
                }
                layer_to_6x6(&ap, C);
                fill_cijkl(&tc, C, ap.rho);
                for (iz = iz1; iz <= iz2; iz++) o->mesh[(size_t)iz * o->nx + ix] = tc;
                iz1 = iz2 + 1;
            }
        }
        for (j = 0; j < nll; j++) { free(an[j]); free(bn[j]); }
        free(an); free(bn); free(L); free(np); free(ratio);
    }
    free(rm.cc); free(rm.ss); free(rm.dd); free(rm.tth);
    free(rm.cc_f); free(rm.ss_f); free(rm.dd_f); free(rm.tth_f);
    return ORC_OK;
}

/* ---------------- GLL / Lagrange (lagrange.c:20-67, 105-131, 256-366) ---- */
static real legendre(int n, real x)
{
    real pn = 1, p0, p1, pn1, pn2;
    int i;
    if (n == 0) return 1;
    if (n == 1) return x;
    p0 = 1; pn2 = p0; p1 = x; pn1 = p1;
    for (i = 2; i <= n; i++) {
        pn = ((2 * i - 1) * x * pn1 - (i - 1) * pn2) / i;
        pn2 = pn1; pn1 = pn;
    }
    return pn;
}

static int gll_points(int np, real *g)
{
    if (np < 3 || np > 6) return fail("hpn must be 3..6", NULL);
    if (np == 3) { g[0] = -1.; g[1] = (real)-sqrt(1 / 5.); g[2] = (real)sqrt(1 / 5.); g[3] = 1.; }
    if (np == 4) { g[0] = -1.; g[1] = (real)-sqrt(15. / 35.); g[2] = 0.; g[3] = (real)sqrt(15. / 35.); g[4] = 1.; }
    if (np == 5 || np == 6) {
        /* roots of P_N'(x) = a x^4 + c x^2 + e (lagrange.c:349-366), with the
         * reference's float coefficients and mixed float/double evaluation */
        real a = (np == 5) ? 315. : 1386., c = (np == 5) ? -210. : -1260., e = (np == 5) ? 15. : 210.;
        real r1 = (real)-sqrt((-c + sqrt(c * c - 4 * a * e)) / 2 / a);
        real r2 = (real)-sqrt((-c - sqrt(c * c - 4 * a * e)) / 2 / a);
        g[0] = -1.;
        if (np == 5) { g[1] = r1; g[2] = r2; g[3] = -r2; g[4] = -r1; g[5] = 1.; }
        else { g[1] = r1; g[2] = r2; g[3] = 0.; g[4] = -r2; g[5] = -r1; g[6] = 1.; }
    }
    return ORC_OK;
}

static void gll_weights(const real *g, int np, real *w)
{
    int i;
    for (i = 0; i <= np; i++) {
        if (i == 0 || i == np) w[i] = (real)(2. / (np * (np + 1)));
        else {
            real t = legendre(np, g[i]);
            real den = np * (np + 1) * t * t;
            w[i] = (real)(2. / den);
        }
    }
}

static real dlag(int Na, int alpha, const real *g, real x)
{
    int i, k;
    real value = 0, down = 1.0, LNi;
    for (i = 0; i <= Na; i++) if (i != alpha) down = down * (g[alpha] - g[i]);
    for (i = 0; i <= Na; i++) {
        LNi = 1;
        if (i != alpha) {
            for (k = 0; k <= Na; k++) if (k != alpha && k != i) LNi = LNi * (x - g[k]);
            value = value + LNi;
        }
    }
    return value / down;
}

/* ---------------- mass and Stacey (sem2d_psvsh.c:1042-1128) -------------- */
static void mass_matrix(Oracle *o)
{
    int i, j, m, n, N = o->hpn;
    size_t np = (size_t)o->nx * o->nz;
    for (i = 0; (size_t)i < np; i++) o->Mass[i] = 0;
    for (i = 0; i < o->nex; i++)
        for (j = 0; j < o->nez; j++)
            for (m = 0; m <= N; m++) {
                real rx = o->gllw[m];
                for (n = 0; n <= N; n++) {
                    real rz = o->gllw[n];
                    size_t idx = (size_t)(j * N + n) * o->nx + i * N + m;
                    o->Mass[idx] = o->Mass[idx] + rx * rz * o->Uni_Je * o->mesh[idx].rho;
                }
            }
    for (i = 0; (size_t)i < np; i++) o->Mass_dt2[i] = o->sdt * o->sdt / o->Mass[i];
}

static void ab_add(real *a, real w, real rho, real v, real Jb, real sdt)
{
    real prod = w * rho * v * Jb * sdt;
    *a = (real)((double)*a + prod / 2.);
}

static void absorb_matrix(Oracle *o)
{
    int ez, ex, be, al, N = o->hpn;
    for (ez = 0; ez < o->nez; ez++)
        for (be = 0; be <= N; be++) {
            size_t idx = (size_t)(ez * N + be) * o->nx;
            const Cmat *m = &o->mesh[idx];
            real vp = (real)sqrt(m->c[0][0][0][0] / m->rho), vs = (real)sqrt(m->c[1][2][1][2] / m->rho);
            ab_add(&o->Ab[idx].u[0], o->gllw[be], m->rho, vp, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[1], o->gllw[be], m->rho, vs, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[2], o->gllw[be], m->rho, vs, o->Uni_Jb, o->sdt);
        }
    for (ex = 0; ex < o->nex; ex++)
        for (al = 0; al <= N; al++) {
            size_t idx = (size_t)ex * N + al;
            const Cmat *m = &o->mesh[idx];
            real vp = (real)sqrt(m->c[0][0][0][0] / m->rho), vs = (real)sqrt(m->c[1][2][1][2] / m->rho);
            ab_add(&o->Ab[idx].u[0], o->gllw[al], m->rho, vs, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[1], o->gllw[al], m->rho, vs, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[2], o->gllw[al], m->rho, vp, o->Uni_Jb, o->sdt);
        }
    for (ez = 0; ez < o->nez; ez++)
        for (be = 0; be <= N; be++) {
            size_t idx = (size_t)(ez * N + be) * o->nx + o->nx - 1;
            const Cmat *m = &o->mesh[idx];
            real vp = (real)sqrt(m->c[0][0][0][0] / m->rho), vs = (real)sqrt(m->c[1][2][1][2] / m->rho);
            ab_add(&o->Ab[idx].u[0], o->gllw[be], m->rho, vp, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[1], o->gllw[be], m->rho, vs, o->Uni_Jb, o->sdt);
            ab_add(&o->Ab[idx].u[2], o->gllw[be], m->rho, vs, o->Uni_Jb, o->sdt);
        }
}

/* ---------------- stiffness (sem2d_psvsh.c:1173-1487) -------------------- */
static void stiff_matrix(Oracle *o)
{
    int ex, ez, alpha, beta, i, N = o->hpn, N1 = o->hpn + 1, nx = o->nx;
    size_t np = (size_t)o->nx * o->nz, g;
    real F0[64][3], F2[64][3];
    const Vec3 *p = o->u;
    for (g = 0; g < np; g++) o->K[g].u[0] = o->K[g].u[1] = o->K[g].u[2] = 0;
    for (ex = 0; ex < o->nex; ex++)
        for (ez = 0; ez < o->nez; ez++) {
            for (alpha = 0; alpha <= N; alpha++)
                for (beta = 0; beta <= N; beta++) {
                    size_t idx = (size_t)(ez * N + beta) * nx + ex * N + alpha;
                    const Cmat *m = &o->mesh[idx];
                    real d[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                    real T[3][3];
                    int th, j;
                    for (th = 0; th <= N; th++) {
                        size_t q = (size_t)(ez * N + beta) * nx + ex * N + th;
                        real D = o->dlagP_JeI[alpha * N1 + th];
                        d[0][0] = d[0][0] + p[q].u[0] * D;
                        d[1][0] = d[1][0] + p[q].u[1] * D;
                        d[2][0] = d[2][0] + p[q].u[2] * D;
                    }
                    for (th = 0; th <= N; th++) {
                        size_t q = (size_t)(ez * N + th) * nx + ex * N + alpha;
                        real D = o->dlagP_JeI[beta * N1 + th];
                        d[0][2] = d[0][2] + p[q].u[0] * D;
                        d[1][2] = d[1][2] + p[q].u[1] * D;
                        d[2][2] = d[2][2] + p[q].u[2] * D;
                    }
                    for (i = 0; i < 3; i++)
                        for (j = 0; j < 3; j += 2) {
                            real s;
                            if (i == 1 && j == 1) { T[i][j] = 0; continue; }
                            s = m->c[i][j][0][0] * d[0][0];
                            s += m->c[i][j][0][1] * (d[0][1] + d[1][0]);
                            s += m->c[i][j][0][2] * (d[2][0] + d[0][2]);
                            s += m->c[i][j][1][1] * d[1][1];
                            s += m->c[i][j][1][2] * (d[1][2] + d[2][1]);
                            s += m->c[i][j][2][2] * d[2][2];
                            T[i][j] = s;
                        }
                    for (i = 0; i < 3; i++) {
                        F0[beta * N1 + alpha][i] = T[i][0] * o->Uni_JeI;
                        F2[beta * N1 + alpha][i] = T[i][2] * o->Uni_JeI;
                    }
                }
            for (alpha = 0; alpha <= N; alpha++)
                for (beta = 0; beta <= N; beta++) {
                    size_t idx = (size_t)(ez * N + beta) * nx + ex * N + alpha;
                    for (i = 0; i < 3; i++) {
                        real it0 = 0, it2 = 0, a;
                        int al, be;
                        for (al = 0; al <= N; al++) it0 = it0 + F0[beta * N1 + al][i] * o->dlagP_Gllw[al * N1 + alpha];
                        for (be = 0; be <= N; be++) it2 = it2 + F2[be * N1 + alpha][i] * o->dlagP_Gllw[be * N1 + beta];
                        a = (it0 * o->gllw[beta] + it2 * o->gllw[alpha]) * o->Uni_Je;
                        o->K[idx].u[i] += a;
                    }
                }
        }
}

/* ---------------- time update (sem2d_psvsh.c:1004-1028, 1834-1892) ------- */
static void absorb_point(Oracle *o, size_t gn, real dt2)
{
    int k;
    for (k = 0; k < 3; k++) {
        real coe = o->Mass[gn] + o->Ab[gn].u[k];
        real coe1 = o->Mass[gn] - o->Ab[gn].u[k];
        real t1 = -dt2 * o->K[gn].u[k];
        double num = (double)t1 + 2. * (double)o->Mass[gn] * (double)o->u[gn].u[k];
        real t3 = coe1 * o->u0[gn].u[k];
        o->u1[gn].u[k] = (real)((num - (double)t3) / (double)coe);
    }
}

static void time_update(Oracle *o)
{
    size_t np = (size_t)o->nx * o->nz, i;
    int k, nx = o->nx, nz = o->nz;
    real dt2 = o->sdt * o->sdt;
    for (k = 0; k < 3; k++)
        for (i = 0; i < np; i++) {
            real t1 = -o->Mass_dt2[i] * o->K[i].u[k];
            o->u1[i].u[k] = (real)((double)t1 + 2. * (double)o->u[i].u[k] - (double)o->u0[i].u[k]);
        }
    for (i = 0; i < (size_t)nz; i++) absorb_point(o, i * nx, dt2);
    for (i = 0; i < (size_t)nx; i++) absorb_point(o, i, dt2);
    for (i = 0; i < (size_t)nz; i++) absorb_point(o, i * nx + nx - 1, dt2);
    for (i = 1; i < (size_t)(3 * o->hpn + 1) && i < (size_t)nx; i++) absorb_point(o, (size_t)(nz - 1) * nx + i, dt2);
}

/* ---------------- boundary taper (sem2d_psvsh.c:1724-1738, 1780-1822) ---- */
/* atten_taper: taper[n] = exp(alpha n), alpha = log10(ass) / (nh log10(2.73));
 * the float build rounds each factor to float as the reference stores it */
static int taper_table(Oracle *o)
{
    int n, nh = o->nh_att;
    o->taper = (real *)malloc(sizeof(real) * (size_t)(nh > 0 ? nh : 1));
    if (!o->taper) return fail("cannot allocate the taper", NULL);
    if (IS_FLOAT) {
        const double alpha = 1.0 / nh * log10((double)o->ass_f) / log10(2.73);
        for (n = 0; n < nh; n++) o->taper[n] = (real)(float)exp((double)(alpha * n));
    } else {
        const double alpha = 1.0 / nh * log10((double)o->ass) / log10(2.73);
        for (n = 0; n < nh; n++) o->taper[n] = (real)exp(alpha * n);
    }
    return ORC_OK;
}

/* atten_wave2: u^{n+1} scaled in the bottom rows (atten > 0), then the left
 * (> 1) and right (> 2) columns above them, then the top rows between those
 * columns (> 3), one multiplication per zone in that order */
static void taper_wave(Oracle *o)
{
    const int nh = o->nh_att, nx = o->nx, nz = o->nz;
    int ix, iz, k;
    for (k = 0; k < 3; k++)
        for (ix = 0; ix < nx; ix++)
            for (iz = 0; iz < nz; iz++) {
                real *p = &o->u1[(size_t)iz * nx + ix].u[k];
                if (o->atten > 0 && iz < nh) *p *= o->taper[nh - iz - 1];
                if (o->atten > 1 && ix < nh && iz >= nh) *p *= o->taper[nh - ix - 1];
                if (o->atten > 2 && ix >= nx - nh && iz >= nh) *p *= o->taper[ix - nx + nh];
                if (o->atten > 3 && iz >= nz - nh && ix < nx - nh && ix >= nh) *p *= o->taper[iz - nz + nh];
            }
}

/* ---------------- GRT boundary injection (sem2d_psvsh.c:1953-2111) ------- */
static void grt_interface_set(Oracle *o)
{
    int i, m, N = o->hpn, nx = o->nx, nz = o->nz, nbl = o->neh * o->hpn;
    for (i = 0; i < nx; i++) { Vec3 *p = &o->u[(size_t)nbl * nx + i]; p->u[0] = p->u[1] = p->u[2] = 0; }
    for (i = 0; i < nz; i++) { Vec3 *p = &o->u[(size_t)i * nx + nbl]; p->u[0] = p->u[1] = p->u[2] = 0; }
    for (i = o->neh; i < o->nex; i++)
        for (m = 0; m <= N; m++) {
            Vec3 *p = &o->u[(size_t)nbl * nx + i * N + m];
            p->u[0] = o->grtuw[i * N + m];
            p->u[1] = o->grtv[i * N + m];
            p->u[2] = -o->grtuw[nx + i * N + m];
        }
    for (i = o->neh; i < o->nez; i++)
        for (m = 0; m <= N; m++) {
            int idz = i * N + m;
            Vec3 *p = &o->u[(size_t)idz * nx + nbl];
            p->u[0] = o->grtuw[2 * nx + idz];
            p->u[1] = o->grtv[nx + idz];
            p->u[2] = -o->grtuw[2 * nx + nz + idz];
        }
}

static void grt_interface_add(Oracle *o)
{
    int i, nx = o->nx, nz = o->nz, nbl = o->neh * o->hpn;
    const real *g = o->grtuw, *g0 = o->grtuw0, *v = o->grtv, *v0 = o->grtv0;
    for (i = nbl; i < nx; i++) {
        Vec3 *p = &o->u[(size_t)nbl * nx + i];
        p->u[0] += -g0[i] + g[i];
        p->u[1] += -v0[i] + v[i];
        p->u[2] += g0[i + nx] - g[i + nx];
    }
    for (i = nbl + 1; i < nz; i++) {
        Vec3 *p = &o->u[(size_t)i * nx + nbl];
        p->u[0] += -g0[2 * nx + i] + g[2 * nx + i];
        p->u[1] += -v0[nx + i] + v[nx + i];
        p->u[2] += g0[2 * nx + nz + i] - g[2 * nx + nz + i];
    }
}

/* ---------------- boundary-trace interpolation (interpl.c:16-91) ---------- */
static int read_record(FILE *f, float *sy, int n, int slot, float *tmp)
{
    int i;
    if (f) {
        if (fread(tmp, sizeof(float), n, f) != (size_t)n) return ORC_ERR;
    } else {
        for (i = 0; i < n; i++) tmp[i] = 0.f;
    }
    for (i = 0; i < n; i++) sy[i * 4 + slot] = tmp[i];
    return ORC_OK;
}

static void guard(real *g, int n)
{   /* sem2d_psvsh.c:433-443, ends read as 0 */
    int i;
    for (i = 0; i < n; i++)
        if (!(g[i] < 10 && g[i] > -10)) {
            real l = (i > 0) ? g[i - 1] : 0, r = (i + 1 < n) ? g[i + 1] : 0;
            g[i] = (l + r) / 2;
        }
}

/* One interpl() call (interpl.c:16-54 with interp_const :59-91).  In
 * sem2d_psvsh.c the P-SV and the SH calls share ONE ns[] ring index array
 * (sem2d_psvsh.c:430-431), so on a step that reads a new record the ring turns
 * once in the P-SV call and once more in the SH call; the taps of each call
 * use the ring as it stands after its own turn. */
static int interpl_one(Oracle *o, int it, FILE *f, float *sy, int n, real *out, float *tmp)
{
    float nst = (float)it;
    float t_f = nst * o->rdt_f;
    int ns0 = (int)(t_f + 0.00001);
    int prev = (int)((nst - 1) * o->rdt_f + 0.00001);
    real w[4];
    int i, j;
    if (ns0 > prev || nst == 0.f) {
        int ns1 = o->ns[0];
        for (j = 0; j < 3; j++) o->ns[j] = o->ns[j + 1];
        o->ns[3] = ns1;
        if (read_record(f, sy, n, o->ns[3], tmp)) return ORC_ERR;
    }
    if (IS_FLOAT) {
        float d1 = t_f - (int)(t_f + 0.00001), d2 = d1 * d1, d3 = d1 * d2;
        w[0] = (real)(-0.5 * d3 + d2 - 0.5 * d1);
        w[1] = (real)(3.0 * d3 - 2.5 * d2 + 1.0);
        w[2] = (real)(-3.0 * d3 + 2.0 * d2 + 0.5 * d1);
        w[3] = (real)(0.5 * (d3 - d2));
    } else {
        double d1 = (double)it * (double)o->rdt - (double)ns0, d2 = d1 * d1, d3 = d1 * d2;
        w[0] = -0.5 * d3 + d2 - 0.5 * d1;
        w[1] = 3.0 * d3 - 2.5 * d2 + 1.0;
        w[2] = -3.0 * d3 + 2.0 * d2 + 0.5 * d1;
        w[3] = 0.5 * (d3 - d2);
    }
    for (i = 0; i < n; i++) {
        real s = 0.0;
        for (j = 0; j < 4; j++) s += w[j] * (real)sy[i * 4 + o->ns[j]];
        out[i] = s;
    }
    return ORC_OK;
}

static int interpl_step(Oracle *o, int it, float *tmp)
{   /* sem2d_psvsh.c:428-444 */
    if (interpl_one(o, it, o->gf, o->sy, o->mtotal, o->grtuw, tmp))
        return fail("P-SV boundary file is short", o->greenfile);
    if (!o->psv_only && interpl_one(o, it, o->shf, o->sy_sh, o->shtotal, o->grtv, tmp))
        return fail("SH boundary file is short", o->shgreenfile);
    guard(o->grtuw, o->mtotal);
    if (!o->psv_only) guard(o->grtv, o->shtotal);
    return ORC_OK;
}

/* ---------------- par -> state ------------------------------------------ */
#define GETI(name, var, must) do { const char *s_ = par_get(&pl, name); \
    if (s_) var = atoi(s_); else if (must) { free(pl.e); return fail("missing par", name); } } while (0)
#define GETF(name, var, varf, must) do { const char *s_ = par_get(&pl, name); \
    if (s_) { varf = (float)atof(s_); var = IS_FLOAT ? (real)varf : (real)atof(s_); } \
    else if (must) { free(pl.e); return fail("missing par", name); } } while (0)
#define GETS(name, var, must) do { const char *s_ = par_get(&pl, name); \
    if (s_) snprintf(var, sizeof var, "%s", s_); else if (must) { free(pl.e); return fail("missing par", name); } } while (0)

static int oracle_setup(Oracle *o, int argc, char **argv)
{
    ParList pl = {0, 0, 0};
    int i, j, N;
    float xmin_f;
    memset(o, 0, sizeof *o);
    o->flat = 1; o->nfil = 1; o->hpn = 5; o->absorb = 1; o->readpars = 1; o->neh = 1;
    o->xtrace = 20; o->idxplot = 20;
    o->ist = 100; o->incre = 50;
    if (par_parse(&pl, argc, argv)) { free(pl.e); return ORC_ERR; }
    GETI("plot_snap", o->plot_snap, 0);
    GETI("startsnap", o->ist, 0);
    GETI("incresnap", o->incre, 0);
    GETI("flat", o->flat, 0);
    GETI("psv_only", o->psv_only, 0);
    GETI("semmodel_full", o->semmodel_full, 0);
    GETS("greenfile", o->greenfile, 1);
    if (!o->psv_only) GETS("shgreenfile", o->shgreenfile, 1);
    GETS("raymodel", o->raymodel, 1);
    GETS("semmodel", o->semmodel, 1);
    GETI("nt", o->nt, 1);
    GETF("dp", o->dp, o->dp_f, 1);
    GETI("nex", o->nex, 1);
    GETF("eh", o->eh, o->eh_f, 1);
    GETF("xmin", o->xmin, xmin_f, 1);
    GETI("nst", o->nst, 1);
    GETF("sdt", o->sdt, o->sdt_f, 1);
    GETI("nfil", o->nfil, 0);
    GETI("hpn", o->hpn, 0);
    GETI("absorb", o->absorb, 0);
    GETI("readpars", o->readpars, 0);
    GETI("neh", o->neh, 0);
    GETI("atten", o->atten, 0);
    o->ass_f = 0.93f;
    o->ass = IS_FLOAT ? (real)o->ass_f : (real)0.93;
    GETF("ass", o->ass, o->ass_f, 0);
    GETI("xtrace", o->xtrace, 0);
    GETF("xbeg", o->xbeg, o->xbeg_f, 1);
    GETF("zbeg", o->zbeg, o->zbeg_f, 0);
    GETI("get_rec", o->get_rec, 0);
    GETI("plot_trace", o->plot_trace, 0);
    if (o->get_rec == 1) GETS("rec_file", o->rec_file, 1);
    GETI("idxplot", o->idxplot, 1);
    GETI("msource", o->msource, 1);
    free(pl.e);
    if (o->msource != 0) return fail("only the GRT boundary source (msource=0) is restated", NULL);
    if (o->atten > 0) {
        o->nh_att = o->neh * o->hpn;
        if (taper_table(o)) return ORC_ERR;
    }
    if (o->nex < 1) return fail("nex must be positive", NULL);
    N = o->hpn;
    if (gll_points(N, o->gllp)) return ORC_ERR;
    gll_weights(o->gllp, N, o->gllw);
    for (i = 0; i <= N; i++)
        for (j = 0; j <= N; j++) o->dlagP[j * (N + 1) + i] = dlag(N, i, o->gllp, o->gllp[j]);
    if (discret(o)) return ORC_ERR;
    o->Uni_Je = (real)(o->eh * o->eh / 4.);
    o->Uni_JeI = (real)(2. / o->eh);
    o->Uni_Jb = (real)(o->eh / 2.);
    for (i = 0; i <= N; i++)
        for (j = 0; j <= N; j++) {
            o->dlagP_JeI[j * (N + 1) + i] = o->dlagP[j * (N + 1) + i] * o->Uni_JeI;
            o->dlagP_Gllw[j * (N + 1) + i] = o->dlagP[j * (N + 1) + i] * o->gllw[j];
        }
    {
        size_t np = (size_t)o->nx * o->nz + 1;
        o->Mass = (real *)calloc(np, sizeof(real));
        o->Mass_dt2 = (real *)calloc(np, sizeof(real));
        o->Ab = (Vec3 *)calloc(np, sizeof(Vec3));
        o->u = (Vec3 *)calloc(np, sizeof(Vec3)); o->u0 = (Vec3 *)calloc(np, sizeof(Vec3));
        o->u1 = (Vec3 *)calloc(np, sizeof(Vec3)); o->K = (Vec3 *)calloc(np, sizeof(Vec3));
        if (!o->Mass || !o->Mass_dt2 || !o->Ab || !o->u || !o->u0 || !o->u1 || !o->K)
            return fail("cannot allocate wavefield", NULL);
    }
    mass_matrix(o);
    if (o->absorb > 0) absorb_matrix(o);

    /* receivers (sem2d_psvsh.c:333-370) */
    if (o->plot_trace) {
        int ixbeg = (int)(o->xbeg_f / o->h_f - 1);
        int izbeg = (int)(o->zbeg_f / o->h_f);
        izbeg += o->nz - 1;
        if (o->zbeg_f == 0.f) izbeg = o->nz - 1;
        if (izbeg > o->nz - 1) izbeg = o->nz - 1;
        if (o->get_rec == 0) {
            o->ntrace = o->xtrace;
            o->rec_off = (long *)calloc(o->ntrace > 0 ? o->ntrace : 1, sizeof(long));
            for (i = 0; i < o->ntrace; i++) o->rec_off[i] = (long)izbeg * o->nx + ixbeg + o->idxplot * i;
        } else {
            FILE *rf = fopen(o->rec_file, "r");
            if (!rf) return fail("cannot open receiver file", o->rec_file);
            if (fscanf(rf, "%d", &o->ntrace) != 1 || o->ntrace < 0) { fclose(rf); return fail("bad receiver file", o->rec_file); }
            o->rec_off = (long *)calloc(o->ntrace > 0 ? o->ntrace : 1, sizeof(long));
            for (i = 0; i < o->ntrace; i++) {
                float rx;
                if (fscanf(rf, "%f", &rx) != 1) { fclose(rf); return fail("short receiver file", o->rec_file); }
                o->rec_off[i] = (long)izbeg * o->nx + (int)(rx / o->h_f);
            }
            fclose(rf);
        }
        for (i = 0; i < o->ntrace; i++)
            if (o->rec_off[i] < 0 || o->rec_off[i] > (long)o->nx * o->nz) return fail("receiver outside the mesh", NULL);
    }

    /* boundary traces (sem2d_psvsh.c:374-396) */
    o->gf = fopen(o->greenfile, "rb");
    if (!o->gf) return fail("cannot open P-SV boundary file", o->greenfile);
    if (!o->psv_only) {
        o->shf = fopen(o->shgreenfile, "rb");
        if (!o->shf) return fail("cannot open SH boundary file", o->shgreenfile);
    }
    o->mtotal = 2 * (o->nx + o->nz);
    o->shtotal = o->nx + o->nz;
    o->grtuw = (real *)calloc(o->mtotal, sizeof(real)); o->grtuw0 = (real *)calloc(o->mtotal, sizeof(real));
    o->grtv = (real *)calloc(o->shtotal, sizeof(real)); o->grtv0 = (real *)calloc(o->shtotal, sizeof(real));
    o->sy = (float *)calloc((size_t)o->mtotal * 4, sizeof(float));
    o->sy_sh = (float *)calloc((size_t)o->shtotal * 4, sizeof(float));
    o->rdt_f = o->sdt_f / o->dp_f;
    o->rdt = o->sdt / o->dp;
    o->nt_sem = (int)((float)((o->nt - 3) * o->dp_f / o->sdt_f));
    for (j = 0; j < 4; j++) o->ns[j] = j;
    return ORC_OK;
}

static void oracle_free(Oracle *o)
{
    if (o->gf) fclose(o->gf);
    if (o->shf) fclose(o->shf);
    free(o->mesh); free(o->Mass); free(o->Mass_dt2); free(o->Ab);
    free(o->u); free(o->u0); free(o->u1); free(o->K); free(o->rec_off);
    free(o->grtuw); free(o->grtuw0); free(o->grtv); free(o->grtv0); free(o->sy); free(o->sy_sh);
    free(o->snaps);
    free(o->taper);
    memset(o, 0, sizeof *o);
}

/* snapshot (sem2d.c:1667-1683): ix = 0, 2, ... outer, iz = 0, 2, ... inner */
static void take_snapshot(Oracle *o, int k)
{
    int ix, iz;
    float *out = o->snaps + (size_t)k * o->nxs * o->nzs * 2;
    for (ix = 0; ix < o->nx; ix += 2)
        for (iz = 0; iz < o->nz; iz += 2) {
            const Vec3 *p = &o->u[(size_t)iz * o->nx + ix];
            float *q = out + ((size_t)(ix / 2) * o->nzs + iz / 2) * 2;
            q[0] = (float)p->u[0];
            q[1] = (float)p->u[1];
        }
    o->snap_taken[k] = 1;
}

static void record(const Oracle *o, float *su, float *sv, float *sw)
{   /* kirrecord_zhl (sem2d_psvsh.c:2116-2160): u, -w, v */
    int i;
    for (i = 0; i < o->ntrace; i++) {
        const Vec3 *p = &o->u[o->rec_off[i]];
        su[i] = (float)p->u[0];
        sw[i] = (float)(-p->u[2]);
        sv[i] = (float)p->u[1];
    }
}

/* the time loop (sem2d_psvsh.c:418-513) */
static int oracle_steps(Oracle *o, int it_begin, int it_end, float *su, float *sv, float *sw)
{
    int it;
    float *tmp = (float *)malloc(sizeof(float) * (size_t)(o->mtotal + 1));
    for (it = it_begin; it < it_end; it++) {
        if (it > 0) {
            memcpy(o->grtuw0, o->grtuw, sizeof(real) * o->mtotal);
            memcpy(o->grtv0, o->grtv, sizeof(real) * o->shtotal);
        }
        if (it < o->nt_sem && interpl_step(o, it, tmp)) { free(tmp); return ORC_ERR; }
        if (it == 0) {
            size_t np = (size_t)o->nx * o->nz + 1;
            memset(o->u, 0, np * sizeof(Vec3));
            memset(o->u0, 0, np * sizeof(Vec3));
            grt_interface_set(o);
        } else {
            Vec3 *t;
            if (it < o->nt_sem) grt_interface_add(o);
            stiff_matrix(o);
            time_update(o);
            if (o->atten > 0) taper_wave(o);
            t = o->u0; o->u0 = o->u; o->u = o->u1; o->u1 = t;
        }
        if (o->plot_trace && su) {
            size_t off = (size_t)(it - it_begin) * o->ntrace;
            record(o, su + off, sv + off, sw + off);
        }
        if (o->plot_snap && o->incre != 0 && it >= o->ist && (it - o->ist) % o->incre == 0 &&
            (it - o->ist) / o->incre < NSNAP) {
            if (!o->snaps) {
                o->nxs = (o->nx + 1) / 2;
                o->nzs = (o->nz + 1) / 2;
                o->snaps = (float *)calloc((size_t)NSNAP * o->nxs * o->nzs * 2, sizeof(float));
                if (!o->snaps) { free(tmp); return fail("cannot allocate snapshots", NULL); }
            }
            take_snapshot(o, (it - o->ist) / o->incre);
        }
    }
    free(tmp);
    return ORC_OK;
}

/* ---------------- exported API (ctypes) ---------------------------------- */
typedef struct { Oracle o; int it; } OracleHandle;

void *oracle_create(int argc, char **argv)
{
    OracleHandle *h = (OracleHandle *)calloc(1, sizeof *h);
    if (!h) return NULL;
    if (oracle_setup(&h->o, argc, argv)) { oracle_free(&h->o); free(h); return NULL; }
    return h;
}
int oracle_dims(void *hv, int *out)
{   /* nx, nz, nez, ntrace, nst, nt_sem, mtotal, shtotal */
    OracleHandle *h = (OracleHandle *)hv;
    out[0] = h->o.nx; out[1] = h->o.nz; out[2] = h->o.nez; out[3] = h->o.ntrace;
    out[4] = h->o.nst; out[5] = h->o.nt_sem; out[6] = h->o.mtotal; out[7] = h->o.shtotal;
    return 0;
}
double oracle_eh(void *hv) { return (double)((OracleHandle *)hv)->o.eh; }
/* run nsteps further steps; seismograms [nsteps][ntrace] each (may be NULL) */
int oracle_run(void *hv, int nsteps, float *su, float *sv, float *sw)
{
    OracleHandle *h = (OracleHandle *)hv;
    int e = h->it + nsteps;
    if (e > h->o.nst) e = h->o.nst;
    if (oracle_steps(&h->o, h->it, e, su, sv, sw)) return ORC_ERR;
    nsteps = e - h->it;
    h->it = e;
    return nsteps;
}
/* snapshot k (the step ist + k*incre) as [nxs][nzs][2]; returns its step, or
 * -1 when it was not taken; dims = {nxs, nzs} */
int oracle_snapshot(void *hv, int k, float *out, int *dims)
{
    OracleHandle *h = (OracleHandle *)hv;
    const Oracle *o = &h->o;
    dims[0] = (o->nx + 1) / 2;
    dims[1] = (o->nz + 1) / 2;
    if (k < 0 || k >= NSNAP || !o->snaps || !o->snap_taken[k]) return -1;
    if (out) memcpy(out, o->snaps + (size_t)k * o->nxs * o->nzs * 2, sizeof(float) * (size_t)o->nxs * o->nzs * 2);
    return o->ist + k * o->incre;
}

/* the newest displacement u^n (after the last step run) as [nx*nz][3] = (x, y, z),
 * for whole-wavefield comparisons at sizes where the seismograms see little */
int oracle_field(void *hv, double *out3)
{
    OracleHandle *h = (OracleHandle *)hv;
    size_t np = (size_t)h->o.nx * h->o.nz, g;
    int c;
    for (g = 0; g < np; g++)
        for (c = 0; c < 3; c++) out3[3 * g + c] = (double)h->o.u[g].u[c];
    return h->it;
}

/* per-point material as 15 coefficients + rho and the Stacey/mass arrays, for set-up checks */
int oracle_material(void *hv, double *out16)
{
    OracleHandle *h = (OracleHandle *)hv;
    size_t np = (size_t)h->o.nx * h->o.nz, g;
    for (g = 0; g < np; g++) {
        const Cmat *m = &h->o.mesh[g];
        static const int vi[5][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 2}, {2, 2}};  /* Voigt 11 12 13 23 33 */
        int a, b, k = 0;
        for (a = 0; a < 5; a++)
            for (b = a; b < 5; b++)
                out16[g * 16 + k++] = (double)m->c[vi[a][0]][vi[a][1]][vi[b][0]][vi[b][1]];
        out16[g * 16 + 15] = (double)m->rho;
    }
    return 0;
}
int oracle_mass(void *hv, double *mass, double *ab3)
{
    OracleHandle *h = (OracleHandle *)hv;
    size_t np = (size_t)h->o.nx * h->o.nz, g;
    for (g = 0; g < np; g++) {
        mass[g] = (double)h->o.Mass[g];
        ab3[3 * g] = (double)h->o.Ab[g].u[0]; ab3[3 * g + 1] = (double)h->o.Ab[g].u[1]; ab3[3 * g + 2] = (double)h->o.Ab[g].u[2];
    }
    return 0;
}
int oracle_receivers(void *hv, long long *off)
{
    OracleHandle *h = (OracleHandle *)hv;
    int i;
    for (i = 0; i < h->o.ntrace; i++) off[i] = h->o.rec_off[i];
    return h->o.ntrace;
}
void oracle_destroy(void *hv)
{
    OracleHandle *h = (OracleHandle *)hv;
    if (!h) return;
    oracle_free(&h->o);
    free(h);
}

#ifdef ORACLE_MAIN
/* drop-in CLI: `oracle_sem2d_psvsh par=run.par [key=value ...]` writes
 * seis.u / seis.w / seis.v in the working directory like the reference. */
int main(int argc, char **argv)
{
    Oracle o;
    FILE *fu = NULL, *fw = NULL, *fv = NULL;
    float *su, *sv, *sw;
    int it;
    if (oracle_setup(&o, argc, argv)) { fprintf(stderr, "oracle: %s\n", orc_errbuf); return 1; }
    su = (float *)calloc(o.ntrace + 1, sizeof(float));
    sv = (float *)calloc(o.ntrace + 1, sizeof(float));
    sw = (float *)calloc(o.ntrace + 1, sizeof(float));
    if (o.plot_trace) {
        fu = fopen("seis.u", "wb"); fw = fopen("seis.w", "wb"); fv = fopen("seis.v", "wb");
        if (!fu || !fw || !fv) { fprintf(stderr, "oracle: cannot open seis.* for writing\n"); return 1; }
    }
    printf("oracle: nx=%d nz=%d nez=%d eh=%.9g nst=%d nt_sem=%d ntrace=%d\n",
           o.nx, o.nz, o.nez, (double)o.eh, o.nst, o.nt_sem, o.ntrace);
    for (it = 0; it < o.nst; it++) {
        if (oracle_steps(&o, it, it + 1, su, sv, sw)) { fprintf(stderr, "oracle: %s\n", orc_errbuf); return 1; }
        if (o.plot_trace) {
            fwrite(su, sizeof(float), o.ntrace, fu);
            fwrite(sw, sizeof(float), o.ntrace, fw);
            fwrite(sv, sizeof(float), o.ntrace, fv);
        }
    }
    if (fu) { fclose(fu); fclose(fw); fclose(fv); }
    for (it = 0; it < NSNAP && o.snaps; it++) {
        /* the reference's text snapshot: "%d %d %e %e\n" (sem2d.c:1677-1681) */
        char name[16];
        FILE *f;
        int ix, iz;
        if (!o.snap_taken[it]) continue;
        snprintf(name, sizeof name, "out%d", it + 1);
        if (!(f = fopen(name, "wt"))) { fprintf(stderr, "oracle: cannot open %s\n", name); return 1; }
        for (ix = 0; ix < o.nx; ix += 2)
            for (iz = 0; iz < o.nz; iz += 2) {
                const float *q = o.snaps + (((size_t)it * o.nxs + ix / 2) * o.nzs + iz / 2) * 2;
                fprintf(f, "%d %d %e %e\n", ix, iz, q[0], q[1]);
            }
        fclose(f);
    }
    free(su); free(sv); free(sw);
    oracle_free(&o);
    return 0;
}
#endif
