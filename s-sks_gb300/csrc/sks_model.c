/*
 * Host set-up of an SEM solve from the reference's par file and model files.
 *
 * Mirrors what main() of semsyn/src/sem2d_psvsh.c does before its time loop,
 * with every real quantity in FP64.  Quantities that decide an integer (the
 * element count nez, the grid row where a layer ends, receiver columns, the
 * number of injection steps, when a boundary record is read) are computed in
 * the reference's float arithmetic so that the mesh and the schedule are the
 * reference's own; the float values come from parsing the same text with
 * strtof, as the reference's fscanf("%f")/atof do.
 *
 * Materials are stored as a table of distinct materials plus a 16-bit index
 * per grid point: the reference's models are layered (every point takes the
 * material of one ray-model or SEM-model layer), so a table of a few entries
 * replaces the 328-byte struct cmatrix per point (sem2d_psvsh.c:545-606).
 */
#include "sks_model.h"
#include "sks.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ERR(code, ...) do { snprintf(err, errlen, __VA_ARGS__); return (code); } while (0)

/* ---------------------------------------------------------------- getpar */
/* Caltech getpar (semsyn/src/getpar/lib/getpar.c): name=value words, par=FILE
 * splices a file of words ('#' comments the rest of a line, quotes group),
 * the last occurrence of a name wins, at most 4 nested par files. */
typedef struct { char *name, *value; } Word;
typedef struct { Word *w; int n, cap; } Words;

static void words_add(Words *ws, const char *name, size_t nl, const char *value, size_t vl)
{
    if (ws->n == ws->cap) {
        ws->cap = ws->cap ? ws->cap * 2 : 32;
        ws->w = (Word *)realloc(ws->w, sizeof(Word) * ws->cap);
    }
    ws->w[ws->n].name = (char *)malloc(nl + 1);
    memcpy(ws->w[ws->n].name, name, nl);
    ws->w[ws->n].name[nl] = 0;
    ws->w[ws->n].value = (char *)malloc(vl + 1);
    memcpy(ws->w[ws->n].value, value, vl);
    ws->w[ws->n].value[vl] = 0;
    ws->n++;
}

static void words_free(Words *ws)
{
    int i;
    for (i = 0; i < ws->n; i++) { free(ws->w[i].name); free(ws->w[i].value); }
    free(ws->w);
    memset(ws, 0, sizeof *ws);
}

static int words_file(Words *ws, const char *path, int depth, char *err, size_t errlen)
{
    FILE *f;
    char line[4096];
    if (depth > 4) ERR(SKS_ERR_ARG, "par files nested deeper than 4 at %s", path);
    f = fopen(path, "r");
    if (!f) ERR(SKS_ERR_IO, "cannot open par file %s", path);
    while (fgets(line, sizeof line, f)) {
        const char *p = line;
        for (;;) {
            const char *n0, *v0;
            size_t nl, vl;
            char q = 0;
            while (*p == ' ' || *p == '\t') p++;
            if (!*p || *p == '\n' || *p == '#') break;
            n0 = p;
            while (*p && *p != '=' && *p != ' ' && *p != '\t' && *p != '\n') p++;
            nl = (size_t)(p - n0);
            if (*p == '=') p++;
            if (*p == '"' || *p == '\'') q = *p++;
            v0 = p;
            if (q) { while (*p && *p != q && *p != '\n') p++; }
            else { while (*p && *p != ' ' && *p != '\t' && *p != '\n') p++; }
            vl = (size_t)(p - v0);
            if (q && *p == q) p++;
            words_add(ws, n0, nl, v0, vl);
            if (nl == 3 && !strncmp(n0, "par", 3)) {
                char sub[1024];
                int rc;
                snprintf(sub, sizeof sub, "%.*s", (int)vl, v0);
                rc = words_file(ws, sub, depth + 1, err, errlen);
                if (rc) { fclose(f); return rc; }
            }
        }
    }
    fclose(f);
    return SKS_OK;
}

static const char *words_get(const Words *ws, const char *name)
{
    int i;
    for (i = ws->n - 1; i >= 0; i--) if (!strcmp(ws->w[i].name, name)) return ws->w[i].value;
    return NULL;
}

/* ------------------------------------------------------------- materials */
static const int VLIST[5] = {0, 5, 4, 3, 2};   /* Voigt 11,12,13,23,33 */

static uint64_t mix64(uint64_t h, uint64_t v)
{
    h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    return h;
}

typedef struct { int *slot; int cap; } MatHash;

static int mat_insert(sks_model *m, MatHash *mh, const double rec[SKS_MAT_STRIDE], uint16_t *out)
{
    uint64_t h = 0;
    int k, i;
    for (k = 0; k < SKS_MAT_STRIDE; k++) {
        uint64_t b;
        double v = rec[k] == 0.0 ? 0.0 : rec[k];   /* fold -0 into +0 */
        memcpy(&b, &v, 8);
        h = mix64(h, b);
    }
    i = (int)(h & (uint64_t)(mh->cap - 1));
    while (mh->slot[i] >= 0) {
        const double *o = m->mat + (size_t)mh->slot[i] * SKS_MAT_STRIDE;
        for (k = 0; k < SKS_MAT_STRIDE; k++) if (!(o[k] == rec[k])) break;
        if (k == SKS_MAT_STRIDE) { *out = (uint16_t)mh->slot[i]; return 0; }
        i = (i + 1) & (mh->cap - 1);
    }
    if (m->nmat >= 65535) return -1;
    if (m->nmat == m->mat_cap) {
        m->mat_cap = m->mat_cap ? m->mat_cap * 2 : 16;
        m->mat = (double *)realloc(m->mat, sizeof(double) * SKS_MAT_STRIDE * m->mat_cap);
    }
    memcpy(m->mat + (size_t)m->nmat * SKS_MAT_STRIDE, rec, sizeof(double) * SKS_MAT_STRIDE);
    mh->slot[i] = m->nmat;
    *out = (uint16_t)m->nmat;
    m->nmat++;
    if (m->nmat * 2 > mh->cap) {       /* grow and rehash */
        int ncap = mh->cap * 2, j;
        int *ns = (int *)malloc(sizeof(int) * ncap);
        for (j = 0; j < ncap; j++) ns[j] = -1;
        for (j = 0; j < mh->cap; j++) {
            int id = mh->slot[j];
            uint64_t hh = 0;
            int q;
            if (id < 0) continue;
            for (k = 0; k < SKS_MAT_STRIDE; k++) {
                uint64_t b;
                double v = m->mat[(size_t)id * SKS_MAT_STRIDE + k];
                v = v == 0.0 ? 0.0 : v;
                memcpy(&b, &v, 8);
                hh = mix64(hh, b);
            }
            q = (int)(hh & (uint64_t)(ncap - 1));
            while (ns[q] >= 0) q = (q + 1) & (ncap - 1);
            ns[q] = id;
        }
        free(mh->slot);
        mh->slot = ns;
        mh->cap = ncap;
    }
    return 0;
}

/* 6x6 Voigt stiffness + rho -> table row */
static void mat_record(const double C[6][6], double rho, double rec[SKS_MAT_STRIDE])
{
    int a, b, k = 0;
    for (a = 0; a < 5; a++)
        for (b = a; b < 5; b++) rec[k++] = C[VLIST[a]][VLIST[b]];
    rec[15] = rho;
}

static int mat_is_iso(const double *r)
{   /* r: C11 C16 C15 C14 C13 | C66 C56 C46 C36 | C55 C45 C35 | C44 C34 | C33 */
    return r[1] == 0 && r[2] == 0 && r[3] == 0 && r[6] == 0 && r[7] == 0 && r[8] == 0 &&
           r[10] == 0 && r[11] == 0 && r[13] == 0 && r[0] == r[14] && r[5] == r[9] && r[9] == r[12];
}

int sks_material_is_isotropic(const double *r) { return mat_is_iso(r); }

/* a SEM-model / ray-model layer: 13 constants (Cijkl_3D, sem2d_psvsh.c:1528-1563)
 * or, with semmodel_full=1, all 21 */
typedef struct { double v[21]; double rho; int full; } LayerC;

static void layer_6x6(const LayerC *L, double C[6][6])
{
    int i, j, k = 0;
    memset(C, 0, sizeof(double) * 36);
    if (L->full) {
        for (i = 0; i < 6; i++) for (j = i; j < 6; j++) { C[i][j] = C[j][i] = L->v[k]; k++; }
        return;
    }
    /* v[]: c11 c12 c13 c16 c22 c23 c26 c33 c36 c44 c45 c55 c66 */
    C[0][0] = L->v[0]; C[0][1] = C[1][0] = L->v[1]; C[0][2] = C[2][0] = L->v[2]; C[0][5] = C[5][0] = L->v[3];
    C[1][1] = L->v[4]; C[1][2] = C[2][1] = L->v[5]; C[1][5] = C[5][1] = L->v[6];
    C[2][2] = L->v[7]; C[2][5] = C[5][2] = L->v[8];
    C[3][3] = L->v[9]; C[3][4] = C[4][3] = L->v[10]; C[4][4] = L->v[11]; C[5][5] = L->v[12];
}

/* ------------------------------------------------------------- ray model */
typedef struct {
    int jo, nrec;
    double *vp, *vs, *rho, *thk;   /* FP64 */
    float *thk_f;                  /* float thickness (decisions) */
} Ray;

static void ray_free(Ray *r) { free(r->vp); free(r->vs); free(r->rho); free(r->thk); free(r->thk_f); }

static int ray_read(Ray *r, const char *path, int flat, char *err, size_t errlen)
{
    /* semsyn/src/readmodel.c:43-109: "jo nb", jo x "vp vs rho thk",
     * "lfinal", rays; nrec = na[nen[0]-2] of the first ray (sem2d_psvsh.c:591) */
    FILE *f = fopen(path, "r");
    int j, k, nb, lfinal, nen0 = 0;
    float *vpf, *vsf, *rhf;
    if (!f) ERR(SKS_ERR_IO, "cannot open ray model %s", path);
    if (fscanf(f, "%d %d", &r->jo, &nb) != 2 || r->jo < 1 || r->jo > 100000) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: bad header", path); }
    r->vp = (double *)calloc(r->jo, sizeof(double)); r->vs = (double *)calloc(r->jo, sizeof(double));
    r->rho = (double *)calloc(r->jo, sizeof(double)); r->thk = (double *)calloc(r->jo, sizeof(double));
    r->thk_f = (float *)calloc(r->jo, sizeof(float));
    vpf = (float *)calloc(r->jo, sizeof(float)); vsf = (float *)calloc(r->jo, sizeof(float)); rhf = (float *)calloc(r->jo, sizeof(float));
    for (j = 0; j < r->jo; j++) {
        char t[4][96];
        if (fscanf(f, "%95s %95s %95s %95s", t[0], t[1], t[2], t[3]) != 4) {
            fclose(f); free(vpf); free(vsf); free(rhf); ERR(SKS_ERR_MODEL, "ray model %s: short layer table", path);
        }
        r->vp[j] = strtod(t[0], NULL); r->vs[j] = strtod(t[1], NULL);
        r->rho[j] = strtod(t[2], NULL); r->thk[j] = strtod(t[3], NULL);
        vpf[j] = strtof(t[0], NULL); vsf[j] = strtof(t[1], NULL); rhf[j] = strtof(t[2], NULL);
        r->thk_f[j] = strtof(t[3], NULL);
    }
    if (flat == 0) {
        /* Earth flattening, readmodel.c:82-95,155-166: q_j = R/(R - z_mid) */
        double *qd = (double *)malloc(sizeof(double) * r->jo), *qf = (double *)malloc(sizeof(double) * r->jo);
        for (j = 0; j < r->jo; j++) {
            double zd = 0, zf = 0;
            for (k = 0; k < j; k++) { zd += r->thk[k]; zf += r->thk_f[k]; }
            zd += 0.5 * r->thk[j]; zf += 0.5 * r->thk_f[j];
            qd[j] = 6371.0 / (6371.0 - zd);
            qf[j] = 6371.0 / (6371.0 - zf);
        }
        for (j = 0; j < r->jo; j++) {
            r->vp[j] *= qd[j]; r->vs[j] *= qd[j]; r->rho[j] *= qd[j]; r->thk[j] *= qd[j];
            r->thk_f[j] = (float)(r->thk_f[j] * qf[j]);
        }
        free(qd); free(qf);
    }
    free(vpf); free(vsf); free(rhf);
    if (fscanf(f, "%d", &lfinal) != 1 || lfinal < 1) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: no rays", path); }
    r->nrec = -1;
    for (j = 0; j < lfinal; j++) {
        int nen, v, cnt;
        if (fscanf(f, "%d", &nen) != 1 || nen < 2) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: bad ray %d", path, j); }
        if (j == 0) nen0 = nen;
        for (k = 0; k < nen; k++) {
            if (fscanf(f, "%d", &v) != 1) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: short ray %d", path, j); }
            if (j == 0 && k == nen0 - 2) r->nrec = v;
        }
        if (fscanf(f, "%d", &cnt) != 1) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: short ray %d", path, j); }
        for (k = 0; k < nen; k++)
            if (fscanf(f, "%d", &v) != 1) { fclose(f); ERR(SKS_ERR_MODEL, "ray model %s: short ray %d", path, j); }
    }
    fclose(f);
    if (r->nrec < 1 || r->nrec > r->jo) ERR(SKS_ERR_MODEL, "ray model %s: last GRT layer %d outside 1..%d", path, r->nrec, r->jo);
    return SKS_OK;
}

/* piecewise-linear interface height lip() (sem2d_psvsh.c:831-846) in float;
 * at the last control point the last segment's end value is used */
static int lip(const float *an, const float *bn, int np, float x, float *out)
{
    int i;
    if (x < an[0] || x > an[np - 1]) return -1;
    *out = bn[np - 1];
    for (i = 0; i + 1 < np; i++)
        if (x >= an[i] && x < an[i + 1]) {
            float s = (bn[i + 1] - bn[i]) / (an[i + 1] - an[i]);
            *out = bn[i] + s * (x - an[i]);
        }
    return 0;
}

static void set_rows(sks_model *m, int ix0, int ix1, int iz0, int iz1, uint16_t id)
{
    int iz, ix;
    for (iz = iz0; iz <= iz1; iz++)
        for (ix = ix0; ix < ix1; ix++) m->mat_id[(size_t)iz * m->nx + ix] = id;
}

static int mesh_and_materials(sks_model *m, char *err, size_t errlen)
{
    Ray r;
    MatHash mh;
    int i, k, rc = SKS_OK, iz1, iz2, nlay1, nlay2, nlaynum, inlay;
    float thick_f = 0.f, thk2_f = 0.f;
    double thick = 0;
    memset(&r, 0, sizeof r);
    rc = ray_read(&r, m->raymodel, m->flat, err, errlen);
    if (rc) { ray_free(&r); return rc; }
    /* box height from the ray model (sem2d_psvsh.c:592-606) */
    if (m->nfil > r.nrec) {
        for (i = r.nrec; i < m->nfil && i < r.jo; i++) { thick_f += r.thk_f[i]; thick += r.thk[i]; }
    } else {
        for (i = m->nfil - 1; i < r.nrec - 1; i++) { thick_f += r.thk_f[i]; thick += r.thk[i]; }
    }
    m->nez = (int)((thick_f - 1.e-3) / m->eh_par_f);
    if (m->nez < 1) { ray_free(&r); ERR(SKS_ERR_MODEL, "ray model gives a box of %.6g km: no element rows of %g km", thick, m->eh_par); }
    m->eh_f = (float)((thick_f - 1.e-3) / m->nez);
    m->eh = (thick - 1.e-3) / m->nez;
    m->nx = m->nex * m->hpn + 1;
    m->nz = m->nez * m->hpn + 1;
    m->h_f = m->eh_f / m->hpn;
    m->h = m->eh / m->hpn;
    m->mat_id = (uint16_t *)calloc((size_t)m->nx * m->nz, sizeof(uint16_t));
    if (!m->mat_id) { ray_free(&r); ERR(SKS_ERR_NOMEM, "cannot allocate %d x %d material indices", m->nx, m->nz); }
    mh.cap = 64;
    mh.slot = (int *)malloc(sizeof(int) * mh.cap);
    for (i = 0; i < mh.cap; i++) mh.slot[i] = -1;

    /* 1-D model by grid rows from the bottom (sem2d_psvsh.c:607-672) */
    nlay1 = (m->nfil > r.nrec) ? r.nrec : r.nrec - 2;
    nlay2 = (m->nfil > r.nrec) ? m->nfil + 200 : m->nfil - 200;
    if (nlay2 < 0) nlay2 = 0;
    nlaynum = abs(nlay2 - nlay1) + 1;
    inlay = (m->nfil > r.nrec) ? 1 : -1;
    iz1 = 0;
    for (k = 0; k < nlaynum; k++) {
        double C[6][6], rec[SKS_MAT_STRIDE], c11, c44, c13;
        LayerC L;
        uint16_t id;
        i = nlay1 + k * inlay;
        if (i < 0 || i >= r.jo) break;
        thk2_f += r.thk_f[i];
        iz2 = (int)((thk2_f + 1.e-3) / m->h_f) + 1;
        if (iz2 > m->nz - 1) iz2 = m->nz - 1;
        if (iz2 < iz1) break;
        c11 = r.vp[i] * r.vp[i] * r.rho[i];
        c44 = r.vs[i] * r.vs[i] * r.rho[i];
        c13 = c11 - 2.0 * c44;
        memset(&L, 0, sizeof L);
        L.v[0] = c11; L.v[1] = c13; L.v[2] = c13; L.v[4] = c11; L.v[5] = c13; L.v[7] = c11;
        L.v[9] = c44; L.v[11] = c44; L.v[12] = c44;
        layer_6x6(&L, C);
        mat_record(C, r.rho[i], rec);
        if (mat_insert(m, &mh, rec, &id)) { rc = SKS_ERR_MODEL; snprintf(err, errlen, "more than 65535 materials"); goto out; }
        set_rows(m, 0, m->nx, iz1, iz2, id);
        iz1 = iz2 + 1;
        if (iz2 == m->nz - 1) break;
    }

    /* SEM model, per grid column (sem2d_psvsh.c:674-799) */
    if (m->readpars == 1) {
        FILE *f = fopen(m->semmodel, "r");
        int nll, first = 0, j, ix, nvals = m->semmodel_full ? 22 : 14;
        LayerC *Ls = NULL, ap;
        int *np = NULL, *ratio = NULL;
        float **an = NULL, **bn = NULL;
        if (!f) { rc = SKS_ERR_IO; snprintf(err, errlen, "cannot open SEM model %s", m->semmodel); goto out; }
        if (fscanf(f, "%d", &nll) != 1 || nll == 0) { fclose(f); rc = SKS_ERR_MODEL; snprintf(err, errlen, "SEM model %s: bad layer count", m->semmodel); goto out; }
        if (nll < 0) { first = 1; nll = -nll; }
        Ls = (LayerC *)calloc(nll, sizeof(LayerC));
        np = (int *)calloc(nll, sizeof(int)); ratio = (int *)calloc(nll, sizeof(int));
        an = (float **)calloc(nll, sizeof(float *)); bn = (float **)calloc(nll, sizeof(float *));
        for (j = 0; j < nll && rc == SKS_OK; j++) {
            int q;
            char t[96];
            if (fscanf(f, "%d", &np[j]) != 1) { rc = SKS_ERR_MODEL; break; }
            for (q = 0; q < nvals; q++) {
                double v;
                if (fscanf(f, "%95s", t) != 1) { rc = SKS_ERR_MODEL; break; }
                v = strtod(t, NULL);
                if (q == nvals - 1) Ls[j].rho = v; else Ls[j].v[q] = v;
            }
            if (rc) break;
            Ls[j].full = m->semmodel_full;
            if (np[j] < 0) { ratio[j] = 1; np[j] = -np[j]; }
            if (np[j] < 1 || np[j] > 1000) { rc = SKS_ERR_MODEL; break; }
            an[j] = (float *)calloc(np[j], sizeof(float)); bn[j] = (float *)calloc(np[j], sizeof(float));
            for (q = 0; q < np[j] && rc == SKS_OK; q++) if (fscanf(f, "%f", &an[j][q]) != 1) rc = SKS_ERR_MODEL;
            for (q = 0; q < np[j] && rc == SKS_OK; q++) if (fscanf(f, "%f", &bn[j][q]) != 1) rc = SKS_ERR_MODEL;
        }
        fclose(f);
        if (rc) snprintf(err, errlen, "SEM model %s: malformed layer %d", m->semmodel, j);
        memset(&ap, 0, sizeof ap);
        for (ix = 0; ix < m->nx && rc == SKS_OK; ix++) {
            float x = ix * m->h_f, dep;
            int jz1 = 0, jz2;
            if (first == 1) {
                if (lip(an[0], bn[0], np[0], x, &dep)) { rc = SKS_ERR_MODEL; snprintf(err, errlen, "SEM model %s: x=%.3f outside layer 0", m->semmodel, x); break; }
                jz1 = (int)((dep + 1.e-3) / m->h_f);
            }
            if (jz1 < 0) jz1 = 0;
            for (j = first; j < nll; j++) {
                double C[6][6], rec[SKS_MAT_STRIDE];
                uint16_t id;
                int q;
                if (lip(an[j], bn[j], np[j], x, &dep)) { rc = SKS_ERR_MODEL; snprintf(err, errlen, "SEM model %s: x=%.3f outside layer %d", m->semmodel, x, j); break; }
                jz2 = (int)((dep + 1.e-3) / m->h_f);
                if (jz2 > m->nz - 1) jz2 = m->nz - 1;
                if (ratio[j]) {          /* coefficients multiply the layer below */
                    for (q = 0; q < 21; q++) ap.v[q] *= Ls[j].v[q];
                    ap.rho *= Ls[j].rho;
                    ap.full = Ls[j].full;
                } else {
                    ap = Ls[j];
                }
                layer_6x6(&ap, C);
                mat_record(C, ap.rho, rec);
                if (mat_insert(m, &mh, rec, &id)) { rc = SKS_ERR_MODEL; snprintf(err, errlen, "more than 65535 materials"); break; }
                if (jz2 >= jz1) set_rows(m, ix, ix + 1, jz1 < 0 ? 0 : jz1, jz2, id);
                jz1 = jz2 + 1;
            }
        }
        for (j = 0; j < nll; j++) { free(an[j]); free(bn[j]); }
        free(an); free(bn); free(Ls); free(np); free(ratio);
    }
out:
    free(mh.slot);
    ray_free(&r);
    if (rc == SKS_OK) {
        m->anisotropic = 0;
        for (i = 0; i < m->nmat; i++)
            if (!mat_is_iso(m->mat + (size_t)i * SKS_MAT_STRIDE)) m->anisotropic = 1;
        for (i = 0; i < m->nmat; i++)
            if (!(m->mat[(size_t)i * SKS_MAT_STRIDE + 15] > 0)) ERR(SKS_ERR_MODEL, "material %d has density %g", i, m->mat[(size_t)i * SKS_MAT_STRIDE + 15]);
    }
    return rc;
}

/* ------------------------------------------------------------- GLL tables */
static double legendre(int n, double x)
{
    double p0 = 1, p1 = x, pn = x;
    int i;
    if (n == 0) return 1;
    for (i = 2; i <= n; i++) { pn = ((2 * i - 1) * x * p1 - (i - 1) * p0) / i; p0 = p1; p1 = pn; }
    return pn;
}

static int gll_tables(sks_model *m, char *err, size_t errlen)
{
    /* GLL points as roots of P_N' (closed forms, lagrange.c:323-366), weights
     * 2/(N(N+1)P_N^2) (lagrange.c:256-276), l'_i(xi_j) (lagrange.c:42-67) */
    int N = m->hpn, i, j, k;
    double *g = m->gllp;
    if (N < 3 || N > 6) ERR(SKS_ERR_ARG, "hpn=%d: the GLL points are defined for degree 3..6", N);
    g[0] = -1.0; g[N] = 1.0;
    if (N == 3) { g[1] = -sqrt(1.0 / 5.0); g[2] = -g[1]; }
    if (N == 4) { g[1] = -sqrt(15.0 / 35.0); g[2] = 0.0; g[3] = -g[1]; }
    if (N == 5 || N == 6) {
        double a = N == 5 ? 315.0 : 1386.0, c = N == 5 ? -210.0 : -1260.0, e = N == 5 ? 15.0 : 210.0;
        double r1 = sqrt((-c + sqrt(c * c - 4 * a * e)) / 2 / a), r2 = sqrt((-c - sqrt(c * c - 4 * a * e)) / 2 / a);
        g[1] = -r1; g[2] = -r2;
        if (N == 5) { g[3] = r2; g[4] = r1; } else { g[3] = 0.0; g[4] = r2; g[5] = r1; }
    }
    for (i = 0; i <= N; i++) {
        double P = legendre(N, g[i]);
        m->gllw[i] = (i == 0 || i == N) ? 2.0 / (N * (N + 1)) : 2.0 / (N * (N + 1) * P * P);
    }
    for (i = 0; i <= N; i++) {            /* l'_i evaluated at xi_j */
        double down = 1.0;
        for (k = 0; k <= N; k++) if (k != i) down *= (g[i] - g[k]);
        for (j = 0; j <= N; j++) {
            double sum = 0.0;
            int q;
            for (q = 0; q <= N; q++) {
                double prod = 1.0;
                if (q == i) continue;
                for (k = 0; k <= N; k++) if (k != i && k != q) prod *= (g[j] - g[k]);
                sum += prod;
            }
            m->dlagP[j * (N + 1) + i] = sum / down;
        }
    }
    return SKS_OK;
}

/* ------------------------------------------------------- mass and Stacey */
static int mass_and_stacey(sks_model *m, char *err, size_t errlen)
{
    /* Mass_Matrix (sem2d_psvsh.c:1042-1071) and Absorb_Matrix (:1093-1160),
     * with their loop orders, in FP64 */
    int N = m->hpn, nx = m->nx, ex, ez, a, b;
    size_t np = (size_t)m->nx * m->nz;
    m->mass = (double *)calloc(np, sizeof(double));
    m->ab = (double *)calloc(3 * np, sizeof(double));
    if (!m->mass || !m->ab) ERR(SKS_ERR_NOMEM, "cannot allocate the mass matrix");
    for (ex = 0; ex < m->nex; ex++)
        for (ez = 0; ez < m->nez; ez++)
            for (a = 0; a <= N; a++)
                for (b = 0; b <= N; b++) {
                    size_t g = (size_t)(ez * N + b) * nx + ex * N + a;
                    m->mass[g] += m->gllw[a] * m->gllw[b] * m->Je * m->mat[(size_t)m->mat_id[g] * SKS_MAT_STRIDE + 15];
                }
    if (m->absorb > 0) {
        int side;
        for (side = 0; side < 3; side++) {        /* left, bottom, right */
            int cnt = side == 1 ? m->nex : m->nez, e, q;
            for (e = 0; e < cnt; e++)
                for (q = 0; q <= N; q++) {
                    size_t g = side == 0 ? (size_t)(e * N + q) * nx
                             : side == 1 ? (size_t)(e * N + q)
                                         : (size_t)(e * N + q) * nx + nx - 1;
                    const double *r = m->mat + (size_t)m->mat_id[g] * SKS_MAT_STRIDE;
                    double rho = r[15], vp = sqrt(r[0] / rho), vs = sqrt(r[12] / rho);
                    double f = m->gllw[q] * rho * m->Jb * m->sdt / 2.0;
                    double vx = side == 1 ? vs : vp, vz = side == 1 ? vp : vs;
                    m->ab[3 * g + 0] += f * vx;
                    m->ab[3 * g + 1] += f * vs;
                    m->ab[3 * g + 2] += f * vz;
                }
        }
    }
    return SKS_OK;
}

/* ------------------------------------------------------------- receivers */
static int receivers(sks_model *m, char *err, size_t errlen)
{
    /* sem2d_psvsh.c:333-370: a surface row izbeg and columns from xbeg/idxplot
     * (get_rec=0) or from rec_file x positions (get_rec=1) */
    int ixbeg, izbeg, i;
    m->ntrace = 0;
    if (!m->plot_trace) return SKS_OK;
    ixbeg = (int)(m->xbeg_f / m->h_f - 1);
    izbeg = (int)(m->zbeg_f / m->h_f);
    izbeg += m->nz - 1;
    if (m->zbeg_f == 0.f) izbeg = m->nz - 1;
    if (izbeg > m->nz - 1) izbeg = m->nz - 1;
    if (m->get_rec == 0) {
        m->ntrace = m->xtrace;
        m->rec_off = (int64_t *)calloc(m->ntrace > 0 ? m->ntrace : 1, sizeof(int64_t));
        for (i = 0; i < m->ntrace; i++) m->rec_off[i] = (int64_t)izbeg * m->nx + ixbeg + (int64_t)m->idxplot * i;
    } else {
        FILE *f = fopen(m->rec_file, "r");
        if (!f) ERR(SKS_ERR_IO, "cannot open receiver file %s", m->rec_file);
        if (fscanf(f, "%d", &m->ntrace) != 1 || m->ntrace < 0) { fclose(f); ERR(SKS_ERR_MODEL, "receiver file %s: bad count", m->rec_file); }
        m->rec_off = (int64_t *)calloc(m->ntrace > 0 ? m->ntrace : 1, sizeof(int64_t));
        for (i = 0; i < m->ntrace; i++) {
            float x;
            if (fscanf(f, "%f", &x) != 1) { fclose(f); ERR(SKS_ERR_MODEL, "receiver file %s: %d of %d positions", m->rec_file, i, m->ntrace); }
            m->rec_off[i] = (int64_t)izbeg * m->nx + (int)(x / m->h_f);
        }
        fclose(f);
    }
    for (i = 0; i < m->ntrace; i++)
        if (m->rec_off[i] < 0 || m->rec_off[i] > (int64_t)m->nx * m->nz)
            ERR(SKS_ERR_MODEL, "receiver %d falls outside the mesh (offset %lld)", i, (long long)m->rec_off[i]);
    return SKS_OK;
}

/* ------------------------------------------------------ boundary schedule */
static void interp_weights(double d, double w[4])
{   /* interp_const() weights, interpl.c:83-88 */
    double d2 = d * d, d3 = d * d2;
    w[0] = -0.5 * d3 + d2 - 0.5 * d;
    w[1] = 3.0 * d3 - 2.5 * d2 + 1.0;
    w[2] = -3.0 * d3 + 2.0 * d2 + 0.5 * d;
    w[3] = 0.5 * (d3 - d2);
}

static int schedule(sks_model *m, char *err, size_t errlen)
{
    /* Ring of four record slots per family with ONE shared index array ns[]
     * (sem2d_psvsh.c:381-396,430-431): on a step that reads a record the P-SV
     * call turns the ring and reads into ns[3], then the SH call turns it
     * again and reads into its own slots at the new ns[3]. */
    int ns[4] = {0, 1, 2, 3}, slot_psv[4] = {-1, -1, -1, -1}, slot_sh[4] = {-1, -1, -1, -1};
    int it, j, fam;
    float rdt_f = m->sdt_f / m->dp_f;
    double rdt = m->sdt / m->dp;
    m->mtotal = 2 * (m->nx + m->nz);
    m->shtotal = m->nx + m->nz;
    m->nt_sem = (int)((float)((m->nt - 3) * m->dp_f / m->sdt_f));
    if (m->nt_sem > m->nst) m->nt_sem = m->nst;
    if (m->nt_sem < 0) m->nt_sem = 0;
    m->nrec_psv = m->nrec_sh = 0;
    if (m->nt_sem == 0) return SKS_OK;
    m->tap_psv = (int32_t *)malloc(sizeof(int32_t) * 4 * m->nt_sem);
    m->tap_sh = (int32_t *)malloc(sizeof(int32_t) * 4 * m->nt_sem);
    m->w_psv = (double *)malloc(sizeof(double) * 4 * m->nt_sem);
    m->w_sh = (double *)malloc(sizeof(double) * 4 * m->nt_sem);
    if (!m->tap_psv || !m->tap_sh || !m->w_psv || !m->w_sh) ERR(SKS_ERR_NOMEM, "cannot allocate the boundary schedule");
    for (it = 0; it < m->nt_sem; it++) {
        float t_f = (float)it * rdt_f;
        int ns0 = (int)(t_f + 0.00001);
        int prev = (int)(((float)it - 1) * rdt_f + 0.00001);
        int advance = (ns0 > prev) || it == 0;
        double w[4];
        interp_weights((double)it * rdt - (double)ns0, w);
        for (fam = 0; fam < 2; fam++) {
            int *slot = fam == 0 ? slot_psv : slot_sh;
            int32_t *tap = (fam == 0 ? m->tap_psv : m->tap_sh) + 4 * it;
            double *wt = (fam == 0 ? m->w_psv : m->w_sh) + 4 * it;
            if (fam == 1 && m->psv_only) {           /* no SH call at all */
                for (j = 0; j < 4; j++) { tap[j] = -1; wt[j] = 0.0; }
                continue;
            }
            if (advance) {
                int t0 = ns[0];
                ns[0] = ns[1]; ns[1] = ns[2]; ns[2] = ns[3]; ns[3] = t0;
                slot[ns[3]] = fam == 0 ? m->nrec_psv++ : m->nrec_sh++;
            }
            for (j = 0; j < 4; j++) { tap[j] = slot[ns[j]]; wt[j] = w[j]; }
        }
    }
    return SKS_OK;
}

/* ----------------------------------------------------------- taper */
/* atten_taper (sem2d_psvsh.c:1724-1738): taper[n] = exp(alpha n) for n < nh =
 * neh*hpn, alpha = log10(ass) / (nh log10(2.73)), so taper[0] = 1 and
 * taper[nh-1] ~ ass.  The float table is the reference's (float ass, each
 * factor rounded to float); the FP64 table takes ass as the par word's double. */
static int taper_tables(sks_model *m, char *err, size_t errlen)
{
    int n;
    const int nh = m->neh * m->hpn;
    m->nh_att = 0;
    if (m->atten <= 0) return SKS_OK;
    if (!(m->ass_f > 0.f)) ERR(SKS_ERR_ARG, "ass=%g: the taper's edge factor must be positive", (double)m->ass_f);
    m->taper_f = (float *)calloc((size_t)nh, sizeof(float));
    m->taper_d = (double *)calloc((size_t)nh, sizeof(double));
    if (!m->taper_f || !m->taper_d) ERR(SKS_ERR_NOMEM, "out of host memory (taper)");
    {
        const double alpha_f = 1.0 / nh * log10((double)m->ass_f) / log10(2.73);
        const double alpha_d = 1.0 / nh * log10(m->ass) / log10(2.73);
        for (n = 0; n < nh; n++) {
            m->taper_f[n] = (float)exp((double)(alpha_f * n));
            m->taper_d[n] = exp(alpha_d * n);
        }
    }
    m->nh_att = nh;
    return SKS_OK;
}

/* ------------------------------------------------------------------ main */
#define PGETI(key, dst, must) do { const char *s_ = words_get(&ws, key); \
    if (s_) (dst) = atoi(s_); else if (must) { rc = SKS_ERR_ARG; snprintf(err, errlen, "par: must specify %s", key); goto done; } } while (0)
#define PGETF(key, dst, dstf, must) do { const char *s_ = words_get(&ws, key); \
    if (s_) { (dst) = atof(s_); (dstf) = (float)atof(s_); } \
    else if (must) { rc = SKS_ERR_ARG; snprintf(err, errlen, "par: must specify %s", key); goto done; } } while (0)
#define PGETS(key, dst, must) do { const char *s_ = words_get(&ws, key); \
    if (s_) snprintf((dst), sizeof(dst), "%s", s_); \
    else if (must) { rc = SKS_ERR_ARG; snprintf(err, errlen, "par: must specify %s", key); goto done; } } while (0)

int sks_model_from_par(sks_model *m, int argc, const char *const *argv, char *err, size_t errlen)
{
    Words ws = {0, 0, 0};
    int rc = SKS_OK, i;
    float xmin_f;
    double xmin;
    memset(m, 0, sizeof *m);
    /* defaults as in sem2d_psvsh.c:46-135 */
    m->flat = 1; m->nfil = 1; m->hpn = 5; m->absorb = 1; m->readpars = 1; m->neh = 1;
    m->ass = 0.93; m->ass_f = 0.93f;
    m->xtrace = 20; m->idxplot = 20;
    m->snap_start = 100; m->snap_incre = 50;
    for (i = 1; i < argc; i++) {
        const char *a = argv[i], *eq;
        while (*a == ' ' || *a == '\t') a++;
        eq = strchr(a, '=');
        if (!eq) { words_add(&ws, a, strlen(a), "", 0); continue; }
        words_add(&ws, a, (size_t)(eq - a), eq + 1, strlen(eq + 1));
        if (eq - a == 3 && !strncmp(a, "par", 3)) {
            rc = words_file(&ws, eq + 1, 1, err, errlen);
            if (rc) goto done;
        }
    }
    PGETI("flat", m->flat, 0);
    PGETI("psv_only", m->psv_only, 0);
    PGETI("semmodel_full", m->semmodel_full, 0);
    PGETS("greenfile", m->greenfile, 1);
    if (!m->psv_only) PGETS("shgreenfile", m->shgreenfile, 1);
    PGETS("raymodel", m->raymodel, 1);
    PGETS("semmodel", m->semmodel, 1);
    PGETI("nt", m->nt, 1);
    PGETF("dp", m->dp, m->dp_f, 1);
    PGETI("nex", m->nex, 1);
    PGETF("eh", m->eh_par, m->eh_par_f, 1);
    PGETF("xmin", xmin, xmin_f, 1);
    PGETI("nst", m->nst, 1);
    PGETF("sdt", m->sdt, m->sdt_f, 1);
    PGETI("nfil", m->nfil, 0);
    PGETI("hpn", m->hpn, 0);
    PGETI("absorb", m->absorb, 0);
    PGETI("readpars", m->readpars, 0);
    PGETI("neh", m->neh, 0);
    PGETI("atten", m->atten, 0);
    PGETF("ass", m->ass, m->ass_f, 0);
    PGETI("xtrace", m->xtrace, 0);
    PGETF("xbeg", m->xbeg, m->xbeg_f, 1);
    PGETF("zbeg", m->zbeg, m->zbeg_f, 0);
    PGETI("get_rec", m->get_rec, 0);
    PGETI("plot_trace", m->plot_trace, 0);
    PGETI("plot_snap", m->plot_snap, 0);
    PGETI("startsnap", m->snap_start, 0);
    PGETI("incresnap", m->snap_incre, 0);
    if (m->get_rec == 1) PGETS("rec_file", m->rec_file, 1);
    PGETI("idxplot", m->idxplot, 1);
    PGETI("msource", m->msource, 1);
    (void)xmin; (void)xmin_f;
    if (m->msource != 0) { rc = SKS_ERR_UNSUPPORTED; snprintf(err, errlen, "msource=%d: only the GRT boundary source (msource=0) is supported", m->msource); goto done; }
    if (m->nex < 3) { rc = SKS_ERR_ARG; snprintf(err, errlen, "nex=%d: at least 3 elements are needed", m->nex); goto done; }
    if (m->nst < 1) { rc = SKS_ERR_ARG; snprintf(err, errlen, "nst=%d must be positive", m->nst); goto done; }
    if (!(m->sdt > 0) || !(m->dp > 0) || !(m->eh_par > 0)) { rc = SKS_ERR_ARG; snprintf(err, errlen, "sdt, dp and eh must be positive"); goto done; }
    if (m->neh < 1) { rc = SKS_ERR_ARG; snprintf(err, errlen, "neh=%d must be at least 1", m->neh); goto done; }
    rc = gll_tables(m, err, errlen);
    if (rc) goto done;
    rc = mesh_and_materials(m, err, errlen);
    if (rc) goto done;
    if (m->neh >= m->nex || m->neh >= m->nez) { rc = SKS_ERR_ARG; snprintf(err, errlen, "neh=%d leaves no interface inside the %dx%d mesh", m->neh, m->nex, m->nez); goto done; }
    m->Je = m->eh * m->eh / 4.0;
    m->JeI = 2.0 / m->eh;
    m->Jb = m->eh / 2.0;
    rc = mass_and_stacey(m, err, errlen);
    if (rc) goto done;
    rc = receivers(m, err, errlen);
    if (rc) goto done;
    rc = taper_tables(m, err, errlen);
    if (rc) goto done;
    rc = schedule(m, err, errlen);
done:
    words_free(&ws);
    if (rc) sks_model_free(m);
    return rc;
}

/* the element size and GLL spacing as the reference computes them in float,
 * and the element rows, from the ray model's box height (sem2d_psvsh.c:592-606;
 * semsyn/plot/uvw2sac.c:137-155 repeats the computation) */
int sks_mesh_spacing(const char *raymodel, int flat, int nfil, float eh_par, int hpn, int *nez, float *eh_f, float *h_f,
                     char *err, size_t errlen)
{
    Ray r;
    int i, rc;
    float thick_f = 0.f;
    memset(&r, 0, sizeof r);
    rc = ray_read(&r, raymodel, flat, err, errlen);
    if (rc) { ray_free(&r); return rc; }
    if (nfil > r.nrec) {
        for (i = r.nrec; i < nfil && i < r.jo; i++) thick_f += r.thk_f[i];
    } else {
        for (i = nfil - 1; i < r.nrec - 1; i++) thick_f += r.thk_f[i];
    }
    ray_free(&r);
    if (!(eh_par > 0.f) || hpn < 1) ERR(SKS_ERR_ARG, "eh=%g hpn=%d", eh_par, hpn);
    *nez = (int)((thick_f - 1.e-3) / eh_par);
    if (*nez < 1) ERR(SKS_ERR_MODEL, "ray model gives a box of %.6g km: no element rows of %g km", thick_f, eh_par);
    *eh_f = (float)((thick_f - 1.e-3) / *nez);
    *h_f = *eh_f / hpn;
    return SKS_OK;
}

/* the values of the named par words (NULL when absent; the last occurrence
 * wins, par=FILE splices files as above); the caller frees them */
int sks_par_lookup(int argc, const char *const *argv, int n, const char *const *names, char **values, char *err,
                   size_t errlen)
{
    Words ws = {0, 0, 0};
    int rc = SKS_OK, i;
    for (i = 0; i < n; i++) values[i] = NULL;
    for (i = 1; i < argc; i++) {
        const char *a = argv[i], *eq;
        while (*a == ' ' || *a == '\t') a++;
        eq = strchr(a, '=');
        if (!eq) { words_add(&ws, a, strlen(a), "", 0); continue; }
        words_add(&ws, a, (size_t)(eq - a), eq + 1, strlen(eq + 1));
        if (eq - a == 3 && !strncmp(a, "par", 3)) {
            rc = words_file(&ws, eq + 1, 1, err, errlen);
            if (rc) break;
        }
    }
    if (!rc)
        for (i = 0; i < n; i++) {
            const char *v = words_get(&ws, names[i]);
            if (v) {
                values[i] = (char *)malloc(strlen(v) + 1);
                strcpy(values[i], v);
            }
        }
    words_free(&ws);
    return rc;
}

void sks_model_free(sks_model *m)
{
    free(m->mat); free(m->mat_id); free(m->mass); free(m->ab); free(m->rec_off);
    free(m->tap_psv); free(m->tap_sh); free(m->w_psv); free(m->w_sh);
    free(m->taper_f); free(m->taper_d);
    memset(m, 0, sizeof *m);
}
