/* Model builder: elastic tensors for SEM models, in FP64.
 *
 * The reference builds anisotropic SEM models with small programs and Perl
 * drivers (semsyn/model/src/any_anisotropy.pl, semsyn/model/models/rot_ela.pl):
 * a 6x6 Voigt matrix is rotated about x3 by elastic_rotate
 * (semsyn/model/src/elastic_rotate.c:84-188), dipped about x2 by elastic_dip
 * (semsyn/model/src/elastic_dip.c:114-170), its velocities are checked with a
 * Jacobi eigen-solver of the Christoffel matrix (semsyn/model/src/cjcbi0.c),
 * and the constants are written into the SEM model file the solver reads
 * (sem2d_psvsh.c:663-713).  Those programs compute in float and print two
 * decimals; here the same transforms run in FP64 on full 6x6 matrices, so a
 * tilted axis keeps all 21 constants (semmodel_full=1).
 */
#include "sks.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

int sks_internal_error_c(int code, const char *msg);   /* sks_solver.cu */

/* Voigt (Musgrave) index of a tensor index pair: 11 22 33 23 13 12
 * (elastic_rotate.c:100-146) */
static const int VOIGT[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
static const int PAIR[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};

/* c'_jkmn = g_jo g_kp g_mq g_nr c_opqr (Crampin 1977, the transform of
 * elastic_rotate.c:148-188): g[j][o] is the cosine between new axis j and old
 * axis o; the sum runs o, p, q, r from the outside in. */
static void transform(const double c[36], double g[3][3], double out[36])
{
    int jk, mn, o, p, q, r;
    double t[36];
    for (jk = 0; jk < 6; jk++) {
        const int j = PAIR[jk][0], k = PAIR[jk][1];
        for (mn = 0; mn < 6; mn++) {
            const int m = PAIR[mn][0], n = PAIR[mn][1];
            double v = 0.0;
            for (o = 0; o < 3; o++)
                for (p = 0; p < 3; p++)
                    for (q = 0; q < 3; q++)
                        for (r = 0; r < 3; r++)
                            v += g[j][o] * g[k][p] * g[m][q] * g[n][r] * c[VOIGT[o][p] * 6 + VOIGT[q][r]];
            t[jk * 6 + mn] = v;
        }
    }
    memcpy(out, t, sizeof t);
}

int sks_elastic_rotate(const double c[36], double angle_deg, double out[36])
{
    /* new x1 at angle_deg from old x1, counter-clockwise about x3 (elastic_rotate.c:148-170) */
    const double a = angle_deg * (M_PI / 180.0), ca = cos(a), sa = sin(a);
    double g[3][3] = {{ca, sa, 0.0}, {-sa, ca, 0.0}, {0.0, 0.0, 1.0}};
    if (!c || !out) return sks_internal_error_c(SKS_ERR_ARG, "elastic_rotate: NULL matrix");
    transform(c, g, out);
    return SKS_OK;
}

int sks_elastic_dip(const double c[36], double angle_deg, double out[36])
{
    /* new x1 at angle_deg from old x1 toward old x3, about x2 (elastic_dip.c:114-135) */
    const double a = angle_deg * (M_PI / 180.0), ca = cos(a), sa = sin(a);
    double g[3][3] = {{ca, 0.0, sa}, {0.0, 1.0, 0.0}, {-sa, 0.0, ca}};
    if (!c || !out) return sks_internal_error_c(SKS_ERR_ARG, "elastic_dip: NULL matrix");
    transform(c, g, out);
    return SKS_OK;
}

/* symmetric 3x3 eigenvalues by cyclic Jacobi rotations (the method cjcbi0.c
 * applies to the Christoffel matrix), descending */
static void jacobi3(double A[3][3], double ev[3])
{
    int sweep, p, q, i;
    for (sweep = 0; sweep < 50; sweep++) {
        const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        if (off <= 1e-30 * (A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2]) || off == 0.0) break;
        for (p = 0; p < 2; p++)
            for (q = p + 1; q < 3; q++) {
                double th, t, cs, sn;
                if (A[p][q] == 0.0) continue;
                th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                cs = 1.0 / sqrt(t * t + 1.0);
                sn = t * cs;
                for (i = 0; i < 3; i++) {   /* columns p, q */
                    const double aip = A[i][p], aiq = A[i][q];
                    A[i][p] = cs * aip - sn * aiq;
                    A[i][q] = sn * aip + cs * aiq;
                }
                for (i = 0; i < 3; i++) {   /* rows p, q */
                    const double api = A[p][i], aqi = A[q][i];
                    A[p][i] = cs * api - sn * aqi;
                    A[q][i] = sn * api + cs * aqi;
                }
            }
    }
    ev[0] = A[0][0]; ev[1] = A[1][1]; ev[2] = A[2][2];
    for (p = 0; p < 2; p++)
        for (q = p + 1; q < 3; q++)
            if (ev[q] > ev[p]) { const double t = ev[p]; ev[p] = ev[q]; ev[q] = t; }
}

int sks_christoffel(const double c[36], double rho, const double dir[3], double v[3])
{
    /* Gamma_ik = c_ijkl n_j n_l / rho; phase velocities sqrt of its eigenvalues */
    double G[3][3], n[3], nn, ev[3];
    int i, j, k, l;
    if (!c || !dir || !v || !(rho > 0.0)) return sks_internal_error_c(SKS_ERR_ARG, "christoffel: NULL argument or rho <= 0");
    nn = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(nn > 0.0)) return sks_internal_error_c(SKS_ERR_ARG, "christoffel: zero direction");
    for (i = 0; i < 3; i++) n[i] = dir[i] / nn;
    for (i = 0; i < 3; i++)
        for (k = 0; k < 3; k++) {
            double s = 0.0;
            for (j = 0; j < 3; j++)
                for (l = 0; l < 3; l++) s += c[VOIGT[i][j] * 6 + VOIGT[k][l]] * n[j] * n[l];
            G[i][k] = s / rho;
        }
    jacobi3(G, ev);
    for (i = 0; i < 3; i++) v[i] = ev[i] > 0.0 ? sqrt(ev[i]) : 0.0;
    return SKS_OK;
}

int sks_semmodel_write(const char *path, int32_t nlayers, const sks_layer_t *layers, int32_t full)
{
    /* the SEM model file the solver reads (sem2d_psvsh.c:663-713): per layer
     * "<points> <constants> <rho>", the interface's x values, its z values;
     * 13 constants (c11 c12 c13 c16 c22 c23 c26 c33 c36 c44 c45 c55 c66, the
     * set Cijkl_3D keeps) or, with full, the 21 of the upper triangle */
    static const int C13[13][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 5}, {1, 1}, {1, 2}, {1, 5},
                                   {2, 2}, {2, 5}, {3, 3}, {3, 4}, {4, 4}, {5, 5}};
    FILE *f;
    int i, j, k;
    if (!path || !layers || nlayers < 1) return sks_internal_error_c(SKS_ERR_ARG, "semmodel_write: no layers");
    for (i = 0; i < nlayers; i++)
        if (layers[i].npts < 1 || !layers[i].x || !layers[i].z || !(layers[i].rho > 0.0))
            return sks_internal_error_c(SKS_ERR_ARG, "semmodel_write: a layer needs control points and rho > 0");
    f = fopen(path, "w");
    if (!f) return sks_internal_error_c(SKS_ERR_IO, "semmodel_write: cannot open the file");
    fprintf(f, "%d\n", nlayers);
    for (i = 0; i < nlayers; i++) {
        const sks_layer_t *L = &layers[i];
        fprintf(f, "%d", L->npts);
        if (full) {
            for (j = 0; j < 6; j++)
                for (k = j; k < 6; k++) fprintf(f, " %.17g", L->c[j * 6 + k]);
        } else {
            for (j = 0; j < 13; j++) fprintf(f, " %.17g", L->c[C13[j][0] * 6 + C13[j][1]]);
        }
        fprintf(f, " %.17g\n", L->rho);
        for (j = 0; j < L->npts; j++) fprintf(f, "%s%.17g", j ? " " : "", L->x[j]);
        fprintf(f, "\n");
        for (j = 0; j < L->npts; j++) fprintf(f, "%s%.17g", j ? " " : "", L->z[j]);
        fprintf(f, "\n");
    }
    if (fclose(f)) return sks_internal_error_c(SKS_ERR_IO, "semmodel_write: write failed");
    return SKS_OK;
}
