/* Boundary traces of a plane wave through a stack of isotropic layers.
 *
 * The reference produces its boundary traces with a generalized-ray
 * generator (semsyn/src/aserpsv_sem.c:319-488, asersh_sem.c, with the
 * Fortran ray sums of semsyn/src/aser.rout_noplot.f) and splits them into the
 * greenfile records (semsyn/src/demult.c:63-78).  Here the incident wave is a
 * plane P, SV or SH wave coming up through a 1-D stack below the SEM box: the
 * upgoing field that reaches the box's bottom medium, with every conversion
 * and reverberation inside the stack, is solved for in the frequency domain
 * with Thomson-Haskell propagators in FP64 and brought back to time by FFT.
 *
 * Stack: entry 0 is the box's bottom medium (unbounded upward; only its
 * upgoing waves are sought), entries 1..n-2 are layers of given thickness
 * going down, entry n-1 is the half-space the wave comes from.  z is up, 0 at
 * the top of entry 1 (the base of entry 0).  The incident wave is referenced
 * to z = 0 as if the half-space reached it, so a stack of identical media
 * passes it unchanged.  Every mode must propagate (p < 1/vp in each medium),
 * so the propagators only carry unit-modulus phases and stay stable.
 *
 * Motion-stress vector b = (u_x, u_z, sigma_xz/(-i w), sigma_zz/(-i w)),
 * continuous across interfaces.  A plane wave u = A pol e^{i w (t - p x - s z)}
 * (s = +eta upgoing, -eta downgoing) has real b per unit amplitude, so each
 * medium's mode matrix E is real.  Polarisations: P along its propagation
 * (p vp, +-eta_p vp); SV upgoing (eta_s vs, -p vs) and downgoing
 * (eta_s vs, p vs); SH u_y, traction mu s u_y.
 */
#include "sks.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

int sks_internal_error_c(int code, const char *msg);   /* sks_solver.cu */

typedef double complex cplx;

static int stack_ok(const sks_stack_layer_t *L, int n, double p)
{
    int j;
    if (!L || n < 2) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: at least 2 media (top, half-space)");
    if (!(p >= 0.0)) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: p must be >= 0");
    for (j = 0; j < n; j++) {
        const sks_stack_layer_t *m = L + j;
        if (!(m->vs > 0.0) || !(m->vp > m->vs) || !(m->rho > 0.0))
            return sks_internal_error_c(SKS_ERR_ARG, "layered wave: each medium needs vp > vs > 0 and rho > 0");
        if (!(p * m->vp < 1.0))
            return sks_internal_error_c(SKS_ERR_ARG, "layered wave: p >= 1/vp in a medium (evanescent P)");
        if (j > 0 && j < n - 1 && !(m->thickness > 0.0))
            return sks_internal_error_c(SKS_ERR_ARG, "layered wave: layer thickness must be positive");
    }
    return SKS_OK;
}

static void etas(const sks_stack_layer_t *m, double p, double *ep, double *es)
{
    *ep = sqrt(1.0 / (m->vp * m->vp) - p * p);
    *es = sqrt(1.0 / (m->vs * m->vs) - p * p);
}

/* columns: P up, SV up, P down, SV down; rows: u_x, u_z, tau_xz, tau_zz */
static void mode_matrix(const sks_stack_layer_t *m, double p, double E[4][4])
{
    double ep, es;
    const double vp = m->vp, vs = m->vs, rho = m->rho, mu = rho * vs * vs;
    const double tzz_p = vp * rho * (1.0 - 2.0 * vs * vs * p * p);
    const double txz_s = mu * vs * (1.0 / (vs * vs) - 2.0 * p * p);   /* mu vs (eta_s^2 - p^2) */
    etas(m, p, &ep, &es);
    E[0][0] = p * vp;                 E[0][1] = es * vs;            E[0][2] = p * vp;                 E[0][3] = es * vs;
    E[1][0] = ep * vp;                E[1][1] = -p * vs;            E[1][2] = -ep * vp;               E[1][3] = p * vs;
    E[2][0] = 2.0 * mu * p * ep * vp; E[2][1] = txz_s;              E[2][2] = -2.0 * mu * p * ep * vp; E[2][3] = -txz_s;
    E[3][0] = tzz_p;                  E[3][1] = -2.0 * mu * p * es * vs; E[3][2] = tzz_p;            E[3][3] = -2.0 * mu * p * es * vs;
}

/* inverse of a real 4x4 by Gauss-Jordan with partial pivoting */
static int invert4(const double A[4][4], double X[4][4])
{
    double a[4][8];
    int i, j, k;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 8; j++) a[i][j] = j < 4 ? A[i][j] : (j - 4 == i ? 1.0 : 0.0);
    for (k = 0; k < 4; k++) {
        int piv = k;
        for (i = k + 1; i < 4; i++)
            if (fabs(a[i][k]) > fabs(a[piv][k])) piv = i;
        if (a[piv][k] == 0.0) return -1;
        if (piv != k)
            for (j = 0; j < 8; j++) { const double t = a[k][j]; a[k][j] = a[piv][j]; a[piv][j] = t; }
        {
            const double d = a[k][k];
            for (j = 0; j < 8; j++) a[k][j] /= d;
        }
        for (i = 0; i < 4; i++) {
            if (i == k) continue;
            const double f = a[i][k];
            if (f != 0.0)
                for (j = 0; j < 8; j++) a[i][j] -= f * a[k][j];
        }
    }
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++) X[i][j] = a[i][j + 4];
    return 0;
}

/* solve A x = B for the columns of B (complex n x n, n <= 4, nb columns), by
 * Gaussian elimination with partial pivoting; A and B are overwritten */
static int csolve(int n, cplx A[4][4], int nb, cplx B[4][2])
{
    int i, j, k;
    for (k = 0; k < n; k++) {
        int piv = k;
        for (i = k + 1; i < n; i++)
            if (cabs(A[i][k]) > cabs(A[piv][k])) piv = i;
        if (cabs(A[piv][k]) == 0.0) return -1;
        if (piv != k) {
            for (j = 0; j < n; j++) { const cplx t = A[k][j]; A[k][j] = A[piv][j]; A[piv][j] = t; }
            for (j = 0; j < nb; j++) { const cplx t = B[k][j]; B[k][j] = B[piv][j]; B[piv][j] = t; }
        }
        for (i = k + 1; i < n; i++) {
            const cplx f = A[i][k] / A[k][k];
            for (j = k; j < n; j++) A[i][j] -= f * A[k][j];
            for (j = 0; j < nb; j++) B[i][j] -= f * B[k][j];
        }
    }
    for (k = n - 1; k >= 0; k--)
        for (j = 0; j < nb; j++) {
            cplx s = B[k][j];
            for (i = k + 1; i < n; i++) s -= A[k][i] * B[i][j];
            B[k][j] = s / A[k][k];
        }
    return 0;
}

/* per-medium tables reused across frequencies */
typedef struct {
    double E[4][4], Ei[4][4];
    double ep, es, mu;
} medium_t;

static int media_tables(const sks_stack_layer_t *L, int n, double p, medium_t *md)
{
    int j;
    for (j = 0; j < n; j++) {
        mode_matrix(L + j, p, md[j].E);
        if (invert4(md[j].E, md[j].Ei))
            return sks_internal_error_c(SKS_ERR_ARG, "layered wave: singular mode matrix");
        etas(L + j, p, &md[j].ep, &md[j].es);
        md[j].mu = L[j].rho * L[j].vs * L[j].vs;
    }
    return SKS_OK;
}

/* coefficients at angular frequency w (> 0 or 0) */
static int coefs_at(const sks_stack_layer_t *L, int n, const medium_t *md, double w, sks_layered_coef_t *c)
{
    cplx M[4][4], H[2][2];
    int i, j, k, l;
    double D = 0.0;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++) M[i][j] = i == j;
    H[0][0] = 1; H[0][1] = 0; H[1][0] = 0; H[1][1] = 1;
    /* M = P_1 P_2 ... P_{n-2}: b(0) = M b(-D) */
    for (l = 1; l <= n - 2; l++) {
        const medium_t *m = md + l;
        const double h = L[l].thickness;
        const cplx lam[4] = {cexp(-I * w * m->ep * h), cexp(-I * w * m->es * h), cexp(I * w * m->ep * h),
                             cexp(I * w * m->es * h)};
        cplx P[4][4], R[4][4];
        for (i = 0; i < 4; i++)
            for (j = 0; j < 4; j++) {
                cplx s = 0;
                for (k = 0; k < 4; k++) s += m->E[i][k] * lam[k] * m->Ei[k][j];
                P[i][j] = s;
            }
        for (i = 0; i < 4; i++)
            for (j = 0; j < 4; j++) {
                cplx s = 0;
                for (k = 0; k < 4; k++) s += M[i][k] * P[k][j];
                R[i][j] = s;
            }
        memcpy(M, R, sizeof M);
        {
            /* SH: E = [[1, 1], [mu es, -mu es]], P = E diag(e^-, e^+) E^-1 */
            const cplx a = cexp(-I * w * m->es * h), b = cexp(I * w * m->es * h);
            const double z = m->mu * m->es;
            cplx Q[2][2], S[2][2];
            Q[0][0] = 0.5 * (a + b);
            Q[0][1] = 0.5 * (a - b) / z;
            Q[1][0] = 0.5 * z * (a - b);
            Q[1][1] = 0.5 * (a + b);
            for (i = 0; i < 2; i++)
                for (j = 0; j < 2; j++) S[i][j] = H[i][0] * Q[0][j] + H[i][1] * Q[1][j];
            memcpy(H, S, sizeof H);
        }
        D += h;
    }
    {
        /* E_0 [tP, tS, 0, 0] - G[:,2] rP - G[:,3] rS = G[:,0] aP' + G[:,1] aS', G = M E_hs */
        const medium_t *hs = md + n - 1, *top = md;
        cplx G[4][4], A[4][4], B[4][2];
        const cplx advp = cexp(I * w * hs->ep * D), advs = cexp(I * w * hs->es * D);
        for (i = 0; i < 4; i++)
            for (j = 0; j < 4; j++) {
                cplx s = 0;
                for (k = 0; k < 4; k++) s += M[i][k] * hs->E[k][j];
                G[i][j] = s;
            }
        for (i = 0; i < 4; i++) {
            A[i][0] = top->E[i][0];
            A[i][1] = top->E[i][1];
            A[i][2] = -G[i][2];
            A[i][3] = -G[i][3];
            B[i][0] = G[i][0] * advp;
            B[i][1] = G[i][1] * advs;
        }
        if (csolve(4, A, 2, B)) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: singular P-SV system");
        for (i = 0; i < 2; i++)
            for (j = 0; j < 2; j++) {
                c->t_psv[i][j][0] = creal(B[i][j]);
                c->t_psv[i][j][1] = cimag(B[i][j]);
                c->r_psv[i][j][0] = creal(B[2 + i][j]);
                c->r_psv[i][j][1] = cimag(B[2 + i][j]);
            }
        /* SH: [1, -Gh0 ; mu0 es0, -Gh1] [tH; rH] = Gu aH', Gu/Gd = H E_hs columns */
        {
            const double zh = hs->mu * hs->es, z0 = top->mu * top->es;
            const cplx gu0 = H[0][0] + H[0][1] * zh, gu1 = H[1][0] + H[1][1] * zh;
            const cplx gd0 = H[0][0] - H[0][1] * zh, gd1 = H[1][0] - H[1][1] * zh;
            cplx As[4][4], Bs[4][2];
            As[0][0] = 1.0;
            As[0][1] = -gd0;
            As[1][0] = z0;
            As[1][1] = -gd1;
            Bs[0][0] = gu0 * advs;
            Bs[1][0] = gu1 * advs;
            if (csolve(2, As, 1, Bs)) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: singular SH system");
            c->t_sh[0] = creal(Bs[0][0]);
            c->t_sh[1] = cimag(Bs[0][0]);
            c->r_sh[0] = creal(Bs[1][0]);
            c->r_sh[1] = cimag(Bs[1][0]);
        }
    }
    return SKS_OK;
}

int sks_layered_coefficients(const sks_stack_layer_t *layers, int32_t n, double p, double omega, sks_layered_coef_t *out)
{
    medium_t *md;
    int rc;
    if (!out) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: NULL output");
    if ((rc = stack_ok(layers, n, p))) return rc;
    md = (medium_t *)malloc(sizeof(medium_t) * (size_t)n);
    if (!md) return sks_internal_error_c(SKS_ERR_NOMEM, "layered wave: out of host memory");
    rc = media_tables(layers, n, p, md);
    if (!rc) rc = coefs_at(layers, n, md, omega, out);
    free(md);
    return rc;
}

/* in-place radix-2 FFT of length nt (a power of 2); sign -1 forward, +1 inverse (unscaled) */
static void fft(cplx *x, int64_t nt, int sign)
{
    int64_t i, j = 0, len;
    for (i = 1; i < nt; i++) {
        int64_t bit = nt >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { const cplx t = x[i]; x[i] = x[j]; x[j] = t; }
    }
    for (len = 2; len <= nt; len <<= 1) {
        const double ang = sign * 2.0 * M_PI / (double)len;
        const int64_t half = len >> 1;
        int64_t k;
        for (k = 0; k < half; k++) {
            /* twiddles from the angle directly, not by repeated products, so
               the error does not grow along the stage */
            const cplx wk = cexp(I * ang * (double)k);
            for (i = k; i < nt; i += len) {
                const cplx u = x[i], v = x[i + half] * wk;
                x[i] = u + v;
                x[i + half] = u - v;
            }
        }
    }
}

int64_t sks_layered_series_length(const sks_stack_layer_t *layers, int32_t n, double p, double f0, double dt, double span)
{
    double tail = 0.0, shift = 0.0;
    int j;
    int64_t nt = 64;
    if (stack_ok(layers, n, p)) return SKS_ERR_ARG;
    if (!(f0 > 0.0) || !(dt > 0.0) || !(span >= 0.0))
        return sks_internal_error_c(SKS_ERR_ARG, "layered wave: needs f0 > 0, dt > 0, span >= 0");
    for (j = 1; j < n - 1; j++) {
        double ep, es, hp, hs;
        etas(layers + j, p, &ep, &es);
        etas(layers + n - 1, p, &hp, &hs);
        tail += layers[j].thickness * (ep + es);
        shift += layers[j].thickness * (ep + es + hp + hs);
    }
    {
        /* reverberations: 12 two-way P+S times of the stack; then the pulse's
           width and the stack's advance or delay against the half-space */
        const double period = span + shift + 12.0 * tail + 8.0 / f0;
        const double want = period / dt;
        if (!(want < (double)(1 << 26)))
            return sks_internal_error_c(SKS_ERR_ARG, "layered wave: the series would exceed 2^26 samples");
        while ((double)nt < want) nt <<= 1;
    }
    return nt;
}

int sks_layered_series(const sks_stack_layer_t *layers, int32_t n, const sks_layered_wave_t *wave, double dt, int64_t nt,
                       double *out)
{
    medium_t *md = NULL;
    cplx *src = NULL, *buf = NULL;
    int rc, m;
    int64_t k, i;
    if (!wave || !out) return sks_internal_error_c(SKS_ERR_ARG, "layered wave: NULL argument");
    if ((rc = stack_ok(layers, n, wave->p))) return rc;
    if (!(wave->f0 > 0.0) || !(dt > 0.0) || nt < 64 || (nt & (nt - 1)))
        return sks_internal_error_c(SKS_ERR_ARG, "layered wave: needs f0 > 0, dt > 0, nt a power of 2 >= 64");
    md = (medium_t *)malloc(sizeof(medium_t) * (size_t)n);
    src = (cplx *)malloc(sizeof(cplx) * (size_t)nt);
    buf = (cplx *)malloc(sizeof(cplx) * (size_t)nt * 3);
    if (!md || !src || !buf) { rc = sks_internal_error_c(SKS_ERR_NOMEM, "layered wave: out of host memory"); goto done; }
    if ((rc = media_tables(layers, n, wave->p, md))) goto done;
    {
        /* Ricker pulse centred at 1.5/f0, the plane-wave generator's */
        const double pf = M_PI * wave->f0, delay = 1.5 / wave->f0;
        for (i = 0; i < nt; i++) {
            const double x = pf * ((double)i * dt - delay), a = x * x;
            src[i] = (1.0 - 2.0 * a) * exp(-a);
        }
    }
    fft(src, nt, -1);
    memset(buf, 0, sizeof(cplx) * (size_t)nt * 3);
    {
        const double dw = 2.0 * M_PI / ((double)nt * dt);
        /* the pulse's spectrum is below 1e-15 of its peak past 6.5 f0 */
        const int64_t kmax = (int64_t)fmin((double)(nt / 2 - 1), ceil(6.5 * 2.0 * M_PI * wave->f0 / dw));
        for (k = 0; k <= kmax; k++) {
            sks_layered_coef_t c;
            cplx tpp, tps, tsp, tss, th, up, us, uh;
            if ((rc = coefs_at(layers, n, md, dw * (double)k, &c))) goto done;
            tpp = c.t_psv[0][0][0] + I * c.t_psv[0][0][1];
            tps = c.t_psv[0][1][0] + I * c.t_psv[0][1][1];
            tsp = c.t_psv[1][0][0] + I * c.t_psv[1][0][1];
            tss = c.t_psv[1][1][0] + I * c.t_psv[1][1][1];
            th = c.t_sh[0] + I * c.t_sh[1];
            up = (tpp * wave->p_amp + tps * wave->sv_amp) * src[k];
            us = (tsp * wave->p_amp + tss * wave->sv_amp) * src[k];
            uh = th * wave->sh_amp * src[k];
            buf[k] = up;
            buf[nt + k] = us;
            buf[2 * nt + k] = uh;
            if (k > 0) {          /* real signals: X(-w) = conj X(w) */
                buf[nt - k] = conj(up);
                buf[2 * nt - k] = conj(us);
                buf[3 * nt - k] = conj(uh);
            } else {
                buf[0] = creal(up);
                buf[nt] = creal(us);
                buf[2 * nt] = creal(uh);
            }
        }
    }
    for (m = 0; m < 3; m++) {
        fft(buf + (size_t)m * nt, nt, 1);
        for (i = 0; i < nt; i++) out[(size_t)m * nt + i] = creal(buf[(size_t)m * nt + i]) / (double)nt;
    }
    rc = SKS_OK;
done:
    free(md);
    free(src);
    free(buf);
    return rc;
}
