/* SAC files of a solve's seismograms: the reference's uvw2sac
 * (semsyn/plot/uvw2sac.c:38-447) as a library call and a program.
 *
 * uvw2sac reads seis.u / seis.v / seis.w, keeps every second record (its
 * output step is twice the SEM step), multiplies by `enlarge` and writes per
 * receiver three SAC files <n>.ce (u, east), <n>.cn (v, north) and <n>.cz
 * (w, vertical), plus log.txt (time and distance ranges) and pm.xy (u, w
 * particle motion).  Its SAC header declaration (sachead.h) and writer are not
 * in the reference tree; the binary layout here is the published SAC version 6
 * header (70 floats, 40 integers, 192 bytes of 8-character fields; unset values
 * -12345, "-12345  "), in the host's byte order, followed by the samples.  The
 * header words are the ones uvw2sac sets (uvw2sac.c:308-333, :366-372,
 * :438-443); everything else stays unset.  The optional convolution with a
 * source time function (Conv_Source=1) calls Fortran routines (stime, convt,
 * diff) that are not in the reference tree and is refused.
 */
#include "sks.h"
#include "sks_model.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int sks_internal_error_c(int code, const char *msg);   /* sks_solver.cu */

/* ---- the SAC version 6 binary header ------------------------------------ */
enum {
    F_DELTA = 0, F_B = 5, F_E = 6, F_O = 7, F_STLA = 31, F_STLO = 32, F_STEL = 33, F_EVLA = 35, F_EVLO = 36,
    F_EVDP = 38, F_GCARC = 53, F_CMPAZ = 57, F_CMPINC = 58, NF = 70
};
enum {
    I_NZYEAR = 0, I_NZJDAY = 1, I_NZHOUR = 2, I_NZMIN = 3, I_NZSEC = 4, I_NZMSEC = 5, I_NVHDR = 6, I_NPTS = 9,
    I_IFTYPE = 15, I_LEVEN = 35, NI = 40
};
#define NC 192                 /* kstnm at byte 0, kevnm (16 bytes) at 8, then 21 fields of 8 */
#define SAC_UNDEF (-12345)
#define SAC_ITIME 1            /* iftype: time series */

void sks_sac_fields_init(sks_sac_fields_t *f)
{
    if (!f) return;
    f->delta = f->b = f->e = f->o = (float)SAC_UNDEF;
    f->evla = f->evlo = f->evdp = (float)SAC_UNDEF;
    f->stla = f->stlo = f->stel = (float)SAC_UNDEF;
    f->gcarc = f->cmpaz = f->cmpinc = (float)SAC_UNDEF;
    f->nzyear = f->nzjday = f->nzhour = f->nzmin = f->nzsec = f->nzmsec = SAC_UNDEF;
    snprintf(f->kstnm, sizeof f->kstnm, "-12345");
}

int sks_sac_write(const char *path, int32_t npts, const float *data, const sks_sac_fields_t *f)
{
    float hf[NF];
    int32_t hi[NI];
    char hc[NC];
    FILE *fp;
    int i;
    size_t n;
    if (!path || !f || npts < 0 || (npts > 0 && !data)) return sks_internal_error_c(SKS_ERR_ARG, "sac_write: bad arguments");
    for (i = 0; i < NF; i++) hf[i] = (float)SAC_UNDEF;
    for (i = 0; i < NI; i++) hi[i] = SAC_UNDEF;
    for (i = 0; i < NC / 8; i++) memcpy(hc + 8 * i, "-12345  ", 8);   /* kstnm, kevnm, 21 more */
    memcpy(hc + 8, "-12345          ", 16);                             /* kevnm is 16 characters */
    hf[F_DELTA] = f->delta; hf[F_B] = f->b; hf[F_E] = f->e; hf[F_O] = f->o;
    hf[F_STLA] = f->stla; hf[F_STLO] = f->stlo; hf[F_STEL] = f->stel;
    hf[F_EVLA] = f->evla; hf[F_EVLO] = f->evlo; hf[F_EVDP] = f->evdp;
    hf[F_GCARC] = f->gcarc; hf[F_CMPAZ] = f->cmpaz; hf[F_CMPINC] = f->cmpinc;
    hi[I_NZYEAR] = f->nzyear; hi[I_NZJDAY] = f->nzjday; hi[I_NZHOUR] = f->nzhour;
    hi[I_NZMIN] = f->nzmin; hi[I_NZSEC] = f->nzsec; hi[I_NZMSEC] = f->nzmsec;
    hi[I_NVHDR] = 6;
    hi[I_NPTS] = npts;
    hi[I_IFTYPE] = SAC_ITIME;
    hi[I_LEVEN] = 1;
    {
        /* kstnm as uvw2sac fills it: a C string copy over the unset value
         * (uvw2sac.c:381, strcpy into the "-12345  " of sac_null) -- the name,
         * a NUL, then what is left of "-12345  "; 8 characters fill the field */
        size_t l = strlen(f->kstnm);
        if (l > 8) l = 8;
        memcpy(hc, f->kstnm, l);
        if (l < 8) hc[l] = '\0';
    }
    fp = fopen(path, "wb");
    if (!fp) return sks_internal_error_c(SKS_ERR_IO, "sac_write: cannot open the file");
    n = fwrite(hf, sizeof(float), NF, fp);
    n += fwrite(hi, sizeof(int32_t), NI, fp);
    n += fwrite(hc, 1, NC, fp);
    if (npts > 0) n += fwrite(data, sizeof(float), (size_t)npts, fp);
    if (fclose(fp) || n != (size_t)(NF + NI + NC + npts)) return sks_internal_error_c(SKS_ERR_IO, "sac_write: write failed");
    return SKS_OK;
}

/* ---- uvw2sac --------------------------------------------------------------- */
enum {
    W_FLAT, W_RAYMODEL, W_NEX, W_NST, W_HPN, W_EH, W_DP, W_SDT, W_NFIL, W_KDT, W_XMIN, W_TSTART, W_XTRACE,
    W_ZTRACE, W_ZBEG, W_IDZPLOT, W_XBEG, W_IDXPLOT, W_ZS, W_GET_REC, W_REC_FILE, W_ENLARGE, W_FIX_REC, W_POS_FILE,
    W_BAZ, W_CONV, NW
};
static const char *const WNAMES[NW] = {
    "flat", "raymodel", "nex", "nst", "hpn", "eh", "dp", "sdt", "nfil", "kdt", "xmin", "tstart", "xtrace",
    "ztrace", "zbeg", "idzplot", "xbeg", "idxplot", "zs", "get_rec", "rec_file", "enlarge", "fix_rec", "pos_file",
    "baz", "Conv_Source"};
/* words uvw2sac requires (mstpar, uvw2sac.c:84-116) */
static const int MUST[] = {W_RAYMODEL, W_NEX, W_NST, W_HPN, W_EH, W_DP, W_ZBEG, W_IDZPLOT, W_XBEG, W_IDXPLOT, W_ZS,
                           W_CONV};

static void path_in(char *out, size_t cap, const char *dir, const char *name)
{
    if (dir && dir[0]) snprintf(out, cap, "%s/%s", dir, name);
    else snprintf(out, cap, "%s", name);
}

int sks_uvw2sac(int argc, const char *const *argv, const char *dir)
{
    char *v[NW];
    char err[512], path[4096];
    int rc, i, j, it, k;
    int flat = 1, nfil = 1, kdt = 1, xtrace = 700, ztrace = 1, get_rec = 0, fix_rec = 0, hpn, nst, nez, idxplot;
    float eh, h, dt = 0.f, xmin = 0.f, tstart = 0.f, xbeg, zs, enlarge = 4.f, baz = 270.f, eh_f;
    const float dis2deg = 111.2f;
    int *ix1 = NULL, ntrace, nt, istep, num, t_m, index;
    float *outu = NULL, *outv = NULL, *outw = NULL, *hold = NULL, *us = NULL, *vs = NULL, *ws = NULL;
    float *longs = NULL;
    char (*names)[64] = NULL;
    FILE *fu = NULL, *fv = NULL, *fw = NULL, *fp = NULL, *fpm = NULL;
    sks_sac_fields_t hd;

    rc = sks_par_lookup(argc, argv, NW, WNAMES, v, err, sizeof err);
    if (rc) return sks_internal_error_c(rc, err);
    for (i = 0; i < (int)(sizeof MUST / sizeof MUST[0]); i++)
        if (!v[MUST[i]]) {
            snprintf(err, sizeof err, "uvw2sac: must specify %s", WNAMES[MUST[i]]);
            rc = sks_internal_error_c(SKS_ERR_ARG, err);
            goto done;
        }
    if (atoi(v[W_CONV]) == 1) {
        rc = sks_internal_error_c(SKS_ERR_UNSUPPORTED,
                                  "uvw2sac: Conv_Source=1 (convolution with a source time function by the Fortran "
                                  "routines stime/convt/diff) is not available");
        goto done;
    }
    if (v[W_FLAT]) flat = atoi(v[W_FLAT]);
    if (v[W_NFIL]) nfil = atoi(v[W_NFIL]);
    if (v[W_KDT]) kdt = atoi(v[W_KDT]);
    if (v[W_XTRACE]) xtrace = atoi(v[W_XTRACE]);
    if (v[W_ZTRACE]) ztrace = atoi(v[W_ZTRACE]);
    if (v[W_GET_REC]) get_rec = atoi(v[W_GET_REC]);
    if (v[W_FIX_REC]) fix_rec = atoi(v[W_FIX_REC]);
    if (v[W_ENLARGE]) enlarge = (float)atof(v[W_ENLARGE]);
    if (v[W_XMIN]) xmin = (float)atof(v[W_XMIN]);
    if (v[W_TSTART]) tstart = (float)atof(v[W_TSTART]);
    if (v[W_BAZ]) baz = (float)atof(v[W_BAZ]);
    if (!v[W_SDT]) { rc = sks_internal_error_c(SKS_ERR_ARG, "uvw2sac: must specify sdt"); goto done; }
    dt = (float)atof(v[W_SDT]);
    hpn = atoi(v[W_HPN]);
    nst = atoi(v[W_NST]);
    eh = (float)atof(v[W_EH]);
    xbeg = (float)atof(v[W_XBEG]);
    zs = (float)atof(v[W_ZS]);
    idxplot = atoi(v[W_IDXPLOT]);
    if (kdt < 1 || nst < 1 || !(dt > 0.f) || xtrace < 1 || ztrace < 1) {
        rc = sks_internal_error_c(SKS_ERR_ARG, "uvw2sac: kdt, nst, sdt, xtrace and ztrace must be positive");
        goto done;
    }
    rc = sks_mesh_spacing(v[W_RAYMODEL], flat, nfil, eh, hpn, &nez, &eh_f, &h, err, sizeof err);
    if (rc) { rc = sks_internal_error_c(rc, err); goto done; }

    /* receivers (uvw2sac.c:160-185): every idxplot-th column from xbeg, or a receiver file */
    ix1 = (int *)malloc(sizeof(int) * (size_t)xtrace);
    if (!ix1) { rc = sks_internal_error_c(SKS_ERR_NOMEM, "uvw2sac: no memory"); goto done; }
    if (get_rec == 1) {
        FILE *rf;
        if (!v[W_REC_FILE]) { rc = sks_internal_error_c(SKS_ERR_ARG, "uvw2sac: must specify rec_file"); goto done; }
        ztrace = 1;
        path_in(path, sizeof path, NULL, v[W_REC_FILE]);
        rf = fopen(path, "rt");
        if (!rf || fscanf(rf, "%d", &xtrace) != 1 || xtrace < 1) {
            if (rf) fclose(rf);
            rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: cannot read the receiver file");
            goto done;
        }
        free(ix1);
        ix1 = (int *)malloc(sizeof(int) * (size_t)xtrace);
        for (i = 0; i < xtrace; i++) {
            float rx = 0.f;
            if (fscanf(rf, "%f", &rx) != 1) { fclose(rf); rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: short receiver file"); goto done; }
            ix1[i] = (int)(rx / h);
        }
        fclose(rf);
    } else {
        const int ixbeg = (int)(xbeg / h);
        for (i = 0; i < xtrace; i++) ix1[i] = ixbeg + idxplot * i;
    }
    if (fix_rec == 1) {
        FILE *pf;
        int ptrace = 0;
        if (!v[W_POS_FILE]) { rc = sks_internal_error_c(SKS_ERR_ARG, "uvw2sac: must specify pos_file"); goto done; }
        pf = fopen(v[W_POS_FILE], "rt");
        if (!pf || fscanf(pf, "%d", &ptrace) != 1 || ptrace != xtrace) {
            if (pf) fclose(pf);
            rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: position file missing or inconsistent with the receivers");
            goto done;
        }
        longs = (float *)malloc(sizeof(float) * (size_t)xtrace);
        names = (char (*)[64])malloc(sizeof *names * (size_t)xtrace);
        for (i = 0; i < xtrace; i++) {
            float la;
            if (fscanf(pf, "%f %f %63s", &longs[i], &la, names[i]) != 3) {
                fclose(pf);
                rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: short position file");
                goto done;
            }
        }
        fclose(pf);
    }

    /* records: every istep-th of nt = nst/kdt (uvw2sac.c:187-271) */
    istep = (int)((dt * 2) / dt / kdt);
    if (istep < 1) istep = 1;
    nt = nst / kdt;
    ntrace = xtrace * ztrace;
    {
        const float t_e = tstart + nt * dt * kdt;
        float x_b, x_e;
        if (get_rec == 1) {
            x_b = (xmin + ix1[0] * h) / dis2deg;
            x_e = (xmin + ix1[xtrace - 1] * h) / dis2deg;
        } else {
            x_b = (xmin + xbeg) / dis2deg;
            x_e = (xmin + xbeg + idxplot * (xtrace - 1) * h) / dis2deg;
        }
        path_in(path, sizeof path, dir, "log.txt");
        fp = fopen(path, "wt");
        if (!fp) { rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: cannot write log.txt"); goto done; }
        fprintf(fp, "%-9.3f %-9.3f\n", tstart, t_e);
        fprintf(fp, "%-9.3f %-9.3f\n", x_b, x_e);
        fclose(fp);
        fp = NULL;
    }
    path_in(path, sizeof path, dir, "seis.u"); fu = fopen(path, "rb");
    path_in(path, sizeof path, dir, "seis.v"); fv = fopen(path, "rb");
    path_in(path, sizeof path, dir, "seis.w"); fw = fopen(path, "rb");
    if (!fu || !fv || !fw) { rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: cannot open seis.u, seis.v and seis.w"); goto done; }
    num = (nt + istep - 1) / istep;
    outu = (float *)malloc(sizeof(float) * (size_t)num * ntrace);
    outv = (float *)malloc(sizeof(float) * (size_t)num * ntrace);
    outw = (float *)malloc(sizeof(float) * (size_t)num * ntrace);
    hold = (float *)malloc(sizeof(float) * (size_t)3 * ntrace);
    if (!outu || !outv || !outw || !hold) { rc = sks_internal_error_c(SKS_ERR_NOMEM, "uvw2sac: no memory"); goto done; }
    num = 0;
    for (it = 0; it < nt; it++) {
        if (fread(hold, sizeof(float), (size_t)ntrace, fu) != (size_t)ntrace ||
            fread(hold + ntrace, sizeof(float), (size_t)ntrace, fv) != (size_t)ntrace ||
            fread(hold + 2 * ntrace, sizeof(float), (size_t)ntrace, fw) != (size_t)ntrace) {
            rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: the seis files hold fewer than nst/kdt records of xtrace*ztrace");
            goto done;
        }
        if (it % istep) continue;
        memcpy(outu + (size_t)num * ntrace, hold, sizeof(float) * (size_t)ntrace);
        memcpy(outv + (size_t)num * ntrace, hold + ntrace, sizeof(float) * (size_t)ntrace);
        memcpy(outw + (size_t)num * ntrace, hold + 2 * ntrace, sizeof(float) * (size_t)ntrace);
        num++;
    }
    t_m = it / istep;
    if (num > t_m) num--;

    /* per receiver: three SAC files and its particle motion (uvw2sac.c:301-447) */
    sks_sac_fields_init(&hd);
    hd.delta = istep * dt * kdt;
    hd.nzyear = 2006; hd.nzjday = 0; hd.nzhour = 0; hd.nzmin = 0; hd.nzsec = 0; hd.nzmsec = 0;
    hd.evla = 0.f;
    hd.evlo = 0.f;
    if (fix_rec == 1) {
        const float gc = get_rec == 1 ? (xmin + ix1[0] * h) / dis2deg : (xmin + xbeg + idxplot * h) / dis2deg;
        if (baz == 270.f) hd.evlo = longs[0] - gc;
        if (baz == 90.f) hd.evlo = longs[0] + gc;
    }
    hd.evdp = zs;
    hd.stla = 0.f;
    hd.stel = 0.f;
    hd.o = -tstart;
    hd.b = 0.f;
    hd.e = num * hd.delta;
    us = (float *)malloc(sizeof(float) * (size_t)(num > 0 ? num : 1));
    vs = (float *)malloc(sizeof(float) * (size_t)(num > 0 ? num : 1));
    ws = (float *)malloc(sizeof(float) * (size_t)(num > 0 ? num : 1));
    if (!us || !vs || !ws) { rc = sks_internal_error_c(SKS_ERR_NOMEM, "uvw2sac: no memory"); goto done; }
    path_in(path, sizeof path, dir, "pm.xy");
    fpm = fopen(path, "wt");
    if (!fpm) { rc = sks_internal_error_c(SKS_ERR_IO, "uvw2sac: cannot write pm.xy"); goto done; }
    index = 0;
    for (i = 0; i < xtrace; i++) {
        const float gcarc = get_rec == 1 ? (xmin + ix1[i] * h) / dis2deg : (xmin + xbeg + idxplot * i * h) / dis2deg;
        for (j = 0; j < ztrace; j++) {
            char base[80], name[4096];
            if (fix_rec == 0) hd.gcarc = gcarc;
            hd.stlo = gcarc;
            if (fix_rec == 1) {
                hd.stlo = longs[i];
                snprintf(base, sizeof base, "%s", names[i]);
            } else {
                snprintf(base, sizeof base, "%d", index);
                path_in(path, sizeof path, dir, "tt.txt");      /* uvw2sac.c:375-380 leaves it behind */
                fp = fopen(path, "wt");
                if (fp) { fprintf(fp, "%d", index); fclose(fp); fp = NULL; }
            }
            snprintf(hd.kstnm, sizeof hd.kstnm, "%.8s", base);
            fprintf(fpm, ">> %-8.2f %-8.2f %-8.2f %d\n", gcarc, hd.b, hd.delta, num);
            for (k = 0; k < num; k++) {
                const size_t off = (size_t)k * ntrace + (size_t)j * xtrace + i;
                us[k] = outu[off] * enlarge;
                vs[k] = outv[off] * enlarge;
                ws[k] = outw[off] * enlarge;
                fprintf(fpm, "%-11.4e %-11.4e\n", us[k], ws[k]);
            }
            hd.cmpaz = 90.f; hd.cmpinc = 90.f;
            snprintf(name, sizeof name, "%s.ce", base); path_in(path, sizeof path, dir, name);
            if ((rc = sks_sac_write(path, num, us, &hd))) goto done;
            hd.cmpaz = 0.f; hd.cmpinc = 90.f;
            snprintf(name, sizeof name, "%s.cn", base); path_in(path, sizeof path, dir, name);
            if ((rc = sks_sac_write(path, num, vs, &hd))) goto done;
            hd.cmpaz = 0.f; hd.cmpinc = 0.f;
            snprintf(name, sizeof name, "%s.cz", base); path_in(path, sizeof path, dir, name);
            if ((rc = sks_sac_write(path, num, ws, &hd))) goto done;
        }
        index++;
    }
    rc = SKS_OK;
done:
    if (fu) fclose(fu);
    if (fv) fclose(fv);
    if (fw) fclose(fw);
    if (fp) fclose(fp);
    if (fpm) fclose(fpm);
    free(ix1); free(outu); free(outv); free(outw); free(hold); free(us); free(vs); free(ws); free(longs); free(names);
    for (i = 0; i < NW; i++) free(v[i]);
    return rc;
}
