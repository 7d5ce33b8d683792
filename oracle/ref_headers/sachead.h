/*
 * Restated declarations for building the reference's seismogram converter
 * (semsyn/plot/uvw2sac.c, sac_rw.c) as a CPU oracle.
 *
 * The reference tree includes "sachead.h" but does not ship it.  uvw2sac and
 * sac_rw use a type SACHEAD whose bytes write_sac() puts at the head of each
 * file (sac_rw.c:100-117), fields set by name (uvw2sac.c:308-333, 366-372,
 * 438-443), and an initialiser sac_null (uvw2sac.c:76).  What is written here
 * is the published SAC version 6 binary header: 70 float words, 40 integer
 * words (35 integers, then leven, lpspol, lovrok, lcalda and one unused),
 * then 8-character fields (kevnm 16) for 192 bytes, 632 bytes in all; every
 * value unset: -12345, "-12345  " (no terminating NUL in an 8-byte field).
 * This header is test infrastructure for the oracle build only.
 */
#ifndef SKS_ORACLE_REF_SACHEAD_H
#define SKS_ORACLE_REF_SACHEAD_H

typedef struct {
    /* float words 0..69 */
    float delta, depmin, depmax, scale, odelta;
    float b, e, o, a, fmt;
    float t0, t1, t2, t3, t4, t5, t6, t7, t8, t9;
    float f;
    float resp0, resp1, resp2, resp3, resp4, resp5, resp6, resp7, resp8, resp9;
    float stla, stlo, stel, stdp;
    float evla, evlo, evel, evdp, mag;
    float user0, user1, user2, user3, user4, user5, user6, user7, user8, user9;
    float dist, az, baz, gcarc;
    float sb, sdelta, depmen, cmpaz, cmpinc;
    float xminimum, xmaximum, yminimum, ymaximum;
    float unused6, unused7, unused8, unused9, unused10, unused11, unused12;
    /* integer words 0..39 */
    int nzyear, nzjday, nzhour, nzmin, nzsec, nzmsec;
    int nvhdr, norid, nevid, npts, nsnpts, nwfid, nxsize, nysize, unused15;
    int iftype, idep, iztype, unused16, iinst, istreg, ievreg, ievtyp, iqual, isynth, imagtyp, imagsrc, ibody;
    int unused20, unused21, unused22, unused23, unused24, unused25, unused26;
    int leven, lpspol, lovrok, lcalda, unused27;
    /* character fields, 192 bytes */
    char kstnm[8], kevnm[16];
    char khole[8], ko[8], ka[8];
    char kt0[8], kt1[8], kt2[8], kt3[8], kt4[8], kt5[8], kt6[8], kt7[8], kt8[8], kt9[8];
    char kf[8], kuser0[8], kuser1[8], kuser2[8];
    char kcmpnm[8], knetwk[8], kdatrd[8], kinst[8];
} SACHEAD;

#define SAC_U_ (-12345.0f)
#define SAC_I_ (-12345)
#define SAC_K_ {'-', '1', '2', '3', '4', '5', ' ', ' '}
static SACHEAD sac_null = {
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_, SAC_U_,
    SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_,
    SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_,
    SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_,
    SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_, SAC_I_,
    SAC_K_, {'-', '1', '2', '3', '4', '5', ' ', ' ', ' ', ' ', ' ', ' ', ' ', ' ', ' ', ' '},
    SAC_K_, SAC_K_, SAC_K_,
    SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_, SAC_K_,
    SAC_K_, SAC_K_, SAC_K_, SAC_K_,
    SAC_K_, SAC_K_, SAC_K_, SAC_K_};
#endif
