/*
 * sks.h — C ABI of the GB300 (sm_103a) SEM time-stepping library.
 *
 * The reference solver `sem2d_psvsh` (semsyn/src/sem2d_psvsh.c) is a program:
 * main() parses a getpar par file, meshes the box and fills per-point
 * materials (discret, :534-828), builds GLL/mass/Stacey tables (:207-330),
 * opens the receivers and the GRT boundary-trace files (:333-416), and then
 * runs the time loop (:418-513) that writes seis.u/seis.w/seis.v.  It has no
 * library interface, uses file-scope globals and exit()s on errors.
 *
 * This ABI is that program cut at its two natural seams, handle based and
 * re-entrant: sks_open_par() is main() up to the time loop, sks_run() is the
 * time loop, and the boundary traces may come from the par file's files
 * (sks_load_boundary_files) or from caller memory (sks_set_boundary).
 * Plain C types only.  Every call returns SKS_OK (0) or a negative status;
 * sks_last_error() describes the last failure of the calling thread.
 * The caller owns every host buffer it passes; the library owns device state.
 * One host thread at a time per handle.
 */
#ifndef SKS_H
#define SKS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference exit()s with -1/-2/-3 or 100 instead:
 * readmodel.c:15-19, sem2d_psvsh.c:591-594,699-702,831-838, getpar.c:560-568) */
#define SKS_OK               0
#define SKS_ERR_ARG         -1   /* bad argument or par value            */
#define SKS_ERR_IO          -2   /* a named input file cannot be read    */
#define SKS_ERR_MODEL       -3   /* ray/SEM model malformed or out of range */
#define SKS_ERR_UNSUPPORTED -4   /* option outside this library's scope  */
#define SKS_ERR_CUDA        -5   /* CUDA runtime failure                 */
#define SKS_ERR_NOMEM       -6   /* host or device allocation failed     */
#define SKS_ERR_BOUNDARY    -7   /* boundary records missing or short    */
#define SKS_ERR_STATE       -8   /* call out of order                    */
#define SKS_ERR_NONFINITE   -9   /* the wavefield stopped being finite   */

/* arithmetic forms */
#define SKS_FP64   0   /* plain FP64 3-level central-difference update      */
#define SKS_FP32C  1   /* FP32 wavefield, Kahan-compensated leapfrog update,
                          FP64 precompute and boundary-trace interpolation */

typedef struct sks_solver sks_solver;

typedef struct {
    int32_t nex, nez, hpn;        /* elements in x and z, GLL degree N    */
    int32_t nx, nz;               /* grid points: nex*N+1, nez*N+1        */
    int32_t nst;                  /* time steps of the whole run          */
    int32_t nt_inject;            /* steps that inject boundary traces    */
    int32_t ntrace;               /* receivers                            */
    int32_t mtotal, shtotal;      /* values per P-SV / SH boundary record */
    int32_t nrec_psv, nrec_sh;    /* boundary records the run consumes    */
    int32_t nmat;                 /* distinct materials                   */
    int32_t anisotropic;          /* 1 if any material is not isotropic   */
    int32_t precision;            /* SKS_FP64 or SKS_FP32C                */
    int32_t step;                 /* next step sks_run() will take        */
    double  eh, h, sdt;           /* element size, GLL spacing, time step */
    int64_t device_bytes;         /* device memory held by the handle     */
    int64_t seam_points;          /* points shared by warp tiles          */
    int32_t tile_rows;            /* element rows per CTA band            */
    int32_t neh;                  /* interface line offset in elements    */
    int32_t iso_rows;             /* element rows whose points are all of
                                     isotropic materials                  */
} sks_info_t;

/* Replaces main() of sem2d_psvsh up to its time loop (sem2d_psvsh.c:82-416):
 * argv holds getpar words ("par=run.par", "nst=2000", ...; argv[0] is the
 * program name and is ignored).  Reads the ray model, the SEM model and the
 * receiver file named there and builds the device state on `device`.  The
 * boundary-trace files are NOT read here (see sks_load_boundary_files).
 * Options the reference has that this library does not run return
 * SKS_ERR_UNSUPPORTED: msource=1 (explosive source).  Every GLL degree the
 * reference accepts runs (hpn = 3..6, lagrange.c:323-328): degree 4 under
 * every tuning, degrees 3, 5 (the reference's default) and 6 with 4-warp
 * CTAs and register cap 0 or 1, alone, in batches (a batch's members share
 * one degree) and in the serving loop.  atten>0 (with ass) runs the
 * reference's boundary taper (atten_wave2, sem2d_psvsh.c:1780-1822). */
int sks_open_par(int argc, const char *const *argv, int precision, int device,
                 sks_solver **out);

/* Reads greenfile/shgreenfile named in the par words (time-major float32
 * records, interpl.c:16-54) and uploads the records the run needs. */
int sks_load_boundary_files(sks_solver *s);

/* Same from caller memory: psv holds nrec_psv records of mtotal floats, sh
 * holds nrec_sh records of shtotal floats (sh may be NULL when the solver was
 * opened with psv_only=1).  Records are copied to the device. */
int sks_set_boundary(sks_solver *s, const float *psv, int32_t nrec_psv,
                     const float *sh, int32_t nrec_sh);

/* Boundary records generated on the device instead of read, each evaluated
 * where the boundary interpolation reads it (the run holds no record table):
 * an upgoing plane P-SV (SV polarisation) and SH wave in the bottom layer, velocity vs (km/s),
 * ray parameter p (s/km), Ricker pulse of dominant frequency f0 (Hz) centred
 * at 1.5/f0 s, sampled every dp (the par file's) on the interface row and
 * column at their GLL node positions (as the reference's generator places
 * them, semsyn/src/aserpsv_sem.c:887-920), in the layout of
 * greenfile/shgreenfile.  Stands in for the
 * reference's boundary-trace producers (semsyn/src/aserpsv_sem.c:319-488 and
 * the record splitting of demult.c:63-78) for plane-wave runs, with no file
 * round trip; the records equal the host generator's (s-sks_gb300/synth.py)
 * up to the rounding of exp. */
typedef struct {
    double vs, p, f0, sv_amp, sh_amp;
} sks_plane_wave_t;
int sks_set_boundary_plane_wave(sks_solver *s, const sks_plane_wave_t *pw);

/* ---- plane waves through a layered stack --------------------------------
 * Boundary records of a plane P, SV or SH wave that comes up through a 1-D
 * stack of isotropic layers below the box: the upgoing P, SV and SH waves it
 * leaves in the box's bottom medium, with every conversion and reverberation
 * inside the stack (Thomson-Haskell propagators in FP64, frequency domain).
 * Stands in for the reference's ray-sum generator
 * (semsyn/src/aserpsv_sem.c:319-488, asersh_sem.c, aser.rout_noplot.f) for
 * plane-wave runs; a stack of identical media gives sks_set_boundary_plane_wave's
 * records.  Stack order: layers[0] the box's bottom medium (unbounded
 * upward), layers[1..n-2] going down with their thickness (km), layers[n-1]
 * the half-space the wave comes from.  Every medium needs vp > vs > 0,
 * rho > 0 and p < 1/vp (all modes propagate).  The incident wave is
 * referenced to the base of layers[0] as if the half-space reached it. */
typedef struct {
    double vp, vs, rho;         /* km/s, km/s, g/cm^3                      */
    double thickness;           /* km; ignored for the first and last entries */
} sks_stack_layer_t;

typedef struct {
    double p, f0;               /* ray parameter (s/km), Ricker frequency (Hz) */
    double p_amp, sv_amp, sh_amp; /* incident amplitudes in the half-space  */
} sks_layered_wave_t;

/* plane-wave coefficients at angular frequency omega (rad/s) for a unit
 * incident wave: t_* the upgoing amplitudes in layers[0] at its base, r_*
 * the downgoing amplitudes in the half-space at its top; [out][in] with 0 =
 * P, 1 = SV; [re, im].  Polarisations: P along its propagation; SV upgoing
 * (eta_s vs, -p vs), downgoing (eta_s vs, p vs) in (x, z up); SH u_y. */
typedef struct {
    double t_psv[2][2][2], r_psv[2][2][2];
    double t_sh[2], r_sh[2];
} sks_layered_coef_t;
int sks_layered_coefficients(const sks_stack_layer_t *layers, int32_t n, double p, double omega,
                             sks_layered_coef_t *out);

/* The upgoing P, SV and SH displacement series in layers[0] at its base and
 * x = 0, for the Ricker pulse centred at 1.5/f0: out[m*nt + i] at time i*dt
 * (m = 0 P, 1 SV, 2 SH), periodic in nt*dt (negative times at the end).
 * sks_layered_series_length gives a power-of-2 nt whose period holds span
 * seconds of record plus the stack's reverberations. */
int64_t sks_layered_series_length(const sks_stack_layer_t *layers, int32_t n, double p, double f0, double dt,
                                  double span);
int sks_layered_series(const sks_stack_layer_t *layers, int32_t n, const sks_layered_wave_t *wave, double dt,
                       int64_t nt, double *out);

/* Boundary records from the layered stack, on the device, in the layout
 * and at the node positions of sks_set_boundary_plane_wave, evaluated where
 * the interpolation reads them (the run holds the mode series, not a record
 * table).  Each value is a series above evaluated at t - p x - eta z (cubic
 * Lagrange between samples dp/4 apart).  All boundary setters refuse a solver
 * that is already a batch member (SKS_ERR_STATE). */
int sks_set_boundary_layered_wave(sks_solver *s, const sks_stack_layer_t *layers, int32_t n,
                                  const sks_layered_wave_t *wave);

/* Replaces the time loop (sem2d_psvsh.c:418-513) for steps
 * [step, step+nsteps): each step writes ntrace floats to each of seis_u
 * (u_x), seis_w (-u_z) and seis_v (u_y), time-major, like kirrecord_zhl
 * (sem2d_psvsh.c:2116-2160).  Buffers hold nsteps*ntrace floats; any may be
 * NULL.  Returns the number of steps taken (>= 0) or a negative status. */
int sks_run(sks_solver *s, int32_t nsteps, float *seis_u, float *seis_v, float *seis_w);

/* Snapshots (plot_snap=1 with startsnap / incresnap in the par words, as in
 * sem2d_psvsh.c:149-150,202-204,483-510): the step startsnap + k*incresnap
 * (k < 26) records (u_x, u_y) of every second grid point, the field the
 * receivers see (after the update, before the next injection), like the
 * reference's snapshot() (sem2d.c:1667-1683), which writes them as text file
 * out<k+1>.  out receives dims[0]*dims[1]*2 floats, [ix/2][iz/2][2] (ix outer,
 * iz inner, as the file lists them); dims = {(nx+1)/2, (nz+1)/2}.  Returns
 * the snapshot's step, or SKS_ERR_STATE when the run has not taken it (or
 * plot_snap=0).  sks_run takes snapshots; batch members cannot have them. */
int sks_snapshot(const sks_solver *s, int32_t k, float *out, int32_t *dims);

/* ---- model builder -----------------------------------------------------
 * Elastic tensors for SEM models in FP64 (the reference's float tools:
 * semsyn/model/src/elastic_rotate.c, elastic_dip.c, cjcbi0.c).  Matrices are
 * 6x6 Voigt, row-major, index order 11 22 33 23 13 12. */
/* new x1 at angle_deg from old x1, counter-clockwise about x3; out may be c */
int sks_elastic_rotate(const double c[36], double angle_deg, double out[36]);
/* new x1 at angle_deg from old x1 toward old x3, about x2; out may be c */
int sks_elastic_dip(const double c[36], double angle_deg, double out[36]);
/* phase velocities along dir (any length): the square roots of the
 * eigenvalues of the Christoffel matrix c_ijkl n_j n_l / rho, descending
 * (qP, then the two quasi-shear waves) */
int sks_christoffel(const double c[36], double rho, const double dir[3], double v[3]);
/* one layer of a SEM model: its stiffness and density, and the control
 * points (x, height above the box bottom, km) of its top interface */
typedef struct {
    double c[36];
    double rho;
    int32_t npts;
    const double *x;
    const double *z;
} sks_layer_t;
/* writes the SEM model file (sem2d_psvsh.c:663-713), bottom layer first:
 * 13 constants per layer as the reference keeps them, or (full != 0) all 21
 * for semmodel_full=1 */
int sks_semmodel_write(const char *path, int32_t nlayers, const sks_layer_t *layers, int32_t full);

/* ---- post-processing ---------------------------------------------------
 * The band-pass and shear-wave splitting the reference's scripts run with SAC
 * and an external Silver-Chan program (applications/test/prem_epi83.pl:96-99,
 * cal_split.pl:7-56), on the device for every receiver of a solve. */
typedef struct {
    double f_lo, f_hi;      /* Butterworth band-pass corners (Hz); f_lo <= 0: no filter */
    int32_t poles;          /* low-pass prototype poles (SAC "n"), 1..8 */
    int32_t passes;         /* 1: forward; 2: forward then backward, zero phase (SAC "p") */
    double before, after;   /* analysis window: s before / after the largest radial amplitude */
    double max_delay;       /* s, delays 0..max_delay in steps of dt */
    double dphi;            /* deg, fast axes -90 + k*dphi */
} sks_split_opts_t;
/* second-order sections of the band-pass for sample interval dt:
 * sos[6k..6k+5] = b0 b1 b2 1 a1 a2; returns the number of sections (= poles) */
int sks_bandpass_design(double f_lo, double f_hi, int32_t poles, double dt, double *sos);
/* device scratch sks_split_traces needs */
int sks_split_scratch(int32_t ntrace, int32_t nt, double dt, const sks_split_opts_t *o, int64_t *work_floats,
                      int64_t *sum_doubles);
/* Band-pass and Silver-Chan (1991, eigenvalue method) splitting of ntrace
 * receivers; every pointer is DEVICE memory: sample t of trace r of the radial
 * (u_x) and transverse (u_y) components at [t*ld + r] (a whole-run
 * seismogram buffer [nst][3][ntrace] is radial = base, transverse = base +
 * ntrace, ld = 3*ntrace); work and sums from sks_split_scratch; out[4r..4r+3]
 * = fast axis (deg from x toward y), delay (samples), lambda2/lambda1, window
 * start (sample).  Queued on stream (0: the default stream). */
int sks_split_traces(const float *radial, const float *transverse, int32_t ntrace, int32_t nt, int64_t ld,
                     double dt, const sks_split_opts_t *o, float *work, double *sums, float *out, void *stream);

/* SAC files of a solve's seismograms, as the reference's uvw2sac writes them
 * (semsyn/plot/uvw2sac.c).  sks_sac_write writes one SAC version 6 binary file
 * (host byte order): the fields below, iftype = time series, leven = 1,
 * nvhdr = 6, npts; every other header word unset (-12345).
 * sks_sac_fields_init sets every field unset. */
typedef struct {
    float delta, b, e, o;          /* sample interval, begin, end, origin (s)   */
    float evla, evlo, evdp;        /* event latitude, longitude, depth          */
    float stla, stlo, stel;        /* station latitude, longitude, elevation    */
    float gcarc, cmpaz, cmpinc;    /* distance (deg), component azimuth, incidence */
    int32_t nzyear, nzjday, nzhour, nzmin, nzsec, nzmsec;   /* reference time  */
    char kstnm[9];                 /* station name (8 characters)               */
} sks_sac_fields_t;

void sks_sac_fields_init(sks_sac_fields_t *f);
int sks_sac_write(const char *path, int32_t npts, const float *data, const sks_sac_fields_t *f);

/* The uvw2sac program: par words as the reference reads them (raymodel, nex,
 * nst, hpn, eh, dp, sdt, kdt, xmin, tstart, xtrace, ztrace, zbeg, idzplot, xbeg,
 * idxplot, zs, get_rec/rec_file, enlarge, fix_rec/pos_file/baz, Conv_Source);
 * reads seis.u/v/w from dir (NULL: the working directory) and writes there, per
 * receiver n, n.ce / n.cn / n.cz (every second record, times enlarge), log.txt
 * and pm.xy.  Conv_Source=1 (a source time function convolved by Fortran
 * routines outside the reference tree) returns SKS_ERR_UNSUPPORTED. */
int sks_uvw2sac(int argc, const char *const *argv, const char *dir);

/* Restart: a solve's state (both displacement buffers, the FP32C increment
 * and compensation, the step, taken snapshots) copied to host memory and
 * back, for checkpoints and for preempting a served solve.  A saved state
 * loads into the same solve or into a new solver opened from the same par
 * words and form (checked: form, mesh, step count); the run then continues
 * exactly as if it had not stopped, under any tuning.  The reference has no
 * restart (its snapshot files, sem2d.c:1667-1683, are for plotting). */
int64_t sks_state_bytes(const sks_solver *s);
int sks_state_save(sks_solver *s, void *host, int64_t bytes);
int sks_state_load(sks_solver *s, const void *host, int64_t bytes);

/* The boundary increments the time loop injects, as GRT_Interface4 adds them
 * (sem2d_psvsh.c:2076-2111) from the interpolated traces of interpl()
 * (interpl.c:16-54): for each step it in [it0, it0+nsteps), the FP64
 * difference g(it+1) - g(it) at every interface-line point -- row nbl for
 * ix >= nbl, then column nbl for iz > nbl, nline = (nx-nbl)+(nz-nbl-1)
 * points -- as (u_x, u_y, u_z) with z up.  out receives nsteps*nline*3
 * doubles (host memory); steps that inject nothing get zeros.  Scratch for
 * the interpolated traces is allocated on the device for the call. */
int sks_line_increments(sks_solver *s, int32_t it0, int32_t nsteps, double *out);

/* The same boundary increments as sks_line_increments(), for callers that
 * cannot allocate device memory when they need them: a serving process that
 * has already divided the GPU's memory among its solves and gives each part
 * only the buffers it owns, a host program whose plugin rules forbid the
 * plugin from allocating, or a latency-critical path that cannot accept the
 * device-wide synchronization cudaMalloc/cudaFree imply.  No counterpart in
 * the reference (which has no library interface).
 *
 * Every pointer is DEVICE memory the caller owns: rec_psv / rec_sh are the
 * boundary records (float32, 2*(nx+nz) and nx+nz values per record), the
 * four-tap schedule (tap_* record indices, -1 for an empty slot; w_* FP64
 * weights; 4 entries per step) covers nsteps+1 consecutive steps s..s+nsteps,
 * and every tap that is not -1 must index a record the caller's rec_psv /
 * rec_sh hold (the kernels read record tap without a bound; the caller's
 * schedule is trusted as sks_setup_schedule writes it),
 * and out receives nsteps*nline*3 doubles: the increment g(s+k+1) - g(s+k)
 * of step s+k at every interface-line point (row nbl for ix >= nbl, then
 * column nbl for iz > nbl; nline = (nx-nbl)+(nz-nbl-1)).  The work is queued
 * on `stream` (a cudaStream_t; NULL for the default stream) and the call
 * returns without waiting for it.
 *
 * It allocates nothing: the FP64 interpolated rows live in one fixed 8 MiB
 * scratch array inside the library, so (nsteps+2)*3*(nx+nz) must not exceed
 * 1048576 or the call fails with SKS_ERR_ARG.  The first call on a device
 * looks the scratch's device address up (cudaGetSymbolAddress) and keeps it
 * for the context current at that call (normally the device's primary
 * context, the one the CUDA runtime uses); a call made in another context (a
 * new primary context after cudaDeviceReset, or a driver-API context the
 * caller made current) looks it up again for that context.  Make the first
 * call in a context before any stream capture.  All calls on a device
 * share the scratch and it keeps the last call's contents (every value a call
 * reads is written by that call first); calls whose work overlaps on the GPU
 * (other streams, other host threads) race on it. */
int sks_line_increments_noalloc(const float *rec_psv, const float *rec_sh, int32_t nx, int32_t nz,
                                int32_t nbl, const int32_t *tap_psv, const double *w_psv,
                                const int32_t *tap_sh, const double *w_sh, int32_t nsteps,
                                double *out, void *stream);

/* Back to step 0 with a zero wavefield (boundary records are kept); clears
 * the non-finite flag. */
int sks_reset(sks_solver *s);

/* Wavefield health.  The step kernels flag a solve whose new displacement at
 * any point is NaN or infinite (or, in the FP32C form, whose components'
 * magnitudes sum past the largest float); the reference has no such check
 * (its only guard replaces an interpolated boundary value outside (-10, 10),
 * NaN included, by its neighbours' mean, sem2d_psvsh.c:432-444; a NaN with a
 * non-finite neighbour, as in a whole NaN record, passes).  sks_run then returns
 * SKS_ERR_NONFINITE after taking its steps (the seismograms are still
 * written), and so does every later run until sks_reset or sks_state_load;
 * sks_batch_run returns it when any member is flagged, and the serving loop
 * fails that request alone.  Returns 1 while the solve is finite as of its
 * last finished run, 0 once flagged. */
int sks_wavefield_finite(const sks_solver *s);

int sks_get_info(const sks_solver *s, sks_info_t *info);

/* ---- host-only set-up (no device needed) ------------------------------
 * sks_setup_open() runs the set-up half of main() (par words, ray and SEM
 * models, mesh, materials, GLL tables, mass, Stacey matrix, receivers and the
 * boundary-record schedule) and keeps it on the host for inspection;
 * sks_open_setup() turns it into a device solver. */
typedef struct sks_setup sks_setup;

int sks_setup_open(int argc, const char *const *argv, sks_setup **out);
int sks_setup_info(const sks_setup *su, sks_info_t *info);

/* Per-point material: nx*nz rows of 16 doubles, the 5x5 block of the Voigt
 * stiffness on the strains (11, 12, 13, 23, 33) stored upper-triangle row by
 * row (C11 C16 C15 C14 C13 C66 C56 C46 C36 C55 C45 C35 C44 C34 C33), then
 * rho: the entries the 2-D stress uses (Stress_ij, sem2d_psvsh.c:1345-1380). */
int sks_setup_material(const sks_setup *su, double *out16);

/* Lumped mass (nx*nz) and Stacey coefficients (3*nx*nz, zero off the
 * absorbing edges) as Mass_Matrix / Absorb_Matrix build them
 * (sem2d_psvsh.c:1042-1128). */
int sks_setup_mass(const sks_setup *su, double *mass, double *ab3);

/* Receiver offsets iz*nx+ix (ntrace values). */
int sks_setup_receivers(const sks_setup *su, int64_t *off);

/* Boundary-record schedule of the injecting steps: per step four record
 * indices (-1: a ring slot never filled) and four FP64 weights for the P-SV
 * and the SH family (interpl.c:16-91, ring shared as in
 * sem2d_psvsh.c:430-431).  Arrays hold 4*nt_inject entries. */
int sks_setup_schedule(const sks_setup *su, int32_t *tap_psv, double *w_psv,
                       int32_t *tap_sh, double *w_sh);

void sks_setup_close(sks_setup *su);

/* Device solver from a set-up; the set-up is consumed (closed) on success
 * and on failure. */
int sks_open_setup(sks_setup *su, int precision, int device, sks_solver **out);

/* ---- tuning -------------------------------------------------------------
 * The step kernel runs one CTA per (column of 6*W-1 elements, band of B
 * element rows); each CTA recomputes one element column of halo.  W (warps
 * per CTA), the band layout, the band-seam method and a register cap are
 * tunable; the default comes from the mesh size and the SM count.
 * Every tuning gives bit-identical results. */
typedef struct {
    int32_t warps_per_block;      /* 2 or 4                                 */
    int32_t band_rows;            /* element rows per CTA band              */
    int32_t zseam;                /* 0: each band recomputes the element row below
                                     it; 1: bands exchange boundary-row partial
                                     forces (the later band sums them)      */
    int32_t register_cap;         /* 0: compiler's choice; 1 / 2: registers capped for
                                     16 / 20 (FP32) or 8 / 12 (FP64) warps per SM */
    int32_t waves;                /* 0: bands of band_rows rows; W > 0: exactly
                                     W waves of CTAs (SMs x resident CTAs x W),
                                     columns split into near-equal bands   */
    int32_t blocks;               /* CTAs per step (output)                 */
    float   ms_per_step;          /* measured by sks_autotune (output)      */
    int32_t pipeline;             /* 1: each 64-step chunk is one launch of
                                     persistent CTAs that take (step, tile)
                                     pairs in order, a tile starting once its
                                     neighbours finished the previous step
                                     (needs waves = 0); 0: one launch per
                                     step                                   */
} sks_tuning_t;

int sks_set_tuning(sks_solver *s, const sks_tuning_t *t);
int sks_get_tuning(const sks_solver *s, sks_tuning_t *t);

/* Times every candidate tuning on `steps` steps of this solve (CUDA events
 * on the solver's stream), keeps the fastest, and leaves the solve where it
 * was: the wavefield, step counter and boundary state are saved before and
 * restored after.  Needs steps+1 steps left in the run. */
int sks_autotune(sks_solver *s, int32_t steps, sks_tuning_t *best);

/* ---- instrumentation --------------------------------------------------
 * Kernel launches issued by sks_run() so far. */
int64_t sks_kernel_launches(const sks_solver *s);

/* Device time in ms of the last sks_run(): CUDA events recorded on the
 * solver's stream before its first and after its last launch. */
double sks_last_run_ms(const sks_solver *s);

/* Per-kernel-class device time: with timing on, every launch is bracketed by
 * CUDA events on the solver's stream and its time added to its class. */
#define SKS_KC_ELEMENT  0   /* fused element force + assembly + update      */
#define SKS_KC_SEAM     1   /* points shared by warp tiles                  */
#define SKS_KC_INJECT   2   /* GRT boundary injection (and step-0 set line) */
#define SKS_KC_RECORD   3   /* receiver sampling                            */
#define SKS_KC_INTERP   4   /* boundary-trace interpolation                 */
#define SKS_KERNEL_CLASSES 5
int sks_enable_kernel_timing(sks_solver *s, int on);   /* also clears the sums */
int sks_kernel_timing(const sks_solver *s, double *ms, int64_t *count);  /* arrays of SKS_KERNEL_CLASSES */

/* Measurement only, not part of a solve: the measured peak FMA throughput
 * of the device's CUDA cores in TFLOP/s (an FMA counts 2 flops), for
 * precision SKS_FP64 (the FP64 pipe the FP64 form is bound by) or SKS_FP32C
 * (FP32): independent FMA chains on every SM, the best of three event-timed
 * launches after one untimed.  The benchmark's FP64 compute roofline divides
 * by it. */
int sks_probe_fma_peak(int device, int precision, double *tflops);

/* Tests of the failure path only, not part of a solve.  The pipelined chunks
 * (tuning pipeline = 1) start a tile once its neighbours have finished the
 * previous step; every such wait gives up after a bounded number of polls,
 * sets an error flag that stops every CTA, and the run returns SKS_ERR_CUDA
 * ("a wait for neighbouring tiles ran out") with the device still usable.
 * These hooks make that happen on purpose: for the next sks_run (or the next
 * batch run) only, tile `tile` of the chunk never marks a step finished and
 * a wait gives up after spin_limit polls (128 ns apart).  The wavefield is
 * then not meaningful; sks_reset (or sks_state_load) starts over.  The
 * solver's tiles are numbered row by row over its CTA grid; a batch's over
 * its members' tiles in member order. */
int sks_test_stall_pipeline(sks_solver *s, int32_t tile, int32_t spin_limit);

/* Destroys the solver; a batch member leaves its batch first. */
void sks_destroy(sks_solver *s);

/* ---- batches ----------------------------------------------------------
 * Many solves advanced together on one GPU.  The reference runs one solve per
 * process (sem2d_psvsh.c:82, launched once per event by the driver scripts,
 * applications/test/prem_epi83.pl:81-82); a batch replaces a set of such
 * processes.  Members are ordinary solvers of one form and device, each with
 * its own mesh, materials, time step, boundary records and step count.  One
 * step of every member is one launch of a persistent kernel (or, with
 * pipeline = 1, the chunk's steps of every member are one launch whose
 * tiles start as their neighbours finish the previous step); a chunk of 64
 * steps (boundary interpolation, increments, the step launches) is one launch
 * of a CUDA graph that the batch captures once and reuses.  A member runs
 * with the batch's tuning, and its seismograms are bit-identical to the same
 * solver run alone with that tuning.  Members keep their wavefields on the
 * device between calls; solvers may join and leave between calls.  A
 * member's tuning belongs to the batch (sks_set_tuning / sks_autotune on a
 * member return SKS_ERR_STATE); sks_run on a member runs it alone. */
typedef struct sks_batch sks_batch;

int sks_batch_create(int precision, int device, sks_batch **out);
/* Joins at the solver's current step; allocates its whole-run seismogram
 * buffer on the device ([nst][3][ntrace] floats) on first joining. */
int sks_batch_add(sks_batch *b, sks_solver *s);
int sks_batch_remove(sks_batch *b, sks_solver *s);
int sks_batch_size(const sks_batch *b);

/* Advances every member by min(nsteps, the steps its run has left).  Member
 * i's new seismogram rows go to su[i], sv[i], sw[i] as sks_run() writes them
 * (any array, or any entry, may be NULL).  Returns the most steps any member
 * took, or a negative status. */
int sks_batch_run(sks_batch *b, int32_t nsteps, float *const *su, float *const *sv, float *const *sw);

/* Tuning shared by the members (waves must be 0: the batch's persistent grid
 * balances the tiles; pipeline 0 or 1).  sks_batch_autotune times every candidate on the
 * members' next `steps` steps and restores their state afterwards. */
int sks_batch_set_tuning(sks_batch *b, const sks_tuning_t *t);
int sks_batch_get_tuning(const sks_batch *b, sks_tuning_t *t);
int sks_batch_autotune(sks_batch *b, int32_t steps, sks_tuning_t *best);

double sks_batch_last_run_ms(const sks_batch *b);     /* events on the batch's stream */
/* The batch form of sks_test_stall_pipeline (tests of the failure path only). */
int sks_batch_test_stall_pipeline(sks_batch *b, int32_t tile, int32_t spin_limit);
int64_t sks_batch_kernel_launches(const sks_batch *b);
/* Destroys the batch; the members stay open and leave it. */
void sks_batch_destroy(sks_batch *b);

/* ---- serving ----------------------------------------------------------
 * Solve requests that arrive at any time (continuous batching).  The
 * reference has no counterpart: one solve is one process (sem2d_psvsh.c:82).
 * A request is a host set-up (the par words, sks_setup_open) plus its form
 * and boundary source.  The server admits queued requests first come first
 * served within each form, while their device-memory footprint fits the
 * budget and the form's running grid points stay within its cap (by default
 * 8 Mi points FP64, 24 Mi FP32C, about twice what fills the GPU; a larger
 * request runs alone), opens them on the device, and runs every admitted
 * request of a form as a member of that form's batch, a quantum of steps per
 * round, the FP32C and FP64 batches on their own streams (FP32C at the higher
 * stream priority: its quanta are short, FP64's long).
 * Requests join and leave between quanta; wavefields stay on the device; a
 * finished request's seismograms are copied once into the caller's arrays
 * and its device memory is freed.  Each result equals the same request run
 * alone with the batch's tuning, bit for bit.  submit() may be called from
 * another thread than step(). */
typedef struct sks_server sks_server;

#define SKS_REQ_QUEUED  0
#define SKS_REQ_RUNNING 1
#define SKS_REQ_DONE    2
#define SKS_REQ_FAILED  3

typedef struct {
    int32_t state;          /* SKS_REQ_*                                      */
    int32_t status;         /* the error status of a failed request           */
    int32_t precision;
    int32_t step, nst;      /* steps taken, steps of the run                  */
    int32_t ntrace;
    double  submit_s;       /* server clock (sks_server_clock), seconds;       */
    double  admit_s;        /*   -1 until it happens                          */
    double  done_s;
    int64_t device_bytes;   /* held while running; the estimate while queued  */
} sks_request_info_t;

/* budget <= 0: 90 % of the device memory free at creation.  quantum_steps:
 * steps per scheduling round (64 = one chunk). */
int sks_server_create(int device, int64_t device_budget_bytes, int32_t quantum_steps, sks_server **out);
/* A form's tuning (as sks_batch_set_tuning).  A tuning other than 4 warps
 * per CTA with register cap 0 or 1 runs GLL degree 4 only: it is refused
 * (SKS_ERR_STATE) while the form has requests of another degree queued or
 * running, and afterwards such submissions of that form are refused. */
int sks_server_set_tuning(sks_server *srv, int precision, const sks_tuning_t *t);
int sks_server_set_active_points(sks_server *srv, int precision, int64_t max_points);
/* Takes the set-up over (also on error).  pw: boundary records generated on
 * the device; NULL: read at admission from the files the par words name
 * (relative names resolved against the working directory at submission).
 * seis_u/v/w: nst*ntrace floats each, filled when the request is done (any
 * may be NULL); they must stay valid until then.  A request of GLL degree 3,
 * 5 or 6 is refused here (SKS_ERR_UNSUPPORTED) when the form's tuning cannot
 * run it.  A request whose wavefield stops being finite fails alone with
 * SKS_ERR_NONFINITE. */
int sks_server_submit(sks_server *srv, sks_setup *su, int precision, const sks_plane_wave_t *pw,
                      float *seis_u, float *seis_v, float *seis_w, int64_t *id);
/* Same with boundary records from a plane wave through a layered stack
 * (sks_set_boundary_layered_wave at admission; the stack is copied). */
int sks_server_submit_layered(sks_server *srv, sks_setup *su, int precision, const sks_stack_layer_t *layers,
                              int32_t n, const sks_layered_wave_t *wave, float *seis_u, float *seis_v,
                              float *seis_w, int64_t *id);
/* One scheduling round: retire requests whose batch quantum finished,
 * admit, launch the idle forms' next quantum.  Returns the requests queued or
 * running (0 when all are done), or a negative status. */
int sks_server_step(sks_server *srv);
int sks_server_request_info(sks_server *srv, int64_t id, sks_request_info_t *info);
int sks_server_release(sks_server *srv, int64_t id);     /* forget a finished request */
double sks_server_clock(const sks_server *srv);          /* seconds since creation */
int64_t sks_server_device_bytes(const sks_server *srv);  /* held by running requests */
void sks_server_destroy(sks_server *srv);

const char *sks_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SKS_H */
