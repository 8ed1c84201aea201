/*
 * c3d.h -- C-ABI of the GB300 (sm_103a) time step for compact3d's
 * incompressible turbulent channel flow.
 *
 * The Fortran driver of compact3d (PROGRAM MAIN, compact3d.f:11-189) keeps
 * its time loop, PARAM.H / COMMON1.FI parameters and wall-model switches.
 * It replaces the body of GETUP (compact3d.f:879-960) and the per-step
 * diagnostics DIVCHECK / CFL / CHKMF / WALLSS with calls into this library
 * through ISO_C_BINDING.  Every argument is a plain pointer, integer or
 * double; there are no C++ or PyTorch types in any signature.
 *
 * Array layouts on the host side are exactly the Fortran ones of the driver
 * (column-major, first index fastest, M1=N1, M2=N2, M3=N3):
 *   U(0:M1,0:M2,0:M3,3), HH(0:M1,0:M2,0:M3,3), SGSVIS(0:M1,0:M2,0:M3),
 *   P(M1,M2,M3), TAUW(0:M1,0:M3,2), TAUB(0:M1,0:M3,2).
 * On the device the state is kept resident between steps in the library's
 * own plane-major layout; c3d_upload / c3d_download convert.
 *
 * Return convention: 0 on success, a negative C3D_E* code on failure.  The
 * library never calls exit() or abort(); c3d_error_string() describes a code
 * and c3d_last_error() gives the message of the most recent failure on the
 * calling thread.  A channel handle is used from one host thread at a time.
 */
#ifndef C3D_H
#define C3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ------------------------------------------------------ */
#define C3D_OK            0
#define C3D_EINVAL      (-1)   /* bad extents, null pointer, unsupported size */
#define C3D_ECUDA       (-2)   /* a CUDA runtime call failed                    */
#define C3D_ENOMEM      (-3)   /* device or pinned-host allocation failed       */
#define C3D_ENOTCONV    (-4)   /* a device iteration cap was hit (wall model)   */
#define C3D_ENONFINITE  (-5)   /* NaN/Inf found by the diagnostics              */
#define C3D_ESTATE      (-6)   /* call made in the wrong state                  */
#define C3D_ENODEV      (-7)   /* no usable CUDA device                         */
#define C3D_EIO         (-8)   /* a checkpoint file could not be written or read */

/* ---- precision forms -------------------------------------------------- */
#define C3D_FP64   0   /* every operation in FP64                              */
#define C3D_MIXED  1   /* FP32 line solves / RHS / FFT; FP64 state, reductions,
                          low-wavenumber Poisson modes and bulk-flow constraint */
#define C3D_MIXED_IR 2 /* C3D_MIXED plus one step of iterative refinement of the
                          pressure solve: the residual div(U)/DT of the corrected
                          field in double-float arithmetic, a second solve and
                          update; the projected field is divergence-free to about
                          FP64 rounding */

/*
 * Grid and model description.  It carries the values the reference keeps in
 * COMMON blocks after SETUP/MESH (compact3d.f:192-443):
 *   /DIM/   N1,N2,N3                       -> n1,n2,n3 (points; cells = n-1)
 *   /SIZE/  ALX,ALY,ALZ,VOL                -> alx,aly,alz,vol
 *   /MESH1/ DX1,DX3 (= N1M/ALX, N3M/ALZ)   -> dx1,dx3
 *   /MESH2/ Y(0:N2)                        -> y     (n2+1 values)
 *   /MESH3/ DY(0:N2),H,HM,HC,HP(1:N2)      -> dy    (n2+1 values, DY(0)=DY(N2)=0)
 *                                             h,hm,hc,hp (n2 values, index J-1)
 *   /MESH4/ DYM,DYC,DYP(1:N2)              -> dym,dyc,dyp (n2 values, index J-1)
 *   /PARA/  RE                             -> re
 *   /FINOUT/ FILES (SGS model)             -> files  (0 none, 1 SGSDY, 2 SGSCS,
 *                                             3 SGSSD)
 *   /WALLMODEL/ WMODEL                     -> wmodel (0 none, 1 WALLMODEL_INSTANT,
 *                                             2 WALLMODEL_IWMLES_SMOOTH, 3 MARUSIC1,
 *                                             4 WALLMODEL_WERNER, 5 PIOMELLI; with 1
 *                                             and 2, Y0 = Y(0) != 0 selects
 *                                             WALLMODEL_ROUGH / _IWMLES_ROUGH
 *                                             (0 < Y0 < DY(1)+DY(2)+DY(3)/2);
 *                                             4 needs N3 <= N1;
 *                                             3 and 5 need Y(1:N2) increasing, see
 *                                             below)
 * The library takes the driver's metric arrays as given; it recomputes only
 * the Poisson metrics of INIWAVE / METRICPOISSON (compact3d.f:9182-9263),
 * which depend on nothing else.
 */
typedef struct c3d_grid {
    int n1, n2, n3;
    double alx, aly, alz, vol;
    double dx1, dx3;
    double re;
    const double *y;
    const double *dy;
    const double *h, *hm, *hc, *hp;
    const double *dym, *dyc, *dyp;
    int files;
    int wmodel;
    int precision;      /* C3D_FP64 or C3D_MIXED */
} c3d_grid;

/* Diagnostics of one step (DIVCHECK, CFL, CHKMF, WALLSS; compact3d.f:9049-9169,
 * 9463-9503, 11077-11143).  Reductions are accumulated in FP64 in every form. */
typedef struct c3d_diag {
    double divmax;      /* DIVCHECK: max |div u|                              */
    double cflm;        /* CFL: max local CFL number / DT                    */
    double flow1;       /* CHKMF: flow rate through plane i=1 (per unit z)   */
    double flow3;       /* CHKMF: flow rate through plane k=1                */
    double wsm[3];      /* WALLSS: plane-mean wall shear / RE / ALY          */
    int    nonfinite;   /* 1 if any NaN/Inf was met in the reductions        */
} c3d_diag;

typedef struct c3d_channel c3d_channel;   /* one channel, device-resident   */
typedef struct c3d_batch   c3d_batch;     /* many channels, one launch      */

/* ---- library ---------------------------------------------------------- */
const char *c3d_error_string(int code);
const char *c3d_last_error(void);
int c3d_version(void);
/* Selects the CUDA device used by channels created afterwards on this thread. */
int c3d_set_device(int device);

/* ---- one channel -------------------------------------------------------
 * c3d_create    replaces SETUP's INIWAVE/METRICPOISSON and allocates the
 *               device state (compact3d.f:192-299, 9182-9263).
 * c3d_upload    copies U, P, HH (and SGSVIS, may be NULL) from Fortran arrays
 *               to the device; PRESG/PRESG3 are passed to c3d_step.
 * c3d_download  copies them back (any pointer may be NULL to skip it).
 * c3d_step      one call of GETUP(U,P,HH,SS,NTIME,PRESG,PRESG3,SGSVIS)
 *               (compact3d.f:879-960): BCOND, RHS1-3 with AB2, GETUH1-3
 *               (Crank-Nicolson ADI), RHSDP, GETDP (FFT Poisson), UPCALC.
 *               dt is COMMON /TSTEP/ DT; presg/presg3 are in-out.
 * c3d_diagnose  DIVCHECK + CFL + CHKMF + WALLSS on the current device state.
 * c3d_getup     drop-in for a driver that keeps the fields on the host:
 *               upload, step, download in one call.
 *
 * LES (files != 0, compact3d.f:931-937): each step zeroes SGSVIS and runs the SGS
 * model (SGSDY, SGSCS or SGSSD) and, with wmodel != 0, the wall model before BCOND; the
 * SGS fluxes and the wall-stress terms enter RHS1-3.  SGSVIS passed to c3d_upload
 * is not used (the step recomputes it); c3d_download / c3d_getup return it.  With
 * wmodel = 0 the step first evaluates WALLSS on the current field, which is what the
 * driver's time loop does right before GETUP (compact3d.f:125), so SGSCS sees the
 * same WSM.  A wall point whose Newton iteration for u_tau exceeds the iteration cap
 * (default 10000; the reference iterates without one) makes c3d_step / c3d_sync
 * return C3D_ENOTCONV after the step completes.  WALLMODEL_WERNER (compact3d.f:
 * 4815-4958) sets both walls' stresses from the Werner-Wengle power law and WSM(1)
 * from the bottom wall; like the reference it takes the x neighbour of a wall point
 * with the z index (IPA(K), IMA(K)), which the reference's index arrays allow only for
 * N3 <= N1, so c3d_create refuses wmodel = 4 on other grids.  SGSSD (files 3,
 * compact3d.f:1502-1948) is the scale-dependent dynamic model: per plane the Germano
 * sums at the test filters 2 DELTA (FILTER) and 4 DELTA (FILTER4) give a quintic
 * (COEFFICIENT) whose largest real root in (0, 2), by the reference's companion-matrix
 * QR iteration with its deflation tolerance 1e-5 (DQRRT/CHHQR), is the scale
 * dependence BETA; the coefficient is the dynamic one at 2 DELTA with BETA in M_ij (the
 * reference's file BETA.plt is not written).  MARUSIC1 (wmodel 3,
 * compact3d.f:4336-4495) and PIOMELLI (wmodel 5, 4960-5110) take u_tau of each wall
 * from the log law on the plane mean of u at a reference plane (MARUSIC1: the Y(J)
 * nearest 0.06; PIOMELLI: the first cell) by the reference's bisection, and set both
 * walls' stresses from the velocity interpolated trilinearly at a point shifted
 * downstream (MARUSIC1: by DELTAP / tan 16 deg; PIOMELLI: not shifted, its DELTP is
 * never set); WSM(1) is the bottom wall's u_tau^2.  They search the Y faces for the
 * interpolation cell, so Y(1:N2) must increase; PIOMELLI's height H(1) climbs by 1e-6
 * per wall point while it lies below YC(1), as the reference's by-reference INDEX_IJK
 * does, and c3d_create refuses grids where it starts more than 2e-3 below.
 * WALLMODEL_IWMLES_SMOOTH (wmodel 2, compact3d.f:3386-4279) is the integral wall model
 * on the bottom wall: its per-point state (filtered velocity and pressure, integrals,
 * u_tau) is initialised at NTIME = 1 (or at the channel's first step with it) from the
 * log law on the mean u of plane 3 and CFLMAX (c3d_set_cflmax, default 1), updated every
 * fifth step (NTIME mod 5 = 0, the NTIME passed to c3d_step) and imposed every step;
 * the spanwise stress the reference writes to TAUW(I,K,3), beyond TAUW, lands on
 * TAUB(I,K,1) of /TAUXYZ/, where it is stored; WSM(1) is the plane mean of
 * |(tauwx, tauwy)|.  Batches refuse it (its schedule follows NTIME).
 * c3d_upload_wall / c3d_download_wall  TAUW, TAUB (0:M1,0:M3,2) of /TAUXYZ/ (the
 *               interior I = 1..N1M, K = 1..N3M of both walls; either may be NULL).
 *               WALLMODEL_INSTANT updates the bottom wall (index 1) and the top
 *               wall keeps what was uploaded, as in the reference; WERNER, MARUSIC1
 *               and PIOMELLI update both walls.
 * c3d_set_wsm / c3d_get_wsm  /WSMEM/ WSM(1:3) as the SGS model reads it and the
 *               wall model writes WSM(1).
 */
int c3d_create(const c3d_grid *grid, c3d_channel **out);
int c3d_destroy(c3d_channel *ch);
int c3d_upload(c3d_channel *ch, const double *u, const double *p,
               const double *hh, const double *sgsvis);
int c3d_download(c3d_channel *ch, double *u, double *p, double *hh,
                 double *sgsvis);
int c3d_upload_wall(c3d_channel *ch, const double *tauw, const double *taub);
int c3d_download_wall(c3d_channel *ch, double *tauw, double *taub);
int c3d_set_wsm(c3d_channel *ch, const double *wsm);
int c3d_get_wsm(c3d_channel *ch, double *wsm);
/* Newton iterations allowed per wall point (>= 1).  No counterpart in the reference,
 * whose loop is unbounded; the cap turns a non-converging point into an error. */
int c3d_set_wall_iter_cap(c3d_channel *ch, int cap);
int c3d_step(c3d_channel *ch, int ntime, double dt,
             double *presg, double *presg3);
int c3d_diagnose(c3d_channel *ch, c3d_diag *out);
int c3d_getup(c3d_channel *ch, double *u, double *p, double *hh,
              double *sgsvis, int ntime, double dt,
              double *presg, double *presg3);
/* Pressure projection of the current velocity (RHSDP + GETDP + UPCALC with
 * U taken as the intermediate velocity and DT = 1, no bulk-flow forcing).
 * Used to make a synthetic initial condition discretely divergence-free. */
int c3d_project(c3d_channel *ch);
/* Page-locks (pins) a host array; a driver calls it once per field array.
 * c3d_upload / c3d_download / c3d_getup then move registered arrays by DMA at the
 * host link's rate through a device staging area with one slot per field (U, P, HH,
 * SGSVIS: about 2.2 GB for 384x257x384, allocated on first use), and c3d_getup
 * overlaps the transfers of HH with the step.  Unregistered arrays go through a
 * one-field staging buffer, one field at a time. */
int c3d_host_register(void *ptr, size_t bytes);
int c3d_host_unregister(void *ptr);
/* Allocates `bytes` of page-locked host memory (cudaHostAlloc, mapped) for a driver's
 * field arrays, and frees it.  Arrays allocated here move at the host link's rate
 * whatever the state of the host's memory; an existing array that c3d_host_register
 * pins keeps the physical pages it happens to have, and on a host whose free memory is
 * fragmented (for example after another process used and released tens of GB) its
 * transfers measured four times slower.  No counterpart in the reference. */
int c3d_host_alloc(size_t bytes, void **ptr);
int c3d_host_free(void *ptr);
/* Blocks until all work queued on the channel's stream has finished. */
int c3d_sync(c3d_channel *ch);
/* Device time of the last c3d_step in milliseconds (CUDA events on the
 * channel's stream), and the number of kernels that step launched. */
int c3d_last_step_stats(c3d_channel *ch, double *ms, int *kernel_launches);

/* Device-resident driving: c3d_step_async queues one GETUP on the channel's
 * stream and returns without waiting; PRESG/PRESG3 stay on the device
 * (c3d_set_presg before the first step, c3d_get_presg to read them, which
 * waits for the queued work). */
int c3d_step_async(c3d_channel *ch, int ntime, double dt);
/* CFLMAX of the driver, which WALLMODEL_IWMLES_SMOOTH's initial filter time scale uses
 * (wm_tR = (CFLMAX ALX / N1M / U) / (DZ / 0.4 / u_tau)); default 1. */
int c3d_set_cflmax(c3d_channel *ch, double cflmax);
int c3d_set_presg(c3d_channel *ch, double presg, double presg3);
int c3d_get_presg(c3d_channel *ch, double *presg, double *presg3);
/* CUDA-event timer on the channel's stream: start, then stop returns the
 * device time between the two marks in milliseconds (waits for the stop). */
int c3d_timer_start(c3d_channel *ch);
int c3d_timer_stop(c3d_channel *ch, double *ms);
/* Per-kernel profile of subsequent steps (CUDA events around every launch).
 * c3d_profile_get returns, for kernel index idx < c3d_profile_count(),
 * its name, accumulated device time, launch count and the algorithmic bytes
 * of one launch (compulsory reads + writes of that kernel). */
/* Diagnostic with no counterpart in the reference: runs the bounded wait that the
 * shared-memory staged x passes use for their bulk copies, on a barrier that nothing
 * arrives on, so that it runs out after limit_ms (0 < limit_ms <= 1000).  It sets the
 * channel's pipeline-error flag as a stalled stage would: the next c3d_sync (and every
 * later step of the channel) returns C3D_ECUDA with the stall message.  It shows that a
 * stalled copy ends in an error code instead of a hung kernel. */
int c3d_pipe_wait_selftest(c3d_channel *ch, double limit_ms);
int c3d_profile(c3d_channel *ch, int enable);
int c3d_profile_count(c3d_channel *ch);
int c3d_profile_get(c3d_channel *ch, int idx, const char **name, double *ms,
                    int *launches, double *bytes_per_launch);

/* ---- allocation-free divergence check ----------------------------------
 * No counterpart in the reference (it is an addition for callers of this
 * library, not a replacement of a compact3d routine).  c3d_divcheck_noalloc
 * computes DIVCHECK's max|div u| (the same operators as c3d_diagnose) for a
 * host velocity U(0:N1,0:N2,0:N3,3) in the driver's Fortran layout, for callers
 * that must not allocate device memory: drivers whose device memory belongs to
 * their own pool allocator, and long-running loops whose footprint must stay
 * fixed after start-up.  It calls no cudaMalloc/cudaFree; its scratch is one
 * static __device__ array of C3D_NOALLOC_MAX_BYTES that every GPU loading the
 * library keeps until exit, so grids whose working set (about 8 bytes x
 * ((N1+1)(N2+1)(N3+1) + 4 (N2+1)(N1-1)(N3-1))) exceeds it return C3D_EINVAL.
 * Only grid->n1..n3, dx1, dx3 and dy are read.  Extents: c3d_create's rules
 * without its FFT-length ones (DIVCHECK has no FFT): N1-1 even, >= 16 and split
 * into 32 lane chunks of 1, 2, 3, 4, 6, 8 or 12; N3-1 a multiple of 16; N2-1 in
 * [4, 4096].  All calls share that scratch: calls that overlap on the GPU race,
 * so serialise them.  The first call on a device looks up the scratch address
 * (cudaGetSymbolAddress).  Every call issues its copies and kernels on the legacy
 * default stream and synchronises it, so no call (the first or any later one) may
 * run while a stream capture is active on that device; the call returns when
 * *divmax is ready. */
#define C3D_NOALLOC_MAX_BYTES (64u * 1024u * 1024u)
int c3d_divcheck_noalloc(const c3d_grid *grid, const double *u, double *divmax);

/* ---- plane statistics --------------------------------------------------------
 * c3d_plane_stats computes, on the device and in FP64, the plane statistics of
 * ENERGY (compact3d.f:10003-10232) for the current state: out[(J-1)*29 + q] for
 * J = 1..N2M with q =
 *    0-2  VM(J,1..3)   mean cell-centre u, v, w
 *    3    PM(J)        mean P
 *    4-6  WM(J,1..3)   mean vorticity (cell centres, ENERGY's stencils)
 *    7-12 VRMS(J,1..6) mean uu, vv, ww, uv, uw, vw
 *    13   PRMS(J)      mean pp          14  PV(J)   mean pv
 *    15-17 WRMS(J,1..3) mean squared vorticity components
 *    18   U2V(J)       mean uuv         19  VW2(J)  mean vww
 *    20-22 VSKEW(J,1..3), 23-25 VFLAT(J,1..3)  third and fourth central moments
 *    26-28 DUDY, DVDY, DWDY mean wall-normal gradients
 * (raw moments as ENERGY stores them; the time averaging of TAVER and the output of
 * WRITEAVG stay with the driver).  ENERGY's spectra and two-point correlations are
 * c3d_plane_spectra's, its quadrant analysis c3d_plane_quadrants' (its budget terms are
 * commented out in the reference). */
int c3d_plane_stats(c3d_channel *ch, double *out);

/* c3d_plane_spectra computes ENERGY's 1-D energy spectra and two-point correlations
 * (compact3d.f:10243-10515) for the current state, in FP64.  vmo (VMO(J,L), 3*N2M
 * values, J fastest; NULL: the instantaneous plane means VM) is the mean the spectra
 * subtract; the reference passes TAVER's running average.  Outputs are Fortran arrays,
 * each may be NULL:
 *   xspec XSPCTR(1:N1M,1:N2M,3)  sum over the x lines of |DFT(v_L - VMO)|^2 / N1M /
 *                                (PI DX1), divided by N3M (wavenumber index I-1)
 *   zspec ZSPCTR(1:N3M,1:N2M,3)  the same along z, / N3M / (PI DX3) / N1M
 *   rxx   RXX(1:N1M,1:N2M,3)     sum_K VP(N1H,J,K) VP(I,J,K) / N3M / (VRMS - VM^2)
 *   rzz   RZZ(1:N3M,1:N2M,3)     sum_I VP(I,J,N3H) VP(I,J,K) / N1M / (VRMS - VM^2)
 *   rxy   RXY(1:N1M,1:N2M,3)     sum_K VP(N1H,1,K) VP(I,J,K) / N3M / the two rms
 * with VP = v_L - VM(J,L), V between J and JPA(J) (JPA(N2M) = N2M), N1H = N1M/2 + 1,
 * N3H = N3M/2 + 1. */
int c3d_plane_spectra(c3d_channel *ch, const double *vmo, double *xspec, double *zspec, double *rxx, double *rzz,
                      double *rxy);

/* c3d_plane_quadrants: ENERGY's quadrant analysis (compact3d.f:10560-10604) for the
 * current state, FP64: out[(J-1)*8 + q] = Q(J,1..4) for q = 0..3, the sums of
 * u'v' over the points of quadrants 1-4 of (u', v') negated and divided by N1M N3M, and
 * QP(J,1..4) for q = 4..7, the quadrants' point fractions, with u' = u - VMP(J,1),
 * v' = v - VMP(J,2) of the cell-centre velocities.  vmp (2*N2M, J fastest) may be NULL:
 * the reference's VMP is a local whose assignments are commented out, zero-valued in
 * practice, which NULL reproduces. */
int c3d_plane_quadrants(c3d_channel *ch, const double *vmp, double *out);

/* c3d_wall_spectrum: ENERGY's 2-D spectrum of the bottom wall's streamwise stress
 * (compact3d.f:10394-10416), SPECTAUW(I,K,1) = |DFT2(TAUW(.,.,1) - utau^2)(I-1,K-1)|^2
 * / N1M / N3M / (PI DX3) / (PI DX1), out Fortran (N1M, N3M), FP64; utau is the friction
 * velocity the driver holds (the reference's sqrt of the averaged wall stress).
 * c3d_corr3d: ENERGY's 3-D two-point correlation (10524-10556), out RXYZ(N1M,N2M,N3M,3)
 * = VP(N1H,N2H,N3H,L) VP(I,J,K,L) / rms(J,L) / rms(N2H,L), VP and rms as for
 * c3d_plane_spectra, N2H = N2M/2 + 1 with ALY = 1 and N2M/4 + 1 otherwise. */
int c3d_wall_spectrum(c3d_channel *ch, double utau, double *out);
int c3d_corr3d(c3d_channel *ch, double *out);

/* ---- Lagrangian particles ------------------------------------------------------
 * The particle routines of the reference (compact3d.f:11817-12894) with their calls in
 * the time loop commented out (GET_PAR at 128, SOURCE_PAR at 1026).  Particles are
 * par[6*q .. 6*q+5] = x, y, z, u, v, w (the reference's PAR(1:6, q)); diam (m), dens and
 * hhh (m) give INIT_PAR's DIAM_P = diam / hhh, MASS_P and TAU_P = dens DIAM_P^2 / 18 RE.
 * c3d_particles_advance: one CALC_UX_4RK step of dt on the device with FORCE_PAR's
 *   Clift-Gauvin drag and gravity and INDEX_IJK / INTERPOLAT of the current field at every
 *   stage (the explicit Euler step when a stage leaves the channel), then BC_PAR's
 *   periodic shifts and top-wall reflection; impact[q] (may be NULL) = 1 for a particle
 *   that reached the bottom wall moving down, where the reference calls SPLASH (its draws
 *   come from RAN2 seeded by CPU_TIME and are left to the driver).  par is updated.
 * c3d_particles_source: SOURCE_PAR's two-way coupling terms for the particles, written to
 *   ruh1..3 (Fortran (0:N1,0:N2,0:N3) each, zero elsewhere). */
int c3d_particles_advance(c3d_channel *ch, int n, double *par, double diam, double dens, double hhh, double dt,
                          int *impact);
int c3d_particles_source(c3d_channel *ch, int n, const double *par, double diam, double dens, double hhh,
                         double *ruh1, double *ruh2, double *ruh3);

/* ---- checkpoint ------------------------------------------------------------
 * The restart pair of the reference, CWRITE / READUP (compact3d.f:741-872), writes a
 * list-directed text file and reads it back unformatted in another loop order, so the
 * two do not round-trip.  These write and read one fixed format that does, straight
 * from and into the device state: Fortran sequential unformatted records (a 4-byte
 * little-endian length before and after each record), REAL*8 values, CWRITE's content
 * and loop order:
 *   1. N1M, N2M, N3M                                    (INTEGER*4 x 3)
 *   2. PRESG, PRESG3                                    (REAL*8 x 2)
 *   3. NTIME                                            (INTEGER*4)
 *   4. TIME                                             (REAL*8)
 *   5. ((( U(I,J,K,1), U(I,J,K,2), U(I,J,K,3), I=1,N1M), J=0,N2), K=1,N3M)
 *   6. ((( P(I,J,K), I=1,N1M), J=1,N2M), K=1,N3M)
 *   7. (((( HH(I,J,K,NV), I=1,N1M), J=1,N2M), K=1,N3M), NV=1,3)   (AB2 history)
 *   8. with an SGS model only: TAUW(0:M1,0:M3,2), TAUB(0:M1,0:M3,2), WSM(3)
 * Records 1 and 7-8 extend CWRITE so that a restart continues the run exactly (the
 * reference restarts with HH = 0).  A record longer than 2^31 - 1 bytes (more than
 * 89 M points per component) is refused with C3D_EINVAL.  c3d_checkpoint_read checks
 * the extents against the channel's grid (C3D_EINVAL) and the length and both markers
 * of every record (C3D_EIO) before it replaces any of the channel's state, then leaves
 * the state as read; if reading still fails after that check, the channel has no state
 * (c3d_step returns C3D_ESTATE) until one is uploaded or read.  A Fortran driver reads
 * the file with one unformatted READ per record, in the order above. */
int c3d_checkpoint_write(c3d_channel *ch, const char *path, int ntime, double time, double presg,
                         double presg3);
int c3d_checkpoint_read(c3d_channel *ch, const char *path, int *ntime, double *time, double *presg,
                        double *presg3);

/* ---- launch schedule -----------------------------------------------------
 * The kernels' launch shapes are chosen per grid shape by an autotuner written for
 * this library (no counterpart in the reference).  A schedule is sixteen ints
 * (C3D_SCHEDULE_LEN):
 *   [0..4] z-line segment length (8, 16, 32) of each z pass: the points each thread
 *       solves sequentially (Thomas-like) before the parallel segments of a z line
 *       meet; or 0: one block per 32 z lines of a plane, each thread one segment of
 *       8, 12 or 16 points, the segments of a line joined exactly through shared
 *       memory (N3M / segment length <= 32; otherwise segments of 16)
 *   [5] rows per block of the x passes (2, 4, 8)
 *   [6] kx columns per block of the z FFT (4, 8, 16), or 0: one warp per kx column,
 *       four-step form (N3M / 32 points per lane in registers, then a 32-point
 *       shuffle FFT across the lanes) when N3M is 32 x 2, 3, 4, 6, 8, 12 or 16
 *   [7], [8] radix order of the x and z FFT plans (0: radix 4 first, 1: radix 3
 *       first, 2: radix 2 only, then 3); [7] = 3 runs the row FFTs of the pressure
 *       x passes in registers (four-step form, no shared memory) and is accepted only
 *       when N1M is a multiple of 64 (N1M / 32 even)
 *   [9] the z pass of the explicit terms as one kernel (0) or as its three sweeps
 *       in three kernels (1)
 *   [10] the x pass of the explicit terms as one kernel (0) or as its u, v and w
 *       pieces in three kernels (1)
 *   [11] x passes whose rows each warp reads from global memory (0) or streams into
 *       shared memory through a ring of 2 or 3 bulk-copy stages (persistent warps;
 *       mixed form, N1M a multiple of 4)
 *   [12] the u, v and w pieces of the explicit x pass (with [10] = 1) read their rows
 *       from global memory (0), or stage every row of a warp's (J, K) in shared memory
 *       by one bulk copy per row before computing (1; N1M even)
 *   [13] the wall-normal Crank-Nicolson factor (TDMAI): one thread per column with
 *       register batches of planes (0), or blocks of 32 or 64 columns whose planes
 *       are staged in shared memory by bulk copies so that each value is read and
 *       written once (falls back to 0 when the tile exceeds shared memory)
 *   [14] lanes per row of the explicit x pieces read from global memory, of the
 *       x pass of the remaining terms, and of the pressure x passes with the
 *       shared-memory row FFT ([7] != 3) and no bulk-copy ring ([11] = 0): 0 (a warp
 *       per row), or the row segment of short rows, accepted only at N1M = 48, 64,
 *       96 (8 lanes) or 128 (16 lanes) with N3M a multiple of 32 / lanes, so that each
 *       lane holds 6 to 12 points and the cross-lane scans of the line solves take 3
 *       or 4 steps instead of 5
 *   [15] the u, v and w pieces of the explicit x pass ([10] = 1), then those of the
 *       explicit z pass ([9] = 1), as three concurrent branches on three streams (1)
 *       or one after another (0); they write disjoint fields.  The per-kernel profile
 *       (c3d_profile) runs them one after another; c3d_autotune sets this knob by
 *       the time of whole unprofiled steps
 * c3d_autotune  times the candidates on a scratch channel of the same grid holding a
 *               copy of this channel's state (so the channel needs its state), keeps
 *               the fastest per kernel group, applies it, and caches it per grid
 *               shape, form and models for the process; `sched` (may be NULL)
 *               receives the result.
 * c3d_set_schedule / c3d_get_schedule  set or read a schedule directly.
 * Channels of a batch are tuned before the batch's first step captures its graph. */
#define C3D_SCHEDULE_LEN 16
int c3d_autotune(c3d_channel *ch, int *sched);
int c3d_get_schedule(c3d_channel *ch, int *sched);
int c3d_set_schedule(c3d_channel *ch, const int *sched);

/* ---- operators one at a time ---------------------------------------------
 * No single routine of the reference corresponds: these are the operators inside
 * RHS1-3 / RHSDP / GETDP, exposed for operator-level checks and measurement.
 * c3d_op_set    loads one field F(0:M1,0:M2,0:M3) (the layout of one component of U)
 *               as the operand, converted to the channel's working precision.
 * c3d_op_apply  applies operator `op` `count` times, each time from the operand to
 *               the result, asynchronously on the channel's stream (time it with
 *               c3d_timer_start / c3d_timer_stop).  The result holds J = 1..N2M
 *               (J = 2..N2M for C3D_OP_DY1); other planes are zero.
 * c3d_op_get    copies the result back in the same layout (periodic ghost columns
 *               filled, wall planes zero).
 *   C3D_OP_DX1  (1,22,1) X = 24 DX1 (F(I+1) - F(I))            CTDMA11, e.g. RHS1 loop 50
 *   C3D_OP_DX2  (1,10,1) X = 12 DX1^2 (F(I-1) - 2F(I) + F(I+1))  CTDMA11, RHS1 loop 20
 *   C3D_OP_IX   (1,6,1)  X = 4 (F(I) + F(I+1))                  CTDMA11, RHS1 loop 50
 *   C3D_OP_DZ1, C3D_OP_DZ2, C3D_OP_IZ   the same along z        CTDMA33
 *   C3D_OP_DY1  (F(J) - F(J-1)) / H(J)                          RHS2 loop 10
 *   C3D_OP_DY2  HP(J) F(J+1) - HC(J) F(J) + HM(J) F(J-1)         RHS1 loop 10
 *   C3D_OP_POISSON  GETDP: DP from RDP = F at J = 1..N2M        compact3d.f:9271-9441
 */
#define C3D_OP_DX1      1
#define C3D_OP_DX2      2
#define C3D_OP_IX       3
#define C3D_OP_DZ1      4
#define C3D_OP_DZ2      5
#define C3D_OP_IZ       6
#define C3D_OP_DY1      7
#define C3D_OP_DY2      8
#define C3D_OP_POISSON  9
int c3d_op_set(c3d_channel *ch, const double *f);
int c3d_op_apply(c3d_channel *ch, int op, int count);
int c3d_op_get(c3d_channel *ch, double *f);

/* ---- batched ensemble --------------------------------------------------
 * Many independent channels (any mix of grid sizes, RE and precision) that
 * advance together.  c3d_batch_step runs one GETUP on every channel as a single
 * CUDA graph (captured on the first call and whenever a channel's DT changes),
 * in one of two forms:
 *   C3D_BATCH_WORKLIST (the default; used when every channel is DNS, FILES = 0,
 *     in one precision, C3D_FP64 or C3D_MIXED): each pass of the step is one
 *     kernel launch over the blocks of all channels whose kernel for that pass
 *     is the same template instance (same x lane chunk N1M/32, same z-FFT
 *     shape), each block working on the channel a device work list names; a
 *     step is about 20 launches for the whole ensemble.  The work-list form
 *     runs a fixed schedule (x rows per block 2, xA and zA in pieces, z
 *     segments of 8, 8, 16, 16, 8 points for zA..zE unless
 *     c3d_batch_set_z_segments says otherwise, the
 *     four-step z FFT where N3M = 32 N1, else tiles of 8, register row FFTs
 *     where N1M is a multiple of 64, rows of 48-128 points in segments of 8 or
 *     16 lanes as schedule knob [14] describes), not the channels' own.
 *   C3D_BATCH_STREAMS (and any other batch): every channel's step, with its own
 *     schedule, on its own stream; the channels run concurrently.
 * presg/presg3 are in-out arrays of nchan values; the call returns when the
 * step is done.  Upload each channel's state with c3d_batch_channel +
 * c3d_upload first.  c3d_batch_set_form chooses the form (the graphs are
 * captured again); c3d_batch_get_form reports the form the next step runs.
 * c3d_batch_set_groups (work-list form; default 2) splits the channels into
 * that many groups, largest first and dealt in turn, each with its own work
 * lists on its own stream, so that the passes of one group run beside those of
 * another instead of every pass waiting for the whole ensemble.
 * c3d_batch_set_z_segments (work-list form) sets the segment length of the z
 * passes zA, zB, zC, zD, zE (seg[0..4], each 8, 16 or 32; a channel whose N3M is
 * not a multiple of it runs 16).  c3d_batch_set_x_warps (work-list form) sets
 * the warps per block of the x passes (2, 4 or 8; default 2).  c3d_batch_set_concurrent
 * (work-list form; default 0) runs the three pieces of the explicit x pass, and then
 * those of the explicit z pass, of each channel group as concurrent branches (1) or one
 * after another (0); the pieces write disjoint fields, so the results do not change.
 * Concurrent pieces pay with one channel group and cost with two (the default), where
 * the groups already overlap.
 */
#define C3D_BATCH_STREAMS   0
#define C3D_BATCH_WORKLIST  1
int c3d_batch_create(int nchan, const c3d_grid *grids, c3d_batch **out);
int c3d_batch_destroy(c3d_batch *b);
int c3d_batch_channel(c3d_batch *b, int index, c3d_channel **ch);
int c3d_batch_step(c3d_batch *b, int ntime, const double *dt,
                   double *presg, double *presg3);
int c3d_batch_sync(c3d_batch *b);
int c3d_batch_set_form(c3d_batch *b, int form);
int c3d_batch_get_form(c3d_batch *b, int *form);
int c3d_batch_set_groups(c3d_batch *b, int groups);
int c3d_batch_set_z_segments(c3d_batch *b, const int *seg);
int c3d_batch_set_x_warps(c3d_batch *b, int warps);
int c3d_batch_set_concurrent(c3d_batch *b, int on);
/* Device time of the last ensemble step (CUDA events around the graph launch) and the
 * number of kernels one ensemble step runs. */
int c3d_batch_last_step_stats(c3d_batch *b, double *ms, int *kernel_launches);

#ifdef __cplusplus
}
#endif
#endif /* C3D_H */
