// c3d_internal.h -- channel state shared by the C-ABI layer and the step kernels.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "../../include/c3d.h"
#include "c3d_dev.cuh"

namespace c3d {

// Radix plan of one FFT length (radices 4, 2, 3 in that order) with its twiddle table
// tw[q] = exp(-2 pi i q / n), q in [0, n).
struct FftPlan {
    int n;
    int nst;
    int rad[16];
    // jj / Ns at stage s (Ns = product of the earlier radices, > 1) as
    // __umulhi(jj, dmag[s]) with dmag = ceil(2^32 / Ns): exact for jj < 2^20 and
    // Ns <= 2^12, and checked for every jj < n when the plan is made
    unsigned dmag[16];
    const double2 *tw64;
    const float2 *tw32;
};

// Storage type of the state (u, v, w, P): FP64 in the FP64 form, double-float pairs
// (hi, lo FP32) in the mixed form.
template <typename R> struct SType;
template <> struct SType<double> { typedef double S; };
template <> struct SType<float> { typedef float2 S; };

// Wall-normal metrics in the working precision, indexed by Fortran J (n2+1 values each):
// the MESH arrays plus rh = 1/H, hdy = DY/2 and rdy = 1/DY, precomputed in FP64 on the
// host (so the FP64 form sees exactly the reference's values) and converted once.
template <typename R>
struct MetR {
    const R *hp, *hc, *hm, *hz, *dyp, *dyc, *dym, *dyz, *h, *rh, *hdy, *rdy, *dy;
};
constexpr int NMETR = 13;

// Everything one step's kernels need, passed by value.  R is the working precision of
// the intermediates (double for the FP64 form, float for the mixed form).
template <typename R>
struct StepArgs {
    typedef typename SType<R>::S S;
    Geo g;
    MetR<R> m;                          // wall-normal metrics in precision R
    // constants in precision R, computed once on the host in FP64:
    // 1/RE, 12 DX1^2, 24 DX1, 12 DX3^2, 24 DX3, 1/DT, 1/(N1M N3M) (inverse-FFT scale)
    R re1, f12x, f24x, f12z, f24z, rdt, xscale;
    S *u, *v, *w, *p;                   // state
    R *hh[3];                           // nonlinear terms of this step (written)
    const R *ho[3];                     // nonlinear terms of the previous step (AB2)
    R *r[3];                            // RUH, then the x/y CN factors in place
    R *exy, *exz, *eyz, *ww1, *wsq;     // edge products and interpolants
    R *rdpz, *g1;                       // z part of div(UH)/DT; x-gradient of DP
    R *dp;                              // pressure increment (planes 1..N2M)
    void *spec;                         // half spectrum [j][kz][kx] of RDP / DP (R complex)
    double *scal;                       // device scalars (see SCAL_*)
    double *part;                       // per-row partial sums for the bulk-flow forcing
    Cyc<R> c6x, c10x, c22x, c6z, c10z, c22z, cnx, cnz;
    const double *ycn;                  // CN wall-normal factors: 3 comps x (A, RBET, GAM) x (n2+1)
    const double *prb, *pgam;           // Poisson factor tables [j][mode], FP64
    const float2 *prbdf, *pgamdf;       // the same as double-float pairs (mixed form)
    const double *pmj;                  // PMJ(J), n2+1 values
    const float2 *pmjdf;                // the same as double-float pairs
    const float2 *bulkw;                // DY(J)/DX3/DX1 as double-float pairs (mixed form)
    FftPlan fx, fz;                     // complex FFT of length N1M/2 (x) and N3M (z)
    const double2 *twx64;               // exp(-2 pi i k / N1M), k in [0, N1M/2]
    const float2 *twx32;
    double dt;                          // DT of the step (1 for the projection)
    int bulk;                           // apply the bulk-flow forcing (GETUP) or not (projection)
    const R *ycnw;                      // the CN wall-normal factors in precision R
};

// ---- work-list launches of a batch of channels -----------------------------------
// One launch of a step pass covers every channel of a group (channels whose kernel for
// that pass is the same template instance with the same block shape): block q of the
// launch runs block (x, y) of channel ch's own grid, whose x extent is gx.
struct BMap { int ch; unsigned x, y, gx; };
// One pass of one channel in the batch form: the batch kernel (its template instance is
// the group key), the block size, dynamic shared memory and the blocks of the channel's
// own grid.  Batch kernels take (const StepArgs<R> *args, const BMap *map).
// run > 0: the pass is piece `piece` (0-2) of a run of three independent passes that the
// work-list capture may launch as concurrent branches (run 1: xA's pieces, run 2: zA's).
struct BKern {
    const void *fn;
    unsigned block;
    size_t smem;
    unsigned nblocks;
    int run = 0, piece = 0;
};

// Blocks of the first level of the bulk-flow reduction; `part` holds 2 N2M N3M per-row
// partials followed by 2 RB block sums.
constexpr int RB = 64;

enum {
    SCAL_PRESG = 0,
    SCAL_PRESG3 = 1,
    SCAL_DMPRESG = 2,
    SCAL_DMPRESG3 = 3,
    SCAL_DIVMAX = 4,
    SCAL_CFL = 5,
    SCAL_FLOW1 = 6,
    SCAL_FLOW3 = 7,
    SCAL_WSM = 8,      // 3 values
    SCAL_NONFIN = 11,
    SCAL_WSMC = 12,    // 3 values: /WSMEM/ WSM as the SGS model and the wall model see it
    SCAL_WALLERR = 15, // 1 when a wall point's Newton iteration hit its cap in the last step
    SCAL_PIPEERR = 16, // 1 when a bulk-copy stage wait gave up (sticky)
    SCAL_COUNT = 17
};

// the shifted-point wall models' scratch: per wall U_ave, UTAU2, TAUW1, CC, DELTS, nfix
// (WS_NPAR slots) and WS_TABN heights YP (the grid check bounds their drift)
constexpr int WS_NPAR = 8;
constexpr int WS_TABN = 4096;

// Launch schedule of one channel, chosen by c3d_autotune per grid shape.
//   zl   z-line segment length of each z pass (zA, zB, zC, zD, zE): each thread runs the
//        recurrences sequentially over zl points (plus the warm-up), the N3M/zl segments
//        of a line run in parallel; this is the split between the sequential (Thomas)
//        and the parallel part of the z solves
//   xw   rows (warps) per block of the x passes
//   twz  kx columns per block of the z FFT
//   fxp, fzp  radix order of the x and z FFT plans (0: radix 4 first, 1: radix 3 first,
//        2: radix 2 only before 3)
//   zsplit  zA fused or split into its three sweeps
//   xsplit  xA fused or split into its u, v and w pieces
struct Tune {
    int zl[5], xw, twz, fxp, fzp;
    int zsplit;   // zA as one kernel (0) or as its three sweeps in three kernels (1)
    int xsplit;   // xA as one kernel (0) or as its u, v, w pieces in three kernels (1)
    int xbulk;    // x passes with rows staged by a bulk-copy ring of this many stages (0: off)
    int xstage;   // xA's pieces read their rows from global memory (0) or stage them in shared memory by bulk copies (1)
    int ycn;      // wall-normal CN factor: one thread per column (0) or shared-memory tiles of 32 or 64 columns
    int xlanes;   // x passes (xA pieces from global memory, xB, xC/xD with the shared-memory FFT) with a row per segment of this many lanes (0: a warp)
    int conc;     // xA's pieces, then zA's pieces, on three streams at once (1) or one after another (0)
};

// Arguments of the pressure refinement (mixed form with C3D_MIXED_IR): double-float
// constants of RHSDP's operators and the scratch for the z part of the residual.
struct RefArgs {
    dfl f24x, f24z, rdt;       // 24 DX1, 24 DX3, 1/DT
    Cyc<dfl> c22x, c22z;       // (1,22,1) solves
    const dfl *rdy;            // 1/DY(J)
    float *rzh, *rzl;          // Dz(w) as double-float pairs
    int updp;                  // add DP2 to P (GETUP) or not (projection)
};

// Arguments of the LES kernels (FILES != 0): fields in the working precision R, plane
// layout like the state; face quantities are stored at the index of their Fortran owner.
template <typename R>
struct LesArgs {
    R *nu;            // SGSVIS at the cell centres (wall planes j = 0, N2 stay zero)
    R *nux, *nuz;     // nu interpolated to the x faces / z faces (1,6,1)
    R *t13;           // tau13 = Ix(Iz(nu)) (du/dz + dw/dx) at (x face, z face)
    R *nuwz;          // nu * Dz(w) at the cell centres
    R *dvdx, *dvdz;   // Dx(v), Dz(v) at the v faces (J >= 2; J = 1, N2 stay zero)
    R *dwdx;          // Dx(w) at (x face, z face)
    R *dyn;           // SGSDY: 21 raw fields of N2M planes
    double *smagc;    // SMAGC(J), n2+1
    R *coef;          // SMAGC(J) * DXYZ^(2/3) in R (SGSCS)
    const double *d23;   // DXYZ^(2/3) per J
    const R *d23r;       // the same in R
    const double *ycs;   // Y(J) + DY(J)/2 per J
    double *tauw, *taub; // wall stresses [w][k][i], w = 0 bottom, 1 top
    double *wpart;       // wall-model per-block partial sums
    int files, wmodel, wall_cap;
    double ifwall;
    R reninv, dx1, dx3;
};

}  // namespace c3d

struct c3d_channel {
    c3d::Geo g;
    int precision;
    int device;
    cudaStream_t stream;
    cudaEvent_t ev0, ev1;
    // overlapped host transfers of c3d_getup: a side stream and the events the step waits
    // for before xB (HH of the previous step uploaded) and records after it (new HH final)
    cudaStream_t side = nullptr;
    cudaEvent_t hh_in = nullptr, hh_out = nullptr;
    bool hh_hooks = false;
    // concurrent pieces (schedule knob 15): two more streams for the u and v pieces of xA
    // and zA, a fork event and their two join events
    cudaStream_t par[2] = {nullptr, nullptr};
    cudaEvent_t pev[3] = {nullptr, nullptr, nullptr};
    double *xfer = nullptr;   // DMA staging area of pinned host arrays (one slot per field)
    double *wtaue = nullptr;  // WALLMODEL_WERNER: TAUWE(I,K,1..4) at the cell centres (4 x N1M N3M)
    // MARUSIC1 / PIOMELLI: Y(0:N2), YC(0:N2), per-wall constants and YP heights; the
    // reference plane ZS of MARUSIC1 (the Y(J) nearest 0.06) and tan(16 deg)
    double *wshift = nullptr;
    // SGSSD: per-plane partial sums of k_sgs_sd_sums (N2M x sdnt x 10) and BETA(0:N2)
    double *specbuf = nullptr;   // c3d_plane_spectra: means and the five output tables
    // WALLMODEL_IWMLES_SMOOTH: per-point state, whether it is set, the accumulated model
    // step, DY(1) + DY(2) + DY(3)/2, the driver's CFLMAX and the NTIME of the step
    double *iwm = nullptr;
    int iwm_ready = 0;
    double iwm_dt = 0.0, iwm_dzp = 0.0, cflmax = 1.0, iwm_y0 = 0.0;
    int ntime = 1;
    double *sdpart = nullptr, *sdbeta = nullptr;
    int sdnt = 0;
    // SGSSD's per-plane root solve and nu run beside BCOND and the RHS passes, which do
    // not read nu: forked after the sums, joined before the SGS fluxes
    cudaStream_t sside = nullptr;
    cudaEvent_t sfork = nullptr, sjoin = nullptr;
    int sjoin_pending = 0;
    // the wall model runs on its own stream beside the SGS model and the RHS passes: forked
    // after the last reader of WSM, joined before the first reader of TAUW/TAUB
    cudaStream_t wside = nullptr;
    cudaEvent_t wfork = nullptr, wjoin = nullptr;
    int wjoin_pending = 0;
    int wzs = 0;
    int wrough = 0;            // WALLMODEL_ROUGH (WMODEL 1 with Y0 != 0) and its KAPA / log(DELTAP / Y0)
    double wklog = 0.0;
    int y_increasing = 0;      // Y(1:N2) increases (the particle and shifted-model searches)
    double wtan16 = 0.0;
    double *stats = nullptr;  // plane statistics table and partial sums (allocated on first use)
    cudaStream_t cs = nullptr;          // copy stream of the DMA transfers
    cudaEvent_t xev[16] = {};           // per-field hand-offs between the copy and compute streams
    // state (double or float2 by precision), scalars and metrics
    void *u, *v, *w, *p, *dp;
    double *scal, *part;
    double *metric;           // 10 arrays of n2+1: dy,h,hp,hc,hm,dyp,dyc,dym,hz,dyz
    void *metr;               // NMETR arrays of n2+1 in the working precision (MetR)
    double *ycn;              // 3 x 3 x (n2+1)
    float *ycn32;             // the same in FP32 (mixed form)
    double *prb, *pgam, *pmj;
    float2 *prbdf, *pgamdf, *pmjdf, *bulkw;
    double *diagbuf;          // FP64 scratch field of the diagnostics
    double2 *tw64;            // x-FFT table, z-FFT table, x post-processing table
    float2 *tw32;
    // working arrays (R = double or float), stored untyped
    void *hh[2][3];
    int cur;                  // index of the current HH set
    void *r[3];
    void *exy, *exz, *eyz, *ww1, *wsq, *rdpz, *g1;
    void *spec;
    double *stage;            // device staging for Fortran-layout transfers
    size_t stage_elems;
    double *pinned;           // pinned host bounce buffer for the host-array path
    size_t pinned_elems;
    double dt_cached;
    int have_state;
    float last_ms;
    int last_launches;
    int nsm;                  // streaming multiprocessors of the device
    c3d::FftPlan fx, fz;
    std::vector<double> ak1, ak3, pcj, ppj, pmjh;
    // LES (FILES != 0): SGS model, wall model and SGS-flux work fields
    int files, wmodel;
    double *tauw, *taub;      // (N1M*N3M*2) device, plane layout [w][k][i]
    void *les[8];             // nu, nux, nuz, t13, nuwz, dvdx, dwdx, dvdz (R, full fields)
    void *dyn;                // SGSDY raw quantities (21 x N2M planes, R)
    double *smagc, *d23, *ycs, *wpart;
    void *coef, *d23r;        // per-J tables in R
    int wall_cap;
    void *opbuf[2];           // operand and result of c3d_op_* (R, full fields)
    int refine;               // mixed form: one refinement step of the pressure solve
    c3d::Tune tune;           // launch schedule (c3d_autotune)
    c3d_grid grid_copy;       // the creation grid with copies of its metric arrays,
    std::vector<double> grid_arrays;   // used to build scratch channels for tuning
    c3d::dfl *rdydf;          // 1/DY(J) as double-float pairs (refinement)
    // per-kernel profiler (CUDA events around every launch when enabled)
    int prof_on;
    int prof_n;                              // events recorded in the current step
    std::vector<cudaEvent_t> prof_ev;        // event pool
    std::vector<int> prof_iv;                // kernel index of interval i
    std::vector<std::string> prof_name;
    std::vector<double> prof_ms, prof_bytes;
    std::vector<int> prof_cnt;
    cudaEvent_t tm0, tm1;                    // c3d_timer_start/stop
};

namespace c3d {
// Kernel launchers of the passes (c3d_xpass.cu, c3d_zpass.cu, c3d_spec.cu).
// which: x passes 0=xA 1=xB 2=xC 3=xD 4=diag; z passes 0=zA 1=zB 2=zC 3=zD 4=zE 5=diag.
template <typename R>
int launch_xpass(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl);
template <typename R>
int launch_zpass(c3d_channel *ch, StepArgs<R> &a, int which, R *d0, R *d1, R *d2, int flag, int *nl);
template <typename R>
int launch_spec(c3d_channel *ch, StepArgs<R> &a, int which, int *nl);   // 0=fwd z FFT 1=poisson 2=inv z FFT
template <typename R>
void set_spec_smem(c3d_channel *ch);
// LES stages (c3d_les.cu): 0 = WALLSS/SGS model/wall model before BCOND, 1 = SGS fluxes.
template <typename R>
int launch_les(c3d_channel *ch, StepArgs<R> &a, LesArgs<R> &l, int stage, int *nl);
// Step drivers (c3d_step.cu)
int launch_step(c3d_channel *ch, double dt, int *launches);
int launch_operator(c3d_channel *ch, int op, int *launches);
template <typename R>
int launch_op(c3d_channel *ch, StepArgs<R> &a, int op, const R *in, R *out, int *nl);   // c3d_ops.cu
int launch_refine(c3d_channel *ch, StepArgs<float> &a, RefArgs &r, int *nl);            // c3d_refine.cu
int launch_project(c3d_channel *ch, int *launches);
int launch_diag(c3d_channel *ch, int *launches);
int launch_pipe_selftest(c3d_channel *ch, double limit_ms);
// Batch form of the DNS step (FILES = 0; precision C3D_FP64 or C3D_MIXED): the passes of
// one channel's step in order (batch_plan), and its StepArgs<R> for the step with DT dt
// written as bytes to dst (batch_args, batch_args_size bytes).
template <typename R> int xpass_bkern(const c3d_channel *ch, int which, int xw, std::vector<BKern> &out);
// Lanes per row segment of the x passes for a channel of N1M x N3M (0: one row per warp).
int x_segment_lanes(int n1m, int n3m);
template <typename R> int zpass_bkern(const c3d_channel *ch, int which, int seg, std::vector<BKern> &out);
template <typename R> int spec_bkern(const c3d_channel *ch, int which, std::vector<BKern> &out);
// Schedule of the work-list form: segment length of the z passes zA..zE and warps per
// block of the x passes.
struct BatchSched {
    int zseg[5];
    int xw;
    int conc;   // the pieces of xA and of zA as concurrent branches of each group (1) or not (0)
};
int batch_plan(c3d_channel *ch, const BatchSched &s, std::vector<BKern> &out);
size_t batch_args_size(const c3d_channel *ch);
void batch_args(c3d_channel *ch, double dt, void *dst);
int launch_poisson_tables(c3d_channel *ch);
// what: 0 U component, 1 P, 2 HH component, 3 SGSVIS (to host), 4 operand (to device),
// 5 operator result (to host)
// ENERGY's plane statistics of the current state into out (N2M x 29, device), with
// `part` as scratch (stats_scratch_doubles(g) doubles hold both)
int launch_stats(c3d_channel *ch, double *out, double *part);
size_t stats_scratch_doubles(const c3d::Geo &g);
// Checkpoint records (CWRITE's order) between the device state and buf; dir 0 packs,
// what 0 U, 1 P, 2 HH (three components)
int launch_ckpt(c3d_channel *ch, int dir, int what, double *buf);
// fort: the Fortran-layout array on the device (the one-field staging buffer by default)
int launch_repack(c3d_channel *ch, int dir, int what, int comp, double *fort = nullptr);  // dir 0: Fortran->device
void set_error(const std::string &msg);
// Records a kernel-boundary mark for the profiler and counts the launch.
void mark(c3d_channel *ch, int *nl, const char *name, double bytes);
// The three pieces of xA or zA as concurrent branches: par_fork makes the two extra streams
// wait for the work so far on the channel's stream, par_join makes the channel's stream
// wait for both.  par_on says whether the pieces run concurrently (knob 15, not while the
// per-kernel profile is on, whose events are recorded on the channel's stream).
bool par_on(const c3d_channel *ch);
int par_fork(c3d_channel *ch);
int par_join(c3d_channel *ch);
// returns C3D_ECUDA with the failing call named when a CUDA runtime call fails
#define CK_RC(call)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));             \
            return C3D_ECUDA;                                                           \
        }                                                                               \
    } while (0)
// the shifted-point wall models' scratch: its size in doubles and the mesh tables
size_t wall_shift_doubles(const Geo &g);
// WALLMODEL_IWMLES_SMOOTH: the state's size in doubles and one step of the model on st
size_t iwm_doubles(const Geo &g);
template <typename R>
int launch_iwm_t(c3d_channel *ch, StepArgs<R> &a, cudaStream_t st, double *tauw, double *taub);
// ENERGY's spectra and correlations (vmo: 3 N2M means; st: the plane statistics table)
int launch_spectra(c3d_channel *ch, const double *vmo, const double *st, double *xs, double *zs, double *rxx,
                   double *rzz, double *rxy);
// ENERGY's quadrant sums into out (8 N2M), part: 8 SB N2M partial sums
int launch_quadrants(c3d_channel *ch, const double *vmp, double *out, double *part);
// ENERGY's 3-D correlation into out (3 N1M N2M N3M) and the wall-stress spectrum
// (c1: (N1M/2 + 1) N3M complex scratch, out: N1M N3M)
int launch_corr3d(c3d_channel *ch, const double *st, double *out);
int launch_wall_spectrum(c3d_channel *ch, double utau, double2 *c1, double *out);
// the particle step (r1 == nullptr) or SOURCE_PAR's terms into r1..r3 for n particles
int launch_particles(c3d_channel *ch, double *par, int n, double diam, double dens, double hhh, double dt, int *impact,
                     double *r1, double *r2, double *r3);
void launch_wall_shift_init(c3d_channel *ch);
void prof_begin(c3d_channel *ch);
int prof_collect(c3d_channel *ch);
}  // namespace c3d
