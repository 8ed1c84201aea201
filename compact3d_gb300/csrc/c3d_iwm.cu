// c3d_iwm.cu -- WALLMODEL_IWMLES_SMOOTH (WMODEL 2 with Y0 = 0, compact3d.f:3386-4279) and
// WALLMODEL_IWMLES_ROUGH (Y0 != 0, 2562-3381), the integral wall model of Yang et al. 2015
// on the bottom wall, FP64.  The rough variant shares the state, schedule, filter and
// left-hand side and replaces the Newton solve and the profile (k_iwm_rough).
//
// Per wall point a state of IW_NS values (the reference's /IWMLES/ arrays, slot-major in
// ch->iwm) persists across steps.  It is initialised at NTIME = 1, or at the channel's
// first step with this model (where the reference would read a zeroed COMMON); every
// fifth step (NTIME mod 5 = 0) the time-filtered velocity and pressure, the integrated
// momentum balance and the Newton solve for (u_tau,x, u_tau,y) are updated with the step
// accumulated since (WM_DT, tracked on the host); every step the stresses are imposed and
// WSM(1) is their plane mean.  Kernels, in order:
//   iwm_sum / iwm_fin   plane sums in a fixed order: u at J = 3 (init), P at J = 1 (mean
//                       pressure), |tau| (WSM(1)); the init also runs the log-law Newton
//   iwm_init            iwm_init_smooth per point (3561-3714)
//   iwm_filter          the temporal filter of u, w and p - <p> (3761-3811)
//   iwm_lhs             convective, pressure-gradient and left-hand-side terms (3814-3875)
//   iwm_newton          the Newton solve with the finite-difference Jacobian and the
//                       equilibrium fallback (3960-4105)
//   iwm_stale           the reference's equilutx/equiluty are locals of the point loop
//                       that only the fallback sets; a point whose linear correction
//                       |A| > 1 takes the values of the last point (I outer, K inner) with
//                       a fallback (zero before the first): a scan in that order
//   iwm_finish          linear corrections, integrals, derivatives, diffusion, stresses
//                       and the filter time scale (4106-4276)
//   iwm_apply           TAUW(I,K,1) = tauwx and TAUW(I,K,3) = tauwy, which the reference
//                       writes beyond TAUW's extent onto TAUB(I,K,1) of /TAUXYZ/: stored
//                       there; per-block sums of sqrt(tauwx^2 + tauwy^2)
// The Newton steps difference the residual over 1e-9 in u_tau, so one rounding of the
// residual moves the Jacobian by about 1e-7 relative: the iterates follow the reference's
// operation order (std::min/max semantics with NaN included) but are not bit-exact.
#include "c3d_kern.cuh"

namespace c3d {

enum {
    IW_UTX, IW_UTY, IW_TAUWX, IW_TAUWY, IW_FTX, IW_FTY, IW_FTMX, IW_FTMY, IW_FP, IW_INTE, IW_INTEM = IW_INTE + 5,
    IW_DIFFX = IW_INTEM + 5, IW_DIFFY, IW_LHSX, IW_LHSY, IW_FUS, IW_TR, IW_DZ, IW_AX, IW_AY, IW_CX, IW_CY,
    IW_UNSX, IW_UNSY, IW_DELI, IW_DELV, IW_DTX, IW_DTY, IW_DBX, IW_DBY, IW_CONVX, IW_CONVY, IW_PRSX, IW_PRSY,
    IW_Z0, IW_NS,
    // device-only: the Newton result before the |A| > 1 reset, the fallback values and flags
    IW_PUTX = IW_NS, IW_PUTY, IW_EQX, IW_EQY, IW_EQ0, IW_STALE, IW_SLOTS
};
enum { IW_LU = 0, IW_LUU = 1, IW_LV = 2, IW_LVV = 3, IW_LUV = 4 };
// scalars after the slots: uinit, usinit, mean P at J = 1
constexpr int IW_SC_UINIT = 0, IW_SC_USINIT = 1, IW_SC_PBAR = 2, IW_NSC = 4;

size_t iwm_doubles(const Geo &g) { return (size_t)IW_SLOTS * g.np + IW_NSC; }

__device__ __forceinline__ double smin(double a, double b) { return b < a ? b : a; }   // std::min
__device__ __forceinline__ double smax(double a, double b) { return a < b ? b : a; }   // std::max
__device__ __forceinline__ double sq(double x) { return x * x; }

// the log-law Newton for u_tau (KAPA 0.4, B 5; compact3d.f:3589-3604, 4079-4091)
__device__ double iwm_loglaw(double U_ave, double DZP, double RE) {
    const double KAPA = 0.4, B = 5.0;
    double U_tau1 = 1.0, U_tau2 = 0.000001, LAMBDA = 1.0;
    for (int it = 0; it < 100000 && fabs(U_tau2 - U_tau1) > 1.0E-6; it++) {
        U_tau1 = U_tau2;
        const double FUtau1 = U_ave / U_tau1 - log(U_tau1 * DZP * RE) / KAPA - B;
        const double FUtau2 = -U_ave / sq(U_tau1) - 1. / KAPA / U_tau1;
        U_tau2 = U_tau1 - LAMBDA * FUtau1 / FUtau2;
        const double FUtau3 = U_ave / U_tau2 - log(U_tau2 * DZP * RE) / KAPA - B;
        if (fabs(FUtau3) > fabs(FUtau1)) LAMBDA = 0.5 * LAMBDA;
    }
    return U_tau1;
}

// iwm_slv_smooth (compact3d.f:3881-3926): the integrated momentum residuals
__device__ void iwm_slv(double lhsx, double lhsy, double Ux, double Uy, double Dz, double utx, double uty,
                        double reinv, double &fx, double &fy) {
    const double vonk = 0.4;
    const double us = pow(pow(utx, 4.0) + pow(uty, 4.0), 0.25);
    const double delv = reinv / us;
    const double deli = smin(11.0 * reinv / us, Dz);
    const double Vel = sqrt(sq(Ux) + sq(Uy));
    const double lg = log(deli / Dz);
    const double Ax = (Ux / us + Ux / Vel / vonk * lg - deli / delv * utx / us) / (1.0 - deli / Dz);
    const double Ay = (Uy / us + Uy / Vel / vonk * lg - deli / delv * uty / us) / (1.0 - deli / Dz);
    const double Cx = Ux / us - Ax, Cy = Uy / us - Ay;
    const double r1 = deli / Dz, r2 = sq(deli) / sq(Dz);
    fx = 0.5 * utx * sq(deli) / delv + us * Dz * (0.5 * Ax * (1.0 - r2) + Cx * (1.0 - r1) -
                                                  1.0 / vonk * Ux / Vel * (1.0 - r1 + r1 * lg)) + lhsx;
    fy = 0.5 * uty * sq(deli) / delv + us * Dz * (0.5 * Ay * (1.0 - r2) + Cy * (1.0 - r1) -
                                                  1.0 / vonk * Uy / Vel * (1.0 - r1 + r1 * lg)) + lhsy;
}

struct IwmArgs {
    double *st;        // IW_SLOTS x np, then IW_NSC scalars
    double *part;      // per-block partial sums
    double *tauw, *taub;
    double *scal;
    Geo g;
    double dzp, cflmax, wm_dt;
    int rough;         // WALLMODEL_IWMLES_ROUGH: Y0 = Y(0) != 0 is the roughness length
    double y0;
};

__device__ __forceinline__ double &S(const IwmArgs &w, int q, int e) { return w.st[(size_t)q * w.g.np + e]; }

// plane sums of one quantity, per block: mode 0 u(I,3,K), 1 P(I,1,K), 2 |tau| from the state
template <typename R>
__global__ void __launch_bounds__(TPB) k_iwm_sum(StepArgs<R> a, IwmArgs w, int mode) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double sh[TPB];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (e < g.np) {
        const int i = e % g.n1m, k = e / g.n1m;
        if (mode == 0) v = ST::dbl(a.u[fidx(g, i, 3, k)]);
        else if (mode == 1) v = ST::dbl(a.p[fidx(g, i, 1, k)]);
        else v = sqrt(sq(S(w, IW_TAUWX, e)) + sq(S(w, IW_TAUWY, e)));
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) w.part[blockIdx.x] = sh[0];
}

// the sums in order; mode 0: uinit and usinit, 1: the mean pressure, 2: WSM(1)
__global__ void k_iwm_fin(IwmArgs w, int nb, int mode) {
    __shared__ double sh[256];
    double x = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) x += w.part[q];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    double *sc = w.st + (size_t)IW_SLOTS * w.g.np;
    const double n = (double)(w.g.n1m * w.g.n3m);
    if (mode == 0) {
        sc[IW_SC_UINIT] = sh[0] / n;
        sc[IW_SC_USINIT] = w.rough ? sc[IW_SC_UINIT] * 0.4 / log(w.dzp / w.y0) : iwm_loglaw(sc[IW_SC_UINIT], w.dzp, w.g.re);
    } else if (mode == 1) {
        sc[IW_SC_PBAR] = sh[0] / (double)w.g.n1m / (double)w.g.n3m;
    } else {
        w.scal[SCAL_WSMC] = sh[0] / n;
    }
}

__global__ void __launch_bounds__(TPB) k_iwm_init(IwmArgs w) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= w.g.np) return;
    const double *sc = w.st + (size_t)IW_SLOTS * w.g.np;
    const double uinit = sc[IW_SC_UINIT], usinit = sc[IW_SC_USINIT], Dzp = w.dzp, vonk = 0.4, reinv = 1.0 / w.g.re;
    for (int q = 0; q < IW_SLOTS; ++q) S(w, q, e) = 0.0;
    S(w, IW_UTX, e) = usinit;
    S(w, IW_TAUWX, e) = sq(usinit);
    S(w, IW_FTX, e) = uinit;
    S(w, IW_FTMX, e) = uinit;
    S(w, IW_INTE + IW_LU, e) = uinit * Dzp;
    S(w, IW_INTE + IW_LUU, e) = sq(uinit) * Dzp;
    S(w, IW_INTEM + IW_LU, e) = uinit * Dzp;
    S(w, IW_INTEM + IW_LUU, e) = sq(uinit) * Dzp;
    S(w, IW_LHSX, e) = -uinit * Dzp;
    S(w, IW_LHSY, e) = -uinit * Dzp;
    S(w, IW_DTX, e) = usinit / vonk / Dzp;
    S(w, IW_FUS, e) = usinit;
    S(w, IW_TR, e) = (w.cflmax * w.g.alx / w.g.n1m / uinit) / (Dzp / vonk / usinit);
    S(w, IW_DZ, e) = Dzp;
    if (w.rough) {   // iwm_init_rough (compact3d.f:2736-2857)
        S(w, IW_DBX, e) = usinit / vonk / w.y0;
        S(w, IW_Z0, e) = w.y0;
    } else {
        S(w, IW_DELI, e) = smin(11.0 * reinv / usinit, Dzp);
        S(w, IW_DELV, e) = reinv / usinit;
    }
}

// iwm_slv_rough (compact3d.f:3031-3052)
__device__ void iwm_slv_rough(double lhsx, double lhsy, double Ux, double Uy, double Dz, double z0, double utx,
                              double uty, double &fx, double &fy) {
    const double vonk = 0.4, lg = log(Dz / z0);
    const double Ax = (Ux - utx / vonk * lg) / ((1.0 - z0 / Dz));
    const double Ay = (Uy - uty / vonk * lg) / ((1.0 - z0 / Dz));
    fx = 1.0 / 2.0 * Dz * Ax * sq(1.0 - z0 / Dz) + 1.0 / vonk * utx * Dz * (z0 / Dz - 1.0 + lg) + lhsx;
    fy = 1.0 / 2.0 * Dz * Ay * sq(1.0 - z0 / Dz) + 1.0 / vonk * uty * Dz * (z0 / Dz - 1.0 + lg) + lhsy;
}

// iwm_calc_wallstress_rough (compact3d.f:3055-3334) per point: the Newton solve with the
// diagonal finite-difference Jacobian, the equilibrium fallback vonk U / log(Dz / z0),
// the rough-wall integrals, derivatives, diffusion and stresses.  Kept as written: the Lvv
// integral has -3 z0^2/Dz^2 where Luu has +3, and tauwy is (vonk * iwmpz0)^2 ... with
// iwmpz0 an undeclared, zero-valued name.
__global__ void __launch_bounds__(TPB) k_iwm_rough(IwmArgs w) {
    const Geo g = w.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const double vonk = 0.4, wm_tol = 0.000001, wm_eps = 0.000000001, wm_dt = w.wm_dt;
    const double lhsx = S(w, IW_LHSX, e), lhsy = S(w, IW_LHSY, e);
    const double Ux = S(w, IW_FTX, e), Uy = S(w, IW_FTY, e), Dz = S(w, IW_DZ, e), z0 = S(w, IW_Z0, e);
    double utx = S(w, IW_UTX, e), uty = S(w, IW_UTY, e), fx, fy, fxp, fyp;
    iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty, fx, fy);
    int iter = 0, eq = 0;
    while (smax(fabs(fx), fabs(fy)) > wm_tol) {
        iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx + wm_eps, uty, fxp, fyp);
        const double a11 = (fxp - fx) / wm_eps, a21 = 0.0;
        iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty + wm_eps, fxp, fyp);
        const double a12 = 0.0, a22 = (fyp - fy) / wm_eps;
        const double det = __dsub_rn(__dmul_rn(a11, a22), __dmul_rn(a12, a21));
        const double nx = utx - __dsub_rn(__dmul_rn(a22, fx), __dmul_rn(a12, fy)) / det;
        const double ny = uty - __dadd_rn(__dmul_rn(-a21, fx), __dmul_rn(a11, fy)) / det;
        utx = nx;
        uty = ny;
        iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty, fx, fy);
        iter = iter + 1;
        if (iter > 1500) {
            eq = 1;
            break;
        }
    }
    if (utx - 1.0 == utx || uty - 1.0 == uty) eq = 1;
    const double lg = log(Dz / z0);
    if (eq) {
        utx = vonk * Ux / lg;
        uty = vonk * Uy / lg;
    }
    double Ax = 0.0, Ay = 0.0;
    if (!eq) {
        Ax = (Ux - utx / vonk * lg) / ((1.0 - z0 / Dz));
        Ay = (Uy - uty / vonk * lg) / ((1.0 - z0 / Dz));
    }
    S(w, IW_UTX, e) = utx;
    S(w, IW_UTY, e) = uty;
    S(w, IW_AX, e) = Ax;
    S(w, IW_AY, e) = Ay;
    for (int q = 0; q < 5; ++q) S(w, IW_INTEM + q, e) = S(w, IW_INTE + q, e);
    const double px = utx, py = uty, r = z0 / Dz;
    const double P4 = 1.0 - 4.0 * r + 3.0 * sq(z0) / sq(Dz) - 2.0 * lg + 4.0 * r * lg;
    const double M4 = 1.0 - 4.0 * r - 3.0 * sq(z0) / sq(Dz) - 2.0 * lg + 4.0 * r * lg;
    const double c3 = (1.0 - r) * (1.0 - r) * (1.0 - r);
    S(w, IW_INTE + IW_LU, e) = 1.0 / 2.0 * Dz * Ax * sq(1.0 - r) + 1.0 / vonk * px * Dz * (r - 1.0 + lg);
    S(w, IW_INTE + IW_LV, e) = 1.0 / 2.0 * Dz * Ay * sq(1.0 - r) + 1.0 / vonk * py * Dz * (r - 1.0 + lg);
    S(w, IW_INTE + IW_LUV, e) = 1.0 / sq(vonk) * px * py * Dz * (1.0 - 2 * r + sq(1.0 - lg)) +
                                1.0 / 3.0 * Ax * Ay * Dz * c3 - 1.0 / 4.0 / vonk * (Ax * py + Ay * px) * Dz * P4;
    S(w, IW_INTE + IW_LUU, e) = 1.0 / sq(vonk) * sq(px) * Dz * (sq(lg - 1.0) - 2.0 * r + 1.0) +
                                1.0 / 3.0 * sq(Ax) * Dz * c3 - 1.0 / 2.0 / vonk * px * Ax * Dz * P4;
    S(w, IW_INTE + IW_LVV, e) = 1.0 / sq(vonk) * sq(py) * Dz * (sq(lg - 1.0) - 2.0 * r + 1.0) +
                                1.0 / 3.0 * sq(Ay) * Dz * c3 - 1.0 / 2.0 / vonk * py * Ay * Dz * M4;
    const double dTx = 1.0 / Dz * (Ax + px / vonk), dTy = 1.0 / Dz * (Ay + py / vonk);
    const double dBx = 1.0 / Dz * Ax + px / vonk / z0, dBy = 1.0 / Dz * Ay + py / vonk / z0;
    S(w, IW_DTX, e) = dTx;
    S(w, IW_DTY, e) = dTy;
    S(w, IW_DBX, e) = dBx;
    S(w, IW_DBY, e) = dBy;
    const double Vel = sqrt(sq(Ux) + sq(Uy));
    const double dVelzT = fabs(Ux / Vel * dTx + Uy / Vel * dTy), dVelzB = sqrt(sq(dBx) + sq(dBy));
    S(w, IW_DIFFX, e) = sq(vonk * Dz) * dVelzT * dTx - sq(vonk * z0) * dVelzB * dBx;
    S(w, IW_DIFFY, e) = sq(vonk * Dz) * dVelzT * dTy - sq(vonk * z0) * dVelzB * dBy;
    double tx, ty;
    if (eq) {
        const double para = sqrt(sq(Ux) + sq(Uy)) * sq(vonk) / sq(lg);
        tx = para * Ux;
        ty = para * Uy;
    } else {
        const double iwmpz0 = 0.0;
        tx = sq(vonk * z0) * dVelzB * dBx;
        ty = sq(vonk * iwmpz0) * dVelzB * dBy;
    }
    S(w, IW_TAUWX, e) = tx;
    S(w, IW_TAUWY, e) = ty;
    const double utaup = pow(sq(tx) + sq(ty), 0.25);
    const double tR = S(w, IW_TR, e);
    const double fus = __dadd_rn(__dmul_rn(S(w, IW_FUS, e), 1.0 - tR), __dmul_rn(utaup, tR));
    S(w, IW_FUS, e) = fus;
    double ntR = wm_dt / (Dz / fus / vonk);
    if (ntR > 1.0) ntR = 1.0;
    S(w, IW_TR, e) = ntR;
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_iwm_filter(StepArgs<R> a, IwmArgs w) {
    typedef St<R> ST;
    const Geo g = a.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const int i = e % g.n1m, k = e / g.n1m;
    const double pbar = w.st[(size_t)IW_SLOTS * g.np + IW_SC_PBAR];
    S(w, IW_FTMX, e) = S(w, IW_FTX, e);
    S(w, IW_FTMY, e) = S(w, IW_FTY, e);
    const double u_inst = ST::dbl(a.u[fidx(g, i, 3, k)]), v_inst = ST::dbl(a.w[fidx(g, i, 3, k)]);
    const double p_inst = ST::dbl(a.p[fidx(g, i, 1, k)]) - pbar, tR = S(w, IW_TR, e);
    S(w, IW_FTX, e) = __dadd_rn(__dmul_rn(S(w, IW_FTX, e), 1.0 - tR), __dmul_rn(u_inst, tR));
    S(w, IW_FTY, e) = __dadd_rn(__dmul_rn(S(w, IW_FTY, e), 1.0 - tR), __dmul_rn(v_inst, tR));
    S(w, IW_FP, e) = __dadd_rn(__dmul_rn(S(w, IW_FP, e), 1.0 - tR), __dmul_rn(p_inst, tR));
}

__global__ void __launch_bounds__(TPB) k_iwm_lhs(IwmArgs w) {
    const Geo g = w.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const int i = e % g.n1m, k = e / g.n1m;
    const int ep = k * g.n1m + (i + 1 == g.n1m ? 0 : i + 1), em = k * g.n1m + (i == 0 ? g.n1m - 1 : i - 1);
    const int kp = (k + 1 == g.n3m ? 0 : k + 1) * g.n1m + i, km = (k == 0 ? g.n3m - 1 : k - 1) * g.n1m + i;
    const double wm_dt = w.wm_dt, DX1 = g.dx1, DX3 = g.dx3;
    S(w, IW_UNSX, e) = (S(w, IW_INTE + IW_LU, e) - S(w, IW_INTEM + IW_LU, e)) / wm_dt;
    S(w, IW_UNSY, e) = (S(w, IW_INTE + IW_LV, e) - S(w, IW_INTEM + IW_LV, e)) / wm_dt;
    auto dx = [&](int q) { return (S(w, q, ep) - S(w, q, em)) * DX1 / 2.0; };
    auto dz = [&](int q) { return (S(w, q, kp) - S(w, q, km)) * DX3 / 2.0; };
    const double uux = dx(IW_INTE + IW_LUU), uvy = dz(IW_INTE + IW_LUV), uvx = dx(IW_INTE + IW_LUV);
    const double vvy = dz(IW_INTE + IW_LVV), ux = dx(IW_INTE + IW_LU), vy = dz(IW_INTE + IW_LV);
    const double convx = __dsub_rn(__dadd_rn(uux, uvy), __dmul_rn(S(w, IW_FTMX, e), __dadd_rn(ux, vy)));
    const double convy = __dsub_rn(__dadd_rn(uvx, vvy), __dmul_rn(S(w, IW_FTMY, e), __dadd_rn(ux, vy)));
    const double Dz = S(w, IW_DZ, e);
    const double prsx = __dadd_rn(__dmul_rn(dx(IW_FP), Dz), __dmul_rn(w.scal[SCAL_PRESG], Dz));
    const double prsy = __dadd_rn(__dmul_rn(dz(IW_FP), Dz), __dmul_rn(w.scal[SCAL_PRESG3], Dz));
    S(w, IW_CONVX, e) = convx;
    S(w, IW_CONVY, e) = convy;
    S(w, IW_PRSX, e) = prsx;
    S(w, IW_PRSY, e) = prsy;
    S(w, IW_LHSX, e) = __dadd_rn(-S(w, IW_INTE + IW_LU, e),
                                 __dmul_rn(wm_dt, __dsub_rn(__dadd_rn(convx, prsx), S(w, IW_DIFFX, e))));
    S(w, IW_LHSY, e) = __dadd_rn(-S(w, IW_INTE + IW_LV, e),
                                 __dmul_rn(wm_dt, __dsub_rn(__dadd_rn(convy, prsy), S(w, IW_DIFFY, e))));
}

__global__ void __launch_bounds__(TPB) k_iwm_newton(IwmArgs w) {
    const Geo g = w.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const double reinv = 1.0 / g.re, vonk = 0.4, wm_tol = 0.000001, wm_eps = 0.000000001;
    const double lhsx = S(w, IW_LHSX, e), lhsy = S(w, IW_LHSY, e);
    const double Ux = S(w, IW_FTX, e), Uy = S(w, IW_FTY, e), Dz = S(w, IW_DZ, e);
    double utx = S(w, IW_UTX, e), uty = S(w, IW_UTY, e), fx, fy, fxp, fyp;
    iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, reinv, fx, fy);
    int iter = 0, eq = 0;
    while (smax(fabs(fx), fabs(fy)) > wm_tol) {
        iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx + wm_eps, uty, reinv, fxp, fyp);
        const double a11 = (fxp - fx) / wm_eps, a21 = (fyp - fy) / wm_eps;
        iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty + wm_eps, reinv, fxp, fyp);
        const double a12 = (fxp - fx) / wm_eps, a22 = (fyp - fy) / wm_eps;
        const double det = __dsub_rn(__dmul_rn(a11, a22), __dmul_rn(a12, a21));
        const double nx = utx - __dsub_rn(__dmul_rn(a22, fx), __dmul_rn(a12, fy)) / det;
        const double ny = uty - __dadd_rn(__dmul_rn(-a21, fx), __dmul_rn(a11, fy)) / det;
        utx = nx;
        uty = ny;
        iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, reinv, fx, fy);
        iter = iter + 1;
        if (iter > 1500) {
            eq = 1;
            break;
        }
    }
    if (utx - 1.0 == utx || uty - 1.0 == uty) eq = 1;
    double eqx = 0.0, eqy = 0.0;
    if (eq) {
        const double U_ave = sqrt(sq(Ux) + sq(Uy));
        const double TAUW1 = sq(iwm_loglaw(U_ave, w.dzp, g.re));
        eqx = TAUW1 * Ux / U_ave;
        eqy = TAUW1 * Uy / U_ave;
        utx = sqrt(fabs(eqx));
        uty = sqrt(fabs(eqy));
    }
    // would the linear correction exceed 1 (the reference then takes the fallback values)
    int stale = 0;
    if (!eq) {
        const double utaup = pow(pow(utx, 4.0) + pow(uty, 4.0), 0.25);
        const double delv = reinv / utaup, deli = smin(11.0 * reinv / utaup, Dz);
        const double Vel = sqrt(sq(Ux) + sq(Uy)), lg = log(deli / Dz);
        const double Ax = (Ux / utaup + Ux / Vel / vonk * lg - deli / delv * utx / utaup) / (1.0 - deli / Dz);
        const double Ay = (Uy / utaup + Uy / Vel / vonk * lg - deli / delv * uty / utaup) / (1.0 - deli / Dz);
        stale = (fabs(Ax) > 1.0 || fabs(Ay) > 1.0) ? 1 : 0;
    }
    S(w, IW_PUTX, e) = utx;
    S(w, IW_PUTY, e) = uty;
    S(w, IW_EQX, e) = eqx;
    S(w, IW_EQY, e) = eqy;
    S(w, IW_EQ0, e) = eq;
    S(w, IW_STALE, e) = stale;
}

// one block of 1024 threads: the fallback values of the last earlier point with a fallback,
// in the reference's loop order I outer, K inner (ord = (I-1) N3M + K-1)
__global__ void __launch_bounds__(1024) k_iwm_stale(IwmArgs w) {
    const Geo g = w.g;
    const int np = g.np, t = threadIdx.x, chunk = (np + 1023) / 1024;
    const int o0 = t * chunk, o1 = min(np, o0 + chunk);
    auto pt = [&](int o) { return (o % g.n3m) * g.n1m + o / g.n3m; };
    __shared__ int last[1024];
    int l = -1;
    for (int o = o0; o < o1; ++o)
        if (S(w, IW_EQ0, pt(o)) != 0.0) l = o;
    last[t] = l;
    __syncthreads();
    if (t == 0) {   // carry into each chunk: the last fallback point of the chunks before
        int c = -1;
        for (int q = 0; q < 1024; ++q) {
            const int v = last[q];
            last[q] = c;
            if (v >= 0) c = v;
        }
    }
    __syncthreads();
    int cur = last[t];
    for (int o = o0; o < o1; ++o) {
        const int e = pt(o);
        if (S(w, IW_EQ0, e) != 0.0) cur = o;
        else if (S(w, IW_STALE, e) != 0.0) {
            S(w, IW_EQX, e) = cur >= 0 ? S(w, IW_EQX, pt(cur)) : 0.0;
            S(w, IW_EQY, e) = cur >= 0 ? S(w, IW_EQY, pt(cur)) : 0.0;
        }
    }
}

__global__ void __launch_bounds__(TPB) k_iwm_finish(IwmArgs w) {
    const Geo g = w.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const double reinv = 1.0 / g.re, vonk = 0.4, wm_dt = w.wm_dt;
    const double Ux = S(w, IW_FTX, e), Uy = S(w, IW_FTY, e), Dz = S(w, IW_DZ, e);
    int eq = S(w, IW_EQ0, e) != 0.0;
    const double px = S(w, IW_PUTX, e), py = S(w, IW_PUTY, e), eqx = S(w, IW_EQX, e), eqy = S(w, IW_EQY, e);
    double utx = px, uty = py;
    const double utaup = pow(pow(px, 4.0) + pow(py, 4.0), 0.25);
    const double delv = reinv / utaup, deli = smin(11.0 * reinv / utaup, Dz);
    const double Vel = sqrt(sq(Ux) + sq(Uy)), lg = log(deli / Dz);
    double Ax = 0.0, Ay = 0.0, Cx = 0.0, Cy = 0.0;
    if (!eq) {
        Ax = (Ux / utaup + Ux / Vel / vonk * lg - deli / delv * px / utaup) / (1.0 - deli / Dz);
        Ay = (Uy / utaup + Uy / Vel / vonk * lg - deli / delv * py / utaup) / (1.0 - deli / Dz);
        Cx = Ux / utaup - Ax;
        Cy = Uy / utaup - Ay;
    }
    if (fabs(Ax) > 1.0 || fabs(Ay) > 1.0) {
        eq = 1;
        utx = sqrt(fabs(eqx));
        uty = sqrt(fabs(eqy));
        Ax = Ay = Cx = Cy = 0.0;
    }
    S(w, IW_UTX, e) = utx;
    S(w, IW_UTY, e) = uty;
    S(w, IW_AX, e) = Ax;
    S(w, IW_AY, e) = Ay;
    S(w, IW_CX, e) = Cx;
    S(w, IW_CY, e) = Cy;
    for (int q = 0; q < 5; ++q) S(w, IW_INTEM + q, e) = S(w, IW_INTE + q, e);
    const double r1 = deli / Dz, r2 = sq(deli) / sq(Dz), r3 = deli * deli * deli / (Dz * Dz * Dz);
    auto lu = [&](double pu, double A, double C, double Uc) {
        return 0.5 * pu * sq(deli) / delv +
               utaup * Dz * (0.5 * A * (1.0 - r2) + C * (1.0 - r1) - 1.0 / vonk * Uc / Vel * (1.0 - r1 + r1 * lg));
    };
    auto luu = [&](double pu, double A, double C, double Uc) {
        return 1.0 / 3.0 * sq(pu) * deli * deli * deli / sq(delv) +
               sq(utaup) * Dz *
                   (-A * Uc / Vel / vonk * r2 * lg + A * (C - 1.0 / 2.0 / vonk * Uc / Vel) * (1.0 - r2) +
                    sq(A) / 3.0 * (1.0 - r3) + sq(C - 1.0 / vonk * Uc / Vel) -
                    r1 * sq(C - Uc / Vel / vonk + Uc / Vel / vonk * lg) + 1.0 / sq(vonk) * sq(Uc) / sq(Vel) * (1.0 - r1));
    };
    S(w, IW_INTE + IW_LU, e) = lu(px, Ax, Cx, Ux);
    S(w, IW_INTE + IW_LV, e) = lu(py, Ay, Cy, Uy);
    S(w, IW_INTE + IW_LUV, e) =
        1.0 / 3.0 * px * py * deli * deli * deli / sq(delv) +
        sq(utaup) * Dz *
            (-1.0 / vonk * (Ax * Uy / Vel + Ay * Ux / Vel) * (0.25 - 0.25 * r2 + 0.5 * sq(deli) / Dz * lg) -
             1.0 / vonk * (Cx * Uy / Vel + Cy * Ux / Vel) * (1.0 - r1 + r1 * lg) -
             Ux * Uy / sq(Vel) / sq(vonk) * (r1 - 2.0 + r1 * sq(lg - 1.0)) + 1.0 / 3.0 * Ax * Ay * (1.0 - r3) +
             0.5 * (Ax * Cy + Ay * Cx) * (1.0 - r2) + Cx * Cy * (1.0 - r1));
    S(w, IW_INTE + IW_LUU, e) = luu(px, Ax, Cx, Ux);
    S(w, IW_INTE + IW_LVV, e) = luu(py, Ay, Cy, Uy);
    double dTx, dTy;
    if (deli < Dz) {
        dTx = utaup / Dz * (Ax + 1.0 / vonk * Ux / Vel);
        dTy = utaup / Dz * (Ay + 1.0 / vonk * Uy / Vel);
    } else {
        dTx = px / delv;
        dTy = py / delv;
    }
    const double dBx = px / delv, dBy = py / delv;
    S(w, IW_DTX, e) = dTx;
    S(w, IW_DTY, e) = dTy;
    S(w, IW_DBX, e) = dBx;
    S(w, IW_DBY, e) = dBy;
    const double dVelzT = fabs(Ux / Vel * dTx + Uy / Vel * dTy);
    if (deli < Dz) {
        S(w, IW_DIFFX, e) = (reinv + sq(vonk * Dz) * dVelzT) * dTx - reinv * dBx;
        S(w, IW_DIFFY, e) = (reinv + sq(vonk * Dz) * dVelzT) * dTy - reinv * dBy;
    } else {
        S(w, IW_DIFFX, e) = 0.0;
        S(w, IW_DIFFY, e) = 0.0;
    }
    if (eq) {
        S(w, IW_TAUWX, e) = eqx;
        S(w, IW_TAUWY, e) = eqy;
    } else if (deli < Dz) {
        S(w, IW_TAUWX, e) = sq(px);
        S(w, IW_TAUWY, e) = sq(py);
    } else {
        S(w, IW_TAUWX, e) = reinv * Ux / Dz;
        S(w, IW_TAUWY, e) = reinv * Uy / Dz;
    }
    const double tR = S(w, IW_TR, e);
    const double fus = __dadd_rn(__dmul_rn(S(w, IW_FUS, e), 1.0 - tR), __dmul_rn(utaup, tR));
    S(w, IW_FUS, e) = fus;
    double ntR = wm_dt / (Dz / fus / vonk);
    if (ntR > 1.0) ntR = 1.0;
    S(w, IW_TR, e) = ntR;
}

__global__ void __launch_bounds__(TPB) k_iwm_apply(IwmArgs w) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= w.g.np) return;
    w.tauw[e] = S(w, IW_TAUWX, e);   // bottom wall (index 1)
    w.taub[e] = S(w, IW_TAUWY, e);   // TAUW(I,K,3) of the reference = TAUB(I,K,1)
}

template <typename R>
int launch_iwm_t(c3d_channel *ch, StepArgs<R> &a, cudaStream_t st, double *tauw, double *taub) {
    const Geo &g = ch->g;
    IwmArgs w;
    w.st = ch->iwm;
    w.part = ch->wpart;
    w.tauw = tauw;
    w.taub = taub;
    w.scal = a.scal;
    w.g = g;
    w.dzp = ch->iwm_dzp;
    w.cflmax = ch->cflmax;
    w.rough = ch->iwm_y0 != 0.0;
    w.y0 = ch->iwm_y0;
    const int nb = nblk(g.np);
    const int ntime = ch->ntime;
    if (ntime == 1 || !ch->iwm_ready) {
        k_iwm_sum<R><<<nb, TPB, 0, st>>>(a, w, 0);
        k_iwm_fin<<<1, 256, 0, st>>>(w, nb, 0);
        k_iwm_init<<<nb, TPB, 0, st>>>(w);
        ch->iwm_dt = 5 * ch->dt_cached;
        ch->iwm_ready = 1;
    }
    if (ntime % 5 == 1) ch->iwm_dt = ch->dt_cached;
    else ch->iwm_dt = ch->iwm_dt + ch->dt_cached;
    w.wm_dt = ch->iwm_dt;
    if (ntime % 5 == 0) {
        k_iwm_sum<R><<<nb, TPB, 0, st>>>(a, w, 1);
        k_iwm_fin<<<1, 256, 0, st>>>(w, nb, 1);
        k_iwm_filter<R><<<nb, TPB, 0, st>>>(a, w);
        k_iwm_lhs<<<nb, TPB, 0, st>>>(w);
        if (w.rough) {
            k_iwm_rough<<<nb, TPB, 0, st>>>(w);
        } else {
            k_iwm_newton<<<nb, TPB, 0, st>>>(w);
            k_iwm_stale<<<1, 1024, 0, st>>>(w);
            k_iwm_finish<<<nb, TPB, 0, st>>>(w);
        }
    }
    k_iwm_apply<<<nb, TPB, 0, st>>>(w);
    k_iwm_sum<R><<<nb, TPB, 0, st>>>(a, w, 2);
    k_iwm_fin<<<1, 256, 0, st>>>(w, nb, 2);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

template int launch_iwm_t<double>(c3d_channel *, StepArgs<double> &, cudaStream_t, double *, double *);
template int launch_iwm_t<float>(c3d_channel *, StepArgs<float> &, cudaStream_t, double *, double *);

}  // namespace c3d
