// c3d_les.cu -- wall-modelled LES on the GPU: the SGS models, the wall model and the SGS
// fluxes of the momentum right-hand sides (FILES != 0, compact3d.f:931-937).
//
//   les_wallss  WALLSS (11077-11143) of the current field into /WSMEM/ WSM, which the
//               driver computes right before GETUP when WMODEL = 0 (compact3d.f:125)
//   sgs_coef    SGSCS's plane coefficient SMAGC(J) DXYZ^(2/3) (1413-1488)
//   sgs_cs      SGSCS: nu = max(coef |S|, -1/RE) with |S| from STRAIN (5558-5689)
//   sgs_raw     SGSDY (1250-1400): per point S_ij, |S|, DELTA^2 |S| S_ij, the cell-centre
//               velocities and their products
//   sgs_dyn     SGSDY: FILTER (5190-5228) of those, M_ij, L_ij, the plane sums, SMAGC(J)
//               and nu, one block per plane
//   sgs_sd_*    SGSSD (1502-1948): both test filters, the Germano sums, the quintic's
//               root by CHHQR (11571-11676) and SMAGC; sgs_apply: nu
//   wall        WALLMODEL_INSTANT (2319-2493): damped Newton for u_tau per wall point
//   wall_rough  WALLMODEL_ROUGH (2496-2558): the rough-wall log law
//   wall_werner WALLMODEL_WERNER (4815-4958): the Werner-Wengle power law, both walls
//   wall_shift* MARUSIC1 (4336-4495) and PIOMELLI (4960-5110): plane-mean log law and
//               INDEX_IJK / INTERPOLAT (12602-12807) at shifted points
//   wall_sum    WSM(1) = plane mean of TAUW1; non-converged points -> error flag
//   les_x1/z1/z2/x2   the SGS fluxes of RHS1/2/3 (6436-6770, 6857-6866, 7088-7393,
//               7774-8111) and the wall-stress terms (6765-6770, 8095-8101)
//   par_*       the particle step and SOURCE_PAR (11882-12470, 2029-2075), which share
//               the MESH02 tables and interpolation of the shifted wall models
// (WALLMODEL_IWMLES_SMOOTH / _ROUGH are in c3d_iwm.cu.)
//
// The reference solves each SGS flux separately (36 compact line solves per step).  The
// sums of fluxes that share an edge viscosity are linear in it, so the kernels form the
// edge stresses once and take one derivative of each:
//   tau13 = Ix(Iz(nu)) (du/dz + dw/dx) at (x face, z face): RHS1 -= Dz(tau13), RHS3 -= Dx(tau13)
//   tau12 = <Ix(nu)>_y (du/dy + dv/dx) at (x face, y face):  RHS2 -= Dx(tau12), RHS1 -= d/dy
//   tau23 = <Iz(nu)>_y (dw/dy + dv/dz) at (y face, z face):  RHS2 -= Dz(tau23), RHS3 -= d/dy
// plus the normal stresses 2 Dx(nu Dx u), 2 d/dy(nu dv/dy), 2 Dz(nu Dz w): 15 solves.  The
// results equal the reference's to rounding.  In the mixed form every difference of the
// state is taken cancellation-free, the strain is formed from values relative to the
// point's own velocity and the Leonard stress from values relative to a per-plane
// constant (the dynamic procedure is Galilean invariant), so FP32 keeps its relative
// accuracy; plane sums, the coefficient and the wall model run in FP64.
#include "c3d_kern.cuh"

namespace c3d {

__device__ __forceinline__ int wrapm(int i, int n) { return i == 0 ? n - 1 : i - 1; }
__device__ __forceinline__ int wrapp(int i, int n) { return i + 1 == n ? 0 : i + 1; }

// ---------------------------------------------------------------------------------
// STRAIN at the cell centre (i, j, k): SR = S11, S12, S13, S22, S23, S33.  Velocities are
// taken relative to (u, v, w) at (i, j, k) (differences are exact in exact arithmetic:
// every quantity below is a difference of averages with unit weight sums).
// ---------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void strain_at(const StepArgs<R> &a, const LesArgs<R> &l, int i, int j, int k,
                                          R (&sr)[6]) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    const Geo &g = a.g;
    const int n1 = g.n1m, n3 = g.n3m, N2 = g.n2;
    const int ip = wrapp(i, n1), im = wrapm(i, n1), kp = wrapp(k, n3), km = wrapm(k, n3);
    const int jp = j + 1, jm = j - 1;
    const S cu = a.u[fidx(g, i, j, k)], cv = a.v[fidx(g, i, j, k)], cw = a.w[fidx(g, i, j, k)];
    auto du = [&](int ii, int jj, int kk) { return ST::d(a.u[fidx(g, ii, jj, kk)], cu); };
    auto dv = [&](int ii, int jj, int kk) { return ST::d(a.v[fidx(g, ii, jj, kk)], cv); };
    auto dw = [&](int ii, int jj, int kk) { return ST::d(a.w[fidx(g, ii, jj, kk)], cw); };
    const bool fjum = (j != 1), fjup = (j != g.n2m);
    const R half = (R)0.5, DX1 = l.dx1, DX3 = l.dx3;
    const R rdy = a.m.rdy[j];
    sr[0] = DX1 * du(ip, j, k);                                   // (U(IP)-U(I))
    {
        R UJP = half * (du(i, jp, k) + du(ip, jp, k));
        R UJC = half * (R(0) + du(ip, j, k));
        R UJM = half * (du(i, jm, k) + du(ip, jm, k));
        R U2, U1;
        if (!l.wmodel) {
            U2 = fjup ? a.m.rh[jp] * (a.m.hdy[j] * UJP + a.m.hdy[jp] * UJC) : half * (du(i, N2, k) + du(ip, N2, k));
            U1 = fjum ? a.m.rh[j] * (a.m.hdy[j] * UJM + a.m.hdy[jm] * UJC) : half * (du(i, 0, k) + du(ip, 0, k));
        } else {
            U2 = fjup ? a.m.rh[jp] * (a.m.hdy[j] * UJP + a.m.hdy[jp] * UJC) : UJC;
            U1 = fjum ? a.m.rh[j] * (a.m.hdy[j] * UJM + a.m.hdy[jm] * UJC) : UJC;
        }
        R VIP = half * (dv(ip, j, k) + dv(ip, jp, k));
        R VIC = half * (R(0) + dv(i, jp, k));
        R VIM = half * (dv(im, j, k) + dv(im, jp, k));
        R V2 = half * (VIP + VIC), V1 = half * (VIM + VIC);
        const R fy = (l.wmodel && (!fjum || !fjup)) ? (R)2.0 * rdy : rdy;
        sr[1] = half * (DX1 * (V2 - V1) + fy * (U2 - U1));
    }
    {
        R UKP = half * (du(i, j, kp) + du(ip, j, kp));
        R UKC = half * (R(0) + du(ip, j, k));
        R UKM = half * (du(i, j, km) + du(ip, j, km));
        R U2 = half * (UKP + UKC), U1 = half * (UKM + UKC);
        R WIP = half * (dw(ip, j, k) + dw(ip, j, kp));
        R WIC = half * (R(0) + dw(i, j, kp));
        R WIM = half * (dw(im, j, k) + dw(im, j, kp));
        R W2 = half * (WIP + WIC), W1 = half * (WIM + WIC);
        sr[2] = half * (DX1 * (W2 - W1) + DX3 * (U2 - U1));
    }
    sr[3] = rdy * dv(i, jp, k);                                    // (V(JP)-V(J))/DY
    {
        R WJP = half * (dw(i, jp, k) + dw(i, jp, kp));
        R WJC = half * (R(0) + dw(i, j, kp));
        R WJM = half * (dw(i, jm, k) + dw(i, jm, kp));
        R W2, W1;
        if (!l.wmodel) {
            W2 = fjup ? a.m.rh[jp] * (a.m.hdy[j] * WJP + a.m.hdy[jp] * WJC) : half * (dw(i, N2, k) + dw(i, N2, kp));
            W1 = fjum ? a.m.rh[j] * (a.m.hdy[j] * WJM + a.m.hdy[jm] * WJC) : half * (dw(i, 0, k) + dw(i, 0, kp));
        } else {
            W2 = fjup ? a.m.rh[jp] * (a.m.hdy[j] * WJP + a.m.hdy[jp] * WJC) : WJC;
            W1 = fjum ? a.m.rh[j] * (a.m.hdy[j] * WJM + a.m.hdy[jm] * WJC) : WJC;
        }
        R VKP = half * (dv(i, j, kp) + dv(i, jp, kp));
        R VKC = half * (R(0) + dv(i, jp, k));
        R VKM = half * (dv(i, j, km) + dv(i, jp, km));
        R V2 = half * (VKP + VKC), V1 = half * (VKM + VKC);
        const R fy = (l.wmodel && (!fjum || !fjup)) ? (R)2.0 * rdy : rdy;
        sr[4] = half * (fy * (W2 - W1) + DX3 * (V2 - V1));
    }
    sr[5] = DX3 * dw(i, j, kp);                                    // (W(KP)-W(K))
}

template <typename R>
__device__ __forceinline__ R sumsq6(const R (&s)[6]) {
    return (R)2.0 * s[1] * s[1] + s[0] * s[0] + (R)2.0 * s[2] * s[2] + s[3] * s[3] + (R)2.0 * s[4] * s[4] +
           s[5] * s[5];
}

// WALLSS into WSM (the SGSCS input): one block, FP64, fixed order.
template <typename R>
__global__ void k_les_wallss(StepArgs<R> a) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double sh[3][256];
    double w1 = 0.0, w2 = 0.0, w3 = 0.0;
    const int n1 = g.n1m, n3 = g.n3m, N2 = g.n2, N2M = g.n2m;
    const double rdy1 = 1.0 / (g.dy[1] * 0.5), rdyv = 1.0 / g.dy[1], rdyt = 1.0 / (g.dy[N2M] * 0.5);
    for (int e = threadIdx.x; e < n1 * n3; e += blockDim.x) {
        const int i = e % n1, k = e / n1, ip = wrapp(i, n1), kp = wrapp(k, n3);
        auto U = [&](const typename SType<R>::S *f, int ii, int jj, int kk) { return ST::dbl(f[fidx(g, ii, jj, kk)]); };
        double uhc = 0.5 * (U(a.u, i, 1, k) + U(a.u, ip, 1, k)), uhw = 0.5 * (U(a.u, i, 0, k) + U(a.u, ip, 0, k));
        double vhc = U(a.v, i, 2, k), vhw = U(a.v, i, 1, k);
        double whc = 0.5 * (U(a.w, i, 1, k) + U(a.w, i, 1, kp)), whw = 0.5 * (U(a.w, i, 0, k) + U(a.w, i, 0, kp));
        double b1 = (uhc - uhw) * rdy1, b2 = (vhc - vhw) * rdyv, b3 = (whc - whw) * rdy1;
        double tc = 0.5 * (U(a.u, i, N2M, k) + U(a.u, ip, N2M, k)), tw = 0.5 * (U(a.u, i, N2, k) + U(a.u, ip, N2, k));
        double t1 = (tc - tw) * rdyt * (g.aly - 1.0);
        w1 += b1 + t1;
        w2 += b2 + t1;
        w3 += b3 + t1;
    }
    sh[0][threadIdx.x] = w1;
    sh[1][threadIdx.x] = w2;
    sh[2][threadIdx.x] = w3;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double nxz = 1.0 / (double)(n1 * n3);
        for (int c = 0; c < 3; ++c) a.scal[SCAL_WSMC + c] = sh[c][0] * nxz / g.re / g.aly;
    }
}

// SGSCS's plane coefficients from WSM: SMAGC(J) = (0.1 (1 - exp(-y+/26)))^2.
template <typename R>
__global__ void k_sgs_coef(StepArgs<R> a, LesArgs<R> l) {
    const Geo g = a.g;
    const double w1 = a.scal[SCAL_WSMC], w3 = a.scal[SCAL_WSMC + 2];
    const double utau = sqrt(sqrt(w1 * w1 + w3 * w3));
    for (int j = 1 + threadIdx.x; j <= g.n2m; j += blockDim.x) {
        const double yp = l.ycs[j] * utau * g.re;
        double cs = 0.1 * (1.0 - exp(-yp / 26.0));
        const double sm = cs * cs;
        l.smagc[j] = sm;
        l.coef[j] = (R)(sm * l.d23[j]);
    }
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_sgs_cs(StepArgs<R> a, LesArgs<R> l) {
    const Geo g = a.g;
    // 32-bit index arithmetic (a field has fewer than 2^31 points)
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (unsigned)g.n2m * (unsigned)g.np) return;
    const unsigned rw = tid / (unsigned)g.n1m, pj = rw / (unsigned)g.n3m;
    const int i = (int)(tid - rw * g.n1m), k = (int)(rw - pj * g.n3m), j = 1 + (int)pj;
    R sr[6];
    strain_at(a, l, i, j, k, sr);
    const R abss = sqrt((R)2.0 * sumsq6(sr));
    const R t = l.coef[j] * abss;
    l.nu[fidx(g, i, j, k)] = t > -l.reninv ? t : -l.reninv;
}

// SGSDY raw quantities: q[0..5] S_ij, q[6..11] DELTA^2|S| S_ij, q[12..14] cell-centre
// velocities (relative to the plane's velocity at (0, j, 0)), q[15..20] their products.
template <typename R>
__global__ void __launch_bounds__(TPB) k_sgs_raw(StepArgs<R> a, LesArgs<R> l) {
    typedef St<R> ST;
    const Geo g = a.g;
    // 32-bit index arithmetic (a field has fewer than 2^31 points)
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (unsigned)g.n2m * (unsigned)g.np) return;
    const unsigned rw = tid / (unsigned)g.n1m, pj = rw / (unsigned)g.n3m;
    const int i = (int)(tid - rw * g.n1m), k = (int)(rw - pj * g.n3m), j = 1 + (int)pj;
    R sr[6];
    strain_at(a, l, i, j, k, sr);
    const R abss = sqrt((R)2.0 * sumsq6(sr));
    l.nu[fidx(g, i, j, k)] = abss;
    const long long fs = (long long)g.n2m * g.np, q0 = tid;
    const R delabs = l.d23r[j] * abss;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        l.dyn[c * fs + q0] = sr[c];
        l.dyn[(6 + c) * fs + q0] = delabs * sr[c];
    }
    const int ip = wrapp(i, g.n1m), kp = wrapp(k, g.n3m);
    const auto cu = a.u[fidx(g, 0, j, 0)], cv = a.v[fidx(g, 0, j, 0)], cw = a.w[fidx(g, 0, j, 0)];
    const R half = (R)0.5;
    const R u1 = (ST::d(a.u[fidx(g, i, j, k)], cu) + ST::d(a.u[fidx(g, ip, j, k)], cu)) * half;
    const R u2 = (ST::d(a.v[fidx(g, i, j, k)], cv) + ST::d(a.v[fidx(g, i, j + 1, k)], cv)) * half;
    const R u3 = (ST::d(a.w[fidx(g, i, j, k)], cw) + ST::d(a.w[fidx(g, i, j, kp)], cw)) * half;
    l.dyn[12 * fs + q0] = u1;
    l.dyn[13 * fs + q0] = u2;
    l.dyn[14 * fs + q0] = u3;
    l.dyn[15 * fs + q0] = u1 * u1;
    l.dyn[16 * fs + q0] = u1 * u2;
    l.dyn[17 * fs + q0] = u1 * u3;
    l.dyn[18 * fs + q0] = u2 * u2;
    l.dyn[19 * fs + q0] = u2 * u3;
    l.dyn[20 * fs + q0] = u3 * u3;
}

// FILTER of one raw quantity at (i, k): Simpson (1,4,1)/6 along x, then along z.
template <typename R>
__device__ __forceinline__ R filt(const R *f, int n1, int n3, int i, int k) {
    const int ip = wrapp(i, n1), im = wrapm(i, n1), kp = wrapp(k, n3), km = wrapm(k, n3);
    const R six = (R)6.0, four = (R)4.0;
    auto T = [&](int kk) {
        const R *r = f + (long long)kk * n1;
        return (r[im] + four * r[i] + r[ip]) / six;
    };
    return (T(km) + four * T(k) + T(kp)) / six;
}

// SGSDY's test-filter stage, the plane sums (FP64, fixed order) and nu, one block per plane.
template <typename R>
__global__ void __launch_bounds__(256) k_sgs_dyn(StepArgs<R> a, LesArgs<R> l) {
    const Geo g = a.g;
    const int j = 1 + blockIdx.x;
    const long long fs = (long long)g.n2m * g.np, pb = (long long)(j - 1) * g.np;
    __shared__ double sn[256], sd[256];
    __shared__ R coefj;
    double snum = 0.0, sden = 0.0;
    const R fd = (R)4.0 * l.d23r[j];
    for (int e = threadIdx.x; e < g.np; e += blockDim.x) {
        const int i = e % g.n1m, k = e / g.n1m;
        R m[6], cf[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            m[c] = filt(l.dyn + c * fs + pb, g.n1m, g.n3m, i, k);
            cf[c] = filt(l.dyn + (6 + c) * fs + pb, g.n1m, g.n3m, i, k);
        }
        const R fdabs = fd * sqrt((R)2.0 * sumsq6(m));
#pragma unroll
        for (int c = 0; c < 6; ++c) m[c] = fdabs * m[c] - cf[c];
        R uc[3], up[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) uc[c] = filt(l.dyn + (12 + c) * fs + pb, g.n1m, g.n3m, i, k);
#pragma unroll
        for (int c = 0; c < 6; ++c) up[c] = filt(l.dyn + (15 + c) * fs + pb, g.n1m, g.n3m, i, k);
        const R L11 = up[0] - uc[0] * uc[0], L12 = up[1] - uc[0] * uc[1], L13 = up[2] - uc[0] * uc[2];
        const R L22 = up[3] - uc[1] * uc[1], L23 = up[4] - uc[1] * uc[2], L33 = up[5] - uc[2] * uc[2];
        const R two = (R)2.0;
        const R sqmm = sumsq6(m);
        const R sqlm = two * L12 * m[1] + L11 * m[0] + two * L13 * m[2] + L22 * m[3] + two * L23 * m[4] + L33 * m[5];
        sden += (double)sqmm;
        snum += (double)sqlm;
    }
    sn[threadIdx.x] = snum;
    sd[threadIdx.x] = sden;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sn[threadIdx.x] += sn[threadIdx.x + s];
            sd[threadIdx.x] += sd[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double nxz = 1.0 / (double)g.np;
        const double sm = -0.5 * (sn[0] * nxz) / (sd[0] * nxz);
        l.smagc[j] = sm;
        coefj = (R)(sm * l.d23[j]);
    }
    __syncthreads();
    const R c = coefj;
    R *nup = l.nu + fidx(g, 0, j, 0);
    for (int e = threadIdx.x; e < g.np; e += blockDim.x) {
        const R t = c * nup[e];
        nup[e] = t > -l.reninv ? t : -l.reninv;
    }
}

// ---------------------------------------------------------------------------------
// SGSSD (compact3d.f:1502-1948), the scale-dependent dynamic model, on SGSDY's raw
// quantities (k_sgs_raw).  k_sgs_sd_sums reads each raw quantity's 5x5 neighbourhood once
// and forms both test filters from it, FILTER (Simpson (1,4,1)/6 in x then z: 2 DELTA) and
// FILTER4 ((1,4,2,4,1)/12: 4 DELTA), then per level the five plane sums of the Germano
// identity, SR1 = DELTA^(2/3) |S~| S~ and COM1 = (DELTA^(2/3) |S| S)~:
//   L.SR1, L.COM1, COM1.COM1, SR1.SR1, SR1.COM1   (2x weight on the off-diagonal terms)
// per block in FP64.  The reference's third pass (the coefficient at 2 DELTA with
// M = 4 BETA DELTA^(2/3) |S~| S~ - COM1, its unclipped BETA) needs no sums of its own: M
// is linear in BETA, so sum(L.M) = 4 BETA sum(L.SR1) - sum(L.COM1) and sum(M.M) =
// 16 BETA^2 sum(SR1.SR1) - 8 BETA sum(SR1.COM1) + sum(COM1.COM1) at the FILTER level.
// k_sgs_sd_coef: per plane COEFFICIENT, DQRRT/CHHQR and SMAGC; k_sgs_apply: nu.
// ---------------------------------------------------------------------------------
constexpr int SD_NS = 10;

// 2 a1 b1 + a0 b0 + 2 a2 b2 + a3 b3 + 2 a4 b4 + a5 b5
template <typename R>
__device__ __forceinline__ R dot6(const R *a, const R *b) {
    return (R)2.0 * a[1] * b[1] + a[0] * b[0] + (R)2.0 * a[2] * b[2] + a[3] * b[3] + (R)2.0 * a[4] * b[4] + a[5] * b[5];
}

// the five sums of one filter level from the filtered S (f[0..5]), COM1 (6..11), UC
// (12..14, relative to a per-plane velocity) and UC products (15..20)
template <typename R>
__device__ __forceinline__ void sd_level(const R *f, R d23, double *acc) {
    R m[6], sr1[6], L[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) m[c] = f[c];
    const R fdabs = d23 * sqrt((R)2.0 * sumsq6(m));
#pragma unroll
    for (int c = 0; c < 6; ++c) sr1[c] = fdabs * m[c];
    const R *uc = f + 12, *up = f + 15, *cf = f + 6;
    L[0] = up[0] - uc[0] * uc[0];
    L[1] = up[1] - uc[0] * uc[1];
    L[2] = up[2] - uc[0] * uc[2];
    L[3] = up[3] - uc[1] * uc[1];
    L[4] = up[4] - uc[1] * uc[2];
    L[5] = up[5] - uc[2] * uc[2];
    acc[0] += (double)dot6(L, sr1);
    acc[1] += (double)dot6(L, cf);
    acc[2] += (double)dot6(cf, cf);
    acc[3] += (double)dot6(sr1, sr1);
    acc[4] += (double)dot6(sr1, cf);
}

// One block per tile of SD_TX x SD_TZ points of a plane (grid: x tiles, z tiles, N2M),
// one thread per point.  Field by field, the tile and a halo of two is staged in shared
// memory, filtered along x by both stencils, then along z at each point; both levels'
// sums go to part[((j - 1) tiles + tile) SD_NS + q].
constexpr int SD_TX = 32, SD_TZ = 16, SD_THREADS = SD_TX * SD_TZ;
template <typename R>
__global__ void __launch_bounds__(SD_THREADS) k_sgs_sd_sums(StepArgs<R> a, LesArgs<R> l, double *part) {
    const Geo g = a.g;
    const int n1 = g.n1m, n3 = g.n3m;
    const int j = 1 + blockIdx.z, i0 = blockIdx.x * SD_TX, k0 = blockIdx.y * SD_TZ;
    const int tx = threadIdx.x % SD_TX, tz = threadIdx.x / SD_TX;
    const long long fs = (long long)g.n2m * g.np, pb = (long long)(j - 1) * g.np;
    // the stencils' divisions by 6 and 12 as products with the rounded reciprocals (a
    // rounding of the last bit; the sums are FP64 and reordered anyway)
    const R four = (R)4.0, two = (R)2.0, r6 = (R)(1.0 / 6.0), r12 = (R)(1.0 / 12.0);
    __shared__ R raw[SD_TZ + 4][SD_TX + 4];
    __shared__ R f3x[SD_TZ + 2][SD_TX], f4x[SD_TZ + 4][SD_TX];
    R f3[21], f4[21];
#pragma unroll 1
    for (int c = 0; c < 21; ++c) {
        const R *f = l.dyn + c * fs + pb;
        for (int q = threadIdx.x; q < (SD_TZ + 4) * (SD_TX + 4); q += SD_THREADS) {
            const int rz = q / (SD_TX + 4), rx = q - rz * (SD_TX + 4);
            int ii = i0 + rx - 2, kk = k0 + rz - 2;
            ii = ii < 0 ? ii + n1 : (ii >= n1 ? ii - n1 : ii);
            kk = kk < 0 ? kk + n3 : (kk >= n3 ? kk - n3 : kk);
            ii = ii < 0 ? ii + n1 : (ii >= n1 ? ii - n1 : ii);   // tiles wider than N1M
            raw[rz][rx] = f[(long long)kk * n1 + ii];
        }
        __syncthreads();
        for (int q = threadIdx.x; q < (SD_TZ + 4) * SD_TX; q += SD_THREADS) {
            const int rz = q / SD_TX, x = q - rz * SD_TX;
            const R *r = &raw[rz][x];
            f4x[rz][x] = (r[0] + four * r[1] + two * r[2] + four * r[3] + r[4]) * r12;
            if (rz >= 1 && rz <= SD_TZ + 2) f3x[rz - 1][x] = (r[1] + four * r[2] + r[3]) * r6;
        }
        __syncthreads();
        f3[c] = (f3x[tz][tx] + four * f3x[tz + 1][tx] + f3x[tz + 2][tx]) * r6;
        f4[c] = (f4x[tz][tx] + four * f4x[tz + 1][tx] + two * f4x[tz + 2][tx] + four * f4x[tz + 3][tx] + f4x[tz + 4][tx]) *
                r12;
    }
    double acc[SD_NS];
#pragma unroll
    for (int q = 0; q < SD_NS; ++q) acc[q] = 0.0;
    if (i0 + tx < n1) {
        const R d23 = l.d23r[j];
        sd_level(f3, d23, acc);
        sd_level(f4, d23, acc + 5);
    }
    // fixed-order reduction: lanes by shuffle, then the block's warps in order
    __shared__ double red[SD_THREADS / 32][SD_NS];
#pragma unroll
    for (int q = 0; q < SD_NS; ++q) {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < SD_NS) {
        double v = 0.0;
        for (int w = 0; w < SD_THREADS / 32; ++w) v += red[w][threadIdx.x];
        const int nt = gridDim.x * gridDim.y, tile = blockIdx.y * gridDim.x + blockIdx.x;
        part[((long long)(j - 1) * nt + tile) * SD_NS + threadIdx.x] = v;
    }
}

// CHHQR (compact3d.f:11571-11676) for the 5x5 companion matrix by one warp, every
// operation rounded as written: eigenvalues of an upper Hessenberg matrix by the Francis
// double-shift QR with the deflation test |A(L,L-1)| <= EPS (|A(L-1,L-1)| + |A(L,L)|), at
// most 60 sweeps per deflation (after which the roots not found stay 0).  A (column-major,
// 1-based) and WR are in shared memory; every lane forms the reflection's scalars, lane t
// updates column K + t (rows K..K+2) and then row L + t (columns K..K+2).
#define SD_M(x, y) __dmul_rn(x, y)
#define SD_A(x, y) __dadd_rn(x, y)
#define SD_S(x, y) __dsub_rn(x, y)
__device__ void sd_chhqr5_warp(double *A, double *WR, double EPS) {
    constexpr int N = 5;
    const int lane = threadIdx.x & 31;
    auto a = [&](int i, int j) -> double & { return A[(i - 1) + N * (j - 1)]; };
    int M = N, IT = 0;
    for (int guard = 0; M > 0 && guard < 1000; ++guard) {
        int L = M;
        while (L > 1 && fabs(a(L, L - 1)) > SD_M(EPS, SD_A(fabs(a(L - 1, L - 1)), fabs(a(L, L))))) L = L - 1;
        if (L == M) {
            if (lane == 0) WR[M - 1] = a(M, M);
            M = M - 1;
            IT = 0;
            continue;
        }
        if (L == M - 1) {
            const double B = -SD_A(a(M, M), a(M - 1, M - 1));
            const double C = SD_S(SD_M(a(M, M), a(M - 1, M - 1)), SD_M(a(M, M - 1), a(M - 1, M)));
            const double W = SD_S(SD_M(B, B), SD_M(4.0, C));
            const double Y = sqrt(fabs(W));
            if (lane == 0) {
                if (W > 0.0) {
                    const double XY = B < 0.0 ? -1.0 : 1.0;
                    WR[M - 1] = SD_S(-B, SD_M(XY, Y)) / 2.0;
                    WR[M - 2] = C / WR[M - 1];
                } else {
                    WR[M - 1] = -B / 2.0;
                    WR[M - 2] = WR[M - 1];
                }
            }
            M = M - 2;
            IT = 0;
            continue;
        }
        if (IT >= 60) return;
        IT = IT + 1;
        __syncwarp();
        if (lane == 0) {
            for (int J = L + 2; J <= M; J++) a(J, J - 2) = 0.0;
            for (int J = L + 3; J <= M; J++) a(J, J - 3) = 0.0;
        }
        __syncwarp();
        for (int K = L; K <= M - 1; K++) {
            double P, Q, R;
            if (K != L) {
                P = a(K, K - 1);
                Q = a(K + 1, K - 1);
                R = K != M - 1 ? a(K + 2, K - 1) : 0.0;
            } else {
                const double X = SD_A(a(M, M), a(M - 1, M - 1));
                const double Y = SD_S(SD_M(a(M - 1, M - 1), a(M, M)), SD_M(a(M - 1, M), a(M, M - 1)));
                P = SD_A(SD_A(SD_M(a(L, L), SD_S(a(L, L), X)), SD_M(a(L, L + 1), a(L + 1, L))), Y);
                Q = SD_M(a(L + 1, L), SD_S(SD_A(a(L, L), a(L + 1, L + 1)), X));
                R = SD_M(a(L + 1, L), a(L + 2, L + 1));
            }
            if (SD_A(SD_A(fabs(P), fabs(Q)), fabs(R)) == 0.0) continue;
            const double XY = P < 0.0 ? -1.0 : 1.0;
            const double S = SD_M(XY, sqrt(SD_A(SD_A(SD_M(P, P), SD_M(Q, Q)), SD_M(R, R))));
            const double E = -Q / S, F = -R / S, X = -P / S;
            const double PS = SD_A(P, S);
            const double Y = SD_S(-X, SD_M(F, R) / PS);
            const double G = SD_M(E, R) / PS;
            const double Z = SD_S(-X, SD_M(E, Q) / PS);
            __syncwarp();
            if (K != L && lane == 0) a(K, K - 1) = -S;
            const int J = K + lane;
            if (J <= M) {
                double p = SD_A(SD_M(X, a(K, J)), SD_M(E, a(K + 1, J)));
                double q = SD_A(SD_M(E, a(K, J)), SD_M(Y, a(K + 1, J)));
                double r = SD_A(SD_M(F, a(K, J)), SD_M(G, a(K + 1, J)));
                if (K != M - 1) {
                    p = SD_A(p, SD_M(F, a(K + 2, J)));
                    q = SD_A(q, SD_M(G, a(K + 2, J)));
                    r = SD_A(r, SD_M(Z, a(K + 2, J)));
                    a(K + 2, J) = r;
                }
                a(K + 1, J) = q;
                a(K, J) = p;
            }
            __syncwarp();
            const int JJ = K + 3 >= M ? M : K + 3;
            const int I = L + lane;
            if (I <= JJ) {
                double p = SD_A(SD_M(X, a(I, K)), SD_M(E, a(I, K + 1)));
                double q = SD_A(SD_M(E, a(I, K)), SD_M(Y, a(I, K + 1)));
                double r = SD_A(SD_M(F, a(I, K)), SD_M(G, a(I, K + 1)));
                if (K != M - 1) {
                    p = SD_A(p, SD_M(F, a(I, K + 2)));
                    q = SD_A(q, SD_M(G, a(I, K + 2)));
                    r = SD_A(r, SD_M(Z, a(I, K + 2)));
                    a(I, K + 2) = r;
                }
                a(I, K + 1) = q;
                a(I, K) = p;
            }
            __syncwarp();
        }
    }
}

// per plane: the sums, COEFFICIENT (compact3d.f:2079-2095), DQRRT's BETA (11548-11569,
// EPS 1.0E-5) and SMAGC; one warp per plane
template <typename R>
__global__ void __launch_bounds__(32) k_sgs_sd_coef(StepArgs<R> a, LesArgs<R> l, const double *part, int nt,
                                                    double *beta) {
    const Geo g = a.g;
    const int j = 1 + blockIdx.x, lane = threadIdx.x;
    __shared__ double Am[25], WR[5], s[SD_NS];
    if (lane < SD_NS) {
        double v = 0.0;
        for (int t = 0; t < nt; ++t) v += part[((long long)(j - 1) * nt + t) * SD_NS + lane];
        s[lane] = v;
    }
    if (lane < 5) WR[lane] = 0.0;
    __syncwarp();
    const double NXZ = 1.0 / (double)(g.n1m * g.n3m);
    const double A1 = -8.0 * s[0] * NXZ, B1 = -2.0 * s[1] * NXZ, C1 = 4.0 * s[2] * NXZ, D1 = 64.0 * s[3] * NXZ,
                 E1 = 32.0 * s[4] * NXZ;
    const double A2 = -32.0 * s[5] * NXZ, B2 = -2.0 * s[6] * NXZ, C2 = 4.0 * s[7] * NXZ, D2 = 1024.0 * s[8] * NXZ,
                 E2 = 128.0 * s[9] * NXZ;
    const double AD = SD_M(A1, D2);
    double PA[5];
    PA[4] = SD_S(SD_M(B2, C1), SD_M(B1, C2)) / AD;
    PA[3] = SD_S(SD_M(A1, C2), SD_M(B2, E1)) / AD;
    PA[2] = SD_S(SD_A(SD_M(B2, D1), SD_M(B1, E2)), SD_M(A2, C1)) / AD;
    PA[1] = SD_S(SD_M(A2, E1), SD_M(A1, E2)) / AD;
    PA[0] = -SD_A(SD_M(A2, D1), SD_M(B1, D2)) / AD;
    if (lane < 25) {   // the companion matrix: first row -PA, ones below the diagonal
        const int i = lane % 5, c = lane / 5;
        Am[lane] = i == 0 ? -PA[c] : (i == c + 1 ? 1.0 : 0.0);
    }
    __syncwarp();
    sd_chhqr5_warp(Am, WR, 1.0E-5);
    __syncwarp();
    double BETA = 0.;
    for (int J = 0; J < 5; J++)
        if (WR[J] > BETA && WR[J] < 2.0) BETA = WR[J];
    if (lane == 0) {
        beta[j] = BETA;
        const double num = SD_S(SD_M(SD_M(4.0, BETA), s[0]), s[1]);
        const double den = SD_A(SD_S(SD_M(SD_M(SD_M(16.0, BETA), BETA), s[3]), SD_M(SD_M(8.0, BETA), s[4])), s[2]);
        const double sm = -0.5 * (num * NXZ) / (den * NXZ);
        l.smagc[j] = sm;
        l.coef[j] = (R)(sm * l.d23[j]);
    }
}
#undef SD_M
#undef SD_A
#undef SD_S

// nu = max(coef(J) |S|, -1/RE) over the N2M planes (|S| left in nu by k_sgs_raw)
template <typename R>
__global__ void __launch_bounds__(TPB) k_sgs_apply(StepArgs<R> a, LesArgs<R> l) {
    const Geo g = a.g;
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (unsigned)g.n2m * (unsigned)g.np) return;
    const int j = 1 + (int)(tid / (unsigned)g.np);
    R *nup = l.nu + (long long)g.np + tid;   // fidx(g, 0, j, 0) + e with j >= 1
    const R t = l.coef[j] * *nup;
    *nup = t > -l.reninv ? t : -l.reninv;
}

// ---------------------------------------------------------------------------------
// WALLMODEL_INSTANT: one thread per bottom-wall point; FP64.  The reference's Newton loop
// has no cap; here a point that has not converged after l.wall_cap iterations is counted
// and the step reports C3D_ENOTCONV.
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall(StepArgs<R> a, LesArgs<R> l) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double ssum[TPB], sbad[TPB];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double tw1 = 0.0, bad = 0.0;
    if (e < g.np) {
        const int i = e % g.n1m, k = e / g.n1m;
        const double u3 = ST::dbl(a.u[fidx(g, i, 3, k)]), w3 = ST::dbl(a.w[fidx(g, i, 3, k)]);
        const double KAPA = 0.41, B = 5.2, RE = g.re;
        const double DELTAP = g.dy[1] + g.dy[2] + g.dy[3] / 2.0;
        const double uave = sqrt(u3 * u3 + w3 * w3);
        double ut1 = 1.0, ut2 = 0.000001, lambda = 1.0;
        // f(ut1) of an iteration is f(ut2) of the one before (same expression, same
        // argument), so each iteration evaluates the log law once
        double f3 = uave / ut2 - log(ut2 * DELTAP * RE) / KAPA - B;
        int it = 0;
        while (fabs(ut2 - ut1) > 1.0e-6) {
            if (++it > l.wall_cap) {
                bad = 1.0;
                break;
            }
            ut1 = ut2;
            const double f1 = f3;
            const double f2 = -uave / (ut1 * ut1) - 1.0 / KAPA / ut1;
            ut2 = ut1 - lambda * f1 / f2;
            f3 = uave / ut2 - log(ut2 * DELTAP * RE) / KAPA - B;
            if (fabs(f3) > fabs(f1)) lambda = 0.5 * lambda;
        }
        tw1 = ut1 * ut1;
        l.tauw[e] = tw1 * u3 / uave;
        l.taub[e] = tw1 * w3 / uave;
    }
    ssum[threadIdx.x] = tw1;
    sbad[threadIdx.x] = bad;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            ssum[threadIdx.x] += ssum[threadIdx.x + s];
            sbad[threadIdx.x] += sbad[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        l.wpart[blockIdx.x] = ssum[0];
        l.wpart[gridDim.x + blockIdx.x] = sbad[0];
    }
}

// WALLMODEL_ROUGH (WMODEL 1 with Y0 = Y(0) != 0, compact3d.f:2496-2558), FP64: the rough-
// wall log law TAUW1 = (0.41 U / log(DELTAP / Y0))^2 per bottom-wall point along the
// velocity of plane 3, with per-block sums of TAUW1 for WSM(1).
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_rough(StepArgs<R> a, LesArgs<R> l, double klog) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double ssum[TPB];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double tw1 = 0.0;
    if (e < g.np) {
        const int i = e % g.n1m, k = e / g.n1m;
        const double u3 = ST::dbl(a.u[fidx(g, i, 3, k)]), w3 = ST::dbl(a.w[fidx(g, i, 3, k)]);
        const double uave = sqrt(__dadd_rn(__dmul_rn(u3, u3), __dmul_rn(w3, w3)));
        const double t = klog * uave;
        tw1 = t * t;
        l.tauw[e] = tw1 * u3 / uave;
        l.taub[e] = tw1 * w3 / uave;
    }
    ssum[threadIdx.x] = tw1;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) ssum[threadIdx.x] += ssum[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        l.wpart[blockIdx.x] = ssum[0];
        l.wpart[gridDim.x + blockIdx.x] = 0.0;
    }
}

// WALLMODEL_WERNER (compact3d.f:4815-4958), FP64: the Werner-Wengle power law at the first
// cell centre of both walls into tw4 (TAUWE(I,K,1..4), four planes of N1M x N3M), with
// per-block sums of the bottom u-stress for WSM(1); the reference's x neighbour taken with
// the z index (IPA(K), F:4852) is kept.  VCASE uses WSM(1) of the step before.
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_werner(StepArgs<R> a, LesArgs<R> l, double *tw4) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double ssum[TPB];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double t1 = 0.0;
    if (e < g.np) {
        const int i = e % g.n1m, k = e / g.n1m;
        const int ik = (k + 1) % g.n1m;            // IPA(K) - 1 (0-based), N3M <= N1M
        const int kp = (k + 1) % g.n3m;
        const double B = 0.1428571429, AB1 = 7.202125274, AB3 = 69.74057973, AB4 = 0.1376936317, AB5 = 1.75;
        const double VCASE = AB3 * (sqrt(fabs(a.scal[SCAL_WSMC])) / 11.81);
        for (int wall = 0; wall < 2; ++wall) {
            const int jw = wall == 0 ? 1 : g.n2m;
            const double DELTAP = g.dy[jw];
            const double U1 = 0.5 * (ST::dbl(a.u[fidx(g, i, jw, k)]) + ST::dbl(a.u[fidx(g, ik, jw, k)]));
            const double U2 = 0.5 * (ST::dbl(a.w[fidx(g, i, jw, k)]) + ST::dbl(a.w[fidx(g, i, jw, kp)]));
            const double VELOCP = sqrt(U1 * U1 + U2 * U2);
            double TAUW1;
            if (VELOCP <= VCASE) {
                TAUW1 = 2. * VELOCP / DELTAP / g.re;
            } else {
                TAUW1 = AB1 * pow(1.0 / DELTAP / g.re, 1. + B);
                TAUW1 = TAUW1 + AB4 * pow(1.0 / DELTAP / g.re, B) * VELOCP;
                TAUW1 = pow(TAUW1, AB5);
            }
            tw4[(2 * wall) * g.np + e] = TAUW1 * (U1 / VELOCP);
            tw4[(2 * wall + 1) * g.np + e] = TAUW1 * (U2 / VELOCP);
            if (wall == 0) t1 = TAUW1 * (U1 / VELOCP);
        }
    }
    ssum[threadIdx.x] = t1;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) ssum[threadIdx.x] += ssum[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        l.wpart[blockIdx.x] = ssum[0];
        l.wpart[gridDim.x + blockIdx.x] = 0.0;
    }
}

// WERNER's averaging to the stress points: TAUW = (TAUWE(I) + TAUWE(IMA(K))) / 2 (the x
// neighbour with the z index again, F:4924), TAUB = (TAUWE(K) + TAUWE(K-1)) / 2, both walls.
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_werner_avg(StepArgs<R> a, LesArgs<R> l, const double *tw4) {
    const Geo g = a.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const int i = e % g.n1m, k = e / g.n1m;
    const int im = (k + g.n1m - 1) % g.n1m;       // IMA(K) - 1
    const int km = (k + g.n3m - 1) % g.n3m;
    const int ei = k * g.n1m + im, ek = km * g.n1m + i;
    for (int wall = 0; wall < 2; ++wall) {
        const double *tu = tw4 + (2 * wall) * g.np, *tw = tw4 + (2 * wall + 1) * g.np;
        l.tauw[wall * g.np + e] = 0.5 * (tu[e] + tu[ei]);
        l.taub[wall * g.np + e] = 0.5 * (tw[e] + tw[ek]);
    }
}

// ---------------------------------------------------------------------------------
// The shifted-point models, FP64: MARUSIC1 (WMODEL 3, compact3d.f:4336-4495) and PIOMELLI
// (WMODEL 5, 4960-5110).  u_tau of each wall from the log law on the plane mean of u at a
// reference plane (bisection), then per wall point the velocity interpolated trilinearly
// (INTERPOLAT, 12602-12760) at a point shifted downstream by DELTS (MARUSIC1: DELTAP /
// tan 16 deg; PIOMELLI: 0, its DELTP is never set) at the height YP.  The mesh of MESH02
// (uniform XG/ZG faces, cell centres XC/YC/ZC) is formed from the grid on the fly with
// the reference's operation order and no contractions, so the cell search and the
// interpolation weights are those of the FP64 restatement.
//
// The scratch ws (layout in WsMesh) holds Y(0:N2), YC(0:N2), per wall WS_NPAR parameters,
// per wall the heights INDEX_IJK leaves in YP call after call, and XG, XC, ZG, ZC(0:N+1)
// (formed once by k_wall_shift_init).  The reference moves YP up by about 1e-6 on every
// call while it is below YC(1) (its arguments are by reference and YP is set once per
// wall), so call c of a wall uses tab[min(c, nfix)].
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double nudge_up(double x) {   // ANINT(X*1E06+0.5)/1E06
    return __ddiv_rn(round(__dadd_rn(__dmul_rn(x, 1E06), 0.5)), 1E06);
}
__device__ __forceinline__ double nudge_dn(double x) {   // ANINT(X*1E06-0.5)/1E06
    return __ddiv_rn(round(__dsub_rn(__dmul_rn(x, 1E06), 0.5)), 1E06);
}
// XG(I) of MESH02 on a uniform grid of n cells over [0, L], I = 1..n+1
__device__ __forceinline__ double ws_face(int I, int n, double L) {
    return I > n ? L : __ddiv_rn(__dmul_rn((double)(I - 1), L), (double)n);
}
// XC(I) = (XG(I+1) + XG(I)) / 2, XC(n+1) = L
__device__ __forceinline__ double ws_ctr(int I, int n, double L) {
    return I > n ? L : __dmul_rn(0.5, __dadd_rn(ws_face(I + 1, n, L), ws_face(I, n, L)));
}
// (B - A) / (HI - LO) * (X - LO) + A, rounded step by step
__device__ __forceinline__ double ws_lerp(double A, double B, double LO, double HI, double X) {
    return __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(B, A), __dsub_rn(HI, LO)), __dsub_rn(X, LO)), A);
}

struct WsMesh {
    const double *Y, *YC, *XG, *XC, *ZG, *ZC;
    const double *V1;  // V(I,1,K) as the step found it (BCOND zeroes it before the model ends)
    double rx, rz;     // N1M / ALX, N3M / ALZ (first guesses of the x and z cells)
    double ix1, ix3;   // 1 / DX1, 1 / DX3
    __host__ __device__ static size_t off_par(const Geo &g) { return 2 * ((size_t)g.n2 + 1); }
    __host__ __device__ static size_t off_tab(const Geo &g) { return off_par(g) + 2 * WS_NPAR; }
    __host__ __device__ static size_t off_xg(const Geo &g) { return off_tab(g) + 2 * (size_t)WS_TABN; }
    __host__ __device__ static size_t off_v1(const Geo &g) { return off_xg(g) + 2 * ((size_t)g.n1m + 2) + 2 * ((size_t)g.n3m + 2); }
    __host__ __device__ static size_t size(const Geo &g) { return off_v1(g) + (size_t)g.np; }
    __host__ static WsMesh of(const Geo &g, const double *ws) {
        WsMesh m;
        m.Y = ws;
        m.YC = ws + g.n2 + 1;
        m.XG = ws + off_xg(g);
        m.XC = m.XG + g.n1m + 2;
        m.ZG = m.XC + g.n1m + 2;
        m.ZC = m.ZG + g.n3m + 2;
        m.V1 = ws + off_v1(g);
        m.rx = g.n1m / g.alx;
        m.rz = g.n3m / g.alz;
        m.ix1 = 1. / g.dx1;
        m.ix3 = 1. / g.dx3;
        return m;
    }
};

// XG, XC (0:N1M+1) and ZG, ZC (0:N3M+1) of MESH02
__global__ void k_wall_shift_init(Geo g, double *ws) {
    double *XG = ws + WsMesh::off_xg(g), *XC = XG + g.n1m + 2, *ZG = XC + g.n1m + 2, *ZC = ZG + g.n3m + 2;
    for (int I = threadIdx.x; I <= g.n1m + 1; I += blockDim.x) {
        XG[I] = I == 0 ? 0.0 : ws_face(I, g.n1m, g.alx);
        XC[I] = I == 0 ? 0.0 : ws_ctr(I, g.n1m, g.alx);
    }
    for (int K = threadIdx.x; K <= g.n3m + 1; K += blockDim.x) {
        ZG[K] = K == 0 ? 0.0 : ws_face(K, g.n3m, g.alz);
        ZC[K] = K == 0 ? 0.0 : ws_ctr(K, g.n3m, g.alz);
    }
}

// PIOMELLI interpolates V between the faces J = 1 and 2 at the bottom wall; the step's
// BCOND sets V(J=1) while the model may still run beside it, so the plane is copied first
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_shift_v1(StepArgs<R> a, double *ws) {
    typedef St<R> ST;
    const Geo g = a.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < g.np) ws[WsMesh::off_v1(g) + e] = ST::dbl(a.v[(long long)g.np + e]);
}

// INDEX_IJK in one direction: the first cell I in 1..n with F(I) <= X <= F(I+1) of the
// increasing faces F(1..n+1); r n / (F(n+1) - F(1)) gives the first guess
__device__ __forceinline__ int ws_cell(double X, const double *F, int n, double r) {
    if (!(X >= F[1] && X <= F[n + 1])) return -1;
    int I = min(n, max(1, (int)((X - F[1]) * r) + 1));
    while (I > 1 && X <= F[I]) --I;
    while (I < n && X > F[I + 1]) ++I;
    return (X >= F[I] && X <= F[I + 1]) ? I : -1;
}

// ... in y (non-uniform): bisection over Y(1..N2)
__device__ __forceinline__ int ws_ycell(double YP, const double *Y, int n2m) {
    int lo = 1, hi = n2m;   // the first J with YP <= Y(J+1)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (YP <= Y[mid + 1]) hi = mid;
        else lo = mid + 1;
    }
    return (YP >= Y[lo] && YP <= Y[lo + 1]) ? lo : -1;
}

// INTERPOLAT of component C (1 u at x faces, 2 v at y faces, 3 w at z faces) at
// (XP, YP, ZP) in cell (IP, JP, KP), Fortran indices; JPA(N2M) = N2M and JMU(1) = 1.
template <typename R>
__device__ double ws_interp(const StepArgs<R> &a, const WsMesh &m, double XP, double YP, double ZP, int IP, int JP,
                            int KP, int C) {
    typedef St<R> ST;
    const Geo &g = a.g;
    const int n1 = g.n1m, n2m = g.n2m, n3 = g.n3m, N2 = g.n2;
    int IUM, IUP, JUM, JUP, KUM, KUP;
    double XUM, XUP, YUM, YUP, ZUM, ZUP;
    const int IPA = IP == n1 ? 1 : IP + 1, IMA = IP == 1 ? n1 : IP - 1;
    if (C == 1) {
        IUM = IP; IUP = IPA; XUM = m.XG[IP]; XUP = m.XG[IUP];
        if (IP == n1) XUP = m.XG[n1 + 1];
    } else if (XP >= m.XC[IP]) {
        IUM = IP; IUP = IPA; XUM = m.XC[IP]; XUP = m.XC[IUP];
        if (IP == n1) XUP = __dadd_rn(m.XC[n1], m.ix1);
    } else {
        IUM = IMA; IUP = IP; XUM = m.XC[IUM]; XUP = m.XC[IP];
        if (IP == 1) XUM = __dsub_rn(m.XC[1], m.ix1);
    }
    const int JPA = JP == n2m ? n2m : JP + 1, JMU = JP == 1 ? 1 : JP - 1;
    if (C == 2) {
        JUM = JP; JUP = JPA; YUM = m.Y[JP]; YUP = m.Y[JUP];
        if (JP == n2m) YUP = m.YC[N2];
    } else if (YP >= m.YC[JP]) {
        JUM = JP; JUP = JPA; YUM = m.YC[JP]; YUP = m.YC[JUP];
        if (JP == n2m) YUP = m.YC[N2];
    } else {
        JUM = JMU; JUP = JP; YUM = m.YC[JUM]; YUP = m.YC[JP];
        if (JP == 1) YUM = m.Y[1];
    }
    const int KPA = KP == n3 ? 1 : KP + 1, KMA = KP == 1 ? n3 : KP - 1;
    if (C == 3) {
        KUM = KP; KUP = KPA; ZUM = m.ZG[KP]; ZUP = m.ZG[KUP];
        if (KP == n3) ZUP = m.ZG[n3 + 1];
    } else if (ZP >= m.ZC[KP]) {
        KUM = KP; KUP = KPA; ZUM = m.ZC[KP]; ZUP = m.ZC[KUP];
        if (KP == n3) ZUP = __dadd_rn(m.ZC[n3], m.ix3);
    } else {
        KUM = KMA; KUP = KP; ZUM = m.ZC[KUM]; ZUP = m.ZC[KP];
        if (KP == 1) ZUM = __dsub_rn(m.ZC[1], m.ix3);
    }
    const typename StepArgs<R>::S *F = C == 1 ? a.u : (C == 2 ? a.v : a.w);
    auto f = [&](int I, int J, int K) {
        return C == 2 && J == 1 && m.V1 ? m.V1[(K - 1) * n1 + (I - 1)] : ST::dbl(F[fidx(g, I - 1, J, K - 1)]);
    };
    const double PHA = f(IUM, JUM, KUM), PHB = f(IUP, JUM, KUM), PHC = f(IUP, JUP, KUM), PHD = f(IUM, JUP, KUM);
    const double PHE = f(IUM, JUM, KUP), PHF = f(IUP, JUM, KUP), PHG = f(IUP, JUP, KUP), PHH = f(IUM, JUP, KUP);
    const double PHAB = ws_lerp(PHA, PHB, XUM, XUP, XP), PHCD = ws_lerp(PHD, PHC, XUM, XUP, XP);
    const double PHEF = ws_lerp(PHE, PHF, XUM, XUP, XP), PHGH = ws_lerp(PHH, PHG, XUM, XUP, XP);
    const double PHABCD = ws_lerp(PHAB, PHCD, YUM, YUP, YP), PHEFGH = ws_lerp(PHEF, PHGH, YUM, YUP, YP);
    return ws_lerp(PHABCD, PHEFGH, ZUM, ZUP, ZP);
}

// per-block sums of u on the two reference planes (jd: bottom, ju: top)
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_shift_mean(StepArgs<R> a, LesArgs<R> l, int jd, int ju) {
    typedef St<R> ST;
    const Geo g = a.g;
    __shared__ double sd[TPB], su[TPB];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0.0, u = 0.0;
    if (e < g.np) {
        const int i = e % g.n1m, k = e / g.n1m;
        d = ST::dbl(a.u[fidx(g, i, jd, k)]);
        u = ST::dbl(a.u[fidx(g, i, ju, k)]);
    }
    sd[threadIdx.x] = d;
    su[threadIdx.x] = u;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sd[threadIdx.x] += sd[threadIdx.x + s];
            su[threadIdx.x] += su[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        l.wpart[blockIdx.x] = sd[0];
        l.wpart[gridDim.x + blockIdx.x] = su[0];
    }
}

// The log-law bisection (compact3d.f:4390-4402, 5017-5029) run by one warp.  The reference
// keeps an anchor end a = U_tau1 and the other end b = U_tau2 and, while |b - a| > 1e-7,
// halves the bracket at m = b/2 + a/2 toward the sign change of f(a) f(m), returning a.
// Each round here covers five of those steps: lane q (1..31) forms the bracket of node q
// of the five-level decision tree with the same midpoint arithmetic and evaluates f at
// its midpoint; the warp then walks the tree with the sequential rule.  Every midpoint
// and every f value is the one the sequential loop computes (f(a) of a step is the f of
// the midpoint that became a), so the result is the same.
__device__ __forceinline__ double loglaw_f(double U_ave, double ut, double DELTAP, double RE) {
    const double KAPA = 0.41, B = 5.2;
    return U_ave / ut - log(ut * DELTAP * RE) / KAPA - B;
}
__device__ __forceinline__ double mid_rn(double a, double b) {
    return __dadd_rn(__dmul_rn(0.5, b), __dmul_rn(0.5, a));
}
__device__ double ws_bisect_warp(double U_ave, double DELTAP, double RE, double a, double b) {
    const int lane = threadIdx.x & 31;
    double fa = loglaw_f(U_ave, a, DELTAP, RE);
    const int depth = lane ? 31 - __clz(lane) : 0;
    for (int round = 0; round < 64 && fabs(b - a) > 0.0000001; ++round) {
        double na = a, nb = b;
        for (int q = depth - 1; q >= 0; --q) {
            const double m = mid_rn(na, nb);
            if ((lane >> q) & 1) na = m;
            else nb = m;
        }
        const double m = mid_rn(na, nb);
        const double fm = lane ? loglaw_f(U_ave, m, DELTAP, RE) : 0.0;
        int node = 1;
        for (int q = 0; q < 5 && fabs(b - a) > 0.0000001; ++q) {
            const double mm = __shfl_sync(FULL, m, node), fmm = __shfl_sync(FULL, fm, node);
            if (fa * fmm <= 0.0) {
                b = mm;
                node = 2 * node;
            } else {
                a = mm;
                fa = fmm;
                node = 2 * node + 1;
            }
        }
    }
    return a;
}

// plane means, u_tau, the per-wall constants and the YP heights; one block of 256
template <typename R>
__global__ void k_wall_shift_fin(StepArgs<R> a, LesArgs<R> l, int nb, double *ws, int zs, double tan16) {
    const Geo g = a.g;
    __shared__ double s[256], b[256];
    double x = 0.0, y = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        x += l.wpart[q];
        y += l.wpart[nb + q];
    }
    s[threadIdx.x] = x;
    b[threadIdx.x] = y;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s[threadIdx.x] += s[threadIdx.x + w];
            b[threadIdx.x] += b[threadIdx.x + w];
        }
        __syncthreads();
    }
    const int wall = threadIdx.x >> 5;   // warp 0: bottom wall, warp 1: top wall
    if (wall >= 2) return;
    const double *YC = ws + (g.n2 + 1);
    double *par = ws + WsMesh::off_par(g) + WS_NPAR * wall;
    double *tab = ws + WsMesh::off_tab(g) + (size_t)WS_TABN * wall;
    const double U_ave = (wall == 0 ? s[0] : b[0]) / (double)(g.n1m * g.n3m);
    const bool mar = l.wmodel == 3;
    double DELTAP, UTAU2, CC = 1.0, DELTS, YP;
    if (mar) {
        DELTAP = YC[zs];
        UTAU2 = ws_bisect_warp(U_ave, DELTAP, g.re, 1.0, 0.000001);
        const double YPLUSML = DELTAP * UTAU2 * g.re, YPLUS1 = g.dy[1] / 2.0 * UTAU2 * g.re;
        const double lg = log(YPLUS1 / YPLUSML);
        CC = __dadd_rn(1.0, __dmul_rn(0.05, __dmul_rn(lg, lg)));
        DELTS = DELTAP / tan16;
        YP = wall == 0 ? DELTAP : YC[g.n2m - zs + 1];
    } else {
        DELTAP = (wall == 0 ? g.dy[1] : g.dy[g.n2m]) / 2.0;
        UTAU2 = ws_bisect_warp(U_ave, DELTAP, g.re, 0.000001, 0.2);
        DELTS = 0.0;
        YP = wall == 0 ? g.h[1] : YC[g.n2m];
    }
    if ((threadIdx.x & 31) != 0) return;
    const double TAUW1 = UTAU2 * UTAU2;
    // YP after each INDEX_IJK call until a call leaves it unchanged
    int nfix = 0;
    for (;; ++nfix) {
        double yn = YP;
        if (yn < YC[1]) yn = nudge_up(yn);
        if (yn > YC[g.n2m]) yn = nudge_dn(yn);
        const bool moved = yn != YP;
        YP = yn;
        tab[nfix] = YP;
        if (!moved || nfix == WS_TABN - 1) break;
    }
    par[0] = U_ave;
    par[1] = UTAU2;
    par[2] = TAUW1;
    par[3] = CC;
    par[4] = DELTS;
    par[5] = (double)nfix;
    if (wall == 0) {
        a.scal[SCAL_WSMC] = TAUW1;
        a.scal[SCAL_WALLERR] = 0.0;
    }
}

// TAUW and TAUB of one wall point per thread (2 N1M N3M threads: wall-major)
template <typename R>
__global__ void __launch_bounds__(TPB) k_wall_shift(StepArgs<R> a, LesArgs<R> l, const double *ws, WsMesh m) {
    const Geo g = a.g;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * g.np) return;
    const int wall = t / g.np, e = t - wall * g.np;
    const int I = e % g.n1m + 1, K = e / g.n1m + 1;
    const double *par = ws + WsMesh::off_par(g) + WS_NPAR * wall;
    const double *tab = ws + WsMesh::off_tab(g) + (size_t)WS_TABN * wall;
    const double U_ave = par[0], UTAU2 = par[1], TAUW1 = par[2], CC = par[3], DELTS = par[4];
    const int nfix = (int)par[5];
    const bool mar = l.wmodel == 3;
    const long long call = 2LL * ((long long)(I - 1) * g.n3m + (K - 1));   // I outer, K inner
    auto point = [&](double XP, double ZP, long long c, int C) -> double {
        if (XP > g.alx) XP = __dsub_rn(XP, g.alx);
        if (XP < m.XC[1]) XP = nudge_up(XP);
        if (XP > m.XC[g.n1m]) XP = nudge_dn(XP);
        if (ZP < m.ZC[1]) ZP = nudge_up(ZP);
        if (ZP > m.ZC[g.n3m]) ZP = nudge_dn(ZP);
        const double YP = tab[c < nfix ? c : nfix];
        const int IP = ws_cell(XP, m.XG, g.n1m, m.rx), KP = ws_cell(ZP, m.ZG, g.n3m, m.rz);
        const int JP = ws_ycell(YP, m.Y, g.n2m);
        if (IP < 0 || JP < 0 || KP < 0) return __longlong_as_double(0x7ff8000000000000LL);   // NaN
        return ws_interp(a, m, XP, YP, ZP, IP, JP, KP, C);
    };
    const double F = point(__dadd_rn(m.XG[I], DELTS), m.ZC[K], call, mar ? 1 : 2);
    const double TW = mar ? __dadd_rn(TAUW1, __dmul_rn(__dmul_rn(__dmul_rn(CC, 0.1), UTAU2), __dsub_rn(F, U_ave)))
                          : __dadd_rn(TAUW1, __dmul_rn(__dmul_rn(0.1, UTAU2), F));
    const double WF = point(__dadd_rn(m.XC[I], DELTS), m.ZG[K], call + 1, 3);
    l.tauw[wall * g.np + e] = TW;
    l.taub[wall * g.np + e] = __dmul_rn(TAUW1, WF) / U_ave;
}

template <typename R>
__global__ void k_wall_sum(StepArgs<R> a, LesArgs<R> l, int nb) {
    __shared__ double s[256], b[256];
    double x = 0.0, y = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        x += l.wpart[q];
        y += l.wpart[nb + q];
    }
    s[threadIdx.x] = x;
    b[threadIdx.x] = y;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s[threadIdx.x] += s[threadIdx.x + w];
            b[threadIdx.x] += b[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.scal[SCAL_WSMC] = s[0] / (double)a.g.np;
        a.scal[SCAL_WALLERR] = b[0] > 0.0 ? 1.0 : 0.0;
        if (l.wmodel == 4) {   // WERNER zeroes WSM(2), WSM(3) (compact3d.f:4938-4940)
            a.scal[SCAL_WSMC + 1] = 0.0;
            a.scal[SCAL_WSMC + 2] = 0.0;
        }
    }
}

// ---------------------------------------------------------------------------------
// les_x1: rows (j, k), j = 1..N2M.  nux = Ix(nu); HH1 -= 2 Dx(nu Dx u); dvdx = Dx(v)
// at the x faces of the v faces J >= 2; dwdx = Dx(w) at the x faces.
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_les_x1(StepArgs<R> a, LesArgs<R> l) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    S *sbS = reinterpret_cast<S *>(smem_raw + wid * stage_bytes(g.n1m, C));
    R *sbR = reinterpret_cast<R *>(sbS);
    const int nrows = g.n2m * g.n3m;
    const R f24 = a.f24x, four = (R)4.0, two = (R)2.0;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k);
        R nv[C], d[C];
        srow_load(nv, l.nu + o, sbR, lane, P);
        {
            R pv = sprev(nv[C - 1], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = four * (nv[t] + (t == 0 ? pv : nv[t - 1]));
            xsolve(d, lane, P, a.c6x);
            srow_store(l.nux + o, d, sbR, lane, P);
        }
        {
            S uc[C];
            srow_load(uc, a.u + o, sbS, lane, P);
            S nx = snext(uc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = f24 * ST::d(t == C - 1 ? nx : uc[t + 1], uc[t]);
            xsolve(d, lane, P, a.c22x);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = nv[t] * d[t];
            R pv = sprev(d[C - 1], lane, P);
            R e[C];
#pragma unroll
            for (int t = 0; t < C; ++t) e[t] = f24 * (d[t] - (t == 0 ? pv : d[t - 1]));
            xsolve(e, lane, P, a.c22x);
            R h[C];
            srow_load(h, a.hh[0] + o, sbR, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) h[t] = h[t] - two * e[t];
            srow_store(a.hh[0] + o, h, sbR, lane, P);
        }
        if (j >= 2) {
            S vc[C];
            srow_load(vc, a.v + o, sbS, lane, P);
            S pv = sprev(vc[C - 1], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = f24 * ST::d(vc[t], t == 0 ? pv : vc[t - 1]);
            xsolve(d, lane, P, a.c22x);
            srow_store(l.dvdx + o, d, sbR, lane, P);
        }
        {
            S wc[C];
            srow_load(wc, a.w + o, sbS, lane, P);
            S pv = sprev(wc[C - 1], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = f24 * ST::d(wc[t], t == 0 ? pv : wc[t - 1]);
            xsolve(d, lane, P, a.c22x);
            srow_store(l.dwdx + o, d, sbR, lane, P);
        }
    }
}

// ---------------------------------------------------------------------------------
// les_z1: columns (i, j), j = 1..N2M.  nuz = Iz(nu); tau13 = Iz(nux) (Dz u + dwdx);
// nuwz = nu Dz(w) at the cell centres; dvdz = Dz(v) at the z faces of the v faces J >= 2.
// ---------------------------------------------------------------------------------
template <typename R>
struct WalkLesZ1 {
    typedef typename SType<R>::S S;
    const R *NU, *NUX; const S *U, *V, *W; int n, s; R f24; bool hv;
    R num, nuxm; S um, vm, wc; int kn, kc;
    __device__ void start(int k) {
        const int kp = zprev(k, n);
        num = NU[kp * s]; nuxm = NUX[kp * s]; um = U[kp * s]; vm = hv ? V[kp * s] : S(); wc = W[k * s];
        kc = k; kn = znext(k, n);
    }
    __device__ void next(R (&d)[5]) {
        const R nuc = NU[kc * s], nuxc = NUX[kc * s];
        const S uc = U[kc * s], wp = W[kn * s];
        d[0] = (R)4.0 * (num + nuc);
        d[1] = (R)4.0 * (nuxm + nuxc);
        d[2] = f24 * St<R>::d(uc, um);
        d[3] = f24 * St<R>::d(wp, wc);
        if (hv) {
            const S vc = V[kc * s];
            d[4] = f24 * St<R>::d(vc, vm);
            vm = vc;
        } else {
            d[4] = R(0);
        }
        num = nuc; nuxm = nuxc; um = uc; wc = wp; kc = kn; kn = znext(kn, n);
    }
    __device__ static int zprev(int k, int n) { return k == 0 ? n - 1 : k - 1; }
    __device__ static int znext(int k, int n) { return k + 1 == n ? 0 : k + 1; }
};

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_les_z1(StepArgs<R> a, LesArgs<R> l) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    R out[5][L];
    const R rr[5] = {a.c6z.r, a.c6z.r, a.c22z.r, a.c22z.r, a.c22z.r};
    const R ss[5] = {a.c6z.s, a.c6z.s, a.c22z.s, a.c22z.s, a.c22z.s};
    WalkLesZ1<R> f{l.nu + o, l.nux + o, a.u + o, a.v + o, a.w + o, n, s, a.f24z, j >= 2};
    zsweep<R, L, WM<R>::M6, 5>(out, k0, n, rr, ss, f);
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const long long kk = o + (long long)(k0 + t) * s;
        l.nuz[kk] = out[0][t];
        l.t13[kk] = out[1][t] * (out[2][t] + l.dwdx[kk]);
        l.nuwz[kk] = l.nu[kk] * out[3][t];
        if (j >= 2) l.dvdz[kk] = out[4][t];
    }
}

// ---------------------------------------------------------------------------------
// les_z2: columns (i, j).  HH1 -= Dz(tau13); HH3 -= 2 Dz(nuwz) + d/dy(nu_yz (dw/dy + dv/dz));
// HH2 -= Dz(tau23) at the v faces J >= 2.
// ---------------------------------------------------------------------------------
template <typename R>
struct WalkLesZ2 {
    typedef typename SType<R>::S S;
    const R *T13, *NWZ, *NZc, *NZm, *DVZ; const S *Wc, *Wm; int n, s; R f24, rhj, hdj, hdjm; bool hv;
    R tc, nwm, t23c; int kn, kc;
    __device__ R tau23(int k) const {
        const R nyz = rhj * (hdj * NZm[k * s] + hdjm * NZc[k * s]);
        return nyz * (rhj * St<R>::d(Wc[k * s], Wm[k * s]) + DVZ[k * s]);
    }
    __device__ void start(int k) {
        tc = T13[k * s]; nwm = NWZ[(k == 0 ? n - 1 : k - 1) * s]; t23c = hv ? tau23(k) : R(0);
        kc = k; kn = (k + 1 == n) ? 0 : k + 1;
    }
    __device__ void next(R (&d)[3]) {
        const R tp = T13[kn * s], nwc = NWZ[kc * s];
        const R t23p = hv ? tau23(kn) : R(0);
        d[0] = f24 * (tp - tc);
        d[1] = f24 * (nwc - nwm);
        d[2] = f24 * (t23p - t23c);
        tc = tp; nwm = nwc; t23c = t23p; kc = kn; kn = (kn + 1 == n) ? 0 : kn + 1;
    }
};

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_les_z2(StepArgs<R> a, LesArgs<R> l) {
    typedef St<R> ST;
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0), om = fidx(g, i, j - 1, 0), op = fidx(g, i, j + 1, 0);
    const bool hv = j >= 2;
    R out[3][L];
    const R rr[3] = {a.c22z.r, a.c22z.r, a.c22z.r}, ss[3] = {a.c22z.s, a.c22z.s, a.c22z.s};
    WalkLesZ2<R> f{l.t13 + o, l.nuwz + o, l.nuz + o, l.nuz + om, l.dvdz + o, a.w + o, a.w + om,
                   n, s, a.f24z, a.m.rh[j], a.m.hdy[j], a.m.hdy[j - 1], hv};
    zsweep<R, L, WM<R>::M22, 3>(out, k0, n, rr, ss, f);
    const bool fjum = (j != 1), fjup = (j != g.n2m);
    const R half = (R)0.5, two = (R)2.0;
    const R f2 = (R)(1.0 - l.ifwall * (fjup ? 0.0 : 1.0) * (g.aly - 1.0));
    const R f1 = (R)(1.0 - l.ifwall * (fjum ? 0.0 : 1.0));
    const R rdy = a.m.rdy[j], rh = a.m.rh[j], rhp = a.m.rh[j + 1];
    const R hdj = a.m.hdy[j], hdjm = a.m.hdy[j - 1], hdjp = a.m.hdy[j + 1];
    const long long w0 = fidx(g, i, 0, 0), wt = fidx(g, i, g.n2, 0);
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int k = k0 + t, km = (k == 0) ? n - 1 : k - 1;
        const long long kk = (long long)k * s, kkm = (long long)km * s;
        const R sj2 = fjup ? rhp * (hdj * l.nuz[op + kk] + hdjp * l.nuz[o + kk])
                           : half * (l.nu[wt + kk] + l.nu[wt + kkm]);
        const R sj1 = fjum ? rh * (hdjm * l.nuz[o + kk] + hdj * l.nuz[om + kk])
                           : half * (l.nu[w0 + kk] + l.nu[w0 + kkm]);
        const R ww22 = rhp * ST::d(a.w[op + kk], a.w[o + kk]);
        const R ww11 = rh * ST::d(a.w[o + kk], a.w[om + kk]);
        const R yflux = rdy * ((f2 * sj2) * (ww22 + l.dvdz[op + kk]) - (f1 * sj1) * (ww11 + l.dvdz[o + kk]));
        R *H1 = a.hh[0] + o + kk, *H2 = a.hh[1] + o + kk, *H3 = a.hh[2] + o + kk;
        *H1 = *H1 - out[0][t];
        *H3 = *H3 - two * out[1][t] - yflux;
        if (hv) *H2 = *H2 - out[2][t];
    }
}

// ---------------------------------------------------------------------------------
// les_x2: rows (j, k).  HH3 -= Dx(tau13); HH2 -= Dx(tau12) + 2 d/dy(nu dv/dy) (J >= 2);
// HH1 -= d/dy(nu_xy (du/dy + dv/dx)); the wall-stress terms of RUH1, RUH3 (IFWALL).
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_les_x2(StepArgs<R> a, LesArgs<R> l) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    S *sbS = reinterpret_cast<S *>(smem_raw + wid * stage_bytes(g.n1m, C));
    R *sbR = reinterpret_cast<R *>(sbS);
    const int nrows = g.n2m * g.n3m;
    const R f24 = a.f24x, half = (R)0.5, two = (R)2.0;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), om = fidx(g, 0, j - 1, k), op = fidx(g, 0, j + 1, k);
        const bool fjum = (j != 1), fjup = (j != g.n2m);
        R d[C];
        {   // HH3 -= Dx(tau13)
            R tc[C];
            srow_load(tc, l.t13 + o, sbR, lane, P);
            R nx = snext(tc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = f24 * ((t == C - 1 ? nx : tc[t + 1]) - tc[t]);
            xsolve(d, lane, P, a.c22x);
            R h[C];
            srow_load(h, a.hh[2] + o, sbR, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) h[t] = h[t] - d[t];
            srow_store(a.hh[2] + o, h, sbR, lane, P);
        }
        S uc[C], um[C];
        srow_load(uc, a.u + o, sbS, lane, P);
        srow_load(um, a.u + om, sbS, lane, P);
        R nxc[C], nxm[C], dvc[C];
        srow_load(nxc, l.nux + o, sbR, lane, P);
        if (j >= 2) {
            srow_load(nxm, l.nux + om, sbR, lane, P);
            srow_load(dvc, l.dvdx + o, sbR, lane, P);
        } else {
#pragma unroll
            for (int t = 0; t < C; ++t) { nxm[t] = R(0); dvc[t] = R(0); }
        }
        if (j >= 2) {   // HH2 -= Dx(tau12) + 2 d/dy(nu dv/dy)
            const R rh = a.m.rh[j], hd = a.m.hdy[j], hdm = a.m.hdy[j - 1];
            R tau[C];
#pragma unroll
            for (int t = 0; t < C; ++t) tau[t] = (rh * (hdm * nxc[t] + hd * nxm[t])) * (rh * ST::d(uc[t], um[t]) + dvc[t]);
            R nx = snext(tau[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = f24 * ((t == C - 1 ? nx : tau[t + 1]) - tau[t]);
            xsolve(d, lane, P, a.c22x);
            S vc[C], vm[C], vp[C];
            srow_load(vc, a.v + o, sbS, lane, P);
            srow_load(vm, a.v + om, sbS, lane, P);
            srow_load(vp, a.v + op, sbS, lane, P);
            R nc[C], nm[C], h[C];
            srow_load(nc, l.nu + o, sbR, lane, P);
            srow_load(nm, l.nu + om, sbR, lane, P);
            srow_load(h, a.hh[1] + o, sbR, lane, P);
            const R rdy = a.m.rdy[j], rdym = a.m.rdy[j - 1];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                const R vis22 = rh * (nc[t] * (rdy * ST::d(vp[t], vc[t])) - nm[t] * (rdym * ST::d(vc[t], vm[t])));
                h[t] = h[t] - d[t] - two * vis22;
            }
            srow_store(a.hh[1] + o, h, sbR, lane, P);
        }
        {   // HH1 -= d/dy(nu_xy (du/dy + dv/dx))
            S up[C];
            srow_load(up, a.u + op, sbS, lane, P);
            R nxp[C], dvp[C], nw[C];
            if (fjup) {
                srow_load(nxp, l.nux + op, sbR, lane, P);
                srow_load(dvp, l.dvdx + op, sbR, lane, P);
            } else {
#pragma unroll
                for (int t = 0; t < C; ++t) { nxp[t] = R(0); dvp[t] = R(0); }
            }
            // wall viscosity (x average of the ghost plane) where the face is a wall
            if (!fjup || !fjum) srow_load(nw, l.nu + (fjup ? fidx(g, 0, 0, k) : fidx(g, 0, g.n2, k)), sbR, lane, P);
            R pw = sprev((!fjup || !fjum) ? nw[C - 1] : R(0), lane, P);
            const R rh = a.m.rh[j], rhp = a.m.rh[j + 1], hd = a.m.hdy[j], hdm = a.m.hdy[j - 1], hdp = a.m.hdy[j + 1];
            const R f2 = (R)(1.0 - l.ifwall * (fjup ? 0.0 : 1.0) * (g.aly - 1.0));
            const R f1 = (R)(1.0 - l.ifwall * (fjum ? 0.0 : 1.0));
            const R rdy = a.m.rdy[j];
            R h[C];
            srow_load(h, a.hh[0] + o, sbR, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                const R wv = (!fjup || !fjum) ? half * (nw[t] + (t == 0 ? pw : nw[t - 1])) : R(0);
                const R sj2 = fjup ? rhp * (hd * nxp[t] + hdp * nxc[t]) : wv;
                const R sj1 = fjum ? rh * (hdm * nxc[t] + hd * nxm[t]) : wv;
                const R uu22 = rhp * ST::d(up[t], uc[t]);
                const R uu11 = rh * ST::d(uc[t], um[t]);
                h[t] = h[t] - rdy * ((f2 * sj2) * (uu22 + dvp[t]) - (f1 * sj1) * (uu11 + dvc[t]));
            }
            srow_store(a.hh[0] + o, h, sbR, lane, P);
        }
        if (l.ifwall && (!fjum || !fjup)) {   // wall-stress terms (IFWALL)
            const double rdy1 = 1.0 / g.dy[1], rdyt = 1.0 / g.dy[g.n2m];
            R r0[C], r2[C];
            srow_load(r0, a.r[0] + o, sbR, lane, P);
            srow_load(r2, a.r[2] + o, sbR, lane, P);
            if (lane < P) {
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    const int i = lane * C + t;
                    const long long e0 = (long long)k * g.n1m + i, e1 = e0 + g.np;
                    double b1 = 0.0, b3 = 0.0;
                    if (!fjum) { b1 += -l.tauw[e0] * rdy1; b3 += -l.taub[e0] * rdy1; }
                    if (!fjup) { b1 += -l.tauw[e1] * rdyt * (g.aly - 1.0); b3 += -l.taub[e1] * rdyt * (g.aly - 1.0); }
                    r0[t] = r0[t] + (R)b1;
                    r2[t] = r2[t] + (R)b3;
                }
            }
            srow_store(a.r[0] + o, r0, sbR, lane, P);
            srow_store(a.r[2] + o, r2, sbR, lane, P);
        }
    }
}

// ---------------------------------------------------------------------------------
// Host-side launch of the LES stages of one step.  stage 0: WALLSS (WMODEL = 0), the SGS
// model and the wall model (before BCOND); stage 1: the SGS fluxes (after zB).
// ---------------------------------------------------------------------------------
template <typename R, int C>
static void launch_les_x(c3d_channel *ch, StepArgs<R> &a, LesArgs<R> &l, int which, int *nl) {
    const size_t sb = (TPB / 32) * stage_bytes(ch->g.n1m, C);
    const int grid = nblk((long long)ch->g.n2m * ch->g.n3m, TPB / 32);
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    if (which == 0) {
        cudaFuncSetAttribute(k_les_x1<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
        k_les_x1<R, C><<<grid, TPB, sb, ch->stream>>>(a, l);
        mark(ch, nl, "les_x1", N * (24 + 6 * Rb));
    } else {
        cudaFuncSetAttribute(k_les_x2<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
        k_les_x2<R, C><<<grid, TPB, sb, ch->stream>>>(a, l);
        mark(ch, nl, "les_x2", N * (16 + 14 * Rb));
    }
}

void launch_wall_shift_init(c3d_channel *ch) {
    k_wall_shift_init<<<1, 256, 0, ch->stream>>>(ch->g, ch->wshift);
}

size_t wall_shift_doubles(const Geo &g) { return WsMesh::size(g); }

template <typename R>
int launch_les(c3d_channel *ch, StepArgs<R> &a, LesArgs<R> &l, int stage, int *nl) {
    cudaStream_t st = ch->stream;
    const Geo &g = ch->g;
    const double N = (double)g.n1m * g.n2m * g.n3m, Rb = sizeof(R);
    if (stage == 0) {
        if (g.n2m < 1) return C3D_EINVAL;
        if (ch->wjoin_pending) {   // a step that stopped between the fork and the join
            CK_RC(cudaStreamWaitEvent(st, ch->wjoin, 0));
            ch->wjoin_pending = 0;
        }
        if (ch->sjoin_pending) {
            CK_RC(cudaStreamWaitEvent(st, ch->sjoin, 0));
            ch->sjoin_pending = 0;
        }
        if (ch->files != 0 && ch->wmodel == 0) {
            k_les_wallss<R><<<1, 256, 0, st>>>(a);
            mark(ch, nl, "les_wallss", 64.0 * g.np);
        }
        // The wall model reads the state and WSM and writes TAUW, TAUB and WSM(1); the SGS
        // model reads WSM (SGSCS's coefficient) and the state, so it runs on a side stream
        // forked after k_sgs_coef and joined before k_les_x2, the first reader of TAUW/TAUB.
        // Of the planes BCOND writes (0, N2 and V at J = 1) the models read only V(J=1)
        // (PIOMELLI), from a copy taken on the main stream before the fork.
        const bool fork = ch->wside && !ch->prof_on && ch->files != 0 && ch->wmodel != 0;
        const cudaStream_t wst = fork ? ch->wside : st;
        auto wall_model = [&]() -> int {
            if (ch->files != 0 && ch->wmodel == 5) {
                k_wall_shift_v1<R><<<nblk(g.np), TPB, 0, st>>>(a, ch->wshift);
                *nl += 1;
            }
            if (fork) {
                CK_RC(cudaEventRecord(ch->wfork, st));
                CK_RC(cudaStreamWaitEvent(wst, ch->wfork, 0));
            }
            if (ch->files != 0 && ch->wmodel == 1 && ch->wrough) {
                const int nb = nblk(g.np);
                k_wall_rough<R><<<nb, TPB, 0, wst>>>(a, l, ch->wklog);
                k_wall_sum<R><<<1, 256, 0, wst>>>(a, l, nb);
                mark(ch, nl, "wall", 24.0 * g.np);
            } else if (ch->files != 0 && ch->wmodel == 1) {
                const int nb = nblk(g.np);
                k_wall<R><<<nb, TPB, 0, wst>>>(a, l);
                k_wall_sum<R><<<1, 256, 0, wst>>>(a, l, nb);
                mark(ch, nl, "wall", 32.0 * g.np);
            } else if (ch->files != 0 && ch->wmodel == 4) {
                const int nb = nblk(g.np);
                k_wall_werner<R><<<nb, TPB, 0, wst>>>(a, l, ch->wtaue);
                k_wall_sum<R><<<1, 256, 0, wst>>>(a, l, nb);
                k_wall_werner_avg<R><<<nb, TPB, 0, wst>>>(a, l, ch->wtaue);
                *nl += 2;
                mark(ch, nl, "wall", 96.0 * g.np);
            } else if (ch->files != 0 && ch->wmodel == 2) {
                int rc2 = launch_iwm_t<R>(ch, a, wst, l.tauw, l.taub);
                if (rc2) return rc2;
                mark(ch, nl, "wall", 64.0 * g.np);
            } else if (ch->files != 0 && (ch->wmodel == 3 || ch->wmodel == 5)) {
                const int nb = nblk(g.np);
                const int jd = ch->wmodel == 3 ? ch->wzs : 1, ju = ch->wmodel == 3 ? g.n2m - ch->wzs + 1 : g.n2m;
                k_wall_shift_mean<R><<<nb, TPB, 0, wst>>>(a, l, jd, ju);
                k_wall_shift_fin<R><<<1, 256, 0, wst>>>(a, l, nb, ch->wshift, ch->wzs, ch->wtan16);
                k_wall_shift<R><<<nblk(2LL * g.np), TPB, 0, wst>>>(a, l, ch->wshift, WsMesh::of(g, ch->wshift));
                *nl += 2;
                // per wall point: u on two planes, eight corners of two components, two stresses
                const double Sb = sizeof(typename StepArgs<R>::S);
                mark(ch, nl, "wall", (2.0 * Sb + 2 * (16 * Sb + 16)) * g.np);
            }
            if (fork) CK_RC(cudaEventRecord(ch->wjoin, wst));
            return 0;
        };
        int rc = 0;
        if (ch->files == 2) {
            k_sgs_coef<R><<<1, 128, 0, st>>>(a, l);
            if ((rc = wall_model())) return rc;
            k_sgs_cs<R><<<nblk((long long)g.n2m * g.np), TPB, 0, st>>>(a, l);
            mark(ch, nl, "sgs_cs", N * (6 * 8 + Rb));
        } else if (ch->files == 1) {
            if ((rc = wall_model())) return rc;
            k_sgs_raw<R><<<nblk((long long)g.n2m * g.np), TPB, 0, st>>>(a, l);
            mark(ch, nl, "sgs_raw", N * (6 * 8 + 22 * Rb));
            k_sgs_dyn<R><<<g.n2m, 256, 0, st>>>(a, l);
            mark(ch, nl, "sgs_dyn", N * 23 * Rb);
        } else if (ch->files == 3) {
            if ((rc = wall_model())) return rc;
            k_sgs_raw<R><<<nblk((long long)g.n2m * g.np), TPB, 0, st>>>(a, l);
            mark(ch, nl, "sgs_raw", N * (6 * 8 + 22 * Rb));
            k_sgs_sd_sums<R><<<dim3((g.n1m + SD_TX - 1) / SD_TX, g.n3m / SD_TZ, g.n2m), SD_THREADS, 0, st>>>(a, l, ch->sdpart);
            mark(ch, nl, "sgs_sd_sums", N * 21 * Rb);
            const bool sfork = ch->sside && !ch->prof_on;
            const cudaStream_t sst = sfork ? ch->sside : st;
            if (sfork) {
                CK_RC(cudaEventRecord(ch->sfork, st));
                CK_RC(cudaStreamWaitEvent(sst, ch->sfork, 0));
            }
            k_sgs_sd_coef<R><<<g.n2m, 32, 0, sst>>>(a, l, ch->sdpart, ch->sdnt, ch->sdbeta);
            k_sgs_apply<R><<<nblk((long long)g.n2m * g.np), TPB, 0, sst>>>(a, l);
            if (sfork) {
                CK_RC(cudaEventRecord(ch->sjoin, sst));
                ch->sjoin_pending = 1;
            }
            *nl += 1;
            mark(ch, nl, "sgs_sd_apply", N * 2 * Rb);
        }
        if (fork) ch->wjoin_pending = 1;
        return 0;
    }
    if (ch->sjoin_pending) {   // nu of this step's SGSSD
        CK_RC(cudaStreamWaitEvent(st, ch->sjoin, 0));
        ch->sjoin_pending = 0;
    }
    switch ((g.n1m + 31) / 32) {
        case 1: launch_les_x<R, 1>(ch, a, l, 0, nl); break;
        case 2: launch_les_x<R, 2>(ch, a, l, 0, nl); break;
        case 3: launch_les_x<R, 3>(ch, a, l, 0, nl); break;
        case 4: launch_les_x<R, 4>(ch, a, l, 0, nl); break;
        case 6: launch_les_x<R, 6>(ch, a, l, 0, nl); break;
        case 8: launch_les_x<R, 8>(ch, a, l, 0, nl); break;
        case 12: launch_les_x<R, 12>(ch, a, l, 0, nl); break;
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
    const long long nz = (long long)g.n2m * (g.n3m / ZL) * g.n1m;
    k_les_z1<R, ZL><<<nblk(nz), TPB, 0, st>>>(a, l);
    mark(ch, nl, "les_z1", N * (24 + 7 * Rb));
    k_les_z2<R, ZL><<<nblk(nz), TPB, 0, st>>>(a, l);
    mark(ch, nl, "les_z2", N * (16 + 12 * Rb));
    if (ch->wjoin_pending) {   // TAUW/TAUB of this step's wall model
        CK_RC(cudaStreamWaitEvent(st, ch->wjoin, 0));
        ch->wjoin_pending = 0;
    }
    switch ((g.n1m + 31) / 32) {
        case 1: launch_les_x<R, 1>(ch, a, l, 1, nl); break;
        case 2: launch_les_x<R, 2>(ch, a, l, 1, nl); break;
        case 3: launch_les_x<R, 3>(ch, a, l, 1, nl); break;
        case 4: launch_les_x<R, 4>(ch, a, l, 1, nl); break;
        case 6: launch_les_x<R, 6>(ch, a, l, 1, nl); break;
        case 8: launch_les_x<R, 8>(ch, a, l, 1, nl); break;
        case 12: launch_les_x<R, 12>(ch, a, l, 1, nl); break;
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
    return 0;
}

template int launch_les<double>(c3d_channel *, StepArgs<double> &, LesArgs<double> &, int, int *);
template int launch_les<float>(c3d_channel *, StepArgs<float> &, LesArgs<float> &, int, int *);

}  // namespace c3d

namespace c3d {

// ---------------------------------------------------------------------------------
// Lagrangian particles (compact3d.f:11882-12470, 2029-2075), FP64, one thread per
// particle: CALC_UX_4RK's step with FORCE_PAR's drag and gravity and INDEX_IJK /
// INTERPOLAT of the three components at every stage, the periodic shifts by DIAM_P and
// the explicit Euler step from the start when a stage leaves the channel; BC_PAR's
// periodic shifts and top-wall reflection, a bottom-wall impact flagged (the reference's
// SPLASH draws from RAN2 seeded by CPU_TIME); SOURCE_PAR's two-way coupling terms,
// deposited with FP64 atomics.  The reference's time loop has GET_PAR and SOURCE_PAR
// commented out (compact3d.f:128, 1026); these run when the driver calls them.
// ---------------------------------------------------------------------------------
struct ParC {
    double D, TAU, MASS, HHH;
};

// INDEX_IJK with its nudges (the coordinates change, as the reference's arguments do)
__device__ __forceinline__ bool ws_locate(const Geo &g, const WsMesh &m, double &XP, double &YP, double &ZP, int &IP,
                                          int &JP, int &KP) {
    if (XP < m.XC[1]) XP = nudge_up(XP);
    if (XP > m.XC[g.n1m]) XP = nudge_dn(XP);
    if (YP < m.YC[1]) YP = nudge_up(YP);
    if (YP > m.YC[g.n2m]) YP = nudge_dn(YP);
    if (ZP < m.ZC[1]) ZP = nudge_up(ZP);
    if (ZP > m.ZC[g.n3m]) ZP = nudge_dn(ZP);
    IP = ws_cell(XP, m.XG, g.n1m, m.rx);
    JP = ws_ycell(YP, m.Y, g.n2m);
    KP = ws_cell(ZP, m.ZG, g.n3m, m.rz);
    return IP >= 0 && JP >= 0 && KP >= 0;
}

template <typename R>
__device__ void par_fluid(const StepArgs<R> &a, const WsMesh &m, double XP, double YP, double ZP, double &UF,
                          double &VF, double &WF) {
    int IP, JP, KP;
    if (!ws_locate(a.g, m, XP, YP, ZP, IP, JP, KP)) {
        UF = VF = WF = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    UF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 1);
    VF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 2);
    WF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 3);
}

// FORCE_PAR (compact3d.f:12320-12350): Clift-Gauvin drag and gravity
__device__ __forceinline__ void force_par(double re, const ParC &c, double UP, double VP, double WP, double UF,
                                          double VF, double WF, double &QU, double &QV, double &QW) {
    const double VISCOS = 0.000015;
    const double REP = sqrt((UF - UP) * (UF - UP) + (VF - VP) * (VF - VP) + (WF - WP) * (WF - WP)) * c.D * re;
    const double FCOR = 1. + 0.15 * pow(REP, 0.687) + 0.0175 * pow(1. + 42500 * pow(REP, -1.16), -1.0);
    QU = FCOR * (UF - UP) / c.TAU;
    const double t = VISCOS * re / c.HHH;
    QV = FCOR * (VF - VP) / c.TAU + (-9.8 / (t * t));
    QW = FCOR * (WF - WP) / c.TAU;
}

template <typename R>
__global__ void __launch_bounds__(TPB) k_par_advance(StepArgs<R> a, WsMesh m, ParC c, double *par, int n, double dt,
                                                     int *impact) {
    const Geo g = a.g;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    double *P = par + 6 * (size_t)q;
    const double D = c.D, ALX = g.alx, ALY = g.aly, ALZ = g.alz;
    double QXRK = 0., QYRK = 0., QZRK = 0., QURK = 0., QVRK = 0., QWRK = 0.;
    double XP = P[0], YP = P[1], ZP = P[2], UP = P[3], VP = P[4], WP = P[5], UF, VF, WF, QU, QV, QW;
    bool euler = YP < 0.5 * D || YP > ALY - 0.5 * D;
    const double cs[3] = {0.5, 0.5, 1.0}, wt[4] = {1.0, 2.0, 2.0, 1.0};
    for (int stg = 0; stg < 4 && !euler; ++stg) {
        if (XP > (ALX - 0.5 * D)) XP = 1.0 * D + XP - ALX;
        if (XP < (0.5 * D)) XP = ALX - D + XP;
        if (ZP > (ALZ - 0.5 * D)) ZP = 1.0 * D + ZP - ALZ;
        if (ZP < (0.5 * D)) ZP = ALZ - D + ZP;
        par_fluid(a, m, XP, YP, ZP, UF, VF, WF);
        force_par(g.re, c, UP, VP, WP, UF, VF, WF, QU, QV, QW);
        QXRK = QXRK + wt[stg] * UP;
        QYRK = QYRK + wt[stg] * VP;
        QZRK = QZRK + wt[stg] * WP;
        QURK = QURK + wt[stg] * QU;
        QVRK = QVRK + wt[stg] * QV;
        QWRK = QWRK + wt[stg] * QW;
        if (stg == 3) break;
        XP = P[0] + cs[stg] * dt * UP;
        YP = P[1] + cs[stg] * dt * VP;
        ZP = P[2] + cs[stg] * dt * WP;
        UP = P[3] + cs[stg] * dt * QU;
        VP = P[4] + cs[stg] * dt * QV;
        WP = P[5] + cs[stg] * dt * QW;
        euler = YP < 0.5 * D || YP > ALY - 0.5 * D;
    }
    if (!euler) {
        XP = P[0] + dt * QXRK / 6.;
        YP = P[1] + dt * QYRK / 6.;
        ZP = P[2] + dt * QZRK / 6.;
        UP = P[3] + dt * QURK / 6.;
        VP = P[4] + dt * QVRK / 6.;
        WP = P[5] + dt * QWRK / 6.;
    } else {
        UP = P[3];
        VP = P[4];
        WP = P[5];
        par_fluid(a, m, P[0], P[1], P[2], UF, VF, WF);
        force_par(g.re, c, UP, VP, WP, UF, VF, WF, QU, QV, QW);
        XP = P[0] + dt * UP;
        YP = P[1] + dt * VP;
        ZP = P[2] + dt * WP;
        UP = P[3] + dt * QU;
        VP = P[4] + dt * QV;
        WP = P[5] + dt * QW;
    }
    if (XP > (ALX - 0.5 * D)) XP = 1.0 * D + XP - ALX;
    if (XP < (0.5 * D)) XP = ALX - D + XP;
    if (ZP > (ALZ - 0.5 * D)) ZP = 1.0 * D + ZP - ALZ;
    if (ZP < (0.5 * D)) ZP = ALZ - D + ZP;
    if (YP > (ALY - 0.5 * D) && VP >= 0.0) {
        VP = -VP;
        YP = 2. * ALY - D - YP;
    }
    P[0] = XP, P[1] = YP, P[2] = ZP, P[3] = UP, P[4] = VP, P[5] = WP;
    if (impact) impact[q] = (YP < (0.5 * D) && VP <= 0.0) ? 1 : 0;
}

// SOURCE_PAR: ruh[3] are Fortran (0:M1,0:M2,0:M3) arrays; h = H(1..N2) by Fortran J
template <typename R>
__global__ void __launch_bounds__(TPB) k_par_source(StepArgs<R> a, WsMesh m, ParC c, const double *par, int n,
                                                    double *r1, double *r2, double *r3) {
    const Geo g = a.g;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double *P = par + 6 * (size_t)q;
    double XP = P[0], YP = P[1], ZP = P[2], QU, QV, QW;
    int IP, JP, KP;
    if (!ws_locate(g, m, XP, YP, ZP, IP, JP, KP)) return;
    const double UF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 1);
    const double VF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 2);
    const double WF = ws_interp(a, m, XP, YP, ZP, IP, JP, KP, 3);
    force_par(g.re, c, P[3], P[4], P[5], UF, VF, WF, QU, QV, QW);
    int IPP = IP, JPP = JP, KPP = KP;
    if (XP > m.XC[IP]) IPP = IP == g.n1m ? 1 : IP + 1;
    if (YP > m.YC[JP]) JPP = JP == g.n2m ? g.n2m : JP + 1;
    if (ZP > m.ZC[KP]) KPP = KP == g.n3m ? 1 : KP + 1;
    const double QQ = 1000.0, t = g.re * 1.5 / 100000 / c.HHH, G = 9.8 / (t * t);
    const long long su1 = g.n1m + 2, su2 = (long long)(g.n1m + 2) * (g.n2 + 1);
    auto iu = [&](int i, int j, int k) { return i + su1 * j + su2 * k; };
    atomicAdd(r1 + iu(IPP, JP, KP), -(c.MASS * QQ * QU * g.dx1 * g.dx3 / g.h[JP]));
    atomicAdd(r2 + iu(IP, JPP, KP), -(c.MASS * QQ * (QV + G) * g.dx1 * g.dx3 / g.h[JPP]));
    atomicAdd(r3 + iu(IP, JP, KPP), -(c.MASS * QQ * QW * g.dx1 * g.dx3 / g.h[JP]));
}

template <typename R>
int launch_particles_t(c3d_channel *ch, StepArgs<R> &a, double *par, int n, double diam, double dens, double hhh,
                       double dt, int *impact, double *r1, double *r2, double *r3) {
    ParC c;
    const double PI = 3.141592653;
    c.D = diam / hhh;
    c.MASS = dens * PI * (c.D * c.D * c.D) / 6.;
    c.TAU = dens * (c.D * c.D) / 18. * ch->g.re;
    c.HHH = hhh;
    WsMesh m = WsMesh::of(ch->g, ch->wshift);
    m.V1 = nullptr;
    const int nb = (n + TPB - 1) / TPB;
    if (r1) k_par_source<R><<<nb, TPB, 0, ch->stream>>>(a, m, c, par, n, r1, r2, r3);
    else k_par_advance<R><<<nb, TPB, 0, ch->stream>>>(a, m, c, par, n, dt, impact);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}
template int launch_particles_t<double>(c3d_channel *, StepArgs<double> &, double *, int, double, double, double, double,
                                        int *, double *, double *, double *);
template int launch_particles_t<float>(c3d_channel *, StepArgs<float> &, double *, int, double, double, double, double,
                                       int *, double *, double *, double *);

}  // namespace c3d
