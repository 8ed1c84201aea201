// c3d_step.cu -- kernels of one GETUP call (compact3d.f:879-960) on sm_103a.
//
// Pass structure of one step (all kernels on the channel's stream):
//   bcond   BCOND (963-1001): wall planes j=0 / j=N2 of u, w; v at j=1 and j=N2.
//   xA      x rows: y-viscous terms, x-viscous compact solves (1,10,1), -dP/dx (1,22,1),
//           d(uu)/dx, d(vv)/dy, and the x-interpolants VV1, WW1 (1,6,1) with the edge
//           product E_xy = VV1 * (u at y faces)                   (RHS1/2/3 pieces)
//   zA      z columns: z-viscous solves, -dP/dz, interpolants UU3, VV3, WW3 (1,6,1) and
//           edge products E_xz = UU3*WW1, E_yz = VV3*(w at y faces), WW3^2
//   zB      z columns: d(uw)/dz, d(vw)/dz, d(ww)/dz (1,22,1)
//   xB      x rows: d(uv)/dx, d(uw)/dx (1,22,1), d(uv)/dy, d(wv)/dy, AB2 combination
//           (-3/2 HH + 1/2 HH_old) and the x factor of Crank-Nicolson (GETUH1-3)
//   ycn     y columns: wall-normal Crank-Nicolson factor, Thomas (TDMAI)
//   zC      z columns: z factor of Crank-Nicolson -> delta; UH = U + delta
//   zD      z columns: compact d(UH3)/dz / DT                      (RHSDP)
//   xC      x rows: RDP = div(UH)/DT and the real-to-complex FFT along x   (RHSDP, GETDP)
//   fftz    z columns of the half spectrum: complex FFT along z            (GETDP)
//   poisson one wall-normal Thomas solve per (kx,kz) mode (TDMAP)          (GETDP)
//   fftz    inverse
//   xD      x rows: complex-to-real FFT -> DP, compact dDP/dx, bulk-flow partial sums
//   reduce  DMPRESG, DMPRESG3 (FP64), PRESG, PRESG3                         (UPCALC)
//   zE      z columns: compact dDP/dz, u/v/w update, P += DP              (UPCALC)
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include "c3d_internal.h"

namespace c3d {

constexpr int TPB = 128;

template <typename R> struct Cx;
template <> struct Cx<double> { typedef double2 T; };
template <> struct Cx<float> { typedef float2 T; };

template <typename C2>
__device__ __forceinline__ C2 cmul(C2 a, C2 b) {
    C2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C2>
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { C2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C2>
__device__ __forceinline__ C2 csub(C2 a, C2 b) { C2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C2>
__device__ __forceinline__ C2 cconj(C2 a) { a.y = -a.y; return a; }
// multiply by (sign * i)
template <typename C2>
__device__ __forceinline__ C2 cmuli(C2 a, int sign) {
    C2 r;
    if (sign < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
    return r;
}

template <typename C2> __device__ __forceinline__ const C2 *twsel(const FftPlan &p);
template <> __device__ __forceinline__ const double2 *twsel<double2>(const FftPlan &p) { return p.tw64; }
template <> __device__ __forceinline__ const float2 *twsel<float2>(const FftPlan &p) { return p.tw32; }

// Radix-p butterfly X_s = sum_r v_r exp(sign 2 pi i r s / p), p in {2,3,4}.
template <typename C2>
__device__ __forceinline__ void dftp(C2 (&v)[4], int p, int sign) {
    typedef decltype(v[0].x) T;
    if (p == 4) {
        C2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        C2 t2 = cadd(v[1], v[3]), t3 = cmuli(csub(v[1], v[3]), sign);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else if (p == 2) {
        C2 a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    } else {
        const T h = (T)0.8660254037844386467637;  // sqrt(3)/2
        C2 t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
        C2 a;
        a.x = v[0].x - (T)0.5 * t.x;
        a.y = v[0].y - (T)0.5 * t.y;
        C2 b = cmuli(u, sign);
        b.x *= h;
        b.y *= h;
        v[0] = cadd(v[0], t);
        v[1] = cadd(a, b);
        v[2] = csub(a, b);
    }
}

// Stockham FFT of `lines` sequences of length pl.n stored at buf[q*es + l*ls]; the
// threads tid..nthr cooperate; `sync` is __syncwarp or __syncthreads.  Returns the
// buffer holding the result (a or b).
template <typename C2, bool BLOCK>
__device__ C2 *fft_smem(C2 *a, C2 *b, const FftPlan &pl, int lines, int es, int ls, int sign,
                        int tid, int nthr) {
    const int n = pl.n;
    const C2 *tw = twsel<C2>(pl);
    int Ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int p = pl.rad[s];
        const int np = n / p;
        const int tstep = n / (Ns * p);
        for (int idx = tid; idx < np * lines; idx += nthr) {
            const int l = idx % lines, jj = idx / lines;
            C2 v[4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (r < p) v[r] = a[(jj + r * np) * es + l * ls];
            const int kq = jj % Ns;
            if (Ns > 1) {
#pragma unroll
                for (int r = 1; r < 4; ++r)
                    if (r < p) {
                        C2 t = __ldg(&tw[kq * r * tstep]);
                        if (sign > 0) t.y = -t.y;
                        v[r] = cmul(v[r], t);
                    }
            }
            dftp(v, p, sign);
            const int base = (jj / Ns) * Ns * p + kq;
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (r < p) b[(base + r * Ns) * es + l * ls] = v[r];
        }
        if (BLOCK) __syncthreads(); else __syncwarp();
        C2 *t = a; a = b; b = t;
        Ns *= p;
    }
    return a;
}

// ---------------------------------------------------------------------------------
// BCOND
// ---------------------------------------------------------------------------------
__global__ void k_bcond(Geo g, double *u, double *v, double *w) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= g.np) return;
    const long long b0 = id, bt = (long long)g.n2 * g.np + id, bm = (long long)g.n2m * g.np + id;
    u[b0] = 0.0;
    v[b0] = 0.0;
    w[b0] = 0.0;
    v[(long long)g.np + id] = 0.0;         // v at J=1 (lower wall)
    u[bt] = u[bm] * (2.0 - g.aly);         // upper wall: no-slip (ALY=2) or free-slip (ALY=1)
    v[bt] = 0.0;
    w[bt] = w[bm] * (2.0 - g.aly);
}

// ---------------------------------------------------------------------------------
// x rows, pass A
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_xA(StepArgs<R> a) {
    const Geo g = a.g;
    const int lane = threadIdx.x & 31;
    const int P = g.n1m / C;
    const int nrows = g.n2m * g.n3m;
    const double RE1 = 1.0 / g.re;
    const R RE1r = (R)RE1;
    for (int row = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), om = fidx(g, 0, j - 1, k), op = fidx(g, 0, j + 1, k);
        R uy[C];
        // ---- u: R1 = visc_y + visc_x/RE - dP/dx - PRESG ; HH1 = d(uu)/dx ----
        {
            double uc[C], um[C], up[C];
            row_load(uc, a.u + o, lane, P);
            row_load(um, a.u + om, lane, P);
            row_load(up, a.u + op, lane, P);
            const double HPj = g.hp[j], HCj = g.hc[j], HMj = g.hm[j];
            R acc[C], d[C];
            {
                double pv = lane_prev(uc[C - 1], lane, P), nx = lane_next(uc[0], lane, P);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    double l = (t == 0) ? pv : uc[t - 1], rr = (t == C - 1) ? nx : uc[t + 1];
                    d[t] = (R)(12.0 * g.dx1q * ((l - 2.0 * uc[t]) + rr));
                }
                xsolve(d, lane, P, a.c10x);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    double vy = RE1 * ((HPj * up[t] - HCj * uc[t]) + HMj * um[t]);
                    acc[t] = (R)vy + RE1r * d[t];
                }
            }
            {
                double pc[C];
                row_load(pc, a.p + o, lane, P);
                double pv = lane_prev(pc[C - 1], lane, P);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    double l = (t == 0) ? pv : pc[t - 1];
                    d[t] = (R)(24.0 * g.dx1 * (pc[t] - l));
                }
                xsolve(d, lane, P, a.c22x);
                const R presg = (R)a.scal[SCAL_PRESG];
#pragma unroll
                for (int t = 0; t < C; ++t) acc[t] = acc[t] - d[t] - presg;
                row_store(a.r[0] + o, acc, lane, P);
            }
            {
                double nx = lane_next(uc[0], lane, P);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    double rr = (t == C - 1) ? nx : uc[t + 1];
                    d[t] = (R)(4.0 * (uc[t] + rr));
                }
                xsolve(d, lane, P, a.c6x);
                R sq[C];
#pragma unroll
                for (int t = 0; t < C; ++t) sq[t] = d[t] * d[t];
                R pv = lane_prev(sq[C - 1], lane, P);
                const R f = (R)(24.0 * g.dx1);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    R l = (t == 0) ? pv : sq[t - 1];
                    d[t] = f * (sq[t] - l);
                }
                xsolve(d, lane, P, a.c22x);
                row_store(a.hh[0] + o, d, lane, P);
            }
            if (j >= 2) {
                const double Hj1 = 1.0 / g.h[j], a1 = g.dy[j] / 2.0, a2 = g.dy[j - 1] / 2.0;
#pragma unroll
                for (int t = 0; t < C; ++t) uy[t] = (R)(Hj1 * (a1 * um[t] + a2 * uc[t]));
            }
        }
        // ---- v (faces J=2..N2M): R2, HH2 = d(vv)/dy, E_xy ----
        if (j >= 2) {
            double vc[C], vm[C], vp[C], pc[C], pm[C];
            row_load(vc, a.v + o, lane, P);
            row_load(vm, a.v + om, lane, P);
            row_load(vp, a.v + op, lane, P);
            row_load(pc, a.p + o, lane, P);
            row_load(pm, a.p + om, lane, P);
            R d[C], acc[C];
            double pv = lane_prev(vc[C - 1], lane, P), nx = lane_next(vc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double l = (t == 0) ? pv : vc[t - 1], rr = (t == C - 1) ? nx : vc[t + 1];
                d[t] = (R)(12.0 * g.dx1q * ((l - 2.0 * vc[t]) + rr));
            }
            xsolve(d, lane, P, a.c10x);
            const double DYPj = g.dyp[j], DYCj = g.dyc[j], DYMj = g.dym[j], Hj = g.h[j];
            const double Hj1 = 1.0 / Hj;
            R hh[C];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double visc = RE1 * ((DYPj * vp[t] - DYCj * vc[t]) + DYMj * vm[t]);
                double pg = (pc[t] - pm[t]) / Hj;
                acc[t] = (R)(-pg + visc) + RE1r * d[t];
                double V2 = 0.5 * (vp[t] + vc[t]), V1 = 0.5 * (vc[t] + vm[t]);
                hh[t] = (R)(Hj1 * (V2 * V2 - V1 * V1));
            }
            row_store(a.r[1] + o, acc, lane, P);
            row_store(a.hh[1] + o, hh, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double l = (t == 0) ? pv : vc[t - 1];
                d[t] = (R)(4.0 * (l + vc[t]));
            }
            xsolve(d, lane, P, a.c6x);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = d[t] * uy[t];
            row_store(a.exy + o, d, lane, P);
        }
        // ---- w: R3 = visc_y + visc_x/RE ; WW1 = w at x faces ----
        {
            double wc[C], wm[C], wp[C];
            row_load(wc, a.w + o, lane, P);
            row_load(wm, a.w + om, lane, P);
            row_load(wp, a.w + op, lane, P);
            R d[C], acc[C];
            double pv = lane_prev(wc[C - 1], lane, P), nx = lane_next(wc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double l = (t == 0) ? pv : wc[t - 1], rr = (t == C - 1) ? nx : wc[t + 1];
                d[t] = (R)(12.0 * g.dx1q * ((l - 2.0 * wc[t]) + rr));
            }
            xsolve(d, lane, P, a.c10x);
            const double HPj = g.hp[j], HCj = g.hc[j], HMj = g.hm[j];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double vy = RE1 * ((HPj * wp[t] - HCj * wc[t]) + HMj * wm[t]);
                acc[t] = (R)vy + RE1r * d[t];
            }
            row_store(a.r[2] + o, acc, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double l = (t == 0) ? pv : wc[t - 1];
                d[t] = (R)(4.0 * (l + wc[t]));
            }
            xsolve(d, lane, P, a.c6x);
            row_store(a.ww1 + o, d, lane, P);
        }
    }
}

// ---------------------------------------------------------------------------------
// z columns: thread per (i, segment of L, plane j)
// ---------------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ bool zcoord(const Geo &g, int jlo, int &i, int &j, int &k0) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nseg = g.n3m / L;
    const long long tot = (long long)(g.n2m - jlo + 1) * nseg * g.n1m;
    if (tid >= tot) return false;
    i = (int)(tid % g.n1m);
    long long rest = tid / g.n1m;
    k0 = (int)(rest % nseg) * L;
    j = jlo + (int)(rest / nseg);
    return true;
}

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_zA(StepArgs<R> a) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const double RE1 = 1.0 / g.re;
    const long long o = fidx(g, i, j, 0);
    const double *U = a.u + o, *V = a.v + o, *W = a.w + o, *Pp = a.p + o;
    R out[L];
    // R1 += (1/RE) * d2u/dz2
    zseg<R, L>(out, k0, n, a.c10z, [&](int kk) {
        int km = kk == 0 ? n - 1 : kk - 1, kp = kk == n - 1 ? 0 : kk + 1;
        return (R)(12.0 * g.dx3q * ((U[km * s] - 2.0 * U[kk * s]) + U[kp * s]));
    });
    {
        R *Rp = a.r[0] + o;
#pragma unroll
        for (int t = 0; t < L; ++t) Rp[(k0 + t) * s] = Rp[(k0 + t) * s] + (R)RE1 * out[t];
    }
    // E_xz = UU3 * WW1 (u interpolated to z faces, w interpolated to x faces)
    zseg<R, L>(out, k0, n, a.c6z, [&](int kk) {
        int km = kk == 0 ? n - 1 : kk - 1;
        return (R)(4.0 * (U[km * s] + U[kk * s]));
    });
    {
        const R *Wx = a.ww1 + o;
        R *E = a.exz + o;
#pragma unroll
        for (int t = 0; t < L; ++t) E[(k0 + t) * s] = out[t] * Wx[(k0 + t) * s];
    }
    // R3: += (1/RE) d2w/dz2 - dP/dz - PRESG3
    zseg<R, L>(out, k0, n, a.c10z, [&](int kk) {
        int km = kk == 0 ? n - 1 : kk - 1, kp = kk == n - 1 ? 0 : kk + 1;
        return (R)(12.0 * g.dx3q * ((W[km * s] - 2.0 * W[kk * s]) + W[kp * s]));
    });
    {
        R pz[L];
        zseg<R, L>(pz, k0, n, a.c22z, [&](int kk) {
            int km = kk == 0 ? n - 1 : kk - 1;
            return (R)(24.0 * g.dx3 * (Pp[kk * s] - Pp[km * s]));
        });
        const R presg3 = (R)a.scal[SCAL_PRESG3];
        R *Rp = a.r[2] + o;
#pragma unroll
        for (int t = 0; t < L; ++t) Rp[(k0 + t) * s] = Rp[(k0 + t) * s] + (R)RE1 * out[t] - pz[t] - presg3;
    }
    // WW3^2 (w interpolated to cell centres in z, squared)
    zseg<R, L>(out, k0, n, a.c6z, [&](int kk) {
        int kp = kk == n - 1 ? 0 : kk + 1;
        return (R)(4.0 * (W[kk * s] + W[kp * s]));
    });
    {
        R *Q = a.wsq + o;
#pragma unroll
        for (int t = 0; t < L; ++t) Q[(k0 + t) * s] = out[t] * out[t];
    }
    if (j >= 2) {
        // R2 += (1/RE) d2v/dz2
        zseg<R, L>(out, k0, n, a.c10z, [&](int kk) {
            int km = kk == 0 ? n - 1 : kk - 1, kp = kk == n - 1 ? 0 : kk + 1;
            return (R)(12.0 * g.dx3q * ((V[km * s] - 2.0 * V[kk * s]) + V[kp * s]));
        });
        {
            R *Rp = a.r[1] + o;
#pragma unroll
            for (int t = 0; t < L; ++t) Rp[(k0 + t) * s] = Rp[(k0 + t) * s] + (R)RE1 * out[t];
        }
        // E_yz = VV3 * (w at y face J)
        zseg<R, L>(out, k0, n, a.c6z, [&](int kk) {
            int km = kk == 0 ? n - 1 : kk - 1;
            return (R)(4.0 * (V[km * s] + V[kk * s]));
        });
        const double Hj1 = 1.0 / g.h[j], a1 = g.dy[j] / 2.0, a2 = g.dy[j - 1] / 2.0;
        const double *Wm = a.w + fidx(g, i, j - 1, 0);
        R *E = a.eyz + o;
#pragma unroll
        for (int t = 0; t < L; ++t) {
            int kk = k0 + t;
            R wy = (R)(Hj1 * (a1 * Wm[kk * s] + a2 * W[kk * s]));
            E[kk * s] = out[t] * wy;
        }
    }
}

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_zB(StepArgs<R> a) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    const R f = (R)(24.0 * g.dx3);
    R out[L];
    {   // HH1 += d(uw)/dz
        const R *E = a.exz + o;
        zseg<R, L>(out, k0, n, a.c22z, [&](int kk) {
            int kp = kk == n - 1 ? 0 : kk + 1;
            return f * (E[kp * s] - E[kk * s]);
        });
        R *H = a.hh[0] + o;
#pragma unroll
        for (int t = 0; t < L; ++t) H[(k0 + t) * s] = H[(k0 + t) * s] + out[t];
    }
    {   // HH3 = d(ww)/dz
        const R *Q = a.wsq + o;
        zseg<R, L>(out, k0, n, a.c22z, [&](int kk) {
            int km = kk == 0 ? n - 1 : kk - 1;
            return f * (Q[kk * s] - Q[km * s]);
        });
        R *H = a.hh[2] + o;
#pragma unroll
        for (int t = 0; t < L; ++t) H[(k0 + t) * s] = out[t];
    }
    if (j >= 2) {   // HH2 += d(vw)/dz
        const R *E = a.eyz + o;
        zseg<R, L>(out, k0, n, a.c22z, [&](int kk) {
            int kp = kk == n - 1 ? 0 : kk + 1;
            return f * (E[kp * s] - E[kk * s]);
        });
        R *H = a.hh[1] + o;
#pragma unroll
        for (int t = 0; t < L; ++t) H[(k0 + t) * s] = H[(k0 + t) * s] + out[t];
    }
}

// ---------------------------------------------------------------------------------
// x rows, pass B: remaining convective terms, AB2, x factor of Crank-Nicolson
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_xB(StepArgs<R> a) {
    const Geo g = a.g;
    const int lane = threadIdx.x & 31;
    const int P = g.n1m / C;
    const int nrows = g.n2m * g.n3m;
    const R f = (R)(24.0 * g.dx1);
    const R dt = (R)a.dt;
    for (int row = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
        const R rdy = (R)(1.0 / g.dy[j]);
        R h1[C], h2[C], h3[C], e[C], d[C];
        row_load(h1, a.hh[0] + o, lane, P);
        row_load(h3, a.hh[2] + o, lane, P);
        // d(uv)/dy for HH1 and d(uv)/dx for HH2 from E_xy at faces j, j+1
        {
            R ep[C];
            if (j >= 2) row_load(e, a.exy + o, lane, P);
            else {
#pragma unroll
                for (int t = 0; t < C; ++t) e[t] = R(0);
            }
            if (j + 1 <= g.n2m) row_load(ep, a.exy + op, lane, P);
            else {
#pragma unroll
                for (int t = 0; t < C; ++t) ep[t] = R(0);
            }
#pragma unroll
            for (int t = 0; t < C; ++t) h1[t] = h1[t] + rdy * (ep[t] - e[t]);
        }
        if (j >= 2) {
            row_load(h2, a.hh[1] + o, lane, P);
            R nx = lane_next(e[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R rr = (t == C - 1) ? nx : e[t + 1];
                d[t] = f * (rr - e[t]);
            }
            xsolve(d, lane, P, a.c22x);
#pragma unroll
            for (int t = 0; t < C; ++t) h2[t] = h2[t] + d[t];
            row_store(a.hh[1] + o, h2, lane, P);
        }
        // d(uw)/dx for HH3 from E_xz
        {
            row_load(e, a.exz + o, lane, P);
            R nx = lane_next(e[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R rr = (t == C - 1) ? nx : e[t + 1];
                d[t] = f * (rr - e[t]);
            }
            xsolve(d, lane, P, a.c22x);
#pragma unroll
            for (int t = 0; t < C; ++t) h3[t] = h3[t] + d[t];
        }
        // d(wv)/dy for HH3 from E_yz at faces j, j+1
        {
            R ep[C];
            if (j >= 2) row_load(e, a.eyz + o, lane, P);
            else {
#pragma unroll
                for (int t = 0; t < C; ++t) e[t] = R(0);
            }
            if (j + 1 <= g.n2m) row_load(ep, a.eyz + op, lane, P);
            else {
#pragma unroll
                for (int t = 0; t < C; ++t) ep[t] = R(0);
            }
#pragma unroll
            for (int t = 0; t < C; ++t) h3[t] = h3[t] + rdy * (ep[t] - e[t]);
        }
        row_store(a.hh[0] + o, h1, lane, P);
        row_store(a.hh[2] + o, h3, lane, P);
        // AB2 + x factor of CN for each component
#pragma unroll 1
        for (int c = 0; c < 3; ++c) {
            if (c == 1 && j < 2) continue;
            const R *hc = (c == 0) ? h1 : (c == 1) ? h2 : h3;
            R rr[C], ho[C];
            row_load(rr, a.r[c] + o, lane, P);
            row_load(ho, a.ho[c] + o, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) rr[t] = (rr[t] - (R)1.5 * hc[t] + (R)0.5 * ho[t]) * dt;
            R pv = lane_prev(rr[C - 1], lane, P), nx = lane_next(rr[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R l = (t == 0) ? pv : rr[t - 1], r2 = (t == C - 1) ? nx : rr[t + 1];
                d[t] = (l + (R)10.0 * rr[t]) + r2;
            }
            xsolve(d, lane, P, a.cnx);
            row_store(a.r[c] + o, d, lane, P);
        }
    }
}

// ---------------------------------------------------------------------------------
// y columns: wall-normal factor of Crank-Nicolson (TDMAI), in place on r[c]
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TPB) k_ycn(StepArgs<R> a) {
    const Geo g = a.g;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= 3LL * g.np) return;
    const int c = (int)(tid / g.np);
    const int col = (int)(tid % g.np);
    const int js = (c == 1) ? 2 : 1;
    const int m = g.n2 + 1;
    const double *A = a.ycn + (c * 3 + 0) * m, *RB = a.ycn + (c * 3 + 1) * m, *GM = a.ycn + (c * 3 + 2) * m;
    R *X = a.r[c] + col;
    const long long s = g.np;
    R xp = X[js * s] * (R)RB[js];
    X[js * s] = xp;
    for (int j = js + 1; j <= g.n2m; ++j) {
        xp = (X[j * s] - (R)A[j] * xp) * (R)RB[j];
        X[j * s] = xp;
    }
    for (int j = g.n2m - 1; j >= js; --j) {
        xp = X[j * s] - xp * (R)GM[j];
        X[j * s] = xp;
    }
}

// ---------------------------------------------------------------------------------
// z columns: z factor of Crank-Nicolson, r[c] -> d[c] (delta)
// ---------------------------------------------------------------------------------
template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_zC(StepArgs<R> a, R *d0, R *d1, R *d2) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    R out[L];
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
        if (c == 1 && j < 2) continue;
        const R *X = a.r[c] + o;
        zseg<R, L>(out, k0, n, a.cnz, [&](int kk) {
            int km = kk == 0 ? n - 1 : kk - 1, kp = kk == n - 1 ? 0 : kk + 1;
            return (X[km * s] + (R)10.0 * X[kk * s]) + X[kp * s];
        });
        R *D = ((c == 0) ? d0 : (c == 1) ? d1 : d2) + o;
#pragma unroll
        for (int t = 0; t < L; ++t) D[(k0 + t) * s] = out[t];
    }
}

// z part of RHSDP: rdpz = compact d(UH3)/dz / DT with UH3 = W + delta3
template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_zD(StepArgs<R> a, const R *d2) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    const double *W = a.w + o;
    const R *D = d2 + o;
    R out[L];
    zseg<R, L>(out, k0, n, a.c22z, [&](int kk) {
        int kp = kk == n - 1 ? 0 : kk + 1;
        return (R)(24.0 * g.dx3 * ((W[kp * s] + (double)D[kp * s]) - (W[kk * s] + (double)D[kk * s])));
    });
    const R rdt = (R)a.dtproj;
    R *Q = a.rdpz + o;
#pragma unroll
    for (int t = 0; t < L; ++t) Q[(k0 + t) * s] = out[t] / rdt;
}

// ---------------------------------------------------------------------------------
// x rows, pass C: RDP = div(UH)/DT and its real-to-complex FFT along x
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_xC(StepArgs<R> a, const R *d0, const R *d1) {
    typedef typename Cx<R>::T C2;
    extern __shared__ unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    C2 *bufa = reinterpret_cast<C2 *>(smem_raw) + wid * 2 * M;
    C2 *bufb = bufa + M;
    R *rbuf = reinterpret_cast<R *>(bufa);
    const int nrows = g.n2m * g.n3m;
    const double dtp = a.dtproj;
    const C2 *twx = nullptr;
    if constexpr (sizeof(R) == 8) twx = reinterpret_cast<const C2 *>(a.twx64);
    else twx = reinterpret_cast<const C2 *>(a.twx32);
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
        R d[C];
        double base[C];
        {
            double uc[C];
            R dd[C];
            row_load(uc, a.u + o, lane, P);
            row_load(dd, d0 + o, lane, P);
            double uh[C];
#pragma unroll
            for (int t = 0; t < C; ++t) uh[t] = uc[t] + (double)dd[t];
            double nx = lane_next(uh[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double rr = (t == C - 1) ? nx : uh[t + 1];
                d[t] = (R)(24.0 * g.dx1 * (rr - uh[t]));
            }
            xsolve(d, lane, P, a.c22x);
        }
        {
            double vp[C], vc[C];
            R dp_[C], dc_[C];
            const bool up = (j + 1 <= g.n2m), lo = (j >= 2);
            if (up) { row_load(vp, a.v + op, lane, P); row_load(dp_, d1 + op, lane, P); }
            if (lo) { row_load(vc, a.v + o, lane, P); row_load(dc_, d1 + o, lane, P); }
            const double rdy = g.dy[j];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                double a2 = up ? vp[t] + (double)dp_[t] : 0.0;
                double a1 = lo ? vc[t] + (double)dc_[t] : 0.0;
                base[t] = ((up ? a2 : 0.0) - (lo ? a1 : 0.0)) / rdy / dtp;
            }
        }
        {
            R zc[C];
            row_load(zc, a.rdpz + o, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R v = (R)base[t] + d[t] / (R)dtp;
                d[t] = v + zc[t];
            }
        }
        // real row -> shared memory as M complex values, FFT, post-process
        if (lane < P) {
#pragma unroll
            for (int t = 0; t < C; ++t) rbuf[lane * C + t] = d[t];
        }
        __syncwarp();
        C2 *Z = fft_smem<C2, false>(bufa, bufb, a.fx, 1, 1, 0, -1, lane, 32);
        C2 *S = reinterpret_cast<C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        for (int kx = lane; kx <= M; kx += 32) {
            C2 zk = Z[kx == M ? 0 : kx], zm = cconj(Z[kx == 0 ? 0 : M - kx]);
            C2 E, O, X;
            E.x = (R)0.5 * (zk.x + zm.x);
            E.y = (R)0.5 * (zk.y + zm.y);
            C2 df = csub(zk, zm);   // O = -i * df / 2
            O.x = (R)0.5 * df.y;
            O.y = (R)-0.5 * df.x;
            X = cadd(E, cmul(twx[kx], O));
            S[kx] = X;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// z columns of the half spectrum: complex FFT along z (tile of TW kx columns per CTA)
// ---------------------------------------------------------------------------------
constexpr int TWZ = 8;
template <typename R>
__global__ void __launch_bounds__(TPB) k_fftz(StepArgs<R> a, int sign) {
    typedef typename Cx<R>::T C2;
    extern __shared__ unsigned char smem_raw[];
    const Geo g = a.g;
    const int n = g.n3m;
    C2 *A = reinterpret_cast<C2 *>(smem_raw), *B = A + n * TWZ;
    const int ntile = (g.n1h + TWZ - 1) / TWZ;
    const int plane = blockIdx.x / ntile, tile = blockIdx.x % ntile;
    const int kx0 = tile * TWZ;
    const int w = min(TWZ, g.n1h - kx0);
    C2 *S = reinterpret_cast<C2 *>(a.spec) + (long long)plane * n * g.n1h + kx0;
    for (int e = threadIdx.x; e < n * TWZ; e += blockDim.x) {
        int q = e / TWZ, l = e % TWZ;
        if (l < w) A[e] = S[(long long)q * g.n1h + l];
        else { A[e].x = 0; A[e].y = 0; }
    }
    __syncthreads();
    C2 *Z = fft_smem<C2, true>(A, B, a.fz, TWZ, TWZ, 1, sign, threadIdx.x, blockDim.x);
    for (int e = threadIdx.x; e < n * TWZ; e += blockDim.x) {
        int q = e / TWZ, l = e % TWZ;
        if (l < w) S[(long long)q * g.n1h + l] = Z[e];
    }
}

// ---------------------------------------------------------------------------------
// One wall-normal Thomas solve per (kx, kz) mode (TDMAP), factors precomputed
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TPB) k_poisson(StepArgs<R> a) {
    typedef typename Cx<R>::T C2;
    const Geo g = a.g;
    const int nm = g.n1h * g.n3m;
    const int mode = blockIdx.x * blockDim.x + threadIdx.x;
    if (mode >= nm) return;
    const int kx = mode % g.n1h, kz = mode / g.n1h;
    const bool selfc = (kx == 0 || kx == g.n1m / 2) && (kz == 0 || kz == g.n3m / 2);
    C2 *S = reinterpret_cast<C2 *>(a.spec) + mode;
    const long long s = nm;
    const double *RB = a.prb + mode, *GM = a.pgam + mode;
    // forward
    C2 v = S[0];
    double xr = (double)v.x, xi = (double)v.y;
    if (mode == 0) xr = 0.0;       // (1,1) mode: first row replaced by x_1 = 0
    double rb = RB[0];
    xr *= rb;
    xi *= rb;
    C2 o;
    o.x = (R)xr; o.y = (R)xi;
    S[0] = o;
    for (int jj = 1; jj < g.n2m; ++jj) {
        C2 q = S[jj * s];
        double am = a.pmj[jj + 1];
        rb = RB[jj * s];
        xr = ((double)q.x - am * xr) * rb;
        xi = ((double)q.y - am * xi) * rb;
        o.x = (R)xr; o.y = (R)xi;
        S[jj * s] = o;
    }
    // backward (x_j -= gam_{j+1} x_{j+1}); keep the running value in FP64
    for (int jj = g.n2m - 2; jj >= 0; --jj) {
        C2 q = S[jj * s];
        double gm = GM[(jj + 1) * s];
        double yr = (double)q.x - gm * xr;
        double yi = (double)q.y - gm * xi;
        xr = yr;
        xi = yi;
        o.x = (R)xr; o.y = selfc ? (R)0 : (R)xi;
        S[jj * s] = o;
    }
    if (selfc) {
        C2 q = S[(g.n2m - 1) * s];
        q.y = (R)0;
        S[(g.n2m - 1) * s] = q;
    }
}

// Poisson factor tables: TDMAP's recurrence for each mode (compact3d.f:9444-9459)
// with A_J = PMJ, B_J = PCJ - AK3 - AK1, C_J = PPJ; mode (0,0) has row 1 = (0,1,0).
__global__ void k_ptables(Geo g, const double *ak1, const double *ak3, const double *pmj,
                          const double *pcj, const double *ppj, double *rb, double *gam) {
    const int nm = g.n1h * g.n3m;
    const int mode = blockIdx.x * blockDim.x + threadIdx.x;
    if (mode >= nm) return;
    const int kx = mode % g.n1h, kz = mode / g.n1h;
    const int kzs = kz <= g.n3m / 2 ? kz : g.n3m - kz;
    const double lam3 = ak3[kzs], lam1 = ak1[kx];
    double B1 = pcj[1] - lam3 - lam1, C1 = ppj[1];
    if (mode == 0) { B1 = 1.0; C1 = 0.0; }
    double bet = B1;
    rb[mode] = 1.0 / bet;
    gam[mode] = 0.0;
    double cprev = C1;
    for (int J = 2; J <= g.n2m; ++J) {
        double gm = cprev / bet;
        bet = (pcj[J] - lam3 - lam1) - pmj[J] * gm;
        gam[(long long)(J - 1) * nm + mode] = gm;
        rb[(long long)(J - 1) * nm + mode] = 1.0 / bet;
        cprev = ppj[J];
    }
}

// ---------------------------------------------------------------------------------
// x rows, pass D: complex-to-real FFT -> DP, compact dDP/dx, bulk-flow partial sums
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_xD(StepArgs<R> a, const R *d0, const R *d2) {
    typedef typename Cx<R>::T C2;
    extern __shared__ unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    C2 *bufa = reinterpret_cast<C2 *>(smem_raw) + wid * 2 * (M + 1);
    C2 *bufb = bufa + (M + 1);
    const int nrows = g.n2m * g.n3m;
    const C2 *twx = nullptr;
    if constexpr (sizeof(R) == 8) twx = reinterpret_cast<const C2 *>(a.twx64);
    else twx = reinterpret_cast<const C2 *>(a.twx32);
    const double scale = 1.0 / ((double)g.n1m * (double)g.n3m);
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k);
        const C2 *S = reinterpret_cast<const C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        for (int kx = lane; kx <= M; kx += 32) bufb[kx] = S[kx];
        __syncwarp();
        for (int kx = lane; kx < M; kx += 32) {
            C2 xk = bufb[kx], xm = cconj(bufb[M - kx]);
            C2 E = cadd(xk, xm);
            C2 O = cmul(csub(xk, xm), cconj(twx[kx]));
            C2 Z;
            Z.x = E.x - O.y;
            Z.y = E.y + O.x;
            bufa[kx] = Z;
        }
        __syncwarp();
        C2 *Zr = fft_smem<C2, false>(bufa, bufb, a.fx, 1, 1, 0, +1, lane, 32);
        const R *rz = reinterpret_cast<const R *>(Zr);
        double dpv[C];
        if (lane < P) {
#pragma unroll
            for (int t = 0; t < C; ++t) dpv[t] = (double)rz[lane * C + t] * scale;
        } else {
#pragma unroll
            for (int t = 0; t < C; ++t) dpv[t] = 0.0;
        }
        __syncwarp();
        row_store(a.dp + o, dpv, lane, P);
        R d[C];
        double pv = lane_prev(dpv[C - 1], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double l = (t == 0) ? pv : dpv[t - 1];
            d[t] = (R)(24.0 * g.dx1 * (dpv[t] - l));
        }
        xsolve(d, lane, P, a.c22x);
        row_store(a.g1 + o, d, lane, P);
        // bulk-flow partial sums: sum_i delta * DY(J)/DX3/DX1 for u and w
        double s1 = 0.0, s3 = 0.0;
        {
            R q1[C], q3[C];
            row_load(q1, d0 + o, lane, P);
            row_load(q3, d2 + o, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                s1 += (double)q1[t];
                s3 += (double)q3[t];
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            s1 += __shfl_down_sync(FULL, s1, off);
            s3 += __shfl_down_sync(FULL, s3, off);
        }
        if (lane == 0) {
            const double wgt = g.dy[j] / g.dx3 / g.dx1;
            a.part[row] = s1 * wgt;
            a.part[nrows + row] = s3 * wgt;
        }
    }
}

// DMPRESG / DMPRESG3 (FP64, fixed summation order), PRESG += DMPRESG
__global__ void k_reduce(StepArgs<double> ad, StepArgs<float> af, int mixed) {
    const Geo g = mixed ? af.g : ad.g;
    double *part = mixed ? af.part : ad.part;
    double *scal = mixed ? af.scal : ad.scal;
    const double dt = mixed ? af.dtproj : ad.dtproj;
    const int bulk = mixed ? af.bulk : ad.bulk;
    const int nrows = g.n2m * g.n3m;
    __shared__ double sh1[1024], sh3[1024];
    double s1 = 0.0, s3 = 0.0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        s1 += part[r];
        s3 += part[nrows + r];
    }
    sh1[threadIdx.x] = s1;
    sh3[threadIdx.x] = s3;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh1[threadIdx.x] += sh1[threadIdx.x + w];
            sh3[threadIdx.x] += sh3[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double dm = bulk ? sh1[0] / g.vol / dt : 0.0;
        double dm3 = bulk ? sh3[0] / g.vol / dt : 0.0;
        scal[SCAL_DMPRESG] = dm;
        scal[SCAL_DMPRESG3] = dm3;
        if (bulk) {
            scal[SCAL_PRESG] = scal[SCAL_PRESG] + dm;
            scal[SCAL_PRESG3] = scal[SCAL_PRESG3] + dm3;
        }
    }
}

// ---------------------------------------------------------------------------------
// z columns, pass E: dDP/dz, velocity update, P += DP   (UPCALC)
// ---------------------------------------------------------------------------------
template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_zE(StepArgs<R> a, const R *d0, const R *d1, const R *d2, int updp) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    const double dt = a.dtproj;
    const double dm = a.scal[SCAL_DMPRESG], dm3 = a.scal[SCAL_DMPRESG3];
    const double *DP = a.dp + o;
    R out[L];
    zseg<R, L>(out, k0, n, a.c22z, [&](int kk) {
        int km = kk == 0 ? n - 1 : kk - 1;
        return (R)(24.0 * g.dx3 * (DP[kk * s] - DP[km * s]));
    });
    double *W = a.w + o, *U = a.u + o, *V = a.v + o, *Pp = a.p + o;
    const R *D0 = d0 + o, *D1 = d1 + o, *D2 = d2 + o, *G1 = a.g1 + o;
    const double *DPm = a.dp + fidx(g, i, j - 1, 0);
    const double Hj = g.h[j];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int kk = (k0 + t) * s;
        W[kk] = (W[kk] + (double)D2[kk]) - dt * (double)out[t] - dt * dm3;
        U[kk] = (U[kk] + (double)D0[kk]) - dt * (double)G1[kk] - dt * dm;
        if (j >= 2) V[kk] = (V[kk] + (double)D1[kk]) - dt * (DP[kk] - DPm[kk]) / Hj;
        if (updp) Pp[kk] = Pp[kk] + DP[kk];
    }
}

// ---------------------------------------------------------------------------------
// Diagnostics: DIVCHECK, CFL, CHKMF, WALLSS
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_diag_x(StepArgs<R> a) {
    const Geo g = a.g;
    const int lane = threadIdx.x & 31;
    const int P = g.n1m / C;
    const int nrows = g.n2m * g.n3m;
    double cmax = 0.0;
    int bad = 0;
    for (int row = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const int kp = (k + 1 == g.n3m) ? 0 : k + 1;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k), okp = fidx(g, 0, j, kp);
        double uc[C], vc[C], vp[C], wc[C], wk[C];
        row_load(uc, a.u + o, lane, P);
        row_load(vc, a.v + o, lane, P);
        row_load(vp, a.v + op, lane, P);
        row_load(wc, a.w + o, lane, P);
        row_load(wk, a.w + okp, lane, P);
        double nx = lane_next(uc[0], lane, P);
        double d[C];
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = 24.0 * g.dx1 * (rr - uc[t]);
        }
        Cyc<double> c22 = {a.c22x.r, a.c22x.s, a.c22x.m};
        if constexpr (sizeof(R) == 4) {
            const double b = 22.0;
            double r = -2.0 / (b + sqrt(b * b - 4.0));
            c22.r = r;
            c22.s = -r;
        }
        xsolve(d, lane, P, c22);
        const double rdy = g.dy[j];
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = (vp[t] - vc[t]) / rdy + d[t];
            double cf = fabs(uc[t] + rr) * 0.5 * g.dx1 + fabs(vc[t] + vp[t]) * 0.5 / rdy + fabs(wc[t] + wk[t]) * 0.5 * g.dx3;
            if (lane < P) {
                if (!isfinite(cf)) bad = 1;
                cmax = fmax(cmax, cf);
            }
        }
        row_store(a.dp + o, d, lane, P);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        cmax = fmax(cmax, __shfl_down_sync(FULL, cmax, off));
        bad |= __shfl_down_sync(FULL, bad, off);
    }
    if (lane == 0) {
        atomic_max_nonneg(&a.scal[SCAL_CFL], cmax);
        if (bad) a.scal[SCAL_NONFIN] = 1.0;
    }
}

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_diag_z(StepArgs<R> a) {
    const Geo g = a.g;
    int i, j, k0;
    double m = 0.0;
    int bad = 0;
    if (zcoord<L>(g, 1, i, j, k0)) {
        const int n = g.n3m, s = g.n1m;
        const long long o = fidx(g, i, j, 0);
        const double *W = a.w + o, *DX = a.dp + o;
        double out[L];
        Cyc<double> c22 = {(double)a.c22z.r, (double)a.c22z.s, a.c22z.m};
        if constexpr (sizeof(R) == 4) {
            const double b = 22.0;
            double r = -2.0 / (b + sqrt(b * b - 4.0));
            c22.r = r;
            c22.s = -r;
            c22.m = (int)ceil(log(1e-17) / log(fabs(r)));
        }
        zseg<double, L>(out, k0, n, c22, [&](int kk) {
            int kp = kk == n - 1 ? 0 : kk + 1;
            return 24.0 * g.dx3 * (W[kp * s] - W[kk * s]);
        });
#pragma unroll
        for (int t = 0; t < L; ++t) {
            double dv = DX[(k0 + t) * s] + out[t];
            if (!isfinite(dv)) bad = 1;
            m = fmax(m, fabs(dv));
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        m = fmax(m, __shfl_down_sync(FULL, m, off));
        bad |= __shfl_down_sync(FULL, bad, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(&a.scal[SCAL_DIVMAX], m);
        if (bad) a.scal[SCAL_NONFIN] = 1.0;
    }
}

// CHKMF and WALLSS: single block, FP64, fixed order.
__global__ void k_diag_sums(Geo g, const double *u, const double *v, const double *w, double *scal) {
    __shared__ double sh[5][256];
    double f1 = 0.0, f3 = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;
    // FLOW1: plane i=0 (I=1) summed over J,K, N1M times; FLOW3: plane k=0 (K=1), N3M times
    for (int e = threadIdx.x; e < g.n2m * g.n3m; e += blockDim.x) {
        int J = 1 + e / g.n3m, k = e % g.n3m;
        f1 += u[fidx(g, 0, J, k)] * g.dy[J] / g.dx3 / g.dx1;
    }
    for (int e = threadIdx.x; e < g.n2m * g.n1m; e += blockDim.x) {
        int J = 1 + e / g.n1m, i = e % g.n1m;
        f3 += w[fidx(g, i, J, 0)] * g.dy[J] / g.dx1 / g.dx3;
    }
    for (int e = threadIdx.x; e < g.np; e += blockDim.x) {
        int k = e / g.n1m, i = e % g.n1m;
        int ip = (i + 1 == g.n1m) ? 0 : i + 1, kp = (k + 1 == g.n3m) ? 0 : k + 1;
        double UHC = 0.5 * (u[fidx(g, i, 1, k)] + u[fidx(g, ip, 1, k)]);
        double UHW = 0.5 * (u[fidx(g, i, 0, k)] + u[fidx(g, ip, 0, k)]);
        double VHC = v[fidx(g, i, 2, k)], VHW = v[fidx(g, i, 1, k)];
        double WHC = 0.5 * (w[fidx(g, i, 1, k)] + w[fidx(g, i, 1, kp)]);
        double WHW = 0.5 * (w[fidx(g, i, 0, k)] + w[fidx(g, i, 0, kp)]);
        double WSB1 = (UHC - UHW) / (g.dy[1] * 0.5), WSB2 = (VHC - VHW) / g.dy[1], WSB3 = (WHC - WHW) / (g.dy[1] * 0.5);
        UHC = 0.5 * (u[fidx(g, i, g.n2m, k)] + u[fidx(g, ip, g.n2m, k)]);
        UHW = 0.5 * (u[fidx(g, i, g.n2, k)] + u[fidx(g, ip, g.n2, k)]);
        double WST1 = (UHC - UHW) / (g.dy[g.n2m] * 0.5);
        w1 += WSB1 + WST1 * (g.aly - 1.0);
        w2 += WSB2 + WST1 * (g.aly - 1.0);
        w3 += WSB3 + WST1 * (g.aly - 1.0);
    }
    sh[0][threadIdx.x] = f1;
    sh[1][threadIdx.x] = f3;
    sh[2][threadIdx.x] = w1;
    sh[3][threadIdx.x] = w2;
    sh[4][threadIdx.x] = w3;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 5; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scal[SCAL_FLOW1] = sh[0][0] * g.n1m / g.alx / g.alz;
        scal[SCAL_FLOW3] = sh[1][0] * g.n3m / g.alx / g.alz;
        const double nxz = 1.0 / ((double)g.n1m * g.n3m);
        scal[SCAL_WSM + 0] = sh[2][0] * nxz / g.re / g.aly;
        scal[SCAL_WSM + 1] = sh[3][0] * nxz / g.re / g.aly;
        scal[SCAL_WSM + 2] = sh[4][0] * nxz / g.re / g.aly;
    }
}

// ---------------------------------------------------------------------------------
// Fortran <-> device repacking
// ---------------------------------------------------------------------------------
// what: 0 = velocity component comp of U(0:N1,0:N2,0:N3,3) (device planes 0..N2),
//       1 = P(N1,N2,N3) (device planes 1..N2M), 2 = HH component comp (planes 1..N2M).
// Upload: one thread per device element reads its Fortran source.
template <typename T>
__global__ void k_unpack(Geo g, int what, int comp, T *dev, const double *fort) {
    const int j0 = (what == 0) ? 0 : 1, j1 = (what == 0) ? g.n2 : g.n2m;
    const long long tot = (long long)(j1 - j0 + 1) * g.np;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= tot) return;
    const int i = (int)(id % g.n1m);
    const int k = (int)((id / g.n1m) % g.n3m);
    const int j = j0 + (int)(id / g.np);
    const long long N1 = g.n1m + 1, N2 = g.n2, N3 = g.n3m + 1;
    long long f;
    if (what == 1) f = i + N1 * ((j - 1) + N2 * (long long)k);
    else f = (i + 1) + (N1 + 1) * (j + (N2 + 1) * (long long)(k + 1));
    dev[fidx(g, i, j, k)] = (T)fort[f];
    (void)N3;
}
// Download: one thread per Fortran element; periodic ghost cells (I=0, I=N1, K=0, K=N3)
// receive the periodic copies, entries outside the device planes receive 0.
template <typename T>
__global__ void k_pack(Geo g, int what, int comp, const T *dev, double *fort) {
    const long long N1 = g.n1m + 1, N2 = g.n2, N3 = g.n3m + 1;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long I, J, K;
    if (what == 1) {
        if (id >= N1 * N2 * N3) return;
        I = 1 + id % N1; J = 1 + (id / N1) % N2; K = 1 + id / (N1 * N2);
    } else {
        if (id >= (N1 + 1) * (N2 + 1) * (N3 + 1)) return;
        I = id % (N1 + 1); J = (id / (N1 + 1)) % (N2 + 1); K = id / ((N1 + 1) * (N2 + 1));
    }
    int i = (int)((I + g.n1m - 1) % g.n1m), k = (int)((K + g.n3m - 1) % g.n3m);
    const int j0 = (what == 0) ? 0 : 1, j1 = (what == 0) ? g.n2 : g.n2m;
    double v = 0.0;
    if (J >= j0 && J <= j1) v = (double)dev[fidx(g, i, (int)J, k)];
    fort[id] = v;
    (void)comp;
}

// ---------------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------------
static int nblk(long long n, int b = TPB) { return (int)((n + b - 1) / b); }

template <typename R>
static StepArgs<R> make_args(c3d_channel *ch, double dt) {
    StepArgs<R> a;
    memset(&a, 0, sizeof(a));
    a.g = ch->g;
    a.u = ch->u; a.v = ch->v; a.w = ch->w; a.p = ch->p;
    const int cur = ch->cur, old = 1 - ch->cur;
    for (int c = 0; c < 3; ++c) {
        a.hh[c] = (R *)ch->hh[cur][c];
        a.ho[c] = (const R *)ch->hh[old][c];
        a.r[c] = (R *)ch->r[c];
    }
    a.exy = (R *)ch->exy; a.exz = (R *)ch->exz; a.eyz = (R *)ch->eyz;
    a.ww1 = (R *)ch->ww1; a.wsq = (R *)ch->wsq; a.rdpz = (R *)ch->rdpz; a.g1 = (R *)ch->g1;
    a.dp = ch->dp; a.spec = ch->spec; a.scal = ch->scal; a.part = ch->part;
    a.ycn = ch->ycn; a.prb = ch->prb; a.pgam = ch->pgam; a.pmj = ch->pmj;
    a.fx = ch->fx; a.fz = ch->fz;
    const int n1h = ch->g.n1h;
    a.twx64 = ch->tw64 + (ch->g.n1m / 2) + ch->g.n3m;
    a.twx32 = ch->tw32 + (ch->g.n1m / 2) + ch->g.n3m;
    (void)n1h;
    a.dt = dt;
    a.dtproj = dt;
    a.bulk = 1;
    // compact operators
    auto mk = [&](double A, double B, bool fp32) {
        Cyc<R> c;
        double beta = B / A;
        double r = -2.0 / (beta + sqrt(beta * beta - 4.0));
        c.r = (R)r;
        c.s = (R)(-r / A);
        double tol = fp32 ? 3e-8 : 1e-17;
        c.m = (int)ceil(log(tol) / log(fabs(r)));
        return c;
    };
    const bool f32 = sizeof(R) == 4;
    a.c6x = mk(1.0, 6.0, f32); a.c10x = mk(1.0, 10.0, f32); a.c22x = mk(1.0, 22.0, f32);
    a.c6z = a.c6x; a.c10z = a.c10x; a.c22z = a.c22x;
    const double RE = ch->g.re;
    const double api = 1.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx1q * (1.0);
    const double aci = 10.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx1q * (-2.0);
    const double apk = 1.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx3q * (1.0);
    const double ack = 10.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx3q * (-2.0);
    a.cnx = mk(api, aci, f32);
    a.cnz = mk(apk, ack, f32);
    return a;
}

template <typename R, int C>
static void launch_x_all(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl) {
    const int nrows = ch->g.n2m * ch->g.n3m;
    int grid = nblk(nrows, TPB / 32);
    cudaStream_t st = ch->stream;
    const int M = ch->g.n1m / 2;
    typedef typename Cx<R>::T C2;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    switch (which) {
        case 0: k_xA<R, C><<<grid, TPB, 0, st>>>(a); mark(ch, nl, "xA", N * (32 + 7 * Rb)); return;
        case 1: k_xB<R, C><<<grid, TPB, 0, st>>>(a); mark(ch, nl, "xB", N * 18 * Rb); return;
        case 2: {
            size_t sm = (size_t)(TPB / 32) * 2 * M * sizeof(C2);
            k_xC<R, C><<<grid, TPB, sm, st>>>(a, p0, p1);
            mark(ch, nl, "xC", N * (16 + 4 * Rb));
            return;
        }
        case 3: {
            size_t sm = (size_t)(TPB / 32) * 2 * (M + 1) * sizeof(C2);
            k_xD<R, C><<<grid, TPB, sm, st>>>(a, p0, p1);
            mark(ch, nl, "xD", N * (8 + 4 * Rb));
            return;
        }
        case 4: k_diag_x<R, C><<<grid, TPB, 0, st>>>(a); mark(ch, nl, "diag_x", N * 48); return;
    }
}

template <typename R>
static int launch_x(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl) {
    switch (ch->g.n1m / 32 + (ch->g.n1m % 32 ? 1 : 0)) {
        case 1: launch_x_all<R, 1>(ch, a, which, p0, p1, nl); break;
        case 2: launch_x_all<R, 2>(ch, a, which, p0, p1, nl); break;
        case 3: launch_x_all<R, 3>(ch, a, which, p0, p1, nl); break;
        case 4: launch_x_all<R, 4>(ch, a, which, p0, p1, nl); break;
        case 6: launch_x_all<R, 6>(ch, a, which, p0, p1, nl); break;
        case 8: launch_x_all<R, 8>(ch, a, which, p0, p1, nl); break;
        case 12: launch_x_all<R, 12>(ch, a, which, p0, p1, nl); break;
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
    return 0;
}

template <typename R> struct ZL { static constexpr int L = 16; };

template <typename R>
static long long zthreads(const c3d_channel *ch) {
    return (long long)ch->g.n2m * (ch->g.n3m / ZL<R>::L) * ch->g.n1m;
}

template <typename R>
static int run_projection_tail(c3d_channel *ch, StepArgs<R> &a, R *d0, R *d1, R *d2, int updp, int *nl) {
    cudaStream_t st = ch->stream;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    constexpr int L = ZL<R>::L;
    typedef typename Cx<R>::T C2;
    const int nz = nblk(zthreads<R>(ch));
    k_zD<R, L><<<nz, TPB, 0, st>>>(a, d2); mark(ch, nl, "zD", N * (8 + 2 * Rb));
    if (launch_x<R>(ch, a, 2, d0, d1, nl)) return C3D_EINVAL;
    const int ntile = (ch->g.n1h + TWZ - 1) / TWZ;
    const size_t smz = 2 * (size_t)ch->g.n3m * TWZ * sizeof(C2);
    k_fftz<R><<<ch->g.n2m * ntile, TPB, smz, st>>>(a, -1); mark(ch, nl, "fftz_fwd", N * 2 * Rb);
    k_poisson<R><<<nblk((long long)ch->g.n1h * ch->g.n3m), TPB, 0, st>>>(a); mark(ch, nl, "poisson", N * (2 * Rb + 8));
    k_fftz<R><<<ch->g.n2m * ntile, TPB, smz, st>>>(a, +1); mark(ch, nl, "fftz_inv", N * 2 * Rb);
    if (launch_x<R>(ch, a, 3, d0, d2, nl)) return C3D_EINVAL;
    StepArgs<double> ad;
    StepArgs<float> af;
    memset(&ad, 0, sizeof(ad));
    memset(&af, 0, sizeof(af));
    if constexpr (sizeof(R) == 8) k_reduce<<<1, 1024, 0, st>>>(a, af, 0);
    else k_reduce<<<1, 1024, 0, st>>>(ad, a, 1);
    mark(ch, nl, "reduce", 16.0 * ch->g.n2m * ch->g.n3m);
    k_zE<R, L><<<nz, TPB, 0, st>>>(a, d0, d1, d2, updp); mark(ch, nl, "zE", N * (72 + 4 * Rb));
    return 0;
}

template <typename R>
static void set_smem_limits(c3d_channel *ch) {
    typedef typename Cx<R>::T C2;
    const size_t smz = 2 * (size_t)ch->g.n3m * TWZ * sizeof(C2);
    cudaFuncSetAttribute(k_fftz<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
}

template <typename R>
static int step_impl(c3d_channel *ch, double dt, int *nl) {
    cudaStream_t st = ch->stream;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    constexpr int L = ZL<R>::L;
    set_smem_limits<R>(ch);
    // rotate the AB2 history: HH of the last step becomes HH_old
    ch->cur = 1 - ch->cur;
    StepArgs<R> a = make_args<R>(ch, dt);
    k_bcond<<<nblk(ch->g.np), TPB, 0, st>>>(ch->g, ch->u, ch->v, ch->w); mark(ch, nl, "bcond", 64.0 * ch->g.np);
    if (launch_x<R>(ch, a, 0, nullptr, nullptr, nl)) return C3D_EINVAL;
    const int nz = nblk(zthreads<R>(ch));
    k_zA<R, L><<<nz, TPB, 0, st>>>(a); mark(ch, nl, "zA", N * (32 + 10 * Rb));
    k_zB<R, L><<<nz, TPB, 0, st>>>(a); mark(ch, nl, "zB", N * 8 * Rb);
    if (launch_x<R>(ch, a, 1, nullptr, nullptr, nl)) return C3D_EINVAL;
    k_ycn<R><<<nblk(3LL * ch->g.np), TPB, 0, st>>>(a); mark(ch, nl, "ycn", N * 6 * Rb);
    // CN z factor: deltas go to exz/eyz/wsq, which the RHS passes no longer need
    R *dd0 = (R *)ch->exz, *dd1 = (R *)ch->eyz, *dd2 = (R *)ch->wsq;
    k_zC<R, L><<<nz, TPB, 0, st>>>(a, dd0, dd1, dd2); mark(ch, nl, "zC", N * 6 * Rb);
    return run_projection_tail<R>(ch, a, dd0, dd1, dd2, 1, nl);
}

int launch_step(c3d_channel *ch, double dt, int *nl) {
    if (ch->precision == C3D_MIXED) return step_impl<float>(ch, dt, nl);
    return step_impl<double>(ch, dt, nl);
}

template <typename R>
static int project_impl(c3d_channel *ch, int *nl) {
    set_smem_limits<R>(ch);
    StepArgs<R> a = make_args<R>(ch, 1.0);
    a.bulk = 0;
    a.dtproj = 1.0;
    R *dd0 = (R *)ch->exz, *dd1 = (R *)ch->eyz, *dd2 = (R *)ch->wsq;
    const size_t bytes = (size_t)ch->g.nf * sizeof(R);
    cudaMemsetAsync(dd0, 0, bytes, ch->stream);
    cudaMemsetAsync(dd1, 0, bytes, ch->stream);
    cudaMemsetAsync(dd2, 0, bytes, ch->stream);
    k_bcond<<<nblk(ch->g.np), TPB, 0, ch->stream>>>(ch->g, ch->u, ch->v, ch->w); mark(ch, nl, "bcond", 64.0 * ch->g.np);
    return run_projection_tail<R>(ch, a, dd0, dd1, dd2, 0, nl);
}

int launch_project(c3d_channel *ch, int *nl) {
    if (ch->precision == C3D_MIXED) return project_impl<float>(ch, nl);
    return project_impl<double>(ch, nl);
}

template <typename R>
static int diag_impl(c3d_channel *ch, int *nl) {
    cudaStream_t st = ch->stream;
    constexpr int L = ZL<R>::L;
    StepArgs<R> a = make_args<R>(ch, 1.0);
    cudaMemsetAsync(ch->scal + SCAL_DIVMAX, 0, 2 * sizeof(double), st);
    cudaMemsetAsync(ch->scal + SCAL_NONFIN, 0, sizeof(double), st);
    if (launch_x<R>(ch, a, 4, nullptr, nullptr, nl)) return C3D_EINVAL;
    k_diag_z<R, L><<<nblk(zthreads<R>(ch)), TPB, 0, st>>>(a); mark(ch, nl, "diag_z", (double)ch->g.n1m * ch->g.n2m * ch->g.n3m * 16);
    k_diag_sums<<<1, 256, 0, st>>>(ch->g, ch->u, ch->v, ch->w, ch->scal); mark(ch, nl, "diag_sums", 64.0 * ch->g.np);
    return 0;
}

int launch_diag(c3d_channel *ch, int *nl) {
    if (ch->precision == C3D_MIXED) return diag_impl<float>(ch, nl);
    return diag_impl<double>(ch, nl);
}

int launch_poisson_tables(c3d_channel *ch) {
    const Geo &g = ch->g;
    const int nm = g.n1h * g.n3m;
    double *tmp = nullptr;
    const int n2 = g.n2;
    if (cudaMalloc(&tmp, sizeof(double) * (size_t)(g.n1m + (g.n3m / 2 + 1) + 3 * (n2 + 1))) != cudaSuccess)
        return C3D_ENOMEM;
    std::vector<double> h;
    h.insert(h.end(), ch->ak1.begin(), ch->ak1.end());
    h.insert(h.end(), ch->ak3.begin(), ch->ak3.end());
    h.insert(h.end(), ch->pmjh.begin(), ch->pmjh.end());
    h.insert(h.end(), ch->pcj.begin(), ch->pcj.end());
    h.insert(h.end(), ch->ppj.begin(), ch->ppj.end());
    cudaMemcpy(tmp, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
    const double *ak1 = tmp, *ak3 = tmp + g.n1m, *pm = ak3 + (g.n3m / 2 + 1), *pc = pm + (n2 + 1),
                 *pp = pc + (n2 + 1);
    k_ptables<<<nblk(nm), TPB, 0, ch->stream>>>(g, ak1, ak3, pm, pc, pp, ch->prb, ch->pgam);
    cudaError_t e = cudaStreamSynchronize(ch->stream);
    cudaFree(tmp);
    return e == cudaSuccess ? 0 : C3D_ECUDA;
}

int launch_repack(c3d_channel *ch, int dir, int what, int comp) {
    const Geo &g = ch->g;
    const int j0 = (what == 0) ? 0 : 1, j1 = (what == 0) ? g.n2 : g.n2m;
    const long long tot_dev = (long long)(j1 - j0 + 1) * g.np;
    const long long N1 = g.n1m + 1, N2 = g.n2, N3 = g.n3m + 1;
    const long long tot_f = (what == 1) ? N1 * N2 * N3 : (N1 + 1) * (N2 + 1) * (N3 + 1);
    cudaStream_t st = ch->stream;
    if (what == 2) {
        void *hp = ch->hh[ch->cur][comp];
        if (ch->precision == C3D_MIXED) {
            if (dir == 0) k_unpack<float><<<nblk(tot_dev), TPB, 0, st>>>(g, 2, comp, (float *)hp, ch->stage);
            else k_pack<float><<<nblk(tot_f), TPB, 0, st>>>(g, 2, comp, (const float *)hp, ch->stage);
        } else {
            if (dir == 0) k_unpack<double><<<nblk(tot_dev), TPB, 0, st>>>(g, 2, comp, (double *)hp, ch->stage);
            else k_pack<double><<<nblk(tot_f), TPB, 0, st>>>(g, 2, comp, (const double *)hp, ch->stage);
        }
        return 0;
    }
    double *dst = (what == 1) ? ch->p : (comp == 0 ? ch->u : comp == 1 ? ch->v : ch->w);
    if (dir == 0) k_unpack<double><<<nblk(tot_dev), TPB, 0, st>>>(g, what, comp, dst, ch->stage);
    else k_pack<double><<<nblk(tot_f), TPB, 0, st>>>(g, what, comp, dst, ch->stage);
    return 0;
}

}  // namespace c3d
