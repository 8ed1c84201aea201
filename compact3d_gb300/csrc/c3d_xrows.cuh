// c3d_xrows.cuh -- bodies of the x-row passes of the step, shared by the single-channel
// kernels (c3d_xpass.cu) and the batch kernels (c3d_xbatch.cu).  A row (j, k) is held by
// a segment of W lanes (W = 32: one warp per row); lane l owns the C consecutive points
// [l*C, l*C+C).
//   xA  RHS1/2/3 pieces along x (compact3d.f:6063-6334, 6784-6900, 7399-7470)
//   xB  remaining convection terms, AB2 and the x factor of Crank-Nicolson
//       (compact3d.f:6765-6775, 7385-7392, 8095-8104, 8218-8627)
//   xC  RHSDP along x and the real-to-complex FFT of RDP along x (8117-8176, 9325-9345)
//   xD  complex-to-real FFT along x, dDP/dx and the bulk-flow partial sums (9408-9441, 1052-1105)
//   diag_x  DIVCHECK x part and CFL (9049-9169)
#pragma once
#include "c3d_kern.cuh"

namespace c3d {

// ---------------------------------------------------------------------------------
// xA
// ---------------------------------------------------------------------------------
// Rows of u, v, w and P at J-1, J, J+1 that the xA pieces read, and their slots in the
// warp's shared-memory stage when the rows are staged by bulk copies.
enum XaRow { XA_UM, XA_UC, XA_UP, XA_PM, XA_PC, XA_VM, XA_VC, XA_VP, XA_WM, XA_WC, XA_WP };
template <int PART>
__host__ __device__ constexpr int xa_slot(int r) {
    return PART == 1 ? (r == XA_UM ? 0 : r == XA_UC ? 1 : r == XA_UP ? 2 : 3)
         : PART == 2 ? (r == XA_VM ? 0 : r == XA_VC ? 1 : r == XA_VP ? 2 : r == XA_PM ? 3 : r == XA_PC ? 4
                        : r == XA_UM ? 5 : 6)
                     : (r == XA_WM ? 0 : r == XA_WC ? 1 : 2);
}
// The row r of (j, k): in global memory at offsets o (J), om (J-1), op (J+1), or slot
// xa_slot(r) of the stage st (rows of n points).
template <bool STG, int PART, typename R>
__device__ __forceinline__ const typename SType<R>::S *xa_src(const StepArgs<R> &a, int r, long long o, long long om,
                                                               long long op, const typename SType<R>::S *st, int n) {
    if constexpr (STG) {
        return st + (size_t)xa_slot<PART>(r) * n;
    } else {
        (void)st; (void)n;
        switch (r) {
            case XA_UM: return a.u + om;
            case XA_UC: return a.u + o;
            case XA_UP: return a.u + op;
            case XA_PM: return a.p + om;
            case XA_PC: return a.p + o;
            case XA_VM: return a.v + om;
            case XA_VC: return a.v + o;
            case XA_VP: return a.v + op;
            case XA_WM: return a.w + om;
            case XA_WC: return a.w + o;
            default: return a.w + op;
        }
    }
}

// Row operand of an x pass: a global row (read through the read-only path) or a row
// already staged in shared memory by bulk copies.
template <bool STG, typename T, int C>
__device__ __forceinline__ void xrow(T (&v)[C], const T *p, T *sb, int lane, int P) {
    if constexpr (STG) crow_load(v, p, lane, P);
    else srow_load(v, p, sb, lane, P);
}

// One row (j, k) of the u (PART 1), v (PART 2, faces J >= 2) or w (PART 3) piece of xA.
template <typename R, int C, int PART, bool STG, int W = 32>
__device__ __forceinline__ void xa_piece(const StepArgs<R> &a, int j, long long o, long long om, long long op,
                                         const typename SType<R>::S *st, typename SType<R>::S *sbS, R *sbR, int lane,
                                         int P) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    const int n = a.g.n1m;
    const R RE1 = a.re1, f12 = a.f12x, f24 = a.f24x, four = (R)4.0;
    const R presg = (R)a.scal[SCAL_PRESG];
    if (PART == 2 && j >= 2) {
        // The v piece on its own, ordered so that few rows are live at once: the y
        // stencils of V (HH2 stored), then -dP/dy, then the x terms of V (R2 stored),
        // then E_xy with u at the y faces.
        const R DYPj = a.m.dyp[j], DYCj = a.m.dyc[j], DYMj = a.m.dym[j], Z0 = a.m.dyz[j];
        const R Hj1 = a.m.rh[j];
        R acc[C];
        {
            S vc[C], vm[C], vp[C];
            xrow<STG>(vc, xa_src<STG, PART>(a, XA_VC, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(vm, xa_src<STG, PART>(a, XA_VM, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(vp, xa_src<STG, PART>(a, XA_VP, o, om, op, st, n), sbS, lane, P);
            R hh[C];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                acc[t] = RE1 * ST::yvisc(DYPj, DYCj, DYMj, Z0, vp[t], vc[t], vm[t]);
                hh[t] = Hj1 * Sten<R>::vv(vp[t], vc[t], vm[t]);
            }
            srow_store(a.hh[1] + o, hh, sbR, lane, P);
        }
        {
            S pc[C], pm[C];
            xrow<STG>(pc, xa_src<STG, PART>(a, XA_PC, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(pm, xa_src<STG, PART>(a, XA_PM, o, om, op, st, n), sbS, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R pg = ST::d(pc[t], pm[t]) * Hj1;
                acc[t] = -pg + acc[t];
            }
        }
        S vc[C];
        xrow<STG>(vc, xa_src<STG, PART>(a, XA_VC, o, om, op, st, n), sbS, lane, P);
        R d[C];
        S pv = sprev<W>(vc[C - 1], lane, P), nx = snext<W>(vc[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S l = (t == 0) ? pv : vc[t - 1], rr = (t == C - 1) ? nx : vc[t + 1];
            d[t] = f12 * ST::d2(l, vc[t], rr);
        }
        xsolve<W>(d, lane, P, a.c10x);
#pragma unroll
        for (int t = 0; t < C; ++t) acc[t] = acc[t] + RE1 * d[t];
        srow_store(a.r[1] + o, acc, sbR, lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S l = (t == 0) ? pv : vc[t - 1];
            d[t] = four * (ST::hi(l) + ST::hi(vc[t]));
        }
        xsolve<W>(d, lane, P, a.c6x);
        {   // u at the y faces
            S uc[C], um[C];
            xrow<STG>(uc, xa_src<STG, PART>(a, XA_UC, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(um, xa_src<STG, PART>(a, XA_UM, o, om, op, st, n), sbS, lane, P);
            const R a1 = a.m.hdy[j], a2 = a.m.hdy[j - 1];
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = d[t] * (Hj1 * (a1 * ST::hi(um[t]) + a2 * ST::hi(uc[t])));
        }
        srow_store(a.exy + o, d, sbR, lane, P);
    }
    if (PART == 1) {
        // The u piece on its own, ordered so that few rows are live at once: the y
        // stencil of U, the x terms of U (HH1 stored), then -dP/dx (R1 stored).
        const R HPj = a.m.hp[j], HCj = a.m.hc[j], HMj = a.m.hm[j], Z0 = a.m.hz[j];
        R acc[C];
        {
            S um[C], up[C], uc0[C];
            xrow<STG>(uc0, xa_src<STG, PART>(a, XA_UC, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(um, xa_src<STG, PART>(a, XA_UM, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(up, xa_src<STG, PART>(a, XA_UP, o, om, op, st, n), sbS, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) acc[t] = RE1 * ST::yvisc(HPj, HCj, HMj, Z0, up[t], uc0[t], um[t]);
        }
        S uc[C];
        xrow<STG>(uc, xa_src<STG, PART>(a, XA_UC, o, om, op, st, n), sbS, lane, P);
        R d[C];
        S pv = sprev<W>(uc[C - 1], lane, P), nx = snext<W>(uc[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S l = (t == 0) ? pv : uc[t - 1], rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = f12 * ST::d2(l, uc[t], rr);
        }
        xsolve<W>(d, lane, P, a.c10x);
#pragma unroll
        for (int t = 0; t < C; ++t) acc[t] = acc[t] + RE1 * d[t];
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = four * (ST::hi(uc[t]) + ST::hi(rr));
        }
        xsolve<W>(d, lane, P, a.c6x);
        R sq[C];
#pragma unroll
        for (int t = 0; t < C; ++t) sq[t] = d[t] * d[t];
        R ps = sprev<W>(sq[C - 1], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            R l = (t == 0) ? ps : sq[t - 1];
            d[t] = f24 * (sq[t] - l);
        }
        xsolve<W>(d, lane, P, a.c22x);
        srow_store(a.hh[0] + o, d, sbR, lane, P);
        {
            S pc[C];
            xrow<STG>(pc, xa_src<STG, PART>(a, XA_PC, o, om, op, st, n), sbS, lane, P);
            S pp = sprev<W>(pc[C - 1], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pp : pc[t - 1];
                d[t] = f24 * ST::d(pc[t], l);
            }
        }
        xsolve<W>(d, lane, P, a.c22x);
#pragma unroll
        for (int t = 0; t < C; ++t) acc[t] = acc[t] - d[t] - presg;
        srow_store(a.r[0] + o, acc, sbR, lane, P);
    }
    if (PART == 3) {
        // The w piece on its own: the y stencil first, then the x terms.
        const R HPj = a.m.hp[j], HCj = a.m.hc[j], HMj = a.m.hm[j], Z0 = a.m.hz[j];
        R acc[C];
        {
            S wm[C], wp[C], wc0[C];
            xrow<STG>(wc0, xa_src<STG, PART>(a, XA_WC, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(wm, xa_src<STG, PART>(a, XA_WM, o, om, op, st, n), sbS, lane, P);
            xrow<STG>(wp, xa_src<STG, PART>(a, XA_WP, o, om, op, st, n), sbS, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) acc[t] = RE1 * ST::yvisc(HPj, HCj, HMj, Z0, wp[t], wc0[t], wm[t]);
        }
        S wc[C];
        xrow<STG>(wc, xa_src<STG, PART>(a, XA_WC, o, om, op, st, n), sbS, lane, P);
        R d[C];
        S pv = sprev<W>(wc[C - 1], lane, P), nx = snext<W>(wc[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S l = (t == 0) ? pv : wc[t - 1], rr = (t == C - 1) ? nx : wc[t + 1];
            d[t] = f12 * ST::d2(l, wc[t], rr);
        }
        xsolve<W>(d, lane, P, a.c10x);
#pragma unroll
        for (int t = 0; t < C; ++t) acc[t] = acc[t] + RE1 * d[t];
        srow_store(a.r[2] + o, acc, sbR, lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S l = (t == 0) ? pv : wc[t - 1];
            d[t] = four * (ST::hi(l) + ST::hi(wc[t]));
        }
        xsolve<W>(d, lane, P, a.c6x);
        srow_store(a.ww1 + o, d, sbR, lane, P);
    }
}

// PART 0 computes the u, v and w pieces in one kernel; PART 1, 2, 3 compute one of them
// (the split form has fewer registers per thread; PART 2 reads the two u rows of the
// y-face interpolant again).  A row is held by a segment of W lanes (W = 32: a warp); with
// W < 32 the 32/W rows of a warp must share J (N3M a multiple of 32/W) so that the warp
// takes the J-dependent branches together.
template <typename R, int C, int PART, int W = 32>
__device__ __forceinline__ void b_xA(const StepArgs<R> &a, const Blk blk) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    static_assert(W == 32 || !C3D_STAGED_ROWS, "rows staged per warp need one row per warp");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & (W - 1), wid = threadIdx.x / W, rpb = (int)blockDim.x / W;
    const int P = g.n1m / C;
    S *sbS = reinterpret_cast<S *>(smem_raw + wid * stage_bytes(g.n1m, C));
    R *sbR = reinterpret_cast<R *>(sbS);
    const int nrows = g.n2m * g.n3m;
    const R RE1 = a.re1, f12 = a.f12x, f24 = a.f24x, four = (R)4.0;
    const R presg = (R)a.scal[SCAL_PRESG];
    for (int row = blk.x * rpb + wid; row < nrows; row += blk.gx * rpb) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), om = fidx(g, 0, j - 1, k), op = fidx(g, 0, j + 1, k);
        {   // every row this warp reads, requested from DRAM at once
            const int rb = g.n1m * (int)sizeof(S);
            if (PART <= 2) { pf_row(a.u + om, rb, lane, W); pf_row(a.u + o, rb, lane, W); pf_row(a.p + o, rb, lane, W); }
            if (PART <= 1) pf_row(a.u + op, rb, lane, W);
            if (PART == 0 || PART == 2) {
                pf_row(a.p + om, rb, lane, W);
                pf_row(a.v + om, rb, lane, W); pf_row(a.v + o, rb, lane, W); pf_row(a.v + op, rb, lane, W);
            }
            if (PART == 0 || PART == 3) { pf_row(a.w + om, rb, lane, W); pf_row(a.w + o, rb, lane, W); pf_row(a.w + op, rb, lane, W); }
        }
        R uy[C];
        if (PART >= 1) {
            xa_piece<R, C, PART, false, W>(a, j, o, om, op, nullptr, sbS, sbR, lane, P);
        }
        // ---- u: R1 = visc_y + visc_x/RE - dP/dx - PRESG ; HH1 = d(uu)/dx ----
        if (PART == 0) {
            S uc[C], um[C], up[C];
            srow_load(uc, a.u + o, sbS, lane, P);
            srow_load(um, a.u + om, sbS, lane, P);
            srow_load(up, a.u + op, sbS, lane, P);
            const R HPj = a.m.hp[j], HCj = a.m.hc[j], HMj = a.m.hm[j], Z0 = a.m.hz[j];
            R acc[C], d[C];
            S pv = sprev<W>(uc[C - 1], lane, P), nx = snext<W>(uc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pv : uc[t - 1], rr = (t == C - 1) ? nx : uc[t + 1];
                d[t] = f12 * ST::d2(l, uc[t], rr);
            }
            xsolve<W>(d, lane, P, a.c10x);
#pragma unroll
            for (int t = 0; t < C; ++t) acc[t] = RE1 * ST::yvisc(HPj, HCj, HMj, Z0, up[t], uc[t], um[t]) + RE1 * d[t];
            {
                S pc[C];
                srow_load(pc, a.p + o, sbS, lane, P);
                S pp = sprev<W>(pc[C - 1], lane, P);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    S l = (t == 0) ? pp : pc[t - 1];
                    d[t] = f24 * ST::d(pc[t], l);
                }
                xsolve<W>(d, lane, P, a.c22x);
#pragma unroll
                for (int t = 0; t < C; ++t) acc[t] = acc[t] - d[t] - presg;
                srow_store(a.r[0] + o, acc, sbR, lane, P);
            }
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S rr = (t == C - 1) ? nx : uc[t + 1];
                d[t] = four * (ST::hi(uc[t]) + ST::hi(rr));
            }
            xsolve<W>(d, lane, P, a.c6x);
            R sq[C];
#pragma unroll
            for (int t = 0; t < C; ++t) sq[t] = d[t] * d[t];
            R ps = sprev<W>(sq[C - 1], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R l = (t == 0) ? ps : sq[t - 1];
                d[t] = f24 * (sq[t] - l);
            }
            xsolve<W>(d, lane, P, a.c22x);
            srow_store(a.hh[0] + o, d, sbR, lane, P);
            if (PART == 0 && j >= 2) {
                const R Hj1 = a.m.rh[j], a1 = a.m.hdy[j], a2 = a.m.hdy[j - 1];
#pragma unroll
                for (int t = 0; t < C; ++t) uy[t] = Hj1 * (a1 * ST::hi(um[t]) + a2 * ST::hi(uc[t]));
            }
        }
        // ---- v (faces J=2..N2M): R2, HH2 = d(vv)/dy, E_xy = VV1 * UY ----
        if (PART == 0 && j >= 2) {
            S vc[C], vm[C], vp[C];
            srow_load(vc, a.v + o, sbS, lane, P);
            srow_load(vm, a.v + om, sbS, lane, P);
            srow_load(vp, a.v + op, sbS, lane, P);
            R d[C], acc[C], hh[C];
            S pv = sprev<W>(vc[C - 1], lane, P), nx = snext<W>(vc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pv : vc[t - 1], rr = (t == C - 1) ? nx : vc[t + 1];
                d[t] = f12 * ST::d2(l, vc[t], rr);
            }
            xsolve<W>(d, lane, P, a.c10x);
            const R DYPj = a.m.dyp[j], DYCj = a.m.dyc[j], DYMj = a.m.dym[j], Z0 = a.m.dyz[j];
            const R Hj = a.m.h[j], Hj1 = a.m.rh[j];
            {
                S pc[C], pm[C];
                srow_load(pc, a.p + o, sbS, lane, P);
                srow_load(pm, a.p + om, sbS, lane, P);
#pragma unroll
                for (int t = 0; t < C; ++t) {
                    R visc = RE1 * ST::yvisc(DYPj, DYCj, DYMj, Z0, vp[t], vc[t], vm[t]);
                    R pg = ST::d(pc[t], pm[t]) * Hj1;
                    acc[t] = (-pg + visc) + RE1 * d[t];
                    hh[t] = Hj1 * Sten<R>::vv(vp[t], vc[t], vm[t]);
                }
            }
            srow_store(a.r[1] + o, acc, sbR, lane, P);
            srow_store(a.hh[1] + o, hh, sbR, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pv : vc[t - 1];
                d[t] = four * (ST::hi(l) + ST::hi(vc[t]));
            }
            xsolve<W>(d, lane, P, a.c6x);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = d[t] * uy[t];
            srow_store(a.exy + o, d, sbR, lane, P);
        }
        // ---- w: R3 = visc_y + visc_x/RE ; WW1 = w at x faces ----
        if (PART == 0) {
            S wc[C], wm[C], wp[C];
            srow_load(wc, a.w + o, sbS, lane, P);
            srow_load(wm, a.w + om, sbS, lane, P);
            srow_load(wp, a.w + op, sbS, lane, P);
            R d[C], acc[C];
            S pv = sprev<W>(wc[C - 1], lane, P), nx = snext<W>(wc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pv : wc[t - 1], rr = (t == C - 1) ? nx : wc[t + 1];
                d[t] = f12 * ST::d2(l, wc[t], rr);
            }
            xsolve<W>(d, lane, P, a.c10x);
            const R HPj = a.m.hp[j], HCj = a.m.hc[j], HMj = a.m.hm[j], Z0 = a.m.hz[j];
#pragma unroll
            for (int t = 0; t < C; ++t) acc[t] = RE1 * ST::yvisc(HPj, HCj, HMj, Z0, wp[t], wc[t], wm[t]) + RE1 * d[t];
            srow_store(a.r[2] + o, acc, sbR, lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                S l = (t == 0) ? pv : wc[t - 1];
                d[t] = four * (ST::hi(l) + ST::hi(wc[t]));
            }
            xsolve<W>(d, lane, P, a.c6x);
            srow_store(a.ww1 + o, d, sbR, lane, P);
        }
    }
}
// At least 3 blocks of XMAXT threads per SM: at most 80 registers, so more rows are in
// flight (the pieces are latency-bound; measured on 384-point rows: 0.742 -> 0.705 ms for
// the three pieces, with a few dozen bytes of spills).
template <typename R, int C, int PART, int W = 32>
__global__ void __launch_bounds__(XMAXT, 3) k_xA(StepArgs<R> a) {
    b_xA<R, C, PART, W>(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// The u, v or w piece of xA with the rows it reads staged in shared memory: lane 0 of
// each warp issues one bulk copy per row (cp.async.bulk, completion counted on one
// mbarrier by bytes), so every row of the warp's (j, k) is in flight at once instead of
// one dependent group after another; the piece then reads the rows from shared memory.
// One row per warp.  Rows staged: u at J-1, J, J+1 and P at J (PART 1); v at J-1, J, J+1,
// P at J-1, J and u at J-1, J (PART 2); w at J-1, J, J+1 (PART 3).  A wait that runs out
// (about a second) sets SCAL_PIPEERR, waits once more for the warp's copies in flight and
// returns.
template <int PART> struct XaStage { static constexpr int rows = PART == 1 ? 4 : PART == 2 ? 7 : 3; };

__host__ __device__ inline size_t xa_stage_bytes(int part, int n1m) {
    return 16 + (size_t)(part == 1 ? 4 : part == 2 ? 7 : 3) * (size_t)n1m * 8;
}

template <typename R, int C, int PART>
__global__ void __launch_bounds__(XMAXT) k_xAs(StepArgs<R> a) {
    typedef typename SType<R>::S S;
    static_assert(sizeof(S) == 8, "state rows are 8-byte values");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    constexpr int NR = XaStage<PART>::rows;
    unsigned char *wb = smem_raw + wid * xa_stage_bytes(PART, g.n1m);
    uint64_t *bar = reinterpret_cast<uint64_t *>(wb);
    S *st = reinterpret_cast<S *>(wb + 16);
    const int row = blockIdx.x * (int)(blockDim.x >> 5) + wid;
    if (row >= g.n2m * g.n3m) return;
    const int j = 1 + row / g.n3m, k = row % g.n3m;
    if (PART == 2 && j < 2) return;
    const long long o = fidx(g, 0, j, k), om = fidx(g, 0, j - 1, k), op = fidx(g, 0, j + 1, k);
    const int n = g.n1m;
    const uint32_t rb = (uint32_t)n * (uint32_t)sizeof(S);
    if (lane == 0) {
        const S *src[NR];
        if constexpr (PART == 1) {
            src[xa_slot<1>(XA_UM)] = a.u + om; src[xa_slot<1>(XA_UC)] = a.u + o; src[xa_slot<1>(XA_UP)] = a.u + op;
            src[xa_slot<1>(XA_PC)] = a.p + o;
        }
        if constexpr (PART == 2) {
            src[xa_slot<2>(XA_VM)] = a.v + om; src[xa_slot<2>(XA_VC)] = a.v + o; src[xa_slot<2>(XA_VP)] = a.v + op;
            src[xa_slot<2>(XA_PM)] = a.p + om; src[xa_slot<2>(XA_PC)] = a.p + o;
            src[xa_slot<2>(XA_UM)] = a.u + om; src[xa_slot<2>(XA_UC)] = a.u + o;
        }
        if constexpr (PART == 3) {
            src[xa_slot<3>(XA_WM)] = a.w + om; src[xa_slot<3>(XA_WC)] = a.w + o; src[xa_slot<3>(XA_WP)] = a.w + op;
        }
        mbar_init(bar, 1);
        mbar_init_fence();
        fence_async_smem();
        mbar_expect_tx(bar, NR * rb);
#pragma unroll
        for (int q = 0; q < NR; ++q) bulk_g2s(st + (size_t)q * n, src[q], rb, bar);
    }
    __syncwarp();
    if (!mbar_wait(bar, 0)) {
        if (lane == 0) a.scal[SCAL_PIPEERR] = 1.0;
        mbar_wait(bar, 0);   // the copies in flight target this warp's stage
        return;
    }
    xa_piece<R, C, PART, true>(a, j, o, om, op, st, nullptr, nullptr, lane, P);
}

// ---------------------------------------------------------------------------------
// xB: remaining convective terms, AB2, x factor of Crank-Nicolson
// ---------------------------------------------------------------------------------
template <typename R, int C, int W = 32>
__device__ __forceinline__ void ab2_cnx(const StepArgs<R> &a, int c, long long o, const R (&hc)[C], R *sb,
                                        int lane, int P, R dt) {
    R rr[C], ho[C], d[C];
    srow_load(rr, a.r[c] + o, sb, lane, P);
    srow_load(ho, a.ho[c] + o, sb, lane, P);
#pragma unroll
    for (int t = 0; t < C; ++t) rr[t] = (rr[t] - (R)1.5 * hc[t] + (R)0.5 * ho[t]) * dt;
    R pv = sprev<W>(rr[C - 1], lane, P), nx = snext<W>(rr[0], lane, P);
#pragma unroll
    for (int t = 0; t < C; ++t) {
        R l = (t == 0) ? pv : rr[t - 1], r2 = (t == C - 1) ? nx : rr[t + 1];
        d[t] = (l + (R)10.0 * rr[t]) + r2;
    }
    xsolve<W>(d, lane, P, a.cnx);
    srow_store(a.r[c] + o, d, sb, lane, P);
}

template <typename R, int C, int W = 32>
__device__ __forceinline__ void b_xB(const StepArgs<R> &a, const Blk blk) {
    static_assert(W == 32 || !C3D_STAGED_ROWS, "rows staged per warp need one row per warp");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & (W - 1), wid = threadIdx.x / W, rpb = (int)blockDim.x / W;
    const int P = g.n1m / C;
    R *sb = reinterpret_cast<R *>(smem_raw + wid * stage_bytes(g.n1m, C));
    const int nrows = g.n2m * g.n3m;
    const R f = a.f24x;
    const R dt = (R)a.dt;
    for (int row = blk.x * rpb + wid; row < nrows; row += blk.gx * rpb) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
        {
            const int rb = g.n1m * (int)sizeof(R);
            pf_row(a.hh[0] + o, rb, lane, W); pf_row(a.hh[1] + o, rb, lane, W); pf_row(a.hh[2] + o, rb, lane, W);
            pf_row(a.exy + o, rb, lane, W); pf_row(a.exy + op, rb, lane, W); pf_row(a.exz + o, rb, lane, W);
            pf_row(a.eyz + o, rb, lane, W); pf_row(a.eyz + op, rb, lane, W);
            for (int c = 0; c < 3; ++c) { pf_row(a.r[c] + o, rb, lane, W); pf_row(a.ho[c] + o, rb, lane, W); }
        }
        const R rdy = a.m.rdy[j];
        R h1[C], h3[C], e[C], ep[C], d[C];
        srow_load(h1, a.hh[0] + o, sb, lane, P);
        srow_load(h3, a.hh[2] + o, sb, lane, P);
        // E_xy at faces j and j+1 (zero on the walls)
        if (j >= 2) srow_load(e, a.exy + o, sb, lane, P);
        else {
#pragma unroll
            for (int t = 0; t < C; ++t) e[t] = R(0);
        }
        if (j + 1 <= g.n2m) srow_load(ep, a.exy + op, sb, lane, P);
        else {
#pragma unroll
            for (int t = 0; t < C; ++t) ep[t] = R(0);
        }
#pragma unroll
        for (int t = 0; t < C; ++t) h1[t] = h1[t] + rdy * (ep[t] - e[t]);   // d(uv)/dy
        srow_store(a.hh[0] + o, h1, sb, lane, P);
        ab2_cnx<R, C, W>(a, 0, o, h1, sb, lane, P, dt);
        if (j >= 2) {
            R h2[C];
            srow_load(h2, a.hh[1] + o, sb, lane, P);
            R nx = snext<W>(e[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R rr = (t == C - 1) ? nx : e[t + 1];
                d[t] = f * (rr - e[t]);
            }
            xsolve<W>(d, lane, P, a.c22x);
#pragma unroll
            for (int t = 0; t < C; ++t) h2[t] = h2[t] + d[t];                 // d(uv)/dx
            srow_store(a.hh[1] + o, h2, sb, lane, P);
            ab2_cnx<R, C, W>(a, 1, o, h2, sb, lane, P, dt);
        }
        // d(uw)/dx from E_xz, d(wv)/dy from E_yz at faces j, j+1
        srow_load(e, a.exz + o, sb, lane, P);
        {
            R nx = snext<W>(e[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                R rr = (t == C - 1) ? nx : e[t + 1];
                d[t] = f * (rr - e[t]);
            }
        }
        xsolve<W>(d, lane, P, a.c22x);
#pragma unroll
        for (int t = 0; t < C; ++t) h3[t] = h3[t] + d[t];
        if (j >= 2) srow_load(e, a.eyz + o, sb, lane, P);
        else {
#pragma unroll
            for (int t = 0; t < C; ++t) e[t] = R(0);
        }
        if (j + 1 <= g.n2m) srow_load(ep, a.eyz + op, sb, lane, P);
        else {
#pragma unroll
            for (int t = 0; t < C; ++t) ep[t] = R(0);
        }
#pragma unroll
        for (int t = 0; t < C; ++t) h3[t] = h3[t] + rdy * (ep[t] - e[t]);
        srow_store(a.hh[2] + o, h3, sb, lane, P);
        ab2_cnx<R, C, W>(a, 2, o, h3, sb, lane, P, dt);
    }
}
template <typename R, int C, int W = 32>
__global__ void __launch_bounds__(XMAXT) k_xB(StepArgs<R> a) {
    b_xB<R, C, W>(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// ---------------------------------------------------------------------------------
// xC: RDP = div(UH)/DT and its real-to-complex FFT along x
// ---------------------------------------------------------------------------------
// Shared-memory layout of one xC stage (mixed and FP64 forms alike): the rows
// U(J), DH1(J), RDPZ(J), V(J), DH2(J), V(J+1), DH2(J+1) of one (J, K).
template <typename R>
struct XcStage {
    typedef typename SType<R>::S S;
    int u, d0, z, vc, dc, vp, dp, bytes;
    __host__ __device__ XcStage(int n) {
        const int sS = n * (int)sizeof(S), sR = n * (int)sizeof(R);
        u = 0; d0 = sS; z = d0 + sR; vc = z + sR; dc = vc + sS; vp = dc + sR; dp = vp + sS; bytes = dp + sR;
    }
};

// One row of xC: the x part of div(UH)/DT from U + DH1 (compact (1,22,1) derivative),
// the y part from V + DH2 on planes J and J+1, plus RDPZ; then the real-to-complex FFT.
template <bool SH, typename R, int C, bool X4 = false, int W = 32>
__device__ __forceinline__ void xc_row(const StepArgs<R> &a, int j, int k, const typename SType<R>::S *u,
                                       const R *d0, const typename SType<R>::S *vc, const R *dc,
                                       const typename SType<R>::S *vp, const R *dp, const R *zr,
                                       unsigned char *sbuf, typename Cx<R>::T *bufa, typename Cx<R>::T *bufb,
                                       int lane) {
    typedef typename SType<R>::S S;
    typedef typename Cx<R>::T C2;
    static_assert(W == 32 || !X4, "the register row FFT spans a warp");
    const Geo &g = a.g;
    const int P = g.n1m / C, M = g.n1m / 2;
    S *sbS = reinterpret_cast<S *>(sbuf);
    R *sbR = reinterpret_cast<R *>(sbuf);
    R *rbuf = reinterpret_cast<R *>(bufa);
    const R rdt = a.rdt, f24 = a.f24x;
    R d[C], base[C];
    {
        S uc[C];
        R dd[C];
        xrow<SH>(uc, u, sbS, lane, P);
        xrow<SH>(dd, d0, sbR, lane, P);
        S nu = snext<W>(uc[0], lane, P);
        R nd = snext<W>(dd[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            S ru = (t == C - 1) ? nu : uc[t + 1];
            R rd = (t == C - 1) ? nd : dd[t + 1];
            d[t] = f24 * Sten<R>::dd(ru, rd, uc[t], dd[t]);
        }
        xsolve<W>(d, lane, P, a.c22x);
    }
    {
        const bool up = (j + 1 <= g.n2m), lo = (j >= 2);
        S vpv[C], vcv[C];
        R dpv[C], dcv[C];
        if (up) { xrow<SH>(vpv, vp, sbS, lane, P); xrow<SH>(dpv, dp, sbR, lane, P); }
        if (lo) { xrow<SH>(vcv, vc, sbS, lane, P); xrow<SH>(dcv, dc, sbR, lane, P); }
        const R ry = a.m.rdy[j] * rdt;   // 1/(DY(J) DT)
        const S zs = S();
#pragma unroll
        for (int t = 0; t < C; ++t) {
            // (FJUP*UH2(J+1) - FJUM*UH2(J))/DY(J), UH2 = V + delta2, UH2 = 0 on the walls
            R dv = Sten<R>::dd(up ? vpv[t] : zs, up ? dpv[t] : R(0), lo ? vcv[t] : zs, lo ? dcv[t] : R(0));
            base[t] = dv * ry;
        }
    }
    {
        R zc[C];
        xrow<SH>(zc, zr, sbR, lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) d[t] = (base[t] + d[t] * rdt) + zc[t];
    }
    const C2 *twx;
    if constexpr (sizeof(R) == 8) twx = reinterpret_cast<const C2 *>(a.twx64);
    else twx = reinterpret_cast<const C2 *>(a.twx32);
    C2 *Sp = reinterpret_cast<C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
    if constexpr (X4) {   // four-step row FFT in registers
        xrow_r2c<R, C>(d, twsel<C2>(a.fx), twx, Sp, lane);
        return;
    }
    // real row -> shared memory as M complex values, FFT, post-process to N1M/2+1 modes
    if (lane < P) {
#pragma unroll
        for (int t = 0; t < C; ++t) rbuf[lane * C + t] = d[t];
    }
    __syncwarp();
    C2 *Z = fft_smem<C2, false, W>(bufa, bufb, a.fx, 0, 1, 0, -1, lane, W);
    for (int kx = lane; kx <= M; kx += W) {
        C2 zk = Z[kx == M ? 0 : kx], zm = cconj(Z[kx == 0 ? 0 : M - kx]);
        C2 E, O;
        E.x = (R)0.5 * (zk.x + zm.x);
        E.y = (R)0.5 * (zk.y + zm.y);
        C2 df = csub(zk, zm);
        O.x = (R)0.5 * df.y;
        O.y = (R)-0.5 * df.x;
        Sp[kx] = cadd(E, cmul(twx[kx], O));
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------------
// xC: RDP = div(UH)/DT and its real-to-complex FFT along x.  NS = 0: every warp reads
// its rows from global memory (one row per warp).  NS >= 2: persistent warps, each with
// an NS-stage bulk-copy ring that fetches the rows of its next NS-1 (J, K) while it
// computes the current one.
// ---------------------------------------------------------------------------------
template <typename R, int C, int NS, bool X4 = false, int W = 32>
__device__ __forceinline__ void b_xC(const StepArgs<R> &a, const R *d0, const R *d1, const Blk blk) {
    typedef typename SType<R>::S S;
    typedef typename Cx<R>::T C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    static_assert(W == 32 || NS == 0, "the bulk-copy ring is per warp");
    const int lane = threadIdx.x & (W - 1), wid = threadIdx.x / W, wpb = (int)blockDim.x / W;
    const int M = g.n1m / 2;
    const int nrows = g.n2m * g.n3m;
    const size_t fbytes = 2 * (size_t)(M + 1) * sizeof(C2);
    if constexpr (NS == 0) {
        const size_t sbytes = stage_bytes(g.n1m, C);
        unsigned char *wb = smem_raw + wid * (sbytes + fbytes);
        C2 *bufa = reinterpret_cast<C2 *>(wb + sbytes);
        for (int row = blk.x * wpb + wid; row < nrows; row += blk.gx * wpb) {
            const int j = 1 + row / g.n3m, k = row % g.n3m;
            const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
            {
                const int rs_ = g.n1m * (int)sizeof(S), rr_ = g.n1m * (int)sizeof(R);
                pf_row(a.u + o, rs_, lane, W); pf_row(d0 + o, rr_, lane, W); pf_row(a.rdpz + o, rr_, lane, W);
                if (j >= 2) { pf_row(a.v + o, rs_, lane, W); pf_row(d1 + o, rr_, lane, W); }
                if (j + 1 <= g.n2m) { pf_row(a.v + op, rs_, lane, W); pf_row(d1 + op, rr_, lane, W); }
            }
            xc_row<false, R, C, X4, W>(a, j, k, a.u + o, d0 + o, a.v + o, d1 + o, a.v + op, d1 + op, a.rdpz + o, wb,
                                    bufa, bufa + (M + 1), lane);
        }
    } else {
        const XcStage<R> L(g.n1m);
        // per warp: NS barriers (16 bytes reserved each), NS stages, the FFT buffers
        // (none for the register row FFT)
        const size_t wbytes = 16 * NS + (size_t)NS * L.bytes + (X4 ? 0 : fbytes);
        unsigned char *wb = smem_raw + wid * wbytes;
        uint64_t *bar = reinterpret_cast<uint64_t *>(wb);
        unsigned char *stg = wb + 16 * NS;
        C2 *bufa = reinterpret_cast<C2 *>(stg + (size_t)NS * L.bytes);
        const int nw = blk.gx * wpb, gw = blk.x * wpb + wid;
        const uint32_t sS = g.n1m * (uint32_t)sizeof(S), sR = g.n1m * (uint32_t)sizeof(R);
        if (lane == 0) {
            for (int s = 0; s < NS; ++s) mbar_init(bar + s, 1);
            mbar_init_fence();
        }
        __syncwarp();
        auto issue = [&](int row, int s) {   // lane 0 only
            const int j = 1 + row / g.n3m, k = row % g.n3m;
            const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
            const bool up = (j + 1 <= g.n2m), lo = (j >= 2);
            unsigned char *st = stg + (size_t)s * L.bytes;
            fence_async_smem();
            mbar_expect_tx(bar + s, sS + 2 * sR + (lo ? sS + sR : 0u) + (up ? sS + sR : 0u));
            bulk_g2s(st + L.u, a.u + o, sS, bar + s);
            bulk_g2s(st + L.d0, d0 + o, sR, bar + s);
            bulk_g2s(st + L.z, a.rdpz + o, sR, bar + s);
            if (lo) { bulk_g2s(st + L.vc, a.v + o, sS, bar + s); bulk_g2s(st + L.dc, d1 + o, sR, bar + s); }
            if (up) { bulk_g2s(st + L.vp, a.v + op, sS, bar + s); bulk_g2s(st + L.dp, d1 + op, sR, bar + s); }
        };
        if (lane == 0)
            for (int s = 0; s < NS - 1; ++s)
                if (gw + s * nw < nrows) issue(gw + s * nw, s);
        int it = 0;
        for (int row = gw; row < nrows; row += nw, ++it) {
            const int s = it % NS;
            const int nrow = row + (NS - 1) * nw;
            if (lane == 0 && nrow < nrows) issue(nrow, (it + NS - 1) % NS);
            if (!mbar_wait(bar + s, (uint32_t)(it / NS) & 1u)) {
                if (lane == 0) a.scal[SCAL_PIPEERR] = 1.0;
                return;
            }
            const int j = 1 + row / g.n3m, k = row % g.n3m;
            const unsigned char *st = stg + (size_t)s * L.bytes;
            xc_row<true, R, C, X4>(a, j, k, reinterpret_cast<const S *>(st + L.u), reinterpret_cast<const R *>(st + L.d0),
                               reinterpret_cast<const S *>(st + L.vc), reinterpret_cast<const R *>(st + L.dc),
                               reinterpret_cast<const S *>(st + L.vp), reinterpret_cast<const R *>(st + L.dp),
                               reinterpret_cast<const R *>(st + L.z), nullptr, bufa, bufa + (M + 1), lane);
        }
    }
}
template <typename R, int C, int NS, bool X4 = false, int W = 32>
__global__ void __launch_bounds__(XMAXT) k_xC(StepArgs<R> a, const R *d0, const R *d1) {
    b_xC<R, C, NS, X4, W>(a, d0, d1, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// ---------------------------------------------------------------------------------
// xD: complex-to-real FFT -> DP, compact dDP/dx, bulk-flow partial sums
// ---------------------------------------------------------------------------------
template <typename R, int C, bool X4 = false, int W = 32>
__device__ __forceinline__ void b_xD(const StepArgs<R> &a, const R *d0, const R *d2, const Blk blk) {
    typedef typename Cx<R>::T C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    static_assert(W == 32 || !X4, "the register row FFT spans a warp");
    const int lane = threadIdx.x & (W - 1), wid = threadIdx.x / W, rpb = (int)blockDim.x / W;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    const size_t sbytes = stage_bytes(g.n1m, C), fbytes = 2 * (size_t)(M + 1) * sizeof(C2);
    unsigned char *wb = smem_raw + wid * (sbytes + fbytes);
    R *sbR = reinterpret_cast<R *>(wb);
    C2 *bufa = reinterpret_cast<C2 *>(wb + sbytes);
    C2 *bufb = bufa + (M + 1);
    const int nrows = g.n2m * g.n3m;
    const C2 *twx;
    if constexpr (sizeof(R) == 8) twx = reinterpret_cast<const C2 *>(a.twx64);
    else twx = reinterpret_cast<const C2 *>(a.twx32);
    const R scale = a.xscale, f24 = a.f24x;
    for (int row = blk.x * rpb + wid; row < nrows; row += blk.gx * rpb) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k);
        const C2 *Sp = reinterpret_cast<const C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        {
            const int rr_ = g.n1m * (int)sizeof(R);
            pf_row(d0 + o, rr_, lane, W); pf_row(d2 + o, rr_, lane, W);
        }
        R dpv[C];
        if constexpr (X4) {   // four-step row FFT in registers
            xrow_c2r<R, C>(dpv, twsel<C2>(a.fx), twx, Sp, lane);
#pragma unroll
            for (int t = 0; t < C; ++t) dpv[t] *= scale;
        } else {
            for (int kx = lane; kx <= M; kx += W) bufb[kx] = Sp[kx];
            __syncwarp();
            for (int kx = lane; kx < M; kx += W) {
                C2 xk = bufb[kx], xm = cconj(bufb[M - kx]);
                C2 E = cadd(xk, xm);
                C2 O = cmul(csub(xk, xm), cconj(twx[kx]));
                C2 Z;
                Z.x = E.x - O.y;
                Z.y = E.y + O.x;
                bufa[kx] = Z;
            }
            __syncwarp();
            C2 *Zr = fft_smem<C2, false, W>(bufa, bufb, a.fx, 0, 1, 0, +1, lane, W);
            const R *rz = reinterpret_cast<const R *>(Zr);
            if (lane < P) {
#pragma unroll
                for (int t = 0; t < C; ++t) dpv[t] = rz[lane * C + t] * scale;
            } else {
#pragma unroll
                for (int t = 0; t < C; ++t) dpv[t] = R(0);
            }
            __syncwarp();
        }
        srow_store(a.dp + o, dpv, sbR, lane, P);
        R d[C];
        R pv = sprev<W>(dpv[C - 1], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            R l = (t == 0) ? pv : dpv[t - 1];
            d[t] = f24 * (dpv[t] - l);
        }
        xsolve<W>(d, lane, P, a.c22x);
        // bulk-flow partial sums below: sum_i delta * DY(J)/DX3/DX1 for u and w
        R q1[C], q3[C];
        srow_load(q1, d0 + o, sbR, lane, P);
        if constexpr (sizeof(R) == 4) {
            // mixed form: the u update's increment delta1 - DT dDP/dx, formed here in the
            // order UPCALC's update forms it in FP32 (zE then adds it, less dm, to U and
            // reads neither delta1 nor dDP/dx)
            const R dt = (R)a.dt;
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = q1[t] - dt * d[t];
        }
        srow_store(a.g1 + o, d, sbR, lane, P);
        srow_load(q3, d2 + o, sbR, lane, P);
        if constexpr (sizeof(R) == 8) {
            R l1 = R(0), l3 = R(0);
#pragma unroll
            for (int t = 0; t < C; ++t) {
                l1 += q1[t];
                l3 += q3[t];
            }
            double s1 = (double)l1, s3 = (double)l3;
#pragma unroll
            for (int off = W / 2; off > 0; off >>= 1) {
                s1 += __shfl_down_sync(FULL, s1, off, W);
                s3 += __shfl_down_sync(FULL, s3, off, W);
            }
            if (lane == 0) {
                const double wgt = g.dy[j] / g.dx3 / g.dx1;
                a.part[row] = s1 * wgt;
                a.part[nrows + row] = s3 * wgt;
            }
        } else {
            // Mixed form: double-float sums (exact two-sums of the FP32 deltas, FP32
            // instructions only) and a double-float weight; the slots of `part` hold
            // float2 pairs that k_reduce1/k_reduce2 combine in the same arithmetic.
            float2 s1 = make_float2(0.f, 0.f), s3 = s1;
#pragma unroll
            for (int t = 0; t < C; ++t) {
                s1 = St<float>::add(s1, q1[t]);
                s3 = St<float>::add(s3, q3[t]);
            }
#pragma unroll
            for (int off = W / 2; off > 0; off >>= 1) {
                float2 o1 = make_float2(__shfl_down_sync(FULL, s1.x, off, W), __shfl_down_sync(FULL, s1.y, off, W));
                float2 o3 = make_float2(__shfl_down_sync(FULL, s3.x, off, W), __shfl_down_sync(FULL, s3.y, off, W));
                s1 = df_add(s1, o1);
                s3 = df_add(s3, o3);
            }
            if (lane == 0) {
                const float2 wgt = a.bulkw[j];
                float2 *pp = reinterpret_cast<float2 *>(a.part);
                pp[row] = df_mul(s1, wgt);
                pp[nrows + row] = df_mul(s3, wgt);
            }
        }
    }
}
template <typename R, int C, bool X4 = false, int W = 32>
__global__ void __launch_bounds__(XMAXT) k_xD(StepArgs<R> a, const R *d0, const R *d2) {
    b_xD<R, C, X4, W>(a, d0, d2, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// ---------------------------------------------------------------------------------
// Diagnostics, x part: DIVCHECK's (V(J+1)-V(J))/DY + compact dU/dx into an FP64
// scratch field, and the CFL maximum.  Always FP64.
// ---------------------------------------------------------------------------------
template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_diag_x(StepArgs<R> a, double *divx, Cyc<double> c22) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    S *sbS = reinterpret_cast<S *>(smem_raw + wid * stage_bytes(g.n1m, C));
    double *sbD = reinterpret_cast<double *>(sbS);
    const int nrows = g.n2m * g.n3m;
    double cmax = 0.0;
    int bad = 0;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const int kp = (k + 1 == g.n3m) ? 0 : k + 1;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k), okp = fidx(g, 0, j, kp);
        S su[C], sv[C], svp[C], sw[C], swk[C];
        srow_load(su, a.u + o, sbS, lane, P);
        srow_load(sv, a.v + o, sbS, lane, P);
        srow_load(svp, a.v + op, sbS, lane, P);
        srow_load(sw, a.w + o, sbS, lane, P);
        srow_load(swk, a.w + okp, sbS, lane, P);
        double uc[C], d[C];
#pragma unroll
        for (int t = 0; t < C; ++t) uc[t] = ST::dbl(su[t]);
        double nx = snext(uc[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = 24.0 * g.dx1 * (rr - uc[t]);
        }
        xsolve(d, lane, P, c22);
        const double dyj = g.dy[j];
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double rr = (t == C - 1) ? nx : uc[t + 1];
            double vc = ST::dbl(sv[t]), vp = ST::dbl(svp[t]);
            d[t] = (vp - vc) / dyj + d[t];
            double cf = fabs(uc[t] + rr) * 0.5 * g.dx1 + fabs(vc + vp) * 0.5 / dyj +
                        fabs(ST::dbl(sw[t]) + ST::dbl(swk[t])) * 0.5 * g.dx3;
            if (lane < P) {
                if (!isfinite(cf)) bad = 1;
                cmax = fmax(cmax, cf);
            }
        }
        srow_store(divx + o, d, sbD, lane, P);
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

}  // namespace c3d
