// c3d_zpass.cu -- z-column passes of the step: one thread per (i, segment of ZL points,
// plane j); consecutive threads take consecutive i, so every access is coalesced.  The
// cyclic compact solves use the warm-up recurrences of zseg (c3d_dev.cuh).
//   zA  RHS1/2/3 pieces along z (compact3d.f:6160-6185, 6337-6433, 6957-7060, 7474-7705)
//   zB  d(uw)/dz, d(vw)/dz, d(ww)/dz (1,22,1)
//   zC  z factor of Crank-Nicolson (CTDMA3I in GETUH1-3)
//   zD  RHSDP along z (8187-8210)
//   zE  UPCALC along z and the velocity / pressure update (1052-1238)
//   diag_z  DIVCHECK z part and max|div| (9099-9128)
#include "c3d_kern.cuh"

namespace c3d {

// ---------------------------------------------------------------------------------
// Column walkers for zsweep: each keeps a sliding window of its stencil inputs in
// registers and loads one new value per position.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int znext(int k, int n) { return (k + 1 == n) ? 0 : k + 1; }
__device__ __forceinline__ int zprev(int k, int n) { return (k == 0) ? n - 1 : k - 1; }

// Prefetch ring of a column: the values at the D positions after the walker's current
// one, loaded D steps before they are used so the loads of consecutive steps overlap.
constexpr int ZPF = 4;
template <typename T>
struct ZRing {
    T v[ZPF];
    int kf;   // position of v[ZPF-1]
    __device__ void fill(const T *col, int k, int n, int s) {
        kf = k;
#pragma unroll
        for (int d = 0; d < ZPF; ++d) {
            kf = znext(kf, n);
            v[d] = col[kf * s];
        }
    }
    // value at the next position; the ring advances by one
    __device__ T pop(const T *col, int n, int s) {
        const T r = v[0];
#pragma unroll
        for (int d = 0; d < ZPF - 1; ++d) v[d] = v[d + 1];
        kf = znext(kf, n);
        v[ZPF - 1] = col[kf * s];
        return r;
    }
};

// Thread coordinates and the line solve of the two z-pass forms: MODE 0, one thread per
// (i, segment of L points, plane) with warm-up recurrences (zsweep); MODE 1, one block per
// (32 consecutive i, plane) with blockDim.y = N3M / L segments and the exact cyclic
// solve (zblock).
template <int L, int MODE>
__device__ __forceinline__ bool zcoords(const Blk blk, const Geo &g, int jlo, int &i, int &j, int &k0) {
    if constexpr (MODE == 1) {
        i = (int)blk.x * 32 + (int)threadIdx.x;
        j = jlo + (int)blk.y;
        k0 = (int)threadIdx.y * L;
        return true;
    } else {
        return zcoord<L>(blk, g, jlo, i, j, k0);
    }
}
template <typename R, int L, int M, int NR, int MODE, typename F>
__device__ __forceinline__ void zsolve(R (&out)[NR][L], int k0, int n, const R (&r)[NR], const R (&s)[NR], F &f) {
    if constexpr (MODE == 1) {
        extern __shared__ __align__(16) unsigned char zsh_raw[];
        zblock<R, L, NR>(out, k0, r, s, f, reinterpret_cast<R *>(zsh_raw));
    } else {
        zsweep<R, L, M, NR>(out, k0, n, r, s, f);
    }
}
// L2 prefetch margin around a thread's positions: the warm-up length (MODE 0) or one point.
template <int MODE>
constexpr int zmargin(int m) { return MODE == 1 ? 1 : m + 1; }

// state column: (1,10,1) RHS f12*(u- - 2u + u+) and (1,6,1) RHS 4*(u- + u) (face k)
template <typename R>
struct WalkVisBack {
    typedef typename SType<R>::S S;
    const S *col; int n, s; R f12; S um, uc; ZRing<S> ru;
    __device__ void start(int k) { um = col[zprev(k, n) * s]; uc = col[k * s]; ru.fill(col, k, n, s); }
    __device__ void next(R (&d)[2]) {
        S up = ru.pop(col, n, s);
        d[0] = f12 * St<R>::d2(um, uc, up);
        d[1] = (R)4.0 * (St<R>::hi(um) + St<R>::hi(uc));
        um = uc; uc = up;
    }
};

// W and P columns: f12*(w- - 2w + w+), 4*(w + w+) (centre k) and f24*(p - p-) (face k)
template <typename R>
struct WalkWP {
    typedef typename SType<R>::S S;
    const S *W, *P; int n, s; R f12, f24; S wm, wc, pm, pc; ZRing<S> rw, rp;
    __device__ void start(int k) {
        wm = W[zprev(k, n) * s]; wc = W[k * s]; pm = P[zprev(k, n) * s]; pc = P[k * s];
        rw.fill(W, k, n, s);
        rp.fill(P, k, n, s);
    }
    __device__ void next(R (&d)[3]) {
        S wp = rw.pop(W, n, s);
        d[0] = f12 * St<R>::d2(wm, wc, wp);
        d[1] = (R)4.0 * (St<R>::hi(wc) + St<R>::hi(wp));
        d[2] = f24 * St<R>::d(pc, pm);
        wm = wc; wc = wp; pm = pc; pc = rp.pop(P, n, s);
    }
};

// zB: f*(Exz+ - Exz), f*(Q - Q-), f*(Eyz+ - Eyz)
template <typename R>
struct WalkZB {
    const R *E1, *Q, *E2; int n, s; R f; R e1, qm, e2; int kn, kc; bool v;
    __device__ void start(int k) {
        e1 = E1[k * s]; qm = Q[zprev(k, n) * s]; e2 = v ? E2[k * s] : R(0); kc = k; kn = znext(k, n);
    }
    __device__ void next(R (&d)[3]) {
        R e1p = E1[kn * s], qc = Q[kc * s], e2p = v ? E2[kn * s] : R(0);
        d[0] = f * (e1p - e1);
        d[1] = f * (qc - qm);
        d[2] = f * (e2p - e2);
        e1 = e1p; qm = qc; e2 = e2p; kc = kn; kn = znext(kn, n);
    }
};

// zC: (x- + 10x) + x+ for the three components
template <typename R>
struct WalkCN {
    const R *X[3]; int n, s; R xm[3], xc[3]; ZRing<R> rx[3];
    __device__ void start(int k) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            xm[c] = X[c][zprev(k, n) * s]; xc[c] = X[c][k * s];
            rx[c].fill(X[c], k, n, s);
        }
    }
    __device__ void next(R (&d)[3]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            R xp = rx[c].pop(X[c], n, s);
            d[c] = (xm[c] + (R)10.0 * xc[c]) + xp;
            xm[c] = xc[c]; xc[c] = xp;
        }
    }
};

// zD: f24*((W+ + D+) - (W + D))
template <typename R>
struct WalkDivZ {
    typedef typename SType<R>::S S;
    const S *W; const R *D; int n, s; R f24; S wc; R dc; ZRing<S> rw; ZRing<R> rd;
    __device__ void start(int k) { wc = W[k * s]; dc = D[k * s]; rw.fill(W, k, n, s); rd.fill(D, k, n, s); }
    __device__ void next(R (&d)[1]) {
        S wp = rw.pop(W, n, s); R dp = rd.pop(D, n, s);
        d[0] = f24 * Sten<R>::dd(wp, dp, wc, dc);
        wc = wp; dc = dp;
    }
};

// zE: f24*(DP - DP-)
template <typename R>
struct WalkGradZ {
    const R *DP; int n, s; R f24; R pm; ZRing<R> rp;
    __device__ void start(int k) { pm = DP[zprev(k, n) * s]; rp.fill(DP, zprev(k, n), n, s); }
    __device__ void next(R (&d)[1]) {
        R pc = rp.pop(DP, n, s);
        d[0] = f24 * (pc - pm);
        pm = pc;
    }
};

// PART 0 runs the three sweeps in one kernel; PART 1, 2, 3 run only the u, the (w, P) or
// the v sweep (the split form has fewer registers per thread and moves the same bytes).
template <typename R, int L, int PART, int MODE>
__device__ __forceinline__ void b_zA(const StepArgs<R> &a, const Blk blk) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoords<L, MODE>(blk, g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const R RE1 = a.re1;
    const long long o = fidx(g, i, j, 0);
    constexpr int M6 = WM<R>::M6;
    if ((g.n1m & 31) == 0) {   // the warp's column windows (32 consecutive i), requested at once
        const int lane = threadIdx.x & 31;
        const long long o0 = fidx(g, i - lane, j, 0), sb = (long long)g.n1m;
        const int ss = 32 * (int)sizeof(S), sr = 32 * (int)sizeof(R);
        if (PART <= 1) {
            pf_cols(a.u + o0, sb * sizeof(S), ss, k0, zmargin<MODE>(M6), L, n, lane);
            pf_cols(a.ww1 + o0, sb * sizeof(R), sr, k0, 0, L, n, lane);
            pf_cols(a.r[0] + o0, sb * sizeof(R), sr, k0, 0, L, n, lane);
        }
        if (PART == 0 || PART == 2) {
            pf_cols(a.w + o0, sb * sizeof(S), ss, k0, zmargin<MODE>(M6), L, n, lane);
            pf_cols(a.p + o0, sb * sizeof(S), ss, k0, zmargin<MODE>(M6), L, n, lane);
            pf_cols(a.r[2] + o0, sb * sizeof(R), sr, k0, 0, L, n, lane);
        }
        if ((PART == 0 || PART == 3) && j >= 2) {
            pf_cols(a.v + o0, sb * sizeof(S), ss, k0, zmargin<MODE>(M6), L, n, lane);
            pf_cols(a.r[1] + o0, sb * sizeof(R), sr, k0, 0, L, n, lane);
            // w at the y face: planes J and J-1 of the segment, read after the solve
            if (PART == 3) pf_cols(a.w + o0, sb * sizeof(S), ss, k0, 0, L, n, lane);
            pf_cols(a.w + fidx(g, i - lane, j - 1, 0), sb * sizeof(S), ss, k0, 0, L, n, lane);
        }
    }
    if (PART == 0 || PART == 1) {   // u: R1 += (1/RE) d2u/dz2 ; E_xz = UU3 * WW1
        R out[2][L];
        const R rr[2] = {a.c10z.r, a.c6z.r}, ss[2] = {a.c10z.s, a.c6z.s};
        WalkVisBack<R> f{a.u + o, n, s, a.f12z};
        zsolve<R, L, M6, 2, MODE>(out, k0, n, rr, ss, f);
        R *Rp = a.r[0] + o, *E = a.exz + o;
        const R *Wx = a.ww1 + o;
#pragma unroll
        for (int t = 0; t < L; ++t) {
            const int kk = (k0 + t) * s;
            Rp[kk] = Rp[kk] + RE1 * out[0][t];
            E[kk] = out[1][t] * Wx[kk];
        }
    }
    if (PART == 0 || PART == 2) {   // w, P: R3 += (1/RE) d2w/dz2 - dP/dz - PRESG3 ; WW3^2
        R out[3][L];
        const R rr[3] = {a.c10z.r, a.c6z.r, a.c22z.r}, ss[3] = {a.c10z.s, a.c6z.s, a.c22z.s};
        WalkWP<R> f{a.w + o, a.p + o, n, s, a.f12z, a.f24z};
        zsolve<R, L, M6, 3, MODE>(out, k0, n, rr, ss, f);
        const R presg3 = (R)a.scal[SCAL_PRESG3];
        R *Rp = a.r[2] + o, *Q = a.wsq + o;
#pragma unroll
        for (int t = 0; t < L; ++t) {
            const int kk = (k0 + t) * s;
            Rp[kk] = Rp[kk] + RE1 * out[0][t] - out[2][t] - presg3;
            Q[kk] = out[1][t] * out[1][t];
        }
    }
    if ((PART == 0 || PART == 3) && j >= 2) {   // v: R2 += (1/RE) d2v/dz2 ; E_yz = VV3 * (w at y face J)
        R out[2][L];
        const R rr[2] = {a.c10z.r, a.c6z.r}, ss[2] = {a.c10z.s, a.c6z.s};
        WalkVisBack<R> f{a.v + o, n, s, a.f12z};
        zsolve<R, L, M6, 2, MODE>(out, k0, n, rr, ss, f);
        const R Hj1 = a.m.rh[j], a1 = a.m.hdy[j], a2 = a.m.hdy[j - 1];
        const S *W = a.w + o, *Wm = a.w + fidx(g, i, j - 1, 0);
        R *Rp = a.r[1] + o, *E = a.eyz + o;
#pragma unroll
        for (int t = 0; t < L; ++t) {
            const int kk = (k0 + t) * s;
            Rp[kk] = Rp[kk] + RE1 * out[0][t];
            R wy = Hj1 * (a1 * ST::hi(Wm[kk]) + a2 * ST::hi(W[kk]));
            E[kk] = out[1][t] * wy;
        }
    }
}
template <typename R, int L, int PART, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 1024 : TPB) k_zA(StepArgs<R> a) {
    b_zA<R, L, PART, MODE>(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

template <typename R, int L, int MODE>
__device__ __forceinline__ void b_zB(const StepArgs<R> &a, const Blk blk) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoords<L, MODE>(blk, g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    if ((g.n1m & 31) == 0) {
        const int lane = threadIdx.x & 31;
        const long long o0 = fidx(g, i - lane, j, 0), sb = (long long)g.n1m;
        pf_cols(a.exz + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
        pf_cols(a.wsq + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
        pf_cols(a.eyz + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
        pf_cols(a.hh[0] + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
        pf_cols(a.hh[1] + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
    }
    R out[3][L];
    const R rr[3] = {a.c22z.r, a.c22z.r, a.c22z.r}, ss[3] = {a.c22z.s, a.c22z.s, a.c22z.s};
    WalkZB<R> f{a.exz + o, a.wsq + o, a.eyz + o, n, s, a.f24z};
    f.v = (j >= 2);
    zsolve<R, L, WM<R>::M22, 3, MODE>(out, k0, n, rr, ss, f);
    R *H1 = a.hh[0] + o, *H2 = a.hh[1] + o, *H3 = a.hh[2] + o;
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int kk = (k0 + t) * s;
        H1[kk] = H1[kk] + out[0][t];          // d(uw)/dz
        H3[kk] = out[1][t];                   // d(ww)/dz
        if (j >= 2) H2[kk] = H2[kk] + out[2][t];   // d(vw)/dz
    }
}
template <typename R, int L, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 1024 : TPB) k_zB(StepArgs<R> a) {
    b_zB<R, L, MODE>(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// z factor of Crank-Nicolson: r[c] -> d[c] for the three components (the v component at
// J=1 is computed from zeros and never read)
template <typename R, int L, int MODE>
__device__ __forceinline__ void b_zC(const StepArgs<R> &a, R *d0, R *d1, R *d2, const Blk blk) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoords<L, MODE>(blk, g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    if ((g.n1m & 31) == 0) {
        const int lane = threadIdx.x & 31;
        const long long o0 = fidx(g, i - lane, j, 0), sb = (long long)g.n1m;
        pf_cols(a.r[0] + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::MCN), L, n, lane);
        pf_cols(a.r[1] + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::MCN), L, n, lane);
        pf_cols(a.r[2] + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::MCN), L, n, lane);
    }
    R out[3][L];
    const R rr[3] = {a.cnz.r, a.cnz.r, a.cnz.r}, ss[3] = {a.cnz.s, a.cnz.s, a.cnz.s};
    WalkCN<R> f;
    f.X[0] = a.r[0] + o; f.X[1] = a.r[1] + o; f.X[2] = a.r[2] + o;
    f.n = n; f.s = s;
    zsolve<R, L, WM<R>::MCN, 3, MODE>(out, k0, n, rr, ss, f);
    R *D0 = d0 + o, *D1 = d1 + o, *D2 = d2 + o;
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int kk = (k0 + t) * s;
        D0[kk] = out[0][t];
        D1[kk] = out[1][t];
        D2[kk] = out[2][t];
    }
}
template <typename R, int L, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 1024 : TPB) k_zC(StepArgs<R> a, R *d0, R *d1, R *d2) {
    b_zC<R, L, MODE>(a, d0, d1, d2, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// z part of RHSDP: rdpz = compact d(UH3)/dz / DT with UH3 = W + delta3
template <typename R, int L, int MODE>
__device__ __forceinline__ void b_zD(const StepArgs<R> &a, const R *d2, const Blk blk) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoords<L, MODE>(blk, g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    if ((g.n1m & 31) == 0) {
        const int lane = threadIdx.x & 31;
        const long long o0 = fidx(g, i - lane, j, 0), sb = (long long)g.n1m;
        pf_cols(a.w + o0, sb * sizeof(typename SType<R>::S), 32 * (int)sizeof(typename SType<R>::S), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
        pf_cols(d2 + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
    }
    R out[1][L];
    const R rr[1] = {a.c22z.r}, ss[1] = {a.c22z.s};
    WalkDivZ<R> f{a.w + o, d2 + o, n, s, a.f24z};
    zsolve<R, L, WM<R>::M22, 1, MODE>(out, k0, n, rr, ss, f);
    const R rdt = a.rdt;
    R *Q = a.rdpz + o;
#pragma unroll
    for (int t = 0; t < L; ++t) Q[(k0 + t) * s] = out[0][t] * rdt;
}
template <typename R, int L, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 1024 : TPB) k_zD(StepArgs<R> a, const R *d2) {
    b_zD<R, L, MODE>(a, d2, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// UPCALC along z and the state update
template <typename R, int L, int MODE>
__device__ __forceinline__ void b_zE(const StepArgs<R> &a, const R *d0, const R *d1, const R *d2, int updp, const Blk blk) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoords<L, MODE>(blk, g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    const R dt = (R)a.dt;
    const R dtdm = dt * (R)a.scal[SCAL_DMPRESG], dtdm3 = dt * (R)a.scal[SCAL_DMPRESG3];
    const R *DP = a.dp + o;
    if ((g.n1m & 31) == 0) {
        const int lane = threadIdx.x & 31;
        const long long o0 = fidx(g, i - lane, j, 0), sb = (long long)g.n1m;
        pf_cols(a.dp + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, zmargin<MODE>(WM<R>::M22), L, n, lane);
        pf_cols(a.u + o0, sb * sizeof(S), 32 * (int)sizeof(S), k0, 0, L, n, lane);
        pf_cols(a.v + o0, sb * sizeof(S), 32 * (int)sizeof(S), k0, 0, L, n, lane);
        pf_cols(a.w + o0, sb * sizeof(S), 32 * (int)sizeof(S), k0, 0, L, n, lane);
        pf_cols(a.p + o0, sb * sizeof(S), 32 * (int)sizeof(S), k0, 0, L, n, lane);
        if (sizeof(R) == 8) pf_cols(d0 + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
        pf_cols(d1 + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
        pf_cols(d2 + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
        pf_cols(a.g1 + o0, sb * sizeof(R), 32 * (int)sizeof(R), k0, 0, L, n, lane);
    }
    R out[1][L];
    const R rr[1] = {a.c22z.r}, ss[1] = {a.c22z.s};
    WalkGradZ<R> f{DP, n, s, a.f24z};
    zsolve<R, L, WM<R>::M22, 1, MODE>(out, k0, n, rr, ss, f);
    S *W = a.w + o, *U = a.u + o, *V = a.v + o, *Pp = a.p + o;
    const R *D0 = d0 + o, *D1 = d1 + o, *D2 = d2 + o, *G1 = a.g1 + o;
    const R *DPm = a.dp + fidx(g, i, j - 1, 0);
    const R rHj = a.m.rh[j];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int kk = (k0 + t) * s;
        W[kk] = Sten<R>::upd(W[kk], D2[kk], dt * out[0][t], dtdm3);
        if constexpr (sizeof(R) == 4) U[kk] = ST::add(U[kk], G1[kk] - dtdm);   // G1: delta1 - DT dDP/dx (xD)
        else U[kk] = Sten<R>::upd(U[kk], D0[kk], dt * G1[kk], dtdm);
        if (j >= 2) V[kk] = Sten<R>::upd(V[kk], D1[kk], dt * (DP[kk] - DPm[kk]) * rHj, R(0));
        if (updp) Pp[kk] = ST::add(Pp[kk], DP[kk]);
    }
}
template <typename R, int L, int MODE>
__global__ void __launch_bounds__(MODE == 1 ? 1024 : TPB) k_zE(StepArgs<R> a, const R *d0, const R *d1, const R *d2, int updp) {
    b_zE<R, L, MODE>(a, d0, d1, d2, updp, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// DIVCHECK z part and max |div| (FP64)
template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_diag_z(StepArgs<R> a, const double *divx, Cyc<double> c22) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    const Geo g = a.g;
    int i, j, k0;
    double m = 0.0;
    int bad = 0;
    if (zcoord<L>(g, 1, i, j, k0)) {
        const int n = g.n3m, s = g.n1m;
        const long long o = fidx(g, i, j, 0);
        const S *W = a.w + o;
        const double *DX = divx + o;
        double out[L];
        zseg<double, L>(out, k0, n, c22, [&](int kk) {
            int kp = kk == n - 1 ? 0 : kk + 1;
            return 24.0 * g.dx3 * (ST::dbl(W[kp * s]) - ST::dbl(W[kk * s]));
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

template <typename R, int L, int MODE>
static int launch_zpass_l(c3d_channel *ch, StepArgs<R> &a, int which, R *d0, R *d1, R *d2, int flag, int *nl);

// Segment length of the block form (MODE 1) for N3M points: the smallest of 8, 12, 16
// that divides N3M into at most 32 segments, or 0 when none does.
int zblock_len(int n3m) {
    for (int L : {8, 12, 16})
        if (n3m % L == 0 && n3m / L <= 32) return L;
    return 0;
}

// ---------------------------------------------------------------------------------
// Batch form: one launch per pass covers every channel (segment form, segments of ZL
// points, which divides every supported N3M); zA as its three sweeps; the work arrays
// are the channel's exz / eyz / wsq as in the step, and zE adds DP to P.
// ---------------------------------------------------------------------------------
template <typename R, int PART, int L>
__global__ void __launch_bounds__(TPB) kb_zA(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_zA<R, L, PART, 0>(A[m.ch], Blk{m.x, m.y, m.gx});
}
template <typename R, int L>
__global__ void __launch_bounds__(TPB) kb_zB(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_zB<R, L, 0>(A[m.ch], Blk{m.x, m.y, m.gx});
}
template <typename R, int L>
__global__ void __launch_bounds__(TPB) kb_zC(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_zC<R, L, 0>(a, a.exz, a.eyz, a.wsq, Blk{m.x, m.y, m.gx});
}
template <typename R, int L>
__global__ void __launch_bounds__(TPB) kb_zD(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_zD<R, L, 0>(a, a.wsq, Blk{m.x, m.y, m.gx});
}
template <typename R, int L>
__global__ void __launch_bounds__(TPB) kb_zE(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_zE<R, L, 0>(a, a.exz, a.eyz, a.wsq, 1, Blk{m.x, m.y, m.gx});
}

template <typename R, int L>
static int zbk(const c3d_channel *ch, int which, std::vector<BKern> &out) {
    const unsigned nb = (unsigned)nblk((long long)ch->g.n2m * (ch->g.n3m / L) * ch->g.n1m);
    switch (which) {
        case 0:
            out.push_back({(const void *)kb_zA<R, 1, L>, TPB, 0, nb, 2, 0});
            out.push_back({(const void *)kb_zA<R, 2, L>, TPB, 0, nb, 2, 1});
            out.push_back({(const void *)kb_zA<R, 3, L>, TPB, 0, nb, 2, 2});
            return 0;
        case 1: out.push_back({(const void *)kb_zB<R, L>, TPB, 0, nb}); return 0;
        case 2: out.push_back({(const void *)kb_zC<R, L>, TPB, 0, nb}); return 0;
        case 3: out.push_back({(const void *)kb_zD<R, L>, TPB, 0, nb}); return 0;
        case 4: out.push_back({(const void *)kb_zE<R, L>, TPB, 0, nb}); return 0;
        default: return C3D_EINVAL;
    }
}

// z pass `which` of a batch channel in segments of L points (8, 16 or 32; 16 where N3M
// is not a multiple of L).
template <typename R>
int zpass_bkern(const c3d_channel *ch, int which, int L, std::vector<BKern> &out) {
    if (ch->g.n3m % ZL != 0) return C3D_EINVAL;
    if (L != 8 && L != 32) L = 16;
    if (ch->g.n3m % L != 0) L = 16;
    if (L == 8) return zbk<R, 8>(ch, which, out);
    if (L == 32) return zbk<R, 32>(ch, which, out);
    return zbk<R, 16>(ch, which, out);
}
template int zpass_bkern<double>(const c3d_channel *, int, int, std::vector<BKern> &);
template int zpass_bkern<float>(const c3d_channel *, int, int, std::vector<BKern> &);

template <typename R>
int launch_zpass(c3d_channel *ch, StepArgs<R> &a, int which, R *d0, R *d1, R *d2, int flag, int *nl) {
    if (which == 5) return launch_zpass_l<R, ZL, 0>(ch, a, which, d0, d1, d2, flag, nl);
    const int zl = ch->tune.zl[which];
    if (zl == 0) {   // block form; a shape it cannot take runs the segment form with L = 16
        switch (zblock_len(ch->g.n3m)) {
            case 8: return launch_zpass_l<R, 8, 1>(ch, a, which, d0, d1, d2, flag, nl);
            case 12: return launch_zpass_l<R, 12, 1>(ch, a, which, d0, d1, d2, flag, nl);
            case 16: return launch_zpass_l<R, 16, 1>(ch, a, which, d0, d1, d2, flag, nl);
            default: return launch_zpass_l<R, 16, 0>(ch, a, which, d0, d1, d2, flag, nl);
        }
    }
    switch (zl) {
        case 8: return launch_zpass_l<R, 8, 0>(ch, a, which, d0, d1, d2, flag, nl);
        case 32: return launch_zpass_l<R, 32, 0>(ch, a, which, d0, d1, d2, flag, nl);
        default: return launch_zpass_l<R, 16, 0>(ch, a, which, d0, d1, d2, flag, nl);
    }
}

template <typename R, int L, int MODE>
static int launch_zpass_l(c3d_channel *ch, StepArgs<R> &a, int which, R *d0, R *d1, R *d2, int flag, int *nl) {
    const long long nt = (long long)ch->g.n2m * (ch->g.n3m / L) * ch->g.n1m;
    // MODE 0: TPB-thread blocks over all threads; MODE 1: (N1M/32, N2M) blocks of 32 x N3M/L
    const dim3 nb = MODE == 1 ? dim3(ch->g.n1m / 32, ch->g.n2m) : dim3(nblk(nt));
    const dim3 TB = MODE == 1 ? dim3(32, ch->g.n3m / L) : dim3(TPB);
    const size_t zsm = MODE == 1 ? 3 * 32 * (size_t)(ch->g.n3m / L + 1) * sizeof(R) : 0;
    cudaStream_t st = ch->stream;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    switch (which) {
        case 0:
            if (ch->tune.zsplit) {   // u, (w, P), v sweeps as three kernels
                // as concurrent branches with knob 15: each writes its own R component and
                // product, and they share only inputs that none of them writes
                const bool cc = par_on(ch);
                int rc;
                if (cc && (rc = par_fork(ch))) return rc;
                k_zA<R, L, 1, MODE><<<nb, TB, zsm, cc ? ch->par[0] : st>>>(a);
                mark(ch, nl, "zA_u", N * (8 + 4 * Rb));    // u; WW1, R1 -> R1, E_xz
                k_zA<R, L, 2, MODE><<<nb, TB, zsm, cc ? ch->par[1] : st>>>(a);
                mark(ch, nl, "zA_wp", N * (16 + 3 * Rb));  // w, P; R3 -> R3, WW3^2
                k_zA<R, L, 3, MODE><<<nb, TB, zsm, st>>>(a);
                mark(ch, nl, "zA_v", N * (16 + 3 * Rb));   // v, w; R2 -> R2, E_yz
                if (cc && (rc = par_join(ch))) return rc;
            } else {
                k_zA<R, L, 0, MODE><<<nb, TB, zsm, st>>>(a);
                mark(ch, nl, "zA", N * (32 + 10 * Rb));
            }
            break;
        case 1: k_zB<R, L, MODE><<<nb, TB, zsm, st>>>(a); mark(ch, nl, "zB", N * 8 * Rb); break;
        case 2: k_zC<R, L, MODE><<<nb, TB, zsm, st>>>(a, d0, d1, d2); mark(ch, nl, "zC", N * 6 * Rb); break;
        case 3: k_zD<R, L, MODE><<<nb, TB, zsm, st>>>(a, d2); mark(ch, nl, "zD", N * (8 + 2 * Rb)); break;
        case 4:   // the mixed form reads delta1 - DT dDP/dx from one field (xD), FP64 both
            k_zE<R, L, MODE><<<nb, TB, zsm, st>>>(a, d0, d1, d2, flag);
            mark(ch, nl, "zE", N * (64 + (sizeof(R) == 4 ? 4 : 5) * Rb));
            break;
        case 5: {
            if (MODE == 1) return C3D_EINVAL;   // the diagnostics run the segment form only
            const double b = 22.0, r = -2.0 / (b + sqrt(b * b - 4.0));
            Cyc<double> c22 = {r, -r, (int)ceil(log(1e-17) / log(fabs(r)))};
            k_diag_z<R, L><<<nb, TB, zsm, st>>>(a, (const double *)d0, c22);
            mark(ch, nl, "diag_z", N * 16);
            break;
        }
        default: return C3D_EINVAL;
    }
    return 0;
}

template int launch_zpass<double>(c3d_channel *, StepArgs<double> &, int, double *, double *, double *, int, int *);
template int launch_zpass<float>(c3d_channel *, StepArgs<float> &, int, float *, float *, float *, int, int *);

}  // namespace c3d
