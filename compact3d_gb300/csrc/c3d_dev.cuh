// c3d_dev.cuh -- device-side layout and line-solver primitives of the GB300 channel step.
//
// Layout in HBM.  Every 3-D field is plane-major: element (i, j, k) of a field lives at
//   ((j * N3M) + k) * N1M + i,   i in [0,N1M), k in [0,N3M), j in [0, N2]
// with i = I-1, k = K-1 and j = J of the reference's Fortran indices.  One x-z plane
// (N1M*N3M values) is contiguous, rows along x are contiguous, and the wall planes
// j = 0 and j = N2 are stored like interior planes.  The periodic x and z directions
// carry no halo: the kernels wrap indices.
//
// Compact (Pade) operators.  The reference solves constant-coefficient cyclic systems
//   a x_{i-1} + b x_i + a x_{i+1} = d_i                 (CTDMA11/33, CTDMA1J/3I)
// by bordered LU.  With beta = b/a and r the root of r^2 + beta r + 1 = 0 with |r| < 1,
//   tridiag(a, b, a) = (-a/r) (1 - r S)(1 - r S^-1)      (S = cyclic shift)
// so x = s * B(F(d)) with s = -r/a, F: y_i = d_i + r y_{i-1} and B: z_i = y_i + r z_{i+1},
// both cyclic.  The kernels evaluate these two first-order recurrences:
//   * along x (contiguous rows): one warp per row (or, for rows of 48-128 points, a
//     segment of 8 or 16 lanes per row), every lane owns C consecutive points, and the
//     cyclic carries between lanes come from shuffle scans of affine maps;
//   * along z (strided columns): one thread per (column, segment of L points); the cyclic
//     start values come from a warm-up of M points, M chosen so |r|^M is below the
//     working precision's rounding unit.
// The result equals the reference's bordered-LU solution to rounding.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace c3d {

constexpr unsigned FULL = 0xffffffffu;

// Coefficients of one constant-coefficient cyclic operator in a given precision.
template <typename R>
struct Cyc {
    R r;      // root of r^2 + (b/a) r + 1 = 0, |r| < 1
    R s;      // output scale -r/a
    int m;    // warm-up length for segment solves
};

// Geometry and constants handed to every kernel by value.
struct Geo {
    int n1m, n2m, n3m, n2;   // cells; n2 = N2 = n2m + 1
    int np;                  // n1m * n3m (plane)
    long long nf;            // (n2 + 1) * np (field)
    int n1h;                 // n1m/2 + 1 (half spectrum along x)
    double dx1, dx3, dx1q, dx3q, re, alx, aly, alz, vol;
    // y metrics indexed by Fortran J (arrays of n2+1 values, entry 0 = DY(0) etc.);
    // hz = HP+HM-HC and dyz = DYP+DYM-DYC are zero up to rounding (used by the mixed form)
    const double *dy, *h, *hp, *hc, *hm, *dyp, *dyc, *dym, *hz, *dyz;
};

__host__ __device__ inline long long fidx(const Geo &g, int i, int j, int k) {
    return ((long long)j * g.n3m + k) * g.n1m + i;
}

// ---------------------------------------------------------------------------------
// x direction: warp per row, lane chunks of C points, P = N1M / C active lanes (the
// lane_* helpers; the kernels' segmented forms use sprev/snext/xsolve with a width).
// ---------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T lane_prev(T last, int lane, int P) {
    int src = (lane == 0) ? P - 1 : lane - 1;
    return __shfl_sync(FULL, last, src);
}
template <typename T>
__device__ __forceinline__ T lane_next(T first, int lane, int P) {
    int src = (lane + 1 >= P) ? 0 : lane + 1;
    return __shfl_sync(FULL, first, src);
}

// Double-float value hi + lo (about 48 significant bits) made of FP32 operations: error-
// free two-sum (Knuth) and FMA-based two-product.  The line solvers are templates on the
// value type, so the same recurrences run in double-float where a result must be
// accurate well below FP32 rounding (the residual of the pressure refinement).
struct dfl {
    float h, l;
    __host__ __device__ dfl() : h(0.f), l(0.f) {}
    __host__ __device__ dfl(float x) : h(x), l(0.f) {}
    __host__ __device__ dfl(float a, float b) : h(a), l(b) {}
    static __host__ dfl from(double x) {
        float a = (float)x;
        return dfl(a, (float)(x - (double)a));
    }
};
__device__ __forceinline__ dfl dfl_norm(float s, float e) {
    float h = s + e;
    return dfl(h, e - (h - s));
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
    float s = a.h + b.h, v = s - a.h;
    float e = (a.h - (s - v)) + (b.h - v);
    return dfl_norm(s, e + (a.l + b.l));
}
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + dfl(-b.h, -b.l); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return dfl_norm(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
    float q1 = a.h / b.h;
    dfl r = a - dfl(q1) * b;
    float q2 = r.h / b.h;
    dfl q = dfl_norm(q1, q2);
    r = a - q * b;
    return q + dfl(r.h / b.h);
}
__device__ __forceinline__ dfl &operator+=(dfl &a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl &operator*=(dfl &a, dfl b) { return a = a * b; }

// Warp shuffles for every value type of the line solvers.
// Shuffles within segments of w lanes (w = 32: the whole warp); lane indexes and
// offsets are relative to the segment.
__device__ __forceinline__ double shfl_up(double v, int d, int w = 32) { return __shfl_up_sync(FULL, v, d, w); }
__device__ __forceinline__ float shfl_up(float v, int d, int w = 32) { return __shfl_up_sync(FULL, v, d, w); }
__device__ __forceinline__ dfl shfl_up(dfl v, int d, int w = 32) {
    return dfl(__shfl_up_sync(FULL, v.h, d, w), __shfl_up_sync(FULL, v.l, d, w));
}
__device__ __forceinline__ double shfl_down(double v, int d, int w = 32) { return __shfl_down_sync(FULL, v, d, w); }
__device__ __forceinline__ float shfl_down(float v, int d, int w = 32) { return __shfl_down_sync(FULL, v, d, w); }
__device__ __forceinline__ dfl shfl_down(dfl v, int d, int w = 32) {
    return dfl(__shfl_down_sync(FULL, v.h, d, w), __shfl_down_sync(FULL, v.l, d, w));
}
__device__ __forceinline__ double shfl_idx(double v, int s, int w = 32) { return __shfl_sync(FULL, v, s, w); }
__device__ __forceinline__ float shfl_idx(float v, int s, int w = 32) { return __shfl_sync(FULL, v, s, w); }
__device__ __forceinline__ dfl shfl_idx(dfl v, int s, int w = 32) {
    return dfl(__shfl_sync(FULL, v.h, s, w), __shfl_sync(FULL, v.l, s, w));
}

// 1 - x rounds to 1 (so that y / (1 - x) is y exactly) for |x| below half an ulp of 1.
__device__ __forceinline__ bool below_half_ulp(float x) { return fabsf(x) < 0x1p-25f; }
__device__ __forceinline__ bool below_half_ulp(double x) { return fabs(x) < 0x1p-54; }
template <typename R>
__device__ __forceinline__ bool below_half_ulp(R) { return false; }

// xsolve for a row whose every lane holds a chunk (P = W): every lane's chunk multiplier is
// r^C, so the scans combine with the constant powers r^(C 2^b) (one shuffle and one
// multiply-add per level), the chunk sweeps carry no multiplier, and the cyclic closure
// y / (1 - r^(C W)) needs no division once r^(C W) is below half an ulp.  The powers are
// formed with the same products, in the same order, as the general form forms its
// multipliers at each level.
template <int W, typename R, int C>
__device__ __forceinline__ void xsolve_full(R (&x)[C], int lane, const Cyc<R> &c) {
    constexpr int LW = W == 32 ? 5 : W == 16 ? 4 : W == 8 ? 3 : 2;
    const R r = c.r;
    R pw[LW + 1];
    {
        R m = R(1);
#pragma unroll
        for (int t = 0; t < C; ++t) m *= r;
        pw[0] = m;
#pragma unroll
        for (int b = 0; b < LW; ++b) pw[b + 1] = pw[b] * pw[b];
    }
    R ml = R(1), mr = R(1);   // r^(C lane) and r^(C (W - 1 - lane))
#pragma unroll
    for (int b = 0; b < LW; ++b) {
        if ((lane >> b) & 1) ml = ml * pw[b];
        if (((W - 1 - lane) >> b) & 1) mr = mr * pw[b];
    }
    const bool exact1 = below_half_ulp(pw[LW]);
    R y = R(0);
#pragma unroll
    for (int t = 0; t < C; ++t) y = x[t] + r * y;
    R e = y;
#pragma unroll
    for (int b = 0; b < LW; ++b) {
        const int off = 1 << b;
        const R ep = shfl_up(e, off, W);
        if (lane >= off) e = e + pw[b] * ep;
    }
    {
        const R et = shfl_idx(e, W - 1, W);
        const R y0 = exact1 ? et : et / (R(1) - pw[LW]);
        const R ex = shfl_up(e, 1, W);
        y = (lane == 0) ? y0 : ex + ml * y0;
    }
#pragma unroll
    for (int t = 0; t < C; ++t) {
        y = x[t] + r * y;
        x[t] = y;
    }
    R z = R(0);
#pragma unroll
    for (int t = C - 1; t >= 0; --t) z = x[t] + r * z;
    e = z;
#pragma unroll
    for (int b = 0; b < LW; ++b) {
        const int off = 1 << b;
        const R en = shfl_down(e, off, W);
        if (lane + off < W) e = e + pw[b] * en;
    }
    {
        const R e0 = shfl_idx(e, 0, W);
        const R z0 = exact1 ? e0 : e0 / (R(1) - pw[LW]);
        const R en1 = shfl_down(e, 1, W);
        z = (lane == W - 1) ? z0 : en1 + mr * z0;
    }
    const R s = c.s;
#pragma unroll
    for (int t = C - 1; t >= 0; --t) {
        z = x[t] + r * z;
        x[t] = s * z;
    }
}

// Cyclic solve on a row held as lane chunks x[0..C) by a segment of W lanes (lane =
// the lane within the segment; W = 32: one row per warp, W < 32: 32/W rows per warp,
// every segment of the warp calling together); in place, returns s*B(F(x)).  P = W takes
// the constant-multiplier form above; P < W (idle lanes) the general one.
template <int W = 32, typename R, int C>
__device__ __forceinline__ void xsolve(R (&x)[C], int lane, int P, const Cyc<R> &c) {
    static_assert(W == 4 || W == 8 || W == 16 || W == 32, "row segments of 4, 8, 16 or 32 lanes");
    if (P == W) {
        xsolve_full<W>(x, lane, c);
        return;
    }
    const bool act = lane < P;
    const R r = c.r;
    R y = R(0), m = R(1);
#pragma unroll
    for (int t = 0; t < C; ++t) {
        y = x[t] + r * y;
        m *= r;
    }
    R e = act ? y : R(0);
    if (!act) m = R(1);
#pragma unroll
    for (int off = 1; off < W; off <<= 1) {
        R ep = shfl_up(e, off, W), mp = shfl_up(m, off, W);
        if (lane >= off) {
            e = e + m * ep;
            m = m * mp;
        }
    }
    {
        R et = shfl_idx(e, W - 1, W), mt = shfl_idx(m, W - 1, W);
        R y0 = et / (R(1) - mt);
        R ex = shfl_up(e, 1, W), mx = shfl_up(m, 1, W);
        y = (lane == 0) ? y0 : ex + mx * y0;
    }
#pragma unroll
    for (int t = 0; t < C; ++t) {
        y = x[t] + r * y;
        x[t] = y;
    }
    R z = R(0);
    m = R(1);
#pragma unroll
    for (int t = C - 1; t >= 0; --t) {
        z = x[t] + r * z;
        m *= r;
    }
    e = act ? z : R(0);
    if (!act) m = R(1);
#pragma unroll
    for (int off = 1; off < W; off <<= 1) {
        R en = shfl_down(e, off, W), mn = shfl_down(m, off, W);
        if (lane + off < W) {
            e = e + m * en;
            m = m * mn;
        }
    }
    {
        R e0 = shfl_idx(e, 0, W), m0 = shfl_idx(m, 0, W);
        R z0 = e0 / (R(1) - m0);
        R en1 = shfl_down(e, 1, W), mn1 = shfl_down(m, 1, W);
        z = (lane == W - 1) ? z0 : en1 + mn1 * z0;
    }
    const R s = c.s;
#pragma unroll
    for (int t = C - 1; t >= 0; --t) {
        z = x[t] + r * z;
        x[t] = s * z;
    }
}

// Lane-chunk load/store of one row (row pointer + lane*C).  Inactive lanes are skipped.
template <int C>
__device__ __forceinline__ void row_load(double (&v)[C], const double *__restrict__ row, int lane, int P) {
    if (lane < P) {
        const double *p = row + lane * C;
        if constexpr (C % 2 == 0) {
#pragma unroll
            for (int t = 0; t < C; t += 2) {
                double2 q = __ldg(reinterpret_cast<const double2 *>(p + t));
                v[t] = q.x;
                v[t + 1] = q.y;
            }
        } else {
#pragma unroll
            for (int t = 0; t < C; ++t) v[t] = __ldg(p + t);
        }
    } else {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = 0.0;
    }
}
template <int C>
__device__ __forceinline__ void row_load(float (&v)[C], const float *__restrict__ row, int lane, int P) {
    if (lane < P) {
        const float *p = row + lane * C;
        if constexpr (C % 4 == 0) {
#pragma unroll
            for (int t = 0; t < C; t += 4) {
                float4 q = __ldg(reinterpret_cast<const float4 *>(p + t));
                v[t] = q.x; v[t + 1] = q.y; v[t + 2] = q.z; v[t + 3] = q.w;
            }
        } else if constexpr (C % 2 == 0) {
#pragma unroll
            for (int t = 0; t < C; t += 2) {
                float2 q = __ldg(reinterpret_cast<const float2 *>(p + t));
                v[t] = q.x; v[t + 1] = q.y;
            }
        } else {
#pragma unroll
            for (int t = 0; t < C; ++t) v[t] = __ldg(p + t);
        }
    } else {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = 0.f;
    }
}
template <typename T, int C>
__device__ __forceinline__ void row_store(T *__restrict__ row, const T (&v)[C], int lane, int P) {
    if (lane < P) {
        T *p = row + lane * C;
#pragma unroll
        for (int t = 0; t < C; ++t) p[t] = v[t];
    }
}

// ---------------------------------------------------------------------------------
// z direction: thread per (column, segment of L points) with warm-up M.
// D(k) is a functor returning the right-hand side at wrapped index k in [0,n).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int wrapi(int q, int n) {
    while (q < 0) q += n;
    while (q >= n) q -= n;
    return q;
}

template <typename R, int L, typename F>
__device__ __forceinline__ void zseg(R (&out)[L], int k0, int n, const Cyc<R> &c, F D) {
    const R r = c.r;
    R y = R(0);
    int kk = wrapi(k0 - c.m, n);
    for (int q = 0; q < c.m; ++q) {
        y = D(kk) + r * y;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R ys[L];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        y = D(kk) + r * y;
        ys[t] = y;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R acc = R(0), pw = R(1);
    for (int q = 0; q < c.m; ++q) {
        y = D(kk) + r * y;
        acc = acc + pw * y;
        pw *= r;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R z = acc;
    const R s = c.s;
#pragma unroll
    for (int t = L - 1; t >= 0; --t) {
        z = ys[t] + r * z;
        out[t] = s * z;
    }
}

// The same with the warm-up length M a compile-time constant, so that every loop unrolls
// and the loads of D can be issued ahead of the recurrence.
template <typename R, int L, int M, typename F>
__device__ __forceinline__ void zsegm(R (&out)[L], int k0, int n, const Cyc<R> &c, F D) {
    const R r = c.r;
    R y = R(0);
    int kk = wrapi(k0 - M, n);
#pragma unroll
    for (int q = 0; q < M; ++q) {
        y = D(kk) + r * y;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R ys[L];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        y = D(kk) + r * y;
        ys[t] = y;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R acc = R(0), pw = R(1);
#pragma unroll
    for (int q = 0; q < M; ++q) {
        y = D(kk) + r * y;
        acc = acc + pw * y;
        pw *= r;
        kk = (kk + 1 == n) ? 0 : kk + 1;
    }
    R z = acc;
    const R s = c.s;
#pragma unroll
    for (int t = L - 1; t >= 0; --t) {
        z = ys[t] + r * z;
        out[t] = s * z;
    }
}

// Several cyclic solves along one column in a single sweep.  The functor f walks the
// column once, in order, from position k0 - M (wrapped): f.start(k) positions it and
// f.next(d) returns the NR right-hand sides at the current position and advances, so it
// can keep a sliding window of the stencil inputs in registers and load one new value per
// position.  Recurrence q uses root r[q] and scale s[q]; M is the largest warm-up needed.
template <typename R, int L, int M, int NR, typename F>
__device__ __forceinline__ void zsweep(R (&out)[NR][L], int k0, int n, const R (&r)[NR], const R (&s)[NR], F &f) {
    f.start(wrapi(k0 - M, n));
    R y[NR], d[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) y[q] = R(0);
#pragma unroll
    for (int t = 0; t < M; ++t) {
        f.next(d);
#pragma unroll
        for (int q = 0; q < NR; ++q) y[q] = d[q] + r[q] * y[q];
    }
    R ys[NR][L];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        f.next(d);
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            y[q] = d[q] + r[q] * y[q];
            ys[q][t] = y[q];
        }
    }
    R acc[NR], pw[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) { acc[q] = R(0); pw[q] = R(1); }
#pragma unroll
    for (int t = 0; t < M; ++t) {
        f.next(d);
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            y[q] = d[q] + r[q] * y[q];
            acc[q] = acc[q] + pw[q] * y[q];
            pw[q] *= r[q];
        }
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        R z = acc[q];
#pragma unroll
        for (int t = L - 1; t >= 0; --t) {
            z = ys[q][t] + r[q] * z;
            out[q][t] = s[q] * z;
        }
    }
}

// Cyclic carries of the segments of the block's z lines (zblock): for every recurrence q
// and line l, a warp takes the nseg segment values v[p] = sh[(q*32 + l)*(nseg+1) + p] in
// its lanes and replaces them by the state entering each segment.  Forward (BACK false):
// Y(p) = v(p-1) + rL Y(p-1) cyclically, i.e. Y(p) = E(p-1) + rL^p Y(0) with the prefix
// E(p) = v(p) + rL E(p-1) and Y(0) = E(nseg-1) / (1 - rL^nseg).  Backward: the mirror
// image, Z(p) = v(p+1) + rL Z(p+1) from the right.  Warp-shuffle scans, log2(32) steps.
template <typename R, int L, int NR, bool BACK>
__device__ __forceinline__ void zcarry(const R (&r)[NR], R *sh) {
    const int lane = threadIdx.x, w = threadIdx.y, nw = blockDim.y, nseg = blockDim.y;
    const int pitch = nseg + 1;
    for (int sidx = w; sidx < 32 * NR; sidx += nw) {
        const int q = sidx >> 5, l = sidx & 31;
        R rq = R(0);
#pragma unroll
        for (int t = 0; t < NR; ++t)
            if (t == q) rq = r[t];
        R rL = R(1);
#pragma unroll
        for (int t = 0; t < L; ++t) rL *= rq;
        R *v = sh + (q * 32 + l) * pitch;
        const int p = BACK ? nseg - 1 - lane : lane;   // position along the scan direction
        const bool act = lane < nseg;
        R e = act ? v[p] : R(0);
        R pw = rL;   // rL^off
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const R ep = shfl_up(e, off);
            if (lane >= off) e = e + pw * ep;
            pw = pw * pw;
        }
        // rL^lane and rL^nseg by repeated squaring
        R pl = R(1), pn = R(1), b = rL;
#pragma unroll
        for (int bit = 0; bit < 6; ++bit) {
            if ((lane >> bit) & 1) pl = pl * b;
            if ((nseg >> bit) & 1) pn = pn * b;
            b = b * b;
        }
        const R tot = shfl_idx(e, nseg - 1);
        const R y0 = tot / (R(1) - pn);
        const R eprev = shfl_up(e, 1);
        const R yin = (lane == 0 ? R(0) : eprev) + pl * y0;
        if (act) v[p] = yin;
    }
}

// Exact cyclic solve of NR recurrences on z lines by one block of 32 lines (threadIdx.x,
// consecutive i) x nseg segments of L points (threadIdx.y; nseg = blockDim.y = N / L,
// at most 32).  Each thread walks only its own segment: a local forward recurrence from
// zero, the carries across the segments of its line (zcarry), the correction
// y(t) += r^(t+1) Y, and the same backward.  sh holds NR*32*(nseg+1) values.  Every
// thread of the block calls it (it synchronises the block).
template <typename R, int L, int NR, typename F>
__device__ __forceinline__ void zblock(R (&out)[NR][L], int k0, const R (&r)[NR], const R (&s)[NR], F &f, R *sh) {
    const int lx = threadIdx.x, seg = threadIdx.y, pitch = blockDim.y + 1;
    f.start(k0);
    R y[NR], d[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) y[q] = R(0);
#pragma unroll
    for (int t = 0; t < L; ++t) {
        f.next(d);
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            y[q] = d[q] + r[q] * y[q];
            out[q][t] = y[q];
        }
    }
    __syncthreads();   // a previous call's readers of sh are done
#pragma unroll
    for (int q = 0; q < NR; ++q) sh[(q * 32 + lx) * pitch + seg] = y[q];
    __syncthreads();
    zcarry<R, L, NR, false>(r, sh);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const R yin = sh[(q * 32 + lx) * pitch + seg];
        R pw = r[q];
#pragma unroll
        for (int t = 0; t < L; ++t) {
            out[q][t] = out[q][t] + pw * yin;
            pw *= r[q];
        }
    }
    __syncthreads();   // sh is reused
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        R z = R(0);
#pragma unroll
        for (int t = L - 1; t >= 0; --t) {
            z = out[q][t] + r[q] * z;
            out[q][t] = z;
        }
        sh[(q * 32 + lx) * pitch + seg] = z;
    }
    __syncthreads();
    zcarry<R, L, NR, true>(r, sh);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const R zin = sh[(q * 32 + lx) * pitch + seg];
        R pw = r[q];
#pragma unroll
        for (int t = L - 1; t >= 0; --t) {
            out[q][t] = s[q] * (out[q][t] + pw * zin);
            pw *= r[q];
        }
    }
}

// Warm-up lengths M = ceil(log(tol)/log|r|) of the Pade operators (1,6,1), (1,10,1),
// (1,22,1) and the Crank-Nicolson operators (b/a > 10, so M <= M10): tol = 1e-17 in FP64,
// 3e-8 in FP32.
template <typename R> struct WM;
template <> struct WM<double> { static constexpr int M6 = 23, M10 = 18, M22 = 13, MCN = 18; };
template <> struct WM<float> { static constexpr int M6 = 10, M10 = 8, M22 = 6, MCN = 8; };

}  // namespace c3d
