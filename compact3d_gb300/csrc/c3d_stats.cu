// c3d_stats.cu -- ENERGY's plane statistics (compact3d.f:10003-10232) on the device, FP64:
// per plane J the cell-centre means, second moments, vorticity statistics, the two third
// moments ENERGY keeps, the third and fourth central moments and the mean wall-normal
// gradients (29 values; the column order is that of c3d_plane_stats in include/c3d.h).
// Each plane is split over SB blocks; partial sums are combined in a fixed order.
#include "c3d_kern.cuh"

namespace c3d {

constexpr int SB = 8;        // blocks per plane
constexpr int STB = 128;     // threads per block
constexpr int NS1 = 23;      // first-pass sums: 20 moments + 3 gradients

template <typename R>
__device__ __forceinline__ double sv(const typename SType<R>::S *a, const Geo &g, int i, int j, int k) {
    return St<R>::dbl(a[fidx(g, i, j, k)]);
}

// Cell-centre velocities, pressure, vorticity and the wall-normal gradients at (i, j, k)
// (0-based i, k; plane j = 1..N2M), as ENERGY's loops 10, 20 and 40.
template <typename R>
__device__ void point_terms(const StepArgs<R> &a, int i, int j, int k, double v[3], double &pp, double w[3],
                            double d[3]) {
    typedef typename SType<R>::S S;
    const Geo &g = a.g;
    const S *U = a.u, *V = a.v, *W = a.w;
    const int ip = i + 1 == g.n1m ? 0 : i + 1, im = i == 0 ? g.n1m - 1 : i - 1;
    const int kp = k + 1 == g.n3m ? 0 : k + 1, km = k == 0 ? g.n3m - 1 : k - 1;
    const int jp = j + 1, jm = j - 1, n2 = g.n2;
    const double FJUM = j > 1 ? 1.0 : 0.0, FJUP = j < g.n2m ? 1.0 : 0.0;
    const double *DY = g.dy, *H = g.h;
    const double DX1 = g.dx1, DX3 = g.dx3;
    // loop 10: vorticity
    double U1KP = 0.5 * (sv<R>(U, g, i, j, kp) + sv<R>(U, g, ip, j, kp));
    double U1KM = 0.5 * (sv<R>(U, g, i, j, km) + sv<R>(U, g, ip, j, km));
    double U2KP = 0.5 * (sv<R>(V, g, i, j, kp) + sv<R>(V, g, i, jp, kp));
    double U2KM = 0.5 * (sv<R>(V, g, i, j, km) + sv<R>(V, g, i, jp, km));
    double U2IP = 0.5 * (sv<R>(V, g, ip, j, k) + sv<R>(V, g, ip, jp, k));
    double U2IM = 0.5 * (sv<R>(V, g, im, j, k) + sv<R>(V, g, im, jp, k));
    double U3IP = 0.5 * (sv<R>(W, g, ip, j, k) + sv<R>(W, g, ip, j, kp));
    double U3IM = 0.5 * (sv<R>(W, g, im, j, k) + sv<R>(W, g, im, j, kp));
    double U1JP = 0.5 * (sv<R>(U, g, i, jp, k) + sv<R>(U, g, ip, jp, k));
    double U1JC = 0.5 * (sv<R>(U, g, i, j, k) + sv<R>(U, g, ip, j, k));
    double U1JM = 0.5 * (sv<R>(U, g, i, jm, k) + sv<R>(U, g, ip, jm, k));
    double U12 = 0.5 / H[jp] * (DY[jp] * U1JC + DY[j] * U1JP);
    double U11 = 0.5 / H[j] * (DY[j] * U1JM + DY[jm] * U1JC);
    const double U1N2 = (sv<R>(U, g, i, n2, k) + sv<R>(U, g, ip, n2, k)) * 0.5;
    const double U10 = (sv<R>(U, g, i, 0, k) + sv<R>(U, g, ip, 0, k)) * 0.5;
    U12 = U12 * FJUP + (1. - FJUP) * U1N2;
    U11 = U11 * FJUM + (1. - FJUM) * U10;
    double U3JP = 0.5 * (sv<R>(W, g, i, jp, k) + sv<R>(W, g, i, jp, kp));
    double U3JC = 0.5 * (sv<R>(W, g, i, j, k) + sv<R>(W, g, i, j, kp));
    double U3JM = 0.5 * (sv<R>(W, g, i, jm, k) + sv<R>(W, g, i, jm, kp));
    double U32 = 0.5 / H[jp] * (DY[jp] * U3JC + DY[j] * U3JP);
    double U31 = 0.5 / H[j] * (DY[j] * U3JM + DY[jm] * U3JC);
    const double U3N2 = (sv<R>(W, g, i, n2, k) + sv<R>(W, g, i, n2, kp)) * 0.5;
    const double U30 = (sv<R>(W, g, i, 0, k) + sv<R>(W, g, i, 0, kp)) * 0.5;
    U32 = U32 * FJUP + (1. - FJUP) * U3N2;
    U31 = U31 * FJUM + (1. - FJUM) * U30;
    const double DV3DX2 = (U32 - U31) / DY[j];
    const double DV2DX3 = (U2KP - U2KM) * 0.5 * DX3;
    const double DV3DX1 = (U3IP - U3IM) * 0.5 * DX1;
    const double DV1DX3 = (U1KP - U1KM) * 0.5 * DX3;
    const double DV2DX1 = (U2IP - U2IM) * 0.5 * DX1;
    const double DV1DX2 = (U12 - U11) / DY[j];
    w[0] = DV3DX2 - DV2DX3;
    w[1] = DV1DX3 - DV3DX1;
    w[2] = DV2DX1 - DV1DX2;
    // loop 20: cell-centre values
    v[0] = U1JC;
    v[1] = (sv<R>(V, g, i, j, k) + sv<R>(V, g, i, jp, k)) * 0.5;
    v[2] = U3JC;
    pp = St<R>::dbl(a.p[fidx(g, i, j, k)]);
    // loop 40: wall-normal gradients (ENERGY writes these interpolants in another order)
    const double U_JP = U1JP, U_JC = U1JC, U_JM = U1JM, W_JP = U3JP, W_JC = U3JC, W_JM = U3JM;
    const double G1 = FJUM * (1.0 / H[j] * (DY[j] * U_JM / 2.0 + DY[jm] * U_JC / 2.0)) + (1. - FJUM) * U10;
    const double G2 = FJUP * (1.0 / H[jp] * (DY[j] * U_JP / 2.0 + DY[jp] * U_JC / 2.0)) + (1. - FJUP) * U1N2;
    const double E1 = FJUM * (1.0 / H[j] * (DY[j] * W_JM / 2.0 + DY[jm] * W_JC / 2.0)) + (1. - FJUM) * U30;
    const double E2 = FJUP * (1.0 / H[jp] * (DY[j] * W_JP / 2.0 + DY[jp] * W_JC / 2.0)) + (1. - FJUP) * U3N2;
    d[0] = (G2 - G1) / DY[j];
    d[1] = (sv<R>(V, g, i, jp, k) - sv<R>(V, g, i, j, k)) / DY[j];
    d[2] = (E2 - E1) / DY[j];
}

__device__ __forceinline__ void block_sums(double *acc, int n, double *sh, double *outp) {
    for (int q = 0; q < n; ++q) sh[q * STB + threadIdx.x] = acc[q];
    __syncthreads();
    for (int s = STB / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int q = 0; q < n; ++q) sh[q * STB + threadIdx.x] += sh[q * STB + threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < n; ++q) outp[q] = sh[q * STB];
}

// pass 1: blockIdx.y = plane J - 1, blockIdx.x = part of the plane; partial sums
template <typename R>
__global__ void __launch_bounds__(STB) k_stats1(StepArgs<R> a, double *part) {
    __shared__ double sh[NS1 * STB];
    const Geo &g = a.g;
    const int j = 1 + blockIdx.y;
    const int chunk = (g.np + SB - 1) / SB, e0 = blockIdx.x * chunk, e1 = min(g.np, e0 + chunk);
    double acc[NS1];
#pragma unroll
    for (int q = 0; q < NS1; ++q) acc[q] = 0.0;
    for (int e = e0 + threadIdx.x; e < e1; e += STB) {
        const int i = e % g.n1m, k = e / g.n1m;
        double v[3], w[3], d[3], pp;
        point_terms<R>(a, i, j, k, v, pp, w, d);
        acc[0] += v[0]; acc[1] += v[1]; acc[2] += v[2]; acc[3] += pp;
        acc[4] += w[0]; acc[5] += w[1]; acc[6] += w[2];
        acc[7] += v[0] * v[0]; acc[8] += v[1] * v[1]; acc[9] += v[2] * v[2];
        acc[10] += v[0] * v[1]; acc[11] += v[0] * v[2]; acc[12] += v[1] * v[2];
        acc[13] += pp * pp; acc[14] += pp * v[1];
        acc[15] += w[0] * w[0]; acc[16] += w[1] * w[1]; acc[17] += w[2] * w[2];
        acc[18] += v[0] * v[0] * v[1]; acc[19] += v[1] * v[2] * v[2];
        acc[20] += d[0]; acc[21] += d[1]; acc[22] += d[2];
    }
    block_sums(acc, NS1, sh, part + ((size_t)blockIdx.y * SB + blockIdx.x) * NS1);
}

// combine pass 1 (fixed order) into the plane's means: out[J][0..19], [26..28]
__global__ void k_stats1_fin(Geo g, const double *part, double *out) {
    const int j = blockIdx.x, q = threadIdx.x;
    if (q >= NS1) return;
    double s = 0.0;
    for (int b = 0; b < SB; ++b) s += part[((size_t)j * SB + b) * NS1 + q];
    const double m = s / ((double)g.n1m * (double)g.n3m);
    out[(size_t)j * 29 + (q < 20 ? q : q + 6)] = m;
}

// pass 2: third and fourth central moments of the cell-centre velocities
template <typename R>
__global__ void __launch_bounds__(STB) k_stats2(StepArgs<R> a, const double *out, double *part) {
    __shared__ double sh[6 * STB];
    const Geo &g = a.g;
    const int j = 1 + blockIdx.y;
    const double m0 = out[(size_t)(j - 1) * 29 + 0], m1 = out[(size_t)(j - 1) * 29 + 1], m2 = out[(size_t)(j - 1) * 29 + 2];
    const int chunk = (g.np + SB - 1) / SB, e0 = blockIdx.x * chunk, e1 = min(g.np, e0 + chunk);
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int e = e0 + threadIdx.x; e < e1; e += STB) {
        const int i = e % g.n1m, k = e / g.n1m;
        const int ip = i + 1 == g.n1m ? 0 : i + 1, kp = k + 1 == g.n3m ? 0 : k + 1;
        const double V1 = (sv<R>(a.u, g, i, j, k) + sv<R>(a.u, g, ip, j, k)) * 0.5 - m0;
        const double V2 = (sv<R>(a.v, g, i, j, k) + sv<R>(a.v, g, i, j + 1, k)) * 0.5 - m1;
        const double V3 = (sv<R>(a.w, g, i, j, k) + sv<R>(a.w, g, i, j, kp)) * 0.5 - m2;
        acc[0] += V1 * V1 * V1; acc[1] += V2 * V2 * V2; acc[2] += V3 * V3 * V3;
        acc[3] += V1 * V1 * V1 * V1; acc[4] += V2 * V2 * V2 * V2; acc[5] += V3 * V3 * V3 * V3;
    }
    block_sums(acc, 6, sh, part + ((size_t)blockIdx.y * SB + blockIdx.x) * 6);
}

__global__ void k_stats2_fin(Geo g, const double *part, double *out) {
    const int j = blockIdx.x, q = threadIdx.x;
    if (q >= 6) return;
    double s = 0.0;
    for (int b = 0; b < SB; ++b) s += part[((size_t)j * SB + b) * 6 + q];
    out[(size_t)j * 29 + 20 + q] = s / ((double)g.n1m * (double)g.n3m);
}

template <typename R>
int launch_stats_t(c3d_channel *ch, StepArgs<R> &a, double *out, double *part) {
    const Geo &g = ch->g;
    const dim3 grid(SB, g.n2m);
    k_stats1<R><<<grid, STB, 0, ch->stream>>>(a, part);
    k_stats1_fin<<<g.n2m, 32, 0, ch->stream>>>(g, part, out);
    k_stats2<R><<<grid, STB, 0, ch->stream>>>(a, out, part);
    k_stats2_fin<<<g.n2m, 32, 0, ch->stream>>>(g, part, out);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

template int launch_stats_t<double>(c3d_channel *, StepArgs<double> &, double *, double *);
template int launch_stats_t<float>(c3d_channel *, StepArgs<float> &, double *, double *);

// ---------------------------------------------------------------------------------
// ENERGY's 1-D spectra and two-point correlations (compact3d.f:10243-10515), FP64.
// Spectra: one block of SPW warps per (plane, component); warp w transforms the lines
// w, w + SPW, ... with the channel's Stockham plans and double twiddles: an x line of
// N1M reals as N1M/2 complex pairs, then the real-input split, giving |X_k|^2 for
// k <= N1M/2 (the rest mirrored); a z line as N3M complex values with zero imaginary
// part.  The warps' sums are added in a fixed order.  Correlations: one block per
// (plane, component); RXX and RXY with a thread per x point summing over K in order,
// RZZ with a warp per z point.
// ---------------------------------------------------------------------------------
constexpr int SPW = 4;

// cell-centre velocity of component L (0..2) at (i, j, k), v between j and jv
template <typename R>
__device__ __forceinline__ double vcell(const StepArgs<R> &a, int L, int i, int j, int k, int jv) {
    const Geo &g = a.g;
    if (L == 0) return (sv<R>(a.u, g, i, j, k) + sv<R>(a.u, g, i + 1 == g.n1m ? 0 : i + 1, j, k)) * 0.5;
    if (L == 1) return (sv<R>(a.v, g, i, j, k) + sv<R>(a.v, g, i, jv, k)) * 0.5;
    return (sv<R>(a.w, g, i, j, k) + sv<R>(a.w, g, i, j, k + 1 == g.n3m ? 0 : k + 1)) * 0.5;
}

// x spectra: dynamic shared memory SPW x (2 (N1M/2) double2 + (N1M/2 + 1) doubles)
template <typename R>
__global__ void __launch_bounds__(32 * SPW) k_spec_x(StepArgs<R> a, const double *vmo, const double2 *twp,
                                                     double *xs) {
    const Geo g = a.g;
    const int j = 1 + blockIdx.x, L = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = g.n1m, M = N / 2;
    extern __shared__ double2 smx[];
    double2 *bufa = smx + (size_t)w * (2 * M), *bufb = bufa + M;
    double *acc = reinterpret_cast<double *>(smx + (size_t)SPW * 2 * M) + (size_t)w * (M + 1);
    const double FS = 3.141592653589793 * g.dx1, mean = vmo[L * g.n2m + (j - 1)];
    for (int q = lane; q <= M; q += 32) acc[q] = 0.0;
    for (int k = w; k < g.n3m; k += SPW) {
        for (int q = lane; q < M; q += 32)
            bufa[q] = make_double2(vcell(a, L, 2 * q, j, k, j + 1) - mean, vcell(a, L, 2 * q + 1, j, k, j + 1) - mean);
        __syncwarp();
        double2 *Z = fft_smem<double2, false>(bufa, bufb, a.fx, 0, 1, 0, -1, lane, 32);
        for (int q = lane; q <= M; q += 32) {
            const double2 zk = Z[q == M ? 0 : q], zc = Z[q == 0 ? 0 : M - q];
            const double2 zm = make_double2(zc.x, -zc.y);
            const double Ex = 0.5 * (zk.x + zm.x), Ey = 0.5 * (zk.y + zm.y);
            const double Ox = 0.5 * (zk.y - zm.y), Oy = -0.5 * (zk.x - zm.x);
            const double2 t = twp[q];   // exp(-2 pi i q / N1M)
            const double Xx = Ex + (t.x * Ox - t.y * Oy), Xy = Ey + (t.x * Oy + t.y * Ox);
            acc[q] += (Xx * Xx + Xy * Xy) / N / FS;
        }
        __syncwarp();
    }
    __syncthreads();
    double *out = xs + (size_t)N * ((j - 1) + (size_t)g.n2m * L);
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
        const int kk = q <= M ? q : N - q;
        double s = 0.0;
        for (int ww = 0; ww < SPW; ++ww)
            s += reinterpret_cast<double *>(smx + (size_t)SPW * 2 * M)[(size_t)ww * (M + 1) + kk];
        out[q] = s / (double)g.n3m;
    }
}

// z spectra: dynamic shared memory SPW x (2 N3M double2 + N3M doubles)
template <typename R>
__global__ void __launch_bounds__(32 * SPW) k_spec_z(StepArgs<R> a, const double *vmo, double *zs) {
    const Geo g = a.g;
    const int j = 1 + blockIdx.x, L = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = g.n3m;
    extern __shared__ double2 smz[];
    double2 *bufa = smz + (size_t)w * (2 * N), *bufb = bufa + N;
    double *accs = reinterpret_cast<double *>(smz + (size_t)SPW * 2 * N), *acc = accs + (size_t)w * N;
    const double FS = 3.141592653589793 * g.dx3, mean = vmo[L * g.n2m + (j - 1)];
    for (int q = lane; q < N; q += 32) acc[q] = 0.0;
    for (int i = w; i < g.n1m; i += SPW) {
        for (int q = lane; q < N; q += 32) bufa[q] = make_double2(vcell(a, L, i, j, q, j + 1) - mean, 0.0);
        __syncwarp();
        const double2 *Z = fft_smem<double2, false>(bufa, bufb, a.fz, 0, 1, 0, -1, lane, 32);
        for (int q = lane; q < N; q += 32) acc[q] += (Z[q].x * Z[q].x + Z[q].y * Z[q].y) / N / FS;
        __syncwarp();
    }
    __syncthreads();
    double *out = zs + (size_t)N * ((j - 1) + (size_t)g.n2m * L);
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
        double s = 0.0;
        for (int ww = 0; ww < SPW; ++ww) s += accs[(size_t)ww * N + q];
        out[q] = s / (double)g.n1m;
    }
}

// correlations; st = the plane statistics table (VM in columns 0..2, VRMS in 7..9)
template <typename R>
__global__ void __launch_bounds__(256) k_corr(StepArgs<R> a, const double *st, double *rxx, double *rzz,
                                             double *rxy) {
    const Geo g = a.g;
    const int j = 1 + blockIdx.x, L = blockIdx.y;
    const int n1h = g.n1m / 2, n3h = g.n3m / 2;   // N1H - 1, N3H - 1 (0-based)
    const double vm = st[(size_t)(j - 1) * 29 + L], var = st[(size_t)(j - 1) * 29 + 7 + L] - vm * vm;
    const double vm1 = st[L], var1 = st[7 + L] - vm1 * vm1;
    const int jv = j == g.n2m ? g.n2m : j + 1, jv1 = g.n2m == 1 ? 1 : 2;   // JPA(J), JPA(1)
    auto vp = [&](int i, int k) { return vcell(a, L, i, j, k, jv) - vm; };
    const size_t o = (size_t)g.n2m * L + (j - 1);
    for (int i = threadIdx.x; i < g.n1m; i += blockDim.x) {
        double rx = 0.0, ry = 0.0;
        for (int k = 0; k < g.n3m; ++k) {
            const double p = vp(i, k);
            rx = rx + vp(n1h, k) * p;
            ry = ry + (vcell(a, L, n1h, 1, k, jv1) - vm1) * p;
        }
        if (rxx) rxx[o * g.n1m + i] = rx / (double)g.n3m / var;
        if (rxy) rxy[o * g.n1m + i] = ry / (double)g.n3m / sqrt(var) / sqrt(var1);
    }
    if (!rzz) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = w; k < g.n3m; k += blockDim.x / 32) {
        double r = 0.0;
        for (int i = lane; i < g.n1m; i += 32) r += vp(i, n3h) * vp(i, k);
        for (int s = 16; s > 0; s >>= 1) r += __shfl_down_sync(0xffffffffu, r, s);
        if (lane == 0) rzz[o * g.n3m + k] = r / (double)g.n1m / var;
    }
}

// ENERGY's quadrant analysis (compact3d.f:10560-10604): per plane the sums of
// u'v' = (u - VMP)(v - VMP) over the points of each sign quadrant of (u', v') and the
// points' counts; cell-centre u and v (V between J and J+1); vmp = VMP(J,1..2) (the
// reference's VMP is a local never assigned: zero-valued in practice).
template <typename R>
__global__ void __launch_bounds__(STB) k_quad(StepArgs<R> a, const double *vmp, double *part) {
    __shared__ double sh[8 * STB];
    const Geo &g = a.g;
    const int j = 1 + blockIdx.y;
    const int chunk = (g.np + SB - 1) / SB, e0 = blockIdx.x * chunk, e1 = min(g.np, e0 + chunk);
    const double m1 = vmp ? vmp[j - 1] : 0.0, m2 = vmp ? vmp[g.n2m + j - 1] : 0.0;
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int e = e0 + threadIdx.x; e < e1; e += STB) {
        const int i = e % g.n1m, k = e / g.n1m;
        const double V1P = vcell(a, 0, i, j, k, j + 1) - m1, V2P = vcell(a, 1, i, j, k, j + 1) - m2;
        const double uv = V1P * V2P;
        if (V1P > 0.0 && V2P > 0.0) { acc[0] += uv; acc[4] += 1.0; }
        if (V1P < 0.0 && V2P > 0.0) { acc[1] += uv; acc[5] += 1.0; }
        if (V1P < 0.0 && V2P < 0.0) { acc[2] += uv; acc[6] += 1.0; }
        if (V1P > 0.0 && V2P < 0.0) { acc[3] += uv; acc[7] += 1.0; }
    }
    block_sums(acc, 8, sh, part + ((size_t)blockIdx.y * SB + blockIdx.x) * 8);
}

// Q(J,1..4) = -sum / (N1M N3M), QP(J,1..4) = count / (N1M N3M): out[(J-1) 8 + q]
__global__ void k_quad_fin(Geo g, const double *part, double *out) {
    const int j = blockIdx.x, q = threadIdx.x;
    if (q >= 8) return;
    double s = 0.0;
    for (int b = 0; b < SB; ++b) s += part[((size_t)j * SB + b) * 8 + q];
    const double NXZ = 1.0 / (double)(g.n1m * g.n3m);
    out[(size_t)j * 8 + q] = q < 4 ? -s * NXZ : s * NXZ;
}

template <typename R>
int launch_quadrants_t(c3d_channel *ch, StepArgs<R> &a, const double *vmp, double *out, double *part) {
    const Geo &g = ch->g;
    k_quad<R><<<dim3(SB, g.n2m), STB, 0, ch->stream>>>(a, vmp, part);
    k_quad_fin<<<g.n2m, 32, 0, ch->stream>>>(g, part, out);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

template int launch_quadrants_t<double>(c3d_channel *, StepArgs<double> &, const double *, double *, double *);
template int launch_quadrants_t<float>(c3d_channel *, StepArgs<float> &, const double *, double *, double *);

// ENERGY's wall-stress spectrum (compact3d.f:10394-10416): the 2-D DFT of the bottom
// wall's TAUW - UTAU^2.  k_wspec_x: a warp per z row, the x transform of N1M reals as
// N1M/2 complex pairs and the real-input split, C1(kx, k) for kx = 0..N1M/2 into c1;
// k_wspec_z: a warp per kx, the z transform and |C|^2 / N1M / N3M / (PI DX3) / (PI DX1)
// at (kx, kz) and, by the conjugate symmetry of real data, at (N1M - kx, -kz).
__global__ void __launch_bounds__(32 * SPW) k_wspec_x(Geo g, FftPlan fx, const double *tauw, double utau,
                                                      const double2 *twp, double2 *c1) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, M = g.n1m / 2;
    const int k = blockIdx.x * SPW + w;
    extern __shared__ double2 smw[];
    double2 *bufa = smw + (size_t)w * (2 * M), *bufb = bufa + M;
    if (k >= g.n3m) return;
    const double t2 = utau * utau;
    const double *row = tauw + (size_t)k * g.n1m;
    for (int q = lane; q < M; q += 32) bufa[q] = make_double2(row[2 * q] - t2, row[2 * q + 1] - t2);
    __syncwarp();
    const double2 *Z = fft_smem<double2, false>(bufa, bufb, fx, 0, 1, 0, -1, lane, 32);
    for (int q = lane; q <= M; q += 32) {
        const double2 zk = Z[q == M ? 0 : q], zc = Z[q == 0 ? 0 : M - q];
        const double2 zm = make_double2(zc.x, -zc.y);
        const double Ex = 0.5 * (zk.x + zm.x), Ey = 0.5 * (zk.y + zm.y);
        const double Ox = 0.5 * (zk.y - zm.y), Oy = -0.5 * (zk.x - zm.x);
        const double2 t = twp[q];
        c1[(size_t)q * g.n3m + k] = make_double2(Ex + (t.x * Ox - t.y * Oy), Ey + (t.x * Oy + t.y * Ox));
    }
}

__global__ void __launch_bounds__(32 * SPW) k_wspec_z(Geo g, FftPlan fz, const double2 *c1, double *out) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, M = g.n1m / 2, N = g.n3m;
    const int kx = blockIdx.x * SPW + w;
    extern __shared__ double2 smw[];
    double2 *bufa = smw + (size_t)w * (2 * N), *bufb = bufa + N;
    if (kx > M) return;
    for (int q = lane; q < N; q += 32) bufa[q] = c1[(size_t)kx * N + q];
    __syncwarp();
    const double2 *Z = fft_smem<double2, false>(bufa, bufb, fz, 0, 1, 0, -1, lane, 32);
    const double s = 1.0 / g.n1m / N / (3.141592653589793 * g.dx3) / (3.141592653589793 * g.dx1);
    for (int q = lane; q < N; q += 32) {
        const double p = (Z[q].x * Z[q].x + Z[q].y * Z[q].y);
        out[(size_t)q * g.n1m + kx] = p * s;
        if (kx > 0 && kx < M) out[(size_t)((N - q) % N) * g.n1m + (g.n1m - kx)] = p * s;
    }
}

// ENERGY's 3-D two-point correlation (compact3d.f:10524-10556), a thread per point:
// RXYZ(I,J,K,L) = VP(N1H,N2H,N3H,L) VP(I,J,K,L) / rms(J) / rms(N2H), Fortran (N1M,N2M,N3M,3)
template <typename R>
__global__ void __launch_bounds__(256) k_corr3d(StepArgs<R> a, const double *st, double *out) {
    const Geo g = a.g;
    const long long n = (long long)g.n1m * g.n2m * g.n3m;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    const int L = (int)(t / n);
    long long r = t - L * n;
    const int i = (int)(r % g.n1m);
    r /= g.n1m;
    const int j = 1 + (int)(r % g.n2m), k = (int)(r / g.n2m);
    const int jh = g.aly == 1.0 ? g.n2m / 2 + 1 : g.n2m / 4 + 1, ih = g.n1m / 2, kh = g.n3m / 2;
    auto vm = [&](int jj) { return st[(size_t)(jj - 1) * 29 + L]; };
    auto rms = [&](int jj) { return sqrt(st[(size_t)(jj - 1) * 29 + 7 + L] - vm(jj) * vm(jj)); };
    auto jpa = [&](int jj) { return jj == g.n2m ? g.n2m : jj + 1; };
    const double ref = vcell(a, L, ih, jh, kh, jpa(jh)) - vm(jh);
    const double vp = vcell(a, L, i, j, k, jpa(j)) - vm(j);
    out[t] = ref * vp / rms(j) / rms(jh);
}

template <typename R>
int launch_corr3d_t(c3d_channel *ch, StepArgs<R> &a, const double *st, double *out) {
    const long long n = 3LL * ch->g.n1m * ch->g.n2m * ch->g.n3m;
    k_corr3d<R><<<(unsigned)((n + 255) / 256), 256, 0, ch->stream>>>(a, st, out);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}
template int launch_corr3d_t<double>(c3d_channel *, StepArgs<double> &, const double *, double *);
template int launch_corr3d_t<float>(c3d_channel *, StepArgs<float> &, const double *, double *);

int launch_wall_spectrum(c3d_channel *ch, double utau, double2 *c1, double *out) {
    const Geo &g = ch->g;
    const int M = g.n1m / 2;
    const size_t smx = (size_t)SPW * 2 * M * sizeof(double2), smz = (size_t)SPW * 2 * g.n3m * sizeof(double2);
    if (cudaFuncSetAttribute(k_wspec_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx) != cudaSuccess ||
        cudaFuncSetAttribute(k_wspec_z, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz) != cudaSuccess)
        return C3D_ECUDA;
    const double2 *twp = ch->tw64 + g.n1m / 2 + g.n3m;
    k_wspec_x<<<(g.n3m + SPW - 1) / SPW, 32 * SPW, smx, ch->stream>>>(g, ch->fx, ch->tauw, utau, twp, c1);
    k_wspec_z<<<(M + 1 + SPW - 1) / SPW, 32 * SPW, smz, ch->stream>>>(g, ch->fz, c1, out);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

template <typename R>
int launch_spectra_t(c3d_channel *ch, StepArgs<R> &a, const double *vmo, const double *st, double *xs, double *zs,
                     double *rxx, double *rzz, double *rxy) {
    const Geo &g = ch->g;
    const dim3 grid(g.n2m, 3);
    if (xs) {
        const int M = g.n1m / 2;
        const size_t sm = (size_t)SPW * (2 * M * sizeof(double2) + (M + 1) * sizeof(double));
        if (cudaFuncSetAttribute(k_spec_x<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return C3D_ECUDA;
        const double2 *twp = ch->tw64 + g.n1m / 2 + g.n3m;   // exp(-2 pi i q / N1M), q = 0..N1M/2
        k_spec_x<R><<<grid, 32 * SPW, sm, ch->stream>>>(a, vmo, twp, xs);
    }
    if (zs) {
        const size_t sm = (size_t)SPW * (2 * g.n3m * sizeof(double2) + g.n3m * sizeof(double));
        if (cudaFuncSetAttribute(k_spec_z<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
            return C3D_ECUDA;
        k_spec_z<R><<<grid, 32 * SPW, sm, ch->stream>>>(a, vmo, zs);
    }
    if (rxx || rzz || rxy) k_corr<R><<<grid, 256, 0, ch->stream>>>(a, st, rxx, rzz, rxy);
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

template int launch_spectra_t<double>(c3d_channel *, StepArgs<double> &, const double *, const double *, double *,
                                      double *, double *, double *, double *);
template int launch_spectra_t<float>(c3d_channel *, StepArgs<float> &, const double *, const double *, double *,
                                     double *, double *, double *, double *);

// Scratch the statistics need on the device: the output table and the partial sums.
size_t stats_scratch_doubles(const Geo &g) { return (size_t)g.n2m * 29 + (size_t)g.n2m * SB * NS1; }

}  // namespace c3d
