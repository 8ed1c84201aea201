// c3d_step.cu -- orchestration of one GETUP call (compact3d.f:879-960) on sm_103a, and
// the small kernels that are neither x nor z passes.
//
// Pass structure of one step (all kernels on the channel's stream):
//   bcond   BCOND (963-1001): wall planes of u, w (j=0, j=N2) and v (j=1, j=N2)
//   xA      x rows: y-viscous terms, x-viscous (1,10,1), -dP/dx (1,22,1), d(uu)/dx,
//           d(vv)/dy, interpolants VV1, WW1 (1,6,1), E_xy = VV1*(u at y faces)
//   zA      z columns: z-viscous, -dP/dz, UU3, VV3, WW3 and E_xz, E_yz, WW3^2
//   zB      z columns: d(uw)/dz, d(vw)/dz, d(ww)/dz
//   xB      x rows: d(uv)/dx, d(uw)/dx, d(uv)/dy, d(wv)/dy, AB2, x factor of CN
//   ycn     y columns: wall-normal factor of CN (TDMAI)
//   zC      z columns: z factor of CN -> delta = UH - U
//   zD, xC  RHSDP and the real-to-complex FFT of RDP along x
//   fftz, poisson, fftz   GETDP in spectral space
//   xD      complex-to-real FFT -> DP, dDP/dx, bulk-flow partial sums
//   reduce  DMPRESG, DMPRESG3 (FP64), PRESG, PRESG3
//   zE      dDP/dz, u/v/w update, P += DP (UPCALC)
#include <string.h>
#include <type_traits>
#include <vector>
#include "c3d_kern.cuh"

namespace c3d {

int launch_ptables(c3d_channel *ch, const double *ak1, const double *ak3, const double *pm, const double *pc,
                   const double *pp);

template <typename R>
__device__ __forceinline__ void b_bcond(Geo g, typename SType<R>::S *u, typename SType<R>::S *v, typename SType<R>::S *w, const Blk blk) {
    typedef typename SType<R>::S S;
    typedef St<R> ST;
    int id = blk.x * blockDim.x + threadIdx.x;
    if (id >= g.np) return;
    const long long b0 = id, bt = (long long)g.n2 * g.np + id, bm = (long long)g.n2m * g.np + id;
    const S z = S();
    const R top = (R)(2.0 - g.aly);      // no-slip (ALY=2) or free-slip (ALY=1) upper wall
    u[b0] = z;
    v[b0] = z;
    w[b0] = z;
    v[(long long)g.np + id] = z;         // v at J=1
    u[bt] = ST::scale(u[bm], top);
    v[bt] = z;
    w[bt] = ST::scale(w[bm], top);
}
template <typename R>
__global__ void k_bcond(Geo g, typename SType<R>::S *u, typename SType<R>::S *v, typename SType<R>::S *w) {
    b_bcond<R>(g, u, v, w, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// Wall-normal CN factor (TDMAI, compact3d.f:8630-8659), one thread per (i, k), in place.
// The factors (A, 1/BET, GAM per J) are in the working precision; the j loops load UY
// planes ahead so that the sequential chain does not wait on memory.
constexpr int UY = 32;   // planes per batch (8: 0.273 ms, 16: 0.265, 32: 0.252 on channel384)
template <typename R>
__device__ __forceinline__ void b_ycn(const StepArgs<R> &a, const R *ycn, const Blk blk) {
    const Geo g = a.g;
    const long long tid = (long long)blk.x * blockDim.x + threadIdx.x;
    if (tid >= 3LL * g.np) return;
    const int c = (int)(tid / g.np);
    const int col = (int)(tid % g.np);
    const int js = (c == 1) ? 2 : 1;
    const int m = g.n2 + 1;
    const R *A = ycn + (c * 3 + 0) * m, *RB = ycn + (c * 3 + 1) * m, *GM = ycn + (c * 3 + 2) * m;
    R *X = a.r[c] + col;
    const long long s = g.np;
    R xp = R(0);
    for (int j0 = js; j0 <= g.n2m; j0 += UY) {
        R q[UY];
#pragma unroll
        for (int u = 0; u < UY; ++u)
            if (j0 + u <= g.n2m) q[u] = X[(j0 + u) * s];
#pragma unroll
        for (int u = 0; u < UY; ++u) {
            const int j = j0 + u;
            if (j <= g.n2m) {
                xp = (j == js) ? q[u] * RB[j] : (q[u] - A[j] * xp) * RB[j];
                q[u] = xp;
            }
        }
#pragma unroll
        for (int u = 0; u < UY; ++u)
            if (j0 + u <= g.n2m) X[(j0 + u) * s] = q[u];
    }
    for (int j0 = g.n2m - 1; j0 >= js; j0 -= UY) {
        R q[UY];
#pragma unroll
        for (int u = 0; u < UY; ++u)
            if (j0 - u >= js) q[u] = X[(j0 - u) * s];
#pragma unroll
        for (int u = 0; u < UY; ++u)
            if (j0 - u >= js) {
                xp = q[u] - xp * GM[j0 - u];
                q[u] = xp;
            }
#pragma unroll
        for (int u = 0; u < UY; ++u)
            if (j0 - u >= js) X[(j0 - u) * s] = q[u];
    }
}
template <typename R>
__global__ void __launch_bounds__(TPB) k_ycn(StepArgs<R> a, const R *ycn) {
    b_ycn<R>(a, ycn, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// The wall-normal CN factor with the columns staged in shared memory: a block owns TX
// consecutive columns (i, k) of one component over all planes; its first warp fetches each
// plane's TX-value row segment by a bulk copy (cp.async.bulk) into the block's tile, in
// YCH chunks of planes each completing on its own mbarrier, so the forward sweep starts on
// the first chunk while the others arrive; the forward sweep writes the tile in place,
// the backward sweep reads it and stores each result once.  Every value crosses DRAM once
// in each direction.  A wait that runs out sets SCAL_PIPEERR and returns after waiting
// (bounded) for the block's copies in flight.
constexpr int YCH = 8;
template <typename R>
__host__ __device__ inline size_t ycn_tile_bytes(int tx, int n2m) {
    // barriers, coefficients (rounded up to 16 bytes: the tile's rows are bulk-copy targets), tile
    return 64 + (((3 * (size_t)n2m * sizeof(R)) + 15) & ~(size_t)15) + (size_t)n2m * tx * sizeof(R);
}

template <typename R, int TX>
__device__ __forceinline__ void b_ycnt(const StepArgs<R> &a, const R *ycn, const Blk blk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int np = g.np, ntile = (np + TX - 1) / TX;
    const int c = (int)blk.x / ntile, q = (int)blk.x % ntile;
    const int col0 = q * TX, ncol = min(TX, np - col0);
    const int js = (c == 1) ? 2 : 1, nj = g.n2m - js + 1;
    const int m = g.n2 + 1;
    const R *A = ycn + (c * 3 + 0) * m, *RBt = ycn + (c * 3 + 1) * m, *GM = ycn + (c * 3 + 2) * m;
    R *X = a.r[c] + col0;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw);
    R *sA = reinterpret_cast<R *>(smem_raw + 64), *sR = sA + nj, *sG = sR + nj;
    R *T = reinterpret_cast<R *>(smem_raw + 64 + (((3 * (size_t)nj * sizeof(R)) + 15) & ~(size_t)15));
    const int t = threadIdx.x;
    const int cpl = (nj + YCH - 1) / YCH;
    const uint32_t rowb = (uint32_t)ncol * (uint32_t)sizeof(R);
    if (t == 0) {
        for (int b = 0; b < YCH; ++b) mbar_init(bar + b, 1);
        mbar_init_fence();
        fence_async_smem();
        for (int b = 0; b < YCH; ++b) {
            const int p0 = b * cpl, p1 = min(nj, p0 + cpl);
            if (p1 > p0) mbar_expect_tx(bar + b, (uint32_t)(p1 - p0) * rowb);
        }
    }
    for (int p = t; p < nj; p += blockDim.x) {
        sA[p] = A[js + p];
        sR[p] = RBt[js + p];
        sG[p] = GM[js + p];
    }
    __syncthreads();   // barriers set up before any copy can complete; coefficients staged
    if (t < 32)
        for (int p = t; p < nj; p += 32) bulk_g2s(T + (size_t)p * TX, X + (long long)(js + p) * np, rowb, bar + p / cpl);
    if (t >= ncol) return;   // no copy targets this thread's column; the block stays until the others end
    R xp = R(0);
    for (int b = 0; b < YCH; ++b) {
        const int p0 = b * cpl, p1 = min(nj, p0 + cpl);
        if (p1 <= p0) break;
        if (!mbar_wait(bar + b, 0)) {
            a.scal[SCAL_PIPEERR] = 1.0;
            for (int b2 = b; b2 < YCH; ++b2)
                if (b2 * cpl < nj) mbar_wait(bar + b2, 0);   // the copies in flight target this tile
            return;
        }
        // eight planes read ahead of the recurrence, so the shared-memory latency is not on
        // its dependent chain
        int p = p0;
        for (; p + 8 <= p1; p += 8) {
            R v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = T[(size_t)(p + u) * TX + t];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int pp = p + u;
                xp = (pp == 0) ? v[u] * sR[pp] : (v[u] - sA[pp] * xp) * sR[pp];
                v[u] = xp;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) T[(size_t)(p + u) * TX + t] = v[u];
        }
        for (; p < p1; ++p) {
            const R v = T[(size_t)p * TX + t];
            xp = (p == 0) ? v * sR[p] : (v - sA[p] * xp) * sR[p];
            T[(size_t)p * TX + t] = xp;
        }
    }
    X[(long long)(js + nj - 1) * np + t] = xp;
    int p = nj - 2;
    for (; p >= 7; p -= 8) {
        R v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = T[(size_t)(p - u) * TX + t];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            xp = v[u] - xp * sG[p - u];
            v[u] = xp;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) X[(long long)(js + p - u) * np + t] = v[u];
    }
    for (; p >= 0; --p) {
        xp = T[(size_t)p * TX + t] - xp * sG[p];
        X[(long long)(js + p) * np + t] = xp;
    }
}
template <typename R, int TX>
__global__ void __launch_bounds__(64) k_ycnt(StepArgs<R> a, const R *ycn) {
    b_ycnt<R, TX>(a, ycn, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// Launches the wall-normal CN factor in the form the schedule names (0: one thread per
// column with register batches; 32 or 64: the shared-memory tiles of that many columns,
// when the tile fits).
template <typename R>
static void launch_ycn(c3d_channel *ch, StepArgs<R> &a, int *nl) {
    const R *ycn = sizeof(R) == 8 ? (const R *)ch->ycn : (const R *)ch->ycn32;
    const int tx = ch->tune.ycn;
    const size_t sm = ycn_tile_bytes<R>(tx == 0 ? 32 : tx, ch->g.n2m);
    if ((tx == 32 || tx == 64) && sm <= 227 * 1024) {
        const int nb = 3 * ((ch->g.np + tx - 1) / tx);
        // the whole shared-memory carve-out, so that as many tiles as fit are resident
        if (tx == 32) {
            cudaFuncSetAttribute(k_ycnt<R, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            cudaFuncSetAttribute(k_ycnt<R, 32>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            k_ycnt<R, 32><<<nb, 32, sm, ch->stream>>>(a, ycn);
        } else {
            cudaFuncSetAttribute(k_ycnt<R, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            cudaFuncSetAttribute(k_ycnt<R, 64>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            k_ycnt<R, 64><<<nb, 64, sm, ch->stream>>>(a, ycn);
        }
    } else {
        k_ycn<R><<<nblk(3LL * ch->g.np), TPB, 0, ch->stream>>>(a, ycn);
    }
    mark(ch, nl, "ycn", (double)ch->g.n1m * ch->g.n2m * ch->g.n3m * 6 * sizeof(R));
}

// DMPRESG / DMPRESG3 in FP64 with a fixed summation order; PRESG += DMPRESG (UPCALC)
// UPCALC's forcing (compact3d.f:1052-1238) from the summed CN increments of u and w.
__device__ __forceinline__ void finish_bulk(Geo g, double t1, double t3, double *scal, double dt, int bulk) {
    double dm = bulk ? t1 / g.vol / dt : 0.0;
    double dm3 = bulk ? t3 / g.vol / dt : 0.0;
    scal[SCAL_DMPRESG] = dm;
    scal[SCAL_DMPRESG3] = dm3;
    if (bulk) {
        scal[SCAL_PRESG] = scal[SCAL_PRESG] + dm;
        scal[SCAL_PRESG3] = scal[SCAL_PRESG3] + dm3;
    }
}

// Bulk-flow sums over the per-row partials in two fixed-order levels: RB blocks each
// reduce a contiguous range of rows (strided per thread, then a tree) into part[2 nrows
// + b] / part[2 nrows + RB + b]; one block then reduces the RB block sums by a tree and
// finishes UPCALC's forcing.  FP64 form: FP64 sums.  Mixed form: the per-row partials
// are double-float pairs summed in double-float arithmetic (FP32 instructions), then the
// FP64 bulk-flow arithmetic.
struct AddF64 {
    typedef double T;
    static __device__ T zero() { return 0.0; }
    static __device__ T add(T a, T b) { return a + b; }
    static __device__ double dbl(T a) { return a; }
};
struct AddDF {
    typedef float2 T;
    static __device__ T zero() { return make_float2(0.f, 0.f); }
    static __device__ T add(T a, T b) { return df_add(a, b); }
    static __device__ double dbl(T a) { return (double)a.x + (double)a.y; }
};

template <typename A>
__device__ __forceinline__ void b_reduce1(Geo g, typename A::T *part, const Blk blk) {
    typedef typename A::T T;
    const int nrows = g.n2m * g.n3m;
    const int chunk = (nrows + RB - 1) / RB, r0 = blk.x * chunk, r1 = min(nrows, r0 + chunk);
    __shared__ T sh1[256], sh3[256];
    T s1 = A::zero(), s3 = A::zero();
    for (int r = r0 + (int)threadIdx.x; r < r1; r += 256) {
        s1 = A::add(s1, part[r]);
        s3 = A::add(s3, part[nrows + r]);
    }
    sh1[threadIdx.x] = s1;
    sh3[threadIdx.x] = s3;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sh1[threadIdx.x] = A::add(sh1[threadIdx.x], sh1[threadIdx.x + w]);
            sh3[threadIdx.x] = A::add(sh3[threadIdx.x], sh3[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * nrows + blk.x] = sh1[0];
        part[2 * nrows + RB + blk.x] = sh3[0];
    }
}
template <typename A>
__global__ void __launch_bounds__(256) k_reduce1(Geo g, typename A::T *part) {
    b_reduce1<A>(g, part, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

template <typename A>
__device__ __forceinline__ void b_reduce2(Geo g, const typename A::T *part, double *scal, double dt, int bulk, const Blk blk) {
    typedef typename A::T T;
    const int nrows = g.n2m * g.n3m;
    __shared__ T sh1[RB], sh3[RB];
    sh1[threadIdx.x] = part[2 * nrows + threadIdx.x];
    sh3[threadIdx.x] = part[2 * nrows + RB + threadIdx.x];
    __syncthreads();
    for (int w = RB / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sh1[threadIdx.x] = A::add(sh1[threadIdx.x], sh1[threadIdx.x + w]);
            sh3[threadIdx.x] = A::add(sh3[threadIdx.x], sh3[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) finish_bulk(g, A::dbl(sh1[0]), A::dbl(sh3[0]), scal, dt, bulk);
}
template <typename A>
__global__ void __launch_bounds__(RB) k_reduce2(Geo g, const typename A::T *part, double *scal, double dt, int bulk) {
    b_reduce2<A>(g, part, scal, dt, bulk, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// CHKMF (compact3d.f:9463-9503) and WALLSS (11077-11143): one block, FP64, fixed order.
template <typename R>
__global__ void k_diag_sums(Geo g, const typename SType<R>::S *u, const typename SType<R>::S *v,
                            const typename SType<R>::S *w, double *scal) {
    typedef St<R> ST;
    __shared__ double sh[5][256];
    double f1 = 0.0, f3 = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0;
    for (int e = threadIdx.x; e < g.n2m * g.n3m; e += blockDim.x) {
        int J = 1 + e / g.n3m, k = e % g.n3m;
        f1 += ST::dbl(u[fidx(g, 0, J, k)]) * g.dy[J] / g.dx3 / g.dx1;
    }
    for (int e = threadIdx.x; e < g.n2m * g.n1m; e += blockDim.x) {
        int J = 1 + e / g.n1m, i = e % g.n1m;
        f3 += ST::dbl(w[fidx(g, i, J, 0)]) * g.dy[J] / g.dx1 / g.dx3;
    }
    for (int e = threadIdx.x; e < g.np; e += blockDim.x) {
        int k = e / g.n1m, i = e % g.n1m;
        int ip = (i + 1 == g.n1m) ? 0 : i + 1, kp = (k + 1 == g.n3m) ? 0 : k + 1;
        auto U = [&](int ii, int jj, int kk) { return ST::dbl(u[fidx(g, ii, jj, kk)]); };
        auto W = [&](int ii, int jj, int kk) { return ST::dbl(w[fidx(g, ii, jj, kk)]); };
        double UHC = 0.5 * (U(i, 1, k) + U(ip, 1, k));
        double UHW = 0.5 * (U(i, 0, k) + U(ip, 0, k));
        double VHC = ST::dbl(v[fidx(g, i, 2, k)]), VHW = ST::dbl(v[fidx(g, i, 1, k)]);
        double WHC = 0.5 * (W(i, 1, k) + W(i, 1, kp));
        double WHW = 0.5 * (W(i, 0, k) + W(i, 0, kp));
        double WSB1 = (UHC - UHW) / (g.dy[1] * 0.5), WSB2 = (VHC - VHW) / g.dy[1], WSB3 = (WHC - WHW) / (g.dy[1] * 0.5);
        UHC = 0.5 * (U(i, g.n2m, k) + U(ip, g.n2m, k));
        UHW = 0.5 * (U(i, g.n2, k) + U(ip, g.n2, k));
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
        scal[SCAL_FLOW1] = sh[0][0] * g.n1m / g.alx / g.alz;   // the reference sums U(1,J,K) N1M times
        scal[SCAL_FLOW3] = sh[1][0] * g.n3m / g.alx / g.alz;
        const double nxz = 1.0 / ((double)g.n1m * g.n3m);
        scal[SCAL_WSM + 0] = sh[2][0] * nxz / g.re / g.aly;
        scal[SCAL_WSM + 1] = sh[3][0] * nxz / g.re / g.aly;
        scal[SCAL_WSM + 2] = sh[4][0] * nxz / g.re / g.aly;
    }
}

// ---------------------------------------------------------------------------------
// Fortran <-> device repacking.  what: 0 = velocity component of U(0:N1,0:N2,0:N3,3)
// (device planes 0..N2), 1 = P(N1,N2,N3) (planes 1..N2M), 2 = HH component (planes 1..N2M).
// ---------------------------------------------------------------------------------
// Grid-stride loops with 32-bit indices (every Fortran array has fewer than 2^31
// elements), four elements per thread and pass with their loads issued first.
template <typename T, typename Conv>
__global__ void k_unpack(Geo g, int what, T *__restrict__ dev, const double *__restrict__ fort, Conv cv) {
    const int j0 = (what == 0) ? 0 : 1, j1 = (what == 0) ? g.n2 : g.n2m;
    const unsigned tot = (unsigned)(j1 - j0 + 1) * (unsigned)g.np;
    const unsigned n1 = g.n1m, n3 = g.n3m, N1 = g.n1m + 1, N2 = g.n2;
    const unsigned st = gridDim.x * blockDim.x;
    for (unsigned b = blockIdx.x * blockDim.x + threadIdx.x; b < tot; b += 4 * st) {
        double v[4];
        unsigned dst[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const unsigned id = b + u * st;
            if (id < tot) {
                const unsigned q = id / n1, i = id - q * n1, jj = q / n3, k = q - jj * n3, j = j0 + jj;
                const unsigned f = (what == 1) ? i + N1 * ((j - 1) + N2 * k) : (i + 1) + (N1 + 1) * (j + (N2 + 1) * (k + 1));
                v[u] = fort[f];
                dst[u] = (j * n3 + k) * n1 + i;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (b + u * st < tot) dev[dst[u]] = cv(v[u]);
    }
}

// Periodic ghost cells (I=0, I=N1, K=0, K=N3) receive the periodic copies; entries
// outside the device planes receive 0.
template <typename T, typename Conv>
__global__ void k_pack(Geo g, int what, const T *__restrict__ dev, double *__restrict__ fort, Conv cv) {
    const unsigned N1 = g.n1m + 1, N2 = g.n2, N3 = g.n3m + 1;
    const unsigned A1 = (what == 1) ? N1 : N1 + 1, A2 = (what == 1) ? N2 : N2 + 1, A3 = (what == 1) ? N3 : N3 + 1;
    const unsigned tot = A1 * A2 * A3, o = (what == 1) ? 1 : 0;
    const int j0 = (what == 0) ? 0 : 1, j1 = (what == 0) ? g.n2 : g.n2m;
    const unsigned st = gridDim.x * blockDim.x;
    for (unsigned b = blockIdx.x * blockDim.x + threadIdx.x; b < tot; b += 4 * st) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const unsigned id = b + u * st;
            v[u] = 0.0;
            if (id < tot) {
                const unsigned q = id / A1, I = id - q * A1 + o, K = q / A2 + o, J = q - (q / A2) * A2 + o;
                const int i = (int)((I + g.n1m - 1) % g.n1m), k = (int)((K + g.n3m - 1) % g.n3m);
                if ((int)J >= j0 && (int)J <= j1) v[u] = cv(dev[fidx(g, i, (int)J, k)]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (b + u * st < tot) fort[b + u * st] = v[u];
    }
}

struct ToF64 { __device__ double operator()(double x) const { return x; } };
struct ToF32 { __device__ float operator()(double x) const { return (float)x; } };
struct ToDF { __device__ float2 operator()(double x) const { return St<float>::from_double(x); } };
struct FromF64 { __device__ double operator()(double x) const { return x; } };
struct FromF32 { __device__ double operator()(float x) const { return (double)x; } };
struct FromDF { __device__ double operator()(float2 x) const { return St<float>::dbl(x); } };

// ---------------------------------------------------------------------------------
// Host-side drivers
// ---------------------------------------------------------------------------------
template <typename R>
static StepArgs<R> make_args(c3d_channel *ch, double dt) {
    typedef typename SType<R>::S S;
    StepArgs<R> a;
    memset((void *)&a, 0, sizeof(a));
    a.g = ch->g;
    {
        const R *b = (const R *)ch->metr;
        const int m = ch->g.n2 + 1;
        const R **dst[NMETR] = {&a.m.hp, &a.m.hc, &a.m.hm, &a.m.hz, &a.m.dyp, &a.m.dyc, &a.m.dym,
                                &a.m.dyz, &a.m.h, &a.m.rh, &a.m.hdy, &a.m.rdy, &a.m.dy};
        for (int q = 0; q < NMETR; ++q) *dst[q] = b + (size_t)q * m;
    }
    a.u = (S *)ch->u; a.v = (S *)ch->v; a.w = (S *)ch->w; a.p = (S *)ch->p;
    const int cur = ch->cur, old = 1 - ch->cur;
    for (int c = 0; c < 3; ++c) {
        a.hh[c] = (R *)ch->hh[cur][c];
        a.ho[c] = (const R *)ch->hh[old][c];
        a.r[c] = (R *)ch->r[c];
    }
    a.exy = (R *)ch->exy; a.exz = (R *)ch->exz; a.eyz = (R *)ch->eyz;
    a.ww1 = (R *)ch->ww1; a.wsq = (R *)ch->wsq; a.rdpz = (R *)ch->rdpz; a.g1 = (R *)ch->g1;
    a.dp = (R *)ch->dp; a.spec = ch->spec; a.scal = ch->scal; a.part = ch->part;
    a.ycn = ch->ycn; a.prb = ch->prb; a.pgam = ch->pgam; a.prbdf = ch->prbdf; a.pgamdf = ch->pgamdf;
    a.pmj = ch->pmj; a.pmjdf = ch->pmjdf; a.bulkw = ch->bulkw;
    a.fx = ch->fx; a.fz = ch->fz;
    a.twx64 = ch->tw64 + (ch->g.n1m / 2) + ch->g.n3m;
    a.twx32 = ch->tw32 + (ch->g.n1m / 2) + ch->g.n3m;
    a.dt = dt;
    a.bulk = 1;
    a.ycnw = sizeof(R) == 8 ? (const R *)ch->ycn : (const R *)ch->ycn32;
    a.re1 = (R)(1.0 / ch->g.re);
    a.f12x = (R)(12.0 * ch->g.dx1q);
    a.f24x = (R)(24.0 * ch->g.dx1);
    a.f12z = (R)(12.0 * ch->g.dx3q);
    a.f24z = (R)(24.0 * ch->g.dx3);
    a.rdt = (R)(1.0 / dt);
    a.xscale = (R)(1.0 / ((double)ch->g.n1m * (double)ch->g.n3m));
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
    // CN x and z factors of GETUH1-3 (compact3d.f:8280-8282, 8314-8316)
    const double api = 1.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx1q * (1.0);
    const double aci = 10.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx1q * (-2.0);
    const double apk = 1.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx3q * (1.0);
    const double ack = 10.0 - dt / 2.0 * (1. / RE) * 12.0 * ch->g.dx3q * (-2.0);
    a.cnx = mk(api, aci, f32);
    a.cnz = mk(apk, ack, f32);
    return a;
}

template <typename R>
static int pressure_and_update(c3d_channel *ch, StepArgs<R> &a, R *d0, R *d1, R *d2, int updp, int *nl) {
    int rc;
    if ((rc = launch_zpass<R>(ch, a, 3, d0, d1, d2, 0, nl))) return rc;       // zD
    if ((rc = launch_xpass<R>(ch, a, 2, d0, d1, nl))) return rc;              // xC
    if ((rc = launch_spec<R>(ch, a, 0, nl))) return rc;                       // fftz fwd
    if ((rc = launch_spec<R>(ch, a, 1, nl))) return rc;                       // poisson
    if ((rc = launch_spec<R>(ch, a, 2, nl))) return rc;                       // fftz inv
    if ((rc = launch_xpass<R>(ch, a, 3, d0, d2, nl))) return rc;              // xD
    if constexpr (sizeof(R) == 8) {
        k_reduce1<AddF64><<<RB, 256, 0, ch->stream>>>(ch->g, ch->part);
        k_reduce2<AddF64><<<1, RB, 0, ch->stream>>>(ch->g, ch->part, ch->scal, a.dt, a.bulk);
    } else {
        k_reduce1<AddDF><<<RB, 256, 0, ch->stream>>>(ch->g, (float2 *)ch->part);
        k_reduce2<AddDF><<<1, RB, 0, ch->stream>>>(ch->g, (const float2 *)ch->part, ch->scal, a.dt, a.bulk);
    }
    ++*nl;   // the reduction is two launches under one profiler mark
    mark(ch, nl, "reduce", 16.0 * ch->g.n2m * ch->g.n3m);
    return launch_zpass<R>(ch, a, 4, d0, d1, d2, updp, nl);                   // zE
}

static RefArgs make_ref_args(c3d_channel *ch, double dt, int updp) {
    RefArgs r;
    r.updp = updp;
    const double b = 22.0, rt = -2.0 / (b + sqrt(b * b - 4.0));
    r.f24x = dfl::from(24.0 * ch->g.dx1);
    r.f24z = dfl::from(24.0 * ch->g.dx3);
    r.rdt = dfl::from(1.0 / dt);
    r.c22x.r = dfl::from(rt);
    r.c22x.s = dfl::from(-rt);
    r.c22x.m = 13;
    r.c22z = r.c22x;
    r.rdy = ch->rdydf;
    r.rzh = (float *)ch->exz;
    r.rzl = (float *)ch->eyz;
    return r;
}

// One refinement step of the pressure solve after UPCALC (mixed form, C3D_MIXED_IR).
template <typename R>
static int refine_pressure(c3d_channel *ch, StepArgs<R> &a, int updp, int *nl) {
    if constexpr (sizeof(R) == 4) {
        if (!ch->refine) return 0;
        RefArgs r = make_ref_args(ch, a.dt, updp);
        return launch_refine(ch, a, r, nl);
    } else {
        (void)ch; (void)a; (void)updp; (void)nl;
        return 0;
    }
}

template <typename R>
static LesArgs<R> make_les_args(c3d_channel *ch) {
    LesArgs<R> l;
    memset((void *)&l, 0, sizeof(l));
    if (ch->files == 0) return l;
    R **f[8] = {&l.nu, &l.nux, &l.nuz, &l.t13, &l.nuwz, &l.dvdx, &l.dwdx, &l.dvdz};
    for (int q = 0; q < 8; ++q) *f[q] = (R *)ch->les[q];
    l.dyn = (R *)ch->dyn;
    l.smagc = ch->smagc;
    l.coef = (R *)ch->coef;
    l.d23 = ch->d23;
    l.d23r = (const R *)ch->d23r;
    l.ycs = ch->ycs;
    l.tauw = ch->tauw;
    l.taub = ch->taub;
    l.wpart = ch->wpart;
    l.files = ch->files;
    l.wmodel = ch->wmodel;
    l.wall_cap = ch->wall_cap;
    l.ifwall = ch->wmodel != 0 ? 1.0 : 0.0;   // WALL_MODEL sets IFWALL = 1 (compact3d.f:1993)
    l.reninv = (R)(1.0 / ch->g.re);
    l.dx1 = (R)ch->g.dx1;
    l.dx3 = (R)ch->g.dx3;
    return l;
}

template <typename R>
static int step_impl(c3d_channel *ch, double dt, int *nl) {
    typedef typename SType<R>::S S;
    set_spec_smem<R>(ch);
    ch->cur = 1 - ch->cur;   // HH of the last step becomes HH_old (GETUP's HH2 <- HH)
    StepArgs<R> a = make_args<R>(ch, dt);
    int rc;
    LesArgs<R> l = make_les_args<R>(ch);
    // GETUP order (compact3d.f:931-940): SGS model and wall model, then BCOND
    if (ch->files != 0 && (rc = launch_les<R>(ch, a, l, 0, nl))) return rc;
    k_bcond<R><<<nblk(ch->g.np), TPB, 0, ch->stream>>>(ch->g, (S *)ch->u, (S *)ch->v, (S *)ch->w);
    mark(ch, nl, "bcond", 64.0 * ch->g.np);
    if ((rc = launch_xpass<R>(ch, a, 0, nullptr, nullptr, nl))) return rc;    // xA
    if ((rc = launch_zpass<R>(ch, a, 0, nullptr, nullptr, nullptr, 0, nl))) return rc;   // zA
    if ((rc = launch_zpass<R>(ch, a, 1, nullptr, nullptr, nullptr, 0, nl))) return rc;   // zB
    if (ch->files != 0 && (rc = launch_les<R>(ch, a, l, 1, nl))) return rc;   // SGS fluxes into HH
    // xB is the first reader of HH_old and the last writer of the new HH: the overlapped
    // transfers of c3d_getup upload the one and download the other around it
    if (ch->hh_hooks) CK_RC(cudaStreamWaitEvent(ch->stream, ch->hh_in, 0));
    if ((rc = launch_xpass<R>(ch, a, 1, nullptr, nullptr, nl))) return rc;    // xB
    if (ch->hh_hooks) CK_RC(cudaEventRecord(ch->hh_out, ch->stream));
    launch_ycn<R>(ch, a, nl);
    // deltas go to exz/eyz/wsq, which the RHS passes no longer need
    R *dd0 = (R *)ch->exz, *dd1 = (R *)ch->eyz, *dd2 = (R *)ch->wsq;
    if ((rc = launch_zpass<R>(ch, a, 2, dd0, dd1, dd2, 0, nl))) return rc;    // zC
    if ((rc = pressure_and_update<R>(ch, a, dd0, dd1, dd2, 1, nl))) return rc;
    return refine_pressure<R>(ch, a, 1, nl);
}

// ---------------------------------------------------------------------------------
// Batch form of the DNS step (the passes of step_impl without SGS model, in order): the
// small kernels here, the x, z and spectral passes from their files.
// ---------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(TPB) kb_bcond(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_bcond<R>(a.g, a.u, a.v, a.w, Blk{m.x, m.y, m.gx});
}
template <typename R>
__global__ void __launch_bounds__(TPB) kb_ycn(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_ycn<R>(a, a.ycnw, Blk{m.x, m.y, m.gx});
}
template <typename R, typename Add>
__global__ void __launch_bounds__(256) kb_reduce1(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_reduce1<Add>(a.g, reinterpret_cast<typename Add::T *>(a.part), Blk{m.x, m.y, m.gx});
}
template <typename R, typename Add>
__global__ void __launch_bounds__(RB) kb_reduce2(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_reduce2<Add>(a.g, reinterpret_cast<const typename Add::T *>(a.part), a.scal, a.dt, a.bulk, Blk{m.x, m.y, m.gx});
}

template <typename R>
static int batch_plan_t(c3d_channel *ch, const BatchSched &bs, std::vector<BKern> &out) {
    const int *zs = bs.zseg;
    typedef typename std::conditional<sizeof(R) == 8, AddF64, AddDF>::type Add;
    const Geo &g = ch->g;
    int rc;
    out.push_back({(const void *)kb_bcond<R>, TPB, 0, (unsigned)nblk(g.np)});
    if ((rc = xpass_bkern<R>(ch, 0, bs.xw, out))) return rc;      // xA (u, v, w)
    if ((rc = zpass_bkern<R>(ch, 0, zs[0], out))) return rc;      // zA (u, w and P, v)
    if ((rc = zpass_bkern<R>(ch, 1, zs[1], out))) return rc;      // zB
    if ((rc = xpass_bkern<R>(ch, 1, bs.xw, out))) return rc;      // xB
    out.push_back({(const void *)kb_ycn<R>, TPB, 0, (unsigned)nblk(3LL * g.np)});
    if ((rc = zpass_bkern<R>(ch, 2, zs[2], out))) return rc;      // zC
    if ((rc = zpass_bkern<R>(ch, 3, zs[3], out))) return rc;      // zD
    if ((rc = xpass_bkern<R>(ch, 2, bs.xw, out))) return rc;      // xC
    if ((rc = spec_bkern<R>(ch, 0, out))) return rc;       // fftz forward
    if ((rc = spec_bkern<R>(ch, 1, out))) return rc;       // Poisson
    if ((rc = spec_bkern<R>(ch, 2, out))) return rc;       // fftz inverse
    if ((rc = xpass_bkern<R>(ch, 3, bs.xw, out))) return rc;      // xD
    out.push_back({(const void *)kb_reduce1<R, Add>, 256, 0, (unsigned)RB});
    out.push_back({(const void *)kb_reduce2<R, Add>, RB, 0, 1u});
    return zpass_bkern<R>(ch, 4, zs[4], out);              // zE
}

int batch_plan(c3d_channel *ch, const BatchSched &s, std::vector<BKern> &out) {
    if (ch->files != 0 || ch->refine) { set_error("the batch form runs DNS channels without refinement"); return C3D_EINVAL; }
    if (ch->precision == C3D_MIXED) return batch_plan_t<float>(ch, s, out);
    return batch_plan_t<double>(ch, s, out);
}

size_t batch_args_size(const c3d_channel *ch) {
    return ch->precision == C3D_MIXED ? sizeof(StepArgs<float>) : sizeof(StepArgs<double>);
}

void batch_args(c3d_channel *ch, double dt, void *dst) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, dt);
        memcpy(dst, &a, sizeof(a));
    } else {
        StepArgs<double> a = make_args<double>(ch, dt);
        memcpy(dst, &a, sizeof(a));
    }
}

template <typename R>
int launch_stats_t(c3d_channel *ch, StepArgs<R> &a, double *out, double *part);

int launch_stats(c3d_channel *ch, double *out, double *part) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
        return launch_stats_t<float>(ch, a, out, part);
    }
    StepArgs<double> a = make_args<double>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_stats_t<double>(ch, a, out, part);
}

template <typename R>
int launch_spectra_t(c3d_channel *ch, StepArgs<R> &a, const double *vmo, const double *st, double *xs, double *zs,
                     double *rxx, double *rzz, double *rxy);

template <typename R>
int launch_particles_t(c3d_channel *ch, StepArgs<R> &a, double *par, int n, double diam, double dens, double hhh,
                       double dt, int *impact, double *r1, double *r2, double *r3);

int launch_particles(c3d_channel *ch, double *par, int n, double diam, double dens, double hhh, double dt, int *impact,
                     double *r1, double *r2, double *r3) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
        return launch_particles_t<float>(ch, a, par, n, diam, dens, hhh, dt, impact, r1, r2, r3);
    }
    StepArgs<double> a = make_args<double>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_particles_t<double>(ch, a, par, n, diam, dens, hhh, dt, impact, r1, r2, r3);
}

template <typename R>
int launch_corr3d_t(c3d_channel *ch, StepArgs<R> &a, const double *st, double *out);

int launch_corr3d(c3d_channel *ch, const double *st, double *out) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
        return launch_corr3d_t<float>(ch, a, st, out);
    }
    StepArgs<double> a = make_args<double>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_corr3d_t<double>(ch, a, st, out);
}

template <typename R>
int launch_quadrants_t(c3d_channel *ch, StepArgs<R> &a, const double *vmp, double *out, double *part);

int launch_quadrants(c3d_channel *ch, const double *vmp, double *out, double *part) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
        return launch_quadrants_t<float>(ch, a, vmp, out, part);
    }
    StepArgs<double> a = make_args<double>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_quadrants_t<double>(ch, a, vmp, out, part);
}

int launch_spectra(c3d_channel *ch, const double *vmo, const double *st, double *xs, double *zs, double *rxx,
                   double *rzz, double *rxy) {
    if (ch->precision == C3D_MIXED) {
        StepArgs<float> a = make_args<float>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
        return launch_spectra_t<float>(ch, a, vmo, st, xs, zs, rxx, rzz, rxy);
    }
    StepArgs<double> a = make_args<double>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_spectra_t<double>(ch, a, vmo, st, xs, zs, rxx, rzz, rxy);
}

template <typename R>
static int operator_impl(c3d_channel *ch, int op, int *nl) {
    StepArgs<R> a = make_args<R>(ch, ch->dt_cached > 0 ? ch->dt_cached : 1.0);
    return launch_op<R>(ch, a, op, (const R *)ch->opbuf[0], (R *)ch->opbuf[1], nl);
}

int launch_operator(c3d_channel *ch, int op, int *nl) {
    if (ch->precision == C3D_MIXED) return operator_impl<float>(ch, op, nl);
    return operator_impl<double>(ch, op, nl);
}

int launch_step(c3d_channel *ch, double dt, int *nl) {
    if (ch->precision == C3D_MIXED) return step_impl<float>(ch, dt, nl);
    return step_impl<double>(ch, dt, nl);
}

template <typename R>
static int project_impl(c3d_channel *ch, int *nl) {
    typedef typename SType<R>::S S;
    set_spec_smem<R>(ch);
    StepArgs<R> a = make_args<R>(ch, 1.0);
    a.bulk = 0;
    R *dd0 = (R *)ch->exz, *dd1 = (R *)ch->eyz, *dd2 = (R *)ch->wsq;
    const size_t bytes = (size_t)ch->g.nf * sizeof(R);
    cudaMemsetAsync(dd0, 0, bytes, ch->stream);
    cudaMemsetAsync(dd1, 0, bytes, ch->stream);
    cudaMemsetAsync(dd2, 0, bytes, ch->stream);
    k_bcond<R><<<nblk(ch->g.np), TPB, 0, ch->stream>>>(ch->g, (S *)ch->u, (S *)ch->v, (S *)ch->w);
    mark(ch, nl, "bcond", 64.0 * ch->g.np);
    int rc = pressure_and_update<R>(ch, a, dd0, dd1, dd2, 0, nl);
    if (rc) return rc;
    return refine_pressure<R>(ch, a, 0, nl);
}

int launch_project(c3d_channel *ch, int *nl) {
    if (ch->precision == C3D_MIXED) return project_impl<float>(ch, nl);
    return project_impl<double>(ch, nl);
}

template <typename R>
static int diag_impl(c3d_channel *ch, int *nl) {
    typedef typename SType<R>::S S;
    StepArgs<R> a = make_args<R>(ch, 1.0);
    cudaMemsetAsync(ch->scal + SCAL_DIVMAX, 0, 2 * sizeof(double), ch->stream);
    cudaMemsetAsync(ch->scal + SCAL_NONFIN, 0, sizeof(double), ch->stream);
    int rc;
    if ((rc = launch_xpass<R>(ch, a, 4, (const R *)ch->diagbuf, nullptr, nl))) return rc;
    if ((rc = launch_zpass<R>(ch, a, 5, (R *)ch->diagbuf, nullptr, nullptr, 0, nl))) return rc;
    k_diag_sums<R><<<1, 256, 0, ch->stream>>>(ch->g, (const S *)ch->u, (const S *)ch->v, (const S *)ch->w, ch->scal);
    mark(ch, nl, "diag_sums", 64.0 * ch->g.np);
    return 0;
}

int launch_diag(c3d_channel *ch, int *nl) {
    if (ch->precision == C3D_MIXED) return diag_impl<float>(ch, nl);
    return diag_impl<double>(ch, nl);
}

int launch_poisson_tables(c3d_channel *ch) {
    const Geo &g = ch->g;
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
    launch_ptables(ch, ak1, ak3, pm, pc, pp);
    cudaError_t e = cudaStreamSynchronize(ch->stream);
    cudaFree(tmp);
    return e == cudaSuccess ? 0 : C3D_ECUDA;
}

int launch_repack(c3d_channel *ch, int dir, int what, int comp, double *fort) {
    double *F = fort ? fort : ch->stage;
    // the repacking kernels loop with four elements per thread and pass: a grid of 16
    // blocks per SM keeps them all active (a full one-element-per-thread grid would
    // evaluate the three idle slots of every thread)
    auto cap = [](int b) { return b < 152 * 16 ? b : 152 * 16; };
    const Geo &g = ch->g;
    const int j0 = (what == 0 || what == 3) ? 0 : 1, j1 = (what == 0 || what == 3) ? g.n2 : g.n2m;
    const long long tot_dev = (long long)(j1 - j0 + 1) * g.np;
    const long long N1 = g.n1m + 1, N2 = g.n2, N3 = g.n3m + 1;
    const long long tot_f = (what == 1) ? N1 * N2 * N3 : (N1 + 1) * (N2 + 1) * (N3 + 1);
    cudaStream_t st = ch->stream;
    const bool mixed = ch->precision == C3D_MIXED;
    const int nb = cap(nblk(dir == 0 ? tot_dev : tot_f));
    if (what == 4 || what == 5) {   // operator operand (to device) / result (to host), working precision
        void *buf = ch->opbuf[what == 4 ? 0 : 1];
        if (!buf || (what == 4) != (dir == 0)) return C3D_EINVAL;
        if (!mixed) {
            if (dir == 0) k_unpack<double><<<cap(nblk((long long)(g.n2 + 1) * g.np)), TPB, 0, st>>>(g, 0, (double *)buf, F, ToF64());
            else k_pack<double><<<nb, TPB, 0, st>>>(g, 0, (const double *)buf, F, FromF64());
        } else {
            if (dir == 0) k_unpack<float><<<cap(nblk((long long)(g.n2 + 1) * g.np)), TPB, 0, st>>>(g, 0, (float *)buf, F, ToF32());
            else k_pack<float><<<nb, TPB, 0, st>>>(g, 0, (const float *)buf, F, FromF32());
        }
        return 0;
    }
    if (what == 3) {   // SGSVIS (0:M1,0:M2,0:M3), device to host only, working precision
        if (dir == 0 || !ch->les[0]) return C3D_EINVAL;
        if (!mixed) k_pack<double><<<nb, TPB, 0, st>>>(g, 0, (const double *)ch->les[0], F, FromF64());
        else k_pack<float><<<nb, TPB, 0, st>>>(g, 0, (const float *)ch->les[0], F, FromF32());
        return 0;
    }
    void *dev = (what == 2) ? ch->hh[ch->cur][comp]
                            : (what == 1) ? ch->p : (comp == 0 ? ch->u : comp == 1 ? ch->v : ch->w);
    if (!mixed) {
        if (dir == 0) k_unpack<double><<<nb, TPB, 0, st>>>(g, what, (double *)dev, F, ToF64());
        else k_pack<double><<<nb, TPB, 0, st>>>(g, what, (const double *)dev, F, FromF64());
    } else if (what == 2) {
        if (dir == 0) k_unpack<float><<<nb, TPB, 0, st>>>(g, what, (float *)dev, F, ToF32());
        else k_pack<float><<<nb, TPB, 0, st>>>(g, what, (const float *)dev, F, FromF32());
    } else {
        if (dir == 0) k_unpack<float2><<<nb, TPB, 0, st>>>(g, what, (float2 *)dev, F, ToDF());
        else k_pack<float2><<<nb, TPB, 0, st>>>(g, what, (const float2 *)dev, F, FromDF());
    }
    return 0;
}

}  // namespace c3d
