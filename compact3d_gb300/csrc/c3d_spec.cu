// c3d_spec.cu -- the spectral part of GETDP (compact3d.f:9271-9441): complex FFT of the
// half spectrum along z, and one wall-normal Thomas solve (TDMAP, 9444-9459) per (kx, kz).
#include "c3d_kern.cuh"

namespace c3d {

// Complex FFT along kz of a tile of `tw` kx columns of one plane, in shared memory.
template <typename R>
__device__ __forceinline__ void b_fftz(const StepArgs<R> &a, int sign, int tw, const Blk blk) {
    typedef typename Cx<R>::T C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int n = g.n3m;
    C2 *A = reinterpret_cast<C2 *>(smem_raw), *B = A + n * tw;
    const int ntile = (g.n1h + tw - 1) / tw;
    const int plane = blk.x / ntile, tile = blk.x % ntile;
    const int kx0 = tile * tw;
    const int w = min(tw, g.n1h - kx0);
    C2 *S = reinterpret_cast<C2 *>(a.spec) + (long long)plane * n * g.n1h + kx0;
    const int lsh = __ffs(tw) - 1, lm = tw - 1;   // tw is a power of 2
    for (int e = threadIdx.x; e < n * tw; e += blockDim.x) {
        const int q = e >> lsh, l = e & lm;
        if (l < w) A[e] = S[q * g.n1h + l];
        else { A[e].x = 0; A[e].y = 0; }
    }
    __syncthreads();
    C2 *Z = fft_smem<C2, true>(A, B, a.fz, lsh, tw, 1, sign, threadIdx.x, blockDim.x);
    for (int e = threadIdx.x; e < n * tw; e += blockDim.x) {
        const int q = e >> lsh, l = e & lm;
        if (l < w) S[q * g.n1h + l] = Z[e];
    }
}
template <typename R>
__global__ void __launch_bounds__(TPB) k_fftz(StepArgs<R> a, int sign, int tw) {
    b_fftz<R>(a, sign, tw, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// Complex FFT along kz, one warp per kx column, for N3M = 32 N1 (four-step form).  The
// block stages a tile of TWW kx columns of one plane in shared memory (coalesced rows,
// padded pitch); a warp holds its column as x[n1] = X(32 n1 + lane), takes the N1-point
// DFT over n1 in registers, multiplies by exp(sign 2 pi i lane k1 / N3M), and finishes
// with a 32-point DFT across the lanes (five decimation-in-frequency shuffle stages),
// after which lane l holds the outputs k1 + N1 bitrev5(l).  Twiddles come from the z
// plan's table exp(-2 pi i j / N3M).
constexpr int TWW = 16;    // kx columns per block
constexpr int FZW = 8;     // warps per block
template <typename R, int N1, int SIGN>
__device__ __forceinline__ void b_fftz4(const StepArgs<R> &a, const Blk blk) {
    typedef typename Cx<R>::T C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2 *T = reinterpret_cast<C2 *>(smem_raw);
    const Geo g = a.g;
    constexpr int n = 32 * N1, pitch = TWW + 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int ntile = (g.n1h + TWW - 1) / TWW;
    const int plane = blk.x / ntile, kx0 = (blk.x % ntile) * TWW;
    const int w = min(TWW, g.n1h - kx0);
    C2 *S = reinterpret_cast<C2 *>(a.spec) + (long long)plane * n * g.n1h + kx0;
    const C2 *tw = twsel<C2>(a.fz);
    auto twd = [&](int j) {   // exp(SIGN 2 pi i j / n)
        C2 t = __ldg(&tw[j]);
        if constexpr (SIGN > 0) t.y = -t.y;
        return t;
    };
    // the tile arrives by asynchronous copies (no register staging), all in flight at once
    for (int e = threadIdx.x; e < n * TWW; e += FZW * 32) {
        const int q = e >> 4, l = e & (TWW - 1);
        if (l < w) cp_async_c2(&T[q * pitch + l], &S[q * g.n1h + l]);
    }
    cp_async_wait_all();
    C2 wn1[N1], tl[N1], ts[5];
#pragma unroll
    for (int j = 0; j < N1; ++j) { wn1[j] = twd(32 * j); tl[j] = twd(lane * j); }
#pragma unroll
    for (int st = 0; st < 5; ++st) {   // stage with half-distance h = 16 >> st: exp(SIGN 2 pi i (lane mod h) / 2h)
        const int h = 16 >> st;
        ts[st] = twd((lane & (h - 1)) * (n / (2 * h)));
    }
    __syncthreads();
    for (int c = wid; c < w; c += FZW) {
        C2 x[N1];
#pragma unroll
        for (int m = 0; m < N1; ++m) x[m] = T[(32 * m + lane) * pitch + c];
        rdft<N1, SIGN, N1>(x, wn1);
#pragma unroll
        for (int k = 1; k < N1; ++k) x[k] = cmul(x[k], tl[k]);
#pragma unroll
        for (int st = 0; st < 5; ++st) {
            const int h = 16 >> st;
            const bool hi = (lane & h) != 0;
#pragma unroll
            for (int k = 0; k < N1; ++k) {
                C2 o;
                o.x = __shfl_xor_sync(0xffffffffu, x[k].x, h);
                o.y = __shfl_xor_sync(0xffffffffu, x[k].y, h);
                x[k] = hi ? cmul(csub(o, x[k]), ts[st]) : cadd(x[k], o);
            }
        }
        __syncwarp();
        // x[k] is frequency k + N1 * bitrev5(lane); it goes to tile row lane + 32 k, so that
        // the 16 lanes of a half-warp write 16 distinct bank pairs (row k + N1 bitrev5(lane)
        // puts them on 2 when N1 = 12), and the copy-out below reads each frequency's row.
#pragma unroll
        for (int k = 0; k < N1; ++k) T[(lane + 32 * k) * pitch + c] = x[k];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * TWW; e += FZW * 32) {
        const int q = e >> 4, l = e & (TWW - 1);
        const int lq = q / N1, kq = q - lq * N1;
        const int row = (int)(__brev((unsigned)lq) >> 27) + 32 * kq;
        if (l < w) S[q * g.n1h + l] = T[row * pitch + l];
    }
}
template <typename R, int N1, int SIGN>
__global__ void __launch_bounds__(FZW * 32) k_fftz4(StepArgs<R> a) {
    b_fftz4<R, N1, SIGN>(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// One Thomas solve per mode (kx, kz) with A_J = PMJ, B_J = PCJ - AK3 - AK1, C_J = PPJ,
// factors tabulated by k_ptables; the (0,0) mode has row 1 = (0, 1, 0 | 0) and the
// imaginary parts of the self-conjugate modes are zero (compact3d.f:9363-9397).
// FP64 form: FP64 arithmetic.  Mixed form: the same recurrences in double-float
// arithmetic (FP32 instructions), with double-float factor tables: on stretched grids the
// low-wavenumber systems are near-singular and an FP32 recurrence loses accuracy.  The
// forward values are stored at the spectrum's precision between the two sweeps.
// The j loops load UJ planes ahead so that the sequential chain does not wait on memory.
constexpr int UJ = 8;

__device__ __forceinline__ void b_poisson64(const StepArgs<double> &a, const Blk blk) {
    const Geo g = a.g;
    const int nm = g.n1h * g.n3m;
    const int mode = blk.x * blockDim.x + threadIdx.x;
    if (mode >= nm) return;
    const int kx = mode % g.n1h, kz = mode / g.n1h;
    const bool selfc = (kx == 0 || kx == g.n1m / 2) && (kz == 0 || kz == g.n3m / 2);
    double2 *S = reinterpret_cast<double2 *>(a.spec) + mode;
    const long long s = nm;
    const int N = g.n2m;
    const double *RB = a.prb + mode, *GM = a.pgam + mode;
    double xr = 0.0, xi = 0.0;
    for (int j0 = 0; j0 < N; j0 += UJ) {
        double2 q[UJ];
        double rb[UJ], am[UJ];
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (j0 + u < N) { q[u] = S[(j0 + u) * s]; rb[u] = RB[(j0 + u) * s]; am[u] = a.pmj[j0 + u + 1]; }
#pragma unroll
        for (int u = 0; u < UJ; ++u) {
            const int jj = j0 + u;
            if (jj < N) {
                double fr = q[u].x;
                if (jj == 0 && mode == 0) fr = 0.0;      // row 1 of the (1,1) mode: x_1 = 0
                if (jj == 0) { xr = fr * rb[u]; xi = q[u].y * rb[u]; }
                else { xr = (fr - am[u] * xr) * rb[u]; xi = (q[u].y - am[u] * xi) * rb[u]; }
                q[u] = make_double2(xr, xi);
            }
        }
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (j0 + u < N) S[(j0 + u) * s] = q[u];
    }
    S[(N - 1) * s] = make_double2(xr, selfc ? 0.0 : xi);
    for (int jt = N - 2; jt >= 0; jt -= UJ) {
        double2 q[UJ];
        double gm[UJ];
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (jt - u >= 0) { q[u] = S[(jt - u) * s]; gm[u] = GM[(jt - u + 1) * s]; }
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (jt - u >= 0) {
                xr = q[u].x - gm[u] * xr;
                xi = q[u].y - gm[u] * xi;
                q[u] = make_double2(xr, selfc ? 0.0 : xi);
            }
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (jt - u >= 0) S[(jt - u) * s] = q[u];
    }
}
__global__ void __launch_bounds__(TPB) k_poisson64(StepArgs<double> a) {
    b_poisson64(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

__device__ __forceinline__ void b_poisson32(const StepArgs<float> &a, const Blk blk) {
    const Geo g = a.g;
    const int nm = g.n1h * g.n3m;
    const int mode = blk.x * blockDim.x + threadIdx.x;
    if (mode >= nm) return;
    const int kx = mode % g.n1h, kz = mode / g.n1h;
    const bool selfc = (kx == 0 || kx == g.n1m / 2) && (kz == 0 || kz == g.n3m / 2);
    float2 *S = reinterpret_cast<float2 *>(a.spec) + mode;
    const long long s = nm;
    const int N = g.n2m;
    const float2 *RB = a.prbdf + mode, *GM = a.pgamdf + mode;
    float2 xr = make_float2(0.f, 0.f), xi = xr;
    // loads issued one batch ahead: (q, rb, am) hold batch j0, (qn, rbn, amn) batch j0+UJ
    float2 q[UJ], rb[UJ], am[UJ], qn[UJ], rbn[UJ], amn[UJ];
#pragma unroll
    for (int u = 0; u < UJ; ++u)
        if (u < N) { q[u] = S[u * s]; rb[u] = RB[u * s]; am[u] = a.pmjdf[u + 1]; }
    for (int j0 = 0; j0 < N; j0 += UJ) {
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (j0 + UJ + u < N) {
                qn[u] = S[(j0 + UJ + u) * s]; rbn[u] = RB[(j0 + UJ + u) * s]; amn[u] = a.pmjdf[j0 + UJ + u + 1];
            }
#pragma unroll
        for (int u = 0; u < UJ; ++u) {
            const int jj = j0 + u;
            if (jj < N) {
                float fr = q[u].x;
                if (jj == 0 && mode == 0) fr = 0.f;
                if (jj == 0) { xr = df_mul(make_float2(fr, 0.f), rb[u]); xi = df_mul(make_float2(q[u].y, 0.f), rb[u]); }
                else {
                    xr = df_mul(df_fsub(fr, df_mul(am[u], xr)), rb[u]);
                    xi = df_mul(df_fsub(q[u].y, df_mul(am[u], xi)), rb[u]);
                }
                q[u] = make_float2(xr.x, xi.x);
            }
        }
#pragma unroll
        for (int u = 0; u < UJ; ++u) {
            if (j0 + u < N) S[(j0 + u) * s] = q[u];
            q[u] = qn[u]; rb[u] = rbn[u]; am[u] = amn[u];
        }
    }
    S[(N - 1) * s] = make_float2(xr.x, selfc ? 0.f : xi.x);
    // backward sweep; its first batch reads values this thread stored above
    float2 gm[UJ], gmn[UJ];
#pragma unroll
    for (int u = 0; u < UJ; ++u)
        if (N - 2 - u >= 0) { q[u] = S[(N - 2 - u) * s]; gm[u] = GM[(N - 1 - u) * s]; }
    for (int jt = N - 2; jt >= 0; jt -= UJ) {
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (jt - UJ - u >= 0) { qn[u] = S[(jt - UJ - u) * s]; gmn[u] = GM[(jt - UJ - u + 1) * s]; }
#pragma unroll
        for (int u = 0; u < UJ; ++u)
            if (jt - u >= 0) {
                xr = df_fsub(q[u].x, df_mul(gm[u], xr));
                xi = df_fsub(q[u].y, df_mul(gm[u], xi));
                q[u] = make_float2(xr.x, selfc ? 0.f : xi.x);
            }
#pragma unroll
        for (int u = 0; u < UJ; ++u) {
            if (jt - u >= 0) S[(jt - u) * s] = q[u];
            q[u] = qn[u]; gm[u] = gmn[u];
        }
    }
}
__global__ void __launch_bounds__(TPB) k_poisson32(StepArgs<float> a) {
    b_poisson32(a, Blk{blockIdx.x, blockIdx.y, gridDim.x});
}

// Factor tables of TDMAP's recurrence for every mode (FP64; double-float copies when rb32 != 0).
__global__ void k_ptables(Geo g, const double *ak1, const double *ak3, const double *pmj, const double *pcj,
                          const double *ppj, double *rb, double *gam, float2 *rb32, float2 *gam32) {
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
    if (rb32) { rb32[mode] = St<float>::from_double(1.0 / bet); gam32[mode] = make_float2(0.f, 0.f); }
    double cprev = C1;
    for (int J = 2; J <= g.n2m; ++J) {
        double gm = cprev / bet;
        bet = (pcj[J] - lam3 - lam1) - pmj[J] * gm;
        const long long q = (long long)(J - 1) * nm + mode;
        gam[q] = gm;
        rb[q] = 1.0 / bet;
        if (rb32) { gam32[q] = St<float>::from_double(gm); rb32[q] = St<float>::from_double(1.0 / bet); }
        cprev = ppj[J];
    }
}

constexpr int TWZ_MAX = 16;   // widest z-FFT tile the autotuner tries

template <typename R>
void set_spec_smem(c3d_channel *ch) {
    typedef typename Cx<R>::T C2;
    const size_t smz = 2 * (size_t)ch->g.n3m * TWZ_MAX * sizeof(C2);
    cudaFuncSetAttribute(k_fftz<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz);
}

// The four-step z FFT for N3M = 32 N1; false when N3M is not of that form.
template <typename R, int SIGN>
static bool launch_fftz4(c3d_channel *ch, StepArgs<R> &a) {
    typedef typename Cx<R>::T C2;
    const Geo &g = ch->g;
    if (g.n3m % 32 != 0) return false;
    const int ntile = (g.n1h + TWW - 1) / TWW;
    const size_t sm = (size_t)g.n3m * (TWW + 1) * sizeof(C2);
    const dim3 grid(g.n2m * ntile), blk(FZW * 32);
    void (*fn)(StepArgs<R>) = nullptr;
    switch (g.n3m / 32) {
        case 2: fn = k_fftz4<R, 2, SIGN>; break;
        case 3: fn = k_fftz4<R, 3, SIGN>; break;
        case 4: fn = k_fftz4<R, 4, SIGN>; break;
        case 6: fn = k_fftz4<R, 6, SIGN>; break;
        case 8: fn = k_fftz4<R, 8, SIGN>; break;
        case 12: fn = k_fftz4<R, 12, SIGN>; break;
        case 16: fn = k_fftz4<R, 16, SIGN>; break;
        default: return false;
    }
    if (sm > 227 * 1024) return false;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    fn<<<grid, blk, sm, ch->stream>>>(a);
    return true;
}

// ---------------------------------------------------------------------------------
// Batch form: the z FFTs of the channels with the same N3M in one launch (the four-step
// warp form when N3M = 32 N1, tiles of 8 kx columns in shared memory otherwise) and the
// Poisson solves of every channel in one launch.
// ---------------------------------------------------------------------------------
constexpr int TW_BATCH = 8;

template <typename R, int N1, int SIGN>
__global__ void __launch_bounds__(FZW * 32) kb_fftz4(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_fftz4<R, N1, SIGN>(A[m.ch], Blk{m.x, m.y, m.gx});
}
template <typename R, int SIGN>
__global__ void __launch_bounds__(TPB) kb_fftz(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_fftz<R>(A[m.ch], SIGN, TW_BATCH, Blk{m.x, m.y, m.gx});
}
__global__ void __launch_bounds__(TPB) kb_poisson64(const StepArgs<double> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_poisson64(A[m.ch], Blk{m.x, m.y, m.gx});
}
__global__ void __launch_bounds__(TPB) kb_poisson32(const StepArgs<float> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_poisson32(A[m.ch], Blk{m.x, m.y, m.gx});
}

template <typename R, int SIGN>
static const void *fftz4_batch_fn(int n1) {
    switch (n1) {
        case 2: return (const void *)kb_fftz4<R, 2, SIGN>;
        case 3: return (const void *)kb_fftz4<R, 3, SIGN>;
        case 4: return (const void *)kb_fftz4<R, 4, SIGN>;
        case 6: return (const void *)kb_fftz4<R, 6, SIGN>;
        case 8: return (const void *)kb_fftz4<R, 8, SIGN>;
        case 12: return (const void *)kb_fftz4<R, 12, SIGN>;
        case 16: return (const void *)kb_fftz4<R, 16, SIGN>;
        default: return nullptr;
    }
}

template <typename R>
int spec_bkern(const c3d_channel *ch, int which, std::vector<BKern> &out) {
    typedef typename Cx<R>::T C2;
    const Geo &g = ch->g;
    if (which == 1) {
        const void *fn = sizeof(R) == 8 ? (const void *)kb_poisson64 : (const void *)kb_poisson32;
        out.push_back({fn, TPB, 0, (unsigned)nblk((long long)g.n1h * g.n3m)});
        return 0;
    }
    if (which != 0 && which != 2) return C3D_EINVAL;
    const void *f4 = nullptr;
    if (g.n3m % 32 == 0) f4 = which == 0 ? fftz4_batch_fn<R, -1>(g.n3m / 32) : fftz4_batch_fn<R, +1>(g.n3m / 32);
    const size_t sm4 = (size_t)g.n3m * (TWW + 1) * sizeof(C2);
    if (f4 && sm4 <= 227 * 1024) {
        out.push_back({f4, FZW * 32, sm4, (unsigned)(g.n2m * ((g.n1h + TWW - 1) / TWW))});
        return 0;
    }
    const size_t smz = 2 * (size_t)g.n3m * TW_BATCH * sizeof(C2);
    const void *fn = which == 0 ? (const void *)kb_fftz<R, -1> : (const void *)kb_fftz<R, +1>;
    out.push_back({fn, TPB, smz, (unsigned)(g.n2m * ((g.n1h + TW_BATCH - 1) / TW_BATCH))});
    return 0;
}
template int spec_bkern<double>(const c3d_channel *, int, std::vector<BKern> &);
template int spec_bkern<float>(const c3d_channel *, int, std::vector<BKern> &);

template <typename R>
int launch_spec(c3d_channel *ch, StepArgs<R> &a, int which, int *nl) {
    typedef typename Cx<R>::T C2;
    cudaStream_t st = ch->stream;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    if (ch->tune.twz == 0 && (which == 0 || which == 2)) {   // four-step form when N3M allows
        if (which == 0 ? launch_fftz4<R, -1>(ch, a) : launch_fftz4<R, +1>(ch, a)) {
            mark(ch, nl, which == 0 ? "fftz_fwd" : "fftz_inv", N * 2 * Rb);
            return 0;
        }
    }
    const int tw = ch->tune.twz == 0 ? 8 : ch->tune.twz;
    const int ntile = (ch->g.n1h + tw - 1) / tw;
    const size_t smz = 2 * (size_t)ch->g.n3m * tw * sizeof(C2);
    switch (which) {
        case 0: k_fftz<R><<<ch->g.n2m * ntile, TPB, smz, st>>>(a, -1, tw); mark(ch, nl, "fftz_fwd", N * 2 * Rb); break;
        case 1:
            if constexpr (sizeof(R) == 8) k_poisson64<<<nblk((long long)ch->g.n1h * ch->g.n3m), TPB, 0, st>>>(a);
            else k_poisson32<<<nblk((long long)ch->g.n1h * ch->g.n3m), TPB, 0, st>>>(a);
            mark(ch, nl, "poisson", N * 2 * Rb + N * 8);
            break;
        case 2: k_fftz<R><<<ch->g.n2m * ntile, TPB, smz, st>>>(a, +1, tw); mark(ch, nl, "fftz_inv", N * 2 * Rb); break;
        default: return C3D_EINVAL;
    }
    return 0;
}

int launch_ptables(c3d_channel *ch, const double *ak1, const double *ak3, const double *pm, const double *pc,
                   const double *pp) {
    const int nm = ch->g.n1h * ch->g.n3m;
    k_ptables<<<nblk(nm), TPB, 0, ch->stream>>>(ch->g, ak1, ak3, pm, pc, pp, ch->prb, ch->pgam, ch->prbdf,
                                                ch->pgamdf);
    return 0;
}

template void set_spec_smem<double>(c3d_channel *);
template void set_spec_smem<float>(c3d_channel *);
template int launch_spec<double>(c3d_channel *, StepArgs<double> &, int, int *);
template int launch_spec<float>(c3d_channel *, StepArgs<float> &, int, int *);

}  // namespace c3d
