// c3d_refine.cu -- one step of iterative refinement of the pressure solve for the mixed
// form (precision C3D_MIXED_IR).
//
// After UPCALC the field U satisfies div(U)/DT = RDP - L(DP) = the residual of the
// discrete Poisson problem (L = div grad with the compact x/z and FD y operators of
// RHSDP, compact3d.f:8117-8214).  In the mixed form RDP, DP and the update are FP32, so
// the residual is of the order of FP32 rounding of the velocity derivatives.  The
// refinement evaluates it in double-float arithmetic (the compact solves of RHSDP
// instantiated on the double-float value type; an FP32 evaluation would be as large as
// the residual itself), solves L(DP2) = residual with the same FFT / Thomas path as the
// main solve, and applies U -= DT grad(DP2), P += DP2 with the exact two-sum update of
// the double-float state.  The bulk-flow forcing is unchanged: sum_i d(DP2)/dx is zero.
//
//   ir_z  Dz(w) at the cell centres, double-float (the z part of RHSDP)
//   ir_x  Dx(u) + (v(J+1) - v(J))/DY + Dz(w), times 1/DT, double-float; rounded to FP32;
//         real-to-complex FFT along x into the spectrum
//   (fftz, poisson, fftz: the spectral solve of the main pressure step)
//   ir_d  complex-to-real FFT along x -> DP2, compact d(DP2)/dx
//   ir_e  compact d(DP2)/dz and the update of u, v, w and P
#include "c3d_kern.cuh"

namespace c3d {

__device__ __forceinline__ dfl sdf(float2 a) { return dfl(a.x, a.y); }

struct WalkIrZ {
    const float2 *W; int n, s; dfl f24; dfl wc; int kn;
    __device__ void start(int k) { wc = sdf(W[k * s]); kn = (k + 1 == n) ? 0 : k + 1; }
    __device__ void next(dfl (&d)[1]) {
        const dfl wp = sdf(W[kn * s]);
        d[0] = f24 * (wp - wc);
        wc = wp; kn = (kn + 1 == n) ? 0 : kn + 1;
    }
};

template <int L>
__global__ void __launch_bounds__(TPB) k_ir_z(StepArgs<float> a, RefArgs r) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    dfl out[1][L];
    const dfl rr[1] = {r.c22z.r}, ss[1] = {r.c22z.s};
    WalkIrZ f{a.w + o, n, s, r.f24z};
    zsweep<dfl, L, 13, 1>(out, k0, n, rr, ss, f);
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const long long kk = o + (long long)(k0 + t) * s;
        r.rzh[kk] = out[0][t].h;
        r.rzl[kk] = out[0][t].l;
    }
}

template <int C>
__global__ void __launch_bounds__(TPB) k_ir_x(StepArgs<float> a, RefArgs r) {
    typedef float2 C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    const size_t sbytes = stage_bytes(g.n1m, C), fbytes = 2 * (size_t)(M + 1) * sizeof(C2);
    unsigned char *wb = smem_raw + wid * (sbytes + fbytes);
    float2 *sbS = reinterpret_cast<float2 *>(wb);
    float *sbR = reinterpret_cast<float *>(wb);
    C2 *bufa = reinterpret_cast<C2 *>(wb + sbytes);
    C2 *bufb = bufa + (M + 1);
    float *rbuf = reinterpret_cast<float *>(bufa);
    const C2 *twx = reinterpret_cast<const C2 *>(a.twx32);
    const int nrows = g.n2m * g.n3m;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
        dfl d[C];
        {
            float2 uc[C];
            srow_load(uc, a.u + o, sbS, lane, P);
            const float2 nu = snext(uc[0], lane, P);
#pragma unroll
            for (int t = 0; t < C; ++t) d[t] = r.f24x * (sdf(t == C - 1 ? nu : uc[t + 1]) - sdf(uc[t]));
            xsolve(d, lane, P, r.c22x);
        }
        float res[C];
        {
            const bool up = (j + 1 <= g.n2m), lo = (j >= 2);
            float2 vp[C], vc[C];
            float zh[C], zl[C];
            if (up) srow_load(vp, a.v + op, sbS, lane, P);
            if (lo) srow_load(vc, a.v + o, sbS, lane, P);
            srow_load(zh, r.rzh + o, sbR, lane, P);
            srow_load(zl, r.rzl + o, sbR, lane, P);
            const dfl ry = r.rdy[j];
#pragma unroll
            for (int t = 0; t < C; ++t) {
                const dfl dv = (up ? sdf(vp[t]) : dfl()) - (lo ? sdf(vc[t]) : dfl());
                const dfl tot = ((d[t] + dv * ry) + dfl(zh[t], zl[t])) * r.rdt;
                res[t] = tot.h;
            }
        }
        if (lane < P) {
#pragma unroll
            for (int t = 0; t < C; ++t) rbuf[lane * C + t] = res[t];
        }
        __syncwarp();
        C2 *Z = fft_smem<C2, false>(bufa, bufb, a.fx, 0, 1, 0, -1, lane, 32);
        C2 *Sp = reinterpret_cast<C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        for (int kx = lane; kx <= M; kx += 32) {
            C2 zk = Z[kx == M ? 0 : kx], zm = cconj(Z[kx == 0 ? 0 : M - kx]);
            C2 E, O;
            E.x = 0.5f * (zk.x + zm.x);
            E.y = 0.5f * (zk.y + zm.y);
            C2 df = csub(zk, zm);
            O.x = 0.5f * df.y;
            O.y = -0.5f * df.x;
            Sp[kx] = cadd(E, cmul(twx[kx], O));
        }
        __syncwarp();
    }
}

template <int C>
__global__ void __launch_bounds__(TPB) k_ir_d(StepArgs<float> a) {
    typedef float2 C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    const size_t sbytes = stage_bytes(g.n1m, C), fbytes = 2 * (size_t)(M + 1) * sizeof(C2);
    unsigned char *wb = smem_raw + wid * (sbytes + fbytes);
    float *sbR = reinterpret_cast<float *>(wb);
    C2 *bufa = reinterpret_cast<C2 *>(wb + sbytes);
    C2 *bufb = bufa + (M + 1);
    const C2 *twx = reinterpret_cast<const C2 *>(a.twx32);
    const float scale = a.xscale, f24 = a.f24x;
    const int nrows = g.n2m * g.n3m;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k);
        const C2 *Sp = reinterpret_cast<const C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        for (int kx = lane; kx <= M; kx += 32) bufb[kx] = Sp[kx];
        __syncwarp();
        for (int kx = lane; kx < M; kx += 32) {
            C2 xk = bufb[kx], xm = cconj(bufb[M - kx]);
            C2 E = cadd(xk, xm);
            C2 O = cmul(csub(xk, xm), cconj(twx[kx]));
            C2 Zv;
            Zv.x = E.x - O.y;
            Zv.y = E.y + O.x;
            bufa[kx] = Zv;
        }
        __syncwarp();
        C2 *Zr = fft_smem<C2, false>(bufa, bufb, a.fx, 0, 1, 0, +1, lane, 32);
        const float *rz = reinterpret_cast<const float *>(Zr);
        float dpv[C], d[C];
#pragma unroll
        for (int t = 0; t < C; ++t) dpv[t] = lane < P ? rz[lane * C + t] * scale : 0.f;
        __syncwarp();
        srow_store(a.dp + o, dpv, sbR, lane, P);
        const float pv = sprev(dpv[C - 1], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) d[t] = f24 * (dpv[t] - (t == 0 ? pv : dpv[t - 1]));
        xsolve(d, lane, P, a.c22x);
        srow_store(a.g1 + o, d, sbR, lane, P);
    }
}

struct WalkIrGrad {
    const float *DP; int n, s; float f24; float pm; int kc;
    __device__ void start(int k) { pm = DP[(k == 0 ? n - 1 : k - 1) * s]; kc = k; }
    __device__ void next(float (&d)[1]) {
        const float pc = DP[kc * s];
        d[0] = f24 * (pc - pm);
        pm = pc; kc = (kc + 1 == n) ? 0 : kc + 1;
    }
};

template <int L>
__global__ void __launch_bounds__(TPB) k_ir_e(StepArgs<float> a, int updp) {
    typedef St<float> ST;
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    const float dt = (float)a.dt;
    float out[1][L];
    const float rr[1] = {a.c22z.r}, ss[1] = {a.c22z.s};
    WalkIrGrad f{a.dp + o, n, s, a.f24z};
    zsweep<float, L, WM<float>::M22, 1>(out, k0, n, rr, ss, f);
    float2 *W = a.w + o, *U = a.u + o, *V = a.v + o, *Pp = a.p + o;
    const float *DP = a.dp + o, *DPm = a.dp + fidx(g, i, j - 1, 0), *G1 = a.g1 + o;
    const float Hj = a.m.h[j];
#pragma unroll
    for (int t = 0; t < L; ++t) {
        const int kk = (k0 + t) * s;
        W[kk] = ST::add(W[kk], -(dt * out[0][t]));
        U[kk] = ST::add(U[kk], -(dt * G1[kk]));
        if (j >= 2) V[kk] = ST::add(V[kk], -(dt * (DP[kk] - DPm[kk]) / Hj));
        if (updp) Pp[kk] = ST::add(Pp[kk], DP[kk]);
    }
}

template <int C>
static void launch_ir_x(c3d_channel *ch, StepArgs<float> &a, RefArgs &r, int which) {
    const int M = ch->g.n1m / 2;
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(M + 1) * sizeof(float2)) * (TPB / 32);
    const int grid = nblk((long long)ch->g.n2m * ch->g.n3m, TPB / 32);
    if (which == 0) {
        cudaFuncSetAttribute(k_ir_x<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
        k_ir_x<C><<<grid, TPB, fb, ch->stream>>>(a, r);
    } else {
        cudaFuncSetAttribute(k_ir_d<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
        k_ir_d<C><<<grid, TPB, fb, ch->stream>>>(a);
    }
}

static int ir_x(c3d_channel *ch, StepArgs<float> &a, RefArgs &r, int which) {
    switch ((ch->g.n1m + 31) / 32) {
        case 1: launch_ir_x<1>(ch, a, r, which); return 0;
        case 2: launch_ir_x<2>(ch, a, r, which); return 0;
        case 3: launch_ir_x<3>(ch, a, r, which); return 0;
        case 4: launch_ir_x<4>(ch, a, r, which); return 0;
        case 6: launch_ir_x<6>(ch, a, r, which); return 0;
        case 8: launch_ir_x<8>(ch, a, r, which); return 0;
        case 12: launch_ir_x<12>(ch, a, r, which); return 0;
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
}

int launch_refine(c3d_channel *ch, StepArgs<float> &a, RefArgs &r, int *nl) {
    const Geo &g = ch->g;
    const double N = (double)g.n1m * g.n2m * g.n3m;
    const long long nz = (long long)g.n2m * (g.n3m / ZL) * g.n1m;
    int rc;
    k_ir_z<ZL><<<nblk(nz), TPB, 0, ch->stream>>>(a, r);
    mark(ch, nl, "ir_z", N * 16);
    if ((rc = ir_x(ch, a, r, 0))) return rc;
    mark(ch, nl, "ir_x", N * (24 + 8 + 8));
    if ((rc = launch_spec<float>(ch, a, 0, nl)) || (rc = launch_spec<float>(ch, a, 1, nl)) ||
        (rc = launch_spec<float>(ch, a, 2, nl)))
        return rc;
    if ((rc = ir_x(ch, a, r, 1))) return rc;
    mark(ch, nl, "ir_d", N * (8 + 8));
    k_ir_e<ZL><<<nblk(nz), TPB, 0, ch->stream>>>(a, r.updp);
    mark(ch, nl, "ir_e", N * (64 + 12));
    return 0;
}

}  // namespace c3d
