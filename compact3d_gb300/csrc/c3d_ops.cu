// c3d_ops.cu -- the step's operators one at a time, on an operand field held by the
// channel: the compact operators along x (CTDMA11, compact3d.f:8952-9000) and z (CTDMA33,
// 9003-9046) with the right-hand sides the momentum routines use, the wall-normal finite
// differences of RHS1/RHS2, and the pressure Poisson solve GETDP (9271-9441).
//
//   DX1  (1,22,1) x = 24 DX1 (F(I+1) - F(I))          e.g. RHS1 loop 50, RHSDP
//   DX2  (1,10,1) x = 12 DX1^2 (F(I-1) - 2F(I) + F(I+1))  RHS1 loop 20
//   IX   (1,6,1)  x = 4 (F(I) + F(I+1))                RHS1 loop 50
//   DZ1, DZ2, IZ  the same along z
//   DY1  (F(J) - F(J-1)) / H(J), J = 2..N2M           RHS2 loop 10
//   DY2  HP(J) F(J+1) - HC(J) F(J) + HM(J) F(J-1)     RHS1 loop 10
//   POISSON  GETDP: F = RDP at J = 1..N2M -> DP
// Every operator reads the planes it needs of the operand and writes planes 1..N2M of the
// result (2..N2M for DY1).
#include "c3d_kern.cuh"

namespace c3d {

template <typename R, int C>
__global__ void __launch_bounds__(TPB) k_op_x(StepArgs<R> a, int op, const R *in, R *out) {
    typedef typename Cx<R>::T C2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geo g = a.g;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int P = g.n1m / C;
    const int M = g.n1m / 2;
    const size_t sbytes = stage_bytes(g.n1m, C), fbytes = 2 * (size_t)(M + 1) * sizeof(C2);
    unsigned char *wb = smem_raw + wid * (sbytes + fbytes);
    R *sb = reinterpret_cast<R *>(wb);
    C2 *bufa = reinterpret_cast<C2 *>(wb + sbytes);
    C2 *bufb = bufa + (M + 1);
    R *rbuf = reinterpret_cast<R *>(bufa);
    const C2 *twx;
    if constexpr (sizeof(R) == 8) twx = reinterpret_cast<const C2 *>(a.twx64);
    else twx = reinterpret_cast<const C2 *>(a.twx32);
    const int nrows = g.n2m * g.n3m;
    for (int row = blockIdx.x * (TPB / 32) + wid; row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k);
        C2 *Sp = reinterpret_cast<C2 *>(a.spec) + ((long long)(j - 1) * g.n3m + k) * g.n1h;
        if (op == C3D_OP_POISSON + 100) {   // spectrum -> real row (C2R), scaled by 1/(N1M N3M)
            for (int kx = lane; kx <= M; kx += 32) bufb[kx] = Sp[kx];
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
            C2 *Zr = fft_smem<C2, false>(bufa, bufb, a.fx, 0, 1, 0, +1, lane, 32);
            const R *rz = reinterpret_cast<const R *>(Zr);
            const R scale = a.xscale;
            R v[C];
#pragma unroll
            for (int t = 0; t < C; ++t) v[t] = lane < P ? rz[lane * C + t] * scale : R(0);
            __syncwarp();
            srow_store(out + o, v, sb, lane, P);
            continue;
        }
        R f[C], d[C];
        srow_load(f, in + o, sb, lane, P);
        const R pv = sprev(f[C - 1], lane, P), nx = snext(f[0], lane, P);
        if (op == C3D_OP_POISSON) {   // real row -> spectrum (R2C)
            if (lane < P) {
#pragma unroll
                for (int t = 0; t < C; ++t) rbuf[lane * C + t] = f[t];
            }
            __syncwarp();
            C2 *Z = fft_smem<C2, false>(bufa, bufb, a.fx, 0, 1, 0, -1, lane, 32);
            for (int kx = lane; kx <= M; kx += 32) {
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
            continue;
        }
        const Cyc<R> *cy = op == C3D_OP_DX1 ? &a.c22x : op == C3D_OP_DX2 ? &a.c10x : &a.c6x;
#pragma unroll
        for (int t = 0; t < C; ++t) {
            const R l = t == 0 ? pv : f[t - 1], r = t == C - 1 ? nx : f[t + 1];
            if (op == C3D_OP_DX1) d[t] = a.f24x * (r - f[t]);
            else if (op == C3D_OP_DX2) d[t] = a.f12x * ((l - (R)2.0 * f[t]) + r);
            else d[t] = (R)4.0 * (f[t] + r);
        }
        xsolve(d, lane, P, *cy);
        srow_store(out + o, d, sb, lane, P);
    }
}

// z columns: one recurrence of the selected operator over a sliding window of the operand.
template <typename R>
struct WalkOpZ {
    const R *F; int n, s, op; R f24, f12; R fm, fc; int kn;
    __device__ void start(int k) { fm = F[(k == 0 ? n - 1 : k - 1) * s]; fc = F[k * s]; kn = (k + 1 == n) ? 0 : k + 1; }
    __device__ void next(R (&d)[1]) {
        const R fp = F[kn * s];
        if (op == C3D_OP_DZ1) d[0] = f24 * (fp - fc);
        else if (op == C3D_OP_DZ2) d[0] = f12 * ((fm - (R)2.0 * fc) + fp);
        else d[0] = (R)4.0 * (fc + fp);
        fm = fc; fc = fp; kn = (kn + 1 == n) ? 0 : kn + 1;
    }
};

template <typename R, int L>
__global__ void __launch_bounds__(TPB) k_op_z(StepArgs<R> a, int op, const R *in, R *out) {
    const Geo g = a.g;
    int i, j, k0;
    if (!zcoord<L>(g, 1, i, j, k0)) return;
    const int n = g.n3m, s = g.n1m;
    const long long o = fidx(g, i, j, 0);
    R res[1][L];
    const Cyc<R> &cy = op == C3D_OP_DZ1 ? a.c22z : op == C3D_OP_DZ2 ? a.c10z : a.c6z;
    const R rr[1] = {cy.r}, ss[1] = {cy.s};
    WalkOpZ<R> f{in + o, n, s, op, a.f24z, a.f12z};
    zsweep<R, L, WM<R>::M6, 1>(res, k0, n, rr, ss, f);
#pragma unroll
    for (int t = 0; t < L; ++t) out[o + (long long)(k0 + t) * s] = res[0][t];
}

// wall-normal finite differences, one thread per point; blockIdx.y is the plane J - 1
template <typename R>
__global__ void __launch_bounds__(TPB) k_op_y(StepArgs<R> a, int op, const R *in, R *out) {
    const Geo g = a.g;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= g.np) return;
    const int j = 1 + (int)blockIdx.y;
    const long long o = (long long)j * g.np + e;
    if (op == C3D_OP_DY1) {
        out[o] = j >= 2 ? (in[o] - in[o - g.np]) * a.m.rh[j] : R(0);
    } else {
        out[o] = (a.m.hp[j] * in[o + g.np] - a.m.hc[j] * in[o]) + a.m.hm[j] * in[o - g.np];
    }
}

template <typename R, int C>
static void launch_op_x(c3d_channel *ch, StepArgs<R> &a, int op, const R *in, R *out) {
    typedef typename Cx<R>::T C2;
    const int M = ch->g.n1m / 2;
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(M + 1) * sizeof(C2)) * (TPB / 32);
    cudaFuncSetAttribute(k_op_x<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
    k_op_x<R, C><<<nblk((long long)ch->g.n2m * ch->g.n3m, TPB / 32), TPB, fb, ch->stream>>>(a, op, in, out);
}

template <typename R>
static int op_x(c3d_channel *ch, StepArgs<R> &a, int op, const R *in, R *out) {
    switch ((ch->g.n1m + 31) / 32) {
        case 1: launch_op_x<R, 1>(ch, a, op, in, out); return 0;
        case 2: launch_op_x<R, 2>(ch, a, op, in, out); return 0;
        case 3: launch_op_x<R, 3>(ch, a, op, in, out); return 0;
        case 4: launch_op_x<R, 4>(ch, a, op, in, out); return 0;
        case 6: launch_op_x<R, 6>(ch, a, op, in, out); return 0;
        case 8: launch_op_x<R, 8>(ch, a, op, in, out); return 0;
        case 12: launch_op_x<R, 12>(ch, a, op, in, out); return 0;
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
}

template <typename R>
int launch_op(c3d_channel *ch, StepArgs<R> &a, int op, const R *in, R *out, int *nl) {
    const Geo &g = ch->g;
    const double N = (double)g.n1m * g.n2m * g.n3m, Rb = sizeof(R);
    int rc = 0;
    switch (op) {
        case C3D_OP_DX1: case C3D_OP_DX2: case C3D_OP_IX:
            rc = op_x<R>(ch, a, op, in, out);
            mark(ch, nl, "op_x", N * 2 * Rb);
            break;
        case C3D_OP_DZ1: case C3D_OP_DZ2: case C3D_OP_IZ:
            k_op_z<R, ZL><<<nblk((long long)g.n2m * (g.n3m / ZL) * g.n1m), TPB, 0, ch->stream>>>(a, op, in, out);
            mark(ch, nl, "op_z", N * 2 * Rb);
            break;
        case C3D_OP_DY1: case C3D_OP_DY2:
            k_op_y<R><<<dim3(nblk(g.np), g.n2m), TPB, 0, ch->stream>>>(a, op, in, out);
            mark(ch, nl, "op_y", N * 2 * Rb);
            break;
        case C3D_OP_POISSON:
            set_spec_smem<R>(ch);
            if ((rc = op_x<R>(ch, a, C3D_OP_POISSON, in, out))) return rc;
            mark(ch, nl, "op_r2c", N * 2 * Rb);
            if ((rc = launch_spec<R>(ch, a, 0, nl)) || (rc = launch_spec<R>(ch, a, 1, nl)) ||
                (rc = launch_spec<R>(ch, a, 2, nl)))
                return rc;
            rc = op_x<R>(ch, a, C3D_OP_POISSON + 100, in, out);
            mark(ch, nl, "op_c2r", N * 2 * Rb);
            break;
        default:
            set_error("unknown operator");
            return C3D_EINVAL;
    }
    return rc;
}

template int launch_op<double>(c3d_channel *, StepArgs<double> &, int, const double *, double *, int *);
template int launch_op<float>(c3d_channel *, StepArgs<float> &, int, const float *, float *, int *);

}  // namespace c3d
