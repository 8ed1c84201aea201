// c3d_kern.cuh -- device helpers shared by the step kernels: state representations,
// coalesced row staging, complex arithmetic and the shared-memory Stockham FFT.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include "c3d_internal.h"

namespace c3d {

constexpr int TPB = 128;
constexpr int XMAXT = 256;   // largest block of the tunable x passes (8 rows)

// ---------------------------------------------------------------------------------
// State representation.
//   FP64 form (R = double): u, v, w, P are FP64 and stencils follow the reference's
//     expressions, e.g. (u_{i-1} - 2 u_i) + u_{i+1}.
//   Mixed form (R = float): u, v, w, P are double-float pairs (hi, lo) of FP32 values,
//     8 bytes like FP64, about 48 significant bits.  Differences of state values are
//     formed exactly as (a.hi - b.hi) + (a.lo - b.lo) and the update U + delta is an FP32
//     two-sum, so the mixed form executes no FP64 instruction on its step path; products
//     and interpolants use hi.
// ---------------------------------------------------------------------------------
template <typename R> struct St;

template <> struct St<double> {
    typedef double S;
    static __device__ __forceinline__ double hi(double a) { return a; }
    static __device__ __forceinline__ double d(double a, double b) { return a - b; }
    static __device__ __forceinline__ double d2(double l, double c, double r) { return (l - 2.0 * c) + r; }
    static __device__ __forceinline__ double add(double a, double x) { return a + x; }
    static __device__ __forceinline__ double dbl(double a) { return a; }
    static __device__ __forceinline__ double scale(double a, double s) { return a * s; }
    static __host__ __device__ __forceinline__ double from_double(double a) { return a; }
    // y-viscous stencil HP u+ - HC u + HM u- as in compact3d.f:6119-6122
    static __device__ __forceinline__ double yvisc(double hp, double hc, double hm, double c0, double up, double uc,
                                                   double um) {
        (void)c0;
        return (hp * up - hc * uc) + hm * um;
    }
};

template <> struct St<float> {
    typedef float2 S;
    static __device__ __forceinline__ float hi(float2 a) { return a.x; }
    static __device__ __forceinline__ float d(float2 a, float2 b) { return (a.x - b.x) + (a.y - b.y); }
    static __device__ __forceinline__ float d2(float2 l, float2 c, float2 r) { return d(l, c) - d(c, r); }
    static __device__ __forceinline__ float2 add(float2 a, float x) {
        float s = a.x + x;
        float v = s - a.x;
        float e = (a.x - (s - v)) + (x - v);   // two-sum error of a.hi + x
        e = e + a.y;
        float h = s + e;
        float l = e - (h - s);
        return make_float2(h, l);
    }
    static __device__ __forceinline__ double dbl(float2 a) { return (double)a.x + (double)a.y; }
    static __device__ __forceinline__ float2 scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
    static __host__ __device__ __forceinline__ float2 from_double(double a) {
        float h = (float)a;
        return make_float2(h, (float)(a - (double)h));
    }
    // HP(u+ - u) - HM(u - u-) + (HP + HM - HC) u: the same stencil without cancellation;
    // c0 = HP + HM - HC is zero up to rounding for every row of MESH.
    static __device__ __forceinline__ float yvisc(float hp, float hc, float hm, float c0, float2 up, float2 uc,
                                                  float2 um) {
        (void)hc;
        return (hp * d(up, uc) - hm * d(uc, um)) + c0 * uc.x;
    }
};

// Double-float arithmetic (FP32 instructions only, about 48 significant bits), used by
// the mixed form where a long recurrence must not lose accuracy (Poisson Thomas sweeps).
__device__ __forceinline__ float2 df_norm(float s, float e) {
    float h = s + e;
    return make_float2(h, e - (h - s));
}
// a * b
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_norm(p, e);
}
// q - t with q a plain float
__device__ __forceinline__ float2 df_fsub(float q, float2 t) {
    float s = q - t.x;
    float v = s - q;
    float e = (q - (s - v)) + (-t.x - v);
    e -= t.y;
    return df_norm(s, e);
}
// a + b (two-sum of the high parts, low parts added to the error term)
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float s = a.x + b.x;
    float v = s - a.x;
    float e = (a.x - (s - v)) + (b.x - v);
    e += a.y + b.y;
    return df_norm(s, e);
}

// Warp shuffles for every state/working type, within segments of w lanes
__device__ __forceinline__ double shfl_any(double v, int src, int w = 32) { return __shfl_sync(FULL, v, src, w); }
__device__ __forceinline__ float shfl_any(float v, int src, int w = 32) { return __shfl_sync(FULL, v, src, w); }
__device__ __forceinline__ dfl shfl_any(dfl v, int src, int w = 32) { return shfl_idx(v, src, w); }
__device__ __forceinline__ float2 shfl_any(float2 v, int src, int w = 32) {
    return make_float2(__shfl_sync(FULL, v.x, src, w), __shfl_sync(FULL, v.y, src, w));
}
// The last value of the previous lane's chunk and the first of the next one, cyclic over
// the P active lanes of a row segment of W lanes.
template <int W = 32, typename T>
__device__ __forceinline__ T sprev(T last, int lane, int P) { return shfl_any(last, (lane == 0) ? P - 1 : lane - 1, W); }
template <int W = 32, typename T>
__device__ __forceinline__ T snext(T first, int lane, int P) { return shfl_any(first, (lane + 1 >= P) ? 0 : lane + 1, W); }

// Stencils shared by both forms, written once per representation.
template <typename R> struct Sten;
template <> struct Sten<double> {
    // (V2^2 - V1^2) with V2 = (v+ + v)/2, V1 = (v + v-)/2  (compact3d.f:6852-6854)
    static __device__ __forceinline__ double vv(double vp, double vc, double vm) {
        double V2 = 0.5 * (vp + vc), V1 = 0.5 * (vc + vm);
        return V2 * V2 - V1 * V1;
    }
    // (a1 + x1) - (a0 + x0): difference of intermediate velocities UH = U + delta
    static __device__ __forceinline__ double dd(double a1, double x1, double a0, double x0) {
        return (a1 + x1) - (a0 + x0);
    }
    // ((a + delta) - dt*g) - dt*dm, the UPCALC update (compact3d.f:1127)
    static __device__ __forceinline__ double upd(double a, double delta, double dtg, double dtdm) {
        return ((a + delta) - dtg) - dtdm;
    }
};
template <> struct Sten<float> {
    static __device__ __forceinline__ float vv(float2 vp, float2 vc, float2 vm) {
        float dv = 0.5f * St<float>::d(vp, vm);
        float sv = 0.5f * ((vp.x + vc.x) + (vc.x + vm.x));
        return dv * sv;
    }
    static __device__ __forceinline__ float dd(float2 a1, float x1, float2 a0, float x0) {
        return St<float>::d(a1, a0) + (x1 - x0);
    }
    static __device__ __forceinline__ float2 upd(float2 a, float delta, float dtg, float dtdm) {
        return St<float>::add(a, (delta - dtg) - dtdm);
    }
};

// ---------------------------------------------------------------------------------
// Coalesced row I/O through a per-warp shared-memory buffer.  Lane l owns the C
// consecutive points [l*C, l*C+C) of a row of n = P*C points; the buffer stores point e
// at e + e/C (one pad slot per chunk) so the chunked reads avoid bank conflicts.
// ---------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T ldro(const T *p) { return *p; }
template <> __device__ __forceinline__ double ldro<double>(const double *p) { return __ldg(p); }
template <> __device__ __forceinline__ float ldro<float>(const float *p) { return __ldg(p); }
template <> __device__ __forceinline__ float2 ldro<float2>(const float2 *p) { return __ldg(p); }

// Direct lane-chunk row I/O: lane l moves its C consecutive elements with the widest
// vector accesses the alignment allows (16, 8 or 4 bytes), without shared memory.
template <typename T, int C>
__device__ __forceinline__ void drow_load(T (&v)[C], const T *__restrict__ g, int lane, int P) {
    constexpr int B = (int)sizeof(T) * C;
    if (lane < P) {
        const T *p = g + lane * C;
        const uintptr_t a = (uintptr_t)p;
        if constexpr (B % 16 == 0) {
            if ((a & 15) == 0) {
                uint4 q[B / 16];
#pragma unroll
                for (int i = 0; i < B / 16; ++i) q[i] = __ldg(reinterpret_cast<const uint4 *>(p) + i);
                memcpy(v, q, B);
                return;
            }
        }
        if constexpr (B % 8 == 0) {
            if ((a & 7) == 0) {
                uint2 q[B / 8];
#pragma unroll
                for (int i = 0; i < B / 8; ++i) q[i] = __ldg(reinterpret_cast<const uint2 *>(p) + i);
                memcpy(v, q, B);
                return;
            }
        }
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = ldro(p + t);
    } else {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = T();
    }
}

template <typename T, int C>
__device__ __forceinline__ void drow_store(T *__restrict__ g, const T (&v)[C], int lane, int P) {
    constexpr int B = (int)sizeof(T) * C;
    if (lane < P) {
        T *p = g + lane * C;
        const uintptr_t a = (uintptr_t)p;
        if constexpr (B % 16 == 0) {
            if ((a & 15) == 0) {
                uint4 q[B / 16];
                memcpy(q, v, B);
#pragma unroll
                for (int i = 0; i < B / 16; ++i) reinterpret_cast<uint4 *>(p)[i] = q[i];
                return;
            }
        }
        if constexpr (B % 8 == 0) {
            if ((a & 7) == 0) {
                uint2 q[B / 8];
                memcpy(q, v, B);
#pragma unroll
                for (int i = 0; i < B / 8; ++i) reinterpret_cast<uint2 *>(p)[i] = q[i];
                return;
            }
        }
#pragma unroll
        for (int t = 0; t < C; ++t) p[t] = v[t];
    }
}

#ifndef C3D_STAGED_ROWS
#define C3D_STAGED_ROWS 0
#endif

template <typename T, int C>
__device__ __forceinline__ void srow_load(T (&v)[C], const T *__restrict__ g, T *sb, int lane, int P) {
    if (!C3D_STAGED_ROWS) {
        (void)sb;
        drow_load(v, g, lane, P);
        return;
    }
    const int n = P * C;
#pragma unroll
    for (int t = 0; t < C; ++t) {
        int e = lane + 32 * t;
        if (e < n) sb[e + e / C] = ldro(g + e);
    }
    __syncwarp();
    if (lane < P) {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = sb[lane * (C + 1) + t];
    } else {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = T();
    }
    __syncwarp();
}

template <typename T, int C>
__device__ __forceinline__ void srow_store(T *__restrict__ g, const T (&v)[C], T *sb, int lane, int P) {
    if (!C3D_STAGED_ROWS) {
        (void)sb;
        drow_store(g, v, lane, P);
        return;
    }
    const int n = P * C;
    if (lane < P) {
#pragma unroll
        for (int t = 0; t < C; ++t) sb[lane * (C + 1) + t] = v[t];
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < C; ++t) {
        int e = lane + 32 * t;
        if (e < n) g[e] = sb[e + e / C];
    }
    __syncwarp();
}

// Lane-chunk row load from a 16-byte aligned shared-memory row (a bulk-copy stage).
template <typename T, int C>
__device__ __forceinline__ void crow_load(T (&v)[C], const T *s, int lane, int P) {
    constexpr int B = (int)sizeof(T) * C;
    if (lane < P) {
        const T *p = s + lane * C;
        if constexpr (B % 16 == 0) {
            uint4 q[B / 16];
#pragma unroll
            for (int i = 0; i < B / 16; ++i) q[i] = reinterpret_cast<const uint4 *>(p)[i];
            memcpy(v, q, B);
        } else if constexpr (B % 8 == 0) {
            uint2 q[B / 8];
#pragma unroll
            for (int i = 0; i < B / 8; ++i) q[i] = reinterpret_cast<const uint2 *>(p)[i];
            memcpy(v, q, B);
        } else {
#pragma unroll
            for (int t = 0; t < C; ++t) v[t] = p[t];
        }
    } else {
#pragma unroll
        for (int t = 0; t < C; ++t) v[t] = T();
    }
}

// Asynchronous global -> shared copy of one complex value (8 or 16 bytes, naturally
// aligned), and the wait for all of this thread's outstanding copies.
template <typename C2>
__device__ __forceinline__ void cp_async_c2(C2 *dst, const C2 *src) {
    static_assert(sizeof(C2) == 8 || sizeof(C2) == 16, "complex of float or double");
    if constexpr (sizeof(C2) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                     "l"(__cvta_generic_to_global(src)) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                     "l"(__cvta_generic_to_global(src)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ---------------------------------------------------------------------------------
// Bulk-copy ring: one lane of a warp streams whole rows (contiguous byte runs) from
// global memory into shared-memory stages with cp.async.bulk; each stage completes on
// its own mbarrier (transaction count = the stage's bytes).  Waits are bounded by the
// global timer and report failure instead of spinning forever.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
// Makes initialised barriers visible to the bulk-copy (async) proxy.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier shared-memory accesses before later async-proxy writes.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}
// Global -> shared bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_addr(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(smem_addr(b)), "r"(parity) : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long gtimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Waits for phase `parity` of barrier b to complete; false after limit_ns (about one
// second by default).
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, unsigned long long limit_ns = 1000000000ull) {
    if (mbar_try_wait(b, parity)) return true;
    const unsigned long long t0 = gtimer_ns();
    while (!mbar_try_wait(b, parity))
        if (gtimer_ns() - t0 > limit_ns) return false;
    return true;
}

// Bytes of the per-warp staging buffer for rows of n1m points.
__host__ __device__ inline size_t stage_bytes(int n1m, int C) { return (size_t)(n1m + n1m / C + 2) * 8; }

// ---------------------------------------------------------------------------------
// Complex helpers and the shared-memory Stockham FFT (radices 4, 2, 3)
// ---------------------------------------------------------------------------------
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
template <typename C2>
__device__ __forceinline__ C2 cmuli(C2 a, int sign) {
    C2 r;
    if (sign < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
    return r;
}

template <typename C2> __device__ __forceinline__ const C2 *twsel(const FftPlan &p);
template <> __device__ __forceinline__ const double2 *twsel<double2>(const FftPlan &p) { return p.tw64; }
template <> __device__ __forceinline__ const float2 *twsel<float2>(const FftPlan &p) { return p.tw32; }

// X_s = sum_r v_r exp(SIGN 2 pi i r s / P), P in {2,3,4}, radix and direction fixed at
// compile time.
template <int P, int SIGN, typename C2>
__device__ __forceinline__ void dftc(C2 (&v)[P]) {
    typedef decltype(v[0].x) T;
    if constexpr (P == 4) {
        C2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        C2 t2 = cadd(v[1], v[3]), t3 = cmuli(csub(v[1], v[3]), SIGN);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else if constexpr (P == 2) {
        C2 a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    } else {
        const T h = (T)0.8660254037844386467637;  // sqrt(3)/2
        C2 t = cadd(v[1], v[2]), u = csub(v[1], v[2]);
        C2 a;
        a.x = v[0].x - (T)0.5 * t.x;
        a.y = v[0].y - (T)0.5 * t.y;
        C2 b = cmuli(u, SIGN);
        b.x *= h;
        b.y *= h;
        v[0] = cadd(v[0], t);
        v[1] = cadd(a, b);
        v[2] = csub(a, b);
    }
}

// In-register DFT of N points (N = 2^a 3^b dividing NT), natural order in and out, by
// recursive radix-4/2/3 decimation in time.  w[j] = exp(SIGN 2 pi i j / NT); every index
// is a compile-time constant, so the recursion unrolls into straight-line code.
template <int N, int SIGN, int NT, typename C2>
__device__ __forceinline__ void rdft(C2 (&x)[N], const C2 (&w)[NT]) {
    if constexpr (N > 1) {
        constexpr int P = (N % 4 == 0) ? 4 : (N % 2 == 0) ? 2 : 3;
        constexpr int M = N / P;
        C2 sub[P][M];
#pragma unroll
        for (int r = 0; r < P; ++r)
#pragma unroll
            for (int m = 0; m < M; ++m) sub[r][m] = x[P * m + r];
#pragma unroll
        for (int r = 0; r < P; ++r) rdft<M, SIGN, NT>(sub[r], w);
#pragma unroll
        for (int k = 0; k < M; ++k) {
            C2 t[P];
#pragma unroll
            for (int r = 0; r < P; ++r) t[r] = (r * k == 0) ? sub[r][k] : cmul(sub[r][k], w[(r * k * (NT / N)) % NT]);
            dftc<P, SIGN>(t);
#pragma unroll
            for (int s = 0; s < P; ++s) x[k + M * s] = t[s];
        }
    }
}

// ---------------------------------------------------------------------------------
// Row FFTs of the x passes in registers (four-step form), for N1M = 64 Q (C = 2Q points
// per lane).  The packed complex row z[m] = x[2m] + i x[2m+1], m < M = 32 Q, sits in the
// lane chunks as z[Q lane + j], j < Q.  Forward: per j a 32-point DFT across the lanes
// (decimation in frequency, five shuffle stages; lane l ends with k1 = bitrev5(l)), the
// twiddle W_M^(j k1), a Q-point DFT over j in registers: lane l holds Z[k1 + 32 k2].
// Inverse: the same steps in reverse order with conjugate twiddles, ending in the lane
// chunks again.  tabM[j] = exp(-2 pi i j / M) is the x plan's table.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

// Real row (lane chunks) -> half spectrum Sp[0..M] (R2C post-processing as in the x pass
// of RHSDP: E + exp(-2 pi i kx / N1M) O).
template <typename R, int C>
__device__ __forceinline__ void xrow_r2c(const R (&d)[C], const typename Cx<R>::T *__restrict__ tabM,
                                         const typename Cx<R>::T *__restrict__ twx, typename Cx<R>::T *Sp, int lane) {
    typedef typename Cx<R>::T C2;
    constexpr int Q = C / 2, M = 32 * Q;
    C2 x[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) { x[j].x = d[2 * j]; x[j].y = d[2 * j + 1]; }
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int h = 16 >> st;
        const bool hi = (lane & h) != 0;
        const C2 w = __ldg(&tabM[(lane & (h - 1)) * (16 * Q / h)]);
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            C2 o;
            o.x = __shfl_xor_sync(0xffffffffu, x[j].x, h);
            o.y = __shfl_xor_sync(0xffffffffu, x[j].y, h);
            x[j] = hi ? cmul(csub(o, x[j]), w) : cadd(x[j], o);
        }
    }
    const int k1 = brev5(lane);
    if constexpr (Q > 1) {
#pragma unroll
        for (int j = 1; j < Q; ++j) x[j] = cmul(x[j], __ldg(&tabM[j * k1]));
        C2 wq[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) wq[j] = __ldg(&tabM[32 * j]);
        rdft<Q, -1, Q>(x, wq);
    }
    const int pl = brev5((32 - k1) & 31);   // lane holding k1' = 32 - k1
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) {
        C2 zo;
        zo.x = __shfl_sync(0xffffffffu, x[Q - 1 - k2].x, pl);
        zo.y = __shfl_sync(0xffffffffu, x[Q - 1 - k2].y, pl);
        if (lane == 0) zo = x[(Q - k2) % Q];   // k1 = 0: Z[M - 32 k2] = Z[32 ((Q - k2) mod Q)]
        const C2 zk = x[k2], zm = cconj(zo);
        const int kx = k1 + 32 * k2;
        C2 E, O;
        E.x = (zk.x + zm.x) * 0.5f;
        E.y = (zk.y + zm.y) * 0.5f;
        const C2 df = csub(zk, zm);
        O.x = df.y * 0.5f;
        O.y = -df.x * 0.5f;
        Sp[kx] = cadd(E, cmul(__ldg(&twx[kx]), O));
    }
    if (lane == 0) {   // Nyquist mode kx = M from Z[0]
        const C2 zk = x[0], zm = cconj(x[0]);
        C2 E, O;
        E.x = (zk.x + zm.x) * 0.5f;
        E.y = (zk.y + zm.y) * 0.5f;
        const C2 df = csub(zk, zm);
        O.x = df.y * 0.5f;
        O.y = -df.x * 0.5f;
        Sp[M] = cadd(E, cmul(__ldg(&twx[M]), O));
    }
}

// Half spectrum Sp[0..M] -> real row in the lane chunks (unscaled; C2R pre-processing as
// in the x pass of GETDP's inverse transform).
template <typename R, int C>
__device__ __forceinline__ void xrow_c2r(R (&d)[C], const typename Cx<R>::T *__restrict__ tabM,
                                         const typename Cx<R>::T *__restrict__ twx, const typename Cx<R>::T *Sp,
                                         int lane) {
    typedef typename Cx<R>::T C2;
    constexpr int Q = C / 2, M = 32 * Q;
    const int k1 = brev5(lane);
    C2 x[Q];
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) {
        const int kx = k1 + 32 * k2;
        const C2 xk = Sp[kx], xm = cconj(Sp[M - kx]);
        const C2 E = cadd(xk, xm);
        const C2 O = cmul(csub(xk, xm), cconj(__ldg(&twx[kx])));
        x[k2].x = E.x - O.y;
        x[k2].y = E.y + O.x;
    }
    if constexpr (Q > 1) {
        C2 wq[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) wq[j] = cconj(__ldg(&tabM[32 * j]));
        rdft<Q, +1, Q>(x, wq);
#pragma unroll
        for (int j = 1; j < Q; ++j) x[j] = cmul(x[j], cconj(__ldg(&tabM[j * k1])));
    }
#pragma unroll
    for (int st = 4; st >= 0; --st) {
        const int h = 16 >> st;
        const bool hi = (lane & h) != 0;
        const C2 w = cconj(__ldg(&tabM[(lane & (h - 1)) * (16 * Q / h)]));
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const C2 t = hi ? cmul(x[j], w) : x[j];
            C2 o;
            o.x = __shfl_xor_sync(0xffffffffu, t.x, h);
            o.y = __shfl_xor_sync(0xffffffffu, t.y, h);
            x[j] = hi ? csub(o, t) : cadd(t, o);
        }
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) { d[2 * j] = x[j].x; d[2 * j + 1] = x[j].y; }
}

// One radix-P Stockham stage: a -> b over 2^lsh interleaved sequences of length n
// (element q of sequence l at q*es + l*ls).  BLOCK = false is one segment of W lanes on
// one sequence (lsh = 0, es = 1, ls = 0, W threads; W < 32: the segments of a warp run
// their own sequences in step), so its index arithmetic folds.
template <int P, int SIGN, bool BLOCK, typename C2, int W = 32>
__device__ __forceinline__ void fft_stage(const C2 *__restrict__ a, C2 *__restrict__ b, const C2 *__restrict__ tw,
                                          int n, int Ns, unsigned mg, int tstep, int lsh, int es, int ls, int tid,
                                          int nthr) {
    if constexpr (!BLOCK) { lsh = 0; es = 1; ls = 0; nthr = W; }
    const int np = n / P, lmask = (1 << lsh) - 1;
    for (int idx = tid; idx < (np << lsh); idx += nthr) {
        const int l = idx & lmask, jj = idx >> lsh;
        const int q = Ns == 1 ? jj : (int)__umulhi((unsigned)jj, mg);   // jj / Ns
        const int kq = jj - q * Ns;
        C2 v[P];
#pragma unroll
        for (int r = 0; r < P; ++r) v[r] = a[(jj + r * np) * es + l * ls];
        if (Ns > 1) {
            const int t1 = kq * tstep;
#pragma unroll
            for (int r = 1; r < P; ++r) {
                C2 t = __ldg(&tw[r * t1]);
                if constexpr (SIGN > 0) t.y = -t.y;
                v[r] = cmul(v[r], t);
            }
        }
        dftc<P, SIGN>(v);
        const int base = q * Ns * P + kq;
#pragma unroll
        for (int r = 0; r < P; ++r) b[(base + r * Ns) * es + l * ls] = v[r];
    }
}

template <typename C2, bool BLOCK, int SIGN, int W = 32>
__device__ __forceinline__ C2 *fft_run(C2 *a, C2 *b, const FftPlan &pl, int lsh, int es, int ls, int tid, int nthr) {
    const int n = pl.n;
    const C2 *tw = twsel<C2>(pl);
    int Ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int p = pl.rad[s];
        const int tstep = n / (Ns * p);
        const unsigned mg = pl.dmag[s];
        if (p == 4) fft_stage<4, SIGN, BLOCK, C2, W>(a, b, tw, n, Ns, mg, tstep, lsh, es, ls, tid, nthr);
        else if (p == 2) fft_stage<2, SIGN, BLOCK, C2, W>(a, b, tw, n, Ns, mg, tstep, lsh, es, ls, tid, nthr);
        else fft_stage<3, SIGN, BLOCK, C2, W>(a, b, tw, n, Ns, mg, tstep, lsh, es, ls, tid, nthr);
        if (BLOCK) __syncthreads(); else __syncwarp();
        C2 *t = a;
        a = b;
        b = t;
        Ns *= p;
    }
    return a;
}

// Stockham FFT of 2^lsh sequences of length pl.n at buf[q*es + l*ls]; threads tid..nthr
// of a segment of W lanes (BLOCK=false: one sequence, lsh = 0, es = 1, ls = 0) or of the
// block (BLOCK=true) cooperate.  Returns the result buffer.
template <typename C2, bool BLOCK, int W = 32>
__device__ __forceinline__ C2 *fft_smem(C2 *a, C2 *b, const FftPlan &pl, int lsh, int es, int ls, int sign, int tid,
                                        int nthr) {
    if (sign < 0) return fft_run<C2, BLOCK, -1, W>(a, b, pl, lsh, es, ls, tid, nthr);
    return fft_run<C2, BLOCK, +1, W>(a, b, pl, lsh, es, ls, tid, nthr);
}

// L2 prefetch of one address (fire and forget)
__device__ __forceinline__ void pf_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The w lanes of a row segment (lane = the lane within it) prefetch `bytes` contiguous
// bytes starting at p into L2 (128-byte lines).
__device__ __forceinline__ void pf_row(const void *p, int bytes, int lane, int w = 32) {
    const char *c = (const char *)p;
    for (int off = lane * 128; off < bytes; off += w * 128) pf_l2(c + off);
}

// The warp prefetches into L2 the window of positions [k0-m, k0+len+m) of the columns it
// covers: lane t takes positions t, t+32, ...; each position is `span` bytes starting at
// base + k*stride_bytes (the warp's 32 consecutive columns).
__device__ __forceinline__ void pf_cols(const void *base, long long stride_bytes, int span, int k0, int m,
                                        int len, int n, int lane) {
    const char *b = (const char *)base;
    for (int t = lane; t < len + 2 * m; t += 32) {
        int k = k0 - m + t;
        k = (k % n + n) % n;
        const char *p = b + (long long)k * stride_bytes;
        pf_l2(p);
        if (span > 128) pf_l2(p + 128);
    }
}

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

inline int nblk(long long n, int b = TPB) { return (int)((n + b - 1) / b); }

// Block coordinates of a kernel body within its channel's own grid: the launch's block
// index for a single channel, the mapped one when a launch covers a batch of channels.
struct Blk { unsigned x, y, gx; };

// z-direction thread mapping: thread per (i, segment of L points, plane j >= jlo)
template <int L>
__device__ __forceinline__ bool zcoord(const Blk blk, const Geo &g, int jlo, int &i, int &j, int &k0) {
    // 32-bit index arithmetic: a grid has fewer than 2^32 threads (N / L points)
    const unsigned tid = blk.x * blockDim.x + threadIdx.x;
    const unsigned nseg = (unsigned)(g.n3m / L), n1 = (unsigned)g.n1m;
    const unsigned tot = (unsigned)(g.n2m - jlo + 1) * nseg * n1;
    if (tid >= tot) return false;
    const unsigned rest = tid / n1;
    i = (int)(tid - rest * n1);
    const unsigned jq = rest / nseg;
    k0 = (int)(rest - jq * nseg) * L;
    j = jlo + (int)jq;
    return true;
}

template <int L>
__device__ __forceinline__ bool zcoord(const Geo &g, int jlo, int &i, int &j, int &k0) {
    return zcoord<L>(Blk{blockIdx.x, blockIdx.y, gridDim.x}, g, jlo, i, j, k0);
}

constexpr int ZL = 16;   // z segment length

}  // namespace c3d
