// c3d_noalloc.cu -- c3d_divcheck_noalloc: DIVCHECK without any device allocation.
//
// Who needs it: a driver that is not allowed to call cudaMalloc, for example one whose
// device memory is owned entirely by its own pool allocator (the library must not grow
// or fragment that heap behind its back), or a long-running production loop whose memory
// footprint has to stay fixed after start-up.  Such a caller still wants the divergence
// check of its host fields between steps.  c3d_diagnose needs a channel, and c3d_create
// allocates the channel's device state; this entry point instead works out of one
// file-scope __device__ array whose size is fixed at build time, C3D_NOALLOC_MAX_BYTES,
// and which every GPU that loads the library holds until the process exits.
//
// Contract
//   * It calls no cudaMalloc, cudaFree or other allocating routine.  It copies the host
//     velocity into the static array, runs the divergence kernels there and copies one
//     double back.
//   * Grids whose working set does not fit the array are rejected with C3D_EINVAL.
//   * The array is shared by every call in the process and keeps the last call's
//     contents; the running maximum is cleared at the start of each call.  Calls that
//     overlap on the GPU (two host threads, or work issued concurrently on other streams
//     while one call runs) race on the array: callers must serialise them.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current).  Make that first
//     call before any stream capture begins on the device.
//   * All work is issued on the legacy default stream and the call returns after it has
//     finished.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <mutex>
#include <string>
#include "../../include/c3d.h"
#include "c3d_dev.cuh"

namespace c3d {
void set_error(const std::string &msg);
}

namespace {

using namespace c3d;

// The scratch: staging for one Fortran velocity component, the three velocity fields in
// plane-major layout, the x part of the divergence, DY and the running maximum.
static __device__ __align__(256) unsigned char g_na_scratch[C3D_NOALLOC_MAX_BYTES];

constexpr int NA_MAXDEV = 64;
static double *g_na_ptr[NA_MAXDEV];
static std::mutex g_na_mutex;

constexpr int TPB = 128;

__global__ void k_na_unpack(Geo g, double *dev, const double *fort) {
    const long long tot = (long long)(g.n2 + 1) * g.np;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= tot) return;
    const int i = (int)(id % g.n1m);
    const int k = (int)((id / g.n1m) % g.n3m);
    const int j = (int)(id / g.np);
    const long long N1 = g.n1m + 1, N2 = g.n2;
    dev[fidx(g, i, j, k)] = fort[(i + 1) + (N1 + 1) * (j + (N2 + 1) * (long long)(k + 1))];
}

// x part: (V(J+1)-V(J))/DY(J) + compact dU/dx, one warp per row (J = 1..N2M).
template <int C>
__global__ void __launch_bounds__(TPB) k_na_divx(Geo g, const double *u, const double *v, double *divx,
                                                 Cyc<double> c22) {
    const int lane = threadIdx.x & 31;
    const int P = g.n1m / C;
    const int nrows = g.n2m * g.n3m;
    for (int row = blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); row < nrows; row += gridDim.x * (TPB / 32)) {
        const int j = 1 + row / g.n3m, k = row % g.n3m;
        const long long o = fidx(g, 0, j, k), op = fidx(g, 0, j + 1, k);
        double uc[C], vc[C], vp[C], d[C];
        row_load(uc, u + o, lane, P);
        row_load(vc, v + o, lane, P);
        row_load(vp, v + op, lane, P);
        double nx = lane_next(uc[0], lane, P);
#pragma unroll
        for (int t = 0; t < C; ++t) {
            double rr = (t == C - 1) ? nx : uc[t + 1];
            d[t] = 24.0 * g.dx1 * (rr - uc[t]);
        }
        xsolve(d, lane, P, c22);
        const double dyj = g.dy[j];
#pragma unroll
        for (int t = 0; t < C; ++t) d[t] = (vp[t] - vc[t]) / dyj + d[t];
        row_store(divx + o, d, lane, P);
    }
}

__device__ __forceinline__ void na_atomic_max(double *addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// z part: + compact dW/dz and the maximum of |div|, one thread per (column, segment).
template <int L>
__global__ void __launch_bounds__(TPB) k_na_divz(Geo g, const double *w, const double *divx, double *out,
                                                 Cyc<double> c22) {
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nseg = g.n3m / L;
    double m = 0.0;
    if (tid < (long long)g.n2m * nseg * g.n1m) {
        const int i = (int)(tid % g.n1m);
        const long long rest = tid / g.n1m;
        const int k0 = (int)(rest % nseg) * L;
        const int j = 1 + (int)(rest / nseg);
        const int n = g.n3m, s = g.n1m;
        const long long o = fidx(g, i, j, 0);
        const double *W = w + o, *DX = divx + o;
        double r[L];
        zseg<double, L>(r, k0, n, c22, [&](int kk) {
            int kp = kk == n - 1 ? 0 : kk + 1;
            return 24.0 * g.dx3 * (W[kp * s] - W[kk * s]);
        });
#pragma unroll
        for (int t = 0; t < L; ++t) {
            double dv = DX[(k0 + t) * s] + r[t];
            m = isfinite(dv) ? fmax(m, fabs(dv)) : INFINITY;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(FULL, m, off));
    if ((threadIdx.x & 31) == 0) na_atomic_max(out, m);
}

int na_fail(int code, const char *msg) {
    set_error(msg);
    return code;
}

size_t al(size_t n) { return (n + 31) & ~size_t(31); }

}  // namespace

extern "C" int c3d_divcheck_noalloc(const c3d_grid *gr, const double *u, double *divmax) {
    if (!gr || !u || !divmax) return na_fail(C3D_EINVAL, "c3d_divcheck_noalloc: null argument");
    if (!gr->dy) return na_fail(C3D_EINVAL, "c3d_divcheck_noalloc: null DY");
    const int n1m = gr->n1 - 1, n2m = gr->n2 - 1, n3m = gr->n3 - 1;
    const int C = (n1m + 31) / 32;
    const bool cok = (C == 1 || C == 2 || C == 3 || C == 4 || C == 6 || C == 8 || C == 12);
    if (!cok || n1m < 16 || n1m % C != 0 || n1m % 2 != 0 || n3m < 16 || n3m % 16 != 0 || n2m < 4 || n2m > 4096)
        return na_fail(C3D_EINVAL, "c3d_divcheck_noalloc: unsupported extents (c3d_create's rules without the "
                                   "FFT lengths: N1-1 even, >= 16, in 32 lane chunks of 1-12 points; N3-1 a "
                                   "multiple of 16; N2-1 in [4, 4096])");
    if (!(gr->dx1 > 0) || !(gr->dx3 > 0)) return na_fail(C3D_EINVAL, "c3d_divcheck_noalloc: DX1, DX3 must be positive");
    // working set in doubles
    const size_t se = (size_t)(gr->n1 + 1) * (gr->n2 + 1) * (gr->n3 + 1);
    const size_t nf = (size_t)(gr->n2 + 1) * n1m * n3m;
    const size_t need = al(se) + 4 * al(nf) + al(gr->n2 + 1) + 32;
    if (need * sizeof(double) > (size_t)C3D_NOALLOC_MAX_BYTES)
        return na_fail(C3D_EINVAL, "c3d_divcheck_noalloc: grid too large for the static scratch "
                                   "(C3D_NOALLOC_MAX_BYTES); use c3d_create / c3d_diagnose");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAXDEV)
        return na_fail(C3D_ENODEV, "c3d_divcheck_noalloc: no current CUDA device");
    double *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mutex);
        if (!g_na_ptr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
            if (e != cudaSuccess || !p)
                return na_fail(C3D_ECUDA, (std::string("c3d_divcheck_noalloc: cudaGetSymbolAddress: ") +
                                           cudaGetErrorString(e)).c_str());
            g_na_ptr[dev] = (double *)p;
        }
        base = g_na_ptr[dev];
    }
    double *stage = base;
    double *fu = stage + al(se), *fv = fu + al(nf), *fw = fv + al(nf), *divx = fw + al(nf);
    double *dy = divx + al(nf), *res = dy + al(gr->n2 + 1);
    Geo g;
    memset(&g, 0, sizeof(g));
    g.n1m = n1m; g.n2m = n2m; g.n3m = n3m; g.n2 = gr->n2;
    g.np = n1m * n3m;
    g.nf = (long long)nf;
    g.dx1 = gr->dx1; g.dx3 = gr->dx3;
    g.dy = dy;
    cudaStream_t st = 0;
    cudaError_t e = cudaMemcpyAsync(dy, gr->dy, sizeof(double) * (gr->n2 + 1), cudaMemcpyHostToDevice, st);
    double *fields[3] = {fu, fv, fw};
    const long long tot = (long long)(g.n2 + 1) * g.np;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) {
        e = cudaMemcpyAsync(stage, u + c * se, sizeof(double) * se, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) k_na_unpack<<<(int)((tot + TPB - 1) / TPB), TPB, 0, st>>>(g, fields[c], stage);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(res, 0, sizeof(double), st);
    if (e != cudaSuccess)
        return na_fail(C3D_ECUDA, (std::string("c3d_divcheck_noalloc: ") + cudaGetErrorString(e)).c_str());
    const double b = 22.0, r = -2.0 / (b + sqrt(b * b - 4.0));
    Cyc<double> c22 = {r, -r, (int)ceil(log(1e-17) / log(fabs(r)))};
    const int nrows = n2m * n3m;
    const int gx = (nrows + TPB / 32 - 1) / (TPB / 32);
    switch (C) {
        case 1: k_na_divx<1><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        case 2: k_na_divx<2><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        case 3: k_na_divx<3><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        case 4: k_na_divx<4><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        case 6: k_na_divx<6><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        case 8: k_na_divx<8><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
        default: k_na_divx<12><<<gx, TPB, 0, st>>>(g, fu, fv, divx, c22); break;
    }
    const long long zt = (long long)n2m * (n3m / 16) * n1m;
    k_na_divz<16><<<(int)((zt + TPB - 1) / TPB), TPB, 0, st>>>(g, fw, divx, res, c22);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(divmax, res, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return na_fail(C3D_ECUDA, (std::string("c3d_divcheck_noalloc: ") + cudaGetErrorString(e)).c_str());
    if (!isfinite(*divmax)) return na_fail(C3D_ENONFINITE, "c3d_divcheck_noalloc: non-finite divergence");
    return 0;
}
