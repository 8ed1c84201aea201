// c3d_ckpt.cu -- device side of the checkpoint format: the fields of the channel state in
// the record order of CWRITE (compact3d.f:832-872), i fastest, then j, then k:
//   what 0: ((( U(I,J,K,1..3), I=1,N1M), J=0,N2), K=1,N3M)   (the three components interleaved)
//   what 1: ((( P(I,J,K), I=1,N1M), J=1,N2M), K=1,N3M)
//   what 2: (((( HH(I,J,K,NV), I=1,N1M), J=1,N2M), K=1,N3M), NV=1,3)   (the AB2 history)
// dir 0 packs the device state into buf (REAL*8), dir 1 unpacks buf into the state.
#include "c3d_kern.cuh"

#include <algorithm>

namespace c3d {

struct CkF64 {
    __device__ static double get(const double *a, long long q) { return a[q]; }
    __device__ static void put(double *a, long long q, double x) { a[q] = x; }
};
struct CkDF {
    __device__ static double get(const float2 *a, long long q) { return St<float>::dbl(a[q]); }
    __device__ static void put(float2 *a, long long q, double x) { a[q] = St<float>::from_double(x); }
};
struct CkF32 {
    __device__ static double get(const float *a, long long q) { return (double)a[q]; }
    __device__ static void put(float *a, long long q, double x) { a[q] = (float)x; }
};

// One field (or one component of U) between the device layout ((j n3m + k) n1m + i) and
// its place in the record: element (i, j, k) at buf[stride * ((k nj + (j - j0)) n1m + i) + off].
template <typename T, typename A>
__global__ void __launch_bounds__(TPB) k_ckpt(Geo g, int dir, T *dev, double *buf, int j0, int nj, int stride,
                                            int off) {
    const long long n = (long long)nj * g.np;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % g.n1m);
        const long long r = e / g.n1m;
        const int k = (int)(r % g.n3m), jj = (int)(r / g.n3m);
        const long long q = fidx(g, i, j0 + jj, k);
        const long long b = (long long)stride * (((long long)k * nj + jj) * g.n1m + i) + off;
        if (dir == 0) buf[b] = A::get(dev, q);
        else A::put(dev, q, buf[b]);
    }
}

template <typename T, typename A>
static void ckpt_field(c3d_channel *ch, int dir, void *dev, double *buf, int j0, int nj, int stride, int off) {
    const long long n = (long long)nj * ch->g.np;
    const int nb = (int)std::min<long long>((n + TPB - 1) / TPB, 152LL * 16);
    k_ckpt<T, A><<<nb, TPB, 0, ch->stream>>>(ch->g, dir, (T *)dev, buf, j0, nj, stride, off);
}

int launch_ckpt(c3d_channel *ch, int dir, int what, double *buf) {
    const Geo &g = ch->g;
    const bool mixed = ch->precision == C3D_MIXED;
    if (what == 0) {
        void *comp[3] = {ch->u, ch->v, ch->w};
        for (int c = 0; c < 3; ++c) {
            if (mixed) ckpt_field<float2, CkDF>(ch, dir, comp[c], buf, 0, g.n2 + 1, 3, c);
            else ckpt_field<double, CkF64>(ch, dir, comp[c], buf, 0, g.n2 + 1, 3, c);
        }
    } else if (what == 1) {
        if (mixed) ckpt_field<float2, CkDF>(ch, dir, ch->p, buf, 1, g.n2m, 1, 0);
        else ckpt_field<double, CkF64>(ch, dir, ch->p, buf, 1, g.n2m, 1, 0);
    } else if (what == 2) {
        const long long nf = (long long)g.n1m * g.n2m * g.n3m;
        for (int c = 0; c < 3; ++c) {
            double *b = buf + c * nf;
            if (mixed) ckpt_field<float, CkF32>(ch, dir, ch->hh[ch->cur][c], b, 1, g.n2m, 1, 0);
            else ckpt_field<double, CkF64>(ch, dir, ch->hh[ch->cur][c], b, 1, g.n2m, 1, 0);
        }
    } else {
        return C3D_EINVAL;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

}  // namespace c3d
