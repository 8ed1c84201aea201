// c3d_xpass.cu -- launchers of the x-row passes for one channel (kernel bodies in
// c3d_xrows.cuh) and the self-test of the staged passes' bounded wait.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include "c3d_xrows.cuh"

namespace c3d {
// The bounded stage wait of the staged x passes, run on a barrier that nothing arrives on
// and no copy targets, so the wait runs out after limit_ns and sets SCAL_PIPEERR exactly
// as a stalled stage would (c3d_pipe_wait_selftest).
__global__ void k_pipe_selftest(double *scal, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncwarp();
    const bool ok = mbar_wait(&bar, 0, limit_ns);
    if (!ok && threadIdx.x == 0) scal[SCAL_PIPEERR] = 1.0;
}

int launch_pipe_selftest(c3d_channel *ch, double limit_ms) {
    k_pipe_selftest<<<1, 32, 0, ch->stream>>>(ch->scal, (unsigned long long)(limit_ms * 1e6));
    return cudaGetLastError() == cudaSuccess ? 0 : C3D_ECUDA;
}

// ---------------------------------------------------------------------------------
// launcher
// ---------------------------------------------------------------------------------
// Grid of a persistent kernel: as many blocks as fit on the device at once (at most
// `want`), from the occupancy calculator, cached per (kernel, block, shared memory).
static int persistent_grid(const void *fn, int nt, size_t smem, int want, int device) {
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, size_t, int>, int> cache;
    const auto key = std::make_tuple(fn, nt, smem, device);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    int per_sm;
    if (it != cache.end()) per_sm = it->second;
    else {
        int nsm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, smem) != cudaSuccess) per_sm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
        per_sm *= nsm;
        cache[key] = per_sm;
    }
    return per_sm > 0 ? std::min(want, per_sm) : 0;
}

// xC through the bulk-copy ring (mixed form); false when this shape cannot use it (rows
// not a multiple of 16 bytes, or the stages do not fit in shared memory).
template <typename R, int C, int NS, bool X4>
static bool launch_xc_bulk(c3d_channel *ch, StepArgs<R> &a, int xw, const R *p0, const R *p1) {
    typedef typename Cx<R>::T C2;
    const Geo &g = ch->g;
    if (g.n1m % 4 != 0) return false;
    const XcStage<R> L(g.n1m);
    const size_t wbytes = 16 * NS + (size_t)NS * L.bytes + (X4 ? 0 : 2 * (size_t)(g.n1m / 2 + 1) * sizeof(C2));
    const size_t smem = wbytes * xw;
    if (smem > 227 * 1024) return false;
    auto fn = k_xC<R, C, NS, X4>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int nrows = g.n2m * g.n3m;
    const int grid = persistent_grid((const void *)fn, xw * 32, smem, nblk(nrows, xw), ch->device);
    if (grid <= 0) return false;
    fn<<<grid, xw * 32, smem, ch->stream>>>(a, p0, p1);
    return true;
}

template <typename R, int C>
static int launch_x_c(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl) {
    typedef typename Cx<R>::T C2;
    int rc = 0;
    const int nrows = ch->g.n2m * ch->g.n3m;
    const int xw = (which == 4) ? TPB / 32 : ch->tune.xw;   // rows (warps) per block
    const int grid = nblk(nrows, xw), nt = xw * 32;
    cudaStream_t st = ch->stream;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    const size_t sb = stage_bytes(ch->g.n1m, C) * xw;
    const int M = ch->g.n1m / 2;
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(M + 1) * sizeof(C2)) * xw;
    switch (which) {
        case 0:
            if (ch->tune.xsplit && ch->tune.xstage && ch->g.n1m % 2 == 0) {
                // the pieces with their rows staged by bulk copies (rows of 16-byte multiples)
                const size_t s1 = xa_stage_bytes(1, ch->g.n1m) * xw, s2 = xa_stage_bytes(2, ch->g.n1m) * xw,
                             s3 = xa_stage_bytes(3, ch->g.n1m) * xw;
                if (s2 > 227 * 1024) { set_error("xA stage exceeds shared memory"); return C3D_EINVAL; }
                cudaFuncSetAttribute(k_xAs<R, C, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1);
                cudaFuncSetAttribute(k_xAs<R, C, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2);
                cudaFuncSetAttribute(k_xAs<R, C, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3);
                const bool cc = par_on(ch);   // the pieces as concurrent branches (knob 15)
                if (cc && (rc = par_fork(ch))) return rc;
                k_xAs<R, C, 1><<<grid, nt, s1, cc ? ch->par[0] : st>>>(a);
                mark(ch, nl, "xA_u", N * (16 + 2 * Rb));
                k_xAs<R, C, 2><<<grid, nt, s2, cc ? ch->par[1] : st>>>(a);
                mark(ch, nl, "xA_v", N * (24 + 3 * Rb));
                k_xAs<R, C, 3><<<grid, nt, s3, st>>>(a);
                mark(ch, nl, "xA_w", N * (8 + 2 * Rb));
                if (cc && (rc = par_join(ch))) return rc;
                break;
            }
            if (ch->tune.xsplit) {   // the u, v and w pieces as three kernels
                cudaFuncSetAttribute(k_xA<R, C, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
                cudaFuncSetAttribute(k_xA<R, C, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
                cudaFuncSetAttribute(k_xA<R, C, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
                const bool cc = par_on(ch);
                if (cc && (rc = par_fork(ch))) return rc;
                k_xA<R, C, 1><<<grid, nt, sb, cc ? ch->par[0] : st>>>(a);
                mark(ch, nl, "xA_u", N * (16 + 2 * Rb));   // u, P; R1, HH1
                k_xA<R, C, 2><<<grid, nt, sb, cc ? ch->par[1] : st>>>(a);
                mark(ch, nl, "xA_v", N * (24 + 3 * Rb));   // v, P, u; R2, HH2, E_xy
                k_xA<R, C, 3><<<grid, nt, sb, st>>>(a);
                mark(ch, nl, "xA_w", N * (8 + 2 * Rb));    // w; R3, WW1
                if (cc && (rc = par_join(ch))) return rc;
                break;
            }
            cudaFuncSetAttribute(k_xA<R, C, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
            k_xA<R, C, 0><<<grid, nt, sb, st>>>(a);
            mark(ch, nl, "xA", N * (32 + 7 * Rb));
            break;
        case 1:
            cudaFuncSetAttribute(k_xB<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
            k_xB<R, C><<<grid, nt, sb, st>>>(a);
            mark(ch, nl, "xB", N * 18 * Rb);
            break;
        case 2: {
            bool done = false;
            if constexpr (sizeof(R) == 4) {
                constexpr bool X4 = (C % 2 == 0);
                if (X4 && ch->tune.fxp == 3 && ch->g.n1m == 32 * C) {
                    if (ch->tune.xbulk == 2) done = launch_xc_bulk<R, C, 2, X4>(ch, a, xw, p0, p1);
                    else if (ch->tune.xbulk == 3) done = launch_xc_bulk<R, C, 3, X4>(ch, a, xw, p0, p1);
                } else {
                    if (ch->tune.xbulk == 2) done = launch_xc_bulk<R, C, 2, false>(ch, a, xw, p0, p1);
                    else if (ch->tune.xbulk == 3) done = launch_xc_bulk<R, C, 3, false>(ch, a, xw, p0, p1);
                }
            }
            // register row FFT (all 32 lanes hold a chunk: N1M = 32 C, C even): no shared memory
            if (!done && C % 2 == 0 && ch->tune.fxp == 3 && ch->g.n1m == 32 * C) {
                k_xC<R, C, 0, (C % 2 == 0)><<<grid, nt, sb, st>>>(a, p0, p1);
                done = true;
            }
            if (!done) {
                cudaFuncSetAttribute(k_xC<R, C, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
                k_xC<R, C, 0><<<grid, nt, fb, st>>>(a, p0, p1);
            }
            mark(ch, nl, "xC", N * (16 + 4 * Rb));
            break;
        }
        case 3:
            if (C % 2 == 0 && ch->tune.fxp == 3 && ch->g.n1m == 32 * C) {
                k_xD<R, C, (C % 2 == 0)><<<grid, nt, sb, st>>>(a, p0, p1);
            } else {
                cudaFuncSetAttribute(k_xD<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
                k_xD<R, C><<<grid, nt, fb, st>>>(a, p0, p1);
            }
            mark(ch, nl, "xD", N * 5 * Rb);
            break;
        case 4: {
            const double b = 22.0, r = -2.0 / (b + sqrt(b * b - 4.0));
            Cyc<double> c22 = {r, -r, (int)ceil(log(1e-17) / log(fabs(r)))};
            cudaFuncSetAttribute(k_diag_x<R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sb);
            k_diag_x<R, C><<<grid, TPB, sb, st>>>(a, (double *)p0, c22);
            mark(ch, nl, "diag_x", N * 48);
            break;
        }
        default: return C3D_EINVAL;
    }
    return 0;
}


// xA's pieces (unless staged), xB, and xC and xD (with the shared-memory row FFT and no
// bulk-copy ring) with a row per segment of W lanes (schedule knob x_row_lanes).  Returns
// 0 when launched, 1 when the schedule runs the pass on whole warps, or an error code.
template <typename R, int C, int W>
static int launch_x_seg(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl) {
    typedef typename Cx<R>::T C2;
    const Tune &t = ch->tune;
    if (which == 0 && (!t.xsplit || t.xstage)) return 1;
    if ((which == 2 || which == 3) && (t.fxp == 3 || t.xbulk)) return 1;
    const int nrows = ch->g.n2m * ch->g.n3m, rpb = t.xw * 32 / W;
    const int grid = nblk(nrows, rpb), nt = t.xw * 32;
    const double N = (double)ch->g.n1m * ch->g.n2m * ch->g.n3m, Rb = sizeof(R);
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(ch->g.n1m / 2 + 1) * sizeof(C2)) * rpb;
    cudaStream_t st = ch->stream;
    if (which == 2) {
        cudaFuncSetAttribute(k_xC<R, C, 0, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
        k_xC<R, C, 0, false, W><<<grid, nt, fb, st>>>(a, p0, p1);
        mark(ch, nl, "xC", N * (16 + 4 * Rb));
        return 0;
    }
    if (which == 3) {
        cudaFuncSetAttribute(k_xD<R, C, false, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fb);
        k_xD<R, C, false, W><<<grid, nt, fb, st>>>(a, p0, p1);
        mark(ch, nl, "xD", N * 5 * Rb);
        return 0;
    }
    if (which == 0) {
        const bool cc = par_on(ch);   // the pieces as concurrent branches (knob 15)
        int rc;
        if (cc && (rc = par_fork(ch))) return rc;
        k_xA<R, C, 1, W><<<grid, nt, 0, cc ? ch->par[0] : st>>>(a);
        mark(ch, nl, "xA_u", N * (16 + 2 * Rb));
        k_xA<R, C, 2, W><<<grid, nt, 0, cc ? ch->par[1] : st>>>(a);
        mark(ch, nl, "xA_v", N * (24 + 3 * Rb));
        k_xA<R, C, 3, W><<<grid, nt, 0, st>>>(a);
        mark(ch, nl, "xA_w", N * (8 + 2 * Rb));
        if (cc && (rc = par_join(ch))) return rc;
    } else {
        k_xB<R, C, W><<<grid, nt, 0, st>>>(a);
        mark(ch, nl, "xB", N * 18 * Rb);
    }
    return 0;
}

template <typename R>
int launch_xpass(c3d_channel *ch, StepArgs<R> &a, int which, const R *p0, const R *p1, int *nl) {
    if (which >= 0 && which <= 3 && ch->tune.xlanes) {
        int r = 1;
        switch (ch->g.n1m) {   // the shapes x_segment_lanes accepts
            case 48: r = launch_x_seg<R, 6, 8>(ch, a, which, p0, p1, nl); break;
            case 64: r = launch_x_seg<R, 8, 8>(ch, a, which, p0, p1, nl); break;
            case 96: r = launch_x_seg<R, 12, 8>(ch, a, which, p0, p1, nl); break;
            case 128: r = launch_x_seg<R, 8, 16>(ch, a, which, p0, p1, nl); break;
            default: break;
        }
        if (r <= 0) return r;
    }
    switch ((ch->g.n1m + 31) / 32) {
        case 1: return launch_x_c<R, 1>(ch, a, which, p0, p1, nl);
        case 2: return launch_x_c<R, 2>(ch, a, which, p0, p1, nl);
        case 3: return launch_x_c<R, 3>(ch, a, which, p0, p1, nl);
        case 4: return launch_x_c<R, 4>(ch, a, which, p0, p1, nl);
        case 6: return launch_x_c<R, 6>(ch, a, which, p0, p1, nl);
        case 8: return launch_x_c<R, 8>(ch, a, which, p0, p1, nl);
        case 12: return launch_x_c<R, 12>(ch, a, which, p0, p1, nl);
        default: set_error("unsupported N1M"); return C3D_EINVAL;
    }
}

template int launch_xpass<double>(c3d_channel *, StepArgs<double> &, int, const double *, const double *, int *);
template int launch_xpass<float>(c3d_channel *, StepArgs<float> &, int, const float *, const float *, int *);

}  // namespace c3d
