// c3d_xbatch.cu -- batch kernels of the x-row passes (kernel bodies in c3d_xrows.cuh):
// one launch per pass and kernel instance over the blocks of many channels.
#include <vector>
#include "c3d_xrows.cuh"

namespace c3d {
// ---------------------------------------------------------------------------------
// Batch form: one launch per pass covers the channels whose x rows split into the same
// lane chunk C (and, for xC and xD, the same row-FFT form).  xw warps per block; xA
// as its u, v and w pieces with rows read from global memory.  The work arrays of the
// pressure passes are the channel's exz / eyz / wsq, as in the step.
// ---------------------------------------------------------------------------------

template <typename R, int C, int PART, int W = 32>
__global__ void __launch_bounds__(XMAXT) kb_xA(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_xA<R, C, PART, W>(A[m.ch], Blk{m.x, m.y, m.gx});
}
template <typename R, int C, int W = 32>
__global__ void __launch_bounds__(XMAXT) kb_xB(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    b_xB<R, C, W>(A[m.ch], Blk{m.x, m.y, m.gx});
}
template <typename R, int C, bool X4, int W = 32>
__global__ void __launch_bounds__(XMAXT) kb_xC(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_xC<R, C, 0, X4, W>(a, a.exz, a.eyz, Blk{m.x, m.y, m.gx});
}
template <typename R, int C, bool X4, int W = 32>
__global__ void __launch_bounds__(XMAXT) kb_xD(const StepArgs<R> *__restrict__ A, const BMap *__restrict__ map) {
    const BMap m = map[blockIdx.x];
    const StepArgs<R> &a = A[m.ch];
    b_xD<R, C, X4, W>(a, a.exz, a.wsq, Blk{m.x, m.y, m.gx});
}

template <typename R, int C>
static int xbk(const c3d_channel *ch, int which, int xw, std::vector<BKern> &out) {
    typedef typename Cx<R>::T C2;
    const int nrows = ch->g.n2m * ch->g.n3m;
    const unsigned nb = (unsigned)nblk(nrows, xw), nt = xw * 32;
    const size_t sb = stage_bytes(ch->g.n1m, C) * xw;
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(ch->g.n1m / 2 + 1) * sizeof(C2)) * xw;
    const bool x4 = (C % 2 == 0) && ch->g.n1m == 32 * C;   // register row FFT (see launch_x_c)
    switch (which) {
        case 0:
            out.push_back({(const void *)kb_xA<R, C, 1>, nt, sb, nb, 1, 0});
            out.push_back({(const void *)kb_xA<R, C, 2>, nt, sb, nb, 1, 1});
            out.push_back({(const void *)kb_xA<R, C, 3>, nt, sb, nb, 1, 2});
            return 0;
        case 1: out.push_back({(const void *)kb_xB<R, C>, nt, sb, nb}); return 0;
        case 2:
            if (x4) out.push_back({(const void *)kb_xC<R, C, (C % 2 == 0)>, nt, sb, nb});
            else out.push_back({(const void *)kb_xC<R, C, false>, nt, fb, nb});
            return 0;
        case 3:
            if (x4) out.push_back({(const void *)kb_xD<R, C, (C % 2 == 0)>, nt, sb, nb});
            else out.push_back({(const void *)kb_xD<R, C, false>, nt, fb, nb});
            return 0;
        default: return C3D_EINVAL;
    }
}

// xA and xB (and xC, xD with the shared-memory row FFT) of a short row in a segment of W
// lanes, 32/W rows per warp: chunks of C = N1M/W points instead of N1M/32, so the two
// cross-lane scans of every line solve take log2(W) steps and are shared by more points
// (rows of 48-128 points leave 2-4 points per lane of a whole warp), and a 24- or
// 48-point FFT keeps most of its W lanes busy.  The rows of a warp share J when N3M is a
// multiple of 32/W.
template <typename R, int C, int W>
static int xbk_seg(const c3d_channel *ch, int which, int xw, std::vector<BKern> &out) {
    typedef typename Cx<R>::T C2;
    const int nrows = ch->g.n2m * ch->g.n3m, rpb = xw * 32 / W;
    const unsigned nb = (unsigned)nblk(nrows, rpb), nt = xw * 32;
    // xC and xD: a stage and the two FFT buffers per row segment
    const size_t fb = (stage_bytes(ch->g.n1m, C) + 2 * (size_t)(ch->g.n1m / 2 + 1) * sizeof(C2)) * rpb;
    switch (which) {
        case 0:
            out.push_back({(const void *)kb_xA<R, C, 1, W>, nt, 0, nb, 1, 0});
            out.push_back({(const void *)kb_xA<R, C, 2, W>, nt, 0, nb, 1, 1});
            out.push_back({(const void *)kb_xA<R, C, 3, W>, nt, 0, nb, 1, 2});
            return 0;
        case 1: out.push_back({(const void *)kb_xB<R, C, W>, nt, 0, nb}); return 0;
        case 2: out.push_back({(const void *)kb_xC<R, C, false, W>, nt, fb, nb}); return 0;
        case 3: out.push_back({(const void *)kb_xD<R, C, false, W>, nt, fb, nb}); return 0;
        default: return C3D_EINVAL;
    }
}

// The row segment of the x passes for N1M (lanes W, chunk C = N1M/W), or 0 for a whole warp.
int x_segment_lanes(int n1m, int n3m) {
    const int w = (n1m == 48 || n1m == 64 || n1m == 96) ? 8 : (n1m == 128) ? 16 : 32;
    return (w < 32 && n3m % (32 / w) == 0) ? w : 0;
}

template <typename R>
int xpass_bkern(const c3d_channel *ch, int which, int xw, std::vector<BKern> &out) {
    // xC and xD keep the warp's register row FFT where N1M is a multiple of 64
    if (x_segment_lanes(ch->g.n1m, ch->g.n3m) && (which <= 1 || ch->g.n1m % 64 != 0)) {
        switch (ch->g.n1m) {
            case 48: return xbk_seg<R, 6, 8>(ch, which, xw, out);
            case 64: return xbk_seg<R, 8, 8>(ch, which, xw, out);
            case 96: return xbk_seg<R, 12, 8>(ch, which, xw, out);
            case 128: return xbk_seg<R, 8, 16>(ch, which, xw, out);
            default: break;
        }
    }
    switch ((ch->g.n1m + 31) / 32) {
        case 1: return xbk<R, 1>(ch, which, xw, out);
        case 2: return xbk<R, 2>(ch, which, xw, out);
        case 3: return xbk<R, 3>(ch, which, xw, out);
        case 4: return xbk<R, 4>(ch, which, xw, out);
        case 6: return xbk<R, 6>(ch, which, xw, out);
        case 8: return xbk<R, 8>(ch, which, xw, out);
        case 12: return xbk<R, 12>(ch, which, xw, out);
        default: return C3D_EINVAL;
    }
}
template int xpass_bkern<double>(const c3d_channel *, int, int, std::vector<BKern> &);
template int xpass_bkern<float>(const c3d_channel *, int, int, std::vector<BKern> &);

}  // namespace c3d
