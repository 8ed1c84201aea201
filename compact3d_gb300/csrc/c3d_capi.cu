#include <cstdio>
// c3d_capi.cu -- the C-ABI of include/c3d.h: channel lifecycle, host<->device transfers,
// the GETUP drop-in step, diagnostics and the batched ensemble.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <vector>
#include "../../include/c3d.h"
#include "c3d_internal.h"

using namespace c3d;

namespace c3d {
static thread_local std::string g_last_error;
static thread_local int g_device = -1;
void set_error(const std::string &msg) { g_last_error = msg; }

bool par_on(const c3d_channel *ch) { return ch->tune.conc && !ch->prof_on; }

int par_fork(c3d_channel *ch) {
    CK_RC(cudaEventRecord(ch->pev[0], ch->stream));
    for (int q = 0; q < 2; ++q) CK_RC(cudaStreamWaitEvent(ch->par[q], ch->pev[0], 0));
    return 0;
}

int par_join(c3d_channel *ch) {
    for (int q = 0; q < 2; ++q) {
        CK_RC(cudaEventRecord(ch->pev[1 + q], ch->par[q]));
        CK_RC(cudaStreamWaitEvent(ch->stream, ch->pev[1 + q], 0));
    }
    return 0;
}

void mark(c3d_channel *ch, int *nl, const char *name, double bytes) {
    (*nl)++;
    if (!ch->prof_on) return;
    int k = -1;
    for (size_t q = 0; q < ch->prof_name.size(); ++q)
        if (ch->prof_name[q] == name) { k = (int)q; break; }
    if (k < 0) {
        k = (int)ch->prof_name.size();
        ch->prof_name.push_back(name);
        ch->prof_ms.push_back(0.0);
        ch->prof_cnt.push_back(0);
        ch->prof_bytes.push_back(bytes);
    }
    if (ch->prof_n + 1 >= (int)ch->prof_ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ch->prof_ev.push_back(e);
    }
    cudaEventRecord(ch->prof_ev[ch->prof_n + 1], ch->stream);
    if ((int)ch->prof_iv.size() <= ch->prof_n) ch->prof_iv.resize(ch->prof_n + 1);
    ch->prof_iv[ch->prof_n] = k;
    ch->prof_n++;
}

void prof_begin(c3d_channel *ch) {
    if (!ch->prof_on) return;
    if (ch->prof_ev.empty()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ch->prof_ev.push_back(e);
    }
    ch->prof_n = 0;
    cudaEventRecord(ch->prof_ev[0], ch->stream);
}

int prof_collect(c3d_channel *ch) {
    if (!ch->prof_on || ch->prof_n == 0) return 0;
    if (cudaEventSynchronize(ch->prof_ev[ch->prof_n]) != cudaSuccess) return C3D_ECUDA;
    for (int i = 0; i < ch->prof_n; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ch->prof_ev[i], ch->prof_ev[i + 1]);
        ch->prof_ms[ch->prof_iv[i]] += ms;
        ch->prof_cnt[ch->prof_iv[i]] += 1;
    }
    ch->prof_n = 0;
    return 0;
}
}  // namespace c3d

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));             \
            return e_ == cudaErrorMemoryAllocation ? C3D_ENOMEM : C3D_ECUDA;            \
        }                                                                               \
    } while (0)

extern "C" {

const char *c3d_error_string(int code) {
    switch (code) {
        case C3D_OK: return "ok";
        case C3D_EINVAL: return "invalid argument (extent, pointer or unsupported size)";
        case C3D_ECUDA: return "CUDA runtime error";
        case C3D_ENOMEM: return "out of device or pinned host memory";
        case C3D_ENOTCONV: return "device iteration cap reached";
        case C3D_ENONFINITE: return "non-finite value in the fields";
        case C3D_ESTATE: return "call made in the wrong state";
        case C3D_ENODEV: return "no usable CUDA device";
        case C3D_EIO: return "checkpoint file could not be written or read";
        default: return "unknown error";
    }
}

const char *c3d_last_error(void) { return c3d::g_last_error.c_str(); }

int c3d_version(void) { return 10000; }

int c3d_set_device(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        set_error("no CUDA device");
        return C3D_ENODEV;
    }
    if (device < 0 || device >= n) {
        set_error("device index out of range");
        return C3D_EINVAL;
    }
    CK(cudaSetDevice(device));
    c3d::g_device = device;
    return 0;
}

}  // extern "C"

namespace {

bool fft_len_ok(int n) {
    if (n < 2) return false;
    while (n % 2 == 0) n /= 2;
    while (n % 3 == 0) n /= 3;
    return n == 1;
}

// Stockham plan of length n = 2^a 3^b: the radices in the order the passes run.
//   variant 0: radix 4 while possible, then 2, then 3
//   variant 1: radix 3 first, then 4, then 2
//   variant 2: radix 2 only, then 3
FftPlan make_plan(int n, int variant) {
    FftPlan p;
    memset(&p, 0, sizeof(p));
    p.n = n;
    int m = n, e3 = 0;
    while (m % 3 == 0) { m /= 3; ++e3; }
    if (variant == 1)
        for (int q = 0; q < e3; ++q) p.rad[p.nst++] = 3;
    if (variant != 2)
        while (m % 4 == 0) { p.rad[p.nst++] = 4; m /= 4; }
    while (m % 2 == 0) { p.rad[p.nst++] = 2; m /= 2; }
    if (variant != 1)
        for (int q = 0; q < e3; ++q) p.rad[p.nst++] = 3;
    // reciprocals ceil(2^32 / Ns) for the index arithmetic of every stage (Ns > 1)
    unsigned ns = 1;
    for (int s = 0; s < p.nst; ++s) {
        p.dmag[s] = ns == 1 ? 0u : (unsigned)(((1ull << 32) + ns - 1) / ns);
        for (unsigned jj = 0; ns > 1 && jj < (unsigned)n; ++jj) {   // exact for every index the stage uses
            const unsigned q = (unsigned)(((unsigned long long)jj * p.dmag[s]) >> 32);
            if (q != jj / ns) { p.nst = -1; return p; }
        }
        ns *= (unsigned)p.rad[s];
    }
    return p;
}

// Supported x extents: N1M = P*C with C = ceil(N1M/32) in {1,2,3,4,6,8,12}.
bool n1_ok(int n1m) {
    int c = (n1m + 31) / 32;
    if (!(c == 1 || c == 2 || c == 3 || c == 4 || c == 6 || c == 8 || c == 12)) return false;
    return n1m % c == 0 && n1m % 2 == 0 && n1m >= 16;
}

template <typename T>
int dalloc(T **p, size_t n) {
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return C3D_ENOMEM;
    }
    return 0;
}

void free_channel(c3d_channel *ch) {
    if (!ch) return;
    void *ptrs[] = {ch->u, ch->v, ch->w, ch->p, ch->dp, ch->scal, ch->part, ch->metric, ch->ycn,
                    ch->prb, ch->pgam, ch->pmj, ch->ycn32, ch->metr, ch->prbdf, ch->pgamdf, ch->pmjdf, ch->bulkw, ch->diagbuf,
                    ch->tw64, ch->tw32, ch->hh[0][0], ch->hh[0][1],
                    ch->hh[0][2], ch->hh[1][0], ch->hh[1][1], ch->hh[1][2], ch->r[0], ch->r[1],
                    ch->r[2], ch->exy, ch->exz, ch->eyz, ch->ww1, ch->wsq, ch->rdpz, ch->g1,
                    ch->spec, ch->stage, ch->tauw, ch->taub, ch->les[0], ch->les[1], ch->les[2],
                    ch->les[3], ch->les[4], ch->les[5], ch->les[6], ch->les[7], ch->dyn, ch->smagc,
                    ch->d23, ch->ycs, ch->wpart, ch->coef, ch->d23r, ch->opbuf[0], ch->opbuf[1], ch->rdydf};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (ch->pinned) cudaFreeHost(ch->pinned);
    for (cudaEvent_t e : ch->prof_ev) cudaEventDestroy(e);
    if (ch->tm0) cudaEventDestroy(ch->tm0);
    if (ch->tm1) cudaEventDestroy(ch->tm1);
    if (ch->stream) cudaStreamDestroy(ch->stream);
    for (cudaStream_t q : ch->par)
        if (q) cudaStreamDestroy(q);
    for (cudaEvent_t e : ch->pev)
        if (e) cudaEventDestroy(e);
    if (ch->side) cudaStreamDestroy(ch->side);
    if (ch->cs) cudaStreamDestroy(ch->cs);
    for (cudaEvent_t e : ch->xev)
        if (e) cudaEventDestroy(e);
    if (ch->xfer) cudaFree(ch->xfer);
    if (ch->wtaue) cudaFree(ch->wtaue);
    if (ch->wshift) cudaFree(ch->wshift);
    if (ch->specbuf) cudaFree(ch->specbuf);
    if (ch->iwm) cudaFree(ch->iwm);
    if (ch->sdpart) cudaFree(ch->sdpart);
    if (ch->sfork) cudaEventDestroy(ch->sfork);
    if (ch->sjoin) cudaEventDestroy(ch->sjoin);
    if (ch->sside) cudaStreamDestroy(ch->sside);
    if (ch->sdbeta) cudaFree(ch->sdbeta);
    if (ch->wfork) cudaEventDestroy(ch->wfork);
    if (ch->wjoin) cudaEventDestroy(ch->wjoin);
    if (ch->wside) cudaStreamDestroy(ch->wside);
    if (ch->stats) cudaFree(ch->stats);
    if (ch->hh_in) cudaEventDestroy(ch->hh_in);
    if (ch->hh_out) cudaEventDestroy(ch->hh_out);
    if (ch->ev0) cudaEventDestroy(ch->ev0);
    if (ch->ev1) cudaEventDestroy(ch->ev1);
    delete ch;
}

// INIWAVE and METRICPOISSON (compact3d.f:9182-9263), restated on the host.
void poisson_metrics(c3d_channel *ch, const c3d_grid *gr) {
    const int N1M = gr->n1 - 1, N2M = gr->n2 - 1, N3M = gr->n3 - 1, N2 = gr->n2;
    const double PI = acos(-1.0);
    const double DX1Q = gr->dx1 * gr->dx1, DX3Q = gr->dx3 * gr->dx3;
    // AK1 indexed by |kx| (0..N1M/2); the reference's table is even in kx.
    ch->ak1.assign(N1M, 0.0);
    for (int I = 1; I <= N1M; I++) {
        int II = I;
        if (I > N1M / 2 + 1) II = I - N1M;
        double ani = (II - 1) * 2.0 * PI;
        double cs = cos(ani / N1M);
        double den = 11.0 + cs;
        ch->ak1[I - 1] = 288.0 * DX1Q * (1.0 - cs) / (den * den);
    }
    const int N3MH = N3M / 2 + 1;
    ch->ak3.assign(N3MH, 0.0);
    for (int K = 1; K <= N3MH; K++) {
        double ank = (K - 1) * 2.0 * PI;
        double cs = cos(ank / N3M);
        double den = 11.0 + cs;
        ch->ak3[K - 1] = 288.0 * DX3Q * (1.0 - cs) / (den * den);
    }
    ch->pmjh.assign(N2 + 1, 0.0);
    ch->pcj.assign(N2 + 1, 0.0);
    ch->ppj.assign(N2 + 1, 0.0);
    const double *DY = gr->dy;
    auto H = [&](int J) { return gr->h[J - 1]; };
    for (int JC = 1; JC <= N2M; JC++) {
        int JP = JC + 1;
        double FJUM = (JC == 1) ? 0.0 : 1.0, FJUP = (JC == N2M) ? 0.0 : 1.0;
        ch->pmjh[JC] = FJUM * FJUP * (1.0 / DY[JC] / H(JC)) + (1. - FJUP) * (1.0 / DY[N2M] / H(N2M));
        ch->pcj[JC] = FJUM * FJUP * (-1.0 / DY[JC] / H(JC) - 1.0 / DY[JC] / H(JP)) +
                      (1. - FJUP) * (-1.0 / DY[N2M] / H(N2M)) + (1. - FJUM) * (-1.0 / DY[1] / H(2));
        ch->ppj[JC] = FJUM * FJUP * (1.0 / DY[JC] / H(JP)) + (1. - FJUM) * (1.0 / DY[1] / H(2));
    }
}

// Wall-normal Crank-Nicolson factors of GETUH1-3 / TDMAI for the current DT.
int upload_ycn(c3d_channel *ch, double dt) {
    const Geo &g = ch->g;
    const int m = g.n2 + 1, N2M = g.n2m;
    std::vector<double> t(9 * (size_t)m, 0.0), hm(m), hc(m), hp(m), dym(m), dyc(m), dyp(m);
    std::vector<double> met(10 * (size_t)m);
    CK(cudaMemcpy(met.data(), ch->metric, met.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const double *HP = met.data() + 2 * m, *HC = met.data() + 3 * m, *HM = met.data() + 4 * m;
    const double *DYP = met.data() + 5 * m, *DYC = met.data() + 6 * m, *DYM = met.data() + 7 * m;
    const double RE = g.re;
    for (int c = 0; c < 3; ++c) {
        double *A = t.data() + (c * 3 + 0) * m, *RB = A + m, *GM = RB + m;
        const int js = (c == 1) ? 2 : 1;
        std::vector<double> Av(m), Bv(m), Cv(m);
        for (int J = js; J <= N2M; ++J) {
            double FJUP = (J == N2M) ? 0.0 : 1.0;
            double FJUM = (c == 1) ? ((J == 2) ? 0.0 : 1.0) : ((J == 1) ? 0.0 : 1.0);
            if (c == 1) {
                Cv[J] = FJUP * (-0.5 * DYP[J] * (1. / RE)) * dt;
                Bv[J] = 1.0 + (+0.5 * DYC[J] * (1. / RE)) * dt;
                Av[J] = FJUM * (-0.5 * DYM[J] * (1. / RE)) * dt;
            } else {
                Cv[J] = FJUP * (-0.5 * HP[J] * (1. / RE)) * dt;
                Bv[J] = 1.0 + (0.5 * HC[J] * (1. / RE)) * dt;
                Av[J] = FJUM * (-0.5 * HM[J] * (1. / RE)) * dt;
            }
        }
        double bet = 1.0 / Bv[js];
        RB[js] = bet;
        GM[js] = Cv[js] * bet;
        A[js] = Av[js];
        for (int J = js + 1; J <= N2M; ++J) {
            bet = 1.0 / (Bv[J] - Av[J] * GM[J - 1]);
            RB[J] = bet;
            GM[J] = Cv[J] * bet;
            A[J] = Av[J];
        }
    }
    std::vector<float> t32(t.size());
    for (size_t q = 0; q < t.size(); ++q) t32[q] = (float)t[q];
    CK(cudaMemcpyAsync(ch->ycn, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    CK(cudaMemcpyAsync(ch->ycn32, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    ch->dt_cached = dt;
    return 0;
}

// MARUSIC1's reference plane ZS (compact3d.f:4380-4385): the last J in 1..N2M whose Y(J)
// is no farther from 0.06 than Y(J-1) and Y(J+1); 0 if there is none
int marusic_plane(const double *y, int n2m) {
    const double ZO = 0.06;
    int zs = 0;
    for (int j = 1; j <= n2m; ++j)
        if (std::fabs(y[j] - ZO) <= std::fabs(y[j + 1] - ZO) && std::fabs(y[j] - ZO) <= std::fabs(y[j - 1] - ZO)) zs = j;
    return zs;
}

int check_grid(const c3d_grid *g) {
    if (!g) { set_error("null grid"); return C3D_EINVAL; }
    const int n1m = g->n1 - 1, n2m = g->n2 - 1, n3m = g->n3 - 1;
    if (!n1_ok(n1m) || !fft_len_ok(n1m / 2)) {
        set_error("N1-1 must be even, >= 16, factor as 2^a*3^b and split into 32 lane chunks of 1,2,3,4,6,8 or 12");
        return C3D_EINVAL;
    }
    if (n3m < 16 || n3m % 16 != 0 || !fft_len_ok(n3m)) {
        set_error("N3-1 must be a multiple of 16 that factors as 2^a*3^b");
        return C3D_EINVAL;
    }
    if (n2m < 4 || n2m > 4096) { set_error("N2-1 must be in [4, 4096]"); return C3D_EINVAL; }
    if ((long long)(n1m + 2) * (n2m + 2) * (n3m + 2) >= (1LL << 31)) {   // kernels index points in 32 bits
        set_error("the arrays U(0:N1,0:N2,0:N3) must have fewer than 2^31 points per component");
        return C3D_EINVAL;
    }
    if (!g->y || !g->dy || !g->h || !g->hm || !g->hc || !g->hp || !g->dym || !g->dyc || !g->dyp) {
        set_error("null metric array");
        return C3D_EINVAL;
    }
    if (!(g->re > 0) || !(g->dx1 > 0) || !(g->dx3 > 0) || !(g->vol > 0) || !(g->alx > 0) || !(g->alz > 0)) {
        set_error("RE, DX1, DX3, VOL, ALX, ALZ must be positive");
        return C3D_EINVAL;
    }
    if (g->precision != C3D_FP64 && g->precision != C3D_MIXED && g->precision != C3D_MIXED_IR) {
        set_error("precision must be C3D_FP64, C3D_MIXED or C3D_MIXED_IR");
        return C3D_EINVAL;
    }
    if (g->files < 0 || g->files > 3) {
        set_error("FILES must be 0 (DNS), 1 (SGSDY), 2 (SGSCS) or 3 (SGSSD)");
        return C3D_EINVAL;
    }
    if (g->wmodel < 0 || g->wmodel > 5) {
        set_error("WMODEL must be 0, 1 (WALLMODEL_INSTANT), 2 (WALLMODEL_IWMLES_SMOOTH), 3 (MARUSIC1), "
                  "4 (WALLMODEL_WERNER) or 5 (PIOMELLI)");
        return C3D_EINVAL;
    }
    if (g->wmodel == 2 && g->y[0] != 0.0 && !(g->y[0] > 0 && g->dy[1] + g->dy[2] + g->dy[3] / 2.0 > g->y[0])) {
        set_error("WALLMODEL_IWMLES_ROUGH (WMODEL 2, Y0 = Y(0) != 0) needs 0 < Y0 < DY(1) + DY(2) + DY(3)/2");
        return C3D_EINVAL;
    }
    if (g->wmodel == 3 || g->wmodel == 5) {
        for (int j = 1; j <= n2m; ++j)
            if (!(g->y[j + 1] > g->y[j])) {
                set_error("WMODEL 3 / 5 (MARUSIC1 / PIOMELLI) search the Y faces: Y(1:N2) must increase");
                return C3D_EINVAL;
            }
        if (g->wmodel == 3 && marusic_plane(g->y, n2m) < 1) {
            set_error("WMODEL 3 (MARUSIC1) needs a plane J in 1..N2-1 whose Y(J) is nearest 0.06");
            return C3D_EINVAL;
        }
        // PIOMELLI's bottom height H(1) climbs by about 1e-6 per wall point while it lies
        // below YC(1); bound that climb (it is zero when Y(1) = 0)
        if (g->wmodel == 5 && 0.5 * (g->y[2] + g->y[1]) - g->h[0] > 2e-3) {
            set_error("WMODEL 5 (PIOMELLI) needs H(1) within 2e-3 of YC(1) = (Y(1) + Y(2)) / 2");
            return C3D_EINVAL;
        }
    }
    if (g->wmodel == 4 && n3m > n1m) {
        set_error("WMODEL 4 (WALLMODEL_WERNER) takes the x neighbour with the z index, so it needs N3-1 <= N1-1");
        return C3D_EINVAL;
    }
    if (g->wmodel == 1 && g->y[0] != 0.0 &&
        !(g->y[0] > 0 && g->dy[1] + g->dy[2] + g->dy[3] / 2.0 > g->y[0])) {
        set_error("WALLMODEL_ROUGH (WMODEL 1, Y0 = Y(0) != 0) needs 0 < Y0 < DY(1) + DY(2) + DY(3)/2");
        return C3D_EINVAL;
    }
    return 0;
}

}  // namespace

extern "C" {

int c3d_create(const c3d_grid *gr, c3d_channel **out) {
    if (!out) { set_error("null output handle"); return C3D_EINVAL; }
    *out = nullptr;
    int rc = check_grid(gr);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("no CUDA device");
        return C3D_ENODEV;
    }
    if (c3d::g_device >= 0) CK(cudaSetDevice(c3d::g_device));
    c3d_channel *ch = new c3d_channel();
    memset((void *)ch, 0, offsetof(c3d_channel, fx));
    ch->fx = FftPlan();
    ch->fz = FftPlan();
    cudaGetDevice(&ch->device);
    cudaDeviceGetAttribute(&ch->nsm, cudaDevAttrMultiProcessorCount, ch->device);
    if (ch->nsm <= 0) ch->nsm = 1;
    ch->precision = gr->precision == C3D_MIXED_IR ? C3D_MIXED : gr->precision;
    ch->refine = gr->precision == C3D_MIXED_IR;
    {   // the creation grid, with its metric arrays copied (scratch channels of the autotuner)
        const int n2 = gr->n2;
        ch->grid_arrays.resize(2 * (size_t)(n2 + 1) + 7 * (size_t)n2);
        double *q = ch->grid_arrays.data();
        ch->grid_copy = *gr;
        auto cp = [&](const double *src, size_t n) { std::copy(src, src + n, q); const double *r = q; q += n; return r; };
        ch->grid_copy.y = cp(gr->y, n2 + 1);
        ch->grid_copy.dy = cp(gr->dy, n2 + 1);
        ch->grid_copy.h = cp(gr->h, n2);
        ch->grid_copy.hm = cp(gr->hm, n2);
        ch->grid_copy.hc = cp(gr->hc, n2);
        ch->grid_copy.hp = cp(gr->hp, n2);
        ch->grid_copy.dym = cp(gr->dym, n2);
        ch->grid_copy.dyc = cp(gr->dyc, n2);
        ch->grid_copy.dyp = cp(gr->dyp, n2);
    }
    Geo &g = ch->g;
    g.n1m = gr->n1 - 1;
    g.n2m = gr->n2 - 1;
    g.n3m = gr->n3 - 1;
    g.n2 = gr->n2;
    g.np = g.n1m * g.n3m;
    g.nf = (long long)(g.n2 + 1) * g.np;
    g.n1h = g.n1m / 2 + 1;
    g.dx1 = gr->dx1;
    g.dx3 = gr->dx3;
    g.dx1q = gr->dx1 * gr->dx1;
    g.dx3q = gr->dx3 * gr->dx3;
    g.re = gr->re;
    g.alx = gr->alx;
    g.aly = gr->aly;
    g.alz = gr->alz;
    g.vol = gr->vol;
    const size_t nf = (size_t)g.nf;
    const size_t rs = (ch->precision == C3D_MIXED) ? sizeof(float) : sizeof(double);
    auto fail = [&](int code) {
        free_channel(ch);
        return code;
    };
    if (cudaStreamCreateWithFlags(&ch->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(C3D_ECUDA);
    for (int q = 0; q < 2; ++q)
        if (cudaStreamCreateWithFlags(&ch->par[q], cudaStreamNonBlocking) != cudaSuccess) return fail(C3D_ECUDA);
    for (int q = 0; q < 3; ++q)
        if (cudaEventCreateWithFlags(&ch->pev[q], cudaEventDisableTiming) != cudaSuccess) return fail(C3D_ECUDA);
    if (cudaEventCreate(&ch->ev0) != cudaSuccess || cudaEventCreate(&ch->ev1) != cudaSuccess ||
        cudaEventCreate(&ch->tm0) != cudaSuccess || cudaEventCreate(&ch->tm1) != cudaSuccess)
        return fail(C3D_ECUDA);
    // state: FP64 (FP64 form) or double-float pairs (mixed form), 8 bytes per value either way
    if (cudaMalloc(&ch->u, nf * 8) != cudaSuccess || cudaMalloc(&ch->v, nf * 8) != cudaSuccess ||
        cudaMalloc(&ch->w, nf * 8) != cudaSuccess || cudaMalloc(&ch->p, nf * 8) != cudaSuccess ||
        cudaMalloc(&ch->dp, nf * rs) != cudaSuccess) {
        set_error("cudaMalloc state");
        return fail(C3D_ENOMEM);
    }
    if (dalloc(&ch->scal, SCAL_COUNT) || dalloc(&ch->part, 2 * (size_t)g.n2m * g.n3m + 2 * RB) ||
        dalloc(&ch->metric, 10 * (size_t)(g.n2 + 1)) || dalloc(&ch->ycn, 9 * (size_t)(g.n2 + 1)) ||
        dalloc(&ch->ycn32, 9 * (size_t)(g.n2 + 1)) ||
        dalloc(&ch->pmj, (size_t)(g.n2 + 1)) || dalloc(&ch->pmjdf, (size_t)(g.n2 + 1)) ||
        dalloc(&ch->bulkw, (size_t)(g.n2 + 1)) ||
        dalloc(&ch->diagbuf, nf))
        return fail(C3D_ENOMEM);
    const size_t nmodes = (size_t)g.n1h * g.n3m;
    if (dalloc(&ch->prb, nmodes * g.n2m) || dalloc(&ch->pgam, nmodes * g.n2m)) return fail(C3D_ENOMEM);
    if (ch->precision == C3D_MIXED) {
        if (dalloc(&ch->prbdf, nmodes * g.n2m) || dalloc(&ch->pgamdf, nmodes * g.n2m)) return fail(C3D_ENOMEM);
    }
    void **work[] = {&ch->hh[0][0], &ch->hh[0][1], &ch->hh[0][2], &ch->hh[1][0], &ch->hh[1][1], &ch->hh[1][2],
                     &ch->r[0], &ch->r[1], &ch->r[2], &ch->exy, &ch->exz, &ch->eyz, &ch->ww1, &ch->wsq,
                     &ch->rdpz, &ch->g1};
    for (void **q : work) {
        if (cudaMalloc(q, nf * rs) != cudaSuccess) { set_error("cudaMalloc work"); return fail(C3D_ENOMEM); }
        cudaMemset(*q, 0, nf * rs);
    }
    if (cudaMalloc(&ch->spec, nmodes * g.n2m * 2 * rs) != cudaSuccess) return fail(C3D_ENOMEM);
    {   // MESH02's Y, YC and face / centre tables (the shifted wall models and the particles)
        const size_t ny = (size_t)g.n2 + 1;
        if (dalloc(&ch->wshift, c3d::wall_shift_doubles(g))) return fail(C3D_ENOMEM);
        std::vector<double> yy(2 * ny, 0.0);
        for (size_t j = 0; j < ny; ++j) yy[j] = gr->y[j];
        yy[ny] = gr->y[0];
        for (int j = 1; j <= g.n2m; ++j) yy[ny + j] = 0.5 * (gr->y[j + 1] + gr->y[j]);
        yy[ny + g.n2] = gr->y[g.n2];
        cudaMemcpy(ch->wshift, yy.data(), 2 * ny * 8, cudaMemcpyHostToDevice);
        c3d::launch_wall_shift_init(ch);
        ch->y_increasing = 1;
        for (int j = 1; j <= g.n2m; ++j)
            if (!(gr->y[j + 1] > gr->y[j])) ch->y_increasing = 0;
    }
    // wall stresses (any FILES/WMODEL: c3d_upload_wall may set them) and the LES fields
    ch->files = gr->files;
    ch->wmodel = gr->wmodel;
    ch->wall_cap = 10000;
    if (dalloc(&ch->tauw, 2 * (size_t)g.np) || dalloc(&ch->taub, 2 * (size_t)g.np)) return fail(C3D_ENOMEM);
    cudaMemset(ch->tauw, 0, 2 * (size_t)g.np * 8);
    cudaMemset(ch->taub, 0, 2 * (size_t)g.np * 8);
    if (ch->files != 0) {
        for (int q = 0; q < 8; ++q) {
            if (cudaMalloc(&ch->les[q], nf * rs) != cudaSuccess) { set_error("cudaMalloc LES"); return fail(C3D_ENOMEM); }
            cudaMemset(ch->les[q], 0, nf * rs);
        }
        if ((ch->files == 1 || ch->files == 3) && cudaMalloc(&ch->dyn, 21 * (size_t)g.n2m * g.np * rs) != cudaSuccess)
            return fail(C3D_ENOMEM);
        if (ch->files == 3) {   // SGSSD: per-plane sums of tiles of 32 x 16 points
            ch->sdnt = ((g.n1m + 31) / 32) * (g.n3m / 16);
            if (dalloc(&ch->sdpart, (size_t)g.n2m * ch->sdnt * 10) || dalloc(&ch->sdbeta, (size_t)g.n2 + 1))
                return fail(C3D_ENOMEM);
            cudaMemset(ch->sdbeta, 0, ((size_t)g.n2 + 1) * 8);
            if (cudaStreamCreateWithFlags(&ch->sside, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&ch->sfork, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&ch->sjoin, cudaEventDisableTiming) != cudaSuccess)
                return fail(C3D_ECUDA);
        }
        const int nbw = (g.np + 127) / 128;   // blocks of k_wall (TPB = 128 threads)
        if (dalloc(&ch->smagc, (size_t)g.n2 + 1) || dalloc(&ch->d23, (size_t)g.n2 + 1) ||
            dalloc(&ch->ycs, (size_t)g.n2 + 1) || dalloc(&ch->wpart, 2 * (size_t)nbw))
            return fail(C3D_ENOMEM);
        if (gr->wmodel == 4 && dalloc(&ch->wtaue, 4 * (size_t)g.np)) return fail(C3D_ENOMEM);
        if (gr->wmodel != 0 &&
            (cudaStreamCreateWithFlags(&ch->wside, cudaStreamNonBlocking) != cudaSuccess ||
             cudaEventCreateWithFlags(&ch->wfork, cudaEventDisableTiming) != cudaSuccess ||
             cudaEventCreateWithFlags(&ch->wjoin, cudaEventDisableTiming) != cudaSuccess))
            return fail(C3D_ECUDA);
        if (gr->wmodel == 2) {
            if (dalloc(&ch->iwm, c3d::iwm_doubles(g))) return fail(C3D_ENOMEM);
            ch->iwm_dzp = gr->dy[1] + gr->dy[2] + gr->dy[3] / 2.0;
            ch->iwm_y0 = gr->y[0];
        }
        if (gr->wmodel == 1 && gr->y[0] != 0.0) {   // WALLMODEL_ROUGH's KAPA / log(DELTAP / Y0)
            ch->wrough = 1;
            ch->wklog = 0.41 / std::log((gr->dy[1] + gr->dy[2] + gr->dy[3] / 2.0) / gr->y[0]);
        }
        if (gr->wmodel == 3 || gr->wmodel == 5) {
            ch->wzs = marusic_plane(gr->y, g.n2m);
            ch->wtan16 = std::tan(16.0 * std::acos(-1.0) / 180);
        }
        if (cudaMalloc(&ch->coef, ((size_t)g.n2 + 1) * rs) != cudaSuccess ||
            cudaMalloc(&ch->d23r, ((size_t)g.n2 + 1) * rs) != cudaSuccess)
            return fail(C3D_ENOMEM);
        cudaMemset(ch->smagc, 0, ((size_t)g.n2 + 1) * 8);
        // DXYZ^(2/3) and the Van Driest height per plane (SGSCS/SGSDY, compact3d.f:1283, 1469)
        std::vector<double> d23(g.n2 + 1, 0.0), ycs(g.n2 + 1, 0.0);
        for (int j = 1; j <= g.n2m; ++j) {
            const double dxyz = 1.0 / gr->dx1 * gr->dy[j] / gr->dx3;
            d23[j] = pow(dxyz, 2. / 3.);
            ycs[j] = gr->y[j] + gr->dy[j] * 0.5;
        }
        cudaMemcpy(ch->d23, d23.data(), d23.size() * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(ch->ycs, ycs.data(), ycs.size() * 8, cudaMemcpyHostToDevice);
        if (ch->precision == C3D_MIXED) {
            std::vector<float> f(d23.begin(), d23.end());
            cudaMemcpy(ch->d23r, f.data(), f.size() * 4, cudaMemcpyHostToDevice);
        } else {
            cudaMemcpy(ch->d23r, d23.data(), d23.size() * 8, cudaMemcpyHostToDevice);
        }
    }
    ch->stage_elems = (size_t)(gr->n1 + 1) * (gr->n2 + 1) * (gr->n3 + 1);
    if (dalloc(&ch->stage, ch->stage_elems)) return fail(C3D_ENOMEM);
    cudaMemset(ch->u, 0, nf * 8);
    cudaMemset(ch->v, 0, nf * 8);
    cudaMemset(ch->w, 0, nf * 8);
    cudaMemset(ch->p, 0, nf * 8);
    cudaMemset(ch->dp, 0, nf * rs);
    cudaMemset(ch->scal, 0, SCAL_COUNT * 8);
    // metrics indexed by Fortran J: dy(0..N2), h/hp/hc/hm/dyp/dyc/dym(1..N2) (entry 0 = 0)
    const int m = g.n2 + 1;
    std::vector<double> met(10 * (size_t)m, 0.0);
    for (int j = 0; j <= g.n2; ++j) met[j] = gr->dy[j];
    const double *src[7] = {gr->h, gr->hp, gr->hc, gr->hm, gr->dyp, gr->dyc, gr->dym};
    for (int q = 0; q < 7; ++q)
        for (int j = 1; j <= g.n2; ++j) met[(q + 1) * (size_t)m + j] = src[q][j - 1];
    // HP+HM-HC and DYP+DYM-DYC: zero up to rounding, they let the mixed form write the
    // wall-normal viscous stencil without cancellation
    for (int j = 1; j <= g.n2; ++j) {
        met[8 * (size_t)m + j] = (gr->hp[j - 1] + gr->hm[j - 1]) - gr->hc[j - 1];
        met[9 * (size_t)m + j] = (gr->dyp[j - 1] + gr->dym[j - 1]) - gr->dyc[j - 1];
    }
    if (cudaMemcpy(ch->metric, met.data(), met.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) return fail(C3D_ECUDA);
    g.dy = ch->metric;
    g.h = ch->metric + m;
    g.hp = ch->metric + 2 * m;
    g.hc = ch->metric + 3 * m;
    g.hm = ch->metric + 4 * m;
    g.dyp = ch->metric + 5 * m;
    g.dyc = ch->metric + 6 * m;
    g.dym = ch->metric + 7 * m;
    g.hz = ch->metric + 8 * m;
    g.dyz = ch->metric + 9 * m;
    {
        // working-precision copies: hp,hc,hm,hz,dyp,dyc,dym,dyz,h,1/h,dy/2,1/dy,dy
        std::vector<double> mr((size_t)NMETR * m, 0.0);
        const int order[9] = {2, 3, 4, 8, 5, 6, 7, 9, 1};   // rows of `met`
        for (int q = 0; q < 9; ++q)
            for (int j = 0; j < m; ++j) mr[(size_t)q * m + j] = met[(size_t)order[q] * m + j];
        for (int j = 0; j < m; ++j) {
            const double hj = met[(size_t)1 * m + j], dyj = met[j];
            mr[(size_t)9 * m + j] = hj != 0.0 ? 1.0 / hj : 0.0;
            mr[(size_t)10 * m + j] = dyj / 2.0;
            mr[(size_t)11 * m + j] = dyj != 0.0 ? 1.0 / dyj : 0.0;
            mr[(size_t)12 * m + j] = dyj;
        }
        const size_t es = rs;
        if (cudaMalloc(&ch->metr, mr.size() * es) != cudaSuccess) return fail(C3D_ENOMEM);
        if (ch->precision == C3D_MIXED) {
            std::vector<float> f(mr.size());
            for (size_t q = 0; q < mr.size(); ++q) f[q] = (float)mr[q];
            cudaMemcpy(ch->metr, f.data(), f.size() * 4, cudaMemcpyHostToDevice);
        } else {
            cudaMemcpy(ch->metr, mr.data(), mr.size() * 8, cudaMemcpyHostToDevice);
        }
    }
    // Poisson metrics and factor tables
    poisson_metrics(ch, gr);
    if (cudaMemcpy(ch->pmj, ch->pmjh.data(), (size_t)m * 8, cudaMemcpyHostToDevice) != cudaSuccess) return fail(C3D_ECUDA);
    {
        std::vector<float2> pdf(m);
        for (int j = 0; j < m; ++j) {
            float h = (float)ch->pmjh[j];
            pdf[j] = make_float2(h, (float)(ch->pmjh[j] - (double)h));
        }
        if (cudaMemcpy(ch->pmjdf, pdf.data(), (size_t)m * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(C3D_ECUDA);
        // weights of the bulk-flow sums (UPCALC): DY(J)/DX3/DX1, FP64 on the host
        for (int j = 0; j < m; ++j) {
            const double wj = gr->dy[j] / gr->dx3 / gr->dx1;
            const float h = (float)wj;
            pdf[j] = make_float2(h, (float)(wj - (double)h));
        }
        if (cudaMemcpy(ch->bulkw, pdf.data(), (size_t)m * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(C3D_ECUDA);
        if (ch->refine) {   // 1/DY(J) for the refinement's residual
            std::vector<dfl> r(m);
            for (int j = 1; j < m - 1; ++j) r[j] = dfl::from(1.0 / gr->dy[j]);
            if (cudaMalloc(&ch->rdydf, (size_t)m * sizeof(dfl)) != cudaSuccess) return fail(C3D_ENOMEM);
            if (cudaMemcpy(ch->rdydf, r.data(), (size_t)m * sizeof(dfl), cudaMemcpyHostToDevice) != cudaSuccess)
                return fail(C3D_ECUDA);
        }
    }
    rc = launch_poisson_tables(ch);
    if (rc) return fail(rc);
    // FFT plans and twiddles: [x: N1M/2][z: N3M][x post-processing: N1M/2+1]
    ch->tune = Tune{{16, 16, 16, 16, 16}, 4, 8, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    ch->fx = make_plan(g.n1m / 2, 0);
    ch->fz = make_plan(g.n3m, 0);
    if (ch->fx.nst < 0 || ch->fz.nst < 0) { set_error("FFT plan index arithmetic"); return fail(C3D_EINVAL); }
    const int nx = g.n1m / 2, nz = g.n3m, np = g.n1m / 2 + 1;
    std::vector<double2> tw(nx + nz + np);
    std::vector<float2> tw32(nx + nz + np);
    for (int q = 0; q < nx; ++q) tw[q] = make_double2(cos(2 * M_PI * q / nx), -sin(2 * M_PI * q / nx));
    for (int q = 0; q < nz; ++q) tw[nx + q] = make_double2(cos(2 * M_PI * q / nz), -sin(2 * M_PI * q / nz));
    for (int q = 0; q < np; ++q)
        tw[nx + nz + q] = make_double2(cos(2 * M_PI * q / g.n1m), -sin(2 * M_PI * q / g.n1m));
    for (size_t q = 0; q < tw.size(); ++q) tw32[q] = make_float2((float)tw[q].x, (float)tw[q].y);
    if (dalloc(&ch->tw64, tw.size()) || dalloc(&ch->tw32, tw32.size())) return fail(C3D_ENOMEM);
    cudaMemcpy(ch->tw64, tw.data(), tw.size() * sizeof(double2), cudaMemcpyHostToDevice);
    cudaMemcpy(ch->tw32, tw32.data(), tw32.size() * sizeof(float2), cudaMemcpyHostToDevice);
    ch->fx.tw64 = ch->tw64;
    ch->fx.tw32 = ch->tw32;
    ch->fz.tw64 = ch->tw64 + nx;
    ch->fz.tw32 = ch->tw32 + nx;
    ch->dt_cached = -1.0;
    ch->cur = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error(std::string("create: ") + cudaGetErrorString(e));
        return fail(C3D_ECUDA);
    }
    *out = ch;
    return 0;
}

int c3d_destroy(c3d_channel *ch) {
    if (!ch) return C3D_EINVAL;
    cudaSetDevice(ch->device);
    cudaStreamSynchronize(ch->stream);
    free_channel(ch);
    return 0;
}

// True when [h, h + bytes) lies in one host allocation registered with c3d_host_register
// (page-locked): such arrays move by DMA at the link's rate.
static bool host_pinned(const void *h, size_t bytes) {
    if (!h || !bytes) return false;
    cudaPointerAttributes a0, a1;
    const char *last = (const char *)h + bytes - 1;
    if (cudaPointerGetAttributes(&a0, h) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return false;
    return (const char *)a1.devicePointer - (const char *)a0.devicePointer == (long long)(bytes - 1);
}

// Device staging area for the DMA transfers of pinned arrays, one slot per Fortran field:
// U(3 components), P, HH(3), SGSVIS; allocated on first use.
struct Xfer {
    size_t n3, np;
    double *base;
    double *u(int c) const { return base + c * n3; }
    double *p() const { return base + 3 * n3; }
    double *hh(int c) const { return base + 3 * n3 + np + c * n3; }
    double *sgs() const { return base + 6 * n3 + np; }
};
static int xfer_area(c3d_channel *ch, Xfer *x) {
    const Geo &g = ch->g;
    x->n3 = ch->stage_elems;
    x->np = (size_t)(g.n1m + 1) * g.n2 * (g.n3m + 1);
    if (!ch->xfer) {
        if (cudaMalloc(&ch->xfer, (7 * x->n3 + x->np) * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            ch->xfer = nullptr;
            set_error("cudaMalloc of the transfer staging area");
            return C3D_ENOMEM;
        }
    }
    x->base = ch->xfer;
    return 0;
}
// Streams and events of the pipelined DMA transfers (created on first use).
static int xfer_streams(c3d_channel *ch) {
    if (!ch->side) {
        CK(cudaStreamCreateWithFlags(&ch->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ch->hh_in, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ch->hh_out, cudaEventDisableTiming));
    }
    if (!ch->cs) {
        CK(cudaStreamCreateWithFlags(&ch->cs, cudaStreamNonBlocking));
        for (cudaEvent_t &e : ch->xev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    return 0;
}
// Host -> device of one field: DMA into its slot on the copy stream, then the unpacking
// kernel on stream st once the copy is done (event ev), so the next field's copy overlaps
// this field's unpacking.
static int up_field(c3d_channel *ch, cudaStream_t st, cudaEvent_t ev, double *slot, const double *h, size_t n,
                    int what, int comp) {
    CK(cudaMemcpyAsync(slot, h, n * sizeof(double), cudaMemcpyHostToDevice, ch->cs));
    CK(cudaEventRecord(ev, ch->cs));
    CK(cudaStreamWaitEvent(st, ev, 0));
    cudaStream_t keep = ch->stream;
    ch->stream = st;
    launch_repack(ch, 0, what, comp, slot);
    ch->stream = keep;
    return 0;
}
// Device -> host of one field: the packing kernel into its slot on stream st, then the DMA
// on the copy stream once it is done (event ev).
static int dn_field(c3d_channel *ch, cudaStream_t st, cudaEvent_t ev, double *slot, double *h, size_t n, int what,
                    int comp) {
    cudaStream_t keep = ch->stream;
    ch->stream = st;
    launch_repack(ch, 1, what, comp, slot);
    ch->stream = keep;
    CK(cudaEventRecord(ev, st));
    CK(cudaStreamWaitEvent(ch->cs, ev, 0));
    CK(cudaMemcpyAsync(h, slot, n * sizeof(double), cudaMemcpyDeviceToHost, ch->cs));
    return 0;
}

static int h2d(c3d_channel *ch, const double *src, size_t n) {
    CK(cudaMemcpyAsync(ch->stage, src, n * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    return 0;
}
static int d2h(c3d_channel *ch, double *dst, size_t n) {
    CK(cudaMemcpyAsync(dst, ch->stage, n * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_upload(c3d_channel *ch, const double *u, const double *p, const double *hh, const double *sgsvis) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    if (sgsvis && ch->files == 0) { set_error("SGSVIS is not used when FILES=0; pass NULL"); return C3D_EINVAL; }
    // With an SGS model, GETUP zeroes SGSVIS and recomputes it every step
    // (compact3d.f:912-933), so an uploaded SGSVIS has no effect and is not copied.
    cudaSetDevice(ch->device);
    const size_t n3 = ch->stage_elems;   // one component of U / HH
    const Geo &g = ch->g;
    const size_t np_ = (size_t)(g.n1m + 1) * g.n2 * (g.n3m + 1);
    const bool pinned = (!u || host_pinned(u, 3 * n3 * 8)) && (!p || host_pinned(p, np_ * 8)) &&
                        (!hh || host_pinned(hh, 3 * n3 * 8));
    int rc = 0;
    Xfer x;
    if (pinned && (rc = xfer_area(ch, &x)) == 0 && (rc = xfer_streams(ch)) == 0) {
        // every field by DMA on the copy stream, each unpacked as soon as it has arrived
        CK(cudaEventRecord(ch->xev[15], ch->stream));   // after earlier work on the slots
        CK(cudaStreamWaitEvent(ch->cs, ch->xev[15], 0));
        for (int c = 0; c < 3 && u; ++c)
            if ((rc = up_field(ch, ch->stream, ch->xev[c], x.u(c), u + c * n3, n3, 0, c))) return rc;
        if (p && (rc = up_field(ch, ch->stream, ch->xev[3], x.p(), p, np_, 1, 0))) return rc;
        for (int c = 0; c < 3 && hh; ++c)
            if ((rc = up_field(ch, ch->stream, ch->xev[4 + c], x.hh(c), hh + c * n3, n3, 2, c))) return rc;
    } else if (rc && rc != C3D_ENOMEM) {
        return rc;
    } else {   // pageable arrays: one field at a time through the one-field staging buffer
        for (int c = 0; c < 3 && u; ++c) {
            if ((rc = h2d(ch, u + c * n3, n3))) return rc;
            launch_repack(ch, 0, 0, c);
        }
        if (p) {
            if ((rc = h2d(ch, p, np_))) return rc;
            launch_repack(ch, 0, 1, 0);
        }
        for (int c = 0; c < 3 && hh; ++c) {
            if ((rc = h2d(ch, hh + c * n3, n3))) return rc;
            launch_repack(ch, 0, 2, c);
        }
    }
    CK(cudaStreamSynchronize(ch->stream));
    CK(cudaGetLastError());
    ch->have_state = 1;
    return 0;
}

int c3d_download(c3d_channel *ch, double *u, double *p, double *hh, double *sgsvis) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    if (sgsvis && ch->files == 0) { set_error("SGSVIS exists only with an SGS model (FILES != 0)"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    const size_t n3 = ch->stage_elems;
    const Geo &g = ch->g;
    const size_t np_ = (size_t)(g.n1m + 1) * g.n2 * (g.n3m + 1);
    const bool pinned = (!u || host_pinned(u, 3 * n3 * 8)) && (!p || host_pinned(p, np_ * 8)) &&
                        (!hh || host_pinned(hh, 3 * n3 * 8)) && (!sgsvis || host_pinned(sgsvis, n3 * 8));
    int rc = 0;
    Xfer x;
    if (pinned && (rc = xfer_area(ch, &x)) == 0 && (rc = xfer_streams(ch)) == 0) {
        // every field packed on the channel's stream and sent by DMA as soon as it is packed
        for (int c = 0; c < 3 && u; ++c)
            if ((rc = dn_field(ch, ch->stream, ch->xev[c], x.u(c), u + c * n3, n3, 0, c))) return rc;
        if (p && (rc = dn_field(ch, ch->stream, ch->xev[3], x.p(), p, np_, 1, 0))) return rc;
        for (int c = 0; c < 3 && hh; ++c)
            if ((rc = dn_field(ch, ch->stream, ch->xev[4 + c], x.hh(c), hh + c * n3, n3, 2, c))) return rc;
        if (sgsvis && (rc = dn_field(ch, ch->stream, ch->xev[7], x.sgs(), sgsvis, n3, 3, 0))) return rc;
        CK(cudaStreamSynchronize(ch->cs));
    } else if (rc && rc != C3D_ENOMEM) {
        return rc;
    } else {
        for (int c = 0; c < 3 && u; ++c) {
            launch_repack(ch, 1, 0, c);
            if ((rc = d2h(ch, u + c * n3, n3))) return rc;
        }
        if (p) {
            launch_repack(ch, 1, 1, 0);
            if ((rc = d2h(ch, p, np_))) return rc;
        }
        for (int c = 0; c < 3 && hh; ++c) {
            launch_repack(ch, 1, 2, c);
            if ((rc = d2h(ch, hh + c * n3, n3))) return rc;
        }
        if (sgsvis) {
            launch_repack(ch, 1, 3, 0);
            if ((rc = d2h(ch, sgsvis, n3))) return rc;
        }
    }
    CK(cudaStreamSynchronize(ch->stream));
    CK(cudaGetLastError());
    return 0;
}

int c3d_host_register(void *ptr, size_t bytes) {
    if (!ptr || !bytes) { set_error("null pointer or zero size"); return C3D_EINVAL; }
    CK(cudaHostRegister(ptr, bytes, cudaHostRegisterMapped));
    return 0;
}

int c3d_host_unregister(void *ptr) {
    if (!ptr) { set_error("null pointer"); return C3D_EINVAL; }
    CK(cudaHostUnregister(ptr));
    return 0;
}

int c3d_host_alloc(size_t bytes, void **ptr) {
    if (!ptr || !bytes) { set_error("null pointer or zero size"); return C3D_EINVAL; }
    *ptr = nullptr;
    if (cudaHostAlloc(ptr, bytes, cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        set_error("cudaHostAlloc failed");
        return C3D_ENOMEM;
    }
    return 0;
}

int c3d_host_free(void *ptr) {
    if (!ptr) { set_error("null pointer"); return C3D_EINVAL; }
    CK(cudaFreeHost(ptr));
    return 0;
}

// TAUW/TAUB(0:M1,0:M3,2): interior I = 1..N1M, K = 1..N3M of both walls move.
static int wall_copy(c3d_channel *ch, double *host, double *dev, bool up) {
    const Geo &g = ch->g;
    const long long N1 = g.n1m + 1, N3 = g.n3m + 1;
    std::vector<double> plane(2 * (size_t)g.np);
    if (up) {
        for (int w = 0; w < 2; ++w)
            for (int k = 0; k < g.n3m; ++k)
                for (int i = 0; i < g.n1m; ++i)
                    plane[(size_t)w * g.np + (size_t)k * g.n1m + i] = host[(i + 1) + (N1 + 1) * ((k + 1) + (N3 + 1) * w)];
        CK(cudaMemcpy(dev, plane.data(), plane.size() * 8, cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemcpy(plane.data(), dev, plane.size() * 8, cudaMemcpyDeviceToHost));
        for (int w = 0; w < 2; ++w)
            for (int k = 0; k < g.n3m; ++k)
                for (int i = 0; i < g.n1m; ++i)
                    host[(i + 1) + (N1 + 1) * ((k + 1) + (N3 + 1) * w)] = plane[(size_t)w * g.np + (size_t)k * g.n1m + i];
    }
    return 0;
}

int c3d_upload_wall(c3d_channel *ch, const double *tauw, const double *taub) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    CK(cudaStreamSynchronize(ch->stream));
    int rc = 0;
    if (tauw && (rc = wall_copy(ch, const_cast<double *>(tauw), ch->tauw, true))) return rc;
    if (taub && (rc = wall_copy(ch, const_cast<double *>(taub), ch->taub, true))) return rc;
    return 0;
}

int c3d_download_wall(c3d_channel *ch, double *tauw, double *taub) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    CK(cudaStreamSynchronize(ch->stream));
    int rc = 0;
    if (tauw && (rc = wall_copy(ch, tauw, ch->tauw, false))) return rc;
    if (taub && (rc = wall_copy(ch, taub, ch->taub, false))) return rc;
    return 0;
}

int c3d_set_wsm(c3d_channel *ch, const double *wsm) {
    if (!ch || !wsm) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    CK(cudaMemcpyAsync(ch->scal + SCAL_WSMC, wsm, 3 * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_get_wsm(c3d_channel *ch, double *wsm) {
    if (!ch || !wsm) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    CK(cudaMemcpyAsync(wsm, ch->scal + SCAL_WSMC, 3 * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_set_wall_iter_cap(c3d_channel *ch, int cap) {
    if (!ch || cap < 1) { set_error("null channel or cap < 1"); return C3D_EINVAL; }
    ch->wall_cap = cap;
    return 0;
}

// After a completed step: the wall model's non-convergence flag (WMODEL = 1 with an SGS model).
static int check_wall_flag(c3d_channel *ch, const double *scal_host) {
    if (scal_host[SCAL_PIPEERR] != 0.0) {
        set_error("a shared-memory bulk-copy stage did not complete within its wait limit");
        return C3D_ECUDA;
    }
    if (ch->files != 0 && ch->wmodel == 1 && !ch->wrough && scal_host[SCAL_WALLERR] != 0.0) {
        set_error("wall model: the Newton iteration for u_tau did not converge within the iteration cap");
        return C3D_ENOTCONV;
    }
    return 0;
}

static int step_common(c3d_channel *ch, double dt, double *presg, double *presg3, bool sync) {
    if (!(dt > 0) || !isfinite(dt)) { set_error("dt must be positive and finite"); return C3D_EINVAL; }
    if (dt != ch->dt_cached) {
        int rc = upload_ycn(ch, dt);
        if (rc) return rc;
    }
    double pg[2] = {presg ? *presg : 0.0, presg3 ? *presg3 : 0.0};
    if (presg && presg3)
        CK(cudaMemcpyAsync(ch->scal + SCAL_PRESG, pg, 2 * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    CK(cudaEventRecord(ch->ev0, ch->stream));
    prof_begin(ch);
    int nl = 0;
    int rc = launch_step(ch, dt, &nl);
    if (rc) return rc;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ch->ev1, ch->stream));
    ch->last_launches = nl;
    if (ch->prof_on) {
        rc = prof_collect(ch);
        if (rc) return rc;
    }
    if (sync) {
        double sc[SCAL_COUNT];
        CK(cudaMemcpyAsync(sc, ch->scal, sizeof(sc), cudaMemcpyDeviceToHost, ch->stream));
        CK(cudaStreamSynchronize(ch->stream));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ch->ev0, ch->ev1);
        ch->last_ms = ms;
        if (presg) *presg = sc[SCAL_PRESG];
        if (presg3) *presg3 = sc[SCAL_PRESG3];
        return check_wall_flag(ch, sc);
    }
    return 0;
}

int c3d_step(c3d_channel *ch, int ntime, double dt, double *presg, double *presg3) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    ch->ntime = ntime;
    if (!presg || !presg3) { set_error("null PRESG/PRESG3"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_step"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    return step_common(ch, dt, presg, presg3, true);
}

int c3d_step_async(c3d_channel *ch, int ntime, double dt) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    ch->ntime = ntime;
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_step_async"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    return step_common(ch, dt, nullptr, nullptr, false);
}

int c3d_set_cflmax(c3d_channel *ch, double cflmax) {
    if (!ch || !(cflmax > 0) || !isfinite(cflmax)) { set_error("CFLMAX must be positive and finite"); return C3D_EINVAL; }
    ch->cflmax = cflmax;
    return 0;
}

int c3d_set_presg(c3d_channel *ch, double presg, double presg3) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    double pg[2] = {presg, presg3};
    CK(cudaMemcpyAsync(ch->scal + SCAL_PRESG, pg, sizeof(pg), cudaMemcpyHostToDevice, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_get_presg(c3d_channel *ch, double *presg, double *presg3) {
    if (!ch || !presg || !presg3) { set_error("null argument"); return C3D_EINVAL; }
    double pg[2];
    CK(cudaMemcpyAsync(pg, ch->scal + SCAL_PRESG, sizeof(pg), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    *presg = pg[0];
    *presg3 = pg[1];
    return 0;
}

int c3d_timer_start(c3d_channel *ch) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    CK(cudaEventRecord(ch->tm0, ch->stream));
    return 0;
}

int c3d_timer_stop(c3d_channel *ch, double *ms) {
    if (!ch || !ms) { set_error("null argument"); return C3D_EINVAL; }
    CK(cudaEventRecord(ch->tm1, ch->stream));
    CK(cudaEventSynchronize(ch->tm1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ch->tm0, ch->tm1));
    *ms = f;
    return 0;
}

int c3d_profile(c3d_channel *ch, int enable) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    ch->prof_on = enable ? 1 : 0;
    ch->prof_name.clear();
    ch->prof_ms.clear();
    ch->prof_cnt.clear();
    ch->prof_bytes.clear();
    ch->prof_n = 0;
    return 0;
}

int c3d_profile_count(c3d_channel *ch) {
    if (!ch) return C3D_EINVAL;
    return (int)ch->prof_name.size();
}

int c3d_profile_get(c3d_channel *ch, int idx, const char **name, double *ms, int *launches,
                    double *bytes_per_launch) {
    if (!ch || idx < 0 || idx >= (int)ch->prof_name.size()) { set_error("bad profile index"); return C3D_EINVAL; }
    if (name) *name = ch->prof_name[idx].c_str();
    if (ms) *ms = ch->prof_ms[idx];
    if (launches) *launches = ch->prof_cnt[idx];
    if (bytes_per_launch) *bytes_per_launch = ch->prof_bytes[idx];
    return 0;
}

int c3d_project(c3d_channel *ch) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_project"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    int nl = 0;
    prof_begin(ch);
    int rc = launch_project(ch, &nl);
    if (!rc) rc = prof_collect(ch);
    if (rc) return rc;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_diagnose(c3d_channel *ch, c3d_diag *out) {
    if (!ch || !out) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    int nl = 0;
    prof_begin(ch);
    int rc = launch_diag(ch, &nl);
    if (!rc) rc = prof_collect(ch);
    if (rc) return rc;
    double s[SCAL_COUNT];
    CK(cudaMemcpyAsync(s, ch->scal, sizeof(s), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    out->divmax = s[SCAL_DIVMAX];
    out->cflm = s[SCAL_CFL];
    out->flow1 = s[SCAL_FLOW1];
    out->flow3 = s[SCAL_FLOW3];
    out->wsm[0] = s[SCAL_WSM];
    out->wsm[1] = s[SCAL_WSM + 1];
    out->wsm[2] = s[SCAL_WSM + 2];
    out->nonfinite = s[SCAL_NONFIN] != 0.0;
    return out->nonfinite ? C3D_ENONFINITE : 0;
}

// c3d_getup with every array mapped: the transfers of HH overlap the step.  The main
// stream unpacks U and P and runs the step; a side stream unpacks HH_old, which the step
// waits for before xB (its first reader), and packs the new HH back once xB (its last
// writer) is done, while the step continues; U, P and SGSVIS are packed after the step.
// c3d_getup with every array pinned: the transfers of HH overlap the step.  The host link
// is the bottleneck (2 x 2.15 GB per step on channel384), so the DMA copies run back to
// back: U and P first on the channel's stream (unpacked, then the step starts), HH_old
// next on a side stream (unpacked there; the step waits for it before xB, its first
// reader), and the new HH back to the host on the side stream as soon as xB (its last
// writer) is done, while the step continues; U, P and SGSVIS follow after the step.
static int getup_overlapped(c3d_channel *ch, const double *u, double *uo, const double *p, double *po,
                            const double *hh, double *hho, double *sgs, double dt, double *presg, double *presg3) {
    int rc;
    Xfer x;
    if ((rc = xfer_area(ch, &x)) || (rc = xfer_streams(ch))) return rc;
    const size_t n3 = x.n3;
    CK(cudaEventRecord(ch->xev[15], ch->stream));   // after earlier work on the slots
    CK(cudaStreamWaitEvent(ch->cs, ch->xev[15], 0));
    for (int c = 0; c < 3; ++c)
        if ((rc = up_field(ch, ch->stream, ch->xev[c], x.u(c), u + c * n3, n3, 0, c))) return rc;
    if ((rc = up_field(ch, ch->stream, ch->xev[3], x.p(), p, x.np, 1, 0))) return rc;
    for (int c = 0; c < 3; ++c)   // HH_old to the buffer the step reads as HH_old (the current one)
        if ((rc = up_field(ch, ch->side, ch->xev[4 + c], x.hh(c), hh + c * n3, n3, 2, c))) return rc;
    CK(cudaEventRecord(ch->hh_in, ch->side));
    ch->have_state = 1;
    ch->hh_hooks = true;
    rc = step_common(ch, dt, presg, presg3, false);
    ch->hh_hooks = false;
    if (rc) return rc;
    CK(cudaStreamWaitEvent(ch->side, ch->hh_out, 0));   // recorded by the step after xB
    for (int c = 0; c < 3; ++c)
        if ((rc = dn_field(ch, ch->side, ch->xev[8 + c], x.hh(c), hho + c * n3, n3, 2, c))) return rc;
    for (int c = 0; c < 3; ++c)
        if ((rc = dn_field(ch, ch->stream, ch->xev[11 + c], x.u(c), uo + c * n3, n3, 0, c))) return rc;
    if ((rc = dn_field(ch, ch->stream, ch->xev[14], x.p(), po, x.np, 1, 0))) return rc;
    if (sgs && (rc = dn_field(ch, ch->stream, ch->xev[7], x.sgs(), sgs, n3, 3, 0))) return rc;
    double sc[SCAL_COUNT];
    CK(cudaMemcpyAsync(sc, ch->scal, sizeof(sc), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    CK(cudaStreamSynchronize(ch->side));
    CK(cudaStreamSynchronize(ch->cs));
    CK(cudaGetLastError());
    float ms_ = 0.f;
    cudaEventElapsedTime(&ms_, ch->ev0, ch->ev1);
    ch->last_ms = ms_;
    *presg = sc[SCAL_PRESG];
    *presg3 = sc[SCAL_PRESG3];
    return check_wall_flag(ch, sc);
}

int c3d_getup(c3d_channel *ch, double *u, double *p, double *hh, double *sgsvis, int ntime, double dt,
              double *presg, double *presg3) {
    if (!ch || !u || !p || !hh) { set_error("null argument"); return C3D_EINVAL; }
    if (!presg || !presg3) { set_error("null PRESG/PRESG3"); return C3D_EINVAL; }
    {
        cudaSetDevice(ch->device);
        const size_t n3 = ch->stage_elems;
        const Geo &g = ch->g;
        const size_t np_ = (size_t)(g.n1m + 1) * g.n2 * (g.n3m + 1);
        double *sg = ch->files != 0 ? sgsvis : nullptr;
        if (host_pinned(u, 3 * n3 * 8) && host_pinned(p, np_ * 8) && host_pinned(hh, 3 * n3 * 8) &&
            (!sg || host_pinned(sg, n3 * 8)) && !ch->prof_on) {
            ch->ntime = ntime;
            if (!(dt > 0) || !isfinite(dt)) { set_error("dt must be positive and finite"); return C3D_EINVAL; }
            return getup_overlapped(ch, u, u, p, p, hh, hh, sg, dt, presg, presg3);
        }
    }
    int rc = c3d_upload(ch, u, p, hh, sgsvis);
    if (rc) return rc;
    rc = c3d_step(ch, ntime, dt, presg, presg3);
    if (rc) return rc;
    return c3d_download(ch, u, p, hh, ch->files != 0 ? sgsvis : nullptr);
}

// ---- checkpoint -----------------------------------------------------------------
}  // extern "C"

namespace {
// One Fortran sequential unformatted record: length, payload, length (4-byte markers).
int rec_write(FILE *f, const void *p, size_t bytes) {
    if (bytes > 0x7fffffffu) { set_error("checkpoint record longer than 2^31-1 bytes"); return C3D_EINVAL; }
    const int32_t m = (int32_t)bytes;
    if (fwrite(&m, 4, 1, f) != 1 || (bytes && fwrite(p, 1, bytes, f) != bytes) || fwrite(&m, 4, 1, f) != 1) {
        set_error("checkpoint write failed");
        return C3D_EIO;
    }
    return 0;
}
int rec_read(FILE *f, void *p, size_t bytes) {
    int32_t m0 = 0, m1 = 0;
    if (fread(&m0, 4, 1, f) != 1 || (size_t)(uint32_t)m0 != bytes) {
        set_error("checkpoint record length does not match the channel's grid");
        return C3D_EIO;
    }
    if ((bytes && fread(p, 1, bytes, f) != bytes) || fread(&m1, 4, 1, f) != 1 || m1 != m0) {
        set_error("checkpoint read failed (truncated file or bad record marker)");
        return C3D_EIO;
    }
    return 0;
}
// Walks the records of an open checkpoint without reading their contents: each record
// must have the expected length and matching markers before and after it.  The file is
// left at its start.
int rec_scan(FILE *f, const std::vector<size_t> &sizes) {
    int rc = 0;
    for (size_t q = 0; q < sizes.size() && !rc; ++q) {
        int32_t m0 = 0, m1 = 0;
        if (fread(&m0, 4, 1, f) != 1 || (size_t)(uint32_t)m0 != sizes[q]) {
            set_error("checkpoint record length does not match the channel's grid");
            rc = C3D_EIO;
        } else if (fseek(f, (long)sizes[q], SEEK_CUR) != 0 || fread(&m1, 4, 1, f) != 1 || m1 != m0) {
            set_error("checkpoint read failed (truncated file or bad record marker)");
            rc = C3D_EIO;
        }
    }
    rewind(f);
    return rc;
}
// A device record through the staging area: packed on the device, copied, written.
int rec_write_dev(c3d_channel *ch, FILE *f, int what, double *slot, size_t n, std::vector<double> &hb) {
    int rc = launch_ckpt(ch, 0, what, slot);
    if (rc) return rc;
    hb.resize(n);
    CK(cudaMemcpyAsync(hb.data(), slot, n * 8, cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return rec_write(f, hb.data(), n * 8);
}
int rec_read_dev(c3d_channel *ch, FILE *f, int what, double *slot, size_t n, std::vector<double> &hb) {
    hb.resize(n);
    int rc = rec_read(f, hb.data(), n * 8);
    if (rc) return rc;
    CK(cudaMemcpyAsync(slot, hb.data(), n * 8, cudaMemcpyHostToDevice, ch->stream));
    rc = launch_ckpt(ch, 1, what, slot);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}
}  // namespace

extern "C" {

int c3d_plane_stats(c3d_channel *ch, double *out) {
    if (!ch || !out) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_plane_stats"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    const size_t ns = stats_scratch_doubles(ch->g), nout = (size_t)ch->g.n2m * 29;
    if (!ch->stats && dalloc(&ch->stats, ns)) return C3D_ENOMEM;
    int rc = launch_stats(ch, ch->stats, ch->stats + nout);
    if (rc) return rc;
    CK(cudaMemcpyAsync(out, ch->stats, nout * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_plane_spectra(c3d_channel *ch, const double *vmo, double *xspec, double *zspec, double *rxx, double *rzz,
                      double *rxy) {
    if (!ch) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_plane_spectra"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    const Geo &g = ch->g;
    const size_t ns = stats_scratch_doubles(g), nout = (size_t)g.n2m * 29;
    const size_t nx = 3 * (size_t)g.n2m * g.n1m, nz = 3 * (size_t)g.n2m * g.n3m, nm = 3 * (size_t)g.n2m;
    if (!ch->stats && dalloc(&ch->stats, ns)) return C3D_ENOMEM;
    if (!ch->specbuf && dalloc(&ch->specbuf, nm + 3 * nx + 2 * nz)) return C3D_ENOMEM;
    double *dvmo = ch->specbuf, *dxs = dvmo + nm, *dzs = dxs + nx, *drxx = dzs + nz, *drzz = drxx + nx,
           *drxy = drzz + nz;
    int rc = launch_stats(ch, ch->stats, ch->stats + nout);
    if (rc) return rc;
    if (vmo) {
        CK(cudaMemcpyAsync(dvmo, vmo, nm * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    } else {   // the instantaneous plane means VM(J, L), columns 0..2 of the statistics table
        for (int L = 0; L < 3; ++L)
            CK(cudaMemcpy2DAsync(dvmo + (size_t)L * g.n2m, sizeof(double), ch->stats + L, 29 * sizeof(double),
                                 sizeof(double), g.n2m, cudaMemcpyDeviceToDevice, ch->stream));
    }
    rc = launch_spectra(ch, dvmo, ch->stats, xspec ? dxs : nullptr, zspec ? dzs : nullptr, rxx ? drxx : nullptr,
                        rzz ? drzz : nullptr, rxy ? drxy : nullptr);
    if (rc) { set_error("spectra kernels"); return rc; }
    if (xspec) CK(cudaMemcpyAsync(xspec, dxs, nx * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    if (zspec) CK(cudaMemcpyAsync(zspec, dzs, nz * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    if (rxx) CK(cudaMemcpyAsync(rxx, drxx, nx * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    if (rzz) CK(cudaMemcpyAsync(rzz, drzz, nz * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    if (rxy) CK(cudaMemcpyAsync(rxy, drxy, nx * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_plane_quadrants(c3d_channel *ch, const double *vmp, double *out) {
    if (!ch || !out) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_plane_quadrants"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    const Geo &g = ch->g;
    // the statistics scratch holds the output (8 N2M) and the partial sums (8 SB N2M)
    if (!ch->stats && dalloc(&ch->stats, stats_scratch_doubles(g))) return C3D_ENOMEM;
    if (!ch->specbuf && dalloc(&ch->specbuf, 3 * (size_t)g.n2m * (1 + 3 * (size_t)g.n1m + 2 * (size_t)g.n3m)))
        return C3D_ENOMEM;
    double *dvmp = nullptr;
    if (vmp) {
        dvmp = ch->specbuf;
        CK(cudaMemcpyAsync(dvmp, vmp, 2 * (size_t)g.n2m * sizeof(double), cudaMemcpyHostToDevice, ch->stream));
    }
    double *dout = ch->stats, *part = ch->stats + 8 * (size_t)g.n2m;
    int rc = launch_quadrants(ch, dvmp, dout, part);
    if (rc) { set_error("quadrant kernels"); return rc; }
    CK(cudaMemcpyAsync(out, dout, 8 * (size_t)g.n2m * sizeof(double), cudaMemcpyDeviceToHost, ch->stream));
    CK(cudaStreamSynchronize(ch->stream));
    return 0;
}

int c3d_wall_spectrum(c3d_channel *ch, double utau, double *out) {
    if (!ch || !out) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    const Geo &g = ch->g;
    const size_t nc = ((size_t)g.n1m / 2 + 1) * g.n3m, np_ = (size_t)g.np;
    double *buf = nullptr;
    if (dalloc(&buf, 2 * nc + np_)) return C3D_ENOMEM;
    double2 *c1 = reinterpret_cast<double2 *>(buf);
    int rc = launch_wall_spectrum(ch, utau, c1, buf + 2 * nc);
    if (!rc && cudaMemcpyAsync(out, buf + 2 * nc, np_ * sizeof(double), cudaMemcpyDeviceToHost, ch->stream) != cudaSuccess)
        rc = C3D_ECUDA;
    if (!rc && cudaStreamSynchronize(ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (rc) set_error("wall spectrum");
    cudaFree(buf);
    return rc;
}

int c3d_corr3d(c3d_channel *ch, double *out) {
    if (!ch || !out) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_corr3d"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    const Geo &g = ch->g;
    const size_t n = 3 * (size_t)g.n1m * g.n2m * g.n3m, nout = (size_t)g.n2m * 29;
    if (!ch->stats && dalloc(&ch->stats, stats_scratch_doubles(g))) return C3D_ENOMEM;
    int rc = launch_stats(ch, ch->stats, ch->stats + nout);
    if (rc) return rc;
    double *buf = nullptr;
    if (dalloc(&buf, n)) return C3D_ENOMEM;
    rc = launch_corr3d(ch, ch->stats, buf);
    if (!rc && cudaMemcpyAsync(out, buf, n * sizeof(double), cudaMemcpyDeviceToHost, ch->stream) != cudaSuccess)
        rc = C3D_ECUDA;
    if (!rc && cudaStreamSynchronize(ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (rc) set_error("3-D correlation");
    cudaFree(buf);
    return rc;
}

static int particles_common(c3d_channel *ch, int n, const double *par, double diam, double dens, double hhh) {
    if (!ch || n < 0 || (n > 0 && !par)) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before the particle calls"); return C3D_ESTATE; }
    if (!(diam > 0) || !(dens > 0) || !(hhh > 0)) { set_error("DIAM, DENS and HHH must be positive"); return C3D_EINVAL; }
    if (!ch->y_increasing) { set_error("the particle interpolation searches the Y faces: Y(1:N2) must increase"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    return 0;
}

int c3d_particles_advance(c3d_channel *ch, int n, double *par, double diam, double dens, double hhh, double dt,
                          int *impact) {
    int rc = particles_common(ch, n, par, diam, dens, hhh);
    if (rc || n == 0) return rc;
    if (!(dt > 0) || !isfinite(dt)) { set_error("dt must be positive and finite"); return C3D_EINVAL; }
    double *dp = nullptr;
    int *di = nullptr;
    if (dalloc(&dp, 6 * (size_t)n)) return C3D_ENOMEM;
    if (dalloc(&di, (size_t)n)) { cudaFree(dp); return C3D_ENOMEM; }
    rc = cudaMemcpyAsync(dp, par, 6 * (size_t)n * 8, cudaMemcpyHostToDevice, ch->stream) == cudaSuccess ? 0 : C3D_ECUDA;
    if (!rc) rc = launch_particles(ch, dp, n, diam, dens, hhh, dt, di, nullptr, nullptr, nullptr);
    if (!rc && cudaMemcpyAsync(par, dp, 6 * (size_t)n * 8, cudaMemcpyDeviceToHost, ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (!rc && impact && cudaMemcpyAsync(impact, di, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, ch->stream) != cudaSuccess)
        rc = C3D_ECUDA;
    if (!rc && cudaStreamSynchronize(ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (rc) set_error("particle step");
    cudaFree(dp);
    cudaFree(di);
    return rc;
}

int c3d_particles_source(c3d_channel *ch, int n, const double *par, double diam, double dens, double hhh,
                         double *ruh1, double *ruh2, double *ruh3) {
    int rc = particles_common(ch, n, par, diam, dens, hhh);
    if (rc) return rc;
    if (!ruh1 || !ruh2 || !ruh3) { set_error("null argument"); return C3D_EINVAL; }
    const Geo &g = ch->g;
    const size_t ns = (size_t)(g.n1m + 2) * (g.n2 + 1) * (g.n3m + 2);
    double *buf = nullptr, *dp = nullptr;
    if (dalloc(&buf, 3 * ns)) return C3D_ENOMEM;
    if (n > 0 && dalloc(&dp, 6 * (size_t)n)) { cudaFree(buf); return C3D_ENOMEM; }
    rc = cudaMemsetAsync(buf, 0, 3 * ns * 8, ch->stream) == cudaSuccess ? 0 : C3D_ECUDA;
    if (!rc && n > 0)
        rc = cudaMemcpyAsync(dp, par, 6 * (size_t)n * 8, cudaMemcpyHostToDevice, ch->stream) == cudaSuccess ? 0 : C3D_ECUDA;
    if (!rc && n > 0) rc = launch_particles(ch, dp, n, diam, dens, hhh, 0.0, nullptr, buf, buf + ns, buf + 2 * ns);
    double *outs[3] = {ruh1, ruh2, ruh3};
    for (int q = 0; q < 3 && !rc; ++q)
        if (cudaMemcpyAsync(outs[q], buf + q * ns, ns * 8, cudaMemcpyDeviceToHost, ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (!rc && cudaStreamSynchronize(ch->stream) != cudaSuccess) rc = C3D_ECUDA;
    if (rc) set_error("particle source");
    cudaFree(buf);
    if (dp) cudaFree(dp);
    return rc;
}

int c3d_checkpoint_write(c3d_channel *ch, const char *path, int ntime, double time, double presg,
                         double presg3) {
    if (!ch || !path) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("the channel has no state to write"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    CK(cudaStreamSynchronize(ch->stream));
    Xfer x;
    int rc = xfer_area(ch, &x);
    if (rc) return rc;
    const Geo &g = ch->g;
    const size_t nu = 3 * (size_t)g.n1m * (g.n2 + 1) * g.n3m, np_ = (size_t)g.n1m * g.n2m * g.n3m;
    FILE *f = fopen(path, "wb");
    if (!f) { set_error(std::string("cannot open ") + path + " for writing"); return C3D_EIO; }
    std::vector<double> hb;
    const int32_t dims[3] = {g.n1m, g.n2m, g.n3m};
    const double pg[2] = {presg, presg3};
    const int32_t nt = ntime;
    if (!(rc = rec_write(f, dims, sizeof(dims))) && !(rc = rec_write(f, pg, sizeof(pg))) &&
        !(rc = rec_write(f, &nt, 4)) && !(rc = rec_write(f, &time, 8)) &&
        !(rc = rec_write_dev(ch, f, 0, x.u(0), nu, hb)) && !(rc = rec_write_dev(ch, f, 1, x.p(), np_, hb)) &&
        !(rc = rec_write_dev(ch, f, 2, x.hh(0), 3 * np_, hb)) && ch->files != 0) {
        const size_t nt_ = (size_t)(g.n1m + 2) * (g.n3m + 2) * 2;
        std::vector<double> w(2 * nt_ + 3);
        if (!(rc = c3d_download_wall(ch, w.data(), w.data() + nt_)) && !(rc = c3d_get_wsm(ch, w.data() + 2 * nt_)))
            rc = rec_write(f, w.data(), w.size() * 8);
    }
    if (fclose(f) != 0 && !rc) { set_error("checkpoint close failed"); rc = C3D_EIO; }
    return rc;
}

int c3d_checkpoint_read(c3d_channel *ch, const char *path, int *ntime, double *time, double *presg,
                        double *presg3) {
    if (!ch || !path) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    CK(cudaStreamSynchronize(ch->stream));
    Xfer x;
    int rc = xfer_area(ch, &x);
    if (rc) return rc;
    const Geo &g = ch->g;
    const size_t nu = 3 * (size_t)g.n1m * (g.n2 + 1) * g.n3m, np_ = (size_t)g.n1m * g.n2m * g.n3m;
    FILE *f = fopen(path, "rb");
    if (!f) { set_error(std::string("cannot open ") + path); return C3D_EIO; }
    const size_t nt_ = (size_t)(g.n1m + 2) * (g.n3m + 2) * 2;
    {   // every record present and whole before any of the channel's state is replaced
        std::vector<size_t> sizes = {12, 16, 4, 8, nu * 8, np_ * 8, 3 * np_ * 8};
        if (ch->files != 0) sizes.push_back((2 * nt_ + 3) * 8);
        int32_t d0[3] = {0, 0, 0};
        if (rec_read(f, d0, sizeof(d0)) == 0 && (d0[0] != g.n1m || d0[1] != g.n2m || d0[2] != g.n3m)) {
            fclose(f);
            set_error("checkpoint grid does not match the channel's");
            return C3D_EINVAL;
        }
        rewind(f);
        if ((rc = rec_scan(f, sizes))) { fclose(f); return rc; }
    }
    std::vector<double> hb;
    int32_t dims[3] = {0, 0, 0}, nt = 0;
    double pg[2] = {0.0, 0.0}, tm = 0.0;
    rc = rec_read(f, dims, sizeof(dims));
    if (!rc && (dims[0] != g.n1m || dims[1] != g.n2m || dims[2] != g.n3m)) {
        set_error("checkpoint grid does not match the channel's");
        rc = C3D_EINVAL;
    }
    if (!rc && !(rc = rec_read(f, pg, sizeof(pg))) && !(rc = rec_read(f, &nt, 4)) && !(rc = rec_read(f, &tm, 8)) &&
        !(rc = rec_read_dev(ch, f, 0, x.u(0), nu, hb)) && !(rc = rec_read_dev(ch, f, 1, x.p(), np_, hb)) &&
        !(rc = rec_read_dev(ch, f, 2, x.hh(0), 3 * np_, hb)) && ch->files != 0) {
        std::vector<double> w(2 * nt_ + 3);
        if (!(rc = rec_read(f, w.data(), w.size() * 8)) && !(rc = c3d_upload_wall(ch, w.data(), w.data() + nt_)))
            rc = c3d_set_wsm(ch, w.data() + 2 * nt_);
    }
    fclose(f);
    if (rc) {
        // a read that failed after the scan (an I/O error) may have replaced part of the
        // state: the channel refuses to step until a complete state is uploaded or read
        ch->have_state = 0;
        return rc;
    }
    ch->have_state = 1;
    if (ntime) *ntime = nt;
    if (time) *time = tm;
    if (presg) *presg = pg[0];
    if (presg3) *presg3 = pg[1];
    return 0;
}

int c3d_op_set(c3d_channel *ch, const double *f) {
    if (!ch || !f) { set_error("null argument"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    const size_t rs = ch->precision == C3D_MIXED ? 4 : 8, nf = (size_t)ch->g.nf;
    for (int q = 0; q < 2; ++q) {
        if (!ch->opbuf[q]) {
            if (cudaMalloc(&ch->opbuf[q], nf * rs) != cudaSuccess) { set_error("cudaMalloc operand"); return C3D_ENOMEM; }
            CK(cudaMemset(ch->opbuf[q], 0, nf * rs));
        }
    }
    int rc = h2d(ch, f, ch->stage_elems);
    if (rc) return rc;
    launch_repack(ch, 0, 4, 0);
    CK(cudaStreamSynchronize(ch->stream));
    CK(cudaGetLastError());
    return 0;
}

int c3d_op_apply(c3d_channel *ch, int op, int count) {
    if (!ch || count < 0) { set_error("null channel or negative count"); return C3D_EINVAL; }
    if (!ch->opbuf[0]) { set_error("c3d_op_set must be called before c3d_op_apply"); return C3D_ESTATE; }
    if (op < C3D_OP_DX1 || op > C3D_OP_POISSON) { set_error("unknown operator"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    int nl = 0;
    for (int q = 0; q < count; ++q) {
        int rc = launch_operator(ch, op, &nl);
        if (rc) return rc;
    }
    CK(cudaGetLastError());
    ch->last_launches = count > 0 ? nl / count : 0;
    return 0;
}

int c3d_op_get(c3d_channel *ch, double *f) {
    if (!ch || !f) { set_error("null argument"); return C3D_EINVAL; }
    if (!ch->opbuf[1]) { set_error("no operator result"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    launch_repack(ch, 1, 5, 0);
    int rc = d2h(ch, f, ch->stage_elems);
    if (rc) return rc;
    CK(cudaGetLastError());
    return 0;
}

int c3d_pipe_wait_selftest(c3d_channel *ch, double limit_ms) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    if (!(limit_ms > 0) || !(limit_ms <= 1000.0)) { set_error("limit_ms must be in (0, 1000]"); return C3D_EINVAL; }
    cudaSetDevice(ch->device);
    return launch_pipe_selftest(ch, limit_ms);
}

int c3d_sync(c3d_channel *ch) {
    if (!ch) return C3D_EINVAL;
    CK(cudaStreamSynchronize(ch->stream));
    double sc[SCAL_COUNT];
    CK(cudaMemcpy(sc, ch->scal, sizeof(sc), cudaMemcpyDeviceToHost));
    return check_wall_flag(ch, sc);
}

int c3d_last_step_stats(c3d_channel *ch, double *ms, int *launches) {
    if (!ch) return C3D_EINVAL;
    if (ms) *ms = ch->last_ms;
    if (launches) *launches = ch->last_launches;
    return 0;
}

// ---- launch-schedule autotuner --------------------------------------------------
// The knobs of Tune are tried one group at a time on a scratch channel of the same grid
// and form holding a copy of the channel's state; each candidate runs one warm-up step
// and five profiled steps, and the candidate with the least summed time of the kernels
// the knob affects is kept.  Results are cached per (grid shape, form, models, device).
}  // extern "C"

namespace {
std::mutex g_tune_mu;
std::map<std::array<int, 8>, Tune> g_tune_cache;

std::array<int, 8> tune_key(const c3d_channel *ch) {
    return {ch->g.n1m, ch->g.n2m, ch->g.n3m, ch->precision, ch->refine, ch->files, ch->wmodel, ch->device};
}

bool tune_ok(const c3d_channel *ch, const Tune &t) {
    bool zl = true;
    for (int q = 0; q < 5; ++q)
        zl = zl && (t.zl[q] == 0 || t.zl[q] == 8 || t.zl[q] == 16 || (t.zl[q] == 32 && ch->g.n3m % 32 == 0));
    const bool xw = t.xw == 2 || t.xw == 4 || t.xw == 8;
    const bool tw = t.twz == 0 || t.twz == 4 || t.twz == 8 || t.twz == 16;
    // x plan 3 (register row FFTs) needs every lane of the warp to hold a chunk of an even
    // length: N1M a multiple of 64
    const bool fx = t.fxp >= 0 && t.fxp <= 2 ? true : (t.fxp == 3 && ch->g.n1m % 64 == 0);
    return zl && xw && tw && fx && t.fzp >= 0 && t.fzp <= 2 && (t.zsplit == 0 || t.zsplit == 1) &&
           (t.xsplit == 0 || t.xsplit == 1) && (t.xbulk == 0 || t.xbulk == 2 || t.xbulk == 3) &&
           (t.xstage == 0 || (t.xstage == 1 && ch->g.n1m % 2 == 0)) && (t.ycn == 0 || t.ycn == 32 || t.ycn == 64) &&
           (t.xlanes == 0 || t.xlanes == x_segment_lanes(ch->g.n1m, ch->g.n3m)) && (t.conc == 0 || t.conc == 1);
}

// Sets the schedule; the FFT plans get the new radix order and keep their twiddle tables.
void apply_tune(c3d_channel *ch, const Tune &t) {
    ch->tune = t;
    FftPlan fx = make_plan(ch->g.n1m / 2, t.fxp), fz = make_plan(ch->g.n3m, t.fzp);
    if (fx.nst < 0 || fz.nst < 0) return;   // cannot happen for N <= 4096; keep the old plans
    fx.tw64 = ch->fx.tw64;
    fx.tw32 = ch->fx.tw32;
    fz.tw64 = ch->fz.tw64;
    fz.tw32 = ch->fz.tw32;
    ch->fx = fx;
    ch->fz = fz;
}

// Time of the kernels `names` over five profiled steps under schedule t, the smaller of
// two such runs (a single run of a few milliseconds moves by a few percent between
// candidates that differ by less).
int time_schedule(c3d_channel *sc, const Tune &t, double dt, const std::vector<std::string> &names, double *cost) {
    apply_tune(sc, t);
    int rc = step_common(sc, dt, nullptr, nullptr, true);
    if (rc && rc != C3D_ENOTCONV) return rc;
    double best = 1e300;
    for (int rep = 0; rep < 2; ++rep) {
        rc = 0;
        c3d_profile(sc, 1);
        for (int q = 0; q < 5 && !rc; ++q) rc = step_common(sc, dt, nullptr, nullptr, false);
        if (rc) { c3d_profile(sc, 0); return rc; }
        CK(cudaStreamSynchronize(sc->stream));
        double c = 0.0;
        for (size_t q = 0; q < sc->prof_name.size(); ++q)
            for (const std::string &n : names)   // a name covers its split pieces (zA -> zA_u, ...)
                if (sc->prof_name[q] == n || sc->prof_name[q].rfind(n + "_", 0) == 0) c += sc->prof_ms[q];
        c3d_profile(sc, 0);
        best = std::min(best, c);
    }
    *cost = best;
    return 0;
}
}  // namespace

extern "C" {

int c3d_get_schedule(c3d_channel *ch, int *sched) {
    if (!ch || !sched) { set_error("null argument"); return C3D_EINVAL; }
    const Tune &t = ch->tune;
    for (int q = 0; q < 5; ++q) sched[q] = t.zl[q];
    sched[5] = t.xw; sched[6] = t.twz; sched[7] = t.fxp; sched[8] = t.fzp; sched[9] = t.zsplit; sched[10] = t.xsplit;
    sched[11] = t.xbulk;
    sched[12] = t.xstage;
    sched[13] = t.ycn;
    sched[14] = t.xlanes;
    sched[15] = t.conc;
    return 0;
}

int c3d_set_schedule(c3d_channel *ch, const int *sched) {
    if (!ch || !sched) { set_error("null argument"); return C3D_EINVAL; }
    Tune t{{sched[0], sched[1], sched[2], sched[3], sched[4]}, sched[5], sched[6], sched[7], sched[8], sched[9],
           sched[10], sched[11], sched[12], sched[13], sched[14], sched[15]};
    if (!tune_ok(ch, t)) { set_error("invalid schedule"); return C3D_EINVAL; }
    apply_tune(ch, t);
    return 0;
}

int c3d_autotune(c3d_channel *ch, int *sched) {
    if (!ch) { set_error("null channel"); return C3D_EINVAL; }
    if (!ch->have_state) { set_error("c3d_upload must be called before c3d_autotune"); return C3D_ESTATE; }
    cudaSetDevice(ch->device);
    const std::array<int, 8> key = tune_key(ch);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            apply_tune(ch, it->second);
            return sched ? c3d_get_schedule(ch, sched) : 0;
        }
    }
    CK(cudaStreamSynchronize(ch->stream));
    c3d_grid gs = ch->grid_copy;
    c3d_channel *sc = nullptr;
    int rc = c3d_create(&gs, &sc);
    if (rc) return rc;
    const size_t rs = ch->precision == C3D_MIXED ? 4 : 8, nf = (size_t)ch->g.nf;
    void *src[] = {ch->u, ch->v, ch->w, ch->p}, *dst[] = {sc->u, sc->v, sc->w, sc->p};
    for (int q = 0; q < 4; ++q) cudaMemcpy(dst[q], src[q], nf * 8, cudaMemcpyDeviceToDevice);
    for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 3; ++c) cudaMemcpy(sc->hh[b][c], ch->hh[b][c], nf * rs, cudaMemcpyDeviceToDevice);
    cudaMemcpy(sc->scal, ch->scal, SCAL_COUNT * 8, cudaMemcpyDeviceToDevice);
    if (ch->files != 0) {
        cudaMemcpy(sc->tauw, ch->tauw, 2 * (size_t)ch->g.np * 8, cudaMemcpyDeviceToDevice);
        cudaMemcpy(sc->taub, ch->taub, 2 * (size_t)ch->g.np * 8, cudaMemcpyDeviceToDevice);
    }
    sc->have_state = 1;
    const double dt = ch->dt_cached > 0 ? ch->dt_cached : 1e-3;
    // knob q: 0-4 the segment length of zA..zE, 5 x rows per block, 6 z-FFT tile, 7/8 plans,
    // 9 zA split, 10 xA split, 11 bulk-copy stages of the x passes, 12 xA rows staged by bulk copies,
    // 13 form of the wall-normal CN factor, 14 lanes per row of the x passes (15, concurrent pieces, below)
    struct Group { int knob; std::vector<int> cand; std::vector<std::string> kernels; };
    const Group groups[] = {
        {9, {0, 1}, {"zA"}}, {10, {0, 1}, {"xA"}}, {12, {0, 1}, {"xA"}}, {14, {0, 8, 16}, {"xA", "xB", "xC", "xD"}},
        {13, {0, 32, 64}, {"ycn"}},
        {0, {0, 8, 16, 32}, {"zA"}}, {1, {0, 8, 16, 32}, {"zB"}}, {2, {0, 8, 16, 32}, {"zC"}},
        {3, {0, 8, 16, 32}, {"zD"}}, {4, {0, 8, 16, 32}, {"zE"}},
        {5, {2, 4, 8}, {"xA", "xB", "xC", "xD"}},
        {6, {0, 4, 8, 16}, {"fftz_fwd", "fftz_inv"}},
        {8, {0, 1, 2}, {"fftz_fwd", "fftz_inv"}},
        {7, {0, 1, 2, 3}, {"xC", "xD"}},
        {11, {0, 2, 3}, {"xC"}},
    };
    auto knob = [](Tune &t, int q) -> int & {
        return q < 5 ? t.zl[q] : q == 5 ? t.xw : q == 6 ? t.twz : q == 7 ? t.fxp : q == 8 ? t.fzp : q == 9 ? t.zsplit
             : q == 10 ? t.xsplit : q == 11 ? t.xbulk : q == 12 ? t.xstage : q == 13 ? t.ycn : q == 14 ? t.xlanes
             : t.conc;
    };
    Tune best = ch->tune;
    for (const Group &gp : groups) {
        double bcost = 1e300;
        int bval = knob(best, gp.knob);
        for (int v : gp.cand) {
            Tune t = best;
            knob(t, gp.knob) = v;
            if (!tune_ok(ch, t)) continue;
            double cost = 0.0;
            rc = time_schedule(sc, t, dt, gp.kernels, &cost);
            if (rc) { c3d_destroy(sc); return rc; }
            if (cost < bcost) { bcost = cost; bval = v; }
        }
        knob(best, gp.knob) = bval;
    }
    // knob 15 by whole-step time: the per-kernel profile runs the pieces one after another,
    // so the concurrent form is chosen on five unprofiled steps (twice each, the minimum)
    if (best.xsplit || best.zsplit) {
        float bms[2] = {1e30f, 1e30f};
        for (int rep = 0; rep < 2; ++rep)
            for (int v = 0; v < 2; ++v) {
                Tune t = best;
                t.conc = v;
                apply_tune(sc, t);
                rc = step_common(sc, dt, nullptr, nullptr, true);
                if (rc && rc != C3D_ENOTCONV) { c3d_destroy(sc); return rc; }
                rc = 0;
                CK(cudaEventRecord(sc->tm0, sc->stream));
                for (int q = 0; q < 5 && !rc; ++q) rc = step_common(sc, dt, nullptr, nullptr, false);
                if (rc) { c3d_destroy(sc); return rc; }
                CK(cudaEventRecord(sc->tm1, sc->stream));
                CK(cudaEventSynchronize(sc->tm1));
                float ms = 0.f;
                CK(cudaEventElapsedTime(&ms, sc->tm0, sc->tm1));
                bms[v] = std::min(bms[v], ms);
            }
        best.conc = bms[1] < bms[0] ? 1 : 0;
    }
    c3d_destroy(sc);
    apply_tune(ch, best);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    return sched ? c3d_get_schedule(ch, sched) : 0;
}

// ---- batched ensemble ----------------------------------------------------------
// Every channel keeps its own stream.  One ensemble step is one CUDA graph: a copy of the
// PRESG/PRESG3 values of all channels from pinned host memory, a scatter kernel, then a
// fork to every channel's stream (the channels' step kernels run concurrently), a join,
// a gather kernel and the copy back.  Graphs are captured per AB2 buffer parity and
// recaptured when a channel's DT changes.
}  // extern "C"

namespace {
__global__ void k_batch_scatter(int n, const double *src, double *const *scal) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        scal[i][SCAL_PRESG] = src[2 * i];
        scal[i][SCAL_PRESG3] = src[2 * i + 1];
    }
}
__global__ void k_batch_gather(int n, double *dst, double *const *scal) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        dst[2 * i] = scal[i][SCAL_PRESG];
        dst[2 * i + 1] = scal[i][SCAL_PRESG3];
    }
}
}  // namespace

struct c3d_batch {
    std::vector<c3d_channel *> ch;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> join;
    double *hpres = nullptr, *dpres = nullptr;
    double **dscal = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    std::vector<double> gdt[2];
    int launches = 0;
    float last_ms = 0.f;
    int form = C3D_BATCH_WORKLIST;            // requested form (c3d_batch_set_form)
    int groups = 2;                           // work-list form: channel groups on their own streams
    BatchSched sched{{8, 8, 16, 16, 8}, 2, 0};   // work-list form: z segments of zA..zE, warps per x block, concurrent pieces
    // work-list form, per AB2 parity: every channel's StepArgs and the block maps
    void *dargs[2] = {nullptr, nullptr};
    size_t nargs[2] = {0, 0};
    BMap *dmap[2] = {nullptr, nullptr};
    size_t nmap[2] = {0, 0};
};

static void batch_free(c3d_batch *b) {
    for (auto *q : b->ch) c3d_destroy(q);
    for (int p = 0; p < 2; ++p)
        if (b->exec[p]) cudaGraphExecDestroy(b->exec[p]);
    for (auto e : b->join) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->hpres) cudaFreeHost(b->hpres);
    if (b->dpres) cudaFree(b->dpres);
    if (b->dscal) cudaFree(b->dscal);
    for (int p = 0; p < 2; ++p) {
        if (b->dargs[p]) cudaFree(b->dargs[p]);
        if (b->dmap[p]) cudaFree(b->dmap[p]);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// The work-list form applies when every channel is DNS (FILES = 0) in the same
// precision, C3D_FP64 or C3D_MIXED.
static bool batch_worklist_ok(const c3d_batch *b) {
    for (auto *c : b->ch)
        if (c->files != 0 || c->refine || c->precision != b->ch[0]->precision) return false;
    return true;
}

static int grow(void **p, size_t *have, size_t need) {
    if (*have >= need && *p) return 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (cudaMalloc(p, need) != cudaSuccess) { set_error("batch: cudaMalloc of the work lists"); return C3D_ENOMEM; }
    *have = need;
    return 0;
}

// Work-list form of the ensemble step: each pass of the step is one launch per group of
// channels whose kernel for that pass is the same template instance with the same block
// shape; block q of a launch runs block map[q].x of channel map[q].ch.  The channels'
// StepArgs (for the parity the step writes and its DT) and the maps live on the device.
static int batch_capture_worklist(c3d_batch *b, const double *dt, int par) {
    const int n = (int)b->ch.size();
    const size_t asz = batch_args_size(b->ch[0]);
    std::vector<unsigned char> args(asz * n);
    std::vector<std::vector<BKern>> plans(n);
    for (int i = 0; i < n; ++i) {
        c3d_channel *c = b->ch[i];
        c->cur = par;   // GETUP's HH2 <- HH: this step writes buffer par
        batch_args(c, dt[i], args.data() + (size_t)i * asz);
        int rc = batch_plan(c, b->sched, plans[i]);
        if (rc) return rc;
        if (plans[i].size() != plans[0].size()) { set_error("batch: channels with different pass lists"); return C3D_EINVAL; }
    }
    // channel groups: G sets of channels (largest first, dealt round-robin), each with
    // its own work list on its own stream, so that the passes of one group overlap those
    // of another; within a launch the channels with the longest wall-normal lines first
    const int G = std::max(1, std::min(b->groups, n));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const Geo &gx = b->ch[x]->g, &gy = b->ch[y]->g;
        if (gx.n2m != gy.n2m) return gx.n2m > gy.n2m;
        return (long long)gx.n1m * gx.n3m > (long long)gy.n1m * gy.n3m;
    });
    std::vector<std::vector<int>> members(G);
    for (int q = 0; q < n; ++q) members[q % G].push_back(order[q]);
    struct Grp { const void *fn; unsigned block; size_t smem, off, cnt; int sg, run, piece; };
    std::vector<Grp> launches;
    std::vector<BMap> map;
    for (int sg = 0; sg < G; ++sg)
        for (size_t p = 0; p < plans[0].size(); ++p) {
            std::vector<Grp> gs;
            for (int i : members[sg]) {
                const BKern &k = plans[i][p];
                size_t q = 0;
                while (q < gs.size() && !(gs[q].fn == k.fn && gs[q].block == k.block)) ++q;
                if (q == gs.size()) gs.push_back({k.fn, k.block, 0, 0, 0, sg, b->sched.conc ? k.run : 0, k.piece});
                gs[q].smem = std::max(gs[q].smem, k.smem);
            }
            for (Grp &gr : gs) {
                gr.off = map.size();
                for (int i : members[sg]) {
                    const BKern &k = plans[i][p];
                    if (k.fn != gr.fn || k.block != gr.block) continue;
                    for (unsigned x = 0; x < k.nblocks; ++x) map.push_back(BMap{i, x, 0u, k.nblocks});
                }
                gr.cnt = map.size() - gr.off;
                launches.push_back(gr);
            }
        }
    int rc = grow(&b->dargs[par], &b->nargs[par], args.size());
    if (!rc) rc = grow((void **)&b->dmap[par], &b->nmap[par], map.size() * sizeof(BMap));
    if (rc) return rc;
    CK(cudaMemcpy(b->dargs[par], args.data(), args.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b->dmap[par], map.data(), map.size() * sizeof(BMap), cudaMemcpyHostToDevice));
    for (const Grp &gr : launches)
        if (gr.smem > 48 * 1024 &&
            cudaFuncSetAttribute(gr.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gr.smem) != cudaSuccess) {
            set_error("batch: shared memory of a work-list kernel");
            return C3D_ECUDA;
        }
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    cudaMemcpyAsync(b->dpres, b->hpres, 2 * n * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    k_batch_scatter<<<(n + 127) / 128, 128, 0, b->stream>>>(n, b->dpres, b->dscal);
    cudaEventRecord(b->fork, b->stream);
    cudaError_t le = cudaSuccess;
    for (int sg = 0; sg < G; ++sg) {
        cudaStream_t s = G == 1 ? b->stream : b->ch[sg]->stream;   // a channel stream, idle meanwhile
        c3d_channel *own = b->ch[sg];   // its two extra streams carry pieces 0 and 1 of a run
        if (G > 1) cudaStreamWaitEvent(s, b->fork, 0);
        int run = 0;
        auto join = [&]() {
            for (int q = 0; q < 2; ++q) {
                cudaEventRecord(own->pev[1 + q], own->par[q]);
                cudaStreamWaitEvent(s, own->pev[1 + q], 0);
            }
        };
        for (const Grp &gr : launches) {
            if (gr.sg != sg) continue;
            if (gr.run != run) {   // a run of independent pieces ends or begins
                if (run) join();
                run = gr.run;
                if (run) {
                    cudaEventRecord(own->pev[0], s);
                    for (int q = 0; q < 2; ++q) cudaStreamWaitEvent(own->par[q], own->pev[0], 0);
                }
            }
            cudaStream_t ls = (run && gr.piece < 2) ? own->par[gr.piece] : s;
            void *A = b->dargs[par];
            BMap *M = b->dmap[par] + gr.off;
            void *kargs[] = {&A, &M};
            cudaError_t e = cudaLaunchKernel(gr.fn, dim3((unsigned)gr.cnt), dim3(gr.block), kargs, gr.smem, ls);
            if (e != cudaSuccess && le == cudaSuccess) le = e;
        }
        if (run) join();
        if (G > 1) {
            cudaEventRecord(b->join[sg], s);
            cudaStreamWaitEvent(b->stream, b->join[sg], 0);
        }
    }
    k_batch_gather<<<(n + 127) / 128, 128, 0, b->stream>>>(n, b->dpres, b->dscal);
    cudaMemcpyAsync(b->hpres, b->dpres, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        set_error(std::string("batch work-list capture: ") + cudaGetErrorString(le != cudaSuccess ? le : e));
        return C3D_ECUDA;
    }
    if (b->exec[par]) cudaGraphExecDestroy(b->exec[par]);
    b->exec[par] = nullptr;
    e = cudaGraphInstantiate(&b->exec[par], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(e));
        return C3D_ECUDA;
    }
    b->gdt[par].assign(dt, dt + n);
    b->launches = (int)launches.size() + 2;
    return 0;
}

// Captures the ensemble step for the parity the channels move to; leaves ch->cur there.
static int batch_capture(c3d_batch *b, const double *dt, int par) {
    if (b->form == C3D_BATCH_WORKLIST && batch_worklist_ok(b)) return batch_capture_worklist(b, dt, par);
    const int n = (int)b->ch.size();
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    int nl = 0;
    cudaMemcpyAsync(b->dpres, b->hpres, 2 * n * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    k_batch_scatter<<<(n + 127) / 128, 128, 0, b->stream>>>(n, b->dpres, b->dscal);
    cudaEventRecord(b->fork, b->stream);
    int rc = 0;
    for (int i = 0; i < n && !rc; ++i) {
        c3d_channel *c = b->ch[i];
        cudaStreamWaitEvent(c->stream, b->fork, 0);
        int keep = c->prof_on;
        c->prof_on = 0;
        rc = launch_step(c, dt[i], &nl);
        c->prof_on = keep;
        cudaEventRecord(b->join[i], c->stream);
        cudaStreamWaitEvent(b->stream, b->join[i], 0);
    }
    k_batch_gather<<<(n + 127) / 128, 128, 0, b->stream>>>(n, b->dpres, b->dscal);
    cudaMemcpyAsync(b->hpres, b->dpres, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) {
        set_error(std::string("batch capture: ") + cudaGetErrorString(e));
        return C3D_ECUDA;
    }
    if (b->exec[par]) cudaGraphExecDestroy(b->exec[par]);
    b->exec[par] = nullptr;
    e = cudaGraphInstantiate(&b->exec[par], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(e));
        return C3D_ECUDA;
    }
    b->gdt[par].assign(dt, dt + n);
    b->launches = nl + 2;
    for (auto *c : b->ch)
        if (c->cur != par) { set_error("batch parity mismatch"); return C3D_ESTATE; }
    return 0;
}

extern "C" {

int c3d_batch_create(int nchan, const c3d_grid *grids, c3d_batch **out) {
    if (!out || !grids || nchan <= 0) { set_error("bad batch arguments"); return C3D_EINVAL; }
    *out = nullptr;
    c3d_batch *b = new c3d_batch();
    for (int i = 0; i < nchan; ++i) {
        c3d_channel *c = nullptr;
        int rc = c3d_create(&grids[i], &c);
        if (rc) {
            batch_free(b);
            return rc;
        }
        b->ch.push_back(c);
        if (grids[i].files != 0 && grids[i].wmodel == 2) {   // its update schedule follows NTIME
            set_error("WMODEL 2 (WALLMODEL_IWMLES_SMOOTH) channels step individually, not in a batch graph");
            batch_free(b);
            return C3D_EINVAL;
        }
    }
    b->join.resize(nchan, nullptr);
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreate(&b->t0) == cudaSuccess && cudaEventCreate(&b->t1) == cudaSuccess &&
              cudaHostAlloc((void **)&b->hpres, 2 * nchan * sizeof(double), cudaHostAllocDefault) == cudaSuccess &&
              cudaMalloc((void **)&b->dpres, 2 * nchan * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void **)&b->dscal, nchan * sizeof(double *)) == cudaSuccess;
    for (int i = 0; ok && i < nchan; ++i)
        ok = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
    if (ok) {
        std::vector<double *> ps(nchan);
        for (int i = 0; i < nchan; ++i) ps[i] = b->ch[i]->scal;
        ok = cudaMemcpy(b->dscal, ps.data(), nchan * sizeof(double *), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (!ok) {
        set_error("batch: stream/event/memory set-up failed");
        batch_free(b);
        return C3D_ECUDA;
    }
    *out = b;
    return 0;
}

int c3d_batch_destroy(c3d_batch *b) {
    if (!b) return C3D_EINVAL;
    cudaStreamSynchronize(b->stream);
    batch_free(b);
    return 0;
}

int c3d_batch_channel(c3d_batch *b, int index, c3d_channel **ch) {
    if (!b || !ch || index < 0 || index >= (int)b->ch.size()) { set_error("bad batch index"); return C3D_EINVAL; }
    *ch = b->ch[index];
    return 0;
}

int c3d_batch_step(c3d_batch *b, int ntime, const double *dt, double *presg, double *presg3) {
    (void)ntime;
    if (!b || !dt || !presg || !presg3) { set_error("null argument"); return C3D_EINVAL; }
    const int n = (int)b->ch.size();
    const int cur = b->ch[0]->cur;
    for (int i = 0; i < n; ++i) {
        c3d_channel *c = b->ch[i];
        if (!c->have_state) { set_error("batch channel without uploaded state"); return C3D_ESTATE; }
        if (c->cur != cur) { set_error("batch channels were stepped separately"); return C3D_ESTATE; }
        if (!(dt[i] > 0) || !isfinite(dt[i])) { set_error("dt must be positive and finite"); return C3D_EINVAL; }
        if (dt[i] != c->dt_cached) {
            int rc = upload_ycn(c, dt[i]);
            if (rc) return rc;
        }
        // the channels' own streams must be idle before the graph runs
        CK(cudaStreamSynchronize(c->stream));
    }
    const int par = 1 - cur;
    for (int i = 0; i < n; ++i) {
        b->hpres[2 * i] = presg[i];
        b->hpres[2 * i + 1] = presg3[i];
    }
    if (!b->exec[par] || b->gdt[par].size() != (size_t)n ||
        !std::equal(b->gdt[par].begin(), b->gdt[par].end(), dt)) {
        int rc = batch_capture(b, dt, par);   // leaves every channel at parity par
        if (rc) return rc;
    } else {
        for (auto *c : b->ch) c->cur = par;
    }
    CK(cudaEventRecord(b->t0, b->stream));
    CK(cudaGraphLaunch(b->exec[par], b->stream));
    CK(cudaEventRecord(b->t1, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    cudaEventElapsedTime(&b->last_ms, b->t0, b->t1);
    for (int i = 0; i < n; ++i) {
        presg[i] = b->hpres[2 * i];
        presg3[i] = b->hpres[2 * i + 1];
    }
    return 0;
}

}  // extern "C"

// A change of the ensemble's form or schedule: wait for the running step and drop the
// captured graphs, so that the next c3d_batch_step captures them again.
static int batch_recapture(c3d_batch *b) {
    CK(cudaStreamSynchronize(b->stream));
    for (int p = 0; p < 2; ++p) {
        if (b->exec[p]) cudaGraphExecDestroy(b->exec[p]);
        b->exec[p] = nullptr;
        b->gdt[p].clear();
    }
    return 0;
}

extern "C" {

int c3d_batch_set_form(c3d_batch *b, int form) {
    if (!b || (form != C3D_BATCH_STREAMS && form != C3D_BATCH_WORKLIST)) { set_error("bad batch form"); return C3D_EINVAL; }
    if (form != b->form)
        if (int rc = batch_recapture(b)) return rc;
    b->form = form;
    return 0;
}

int c3d_batch_set_groups(c3d_batch *b, int groups) {
    if (!b || groups < 1 || groups > 64) { set_error("groups must be in [1, 64]"); return C3D_EINVAL; }
    if (groups != b->groups)
        if (int rc = batch_recapture(b)) return rc;
    b->groups = groups;
    return 0;
}

int c3d_batch_set_z_segments(c3d_batch *b, const int *seg) {
    if (!b || !seg) { set_error("null argument"); return C3D_EINVAL; }
    for (int q = 0; q < 5; ++q)
        if (seg[q] != 8 && seg[q] != 16 && seg[q] != 32) { set_error("z segment lengths must be 8, 16 or 32"); return C3D_EINVAL; }
    if (int rc = batch_recapture(b)) return rc;
    for (int q = 0; q < 5; ++q) b->sched.zseg[q] = seg[q];
    return 0;
}

int c3d_batch_set_concurrent(c3d_batch *b, int on) {
    if (!b || (on != 0 && on != 1)) { set_error("concurrent must be 0 or 1"); return C3D_EINVAL; }
    if (int rc = batch_recapture(b)) return rc;
    b->sched.conc = on;
    return 0;
}

int c3d_batch_set_x_warps(c3d_batch *b, int warps) {
    if (!b || (warps != 2 && warps != 4 && warps != 8)) { set_error("x warps per block must be 2, 4 or 8"); return C3D_EINVAL; }
    if (int rc = batch_recapture(b)) return rc;
    b->sched.xw = warps;
    return 0;
}

int c3d_batch_get_form(c3d_batch *b, int *form) {
    if (!b || !form) { set_error("null argument"); return C3D_EINVAL; }
    *form = (b->form == C3D_BATCH_WORKLIST && batch_worklist_ok(b)) ? C3D_BATCH_WORKLIST : C3D_BATCH_STREAMS;
    return 0;
}

int c3d_batch_sync(c3d_batch *b) {
    if (!b) return C3D_EINVAL;
    CK(cudaStreamSynchronize(b->stream));
    for (auto *q : b->ch) {
        int rc = c3d_sync(q);
        if (rc) return rc;
    }
    return 0;
}

int c3d_batch_last_step_stats(c3d_batch *b, double *ms, int *kernel_launches) {
    if (!b) return C3D_EINVAL;
    if (ms) *ms = b->last_ms;
    if (kernel_launches) *kernel_launches = b->launches;
    return 0;
}

}  // extern "C"
