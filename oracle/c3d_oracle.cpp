// c3d_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// FP64 CPU restatement of compact3d's channel-flow time step (RuifengHu/compact3d,
// file compact3d.f; citations are compact3d.f:line).  It is the parity checker for
// the CUDA library and the timed CPU baseline of bench.py.  Nothing in the product
// path links or calls it.
//
// Parity status: UNPINNED.  The reference ships no tests, fixtures or golden vectors,
// and it cannot be built in this environment (it is Fortran 77 with FFTW and no
// Fortran compiler or FFTW is installed).  This restatement is therefore checked
// against known answers (modified wavenumbers of the compact operators, dense solves,
// numpy.fft, Poisson round trips, divergence after projection, laminar steady state).
//
// Conventions kept from the reference:
//   * loop order, operation order and parenthesisation of every arithmetic expression
//     follow the Fortran source (compile with -ffp-contract=off so no FMA is formed);
//   * FP64 everywhere (the reference is assumed built with 8-byte default REAL);
//   * arrays use the Fortran layouts U(0:M1,0:M2,0:M3,3), P(M1,M2,M3) with M1=N1,
//     M2=N2, M3=N3, column-major;
//   * OpenMP parallel loops where the reference has !$omp directives;
//   * global sums are taken per outer index and then added in index order, so results
//     do not depend on the thread count (the reference's OpenMP reductions do).
//   * FFTW (a third-party dependency the reference calls through dfftw_plan_dft_2d /
//     dfftw_execute_dft, compact3d.f:9315-9333, version not pinned anywhere) is
//     replaced by a mixed-radix complex FFT written from the DFT definition with
//     FFTW's conventions: forward exponent -1, backward +1, unnormalised.
#include <cmath>
#include <complex>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/c3d.h"

namespace {

typedef std::complex<double> cplx;

struct Orc {
    int N1, N2, N3, N1M, N2M, N3M, N1MH, N3MH;
    double ALX, ALY, ALZ, VOL, DX1, DX3, DX1Q, DX3Q, RE;
    int FILES, WMODEL;
    int IFWALL;
    // 1-based Fortran vectors (index 0 allowed where the reference declares 0:)
    std::vector<double> Y, DY, H, HM, HC, HP, DYM, DYC, DYP;
    std::vector<int> IPA, IMA, KPA, KMA, JPA, JMU, JMV;
    std::vector<double> FJPA, FJMU, FJMV;
    std::vector<double> AK1, AK3, PMJ, PCJ, PPJ;
    std::vector<double> UBC;          // UBC(0:M1,0:M3,3,2)
    std::vector<double> TAUW, TAUB;   // (0:M1,0:M3,2)
    double WSM[3] = {0.0, 0.0, 0.0};  // /WSMEM/ WSM(1:3) as the SGS model and wall model see it
    double TAOW = 0.0;                // /WALLTAO/ TAOW
    std::vector<double> SMAGC;        // /SGSMEAN/ SMAGC(1:N2M)
    std::vector<double> BETA;         // SGSSD's scale-dependence BETA per plane (unclipped)
    std::vector<double> IWM;          // WALLMODEL_IWMLES_SMOOTH's per-point state (IW_NS x N1M N3M)
    double WM_DT = 0.0, CFLMAX = 1.0; // its accumulated step and the driver's CFLMAX
    int iwm_ready = 0;
    std::vector<double> SGS;          // SGSVIS when the caller passes none
    int wall_iter_cap = 10000;        // Newton iterations allowed per wall point
    // work arrays of GETUP / UHCALC / DPCALC
    std::vector<double> UH, HH2, RUH1, RUH2, RUH3, DP, RDP;
    std::vector<double> FRDP, FDP;    // (M1,M2,M3MD)
    std::vector<cplx> COEF;           // (M1M,M3M,M2)

    long su1, su2, su3;               // strides of (0:M1,0:M2,0:M3)
    long sp1, sp2;                    // strides of (M1,M2,M3)

    inline long iu(int i, int j, int k) const { return i + su1 * j + su2 * (long)k; }
    inline long iuc(int i, int j, int k, int c) const { return iu(i, j, k) + su3 * (long)(c - 1); }
    inline long ip(int i, int j, int k) const { return (i - 1) + sp1 * (j - 1) + sp2 * (long)(k - 1); }
    inline long itw(int i, int k, int w) const { return i + (long)(N1 + 1) * k + (long)(N1 + 1) * (N3 + 1) * (w - 1); }
    inline long iubc(int i, int k, int c, int w) const {
        return i + (long)(N1 + 1) * k + (long)(N1 + 1) * (N3 + 1) * ((c - 1) + 3 * (w - 1));
    }
};

// ----------------------------------------------------------------------------------
// Line solvers (compact3d.f:8630-9046, 9444-9459).  Arrays are 1-based.
// ----------------------------------------------------------------------------------

// CTDMA11 / CTDMA33: cyclic tridiagonal, bordered LU with divisions (compact3d.f:8952-9046).
void ctdma_bordered(int n, const double *A, const double *B, const double *C,
                    const double *D, double *X) {
    thread_local std::vector<double> s;
    s.resize(5 * (size_t)(n + 1));
    double *Z = s.data(), *BETA = Z + (n + 1), *P = BETA + (n + 1), *GAMA = P + (n + 1),
           *Q = GAMA + (n + 1);
    BETA[1] = B[1];
    GAMA[1] = C[1] / BETA[1];
    for (int i = 2; i <= n - 1; i++) {
        BETA[i] = B[i] - A[i] * GAMA[i - 1];
        GAMA[i] = C[i] / BETA[i];
    }
    P[1] = C[n];
    Q[1] = A[1] / BETA[1];
    for (int i = 2; i <= n - 2; i++) {
        P[i] = -P[i - 1] * GAMA[i - 1];
        Q[i] = -A[i] * Q[i - 1] / BETA[i];
    }
    P[n - 1] = A[n] - P[n - 2] * GAMA[n - 2];
    Q[n - 1] = (C[n - 1] - A[n - 1] * Q[n - 2]) / BETA[n - 1];
    P[n] = B[n];
    for (int i = 1; i <= n - 1; i++) P[n] = P[n] - P[i] * Q[i];
    Z[1] = D[1] / BETA[1];
    for (int i = 2; i <= n - 1; i++) Z[i] = (D[i] - A[i] * Z[i - 1]) / BETA[i];
    Z[n] = D[n];
    for (int i = 1; i <= n - 1; i++) Z[n] = Z[n] - P[i] * Z[i];
    Z[n] = Z[n] / P[n];
    X[n] = Z[n];
    X[n - 1] = Z[n - 1] - Q[n - 1] * X[n];
    for (int i = n - 2; i >= 1; i--) X[i] = Z[i] - GAMA[i] * X[i + 1] - Q[i] * X[n];
}

// CTDMA1J / CTDMA3I per line: cyclic bordered LU with reciprocals (compact3d.f:8662-8809).
// D and X may alias (the reference passes the same array).
void ctdma_recip(int NS, int NF, const double *A, const double *B, const double *C,
                 const double *D, double *X) {
    thread_local std::vector<double> s;
    s.resize(3 * (size_t)(NF + 2));
    double *GAM = s.data(), *P = GAM + (NF + 2), *Q = P + (NF + 2);
    int I = NS;
    double BET1 = 1.0 / B[I];
    GAM[I] = C[I] * BET1;
    X[I] = D[I] * BET1;
    P[I] = C[NF];
    Q[I] = A[I] * BET1;
    for (I = NS + 1; I <= NF - 1; I++) {
        BET1 = 1.0 / (B[I] - A[I] * GAM[I - 1]);
        GAM[I] = C[I] * BET1;
        P[I] = -P[I - 1] * GAM[I - 1];
        Q[I] = -A[I] * BET1 * Q[I - 1];
        X[I] = (D[I] - A[I] * X[I - 1]) * BET1;
    }
    BET1 = 1.0 / (B[NF - 1] - A[NF - 1] * GAM[NF - 2]);
    P[NF - 1] = A[NF] - P[NF - 2] * GAM[NF - 2];
    Q[NF - 1] = (C[NF - 1] - A[NF - 1] * Q[NF - 2]) * BET1;
    X[NF] = D[NF];
    P[NF] = B[NF];
    for (I = NS; I <= NF - 1; I++) {
        X[NF] = X[NF] - P[I] * X[I];
        P[NF] = P[NF] - P[I] * Q[I];
    }
    X[NF] = X[NF] / P[NF];
    GAM[NF - 1] = 0.0;
    for (I = NF - 1; I >= NS; I--) X[I] = X[I] - GAM[I] * X[I + 1] - Q[I] * X[NF];
}

// TDMAI per line (compact3d.f:8630-8659): Thomas, reciprocal form.  D and X may alias.
void tdmai_line(int NS, int NF, const double *A, const double *B, const double *C,
                const double *D, double *X) {
    thread_local std::vector<double> s;
    s.resize((size_t)NF + 2);
    double *GAM = s.data();
    int J = NS;
    double BET = 1.0 / B[J];
    GAM[J] = C[J] * BET;
    X[J] = D[J] * BET;
    for (J = NS + 1; J <= NF; J++) {
        BET = 1.0 / (B[J] - A[J] * GAM[J - 1]);
        GAM[J] = C[J] * BET;
        X[J] = (D[J] - A[J] * X[J - 1]) * BET;
    }
    for (J = NF - 1; J >= NS; J--) X[J] = X[J] - X[J + 1] * GAM[J];
}

// TDMAP (compact3d.f:9444-9459): Thomas with divisions.  R and X may alias.
void tdmap(const double *A, const double *B, const double *C, const double *R, int N, double *X) {
    thread_local std::vector<double> s;
    s.resize((size_t)N + 2);
    double *GAM = s.data();
    double BET = B[1];
    X[1] = R[1] / BET;
    for (int J = 2; J <= N; J++) {
        GAM[J] = C[J - 1] / BET;
        BET = B[J] - A[J] * GAM[J];
        X[J] = (R[J] - A[J] * X[J - 1]) / BET;
    }
    for (int J = N - 1; J >= 1; J--) X[J] = X[J] - GAM[J + 1] * X[J + 1];
}

// Convenience wrappers for the constant-coefficient calls of CTDMA11/CTDMA33.
struct ConstLine {
    std::vector<double> A, B, C;
    void set(int n, double a, double b, double c) {
        A.assign(n + 1, a);
        B.assign(n + 1, b);
        C.assign(n + 1, c);
    }
};

// ----------------------------------------------------------------------------------
// FFT: mixed-radix complex DFT, FFTW conventions (forward exponent -1, unnormalised).
// ----------------------------------------------------------------------------------
void fft_rec(int n, int sign, const cplx *in, long istride, cplx *out, cplx *scratch) {
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = 0;
    for (int q : {4, 2, 3, 5, 7})
        if (n % q == 0) {
            p = q;
            break;
        }
    if (p == 0) {  // naive DFT for any other prime factor
        for (int k = 0; k < n; k++) {
            cplx acc(0.0, 0.0);
            for (int j = 0; j < n; j++) {
                double ang = sign * 2.0 * M_PI * (double)((long)j * k % n) / n;
                acc += in[j * istride] * cplx(std::cos(ang), std::sin(ang));
            }
            out[k] = acc;
        }
        return;
    }
    int m = n / p;
    // decimation in time: sub-sequences in[r + p*j], j=0..m-1
    for (int r = 0; r < p; r++) fft_rec(m, sign, in + r * istride, istride * p, scratch + r * m, out);
    for (int k = 0; k < m; k++) {
        cplx t[8];
        for (int r = 0; r < p; r++) {
            double ang = sign * 2.0 * M_PI * (double)(r * k) / n;
            t[r] = scratch[r * m + k] * cplx(std::cos(ang), std::sin(ang));
        }
        for (int s = 0; s < p; s++) {
            cplx acc(0.0, 0.0);
            for (int r = 0; r < p; r++) {
                double ang = sign * 2.0 * M_PI * (double)((r * s) % p) / p;
                acc += t[r] * cplx(std::cos(ang), std::sin(ang));
            }
            out[k + s * m] = acc;
        }
    }
}

void fft1d(int n, int sign, cplx *data, long stride) {
    thread_local std::vector<cplx> a, b, c;
    a.resize(n);
    b.resize(n);
    c.resize(n);
    for (int i = 0; i < n; i++) a[i] = data[i * stride];
    fft_rec(n, sign, a.data(), 1, b.data(), c.data());
    for (int i = 0; i < n; i++) data[i * stride] = b[i];
}

// 2-D DFT of a Fortran array COEF(n1,n3) (n1 fastest), as dfftw_plan_dft_2d(n1,n3).
void dft2d(int n1, int n3, cplx *a, int sign) {
    for (int k = 0; k < n3; k++) fft1d(n1, sign, a + (long)k * n1, 1);
    for (int i = 0; i < n1; i++) fft1d(n3, sign, a + i, n1);
}

// ----------------------------------------------------------------------------------
// Setup: INDICES (compact3d.f:446-494), INIWAVE (9182-9228), METRICPOISSON (9239-9263)
// ----------------------------------------------------------------------------------
void setup_indices(Orc &g) {
    int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    g.IPA.assign(g.N1 + 1, 0);
    g.IMA.assign(g.N1 + 1, 0);
    g.KPA.assign(g.N3 + 1, 0);
    g.KMA.assign(g.N3 + 1, 0);
    g.JPA.assign(g.N2 + 1, 0);
    g.JMU.assign(g.N2 + 1, 0);
    g.JMV.assign(g.N2 + 1, 0);
    g.FJPA.assign(g.N2 + 1, 0.0);
    g.FJMU.assign(g.N2 + 1, 0.0);
    g.FJMV.assign(g.N2 + 1, 0.0);
    for (int ic = 1; ic <= N1M; ic++) {
        g.IPA[ic] = ic + 1;
        g.IMA[ic] = ic - 1;
    }
    g.IPA[N1M] = 1;
    g.IMA[1] = N1M;
    for (int kc = 1; kc <= N3M; kc++) {
        g.KPA[kc] = kc + 1;
        g.KMA[kc] = kc - 1;
    }
    g.KPA[N3M] = 1;
    g.KMA[1] = N3M;
    for (int jc = 1; jc <= N2M; jc++) {
        g.JPA[jc] = jc + 1;
        g.JMU[jc] = jc - 1;
        g.JMV[jc] = jc - 1;
    }
    g.JPA[N2M] = N2M;
    g.JMU[1] = 1;
    g.JMV[2] = 2;
    for (int jc = 1; jc <= N2M; jc++) {
        g.FJPA[jc] = g.JPA[jc] - jc;
        g.FJMU[jc] = jc - g.JMU[jc];
        g.FJMV[jc] = jc - g.JMV[jc];
    }
}

void setup_wave(Orc &g) {
    int N1M = g.N1M, N3M = g.N3M;
    g.N3MH = N3M / 2 + 1;
    g.N1MH = N1M / 2 + 1;
    double PI = std::acos(-1.0);
    std::vector<double> ANI(g.N1 + 1), ANK(g.N3 + 1);
    g.AK1.assign(g.N1 + 1, 0.0);
    g.AK3.assign(g.N3MH + 1, 0.0);
    for (int I = 1; I <= N1M; I++) {
        int II = I;
        if (I > N1M / 2 + 1) II = I - N1M;
        ANI[I] = (II - 1) * 2.0 * PI;
    }
    for (int II = 1; II <= N1M; II++) {
        double cs = std::cos(ANI[II] / N1M);
        double den = (11.0 + cs);
        g.AK1[II] = 288.0 * g.DX1Q * (1.0 - cs) / (den * den);
    }
    for (int K = 1; K <= g.N3MH; K++) ANK[K] = (K - 1) * 2.0 * PI;
    for (int KK = 1; KK <= g.N3MH; KK++) {
        double cs = std::cos(ANK[KK] / N3M);
        double den = (11.0 + cs);
        g.AK3[KK] = 288.0 * g.DX3Q * (1.0 - cs) / (den * den);
    }
    // METRICPOISSON
    int N2M = g.N2M;
    g.PMJ.assign(g.N2 + 1, 0.0);
    g.PCJ.assign(g.N2 + 1, 0.0);
    g.PPJ.assign(g.N2 + 1, 0.0);
    const double *DY = g.DY.data(), *H = g.H.data();
    for (int JC = 1; JC <= N2M; JC++) {
        int JP = JC + 1;
        double FJUM = g.FJMU[JC], FJUP = g.FJPA[JC];
        g.PMJ[JC] = FJUM * FJUP * (1.0 / DY[JC] / H[JC]) + (1. - FJUP) * (1.0 / DY[N2M] / H[N2M]);
        g.PCJ[JC] = FJUM * FJUP * (-1.0 / DY[JC] / H[JC] - 1.0 / DY[JC] / H[JP]) +
                    (1. - FJUP) * (-1.0 / DY[N2M] / H[N2M]) + (1. - FJUM) * (-1.0 / DY[1] / H[2]);
        g.PPJ[JC] = FJUM * FJUP * (1.0 / DY[JC] / H[JP]) + (1. - FJUM) * (1.0 / DY[1] / H[2]);
    }
}

// ----------------------------------------------------------------------------------
// BCOND (compact3d.f:963-1001)
// ----------------------------------------------------------------------------------
void bcond(Orc &g, double *U, double *SGSVIS) {
    int N1M = g.N1M, N3M = g.N3M, N2 = g.N2, N2M = g.N2M;
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            g.UBC[g.iubc(I, K, 1, 1)] = 0.0;
            g.UBC[g.iubc(I, K, 2, 1)] = 0.0;
            g.UBC[g.iubc(I, K, 3, 1)] = 0.0;
            U[g.iuc(I, 0, K, 1)] = g.UBC[g.iubc(I, K, 1, 1)];
            U[g.iuc(I, 0, K, 2)] = g.UBC[g.iubc(I, K, 2, 1)];
            U[g.iuc(I, 0, K, 3)] = g.UBC[g.iubc(I, K, 3, 1)];
            g.UBC[g.iubc(I, K, 1, 2)] = U[g.iuc(I, N2M, K, 1)] * (2.0 - g.ALY);
            g.UBC[g.iubc(I, K, 2, 2)] = 0.0;
            g.UBC[g.iubc(I, K, 3, 2)] = U[g.iuc(I, N2M, K, 3)] * (2.0 - g.ALY);
            U[g.iuc(I, N2, K, 1)] = g.UBC[g.iubc(I, K, 1, 2)];
            U[g.iuc(I, N2, K, 2)] = g.UBC[g.iubc(I, K, 2, 2)];
            U[g.iuc(I, N2, K, 3)] = g.UBC[g.iubc(I, K, 3, 2)];
            // The reference tests an undeclared local FILES here (always zero-valued in
            // practice), so SGSVIS's wall planes are left to the SGS routines.
            (void)SGSVIS;
        }
}

// ----------------------------------------------------------------------------------
// RHS1 (compact3d.f:6063-6782), DNS terms.  The SGS-flux terms (6436-6763) add exact
// zeros when SGSVIS == 0, which is the case for FILES == 0 (GETUP zeroes SGSVIS).
// ----------------------------------------------------------------------------------
void sgs_rhs1(Orc &g, const double *U, double *HH, const double *SGSVIS);
void sgs_rhs2_vis22(Orc &g, const double *U, double *HH, const double *SGSVIS);
void sgs_rhs2(Orc &g, const double *U, double *HH, const double *SGSVIS);
void sgs_rhs3(Orc &g, const double *U, double *HH, const double *SGSVIS);

void rhs1(Orc &g, const double *U, const double *P, double *HH, const double *HH2,
          double *RUH1, double PRESG, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double RE = g.RE, DX1 = g.DX1, DX3 = g.DX3, DX1Q = g.DX1Q, DX3Q = g.DX3Q;
    const double *DY = g.DY.data(), *H = g.H.data(), *HP = g.HP.data(), *HC = g.HC.data(),
                 *HM = g.HM.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };

    // 10: viscous term (1/RE) d2u/dy2
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++) {
            int JP = J + 1, JM = J - 1;
            for (int I = 1; I <= N1M; I++) {
                double VISCOS = (1. / RE) * (HP[J] * u(I, JP, K, 1) - HC[J] * u(I, J, K, 1) +
                                             HM[J] * u(I, JM, K, 1));
                RUH1[g.iu(I, J, K)] = VISCOS;
            }
        }
    ConstLine L10x, L10z, L22x, L6x, L6z, L22z;
    L10x.set(N1M, 1.0, 10.0, 1.0);
    L10z.set(N3M, 1.0, 10.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);

    // 20: (1/RE) d2u/dx2
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 2; I <= N1M - 1; I++)
                D1[I] = 12. * DX1Q * (u(I - 1, J, K, 1) - 2. * u(I, J, K, 1) + u(I + 1, J, K, 1));
            D1[1] = 12. * DX1Q * (u(N1M, J, K, 1) - 2. * u(1, J, K, 1) + u(2, J, K, 1));
            D1[N1M] = 12. * DX1Q * (u(N1M - 1, J, K, 1) - 2. * u(N1M, J, K, 1) + u(1, J, K, 1));
            ctdma_bordered(N1M, L10x.A.data(), L10x.B.data(), L10x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) RUH1[g.iu(I, J, K)] = RUH1[g.iu(I, J, K)] + (1. / RE) * X1[I];
        }
    }
    // 30: (1/RE) d2u/dz2
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 2; K <= N3M - 1; K++)
                D3[K] = 12. * DX3Q * (u(I, J, K - 1, 1) - 2. * u(I, J, K, 1) + u(I, J, K + 1, 1));
            D3[1] = 12. * DX3Q * (u(I, J, N3M, 1) - 2. * u(I, J, 1, 1) + u(I, J, 2, 1));
            D3[N3M] = 12. * DX3Q * (u(I, J, N3M - 1, 1) - 2. * u(I, J, N3M, 1) + u(I, J, 1, 1));
            ctdma_bordered(N3M, L10z.A.data(), L10z.B.data(), L10z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) RUH1[g.iu(I, J, K)] = RUH1[g.iu(I, J, K)] + (1. / RE) * X3[K];
        }
    }
    // 40: pressure gradient
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 2; I <= N1M; I++)
                D1[I] = 24. * DX1 * (-P[g.ip(I - 1, J, K)] + P[g.ip(I, J, K)]);
            D1[1] = 24. * DX1 * (-P[g.ip(N1M, J, K)] + P[g.ip(1, J, K)]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) RUH1[g.iu(I, J, K)] = RUH1[g.iu(I, J, K)] - X1[I] - PRESG;
        }
    }
    // d(UV)/dy
    {
        std::vector<double> VV1((size_t)(N1M + 1) * (N2M + 2));
        auto vv1 = [&](int i, int j) -> double & { return VV1[i + (size_t)(N1M + 1) * j]; };
        for (int K = 1; K <= N3M; K++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4.0 * (u(I - 1, J, K, 2) + u(I, J, K, 2));
                D1[1] = 4.0 * (u(N1M, J, K, 2) + u(1, J, K, 2));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) vv1(I, J) = X1[I];
            }
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                int JP = J + 1, JM = J - 1;
                double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                for (int I = 1; I <= N1M; I++) {
                    double U2 = FJUP * 1.0 / H[JP] * (DY[J] / 2. * u(I, JP, K, 1) + DY[JP] / 2. * u(I, J, K, 1)) +
                                (1. - FJUP) * u(I, N2, K, 1);
                    double U1 = FJUM * 1.0 / H[J] * (DY[JM] / 2. * u(I, J, K, 1) + DY[J] / 2. * u(I, JM, K, 1)) +
                                (1. - FJUM) * u(I, 0, K, 1);
                    double V2 = (J == N2M) ? 0.0 : vv1(I, JP);
                    double V1 = (J == 1) ? 0.0 : vv1(I, J);
                    long id = g.iuc(I, J, K, 1);
                    HH[id] = HH[id] + 1. / DY[J] * (V2 * U2 - V1 * U1);
                }
            }
        }
    }
    // 50: d(UU)/dx
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1), UU1(N1M + 1), D11(N1M + 1), X11(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 1; I <= N1M - 1; I++) D1[I] = 4.0 * (u(I, J, K, 1) + u(I + 1, J, K, 1));
            D1[N1M] = 4.0 * (u(N1M, J, K, 1) + u(1, J, K, 1));
            ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) UU1[I] = X1[I];
            for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (UU1[I] * UU1[I] - UU1[I - 1] * UU1[I - 1]);
            D11[1] = 24. * DX1 * (UU1[1] * UU1[1] - UU1[N1M] * UU1[N1M]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
            for (int I = 1; I <= N1M; I++) {
                long id = g.iuc(I, J, K, 1);
                HH[id] = HH[id] + X11[I];
            }
        }
    }
    // 60: d(UW)/dz
    {
        std::vector<double> UU3((size_t)(N1M + 1) * (N3M + 1)), WW1((size_t)(N1M + 1) * (N3M + 1));
        auto uu3 = [&](int i, int k) -> double & { return UU3[i + (size_t)(N1M + 1) * k]; };
        auto ww1 = [&](int i, int k) -> double & { return WW1[i + (size_t)(N1M + 1) * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (u(I, J, K - 1, 1) + u(I, J, K, 1));
                D3[1] = 4. * (u(I, J, N3M, 1) + u(I, J, 1, 1));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) uu3(I, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (u(I - 1, J, K, 3) + u(I, J, K, 3));
                D1[1] = 4. * (u(N1M, J, K, 3) + u(1, J, K, 3));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) ww1(I, K) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D33(N3M + 1), X33(N3M + 1);
                for (int K = 1; K <= N3M - 1; K++)
                    D33[K] = 24. * DX3 * (-uu3(I, K) * ww1(I, K) + uu3(I, K + 1) * ww1(I, K + 1));
                D33[N3M] = 24. * DX3 * (-uu3(I, N3M) * ww1(I, N3M) + uu3(I, 1) * ww1(I, 1));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) {
                    long id = g.iuc(I, J, K, 1);
                    HH[id] = HH[id] + X33[K];
                }
            }
        }
    }
    // 61-73: SGS-flux terms (only when an SGS model is active; otherwise they add zeros)
    if (SGSVIS) sgs_rhs1(g, U, HH, SGSVIS);
    // 71/73: AB2 and wall-stress boundary term
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++) {
            double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
            for (int I = 1; I <= N1M; I++) {
                double BC_DOWN = -g.TAUW[g.itw(I, K, 1)] / DY[1] * g.IFWALL;
                double BC_UP = -g.TAUW[g.itw(I, K, 2)] / DY[N2M] * g.IFWALL * (g.ALY - 1.);
                double BC = (1. - FJUM) * BC_DOWN + (1. - FJUP) * BC_UP;
                long id = g.iu(I, J, K);
                RUH1[id] = RUH1[id] - 3. / 2. * HH[g.iuc(I, J, K, 1)] + 1. / 2. * HH2[g.iuc(I, J, K, 1)] + BC;
            }
        }
}

// RHS2 (compact3d.f:6784-7396), DNS terms.
void rhs2(Orc &g, const double *U, const double *P, double *HH, const double *HH2, double *RUH2,
          const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double RE = g.RE, DX1 = g.DX1, DX3 = g.DX3, DX1Q = g.DX1Q, DX3Q = g.DX3Q;
    const double *DY = g.DY.data(), *H = g.H.data(), *DYP = g.DYP.data(), *DYC = g.DYC.data(),
                 *DYM = g.DYM.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    ConstLine L10x, L10z, L22x, L6x, L6z, L22z;
    L10x.set(N1M, 1.0, 10.0, 1.0);
    L10z.set(N3M, 1.0, 10.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);
    // 10
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 2; J <= N2M; J++) {
            int JP = J + 1, JM = J - 1;
            for (int I = 1; I <= N1M; I++) {
                double VISCOS = (1. / RE) * (DYP[J] * u(I, JP, K, 2) - DYC[J] * u(I, J, K, 2) + DYM[J] * u(I, JM, K, 2));
                double PRESSG2 = (P[g.ip(I, J, K)] - P[g.ip(I, JM, K)]) / H[J];
                RUH2[g.iu(I, J, K)] = -PRESSG2 + VISCOS;
                double V2 = 0.5 * (u(I, JP, K, 2) + u(I, J, K, 2));
                double V1 = 0.5 * (u(I, J, K, 2) + u(I, JM, K, 2));
                long id = g.iuc(I, J, K, 2);
                HH[id] = HH[id] + 1. / H[J] * (V2 * V2 - V1 * V1);
            }
        }
    // 10 (continued): D(SGS*DV/DY)/DY, after the convection term of the same point
    if (SGSVIS) sgs_rhs2_vis22(g, U, HH, SGSVIS);
    // 20
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 2; J <= N2M; J++) {
            for (int I = 2; I <= N1M - 1; I++)
                D1[I] = 12. * DX1Q * (u(I - 1, J, K, 2) - 2. * u(I, J, K, 2) + u(I + 1, J, K, 2));
            D1[1] = 12. * DX1Q * (u(N1M, J, K, 2) - 2. * u(1, J, K, 2) + u(2, J, K, 2));
            D1[N1M] = 12. * DX1Q * (u(N1M - 1, J, K, 2) - 2. * u(N1M, J, K, 2) + u(1, J, K, 2));
            ctdma_bordered(N1M, L10x.A.data(), L10x.B.data(), L10x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) RUH2[g.iu(I, J, K)] = RUH2[g.iu(I, J, K)] + (1. / RE) * X1[I];
        }
    }
    // 30
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 2; J <= N2M; J++) {
            for (int K = 2; K <= N3M - 1; K++)
                D3[K] = 12. * DX3Q * (u(I, J, K - 1, 2) - 2. * u(I, J, K, 2) + u(I, J, K + 1, 2));
            D3[1] = 12. * DX3Q * (u(I, J, N3M, 2) - 2. * u(I, J, 1, 2) + u(I, J, 2, 2));
            D3[N3M] = 12. * DX3Q * (u(I, J, N3M - 1, 2) - 2. * u(I, J, N3M, 2) + u(I, J, 1, 2));
            ctdma_bordered(N3M, L10z.A.data(), L10z.B.data(), L10z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) RUH2[g.iu(I, J, K)] = RUH2[g.iu(I, J, K)] + (1. / RE) * X3[K];
        }
    }
    // 50: d(UV)/dx
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> VV1((size_t)(N1M + 2) * (N2M + 1)), UU2((size_t)(N1M + 2) * (N2M + 1));
        auto vv1 = [&](int i, int j) -> double & { return VV1[i + (size_t)(N1M + 2) * j]; };
        auto uu2 = [&](int i, int j) -> double & { return UU2[i + (size_t)(N1M + 2) * j]; };
#pragma omp parallel for
        for (int J = 2; J <= N2M; J++) {
            std::vector<double> D1(N1M + 1), X1(N1M + 1);
            for (int I = 2; I <= N1M; I++) D1[I] = 4. * (u(I - 1, J, K, 2) + u(I, J, K, 2));
            D1[1] = 4. * (u(N1M, J, K, 2) + u(1, J, K, 2));
            ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) vv1(I, J) = X1[I];
        }
#pragma omp parallel for
        for (int I = 1; I <= N1M; I++)
            for (int J = 2; J <= N2M; J++)
                uu2(I, J) = 1. / H[J] * (DY[J] / 2. * u(I, J - 1, K, 1) + DY[J - 1] / 2. * u(I, J, K, 1));
#pragma omp parallel for
        for (int J = 2; J <= N2M; J++) {
            std::vector<double> D11(N1M + 1), X11(N1M + 1);
            for (int I = 1; I <= N1M - 1; I++)
                D11[I] = 24. * DX1 * (-uu2(I, J) * vv1(I, J) + uu2(I + 1, J) * vv1(I + 1, J));
            D11[N1M] = 24. * DX1 * (-uu2(N1M, J) * vv1(N1M, J) + uu2(1, J) * vv1(1, J));
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
            for (int I = 1; I <= N1M; I++) {
                long id = g.iuc(I, J, K, 2);
                HH[id] = HH[id] + X11[I];
            }
        }
    }
    // 60: d(VW)/dz
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> VV3((size_t)(N2M + 1) * (N3M + 2)), WW2((size_t)(N2M + 1) * (N3M + 2));
        auto vv3 = [&](int j, int k) -> double & { return VV3[j + (size_t)(N2M + 1) * k]; };
        auto ww2 = [&](int j, int k) -> double & { return WW2[j + (size_t)(N2M + 1) * k]; };
#pragma omp parallel for
        for (int J = 2; J <= N2M; J++) {
            std::vector<double> D3(N3M + 1), X3(N3M + 1);
            for (int K = 2; K <= N3M; K++) D3[K] = 4. * (u(I, J, K - 1, 2) + u(I, J, K, 2));
            D3[1] = 4. * (u(I, J, N3M, 2) + u(I, J, 1, 2));
            ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) vv3(J, K) = X3[K];
        }
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++)
            for (int J = 2; J <= N2M; J++)
                ww2(J, K) = 1. / H[J] * (DY[J] / 2. * u(I, J - 1, K, 3) + DY[J - 1] / 2. * u(I, J, K, 3));
#pragma omp parallel for
        for (int J = 2; J <= N2M; J++) {
            std::vector<double> D33(N3M + 1), X33(N3M + 1);
            for (int K = 1; K <= N3M - 1; K++)
                D33[K] = 24. * DX3 * (-vv3(J, K) * ww2(J, K) + vv3(J, K + 1) * ww2(J, K + 1));
            D33[N3M] = 24. * DX3 * (-vv3(J, N3M) * ww2(J, N3M) + vv3(J, 1) * ww2(J, 1));
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
            for (int K = 1; K <= N3M; K++) {
                long id = g.iuc(I, J, K, 2);
                HH[id] = HH[id] + X33[K];
            }
        }
    }
    // SGS-flux terms, then 61-65: AB2
    if (SGSVIS) sgs_rhs2(g, U, HH, SGSVIS);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 2; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) {
                long id = g.iu(I, J, K);
                RUH2[id] = RUH2[id] - 3. / 2. * HH[g.iuc(I, J, K, 2)] + 1. / 2. * HH2[g.iuc(I, J, K, 2)];
            }
}

// RHS3 (compact3d.f:7399-8114), DNS terms.
void rhs3(Orc &g, const double *U, const double *P, double *HH, const double *HH2, double *RUH3,
          double PRESG3, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double RE = g.RE, DX1 = g.DX1, DX3 = g.DX3, DX1Q = g.DX1Q, DX3Q = g.DX3Q;
    const double *DY = g.DY.data(), *H = g.H.data(), *HP = g.HP.data(), *HC = g.HC.data(),
                 *HM = g.HM.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    ConstLine L10x, L10z, L22x, L6x, L6z, L22z;
    L10x.set(N1M, 1.0, 10.0, 1.0);
    L10z.set(N3M, 1.0, 10.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++) {
            int JP = J + 1, JM = J - 1;
            for (int I = 1; I <= N1M; I++) {
                double VISCOS = (1. / RE) * (HP[J] * u(I, JP, K, 3) - HC[J] * u(I, J, K, 3) + HM[J] * u(I, JM, K, 3));
                RUH3[g.iu(I, J, K)] = VISCOS;
            }
        }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 2; I <= N1M - 1; I++)
                D1[I] = 12. * DX1Q * (u(I - 1, J, K, 3) - 2. * u(I, J, K, 3) + u(I + 1, J, K, 3));
            D1[1] = 12. * DX1Q * (u(N1M, J, K, 3) - 2. * u(1, J, K, 3) + u(2, J, K, 3));
            D1[N1M] = 12. * DX1Q * (u(N1M - 1, J, K, 3) - 2. * u(N1M, J, K, 3) + u(1, J, K, 3));
            ctdma_bordered(N1M, L10x.A.data(), L10x.B.data(), L10x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) RUH3[g.iu(I, J, K)] = RUH3[g.iu(I, J, K)] + (1. / RE) * X1[I];
        }
    }
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 2; K <= N3M - 1; K++)
                D3[K] = 12. * DX3Q * (u(I, J, K - 1, 3) - 2. * u(I, J, K, 3) + u(I, J, K + 1, 3));
            D3[1] = 12. * DX3Q * (u(I, J, N3M, 3) - 2. * u(I, J, 1, 3) + u(I, J, 2, 3));
            D3[N3M] = 12. * DX3Q * (u(I, J, N3M - 1, 3) - 2. * u(I, J, N3M, 3) + u(I, J, 1, 3));
            ctdma_bordered(N3M, L10z.A.data(), L10z.B.data(), L10z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) RUH3[g.iu(I, J, K)] = RUH3[g.iu(I, J, K)] + (1. / RE) * X3[K];
        }
    }
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 2; K <= N3M; K++) D3[K] = 24. * DX3 * (-P[g.ip(I, J, K - 1)] + P[g.ip(I, J, K)]);
            D3[1] = 24. * DX3 * (-P[g.ip(I, J, N3M)] + P[g.ip(I, J, 1)]);
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) RUH3[g.iu(I, J, K)] = RUH3[g.iu(I, J, K)] - X3[K] - PRESG3;
        }
    }
    // d(WV)/dy
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> VV3((size_t)(N2M + 2) * (N3M + 1));
        auto vv3 = [&](int j, int k) -> double & { return VV3[j + (size_t)(N2M + 2) * k]; };
#pragma omp parallel for
        for (int J = 1; J <= N2M; J++) {
            std::vector<double> D3(N3M + 1), X3(N3M + 1);
            for (int K = 2; K <= N3M; K++) D3[K] = 4.0 * (u(I, J, K - 1, 2) + u(I, J, K, 2));
            D3[1] = 4.0 * (u(I, J, N3M, 2) + u(I, J, 1, 2));
            ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) vv3(J, K) = X3[K];
        }
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++)
            for (int J = 1; J <= N2M; J++) {
                int JP = J + 1, JM = J - 1;
                double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                double W2 = FJUP * 1.0 / H[JP] * (DY[JP] / 2. * u(I, J, K, 3) + DY[J] / 2. * u(I, JP, K, 3)) +
                            (1. - FJUP) * u(I, N2, K, 3);
                double W1 = FJUM * 1.0 / H[J] * (DY[J] / 2. * u(I, JM, K, 3) + DY[JM] / 2. * u(I, J, K, 3)) +
                            (1. - FJUM) * u(I, 0, K, 3);
                double V2 = (J == N2M) ? 0.0 : vv3(JP, K);
                double V1 = (J == 1) ? 0.0 : vv3(J, K);
                long id = g.iuc(I, J, K, 3);
                HH[id] = HH[id] + 1. / DY[J] * (V2 * W2 - V1 * W1);
            }
    }
    // 50: d(WW)/dz
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1), WW3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 1; K <= N3M - 1; K++) D3[K] = 4. * (u(I, J, K, 3) + u(I, J, K + 1, 3));
            D3[N3M] = 4. * (u(I, J, N3M, 3) + u(I, J, 1, 3));
            ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) WW3[K] = X3[K];
            for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (WW3[K] * WW3[K] - WW3[K - 1] * WW3[K - 1]);
            D33[1] = 24. * DX3 * (WW3[1] * WW3[1] - WW3[N3M] * WW3[N3M]);
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
            for (int K = 1; K <= N3M; K++) {
                long id = g.iuc(I, J, K, 3);
                HH[id] = HH[id] + X33[K];
            }
        }
    }
    // 60: d(UW)/dx
    {
        std::vector<double> UU3((size_t)(N1M + 2) * (N3M + 1)), WW1((size_t)(N1M + 2) * (N3M + 1));
        auto uu3 = [&](int i, int k) -> double & { return UU3[i + (size_t)(N1M + 2) * k]; };
        auto ww1 = [&](int i, int k) -> double & { return WW1[i + (size_t)(N1M + 2) * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (u(I, J, K - 1, 1) + u(I, J, K, 1));
                D3[1] = 4. * (u(I, J, N3M, 1) + u(I, J, 1, 1));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) uu3(I, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (u(I - 1, J, K, 3) + u(I, J, K, 3));
                D1[1] = 4. * (u(N1M, J, K, 3) + u(1, J, K, 3));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) ww1(I, K) = X1[I];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D11(N1M + 1), X11(N1M + 1);
                for (int I = 1; I <= N1M - 1; I++)
                    D11[I] = 24. * DX1 * (-uu3(I, K) * ww1(I, K) + uu3(I + 1, K) * ww1(I + 1, K));
                D11[N1M] = 24. * DX1 * (-uu3(N1M, K) * ww1(N1M, K) + uu3(1, K) * ww1(1, K));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) {
                    long id = g.iuc(I, J, K, 3);
                    HH[id] = HH[id] + X11[I];
                }
            }
        }
    }
    // SGS-flux terms
    if (SGSVIS) sgs_rhs3(g, U, HH, SGSVIS);
    // 71-73: AB2 and wall-stress boundary term
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++) {
            double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
            for (int I = 1; I <= N1M; I++) {
                double BC_DOWN = -g.TAUB[g.itw(I, K, 1)] / DY[1] * g.IFWALL;
                double BC_UP = -g.TAUB[g.itw(I, K, 2)] / DY[N2M] * g.IFWALL * (g.ALY - 1.);
                double BC = (1. - FJUM) * BC_DOWN + (1. - FJUP) * BC_UP;
                long id = g.iu(I, J, K);
                RUH3[id] = RUH3[id] - 3. / 2. * HH[g.iuc(I, J, K, 3)] + 1. / 2. * HH2[g.iuc(I, J, K, 3)] + BC;
            }
        }
}

// ----------------------------------------------------------------------------------
// SGS-flux terms of RHS1/2/3 (compact3d.f:6436-6770, 6857-6866 and 7088-7393,
// 7774-8111).  SGSVIS(0:M1,0:M2,0:M3) holds the eddy viscosity at cell centres; its
// wall planes J=0 and J=N2 are zero (GETUP zeroes them and no routine on the path
// assigns them).  Work arrays the reference indexes one past their declared extent
// (SGSVIS1(I,N2), UU12(I,N2), SGSVISW2(N2,K), VV32(N2,K) at J=N2M, and index 0 at J=1)
// enter only multiplied by FJPA/FJMU = 0 or by a zero wall viscosity; they are zero here.
// ----------------------------------------------------------------------------------
void sgs_rhs1(Orc &g, const double *U, double *HH, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double DX1 = g.DX1, DX3 = g.DX3, ALY = g.ALY, IFWALL = g.IFWALL;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    auto sv = [&](int i, int j, int k) { return SGSVIS[g.iu(i, j, k)]; };
    ConstLine L6x, L6z, L22x, L22z;
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    // 61: D(SGS*(DU/DX))/DX
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D11(N1M + 1), X11(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 1; I <= N1M - 1; I++) D11[I] = 24. * DX1 * (u(I + 1, J, K, 1) - u(I, J, K, 1));
            D11[N1M] = 24. * DX1 * (u(1, J, K, 1) - u(N1M, J, K, 1));
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
            for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (sv(I, J, K) * X11[I] - sv(I - 1, J, K) * X11[I - 1]);
            D11[1] = 24. * DX1 * (sv(1, J, K) * X11[1] - sv(N1M, J, K) * X11[N1M]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
            for (int I = 1; I <= N1M; I++) HH[g.iuc(I, J, K, 1)] = HH[g.iuc(I, J, K, 1)] - 2. * X11[I];
        }
    }
    // 65-67: D(SGS*(DU/DZ))/DZ
    {
        std::vector<double> S2((size_t)(N1M + 1) * (N3M + 1));
        auto s2 = [&](int i, int k) -> double & { return S2[i + (size_t)(N1M + 1) * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) s2(I, K) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (s2(I, K) + s2(I, K - 1));
                D3[1] = 4. * (s2(I, 1) + s2(I, N3M));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (u(I, J, K, 1) - u(I, J, K - 1, 1));
                D33[1] = 24. * DX3 * (u(I, J, 1, 1) - u(I, J, N3M, 1));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M - 1; K++) D33[K] = 24. * DX3 * (X33[K + 1] * X3[K + 1] - X33[K] * X3[K]);
                D33[N3M] = 24. * DX3 * (X33[1] * X3[1] - X33[N3M] * X3[N3M]);
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) HH[g.iuc(I, J, K, 1)] = HH[g.iuc(I, J, K, 1)] - X33[K];
            }
        }
    }
    // 62-64: D(SGS*(DU/DY))/DY and 68-70: D(SGS*(DV/DX))/DY
    {
        std::vector<double> S1((size_t)(N1M + 1) * (N2 + 1), 0.0), S12((size_t)(N1M + 1) * (N2 + 1), 0.0),
            UU12((size_t)(N1M + 1) * (N2 + 1), 0.0);
        auto s1 = [&](int i, int j) -> double & { return S1[i + (size_t)(N1M + 1) * j]; };
        auto s12 = [&](int i, int j) -> double & { return S12[i + (size_t)(N1M + 1) * j]; };
        auto uu12 = [&](int i, int j) -> double & { return UU12[i + (size_t)(N1M + 1) * j]; };
        for (int K = 1; K <= N3M; K++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) s1(I, J) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                const int IM = g.IMA[I];
                for (int J = 1; J <= N2M; J++) {
                    const int JP = J + 1, JM = J - 1;
                    const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                    double SGSJ2 = FJUP * 1. / H[JP] * (DY[J] / 2. * s1(I, JP) + DY[JP] / 2. * s1(I, J)) +
                                   (1. - FJUP) * 0.5 * (sv(I, N2, K) + sv(IM, N2, K));
                    double SGSJ1 = FJUM * 1. / H[J] * (DY[JM] / 2. * s1(I, J) + DY[J] / 2. * s1(I, JM)) +
                                   (1. - FJUM) * 0.5 * (sv(I, 0, K) + sv(IM, 0, K));
                    double UU22 = (u(I, JP, K, 1) - u(I, J, K, 1)) / H[JP];
                    double UU11 = (u(I, J, K, 1) - u(I, JM, K, 1)) / H[J];
                    double SGSDUY = 1. / DY[J] * ((1. - IFWALL * (1. - FJUP) * (ALY - 1.)) * SGSJ2 * UU22 -
                                                  (1. - IFWALL * (1. - FJUM)) * SGSJ1 * UU11);
                    HH[g.iuc(I, J, K, 1)] = HH[g.iuc(I, J, K, 1)] - SGSDUY;
                }
            }
        }
        for (int K = 1; K <= N3M; K++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1), D11(N1M + 1), X11(N1M + 1);
                for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (u(I, J, K, 2) - u(I - 1, J, K, 2));
                D11[1] = 24. * DX1 * (u(1, J, K, 2) - u(N1M, J, K, 2));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) uu12(I, J) = X11[I];
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) s12(I, J) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                const int IM = g.IMA[I];
                for (int J = 1; J <= N2M; J++) {
                    const int JP = J + 1, JM = J - 1;
                    const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                    double SGSJ2 = FJUP * 1.0 / H[JP] * (DY[J] / 2. * s12(I, JP) + DY[JP] / 2. * s12(I, J)) +
                                   (1. - FJUP) * 0.5 * (sv(I, N2, K) + sv(IM, N2, K));
                    double SGSJ1 = FJUM * 1.0 / H[J] * (DY[JM] / 2. * s12(I, J) + DY[J] / 2. * s12(I, JM)) +
                                   (1. - FJUM) * 0.5 * (sv(I, 0, K) + sv(IM, 0, K));
                    double SGSDUXY = 1.0 / DY[J] * ((1. - IFWALL * (1. - FJUP) * (ALY - 1.)) * SGSJ2 * uu12(I, JP) -
                                                    (1. - IFWALL * (1. - FJUM)) * SGSJ1 * uu12(I, J));
                    HH[g.iuc(I, J, K, 1)] = HH[g.iuc(I, J, K, 1)] - SGSDUXY;
                }
            }
        }
    }
    // 71-73: D(SGS*(DW/DX))/DZ (the AB2 update and wall term follow in rhs1)
    {
        std::vector<double> S13((size_t)(N1M + 1) * (N3M + 1)), WW13((size_t)(N1M + 1) * (N3M + 1));
        auto s13 = [&](int i, int k) -> double & { return S13[i + (size_t)(N1M + 1) * k]; };
        auto ww13 = [&](int i, int k) -> double & { return WW13[i + (size_t)(N1M + 1) * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1), D11(N1M + 1), X11(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) s13(I, K) = X1[I];
                for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (u(I, J, K, 3) - u(I - 1, J, K, 3));
                D11[1] = 24. * DX1 * (u(1, J, K, 3) - u(N1M, J, K, 3));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) ww13(I, K) = X11[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (s13(I, K) + s13(I, K - 1));
                D3[1] = 4. * (s13(I, 1) + s13(I, N3M));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M - 1; K++) D33[K] = 24. * DX3 * (ww13(I, K + 1) * X3[K + 1] - ww13(I, K) * X3[K]);
                D33[N3M] = 24. * DX3 * (ww13(I, 1) * X3[1] - ww13(I, N3M) * X3[N3M]);
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) HH[g.iuc(I, J, K, 1)] = HH[g.iuc(I, J, K, 1)] - X33[K];
            }
        }
    }
}

// RHS2 loop 10, second half (compact3d.f:6857-6866): D(SGS*DV/DY)/DY at the v faces.
void sgs_rhs2_vis22(Orc &g, const double *U, double *HH, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 2; J <= N2M; J++) {
            const int JP = J + 1, JM = J - 1;
            for (int I = 1; I <= N1M; I++) {
                double SGSJ2 = SGSVIS[g.iu(I, J, K)];
                double SGSJ1 = SGSVIS[g.iu(I, JM, K)];
                double V2 = 1. / DY[J] * (u(I, JP, K, 2) - u(I, J, K, 2));
                double V1 = 1. / DY[JM] * (u(I, J, K, 2) - u(I, JM, K, 2));
                double VIS22 = 1.0 / H[J] * (SGSJ2 * V2 - SGSJ1 * V1);
                HH[g.iuc(I, J, K, 2)] = HH[g.iuc(I, J, K, 2)] - 2. * VIS22;
            }
        }
}

// RHS2 (compact3d.f:7088-7393): the four cross-derivative SGS fluxes at the v faces.
void sgs_rhs2(Orc &g, const double *U, double *HH, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double DX1 = g.DX1, DX3 = g.DX3;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    auto sv = [&](int i, int j, int k) { return SGSVIS[g.iu(i, j, k)]; };
    ConstLine L6x, L6z, L22x, L22z;
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    const size_t PX = (size_t)(N1M + 2), PJ = (size_t)(N2M + 2);
    // D(SGS*(DU/DY))/DX
    {
        std::vector<double> SV1(PX * PJ), SV21(PX * PJ), VV21(PX * PJ);
        auto sv1 = [&](int i, int j) -> double & { return SV1[i + PX * j]; };
        auto sv21 = [&](int i, int j) -> double & { return SV21[i + PX * j]; };
        auto vv21 = [&](int i, int j) -> double & { return VV21[i + PX * j]; };
        for (int K = 1; K <= N3M; K++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) sv1(I, J) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++)
                for (int J = 2; J <= N2M; J++) {
                    sv21(I, J) = 1. / H[J] * (DY[J - 1] / 2. * sv1(I, J) + DY[J] / 2. * sv1(I, J - 1));
                    vv21(I, J) = 1. / H[J] * (u(I, J, K, 1) - u(I, J - 1, K, 1));
                }
#pragma omp parallel for
            for (int J = 2; J <= N2M; J++) {
                std::vector<double> D11(N1M + 1), X11(N1M + 1);
                for (int I = 1; I <= N1M - 1; I++)
                    D11[I] = 24. * DX1 * (sv21(I + 1, J) * vv21(I + 1, J) - sv21(I, J) * vv21(I, J));
                D11[N1M] = 24. * DX1 * (sv21(1, J) * vv21(1, J) - sv21(N1M, J) * vv21(N1M, J));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) HH[g.iuc(I, J, K, 2)] = HH[g.iuc(I, J, K, 2)] - X11[I];
            }
        }
    }
    // D(SGS*(DW/DY))/DZ
    {
        const size_t PK = (size_t)(N3M + 2);
        std::vector<double> S3(PJ * PK), SV23(PJ * PK), VV32(PJ * PK);
        auto s3 = [&](int j, int k) -> double & { return S3[j + PJ * k]; };
        auto sv23 = [&](int j, int k) -> double & { return SV23[j + PJ * k]; };
        auto vv32 = [&](int j, int k) -> double & { return VV32[j + PJ * k]; };
        for (int I = 1; I <= N1M; I++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K - 1) + sv(I, J, K));
                D3[1] = 4. * (sv(I, J, N3M) + sv(I, J, 1));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) s3(J, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++)
                for (int J = 2; J <= N2M; J++) {
                    sv23(J, K) = 1. / H[J] * (DY[J] / 2. * s3(J - 1, K) + DY[J - 1] / 2. * s3(J, K));
                    vv32(J, K) = 1. / H[J] * (u(I, J, K, 3) - u(I, J - 1, K, 3));
                }
#pragma omp parallel for
            for (int J = 2; J <= N2M; J++) {
                std::vector<double> D33(N3M + 1), X33(N3M + 1);
                for (int K = 1; K <= N3M - 1; K++)
                    D33[K] = 24. * DX3 * (sv23(J, K + 1) * vv32(J, K + 1) - sv23(J, K) * vv32(J, K));
                D33[N3M] = 24. * DX3 * (sv23(J, 1) * vv32(J, 1) - sv23(J, N3M) * vv32(J, N3M));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) HH[g.iuc(I, J, K, 2)] = HH[g.iuc(I, J, K, 2)] - X33[K];
            }
        }
    }
    // D(SGS*(DV/DZ))/DZ
    {
        const size_t PK = (size_t)(N3M + 2);
        std::vector<double> SV3(PJ * PK), VV23(PJ * PK), SV32(PJ * PK);
        auto sv3 = [&](int j, int k) -> double & { return SV3[j + PJ * k]; };
        auto vv23 = [&](int j, int k) -> double & { return VV23[j + PJ * k]; };
        auto sv32 = [&](int j, int k) -> double & { return SV32[j + PJ * k]; };
        for (int I = 1; I <= N1M; I++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K - 1) + sv(I, J, K));
                D3[1] = 4. * (sv(I, J, N3M) + sv(I, J, 1));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) sv3(J, K) = X3[K];
                for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (u(I, J, K, 2) - u(I, J, K - 1, 2));
                D33[1] = 24. * DX3 * (u(I, J, 1, 2) - u(I, J, N3M, 2));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) vv23(J, K) = X33[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++)
                for (int J = 2; J <= N2M; J++)
                    sv32(J, K) = 1. / H[J] * (DY[J] / 2. * sv3(J - 1, K) + DY[J - 1] / 2. * sv3(J, K));
#pragma omp parallel for
            for (int J = 2; J <= N2M; J++) {
                std::vector<double> D33(N3M + 1), X33(N3M + 1);
                for (int K = 1; K <= N3M - 1; K++)
                    D33[K] = 24. * DX3 * (sv32(J, K + 1) * vv23(J, K + 1) - sv32(J, K) * vv23(J, K));
                D33[N3M] = 24. * DX3 * (sv32(J, 1) * vv23(J, 1) - sv32(J, N3M) * vv23(J, N3M));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) HH[g.iuc(I, J, K, 2)] = HH[g.iuc(I, J, K, 2)] - X33[K];
            }
        }
    }
    // D(SGS*(DV/DX))/DX
    {
        std::vector<double> VV12(PX * PJ), SV12(PX * PJ), SV22(PX * PJ);
        auto vv12 = [&](int i, int j) -> double & { return VV12[i + PX * j]; };
        auto sv12 = [&](int i, int j) -> double & { return SV12[i + PX * j]; };
        auto sv22 = [&](int i, int j) -> double & { return SV22[i + PX * j]; };
        for (int K = 1; K <= N3M; K++) {
#pragma omp parallel for
            for (int J = 2; J <= N2M; J++) {
                std::vector<double> D11(N1M + 1), X11(N1M + 1);
                for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (u(I, J, K, 2) - u(I - 1, J, K, 2));
                D11[1] = 24. * DX1 * (u(1, J, K, 2) - u(N1M, J, K, 2));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) vv12(I, J) = X11[I];
            }
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sv(I, J, K) + sv(I - 1, J, K));
                D1[1] = 4. * (sv(1, J, K) + sv(N1M, J, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M; I++) sv12(I, J) = X1[I];
            }
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++)
                for (int J = 2; J <= N2M; J++)
                    sv22(I, J) = 1.0 / H[J] * (DY[J - 1] / 2. * sv12(I, J) + DY[J] / 2. * sv12(I, J - 1));
#pragma omp parallel for
            for (int J = 2; J <= N2M; J++) {
                std::vector<double> D11(N1M + 1), X11(N1M + 1);
                for (int I = 1; I <= N1M - 1; I++)
                    D11[I] = 24. * DX1 * (sv22(I + 1, J) * vv12(I + 1, J) - sv22(I, J) * vv12(I, J));
                D11[N1M] = 24. * DX1 * (sv22(1, J) * vv12(1, J) - sv22(N1M, J) * vv12(N1M, J));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) HH[g.iuc(I, J, K, 2)] = HH[g.iuc(I, J, K, 2)] - X11[I];
            }
        }
    }
}

// RHS3 (compact3d.f:7774-8111): SGS fluxes at the w faces.
void sgs_rhs3(Orc &g, const double *U, double *HH, const double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double DX1 = g.DX1, DX3 = g.DX3, ALY = g.ALY, IFWALL = g.IFWALL;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    auto sv = [&](int i, int j, int k) { return SGSVIS[g.iu(i, j, k)]; };
    ConstLine L6x, L6z, L22x, L22z;
    L6x.set(N1M, 1.0, 6.0, 1.0);
    L6z.set(N3M, 1.0, 6.0, 1.0);
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
    const size_t PX = (size_t)(N1M + 2), PK = (size_t)(N3M + 2), PJ = (size_t)(N2 + 2);
    // 61-63: D(SGS*(DW/DX))/DX
    {
        std::vector<double> SW3(PX * PK);
        auto sw3 = [&](int i, int k) -> double & { return SW3[i + PX * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K - 1) + sv(I, J, K));
                D3[1] = 4. * (sv(I, J, N3M) + sv(I, J, 1));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) sw3(I, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1), D11(N1M + 1), X11(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (sw3(I - 1, K) + sw3(I, K));
                D1[1] = 4. * (sw3(N1M, K) + sw3(1, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 2; I <= N1M; I++) D11[I] = 24. * DX1 * (u(I, J, K, 3) - u(I - 1, J, K, 3));
                D11[1] = 24. * DX1 * (u(1, J, K, 3) - u(N1M, J, K, 3));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M - 1; I++) D11[I] = 24. * DX1 * (X1[I + 1] * X11[I + 1] - X1[I] * X11[I]);
                D11[N1M] = 24. * DX1 * (X1[1] * X11[1] - X1[N1M] * X11[N1M]);
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) HH[g.iuc(I, J, K, 3)] = HH[g.iuc(I, J, K, 3)] - X11[I];
            }
        }
    }
    // 64-66: D(SGS*(DW/DY))/DY
    {
        std::vector<double> SW2(PJ * PK, 0.0);
        auto sw2 = [&](int j, int k) -> double & { return SW2[j + PJ * k]; };
        for (int I = 1; I <= N1M; I++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1);
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K) + sv(I, J, K - 1));
                D3[1] = 4. * (sv(I, J, 1) + sv(I, J, N3M));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) sw2(J, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                const int KM = g.KMA[K];
                for (int J = 1; J <= N2M; J++) {
                    const int JP = J + 1, JM = J - 1;
                    const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                    double WW22 = 1. / H[JP] * (u(I, JP, K, 3) - u(I, J, K, 3));
                    double WW11 = 1. / H[J] * (u(I, J, K, 3) - u(I, JM, K, 3));
                    double SGSJ1 = FJUM * 1. / H[J] * (DY[JM] / 2. * sw2(J, K) + DY[J] / 2. * sw2(JM, K)) +
                                   (1. - FJUM) * 0.5 * (sv(I, 0, K) + sv(I, 0, KM));
                    double SGSJ2 = FJUP * 1.0 / H[JP] * (DY[J] / 2. * sw2(JP, K) + DY[JP] / 2. * sw2(J, K)) +
                                   (1. - FJUP) * 0.5 * (sv(I, N2, K) + sv(I, N2, KM));
                    double SGSDWY = 1. / DY[J] * ((1. - IFWALL * (1. - FJUP) * (ALY - 1.)) * SGSJ2 * WW22 -
                                                  (1. - IFWALL * (1. - FJUM)) * SGSJ1 * WW11);
                    HH[g.iuc(I, J, K, 3)] = HH[g.iuc(I, J, K, 3)] - SGSDWY;
                }
            }
        }
    }
    // 67: D(SGS*(DW/DZ))/DZ
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D33(N3M + 1), X33(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 1; K <= N3M - 1; K++) D33[K] = 24. * DX3 * (u(I, J, K + 1, 3) - u(I, J, K, 3));
            D33[N3M] = 24. * DX3 * (u(I, J, 1, 3) - u(I, J, N3M, 3));
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
            for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (X33[K] * sv(I, J, K) - X33[K - 1] * sv(I, J, K - 1));
            D33[1] = 24. * DX3 * (X33[1] * sv(I, J, 1) - X33[N3M] * sv(I, J, N3M));
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
            for (int K = 1; K <= N3M; K++) HH[g.iuc(I, J, K, 3)] = HH[g.iuc(I, J, K, 3)] - 2. * X33[K];
        }
    }
    // 68-70: D(SGS*(DU/DZ))/DX
    {
        std::vector<double> UU31(PX * PK), S31(PX * PK);
        auto uu31 = [&](int i, int k) -> double & { return UU31[i + PX * k]; };
        auto s31 = [&](int i, int k) -> double & { return S31[i + PX * k]; };
        for (int J = 1; J <= N2M; J++) {
#pragma omp parallel for
            for (int I = 1; I <= N1M; I++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
                for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (u(I, J, K, 1) - u(I, J, K - 1, 1));
                D33[1] = 24. * DX3 * (u(I, J, 1, 1) - u(I, J, N3M, 1));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) uu31(I, K) = X33[K];
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K) + sv(I, J, K - 1));
                D3[1] = 4. * (sv(I, J, 1) + sv(I, J, N3M));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) s31(I, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                std::vector<double> D1(N1M + 1), X1(N1M + 1), D11(N1M + 1), X11(N1M + 1);
                for (int I = 2; I <= N1M; I++) D1[I] = 4. * (s31(I, K) + s31(I - 1, K));
                D1[1] = 4. * (s31(1, K) + s31(N1M, K));
                ctdma_bordered(N1M, L6x.A.data(), L6x.B.data(), L6x.C.data(), D1.data(), X1.data());
                for (int I = 1; I <= N1M - 1; I++) D11[I] = 24. * DX1 * (X1[I + 1] * uu31(I + 1, K) - X1[I] * uu31(I, K));
                D11[N1M] = 24. * DX1 * (X1[1] * uu31(1, K) - X1[N1M] * uu31(N1M, K));
                ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D11.data(), X11.data());
                for (int I = 1; I <= N1M; I++) HH[g.iuc(I, J, K, 3)] = HH[g.iuc(I, J, K, 3)] - X11[I];
            }
        }
    }
    // 71-73: D(SGS*(DV/DZ))/DY (the AB2 update and wall term follow in rhs3)
    {
        std::vector<double> VV32(PJ * PK, 0.0), S32(PJ * PK, 0.0);
        auto vv32 = [&](int j, int k) -> double & { return VV32[j + PJ * k]; };
        auto s32 = [&](int j, int k) -> double & { return S32[j + PJ * k]; };
        for (int I = 1; I <= N1M; I++) {
#pragma omp parallel for
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> D3(N3M + 1), X3(N3M + 1), D33(N3M + 1), X33(N3M + 1);
                for (int K = 2; K <= N3M; K++) D33[K] = 24. * DX3 * (u(I, J, K, 2) - u(I, J, K - 1, 2));
                D33[1] = 24. * DX3 * (u(I, J, 1, 2) - u(I, J, N3M, 2));
                ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D33.data(), X33.data());
                for (int K = 1; K <= N3M; K++) vv32(J, K) = X33[K];
                for (int K = 2; K <= N3M; K++) D3[K] = 4. * (sv(I, J, K) + sv(I, J, K - 1));
                D3[1] = 4. * (sv(I, J, 1) + sv(I, J, N3M));
                ctdma_bordered(N3M, L6z.A.data(), L6z.B.data(), L6z.C.data(), D3.data(), X3.data());
                for (int K = 1; K <= N3M; K++) s32(J, K) = X3[K];
            }
#pragma omp parallel for
            for (int K = 1; K <= N3M; K++) {
                const int KM = g.KMA[K];
                for (int J = 1; J <= N2M; J++) {
                    const int JP = J + 1, JM = J - 1;
                    const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
                    double SGSJ2 = FJUP * 1.0 / H[JP] * (DY[J] / 2. * s32(JP, K) + DY[JP] / 2. * s32(J, K)) +
                                   (1. - FJUP) * 0.5 * (sv(I, N2, K) + sv(I, N2, KM));
                    double SGSJ1 = FJUM * 1.0 / H[J] * (DY[JM] / 2. * s32(J, K) + DY[J] / 2. * s32(JM, K)) +
                                   (1. - FJUM) * 0.5 * (sv(I, 0, K) + sv(I, 0, KM));
                    double SGSDVY = 1.0 / DY[J] * ((1. - IFWALL * (1. - FJUP) * (ALY - 1.)) * SGSJ2 * vv32(JP, K) -
                                                   (1. - IFWALL * (1. - FJUM)) * SGSJ1 * vv32(J, K));
                    HH[g.iuc(I, J, K, 3)] = HH[g.iuc(I, J, K, 3)] - SGSDVY;
                }
            }
        }
    }
}

// ----------------------------------------------------------------------------------
// SGS models and the wall model (compact3d.f:1250-1488, 5190-5228, 5558-5689,
// 2319-2493, 11077-11143).
// ----------------------------------------------------------------------------------

// STRAIN (compact3d.f:5558-5689): strain-rate tensor at the cell centres of plane J,
// SR(I,K,1..6) = S11, S12, S13, S22, S23, S33, stored SR[(I-1) + N1M*((K-1) + N3M*(c-1))].
void strain(Orc &g, const double *U, std::vector<double> &SR, int J) {
    const int N1M = g.N1M, N3M = g.N3M, N2 = g.N2, N2M = g.N2M;
    const double DX1 = g.DX1, DX3 = g.DX3;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    auto sr = [&](int i, int k, int c) -> double & { return SR[(i - 1) + (size_t)N1M * ((k - 1) + (size_t)N3M * (c - 1))]; };
    const int JP = J + 1, JM = J - 1;
    const int FJUM = (int)g.FJMU[J], FJUP = (int)g.FJPA[J];
    const bool wm = g.WMODEL != 0;
    for (int K = 1; K <= N3M; K++) {
        const int KP = g.KPA[K], KM = g.KMA[K];
        for (int I = 1; I <= N1M; I++) {
            const int IP = g.IPA[I], IM = g.IMA[I];
            double U2 = u(IP, J, K, 1), U1 = u(I, J, K, 1);
            sr(I, K, 1) = DX1 * (U2 - U1);
            double UJP = 0.5 * (u(I, JP, K, 1) + u(IP, JP, K, 1));
            double UJC = 0.5 * (u(I, J, K, 1) + u(IP, J, K, 1));
            double UJM = 0.5 * (u(I, JM, K, 1) + u(IP, JM, K, 1));
            if (!wm) {
                U2 = FJUP * 1.0 / H[JP] * (DY[J] / 2.0 * UJP + DY[JP] / 2.0 * UJC) +
                     (1. - FJUP) * 0.5 * (u(I, N2, K, 1) + u(IP, N2, K, 1));
                U1 = FJUM * 1.0 / H[J] * (DY[J] / 2.0 * UJM + DY[JM] / 2.0 * UJC) +
                     (1. - FJUM) * 0.5 * (u(I, 0, K, 1) + u(IP, 0, K, 1));
            } else {
                U2 = FJUP * 1.0 / H[JP] * (DY[J] / 2.0 * UJP + DY[JP] / 2.0 * UJC) + (1. - FJUP) * UJC;
                U1 = FJUM * 1.0 / H[J] * (DY[J] / 2.0 * UJM + DY[JM] / 2.0 * UJC) + (1. - FJUM) * UJC;
            }
            double VIP = 0.5 * (u(IP, J, K, 2) + u(IP, JP, K, 2));
            double VIC = 0.5 * (u(I, J, K, 2) + u(I, JP, K, 2));
            double VIM = 0.5 * (u(IM, J, K, 2) + u(IM, JP, K, 2));
            double V2 = 0.5 * (VIP + VIC), V1 = 0.5 * (VIM + VIC);
            if (!wm || (J != 1 && J != N2M)) sr(I, K, 2) = 0.5 * (DX1 * (V2 - V1) + 1.0 / DY[J] * (U2 - U1));
            else sr(I, K, 2) = 0.5 * (DX1 * (V2 - V1) + 2.0 / DY[J] * (U2 - U1));
            double UKP = 0.5 * (u(I, J, KP, 1) + u(IP, J, KP, 1));
            double UKC = 0.5 * (u(I, J, K, 1) + u(IP, J, K, 1));
            double UKM = 0.5 * (u(I, J, KM, 1) + u(IP, J, KM, 1));
            U2 = 0.5 * (UKP + UKC);
            U1 = 0.5 * (UKM + UKC);
            double WIP = 0.5 * (u(IP, J, K, 3) + u(IP, J, KP, 3));
            double WIC = 0.5 * (u(I, J, K, 3) + u(I, J, KP, 3));
            double WIM = 0.5 * (u(IM, J, K, 3) + u(IM, J, KP, 3));
            double W2 = 0.5 * (WIP + WIC), W1 = 0.5 * (WIM + WIC);
            sr(I, K, 3) = 0.5 * (DX1 * (W2 - W1) + DX3 * (U2 - U1));
            V2 = u(I, JP, K, 2);
            V1 = u(I, J, K, 2);
            sr(I, K, 4) = 1.0 / DY[J] * (V2 - V1);
            double WJP = 0.5 * (u(I, JP, K, 3) + u(I, JP, KP, 3));
            double WJC = 0.5 * (u(I, J, K, 3) + u(I, J, KP, 3));
            double WJM = 0.5 * (u(I, JM, K, 3) + u(I, JM, KP, 3));
            if (!wm) {
                W2 = FJUP * 1.0 / H[JP] * (DY[J] / 2.0 * WJP + DY[JP] / 2.0 * WJC) +
                     (1. - FJUP) * 0.5 * (u(I, N2, K, 3) + u(I, N2, KP, 3));
                W1 = FJUM * 1.0 / H[J] * (DY[J] / 2.0 * WJM + DY[JM] / 2.0 * WJC) +
                     (1. - FJUM) * 0.5 * (u(I, 0, K, 3) + u(I, 0, KP, 3));
            } else {
                W2 = FJUP * 1.0 / H[JP] * (DY[J] / 2.0 * WJP + DY[JP] / 2.0 * WJC) + (1. - FJUP) * WJC;
                W1 = FJUM * 1.0 / H[J] * (DY[J] / 2.0 * WJM + DY[JM] / 2.0 * WJC) + (1. - FJUM) * WJC;
            }
            double VKP = 0.5 * (u(I, J, KP, 2) + u(I, JP, KP, 2));
            double VKC = 0.5 * (u(I, J, K, 2) + u(I, JP, K, 2));
            double VKM = 0.5 * (u(I, J, KM, 2) + u(I, JP, KM, 2));
            V2 = 0.5 * (VKP + VKC);
            V1 = 0.5 * (VKM + VKC);
            if (!wm || (J != 1 && J != N2M)) sr(I, K, 5) = 0.5 * (1.0 / DY[J] * (W2 - W1) + DX3 * (V2 - V1));
            else sr(I, K, 5) = 0.5 * (2.0 / DY[J] * (W2 - W1) + DX3 * (V2 - V1));
            W2 = u(I, J, KP, 3);
            W1 = u(I, J, K, 3);
            sr(I, K, 6) = DX3 * (W2 - W1);
        }
    }
}

// FILTER (compact3d.f:5190-5228): Simpson (1,4,1)/6 in x, then in z, for N components.
void filter(Orc &g, std::vector<double> &F, int N) {
    const int N1M = g.N1M, N3M = g.N3M;
    std::vector<double> T((size_t)N1M * N3M);
    for (int L = 1; L <= N; L++) {
        double *f = F.data() + (size_t)N1M * N3M * (L - 1);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I], IM = g.IMA[I];
                double FM = f[(IM - 1) + (size_t)N1M * (K - 1)], FC = f[(I - 1) + (size_t)N1M * (K - 1)],
                       FP = f[(IP - 1) + (size_t)N1M * (K - 1)];
                T[(I - 1) + (size_t)N1M * (K - 1)] = (FM + 4.0 * FC + FP) / 6.0;
            }
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K], KM = g.KMA[K];
            for (int I = 1; I <= N1M; I++) {
                double FM = T[(I - 1) + (size_t)N1M * (KM - 1)], FC = T[(I - 1) + (size_t)N1M * (K - 1)],
                       FP = T[(I - 1) + (size_t)N1M * (KP - 1)];
                f[(I - 1) + (size_t)N1M * (K - 1)] = (FM + 4.0 * FC + FP) / 6.0;
            }
        }
    }
}

inline double sumsq6(const double s1, const double s2, const double s3, const double s4, const double s5,
                     const double s6) {
    return 2. * s2 * s2 + s1 * s1 + 2. * s3 * s3 + s4 * s4 + 2. * s5 * s5 + s6 * s6;
}

// SGSDY (compact3d.f:1250-1400): dynamic Smagorinsky, plane-averaged coefficient, clipped.
void sgsdy(Orc &g, const double *U, double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const size_t NP = (size_t)N1M * N3M;
    const double NXZ = 1.0 / (double)(N1M * N3M), RENINV = 1. / g.RE;
    std::vector<double> SR(NP * 6), COM(NP * 6), UC(NP * 3);
    for (int J = 1; J <= N2M; J++) {
        const double DXYZ = 1.0 / g.DX1 * g.DY[J] / g.DX3;
        strain(g, U, SR, J);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double DELTA2 = std::pow(DXYZ, 2. / 3.);
                double SUMSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                double ABSSR = std::sqrt(2. * SUMSR);
                SGSVIS[g.iu(I, J, K)] = ABSSR;
                double DELABS = DELTA2 * ABSSR;
                for (int c = 0; c < 6; c++) COM[q + c * NP] = DELABS * SR[q + c * NP];
            }
        filter(g, COM, 6);
        filter(g, SR, 6);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double SUMFSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                double ABSFSR = std::sqrt(2. * SUMFSR);
                double FDXYZ = 4.0 * std::pow(DXYZ, 2. / 3.);
                double FDABS = FDXYZ * ABSFSR;
                for (int c = 0; c < 6; c++) SR[q + c * NP] = FDABS * SR[q + c * NP] - COM[q + c * NP];
            }
        const int JP = J + 1;
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double a = (U[g.iuc(I, J, K, 1)] + U[g.iuc(IP, J, K, 1)]) * 0.5;
                double b = (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
                double c = (U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, KP, 3)]) * 0.5;
                UC[q] = a;
                UC[q + NP] = b;
                UC[q + 2 * NP] = c;
                COM[q] = a * a;
                COM[q + NP] = a * b;
                COM[q + 2 * NP] = a * c;
                COM[q + 3 * NP] = b * b;
                COM[q + 4 * NP] = b * c;
                COM[q + 5 * NP] = c * c;
            }
        }
        filter(g, UC, 3);
        filter(g, COM, 6);
        // 40: the plane sums (an OpenMP reduction in the reference; fixed order here)
        double SUMNUM = 0., SUMDEN = 0.;
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                const double u1 = UC[q], u2 = UC[q + NP], u3 = UC[q + 2 * NP];
                double XL11 = COM[q] - u1 * u1, XL12 = COM[q + NP] - u1 * u2, XL13 = COM[q + 2 * NP] - u1 * u3;
                double XL22 = COM[q + 3 * NP] - u2 * u2, XL23 = COM[q + 4 * NP] - u2 * u3,
                       XL33 = COM[q + 5 * NP] - u3 * u3;
                const double *m = &SR[q];
                double SQMM = sumsq6(m[0], m[NP], m[2 * NP], m[3 * NP], m[4 * NP], m[5 * NP]);
                double SQLM = 2. * XL12 * m[NP] + XL11 * m[0] + 2. * XL13 * m[2 * NP] + XL22 * m[3 * NP] +
                              2. * XL23 * m[4 * NP] + XL33 * m[5 * NP];
                SUMDEN = SUMDEN + SQMM;
                SUMNUM = SUMNUM + SQLM;
            }
        SUMNUM = SUMNUM * NXZ;
        SUMDEN = SUMDEN * NXZ;
        g.SMAGC[J] = -0.5 * SUMNUM / SUMDEN;
        const double CS_DAMPING = 1.0;
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                double TURBV = g.SMAGC[J] * std::pow(DXYZ, 2. / 3.) * SGSVIS[g.iu(I, J, K)];
                double s = std::max(TURBV, -RENINV);
                SGSVIS[g.iu(I, J, K)] = s * CS_DAMPING;
            }
    }
}

// SGSCS (compact3d.f:1413-1488): Smagorinsky with Van Driest damping, C_s = 0.1.
void sgscs(Orc &g, const double *U, double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const size_t NP = (size_t)N1M * N3M;
    const double RENINV = 1. / g.RE;
    std::vector<double> SR(NP * 6);
    const double UTAU = std::sqrt(std::sqrt(g.WSM[0] * g.WSM[0] + g.WSM[2] * g.WSM[2]));
    for (int J = 1; J <= N2M; J++) {
        const double DXYZ = 1.0 / g.DX1 * g.DY[J] / g.DX3;
        strain(g, U, SR, J);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double SUMSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                SGSVIS[g.iu(I, J, K)] = std::sqrt(2. * SUMSR);
            }
        double CS = 0.1;
        const double A_plus = 26.0;
        const double Y_plus = (g.Y[J] + g.DY[J] * 0.5) * UTAU * g.RE;
        CS = CS * (1 - std::exp(-Y_plus / A_plus));
        g.SMAGC[J] = CS * CS;
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                double TURBV = g.SMAGC[J] * std::pow(DXYZ, 2. / 3.) * SGSVIS[g.iu(I, J, K)];
                SGSVIS[g.iu(I, J, K)] = std::max(TURBV, -RENINV);
            }
    }
}

// FILTER4 (compact3d.f:5481-5545): five-point (1,4,2,4,1)/12 in x, then in z, periodic.
void filter4(Orc &g, std::vector<double> &F, int N) {
    const int N1M = g.N1M, N3M = g.N3M;
    std::vector<double> T((size_t)N1M * N3M);
    auto wrap = [](int i, int n) { return i < 1 ? i + n : (i > n ? i - n : i); };
    for (int L = 1; L <= N; L++) {
        double *f = F.data() + (size_t)N1M * N3M * (L - 1);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                auto at = [&](int i) { return f[(wrap(i, N1M) - 1) + (size_t)N1M * (K - 1)]; };
                T[(I - 1) + (size_t)N1M * (K - 1)] = (at(I - 2) + 4.0 * at(I - 1) + 2.0 * at(I) + 4.0 * at(I + 1) + at(I + 2)) / 12.0;
            }
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                auto at = [&](int k) { return T[(I - 1) + (size_t)N1M * (wrap(k, N3M) - 1)]; };
                f[(I - 1) + (size_t)N1M * (K - 1)] = (at(K - 2) + 4.0 * at(K - 1) + 2.0 * at(K) + 4.0 * at(K + 1) + at(K + 2)) / 12.0;
            }
    }
}

// CHHQR (compact3d.f:11571-11676): eigenvalues (WR, WI) of the N x N upper Hessenberg
// matrix A (column-major, A(i,j) = A[(i-1) + N (j-1)], overwritten) by the Francis
// double-shift QR iteration.  The active block is rows L..M; a subdiagonal entry with
// |A(L,L-1)| <= EPS (|A(L-1,L-1)| + |A(L,L)|) splits it; a 1x1 block gives a real root, a
// 2x2 block a pair from its quadratic; otherwise one double-shift sweep of 3x3
// Householder reflections chases the bulge from L to M.  At most 60 sweeps per
// deflation; returns 0 on that failure (roots not yet found are left as they were).
int chhqr(double *A, int N, double *WR, double *WI, double EPS) {
    auto a = [&](int i, int j) -> double & { return A[(i - 1) + (size_t)N * (j - 1)]; };
    int M = N, IT = 0;
    while (M > 0) {
        int L = M;
        while (L > 1 && std::fabs(a(L, L - 1)) > EPS * (std::fabs(a(L - 1, L - 1)) + std::fabs(a(L, L)))) L = L - 1;
        if (L == M) {
            WR[M - 1] = a(M, M);
            WI[M - 1] = 0.0;
            M = M - 1;
            IT = 0;
            continue;
        }
        if (L == M - 1) {
            const double B = -(a(M, M) + a(M - 1, M - 1));
            const double C = a(M, M) * a(M - 1, M - 1) - a(M, M - 1) * a(M - 1, M);
            const double W = B * B - 4 * C;
            const double Y = std::sqrt(std::fabs(W));
            if (W > 0.0) {
                const double XY = B < 0.0 ? -1.0 : 1.0;
                WR[M - 1] = (-B - XY * Y) / 2.0;
                WR[M - 2] = C / WR[M - 1];
                WI[M - 1] = 0.0;
                WI[M - 2] = 0.0;
            } else {
                WR[M - 1] = -B / 2.0;
                WR[M - 2] = WR[M - 1];
                WI[M - 1] = Y / 2.0;
                WI[M - 2] = -WI[M - 1];
            }
            M = M - 2;
            IT = 0;
            continue;
        }
        if (IT >= 60) return 0;
        IT = IT + 1;
        for (int J = L + 2; J <= M; J++) a(J, J - 2) = 0.0;
        for (int J = L + 3; J <= M; J++) a(J, J - 3) = 0.0;
        for (int K = L; K <= M - 1; K++) {
            double P, Q, R;
            if (K != L) {
                P = a(K, K - 1);
                Q = a(K + 1, K - 1);
                R = K != M - 1 ? a(K + 2, K - 1) : 0.0;
            } else {   // first column of (H - s1)(H - s2) from the trailing 2x2 block
                const double X = a(M, M) + a(M - 1, M - 1);
                const double Y = a(M - 1, M - 1) * a(M, M) - a(M - 1, M) * a(M, M - 1);
                P = a(L, L) * (a(L, L) - X) + a(L, L + 1) * a(L + 1, L) + Y;
                Q = a(L + 1, L) * (a(L, L) + a(L + 1, L + 1) - X);
                R = a(L + 1, L) * a(L + 2, L + 1);
            }
            if (std::fabs(P) + std::fabs(Q) + std::fabs(R) == 0.0) continue;
            const double XY = P < 0.0 ? -1.0 : 1.0;
            const double S = XY * std::sqrt(P * P + Q * Q + R * R);
            if (K != L) a(K, K - 1) = -S;
            const double E = -Q / S, F = -R / S, X = -P / S;
            const double Y = -X - F * R / (P + S);
            const double G = E * R / (P + S);
            const double Z = -X - E * Q / (P + S);
            for (int J = K; J <= M; J++) {   // rows K..K+2 from the left
                double p = X * a(K, J) + E * a(K + 1, J);
                double q = E * a(K, J) + Y * a(K + 1, J);
                double r = F * a(K, J) + G * a(K + 1, J);
                if (K != M - 1) {
                    p = p + F * a(K + 2, J);
                    q = q + G * a(K + 2, J);
                    r = r + Z * a(K + 2, J);
                    a(K + 2, J) = r;
                }
                a(K + 1, J) = q;
                a(K, J) = p;
            }
            const int JJ = K + 3 >= M ? M : K + 3;
            for (int I = L; I <= JJ; I++) {   // columns K..K+2 from the right
                double p = X * a(I, K) + E * a(I, K + 1);
                double q = E * a(I, K) + Y * a(I, K + 1);
                double r = F * a(I, K) + G * a(I, K + 1);
                if (K != M - 1) {
                    p = p + F * a(I, K + 2);
                    q = q + G * a(I, K + 2);
                    r = r + Z * a(I, K + 2);
                    a(I, K + 2) = r;
                }
                a(I, K + 1) = q;
                a(I, K) = p;
            }
        }
    }
    return 1;
}

// DQRRT (compact3d.f:11548-11569): the roots of x^N + PA(1) x^(N-1) + ... + PA(N) as the
// eigenvalues of the companion matrix (first row -PA, ones on the subdiagonal); BETA is
// the largest real part in (0, 2), 0 if there is none (complex roots count by their real
// part, as in the reference's scan).
double dqrrt(const double *PA, int N, double EPS) {
    std::vector<double> B((size_t)N * N, 0.0), WR(N, 0.0), WI(N, 0.0);
    for (int J = 1; J <= N; J++) B[(size_t)N * (J - 1)] = -PA[J - 1];
    for (int I = 1; I <= N - 1; I++) B[I + (size_t)N * (I - 1)] = 1.0;
    chhqr(B.data(), N, WR.data(), WI.data(), EPS);
    double BETA = 0.;
    for (int J = 0; J < N; J++)
        if (WR[J] > BETA && WR[J] < 2.0) BETA = WR[J];
    return BETA;
}

// COEFFICIENT (compact3d.f:2079-2095): the quintic of the scale-dependent model,
// PA(1..5) of x^5 + PA(1) x^4 + ... + PA(5), from the plane sums of the two test filters.
void coefficient(double A1, double B1, double C1, double D1, double E1, double A2, double B2, double C2,
                 double D2, double E2, double *PA) {
    PA[4] = (B2 * C1 - B1 * C2) / (A1 * D2);
    PA[3] = (A1 * C2 - B2 * E1) / (A1 * D2);
    PA[2] = (B2 * D1 + B1 * E2 - A2 * C1) / (A1 * D2);
    PA[1] = (A2 * E1 - A1 * E2) / (A1 * D2);
    PA[0] = -(A2 * D1 + B1 * D2) / (A1 * D2);
}

// SGSSD (compact3d.f:1502-1948): the scale-dependent dynamic model.  Per plane, the
// Germano identity at the test filters 2 DELTA (FILTER) and 4 DELTA (FILTER4) gives the
// sums A..E of each; the scale-dependence BETA solves the quintic of COEFFICIENT (DQRRT,
// EPS 1.0E-5); the coefficient is then the dynamic one at 2 DELTA with
// M_ij = 4 DELTA^(2/3) BETA |S~| S~_ij - (DELTA^(2/3) |S| S_ij)~ (the unclipped BETA; the
// reference clips only the copy BETAZ it writes to a file every 100 steps).
void sgssd(Orc &g, const double *U, double *SGSVIS) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const size_t NP = (size_t)N1M * N3M;
    const double NXZ = 1.0 / (double)(N1M * N3M), RENINV = 1. / g.RE;
    std::vector<double> SR(NP * 6), COM(NP * 6), COM1(NP * 6), SR1(NP * 6), UC(NP * 3);
    g.BETA.assign((size_t)g.N2 + 1, 0.0);
    for (int J = 1; J <= N2M; J++) {
        const double DXYZ = 1.0 / g.DX1 * g.DY[J] / g.DX3;
        // one test filter (FILTER or FILTER4) of the raw quantities, then its five sums
        auto level = [&](bool four, double sa, double sd, double se, double &A, double &B, double &C, double &D, double &E) {
            strain(g, U, SR, J);
            for (size_t q = 0; q < NP; q++) {
                double DELTA2 = std::pow(DXYZ, 2. / 3.);
                double SUMSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                double ABSSR = std::sqrt(2. * SUMSR);
                double DELABS = DELTA2 * ABSSR;
                for (int c = 0; c < 6; c++) COM1[q + c * NP] = DELABS * SR[q + c * NP];
            }
            if (four) {
                filter4(g, COM1, 6);
                filter4(g, SR, 6);
            } else {
                filter(g, COM1, 6);
                filter(g, SR, 6);
            }
            for (size_t q = 0; q < NP; q++) {
                double SUMFSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                double ABSFSR = std::sqrt(2. * SUMFSR);
                double FDXYZ = std::pow(DXYZ, 2. / 3.);
                double FDABS = FDXYZ * ABSFSR;
                for (int c = 0; c < 6; c++) SR1[q + c * NP] = FDABS * SR[q + c * NP];
            }
            const int JP = J + 1;
            for (int K = 1; K <= N3M; K++) {
                const int KP = g.KPA[K];
                for (int I = 1; I <= N1M; I++) {
                    const int IP = g.IPA[I];
                    const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                    double a = (U[g.iuc(I, J, K, 1)] + U[g.iuc(IP, J, K, 1)]) * 0.5;
                    double b = (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
                    double c = (U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, KP, 3)]) * 0.5;
                    UC[q] = a;
                    UC[q + NP] = b;
                    UC[q + 2 * NP] = c;
                    COM[q] = a * a;
                    COM[q + NP] = a * b;
                    COM[q + 2 * NP] = a * c;
                    COM[q + 3 * NP] = b * b;
                    COM[q + 4 * NP] = b * c;
                    COM[q + 5 * NP] = c * c;
                }
            }
            if (four) {
                filter4(g, UC, 3);
                filter4(g, COM, 6);
            } else {
                filter(g, UC, 3);
                filter(g, COM, 6);
            }
            A = 0.0, B = 0.0, C = 0.0, D = 0.0, E = 0.0;
            for (size_t q = 0; q < NP; q++) {
                const double u1 = UC[q], u2 = UC[q + NP], u3 = UC[q + 2 * NP];
                const double X11 = COM[q] - u1 * u1, X12 = COM[q + NP] - u1 * u2, X13 = COM[q + 2 * NP] - u1 * u3;
                const double X22 = COM[q + 3 * NP] - u2 * u2, X23 = COM[q + 4 * NP] - u2 * u3,
                             X33 = COM[q + 5 * NP] - u3 * u3;
                const double *s = &SR1[q], *m = &COM1[q];
                A = A + 2. * X12 * s[NP] + X11 * s[0] + 2. * X13 * s[2 * NP] + X22 * s[3 * NP] + 2. * X23 * s[4 * NP] + X33 * s[5 * NP];
                B = B + 2. * X12 * m[NP] + X11 * m[0] + 2. * X13 * m[2 * NP] + X22 * m[3 * NP] + 2. * X23 * m[4 * NP] + X33 * m[5 * NP];
            }
            for (size_t q = 0; q < NP; q++) {
                const double *s = &SR1[q], *m = &COM1[q];
                C = C + 2. * m[NP] * m[NP] + m[0] * m[0] + 2. * m[2 * NP] * m[2 * NP] + m[3 * NP] * m[3 * NP] +
                    2. * m[4 * NP] * m[4 * NP] + m[5 * NP] * m[5 * NP];
                D = D + 2. * s[NP] * s[NP] + s[0] * s[0] + 2. * s[2 * NP] * s[2 * NP] + s[3 * NP] * s[3 * NP] +
                    2. * s[4 * NP] * s[4 * NP] + s[5 * NP] * s[5 * NP];
                E = E + 2. * s[NP] * m[NP] + s[0] * m[0] + 2. * s[2 * NP] * m[2 * NP] + s[3 * NP] * m[3 * NP] +
                    2. * s[4 * NP] * m[4 * NP] + s[5 * NP] * m[5 * NP];
            }
            A = sa * A * NXZ;
            B = -2.0 * B * NXZ;
            C = 4.0 * C * NXZ;
            D = sd * D * NXZ;
            E = se * E * NXZ;
        };
        double A1, B1, C1, D1, E1, A2, B2, C2, D2, E2, PA[5];
        level(false, -8.0, 64.0, 32.0, A1, B1, C1, D1, E1);
        level(true, -32.0, 1024.0, 128.0, A2, B2, C2, D2, E2);
        coefficient(A1, B1, C1, D1, E1, A2, B2, C2, D2, E2, PA);
        const double BETA = dqrrt(PA, 5, 1.0E-5);
        g.BETA[J] = BETA;
        // the coefficient at 2 DELTA with the scale-dependent M_ij
        strain(g, U, SR, J);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double DELTA2 = std::pow(DXYZ, 2. / 3.);
                double SUMSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
                double ABSSR = std::sqrt(2. * SUMSR);
                SGSVIS[g.iu(I, J, K)] = ABSSR;
                double DELABS = DELTA2 * ABSSR;
                for (int c = 0; c < 6; c++) COM[q + c * NP] = DELABS * SR[q + c * NP];
            }
        filter(g, COM, 6);
        filter(g, SR, 6);
        for (size_t q = 0; q < NP; q++) {
            double SUMFSR = sumsq6(SR[q], SR[q + NP], SR[q + 2 * NP], SR[q + 3 * NP], SR[q + 4 * NP], SR[q + 5 * NP]);
            double ABSFSR = std::sqrt(2. * SUMFSR);
            double FDXYZ = 4.0 * std::pow(DXYZ, 2. / 3.) * BETA;
            double FDABS = FDXYZ * ABSFSR;
            for (int c = 0; c < 6; c++) SR[q + c * NP] = FDABS * SR[q + c * NP] - COM[q + c * NP];
        }
        const int JP = J + 1;
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                const size_t q = (I - 1) + (size_t)N1M * (K - 1);
                double a = (U[g.iuc(I, J, K, 1)] + U[g.iuc(IP, J, K, 1)]) * 0.5;
                double b = (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
                double c = (U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, KP, 3)]) * 0.5;
                UC[q] = a;
                UC[q + NP] = b;
                UC[q + 2 * NP] = c;
                COM[q] = a * a;
                COM[q + NP] = a * b;
                COM[q + 2 * NP] = a * c;
                COM[q + 3 * NP] = b * b;
                COM[q + 4 * NP] = b * c;
                COM[q + 5 * NP] = c * c;
            }
        }
        filter(g, UC, 3);
        filter(g, COM, 6);
        double SUMNUM = 0., SUMDEN = 0.;
        for (size_t q = 0; q < NP; q++) {
            const double u1 = UC[q], u2 = UC[q + NP], u3 = UC[q + 2 * NP];
            double XL11 = COM[q] - u1 * u1, XL12 = COM[q + NP] - u1 * u2, XL13 = COM[q + 2 * NP] - u1 * u3;
            double XL22 = COM[q + 3 * NP] - u2 * u2, XL23 = COM[q + 4 * NP] - u2 * u3, XL33 = COM[q + 5 * NP] - u3 * u3;
            const double *m = &SR[q];
            double SQMM = sumsq6(m[0], m[NP], m[2 * NP], m[3 * NP], m[4 * NP], m[5 * NP]);
            double SQLM = 2. * XL12 * m[NP] + XL11 * m[0] + 2. * XL13 * m[2 * NP] + XL22 * m[3 * NP] +
                          2. * XL23 * m[4 * NP] + XL33 * m[5 * NP];
            SUMDEN = SUMDEN + SQMM;
            SUMNUM = SUMNUM + SQLM;
        }
        SUMNUM = SUMNUM * NXZ;
        SUMDEN = SUMDEN * NXZ;
        g.SMAGC[J] = -0.5 * SUMNUM / SUMDEN;
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                double TURBV = g.SMAGC[J] * std::pow(DXYZ, 2. / 3.) * SGSVIS[g.iu(I, J, K)];
                SGSVIS[g.iu(I, J, K)] = std::max(TURBV, -RENINV) * 1.0;
            }
    }
}

// WALLSS (compact3d.f:11077-11143): plane-mean wall shear into wsm[0..2] (/WSMEM/ WSM),
// one running sum in K, I order.  The reference adds the top wall's u-shear WST(I,K,1)
// to all three components (scaled by ALY-1).
void wallss_common(Orc &g, const double *U, double *wsm) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    double W1 = 0.0, W2 = 0.0, W3 = 0.0;
    const double *DY = g.DY.data();
    double NXZ = 1.0 / (double)(N1M * N3M);
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    for (int K = 1; K <= N3M; K++) {
        int KP = g.KPA[K];
        for (int I = 1; I <= N1M; I++) {
            int IP = g.IPA[I];
            double UHC = 0.5 * (u(I, 1, K, 1) + u(IP, 1, K, 1));
            double UHW = 0.5 * (u(I, 0, K, 1) + u(IP, 0, K, 1));
            double VHC = u(I, 2, K, 2);
            double VHW = u(I, 1, K, 2);
            double WHC = 0.5 * (u(I, 1, K, 3) + u(I, 1, KP, 3));
            double WHW = 0.5 * (u(I, 0, K, 3) + u(I, 0, KP, 3));
            double WSB1 = (UHC - UHW) / (DY[1] * 0.5);
            double WSB2 = (VHC - VHW) / DY[1];
            double WSB3 = (WHC - WHW) / (DY[1] * 0.5);
            UHC = 0.5 * (u(I, N2M, K, 1) + u(IP, N2M, K, 1));
            UHW = 0.5 * (u(I, N2, K, 1) + u(IP, N2, K, 1));
            double WST1 = (UHC - UHW) / (DY[N2M] * 0.5);
            W1 = W1 + WSB1 + WST1 * (g.ALY - 1.0);
            W2 = W2 + WSB2 + WST1 * (g.ALY - 1.0);
            W3 = W3 + WSB3 + WST1 * (g.ALY - 1.0);
        }
    }
    wsm[0] = W1 * NXZ / g.RE / g.ALY;
    wsm[1] = W2 * NXZ / g.RE / g.ALY;
    wsm[2] = W3 * NXZ / g.RE / g.ALY;
}

// WALLMODEL_INSTANT (compact3d.f:2319-2493): per wall point, u_tau from the log law at
// the third cell centre by damped Newton iterations; bottom wall only (the top-wall
// stresses TAUW(.,.,2), TAUB(.,.,2) are left as they are).  The reference iterates
// without a cap; here the cap `wall_iter_cap` makes a non-converging point an error.
// WALLMODEL_ROUGH (WMODEL 1 with Y0 = Y(0) != 0, compact3d.f:2496-2558): the rough-wall
// log law u_tau = KAPA U / log(DELTAP / Y0) on the bottom wall, KAPA = 0.41.
int wallmodel_rough(Orc &g, const double *U) {
    const int N1M = g.N1M, N3M = g.N3M;
    const double KAPA = 0.41, Y0 = g.Y[0];
    const double DELTAP = g.DY[1] + g.DY[2] + g.DY[3] / 2.0;
    double WSM1 = 0.0;
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            const double u = U[g.iuc(I, 3, K, 1)], w = U[g.iuc(I, 3, K, 3)];
            const double U_ave = std::sqrt(std::pow(u, 2.) + std::pow(w, 2.));
            const double TAUW1 = std::pow(KAPA / std::log(DELTAP / Y0) * U_ave, 2.0);
            WSM1 = WSM1 + TAUW1;
            g.TAUW[g.itw(I, K, 1)] = TAUW1 * u / U_ave;
            g.TAUB[g.itw(I, K, 1)] = TAUW1 * w / U_ave;
        }
    g.WSM[0] = WSM1 / (double)(N1M * N3M);
    g.TAOW = g.WSM[0];
    return 0;
}

int wallmodel_instant(Orc &g, const double *U) {
    const int N1M = g.N1M, N3M = g.N3M;
    const double KAPA = 0.41, B = 5.2;
    const double DELTAP = g.DY[1] + g.DY[2] + g.DY[3] / 2.0;
    const double RE = g.RE;
    int bad = 0;
    double wsum = 0.0;
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            const double u3 = U[g.iuc(I, 3, K, 1)], w3 = U[g.iuc(I, 3, K, 3)];
            double U_ave = std::sqrt(u3 * u3 + w3 * w3);
            double U_tau1 = 1.0, U_tau2 = 0.000001, FUtau3 = 1.0, FUtau1 = 0.1, LAMBDA = 1.0;
            int it = 0;
            while (std::fabs(U_tau2 - U_tau1) > 1.0E-6) {
                if (++it > g.wall_iter_cap) {
                    bad = 1;
                    break;
                }
                U_tau1 = U_tau2;
                FUtau1 = U_ave / U_tau1 - std::log(U_tau1 * DELTAP * RE) / KAPA - B;
                double FUtau2 = -U_ave / (U_tau1 * U_tau1) - 1. / KAPA / U_tau1;
                U_tau2 = U_tau1 - LAMBDA * FUtau1 / FUtau2;
                FUtau3 = U_ave / U_tau2 - std::log(U_tau2 * DELTAP * RE) / KAPA - B;
                if (std::fabs(FUtau3) > std::fabs(FUtau1)) LAMBDA = 0.5 * LAMBDA;
            }
            double TAUW1 = U_tau1 * U_tau1;
            wsum = wsum + TAUW1;
            g.TAUW[g.itw(I, K, 1)] = TAUW1 * u3 / U_ave;
            g.TAUB[g.itw(I, K, 1)] = TAUW1 * w3 / U_ave;
        }
    g.WSM[0] = wsum / (double)(N1M * N3M);
    g.TAOW = g.WSM[0];
    return bad ? C3D_ENOTCONV : 0;
}

// WALLMODEL_WERNER (compact3d.f:4815-4958): Werner-Wengle power law at the first cell
// centre of both walls, TAUWE(I,K,1..4) at the cell centres, then averaged to the stress
// points; WSM(1) = plane mean of the bottom u-stress.  The reference takes the x neighbour
// with the z loop variable (IP = IPA(J) and IP = IMA(J), J the z index; F:4852, 4881, 4924),
// which this restatement keeps; the INDX arrays have N1M entries, so it needs N3M <= N1M.
int wallmodel_werner(Orc &g, const double *U) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double B = 0.1428571429, AB1 = 7.202125274, AB3 = 69.74057973, AB4 = 0.1376936317, AB5 = 1.75;
    const double RE = g.RE;
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    std::vector<double> TAUWE((size_t)(N1M + 1) * (N3M + 1) * 4, 0.0);
    auto te = [&](int i, int k, int q) -> double & { return TAUWE[((size_t)q * (N3M + 1) + k) * (N1M + 1) + i]; };
    const double TEMP = std::sqrt(std::fabs(g.WSM[0])) / 11.81;   // WSM(1) of the step before
    const double VCASE = AB3 * TEMP;
    for (int wall = 0; wall < 2; ++wall) {
        const int JW = wall == 0 ? 1 : N2M;
        const double DELTAP = g.DY[JW];
        for (int J = 1; J <= N3M; J++) {
            const int KP = g.KPA[J];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[J];
                const double U1 = 0.5 * (u(I, JW, J, 1) + u(IP, JW, J, 1));
                const double U2 = 0.5 * (u(I, JW, J, 3) + u(I, JW, KP, 3));
                const double VELOCP = std::sqrt(U1 * U1 + U2 * U2);
                double TAUW1;
                if (VELOCP <= VCASE) {
                    TAUW1 = 2. * VELOCP / DELTAP / RE;
                } else {
                    TAUW1 = AB1 * std::pow(1.0 / DELTAP / RE, 1. + B);
                    TAUW1 = TAUW1 + AB4 * std::pow(1.0 / DELTAP / RE, B) * VELOCP;
                    TAUW1 = std::pow(TAUW1, AB5);
                }
                te(I, J, 2 * wall) = TAUW1 * (U1 / VELOCP);
                te(I, J, 2 * wall + 1) = TAUW1 * (U2 / VELOCP);
            }
        }
    }
    for (int J = 1; J <= N3M; J++) {
        const int KP = g.KMA[J];
        for (int I = 1; I <= N1M; I++) {
            const int IP = g.IMA[J];
            g.TAUW[g.itw(I, J, 1)] = 0.5 * (te(I, J, 0) + te(IP, J, 0));
            g.TAUB[g.itw(I, J, 1)] = 0.5 * (te(I, J, 1) + te(I, KP, 1));
            g.TAUW[g.itw(I, J, 2)] = 0.5 * (te(I, J, 2) + te(IP, J, 2));
            g.TAUB[g.itw(I, J, 2)] = 0.5 * (te(I, J, 3) + te(I, KP, 3));
        }
    }
    double w1 = 0.0;
    for (int J = 1; J <= N3M; J++)
        for (int I = 1; I <= N1M; I++) w1 = w1 + te(I, J, 0);
    g.WSM[0] = w1 / (double)(N1M * N3M);
    g.WSM[1] = 0.0;
    g.WSM[2] = 0.0;
    g.TAOW = g.WSM[0];
    return 0;
}

// MESH02's coordinates (compact3d.f:322-380): faces XG, ZG of the uniform x and z grids,
// centres XC, YC, ZC; indices as in Fortran.
struct Mesh02 {
    std::vector<double> XG, XC, YC, ZG, ZC;
};
static Mesh02 mesh02(const Orc &g) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    Mesh02 m;
    m.XG.assign(N1M + 2, 0.0);
    m.XC.assign(N1M + 2, 0.0);
    m.ZG.assign(N3M + 2, 0.0);
    m.ZC.assign(N3M + 2, 0.0);
    m.YC.assign(N2 + 1, 0.0);
    for (int I = 1; I <= N1M; I++) m.XG[I] = (double)(I - 1) * g.ALX / (double)N1M;
    m.XG[N1M + 1] = g.ALX;
    for (int K = 1; K <= N3M; K++) m.ZG[K] = (double)(K - 1) * g.ALZ / (double)N3M;
    m.ZG[N3M + 1] = g.ALZ;
    for (int I = 1; I <= N1M; I++) m.XC[I] = 0.5 * (m.XG[I + 1] + m.XG[I]);
    m.XC[N1M + 1] = m.XG[N1M + 1];
    for (int K = 1; K <= N3M; K++) m.ZC[K] = 0.5 * (m.ZG[K + 1] + m.ZG[K]);
    m.ZC[N3M + 1] = m.ZG[N3M + 1];
    m.YC[0] = g.Y[0];
    for (int J = 1; J <= N2M; J++) m.YC[J] = 0.5 * (g.Y[J + 1] + g.Y[J]);
    m.YC[N2] = g.Y[N2];
    return m;
}

// INDEX_IJK (compact3d.f:12763-12807): a point outside the outermost cell centres is moved
// by ANINT(... +- 0.5)/1E6 (the coordinates are changed in the caller, as the reference's
// by-reference arguments are), then the first cell whose faces bracket it in each direction.
static void index_ijk(const Orc &g, const Mesh02 &m, double &XP, double &YP, double &ZP, int &IP, int &JP, int &KP) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    if (XP < m.XC[1]) XP = std::round(XP * 1E06 + 0.5) / 1E06;
    if (XP > m.XC[N1M]) XP = std::round(XP * 1E06 - 0.5) / 1E06;
    if (YP < m.YC[1]) YP = std::round(YP * 1E06 + 0.5) / 1E06;
    if (YP > m.YC[N2M]) YP = std::round(YP * 1E06 - 0.5) / 1E06;
    if (ZP < m.ZC[1]) ZP = std::round(ZP * 1E06 + 0.5) / 1E06;
    if (ZP > m.ZC[N3M]) ZP = std::round(ZP * 1E06 - 0.5) / 1E06;
    IP = JP = KP = -1;
    for (int I = 1; I <= N1M && IP == -1; I++)
        if (XP >= m.XG[I] && XP <= m.XG[I + 1]) IP = I;
    for (int J = 1; J <= N2M && JP == -1; J++)
        if (YP >= g.Y[J] && YP <= g.Y[J + 1]) JP = J;
    for (int K = 1; K <= N3M && KP == -1; K++)
        if (ZP >= m.ZG[K] && ZP <= m.ZG[K + 1]) KP = K;
}

// INTERPOLAT (compact3d.f:12602-12760): trilinear interpolation of velocity component C
// (1 u at x faces, 2 v at y faces, 3 w at z faces) at (XP, YP, ZP) in cell (IP, JP, KP).
static double interpolat(const Orc &g, const Mesh02 &m, double XP, double YP, double ZP, int IP, int JP, int KP,
                         const double *U, int C) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2, N1 = g.N1, N3 = g.N3;
    int IUM, IUP, JUM, JUP, KUM, KUP;
    double XUM, XUP, YUM, YUP, ZUM, ZUP;
    if (C == 1) {
        IUM = IP; IUP = g.IPA[IP]; XUM = m.XG[IP]; XUP = m.XG[IUP];
        if (IP == N1M) XUP = m.XG[N1];
    } else if (XP >= m.XC[IP]) {
        IUM = IP; IUP = g.IPA[IP]; XUM = m.XC[IP]; XUP = m.XC[IUP];
        if (IP == N1M) XUP = m.XC[N1M] + 1. / g.DX1;
    } else {
        IUM = g.IMA[IP]; IUP = IP; XUM = m.XC[IUM]; XUP = m.XC[IP];
        if (IP == 1) XUM = m.XC[1] - 1. / g.DX1;
    }
    if (C == 2) {
        JUM = JP; JUP = g.JPA[JP]; YUM = g.Y[JP]; YUP = g.Y[JUP];
        if (JP == N2M) YUP = m.YC[N2];
    } else if (YP >= m.YC[JP]) {
        JUM = JP; JUP = g.JPA[JP]; YUM = m.YC[JP]; YUP = m.YC[JUP];
        if (JP == N2M) YUP = m.YC[N2];
    } else {
        JUM = g.JMU[JP]; JUP = JP; YUM = m.YC[JUM]; YUP = m.YC[JP];
        if (JP == 1) YUM = g.Y[1];
    }
    if (C == 3) {
        KUM = KP; KUP = g.KPA[KP]; ZUM = m.ZG[KP]; ZUP = m.ZG[KUP];
        if (KP == N3M) ZUP = m.ZG[N3];
    } else if (ZP >= m.ZC[KP]) {
        KUM = KP; KUP = g.KPA[KP]; ZUM = m.ZC[KP]; ZUP = m.ZC[KUP];
        if (KP == N3M) ZUP = m.ZC[N3M] + 1. / g.DX3;
    } else {
        KUM = g.KMA[KP]; KUP = KP; ZUM = m.ZC[KUM]; ZUP = m.ZC[KP];
        if (KP == 1) ZUM = m.ZC[1] - 1. / g.DX3;
    }
    auto u = [&](int i, int j, int k) { return U[g.iuc(i, j, k, C)]; };
    const double PHA = u(IUM, JUM, KUM), PHB = u(IUP, JUM, KUM), PHC = u(IUP, JUP, KUM), PHD = u(IUM, JUP, KUM);
    const double PHE = u(IUM, JUM, KUP), PHF = u(IUP, JUM, KUP), PHG = u(IUP, JUP, KUP), PHH = u(IUM, JUP, KUP);
    const double PHAB = (PHB - PHA) / (XUP - XUM) * (XP - XUM) + PHA;
    const double PHCD = (PHC - PHD) / (XUP - XUM) * (XP - XUM) + PHD;
    const double PHEF = (PHF - PHE) / (XUP - XUM) * (XP - XUM) + PHE;
    const double PHGH = (PHG - PHH) / (XUP - XUM) * (XP - XUM) + PHH;
    const double PHABCD = (PHCD - PHAB) / (YUP - YUM) * (YP - YUM) + PHAB;
    const double PHEFGH = (PHGH - PHEF) / (YUP - YUM) * (YP - YUM) + PHEF;
    return (PHEFGH - PHABCD) / (ZUP - ZUM) * (ZP - ZUM) + PHABCD;
}

// The bisection for u_tau of the log law on a plane-mean velocity (compact3d.f:5017-5029,
// 4390-4402): the lower end of the final bracket.
static double utau_bisect(double U_ave, double DELTAP, double RE, double U_tau1, double U_tau2) {
    const double KAPA = 0.41, B = 5.2;
    while (std::fabs(U_tau2 - U_tau1) > 0.0000001) {
        double TEMP = 0.5 * U_tau2 + 0.5 * U_tau1;
        const double FUtau1 = U_ave / U_tau1 - std::log(U_tau1 * DELTAP * RE) / KAPA - B;
        const double FUtau2 = U_ave / TEMP - std::log(TEMP * DELTAP * RE) / KAPA - B;
        TEMP = FUtau1 * FUtau2;
        if (TEMP <= 0.0) U_tau2 = 0.5 * U_tau2 + 0.5 * U_tau1;
        else U_tau1 = 0.5 * U_tau2 + 0.5 * U_tau1;
    }
    return U_tau1;
}

// The shifted-point models: PIOMELLI (WMODEL 5, compact3d.f:4960-5110) and MARUSIC1
// (WMODEL 3, 4336-4495).  u_tau of each wall from the log law on a plane-mean u, then per
// wall point the velocity interpolated at a point shifted downstream by DELTS.  PIOMELLI
// computes its y+ from DELTP, a variable the routine never sets (F:5035, 5088); it is taken
// as zero, so its shift DELTS is zero.  MARUSIC1's outer plane ZS is the plane nearest
// y = 0.06 (the last J found by its loop).
int wallmodel_shifted(Orc &g, const double *U) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double RE = g.RE, PI = std::acos(-1.0);
    const bool mar = g.WMODEL == 3;
    const Mesh02 m = mesh02(g);
    int ZS = -1;
    if (mar) {
        const double ZO = 0.06;
        for (int J = 1; J <= N2M; J++)
            if (std::fabs(g.Y[J] - ZO) <= std::fabs(g.Y[J + 1] - ZO) && std::fabs(g.Y[J] - ZO) <= std::fabs(g.Y[J - 1] - ZO))
                ZS = J;
        if (ZS < 1) return C3D_EINVAL;
    }
    const int jd = mar ? ZS : 1, ju = mar ? N2M - ZS + 1 : N2M;
    double U1DOWN = 0.0, U1UP = 0.0;
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            U1DOWN = U1DOWN + U[g.iuc(I, jd, K, 1)];
            U1UP = U1UP + U[g.iuc(I, ju, K, 1)];
        }
    U1DOWN = U1DOWN / (double)(N1M * N3M);
    U1UP = U1UP / (double)(N1M * N3M);
    for (int wall = 1; wall <= 2; wall++) {
        const double U_ave = wall == 1 ? U1DOWN : U1UP;
        double DELTAP, UTAU2, TAUW1, DELTS, CC = 1.0, YP;
        if (mar) {
            DELTAP = m.YC[ZS];
            UTAU2 = utau_bisect(U_ave, DELTAP, RE, 1.0, 0.000001);
            TAUW1 = UTAU2 * UTAU2;
            const double YPLUSML = DELTAP * UTAU2 * RE, YPLUS1 = g.DY[1] / 2.0 * UTAU2 * RE;
            CC = 1.0 + 0.05 * std::pow(std::log(YPLUS1 / YPLUSML), 2);
            DELTS = DELTAP / std::tan(16.0 * PI / 180);
            YP = wall == 1 ? DELTAP : m.YC[N2M - ZS + 1];
        } else {
            DELTAP = (wall == 1 ? g.DY[1] : g.DY[N2M]) / 2.0;
            UTAU2 = utau_bisect(U_ave, DELTAP, RE, 0.000001, 0.2);
            TAUW1 = UTAU2 * UTAU2;
            DELTS = 0.0;   // y+ from the unset DELTP
            YP = wall == 1 ? g.H[1] : m.YC[N2M];
        }
        if (wall == 1) {
            g.TAOW = TAUW1;
            g.WSM[0] = TAUW1;
        }
        for (int I = 1; I <= N1M; I++)
            for (int K = 1; K <= N3M; K++) {
                int IP, JP, KP;
                double XP = m.XG[I] + DELTS;
                if (XP > g.ALX) XP = XP - g.ALX;
                double ZP = m.ZC[K];
                index_ijk(g, m, XP, YP, ZP, IP, JP, KP);
                if (IP < 0 || JP < 0 || KP < 0) return C3D_EINVAL;
                const double F = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, mar ? 1 : 2);
                g.TAUW[g.itw(I, K, wall)] = mar ? TAUW1 + CC * 0.1 * UTAU2 * (F - U_ave) : TAUW1 + 0.1 * UTAU2 * F;
                XP = m.XC[I] + DELTS;
                if (XP > g.ALX) XP = XP - g.ALX;
                ZP = m.ZG[K];
                index_ijk(g, m, XP, YP, ZP, IP, JP, KP);
                if (IP < 0 || JP < 0 || KP < 0) return C3D_EINVAL;
                const double WF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 3);
                g.TAUB[g.itw(I, K, wall)] = TAUW1 * WF / U_ave;
            }
    }
    return 0;
}

// ----------------------------------------------------------------------------------
// WALLMODEL_IWMLES_SMOOTH (WMODEL 2 with Y0 = 0, compact3d.f:3386-4279), the integral
// wall model of Yang et al. 2015 on the bottom wall.  Per wall point a state of IWM_NS
// values (the reference's /IWMLES/ arrays) persists across steps: it is initialised at
// NTIME = 1 (or at the first call, where the reference would read a zeroed COMMON), the
// time-filtered velocity and pressure, the integrals and the stresses are recomputed every
// iwm_ntime_skip = 5 steps (NTIME mod 5 = 0) with the step WM_DT accumulated since, and
// TAUW is imposed every step.  The reference stores the spanwise stress in TAUW(I,K,3),
// beyond TAUW's extent (0:M1,0:M3,2); in /TAUXYZ/ that element is TAUB(I,K,1), which is
// where it is stored here.  WSM(1) = TAOW is the plane mean of sqrt(tauwx^2 + tauwy^2).
// ----------------------------------------------------------------------------------
enum {
    IW_UTX, IW_UTY, IW_TAUWX, IW_TAUWY, IW_FTX, IW_FTY, IW_FTMX, IW_FTMY, IW_FP, IW_INTE, IW_INTEM = IW_INTE + 5,
    IW_DIFFX = IW_INTEM + 5, IW_DIFFY, IW_LHSX, IW_LHSY, IW_FUS, IW_TR, IW_DZ, IW_AX, IW_AY, IW_CX, IW_CY,
    IW_UNSX, IW_UNSY, IW_DELI, IW_DELV, IW_DTX, IW_DTY, IW_DBX, IW_DBY, IW_CONVX, IW_CONVY, IW_PRSX, IW_PRSY,
    IW_Z0, IW_NS
};
// integral indices iwm_Lu = 1, iwm_Luu = 2, iwm_Lv = 3, iwm_Lvv = 4, iwm_Luv = 5
enum { IW_LU = 0, IW_LUU = 1, IW_LV = 2, IW_LVV = 3, IW_LUV = 4 };

// the Newton iteration for u_tau on the log law U/u - log(u DZP RE)/KAPA - B (KAPA 0.4,
// B 5), as in iwm_init_smooth and the equilibrium fallback (compact3d.f:3589-3604, 4079-4091)
static double iwm_loglaw(double U_ave, double DZP, double RE) {
    const double KAPA = 0.4, B = 5.0;
    double U_tau1 = 1.0, U_tau2 = 0.000001, LAMBDA = 1.0;
    for (int it = 0; it < 100000 && std::fabs(U_tau2 - U_tau1) > 1.0E-6; it++) {
        U_tau1 = U_tau2;
        const double FUtau1 = U_ave / U_tau1 - std::log(U_tau1 * DZP * RE) / KAPA - B;
        const double FUtau2 = -U_ave / std::pow(U_tau1, 2.0) - 1. / KAPA / U_tau1;
        U_tau2 = U_tau1 - LAMBDA * FUtau1 / FUtau2;
        const double FUtau3 = U_ave / U_tau2 - std::log(U_tau2 * DZP * RE) / KAPA - B;
        if (std::fabs(FUtau3) > std::fabs(FUtau1)) LAMBDA = 0.5 * LAMBDA;
    }
    return U_tau1;
}

// iwm_slv_smooth (compact3d.f:3881-3926): the integrated momentum residuals (fx, fy)
static void iwm_slv(double lhsx, double lhsy, double Ux, double Uy, double Dz, double utx, double uty, double RE,
                    double &fx, double &fy) {
    const double vonk = 0.4, reinv = 1.0 / RE;
    const double us = std::pow(std::pow(utx, 4.0) + std::pow(uty, 4.0), 0.25);
    const double delv = reinv / us;
    const double deli = std::min(11.0 * reinv / us, Dz);
    const double Vel = std::sqrt(std::pow(Ux, 2.0) + std::pow(Uy, 2.0));
    const double Ax = (Ux / us + Ux / Vel / vonk * std::log(deli / Dz) - deli / delv * utx / us) / (1.0 - deli / Dz);
    const double Ay = (Uy / us + Uy / Vel / vonk * std::log(deli / Dz) - deli / delv * uty / us) / (1.0 - deli / Dz);
    const double Cx = Ux / us - Ax, Cy = Uy / us - Ay;
    const double inteLu = 0.5 * utx * std::pow(deli, 2.0) / delv +
                          us * Dz * (0.5 * Ax * (1.0 - std::pow(deli, 2.0) / std::pow(Dz, 2.0)) + Cx * (1.0 - deli / Dz) -
                                     1.0 / vonk * Ux / Vel * (1.0 - deli / Dz + deli / Dz * std::log(deli / Dz)));
    const double inteLv = 0.5 * uty * std::pow(deli, 2.0) / delv +
                          us * Dz * (0.5 * Ay * (1.0 - std::pow(deli, 2.0) / std::pow(Dz, 2.0)) + Cy * (1.0 - deli / Dz) -
                                     1.0 / vonk * Uy / Vel * (1.0 - deli / Dz + deli / Dz * std::log(deli / Dz)));
    fx = inteLu + lhsx;
    fy = inteLv + lhsy;
}

// iwm_slv_rough (compact3d.f:3031-3052)
static void iwm_slv_rough(double lhsx, double lhsy, double Ux, double Uy, double Dz, double z0, double utx, double uty,
                          double &fx, double &fy) {
    const double vonk = 0.4;
    const double Ax = (Ux - utx / vonk * std::log(Dz / z0)) / ((1.0 - z0 / Dz));
    const double Ay = (Uy - uty / vonk * std::log(Dz / z0)) / ((1.0 - z0 / Dz));
    const double inteLu = 1.0 / 2.0 * Dz * Ax * std::pow(1.0 - z0 / Dz, 2.0) +
                          1.0 / vonk * utx * Dz * (z0 / Dz - 1.0 + std::log(Dz / z0));
    const double inteLv = 1.0 / 2.0 * Dz * Ay * std::pow(1.0 - z0 / Dz, 2.0) +
                          1.0 / vonk * uty * Dz * (z0 / Dz - 1.0 + std::log(Dz / z0));
    fx = inteLu + lhsx;
    fy = inteLv + lhsy;
}

// iwm_calc_wallstress_rough (compact3d.f:3055-3334): a Newton solve with the diagonal
// finite-difference Jacobian (a12 = a21 = 0), the equilibrium law vonk U / log(Dz / z0)
// as fallback, the rough-wall integrals and stresses.  Kept as written: the Lvv integral
// has -3 z0^2/Dz^2 where Luu has +3, and tauwy is (vonk * iwmpz0)^2 ... with iwmpz0 an
// undeclared, zero-valued name, so tauwy = 0 (times dVelzB dudzB) off the fallback.
template <typename ST>
static void iwm_wallstress_rough(Orc &g, ST &st, double Y0, double wm_dt) {
    const int N1M = g.N1M, N3M = g.N3M;
    const double vonk = 0.4, wm_tol = 0.000001, wm_eps = 0.000000001;
    const int MaxIter = 1500;
    (void)Y0;
    for (int I = 1; I <= N1M; I++)
        for (int K = 1; K <= N3M; K++) {
            const double lhsx = st(I, K, IW_LHSX), lhsy = st(I, K, IW_LHSY);
            const double Ux = st(I, K, IW_FTX), Uy = st(I, K, IW_FTY), Dz = st(I, K, IW_DZ), z0 = st(I, K, IW_Z0);
            double &utx = st(I, K, IW_UTX), &uty = st(I, K, IW_UTY);
            double fx, fy, fxp, fyp;
            iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty, fx, fy);
            int iter = 0, equil_flag = 0;
            while (std::max(std::fabs(fx), std::fabs(fy)) > wm_tol) {
                iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx + wm_eps, uty, fxp, fyp);
                const double a11 = (fxp - fx) / wm_eps, a21 = 0.0;
                iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty + wm_eps, fxp, fyp);
                const double a12 = 0.0, a22 = (fyp - fy) / wm_eps;
                const double det = a11 * a22 - a12 * a21;
                const double nx = utx - (a22 * fx - a12 * fy) / det;
                const double ny = uty - (-a21 * fx + a11 * fy) / det;
                utx = nx;
                uty = ny;
                iwm_slv_rough(lhsx, lhsy, Ux, Uy, Dz, z0, utx, uty, fx, fy);
                iter = iter + 1;
                if (iter > MaxIter) {
                    equil_flag = 1;
                    break;
                }
            }
            if (utx - 1.0 == utx || uty - 1.0 == uty) equil_flag = 1;
            const double lg = std::log(Dz / z0);
            const double equilutx = vonk * Ux / lg, equiluty = vonk * Uy / lg;
            if (equil_flag == 1) {
                utx = equilutx;
                uty = equiluty;
            }
            double Ax = 0.0, Ay = 0.0;
            if (equil_flag != 1) {
                Ax = (Ux - utx / vonk * lg) / ((1.0 - z0 / Dz));
                Ay = (Uy - uty / vonk * lg) / ((1.0 - z0 / Dz));
            }
            st(I, K, IW_AX) = Ax;
            st(I, K, IW_AY) = Ay;
            for (int q = 0; q < 5; q++) st(I, K, IW_INTEM + q) = st(I, K, IW_INTE + q);
            const double px = utx, py = uty, r = z0 / Dz;
            const double P4 = 1.0 - 4.0 * r + 3.0 * std::pow(z0, 2.0) / std::pow(Dz, 2.0) - 2.0 * lg + 4.0 * r * lg;
            const double M4 = 1.0 - 4.0 * r - 3.0 * std::pow(z0, 2.0) / std::pow(Dz, 2.0) - 2.0 * lg + 4.0 * r * lg;
            st(I, K, IW_INTE + IW_LU) = 1.0 / 2.0 * Dz * Ax * std::pow(1.0 - r, 2.0) + 1.0 / vonk * px * Dz * (r - 1.0 + lg);
            st(I, K, IW_INTE + IW_LV) = 1.0 / 2.0 * Dz * Ay * std::pow(1.0 - r, 2.0) + 1.0 / vonk * py * Dz * (r - 1.0 + lg);
            st(I, K, IW_INTE + IW_LUV) = 1.0 / std::pow(vonk, 2.0) * px * py * Dz * (1.0 - 2 * r + std::pow(1.0 - lg, 2.0)) +
                                         1.0 / 3.0 * Ax * Ay * Dz * std::pow(1.0 - r, 3.0) -
                                         1.0 / 4.0 / vonk * (Ax * py + Ay * px) * Dz * P4;
            st(I, K, IW_INTE + IW_LUU) = 1.0 / std::pow(vonk, 2.0) * std::pow(px, 2.0) * Dz *
                                             (std::pow(lg - 1.0, 2.0) - 2.0 * r + 1.0) +
                                         1.0 / 3.0 * std::pow(Ax, 2.0) * Dz * std::pow(1.0 - r, 3.0) -
                                         1.0 / 2.0 / vonk * px * Ax * Dz * P4;
            st(I, K, IW_INTE + IW_LVV) = 1.0 / std::pow(vonk, 2.0) * std::pow(py, 2.0) * Dz *
                                             (std::pow(lg - 1.0, 2.0) - 2.0 * r + 1.0) +
                                         1.0 / 3.0 * std::pow(Ay, 2.0) * Dz * std::pow(1.0 - r, 3.0) -
                                         1.0 / 2.0 / vonk * py * Ay * Dz * M4;
            const double dTx = 1.0 / Dz * (Ax + px / vonk), dTy = 1.0 / Dz * (Ay + py / vonk);
            const double dBx = 1.0 / Dz * Ax + px / vonk / z0, dBy = 1.0 / Dz * Ay + py / vonk / z0;
            st(I, K, IW_DTX) = dTx;
            st(I, K, IW_DTY) = dTy;
            st(I, K, IW_DBX) = dBx;
            st(I, K, IW_DBY) = dBy;
            const double Vel = std::sqrt(std::pow(Ux, 2.0) + std::pow(Uy, 2.0));
            const double dVelzT = std::fabs(Ux / Vel * dTx + Uy / Vel * dTy);
            const double dVelzB = std::sqrt(std::pow(dBx, 2.0) + std::pow(dBy, 2.0));
            st(I, K, IW_DIFFX) = std::pow(vonk * Dz, 2.0) * dVelzT * dTx - std::pow(vonk * z0, 2.0) * dVelzB * dBx;
            st(I, K, IW_DIFFY) = std::pow(vonk * Dz, 2.0) * dVelzT * dTy - std::pow(vonk * z0, 2.0) * dVelzB * dBy;
            if (equil_flag == 1) {
                const double equilWMpara = std::sqrt(std::pow(Ux, 2.0) + std::pow(Uy, 2.0)) * std::pow(vonk, 2.0) /
                                           std::pow(lg, 2.0);
                st(I, K, IW_TAUWX) = equilWMpara * Ux;
                st(I, K, IW_TAUWY) = equilWMpara * Uy;
            } else {
                const double iwmpz0 = 0.0;
                st(I, K, IW_TAUWX) = std::pow(vonk * z0, 2.0) * dVelzB * dBx;
                st(I, K, IW_TAUWY) = std::pow(vonk * iwmpz0, 2.0) * dVelzB * dBy;
            }
            const double utaup = std::pow(std::pow(st(I, K, IW_TAUWX), 2.0) + std::pow(st(I, K, IW_TAUWY), 2.0), 0.25);
            st(I, K, IW_FUS) = st(I, K, IW_FUS) * (1.0 - st(I, K, IW_TR)) + utaup * st(I, K, IW_TR);
            st(I, K, IW_TR) = wm_dt / (st(I, K, IW_DZ) / st(I, K, IW_FUS) / vonk);
            if (st(I, K, IW_TR) > 1.0) st(I, K, IW_TR) = 1.0;
        }
}

int wallmodel_iwmles(Orc &g, const double *U, const double *P, int NTIME, double DT, double PRESG, double PRESG3) {
    const int N1M = g.N1M, N3M = g.N3M;
    const size_t NP = (size_t)N1M * N3M;
    const double RE = g.RE, reinv = 1.0 / RE, vonk = 0.4;
    auto st = [&](int I, int K, int q) -> double & { return g.IWM[(size_t)q * NP + (I - 1) + (size_t)N1M * (K - 1)]; };
    const double Dzp = g.DY[1] + g.DY[2] + g.DY[3] / 2.0;
    // WALLMODEL_IWMLES_ROUGH (Y0 = Y(0) != 0, compact3d.f:2562-3381): the same filter, left-
    // hand side and schedule with the rough-wall profile (roughness length z0 = Y0)
    const bool rough = g.Y[0] != 0.0;
    const double Y0 = g.Y[0];
    if (NTIME == 1 || !g.iwm_ready) {   // iwm_init_smooth / iwm_init_rough (3561-3714, 2736-2857)
        g.IWM.assign(NP * IW_NS, 0.0);
        double uinit = 0.0;
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) uinit = uinit + U[g.iuc(I, 3, K, 1)];
        uinit = uinit / (double)(N1M * N3M);
        const double usinit = rough ? uinit * vonk / std::log(Dzp / Y0) : iwm_loglaw(uinit, Dzp, RE);
        for (int I = 1; I <= N1M; I++)
            for (int K = 1; K <= N3M; K++) {
                st(I, K, IW_UTX) = usinit;
                st(I, K, IW_TAUWX) = std::pow(usinit, 2.0);
                st(I, K, IW_FTX) = uinit;
                st(I, K, IW_FTMX) = uinit;
                st(I, K, IW_INTE + IW_LU) = uinit * Dzp;
                st(I, K, IW_INTE + IW_LUU) = std::pow(uinit, 2.0) * Dzp;
                st(I, K, IW_INTEM + IW_LU) = uinit * Dzp;
                st(I, K, IW_INTEM + IW_LUU) = std::pow(uinit, 2.0) * Dzp;
                st(I, K, IW_LHSX) = -uinit * Dzp;
                st(I, K, IW_LHSY) = -uinit * Dzp;
                st(I, K, IW_DTX) = usinit / vonk / Dzp;
                st(I, K, IW_FUS) = usinit;
                st(I, K, IW_TR) = (g.CFLMAX * g.ALX / N1M / uinit) / (Dzp / vonk / usinit);
                st(I, K, IW_DZ) = Dzp;
                if (rough) {
                    st(I, K, IW_DBX) = usinit / vonk / Y0;
                    st(I, K, IW_Z0) = Y0;
                } else {
                    st(I, K, IW_DELI) = std::min(11.0 * reinv / usinit, Dzp);
                    st(I, K, IW_DELV) = reinv / usinit;
                }
            }
        g.WM_DT = 5 * DT;
        g.iwm_ready = 1;
    }
    // iwm_wallstress_smooth (compact3d.f:3489-3557)
    if (NTIME % 5 == 1) g.WM_DT = DT;
    else g.WM_DT = g.WM_DT + DT;
    const double wm_dt = g.WM_DT;
    int status = 0;
    if (NTIME % 5 == 0) {
        // iwm_calc_lhs_smooth (3718-3877)
        double p_bar = 0.0;
        for (int I = 1; I <= N1M; I++)
            for (int K = 1; K <= N3M; K++) p_bar = p_bar + P[g.ip(I, 1, K)];
        p_bar = p_bar / (double)N1M / (double)N3M;
        for (int I = 1; I <= N1M; I++)
            for (int K = 1; K <= N3M; K++) {
                st(I, K, IW_FTMX) = st(I, K, IW_FTX);
                st(I, K, IW_FTMY) = st(I, K, IW_FTY);
                const double u_inst = U[g.iuc(I, 3, K, 1)], v_inst = U[g.iuc(I, 3, K, 3)];
                const double p_inst = P[g.ip(I, 1, K)] - p_bar, tR = st(I, K, IW_TR);
                st(I, K, IW_FTX) = st(I, K, IW_FTX) * (1.0 - tR) + u_inst * tR;
                st(I, K, IW_FTY) = st(I, K, IW_FTY) * (1.0 - tR) + v_inst * tR;
                st(I, K, IW_FP) = st(I, K, IW_FP) * (1.0 - tR) + p_inst * tR;
            }
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K], KM = g.KMA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I], IM = g.IMA[I];
                st(I, K, IW_UNSX) = (st(I, K, IW_INTE + IW_LU) - st(I, K, IW_INTEM + IW_LU)) / wm_dt;
                st(I, K, IW_UNSY) = (st(I, K, IW_INTE + IW_LV) - st(I, K, IW_INTEM + IW_LV)) / wm_dt;
                const double uux = (st(IP, K, IW_INTE + IW_LUU) - st(IM, K, IW_INTE + IW_LUU)) * g.DX1 / 2.0;
                const double uvy = (st(I, KP, IW_INTE + IW_LUV) - st(I, KM, IW_INTE + IW_LUV)) * g.DX3 / 2.0;
                const double uvx = (st(IP, K, IW_INTE + IW_LUV) - st(IM, K, IW_INTE + IW_LUV)) * g.DX1 / 2.0;
                const double vvy = (st(I, KP, IW_INTE + IW_LVV) - st(I, KM, IW_INTE + IW_LVV)) * g.DX3 / 2.0;
                const double ux = (st(IP, K, IW_INTE + IW_LU) - st(IM, K, IW_INTE + IW_LU)) * g.DX1 / 2.0;
                const double vy = (st(I, KP, IW_INTE + IW_LV) - st(I, KM, IW_INTE + IW_LV)) * g.DX3 / 2.0;
                st(I, K, IW_CONVX) = uux + uvy - st(I, K, IW_FTMX) * (ux + vy);
                st(I, K, IW_CONVY) = uvx + vvy - st(I, K, IW_FTMY) * (ux + vy);
                const double Dz = st(I, K, IW_DZ);
                st(I, K, IW_PRSX) = (st(IP, K, IW_FP) - st(IM, K, IW_FP)) * g.DX1 / 2.0 * Dz + PRESG * Dz;
                st(I, K, IW_PRSY) = (st(I, KP, IW_FP) - st(I, KM, IW_FP)) * g.DX3 / 2.0 * Dz + PRESG3 * Dz;
                st(I, K, IW_LHSX) = -st(I, K, IW_INTE + IW_LU) +
                                    wm_dt * (st(I, K, IW_CONVX) + st(I, K, IW_PRSX) - st(I, K, IW_DIFFX));
                st(I, K, IW_LHSY) = -st(I, K, IW_INTE + IW_LV) +
                                    wm_dt * (st(I, K, IW_CONVY) + st(I, K, IW_PRSY) - st(I, K, IW_DIFFY));
            }
        }
        if (rough) iwm_wallstress_rough(g, st, Y0, wm_dt);
        // iwm_calc_wallstress_smooth (3930-4279)
        const double KAPA = 0.4, B = 5.0, deltap = Dzp;
        const int MaxIter = 1500;
        const double wm_tol = 0.000001, wm_eps = 0.000000001;
        (void)KAPA;
        (void)B;
        // equilutx/equiluty are locals of the point loop that only the equilibrium fallback
        // sets: a point whose linear correction |A| > 1 sends it to that branch without a
        // fallback of its own takes the values of the last point (I outer, K inner) that
        // had one (zero before the first)
        double equilutx = 0.0, equiluty = 0.0;
        for (int I = 1; I <= (rough ? 0 : N1M); I++)
            for (int K = 1; K <= N3M; K++) {
                const double lhsx = st(I, K, IW_LHSX), lhsy = st(I, K, IW_LHSY);
                const double Ux = st(I, K, IW_FTX), Uy = st(I, K, IW_FTY), Dz = st(I, K, IW_DZ);
                double &utx = st(I, K, IW_UTX), &uty = st(I, K, IW_UTY);
                double fx, fy, fxp, fyp;
                iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, RE, fx, fy);
                int iter = 0, equil_flag = 0;
                while (std::max(std::fabs(fx), std::fabs(fy)) > wm_tol) {
                    iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx + wm_eps, uty, RE, fxp, fyp);
                    const double a11 = (fxp - fx) / wm_eps, a21 = (fyp - fy) / wm_eps;
                    iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty + wm_eps, RE, fxp, fyp);
                    const double a12 = (fxp - fx) / wm_eps, a22 = (fyp - fy) / wm_eps;
                    const double det = a11 * a22 - a12 * a21;
                    const double nx = utx - (a22 * fx - a12 * fy) / det;
                    const double ny = uty - (-a21 * fx + a11 * fy) / det;
                    utx = nx;
                    uty = ny;
                    iwm_slv(lhsx, lhsy, Ux, Uy, Dz, utx, uty, RE, fx, fy);
                    iter = iter + 1;
                    if (iter > MaxIter) {
                        equil_flag = 1;
                        break;
                    }
                }
                if (utx - 1.0 == utx || uty - 1.0 == uty) equil_flag = 1;
                if (equil_flag == 1) {
                    const double U_ave = std::sqrt(std::pow(Ux, 2.) + std::pow(Uy, 2.));
                    const double U_tau1 = iwm_loglaw(U_ave, deltap, RE);
                    const double TAUW1 = std::pow(U_tau1, 2);
                    equilutx = TAUW1 * Ux / U_ave;
                    equiluty = TAUW1 * Uy / U_ave;
                    utx = std::sqrt(std::fabs(equilutx));
                    uty = std::sqrt(std::fabs(equiluty));
                }
                const double wmputx = utx, wmputy = uty, wmpDz = Dz;
                const double utaup = std::pow(std::pow(wmputx, 4.0) + std::pow(wmputy, 4.0), 0.25);
                const double wmpdelv = reinv / utaup;
                const double wmpdeli = std::min(11.0 * reinv / utaup, wmpDz);
                const double wmpUx = Ux, wmpUy = Uy;
                const double wmpVel = std::sqrt(std::pow(wmpUx, 2.0) + std::pow(wmpUy, 2.0));
                double wmpAx = 0.0, wmpAy = 0.0, wmpCx = 0.0, wmpCy = 0.0;
                const double lg = std::log(wmpdeli / wmpDz);
                if (equil_flag != 1) {
                    wmpAx = (wmpUx / utaup + wmpUx / wmpVel / vonk * lg - wmpdeli / wmpdelv * wmputx / utaup) /
                            (1.0 - wmpdeli / wmpDz);
                    wmpAy = (wmpUy / utaup + wmpUy / wmpVel / vonk * lg - wmpdeli / wmpdelv * wmputy / utaup) /
                            (1.0 - wmpdeli / wmpDz);
                    wmpCx = wmpUx / utaup - wmpAx;
                    wmpCy = wmpUy / utaup - wmpAy;
                }
                double px = wmputx, py = wmputy;   // the values the integrals below use
                if (std::fabs(wmpAx) > 1.0 || std::fabs(wmpAy) > 1.0) {
                    equil_flag = 1;
                    utx = std::sqrt(std::fabs(equilutx));
                    uty = std::sqrt(std::fabs(equiluty));
                    wmpAx = 0.0;
                    wmpAy = 0.0;
                    wmpCx = 0.0;
                    wmpCy = 0.0;
                }
                st(I, K, IW_AX) = wmpAx;
                st(I, K, IW_AY) = wmpAy;
                st(I, K, IW_CX) = wmpCx;
                st(I, K, IW_CY) = wmpCy;
                for (int q = 0; q < 5; q++) st(I, K, IW_INTEM + q) = st(I, K, IW_INTE + q);
                st(I, K, IW_INTE + IW_LU) =
                    0.5 * px * std::pow(wmpdeli, 2.0) / wmpdelv +
                    utaup * wmpDz *
                        (0.5 * wmpAx * (1.0 - std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0)) +
                         wmpCx * (1.0 - wmpdeli / wmpDz) -
                         1.0 / vonk * wmpUx / wmpVel * (1.0 - wmpdeli / wmpDz + wmpdeli / wmpDz * lg));
                st(I, K, IW_INTE + IW_LV) =
                    0.5 * py * std::pow(wmpdeli, 2.0) / wmpdelv +
                    utaup * wmpDz *
                        (0.5 * wmpAy * (1.0 - std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0)) +
                         wmpCy * (1.0 - wmpdeli / wmpDz) -
                         1.0 / vonk * wmpUy / wmpVel * (1.0 - wmpdeli / wmpDz + wmpdeli / wmpDz * lg));
                st(I, K, IW_INTE + IW_LUV) =
                    1.0 / 3.0 * px * py * std::pow(wmpdeli, 3.0) / std::pow(wmpdelv, 2.0) +
                    std::pow(utaup, 2.0) * wmpDz *
                        (-1.0 / vonk * (wmpAx * wmpUy / wmpVel + wmpAy * wmpUx / wmpVel) *
                             (0.25 - 0.25 * std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0) +
                              0.5 * std::pow(wmpdeli, 2.0) / wmpDz * lg) -
                         1.0 / vonk * (wmpCx * wmpUy / wmpVel + wmpCy * wmpUx / wmpVel) *
                             (1.0 - wmpdeli / wmpDz + wmpdeli / wmpDz * lg) -
                         wmpUx * wmpUy / std::pow(wmpVel, 2.0) / std::pow(vonk, 2.0) *
                             (wmpdeli / wmpDz - 2.0 + wmpdeli / wmpDz * std::pow(lg - 1.0, 2.0)) +
                         1.0 / 3.0 * wmpAx * wmpAy * (1.0 - std::pow(wmpdeli, 3.0) / std::pow(wmpDz, 3.0)) +
                         0.5 * (wmpAx * wmpCy + wmpAy * wmpCx) * (1.0 - std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0)) +
                         wmpCx * wmpCy * (1.0 - wmpdeli / wmpDz));
                auto inte_sq = [&](double pu, double A, double C, double Uc) {   // Eq. C20, x or y
                    return 1.0 / 3.0 * std::pow(pu, 2.0) * std::pow(wmpdeli, 3.0) / std::pow(wmpdelv, 2.0) +
                           std::pow(utaup, 2.0) * wmpDz *
                               (-A * Uc / wmpVel / vonk * std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0) * lg +
                                A * (C - 1.0 / 2.0 / vonk * Uc / wmpVel) * (1.0 - std::pow(wmpdeli, 2.0) / std::pow(wmpDz, 2.0)) +
                                std::pow(A, 2.0) / 3.0 * (1.0 - std::pow(wmpdeli, 3.0) / std::pow(wmpDz, 3.0)) +
                                std::pow(C - 1.0 / vonk * Uc / wmpVel, 2.0) -
                                wmpdeli / wmpDz * std::pow(C - Uc / wmpVel / vonk + Uc / wmpVel / vonk * lg, 2.0) +
                                1.0 / std::pow(vonk, 2.0) * std::pow(Uc, 2.0) / std::pow(wmpVel, 2.0) * (1.0 - wmpdeli / wmpDz));
                };
                st(I, K, IW_INTE + IW_LUU) = inte_sq(px, wmpAx, wmpCx, wmpUx);
                st(I, K, IW_INTE + IW_LVV) = inte_sq(py, wmpAy, wmpCy, wmpUy);
                double dTx, dTy;
                if (wmpdeli < wmpDz) {
                    dTx = utaup / wmpDz * (wmpAx + 1.0 / vonk * wmpUx / wmpVel);
                    dTy = utaup / wmpDz * (wmpAy + 1.0 / vonk * wmpUy / wmpVel);
                } else {
                    dTx = px / wmpdelv;
                    dTy = py / wmpdelv;
                }
                const double dBx = px / wmpdelv, dBy = py / wmpdelv;
                st(I, K, IW_DTX) = dTx;
                st(I, K, IW_DTY) = dTy;
                st(I, K, IW_DBX) = dBx;
                st(I, K, IW_DBY) = dBy;
                const double dVelzT = std::fabs(wmpUx / wmpVel * dTx + wmpUy / wmpVel * dTy);
                if (wmpdeli < wmpDz) {
                    st(I, K, IW_DIFFX) = (reinv + std::pow(vonk * wmpDz, 2.0) * dVelzT) * dTx - reinv * dBx;
                    st(I, K, IW_DIFFY) = (reinv + std::pow(vonk * wmpDz, 2.0) * dVelzT) * dTy - reinv * dBy;
                } else {
                    st(I, K, IW_DIFFX) = 0.0;
                    st(I, K, IW_DIFFY) = 0.0;
                }
                if (equil_flag == 1) {
                    st(I, K, IW_TAUWX) = equilutx;
                    st(I, K, IW_TAUWY) = equiluty;
                } else if (wmpdeli < wmpDz) {
                    st(I, K, IW_TAUWX) = std::pow(px, 2.0);
                    st(I, K, IW_TAUWY) = std::pow(py, 2.0);
                } else {
                    st(I, K, IW_TAUWX) = reinv * wmpUx / wmpDz;
                    st(I, K, IW_TAUWY) = reinv * wmpUy / wmpDz;
                }
                st(I, K, IW_FUS) = st(I, K, IW_FUS) * (1.0 - st(I, K, IW_TR)) + utaup * st(I, K, IW_TR);
                st(I, K, IW_TR) = wm_dt / (st(I, K, IW_DZ) / st(I, K, IW_FUS) / vonk);
                if (st(I, K, IW_TR) > 1.0) st(I, K, IW_TR) = 1.0;
            }
    }
    // every step: the stresses and WSM(1) (3541-3556, 3466-3479)
    double WSM1 = 0.0;
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            g.TAUW[g.itw(I, K, 1)] = st(I, K, IW_TAUWX);
            g.TAUB[g.itw(I, K, 1)] = st(I, K, IW_TAUWY);
            WSM1 = WSM1 + std::sqrt(std::pow(g.TAUW[g.itw(I, K, 1)], 2.) + std::pow(g.TAUB[g.itw(I, K, 1)], 2.));
        }
    g.WSM[0] = WSM1 / (double)(N1M * N3M);
    g.TAOW = g.WSM[0];
    return status;
}

// The wall model WALL_MODEL dispatches to (compact3d.f:1982-2011) for WMODEL = 1..5.
int wallmodel(Orc &g, const double *U, const double *P = nullptr, int NTIME = 1, double DT = 0.0, double PRESG = 0.0,
              double PRESG3 = 0.0) {
    if (g.WMODEL == 4) return wallmodel_werner(g, U);
    if (g.WMODEL == 3 || g.WMODEL == 5) return wallmodel_shifted(g, U);
    if (g.WMODEL == 2) return P ? wallmodel_iwmles(g, U, P, NTIME, DT, PRESG, PRESG3) : C3D_EINVAL;
    if (g.Y[0] != 0.0) return wallmodel_rough(g, U);
    return wallmodel_instant(g, U);
}

// ----------------------------------------------------------------------------------
// GETUH1/2/3 (compact3d.f:8218-8627): Crank-Nicolson delta form, approximate
// factorisation y -> x -> z (u, v) and y -> z -> x (w), then UH = U + delta.
// ----------------------------------------------------------------------------------
void getuh(Orc &g, const double *U, double *UH, const double *RUH, int comp, double DT) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double RE = g.RE, DX1Q = g.DX1Q, DX3Q = g.DX3Q;
    const int JS = (comp == 2) ? 2 : 1;
    // y: TDMAI over J for every (I,K)
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> A(N2M + 2), B(N2M + 2), C(N2M + 2), R(N2M + 2);
        for (int I = 1; I <= N1M; I++) {
            for (int J = JS; J <= N2M; J++) {
                double FJUM = (comp == 2) ? g.FJMV[J] : g.FJMU[J];
                double FJUP = g.FJPA[J];
                if (comp == 2) {
                    C[J] = FJUP * (-0.5 * g.DYP[J] * (1. / RE)) * DT;
                    B[J] = 1.0 + (+0.5 * g.DYC[J] * (1. / RE)) * DT;
                    A[J] = FJUM * (-0.5 * g.DYM[J] * (1. / RE)) * DT;
                    R[J] = DT * RUH[g.iu(I, J, K)];
                } else {
                    C[J] = FJUP * (-0.5 * g.HP[J] * (1. / RE)) * DT;
                    B[J] = 1.0 + (0.5 * g.HC[J] * (1. / RE)) * DT;
                    A[J] = FJUM * (-0.5 * g.HM[J] * (1. / RE)) * DT;
                    R[J] = RUH[g.iu(I, J, K)] * DT;
                }
            }
            tdmai_line(JS, N2M, A.data(), B.data(), C.data(), R.data(), R.data());
            for (int J = JS; J <= N2M; J++) UH[g.iuc(I, J, K, comp)] = R[J];
        }
    }
    const double api = 1.0 - DT / 2.0 * (1. / RE) * 12.0 * DX1Q * (1.0);
    const double aci = 10.0 - DT / 2.0 * (1. / RE) * 12.0 * DX1Q * (-2.0);
    const double apk = 1.0 - DT / 2.0 * (1. / RE) * 12.0 * DX3Q * (1.0);
    const double ack = 10.0 - DT / 2.0 * (1. / RE) * 12.0 * DX3Q * (-2.0);
    auto xsweep = [&]() {
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++) {
            std::vector<double> A(N1M + 2, api), B(N1M + 2, aci), C(N1M + 2, api), R(N1M + 2);
            for (int J = JS; J <= N2M; J++) {
                for (int I = 1; I <= N1M; I++) {
                    int im = (I == 1) ? N1M : I - 1, ipp = (I == N1M) ? 1 : I + 1;
                    R[I] = UH[g.iuc(im, J, K, comp)] + 10.0 * UH[g.iuc(I, J, K, comp)] + UH[g.iuc(ipp, J, K, comp)];
                }
                ctdma_recip(1, N1M, A.data(), B.data(), C.data(), R.data(), R.data());
                for (int I = 1; I <= N1M; I++) UH[g.iuc(I, J, K, comp)] = R[I];
            }
        }
    };
    auto zsweep = [&]() {
#pragma omp parallel for
        for (int J = JS; J <= N2M; J++) {
            std::vector<double> A(N3M + 2, apk), B(N3M + 2, ack), C(N3M + 2, apk), R(N3M + 2), X(N3M + 2);
            for (int I = 1; I <= N1M; I++) {
                for (int K = 1; K <= N3M; K++) {
                    int km = (K == 1) ? N3M : K - 1, kp = (K == N3M) ? 1 : K + 1;
                    R[K] = UH[g.iuc(I, J, km, comp)] + 10.0 * UH[g.iuc(I, J, K, comp)] + UH[g.iuc(I, J, kp, comp)];
                }
                ctdma_recip(1, N3M, A.data(), B.data(), C.data(), R.data(), X.data());
                for (int K = 1; K <= N3M; K++) UH[g.iuc(I, J, K, comp)] = X[K];
            }
        }
    };
    if (comp == 3) {
        zsweep();
        xsweep();
    } else {
        xsweep();
        zsweep();
    }
    (void)U;
}

// RHSDP (compact3d.f:8117-8214)
void rhsdp(Orc &g, double *RDP, const double *UH, double DT) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double DX1 = g.DX1, DX3 = g.DX3;
    const double *DY = g.DY.data();
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++) {
            int JP = J + 1;
            double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
            for (int I = 1; I <= N1M; I++) {
                double DIVUH = (FJUP * UH[g.iuc(I, JP, K, 2)] - FJUM * UH[g.iuc(I, J, K, 2)]) / DY[J];
                double CBC = (1. - FJUM) * g.UBC[g.iubc(I, K, 2, 1)] / DY[J] -
                             (1. - FJUP) * g.UBC[g.iubc(I, K, 2, 2)] / DY[J];
                RDP[g.ip(I, J, K)] = (DIVUH - CBC) / DT;
            }
        }
    ConstLine L22x, L22z;
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 1; I <= N1M - 1; I++)
                D1[I] = 24. * DX1 * (UH[g.iuc(I + 1, J, K, 1)] - UH[g.iuc(I, J, K, 1)]);
            D1[N1M] = 24. * DX1 * (UH[g.iuc(1, J, K, 1)] - UH[g.iuc(N1M, J, K, 1)]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) RDP[g.ip(I, J, K)] = RDP[g.ip(I, J, K)] + X1[I] / DT;
        }
    }
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 1; K <= N3M - 1; K++)
                D3[K] = 24. * DX3 * (UH[g.iuc(I, J, K + 1, 3)] - UH[g.iuc(I, J, K, 3)]);
            D3[N3M] = 24. * DX3 * (UH[g.iuc(I, J, 1, 3)] - UH[g.iuc(I, J, N3M, 3)]);
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) RDP[g.ip(I, J, K)] = RDP[g.ip(I, J, K)] + X3[K] / DT;
        }
    }
}

// GETDP (compact3d.f:9271-9441)
void getdp(Orc &g, double *DP, const double *RDP) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N1MH = g.N1MH, N3MH = g.N3MH;
    const long M3MD = N3M + 2;
    auto coef = [&](int i, int k, int j) -> cplx & {
        return g.COEF[(i - 1) + (size_t)N1M * ((k - 1) + (size_t)N3M * (j - 1))];
    };
    auto frdp = [&](int i, int j, int kk) -> double & {
        return g.FRDP[(i - 1) + (size_t)g.N1 * ((j - 1) + (size_t)g.N2 * (kk - 1))];
    };
    auto fdp = [&](int i, int j, int kk) -> double & {
        return g.FDP[(i - 1) + (size_t)g.N1 * ((j - 1) + (size_t)g.N2 * (kk - 1))];
    };
    (void)M3MD;
#pragma omp parallel for
    for (int J = 1; J <= N2M; J++) {
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) coef(I, K, J) = cplx(RDP[g.ip(I, J, K)], 0.0);
        dft2d(N1M, N3M, &coef(1, 1, J), -1);
        for (int K = 1; K <= N3MH; K++) {
            int KR = 2 * K - 1, KI = 2 * K;
            for (int I = 1; I <= N1M; I++) {
                frdp(I, J, KR) = coef(I, K, J).real();
                frdp(I, J, KI) = coef(I, K, J).imag();
            }
        }
    }
    // real parts
#pragma omp parallel for
    for (int K = 1; K <= N3MH; K++) {
        int KR = 2 * K - 1;
        std::vector<double> CMJ(N2M + 1), CCJ(N2M + 1), CPJ(N2M + 1), CFJ(N2M + 1);
        for (int I = 1; I <= N1M; I++) {
            for (int J = 1; J <= N2M; J++) {
                CMJ[J] = g.PMJ[J];
                CCJ[J] = g.PCJ[J] - g.AK3[K] - g.AK1[I];
                CPJ[J] = g.PPJ[J];
                CFJ[J] = frdp(I, J, KR);
                if (I == 1 && K == 1) {
                    CMJ[1] = 0.0;
                    CCJ[1] = 1.0;
                    CPJ[1] = 0.0;
                    CFJ[1] = 0.0;
                }
            }
            tdmap(CMJ.data(), CCJ.data(), CPJ.data(), CFJ.data(), N2M, CFJ.data());
            for (int J = 1; J <= N2M; J++) fdp(I, J, KR) = CFJ[J];
        }
    }
    // imaginary parts
#pragma omp parallel for
    for (int K = 1; K <= N3MH; K++) {
        int KI = 2 * K;
        std::vector<double> CMJ(N2M + 1), CCJ(N2M + 1), CPJ(N2M + 1), CFJ(N2M + 1);
        for (int I = 1; I <= N1M; I++) {
            for (int J = 1; J <= N2M; J++) {
                CMJ[J] = g.PMJ[J];
                CCJ[J] = g.PCJ[J] - g.AK3[K] - g.AK1[I];
                CPJ[J] = g.PPJ[J];
                CFJ[J] = frdp(I, J, KI);
                if ((I == 1 && K == 1) || (I == 1 && K == N3MH) || (I == N1MH && K == 1) ||
                    (I == N1MH && K == N3MH)) {
                    CMJ[J] = 0.0;
                    CCJ[J] = 1.0;
                    CPJ[J] = 0.0;
                    CFJ[J] = 0.0;
                }
            }
            tdmap(CMJ.data(), CCJ.data(), CPJ.data(), CFJ.data(), N2M, CFJ.data());
            for (int J = 1; J <= N2M; J++) fdp(I, J, KI) = CFJ[J];
        }
    }
    // inverse
#pragma omp parallel for
    for (int J = 1; J <= N2M; J++) {
        for (int K = 1; K <= N3MH; K++) {
            int KR = 2 * K - 1, KI = 2 * K;
            for (int I = 1; I <= N1M; I++) coef(I, K, J) = cplx(fdp(I, J, KR), fdp(I, J, KI));
        }
        for (int K = N3MH + 1; K <= N3M; K++) {
            int KK = N3M - K + 2;
            for (int I = 1; I <= N1M; I++) {
                int II = N1M - I + 2;
                if (I == 1) II = 1;
                coef(I, K, J) = std::conj(coef(II, KK, J));
            }
        }
        dft2d(N1M, N3M, &coef(1, 1, J), +1);
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) DP[g.ip(I, J, K)] = coef(I, K, J).real() / (double)(N1M * N3M);
    }
}

// UPCALC (compact3d.f:1052-1238)
void upcalc(Orc &g, double *U, double *P, const double *UH, const double *DP, double DT,
            double *PRESG, double *PRESG3, bool bulk_forcing) {
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double DX1 = g.DX1, DX3 = g.DX3;
    const double *DY = g.DY.data(), *H = g.H.data();
    std::vector<double> pf(N3M + 1), pd(N3M + 1);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        double f = 0.0, d = 0.0;
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) {
                int IM = g.IMA[I];
                f = f + U[g.iuc(I, J, K, 1)] * DY[J] / DX3 / DX1;
                d = d + UH[g.iuc(I, J, K, 1)] * DY[J] / DX3 / DX1 -
                    DT * (DP[g.ip(I, J, K)] - DP[g.ip(IM, J, K)]) * DY[J] / DX3;
            }
        pf[K] = f;
        pd[K] = d;
    }
    double FLOW1 = 0.0, DMPRESG = 0.0;
    for (int K = 1; K <= N3M; K++) {
        FLOW1 += pf[K];
        DMPRESG += pd[K];
    }
    DMPRESG = (DMPRESG - FLOW1) / g.VOL / DT;
    if (!bulk_forcing) DMPRESG = 0.0;
    ConstLine L22x, L22z;
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 2; I <= N1M; I++) D1[I] = 24. * DX1 * (-DP[g.ip(I - 1, J, K)] + DP[g.ip(I, J, K)]);
            D1[1] = 24. * DX1 * (-DP[g.ip(N1M, J, K)] + DP[g.ip(1, J, K)]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) U[g.iuc(I, J, K, 1)] = UH[g.iuc(I, J, K, 1)] - DT * X1[I] - DT * DMPRESG;
        }
    }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            U[g.iuc(I, 0, K, 1)] = g.UBC[g.iubc(I, K, 1, 1)];
            U[g.iuc(I, N2, K, 1)] = g.UBC[g.iubc(I, K, 1, 2)];
        }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 2; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++)
                U[g.iuc(I, J, K, 2)] = UH[g.iuc(I, J, K, 2)] - DT * (DP[g.ip(I, J, K)] - DP[g.ip(I, J - 1, K)]) / H[J];
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            U[g.iuc(I, 1, K, 2)] = g.UBC[g.iubc(I, K, 2, 1)];
            U[g.iuc(I, N2, K, 2)] = g.UBC[g.iubc(I, K, 2, 2)];
        }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        int KM = g.KMA[K];
        double f = 0.0, d = 0.0;
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) {
                f = f + U[g.iuc(I, J, K, 3)] * DY[J] / DX1 / DX3;
                d = d + UH[g.iuc(I, J, K, 3)] * DY[J] / DX3 / DX1 -
                    DT * (DP[g.ip(I, J, K)] - DP[g.ip(I, J, KM)]) * DY[J] / DX1;
            }
        pf[K] = f;
        pd[K] = d;
    }
    double FLOW3 = 0.0, DMPRESG3 = 0.0;
    for (int K = 1; K <= N3M; K++) {
        FLOW3 += pf[K];
        DMPRESG3 += pd[K];
    }
    DMPRESG3 = (DMPRESG3 - FLOW3) / g.VOL / DT;
    if (!bulk_forcing) DMPRESG3 = 0.0;
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int K = 2; K <= N3M; K++) D3[K] = 24. * DX3 * (-DP[g.ip(I, J, K - 1)] + DP[g.ip(I, J, K)]);
            D3[1] = 24. * DX3 * (-DP[g.ip(I, J, N3M)] + DP[g.ip(I, J, 1)]);
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) U[g.iuc(I, J, K, 3)] = UH[g.iuc(I, J, K, 3)] - DT * X3[K] - DT * DMPRESG3;
        }
    }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) {
            U[g.iuc(I, 0, K, 3)] = g.UBC[g.iubc(I, K, 3, 1)];
            U[g.iuc(I, N2, K, 3)] = g.UBC[g.iubc(I, K, 3, 2)];
        }
    if (P) {
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++)
            for (int J = 1; J <= N2M; J++)
                for (int I = 1; I <= N1M; I++) P[g.ip(I, J, K)] = P[g.ip(I, J, K)] + DP[g.ip(I, J, K)];
    }
    if (PRESG) *PRESG = *PRESG + DMPRESG;
    if (PRESG3) *PRESG3 = *PRESG3 + DMPRESG3;
}

}  // namespace

// ==================================================================================
// extern "C" interface used by the tests (ctypes) and by bench.py's CPU baseline.
// ==================================================================================
extern "C" {

struct orc_handle;

void *orc_create(const c3d_grid *gr) {
    if (!gr || gr->n1 < 5 || gr->n2 < 4 || gr->n3 < 5) return nullptr;
    Orc *g = new Orc();
    g->N1 = gr->n1;
    g->N2 = gr->n2;
    g->N3 = gr->n3;
    g->N1M = g->N1 - 1;
    g->N2M = g->N2 - 1;
    g->N3M = g->N3 - 1;
    g->ALX = gr->alx;
    g->ALY = gr->aly;
    g->ALZ = gr->alz;
    g->VOL = gr->vol;
    g->DX1 = gr->dx1;
    g->DX3 = gr->dx3;
    g->DX1Q = g->DX1 * g->DX1;
    g->DX3Q = g->DX3 * g->DX3;
    g->RE = gr->re;
    g->FILES = gr->files;
    g->WMODEL = gr->wmodel;
    g->IFWALL = 0;
    int N2 = g->N2;
    g->Y.assign(gr->y, gr->y + N2 + 1);
    g->DY.assign(gr->dy, gr->dy + N2 + 1);
    auto one = [&](std::vector<double> &v, const double *src) {
        v.assign(N2 + 1, 0.0);
        for (int j = 1; j <= N2; j++) v[j] = src[j - 1];
    };
    one(g->H, gr->h);
    one(g->HM, gr->hm);
    one(g->HC, gr->hc);
    one(g->HP, gr->hp);
    one(g->DYM, gr->dym);
    one(g->DYC, gr->dyc);
    one(g->DYP, gr->dyp);
    setup_indices(*g);
    setup_wave(*g);
    g->su1 = g->N1 + 1;
    g->su2 = (long)(g->N1 + 1) * (g->N2 + 1);
    g->su3 = g->su2 * (g->N3 + 1);
    g->sp1 = g->N1;
    g->sp2 = (long)g->N1 * g->N2;
    size_t nu = (size_t)g->su3 * 3, ns = (size_t)g->su3, np = (size_t)g->sp2 * g->N3;
    g->UBC.assign((size_t)(g->N1 + 1) * (g->N3 + 1) * 6, 0.0);
    g->TAUW.assign((size_t)(g->N1 + 1) * (g->N3 + 1) * 2, 0.0);
    g->TAUB.assign((size_t)(g->N1 + 1) * (g->N3 + 1) * 2, 0.0);
    g->SMAGC.assign((size_t)g->N2 + 1, 0.0);
    g->UH.assign(nu, 0.0);
    g->HH2.assign(nu, 0.0);
    g->RUH1.assign(ns, 0.0);
    g->RUH2.assign(ns, 0.0);
    g->RUH3.assign(ns, 0.0);
    g->DP.assign(np, 0.0);
    g->RDP.assign(np, 0.0);
    g->FRDP.assign((size_t)g->N1 * g->N2 * (g->N3M + 2), 0.0);
    g->FDP.assign((size_t)g->N1 * g->N2 * (g->N3M + 2), 0.0);
    g->COEF.assign((size_t)g->N1M * g->N3M * g->N2M, cplx(0, 0));
    return g;
}

void orc_destroy(void *h) { delete (Orc *)h; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_wall(void *h, const double *tauw, const double *taub, int ifwall) {
    Orc &g = *(Orc *)h;
    if (tauw) std::memcpy(g.TAUW.data(), tauw, g.TAUW.size() * sizeof(double));
    if (taub) std::memcpy(g.TAUB.data(), taub, g.TAUB.size() * sizeof(double));
    g.IFWALL = ifwall;
}

// TAUW, TAUB (0:M1,0:M3,2) and /WSMEM/ WSM(1:3) as the step left them (null: skip).
void orc_get_wall(void *h, double *tauw, double *taub, double *wsm) {
    Orc &g = *(Orc *)h;
    if (tauw) std::memcpy(tauw, g.TAUW.data(), g.TAUW.size() * sizeof(double));
    if (taub) std::memcpy(taub, g.TAUB.data(), g.TAUB.size() * sizeof(double));
    if (wsm) std::memcpy(wsm, g.WSM, 3 * sizeof(double));
}
void orc_set_wsm(void *h, const double *wsm) { std::memcpy(((Orc *)h)->WSM, wsm, 3 * sizeof(double)); }
void orc_set_wall_iter_cap(void *h, int cap) { ((Orc *)h)->wall_iter_cap = cap; }

// The SGS model alone (SGSDY for FILES=1, SGSCS for FILES=2, SGSSD for FILES=3) on U, after GETUP's zeroing
// of SGSVIS; smagc (length N2M, may be null) receives SMAGC(1:N2M).
// DQRRT's BETA for x^n + pa[0] x^(n-1) + ... + pa[n-1] (n <= 8), EPS as given; wr/wi
// (may be null) receive CHHQR's eigenvalues and the return value is CHHQR's flag.
int orc_dqrrt(const double *pa, int n, double eps, double *beta, double *wr, double *wi) {
    if (n < 1 || n > 8) return -1;
    std::vector<double> B((size_t)n * n, 0.0), WR(n, 0.0), WI(n, 0.0);
    for (int J = 1; J <= n; J++) B[(size_t)n * (J - 1)] = -pa[J - 1];
    for (int I = 1; I <= n - 1; I++) B[I + (size_t)n * (I - 1)] = 1.0;
    const int ok = chhqr(B.data(), n, WR.data(), WI.data(), eps);
    for (int J = 0; J < n; J++) {
        if (wr) wr[J] = WR[J];
        if (wi) wi[J] = WI[J];
    }
    *beta = dqrrt(pa, n, eps);
    return ok;
}

// FILTER (four = 0) or FILTER4 (four = 1) in place on n fields of N1M x N3M (x fastest)
void orc_filter(void *h, int four, double *F, int n) {
    Orc &g = *(Orc *)h;
    std::vector<double> v(F, F + (size_t)g.N1M * g.N3M * n);
    if (four) filter4(g, v, n);
    else filter(g, v, n);
    std::copy(v.begin(), v.end(), F);
}

// WALLMODEL_IWMLES_SMOOTH: the driver's CFLMAX (its initial filter time scale) and the
// per-point state (IW_NS slots of N1M N3M values, I fastest)
void orc_set_cflmax(void *h, double cflmax) { ((Orc *)h)->CFLMAX = cflmax; }
int orc_iwm_slots() { return IW_NS; }
void orc_get_iwm(void *h, double *out) {
    Orc &g = *(Orc *)h;
    std::copy(g.IWM.begin(), g.IWM.end(), out);
}

// ----------------------------------------------------------------------------------
// Lagrangian particles (compact3d.f:11817-12894, 2029-2075).  The reference's time loop
// has the calls commented out (GET_PAR at 128, SOURCE_PAR at 1026); these restate its
// deterministic part for the tests: CALC_UX_4RK's step (FORCE_PAR's Clift-Gauvin drag
// and gravity, INDEX_IJK/INTERPOLAT at every stage, the periodic shifts by DIAM_P, the
// explicit Euler step from the start when a stage leaves the channel), BC_PAR's periodic
// shifts and top-wall reflection, with a bottom-wall impact flagged (the reference
// calls SPLASH there, which draws from RAN2 seeded by CPU_TIME), and SOURCE_PAR's
// two-way coupling terms.  PAR is (6, N): x, y, z, u, v, w.
// ----------------------------------------------------------------------------------
struct ParConst {
    double DIAM_P, TAU_P, MASS_P, HHH;
};
static ParConst par_const(const Orc &g, double diam_m, double dens, double hhh) {
    ParConst c;
    const double PI = 3.141592653;   // INIT_PAR's PI
    c.DIAM_P = diam_m / hhh;
    c.MASS_P = dens * PI * std::pow(c.DIAM_P, 3) / 6.;
    c.TAU_P = dens * std::pow(c.DIAM_P, 2) / 18. * g.RE;
    c.HHH = hhh;
    return c;
}

// FORCE_PAR (compact3d.f:12320-12350)
static void force_par(const Orc &g, const ParConst &c, double UP, double VP, double WP, double UF, double VF,
                      double WF, double &QU, double &QV, double &QW) {
    const double VISCOS = 0.000015;
    const double REP = std::sqrt(std::pow(UF - UP, 2) + std::pow(VF - VP, 2) + std::pow(WF - WP, 2)) * c.DIAM_P * g.RE;
    const double FCOR = 1. + 0.15 * std::pow(REP, 0.687) + 0.0175 * std::pow(1. + 42500 * std::pow(REP, -1.16), -1);
    QU = FCOR * (UF - UP) / c.TAU_P;
    QV = -9.8 / std::pow(VISCOS * g.RE / c.HHH, 2);
    QV = FCOR * (VF - VP) / c.TAU_P + QV;
    QW = FCOR * (WF - WP) / c.TAU_P;
}

// the fluid velocity at a particle; a point INDEX_IJK finds no cell for (a particle left
// below the bottom wall, which the reference hands to SPLASH) gets NaN, where the
// reference would read outside its arrays
static void par_fluid(const Orc &g, const Mesh02 &m, const double *U, double XP, double YP, double ZP, double &UF,
                      double &VF, double &WF) {
    int IP, JP, KP;
    index_ijk(g, m, XP, YP, ZP, IP, JP, KP);
    if (IP < 0 || JP < 0 || KP < 0) {
        UF = VF = WF = std::nan("");
        return;
    }
    UF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 1);
    VF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 2);
    WF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 3);
}

void orc_particles_advance(void *h, const double *U, int n, double *PAR, double diam_m, double dens, double hhh,
                           double DT_P, int *impact) {
    Orc &g = *(Orc *)h;
    const Mesh02 m = mesh02(g);
    const ParConst c = par_const(g, diam_m, dens, hhh);
    const double D = c.DIAM_P, ALX = g.ALX, ALY = g.ALY, ALZ = g.ALZ;
    auto wrap = [&](double &XP, double &ZP, double one) {
        if (XP > (ALX - 0.5 * D)) XP = one * D + XP - ALX;
        if (XP < (0.5 * D)) XP = ALX - D + XP;
        if (ZP > (ALZ - 0.5 * D)) ZP = one * D + ZP - ALZ;
        if (ZP < (0.5 * D)) ZP = ALZ - D + ZP;
    };
    for (int II = 0; II < n; II++) {
        double *P = PAR + 6 * (size_t)II;
        double QXRK = 0., QYRK = 0., QZRK = 0., QURK = 0., QVRK = 0., QWRK = 0.;
        double XP = P[0], YP = P[1], ZP = P[2], UP = P[3], VP = P[4], WP = P[5], UF, VF, WF, QU, QV, QW;
        bool euler = YP < 0.5 * D || YP > ALY - 0.5 * D;
        const double cs[4] = {0.5, 0.5, 1.0, 0.0}, ws[4] = {1.0, 2.0, 2.0, 1.0};
        for (int stg = 0; stg < 4 && !euler; stg++) {
            wrap(XP, ZP, 1.0);
            par_fluid(g, m, U, XP, YP, ZP, UF, VF, WF);
            force_par(g, c, UP, VP, WP, UF, VF, WF, QU, QV, QW);
            QXRK = QXRK + ws[stg] * UP;
            QYRK = QYRK + ws[stg] * VP;
            QZRK = QZRK + ws[stg] * WP;
            QURK = QURK + ws[stg] * QU;
            QVRK = QVRK + ws[stg] * QV;
            QWRK = QWRK + ws[stg] * QW;
            if (stg == 3) break;
            XP = P[0] + cs[stg] * DT_P * UP;
            YP = P[1] + cs[stg] * DT_P * VP;
            ZP = P[2] + cs[stg] * DT_P * WP;
            UP = P[3] + cs[stg] * DT_P * QU;
            VP = P[4] + cs[stg] * DT_P * QV;
            WP = P[5] + cs[stg] * DT_P * QW;
            euler = YP < 0.5 * D || YP > ALY - 0.5 * D;
        }
        if (!euler) {
            XP = P[0] + DT_P * QXRK / 6.;
            YP = P[1] + DT_P * QYRK / 6.;
            ZP = P[2] + DT_P * QZRK / 6.;
            UP = P[3] + DT_P * QURK / 6.;
            VP = P[4] + DT_P * QVRK / 6.;
            WP = P[5] + DT_P * QWRK / 6.;
        } else {   // label 100: explicit Euler from the particle's state
            UP = P[3];
            VP = P[4];
            WP = P[5];
            par_fluid(g, m, U, P[0], P[1], P[2], UF, VF, WF);
            force_par(g, c, UP, VP, WP, UF, VF, WF, QU, QV, QW);
            XP = P[0] + DT_P * UP;
            YP = P[1] + DT_P * VP;
            ZP = P[2] + DT_P * WP;
            UP = P[3] + DT_P * QU;
            VP = P[4] + DT_P * QV;
            WP = P[5] + DT_P * QW;
        }
        P[0] = XP, P[1] = YP, P[2] = ZP, P[3] = UP, P[4] = VP, P[5] = WP;
        // BC_PAR (12352-12470)
        if (P[0] > (ALX - 0.5 * D)) P[0] = 1.0 * D + P[0] - ALX;
        if (P[0] < (0.5 * D)) P[0] = ALX - D + P[0];
        if (P[2] > (ALZ - 0.5 * D)) P[2] = 1.0 * D + P[2] - ALZ;
        if (P[2] < (0.5 * D)) P[2] = ALZ - D + P[2];
        if (P[1] > (ALY - 0.5 * D) && P[4] >= 0.0) {
            P[4] = -P[4];
            P[1] = 2. * ALY - D - P[1];
        }
        impact[II] = (P[1] < (0.5 * D) && P[4] <= 0.0) ? 1 : 0;
    }
}

// SOURCE_PAR (compact3d.f:2029-2075): the terms the particles add to RUH1..3 (Fortran
// (0:M1,0:M2,0:M3) each, added to what is passed), QQ = 1000 and gravity G.
void orc_particles_source(void *h, const double *U, int n, const double *PAR, double diam_m, double dens, double hhh,
                          double *RUH1, double *RUH2, double *RUH3) {
    Orc &g = *(Orc *)h;
    const Mesh02 m = mesh02(g);
    const ParConst c = par_const(g, diam_m, dens, hhh);
    const double QQ = 1000.0, G = 9.8 / std::pow(g.RE * 1.5 / 100000 / hhh, 2);
    for (int II = 0; II < n; II++) {
        const double *P = PAR + 6 * (size_t)II;
        double XP = P[0], YP = P[1], ZP = P[2], UF, VF, WF, QU, QV, QW;
        int IP, JP, KP;
        index_ijk(g, m, XP, YP, ZP, IP, JP, KP);
        if (IP < 0 || JP < 0 || KP < 0) continue;   // outside the channel: no cell to deposit in
        UF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 1);
        VF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 2);
        WF = interpolat(g, m, XP, YP, ZP, IP, JP, KP, U, 3);
        force_par(g, c, P[3], P[4], P[5], UF, VF, WF, QU, QV, QW);
        int IPP = IP, JPP = JP, KPP = KP;
        if (XP > m.XC[IP]) IPP = g.IPA[IP];
        if (YP > m.YC[JP]) JPP = g.JPA[JP];
        if (ZP > m.ZC[KP]) KPP = g.KPA[KP];
        RUH1[g.iu(IPP, JP, KP)] -= c.MASS_P * QQ * QU * g.DX1 * g.DX3 / g.H[JP];
        RUH2[g.iu(IP, JPP, KP)] -= c.MASS_P * QQ * (QV + G) * g.DX1 * g.DX3 / g.H[JPP];
        RUH3[g.iu(IP, JP, KPP)] -= c.MASS_P * QQ * QW * g.DX1 * g.DX3 / g.H[JP];
    }
}

// SGSSD's BETA(1:N2M) of the last SGS evaluation
void orc_get_beta(void *h, double *beta) {
    Orc &g = *(Orc *)h;
    for (int J = 1; J <= g.N2M; J++) beta[J - 1] = J < (int)g.BETA.size() ? g.BETA[J] : 0.0;
}

int orc_sgs(void *h, const double *U, double *SGSVIS, double *smagc) {
    Orc &g = *(Orc *)h;
    for (int K = 1; K <= g.N3; K++)
        for (int J = 0; J <= g.N2; J++)
            for (int I = 1; I <= g.N1; I++) SGSVIS[g.iu(I, J, K)] = 0.0;
    if (g.FILES == 1) sgsdy(g, U, SGSVIS);
    else if (g.FILES == 2) sgscs(g, U, SGSVIS);
    else if (g.FILES == 3) sgssd(g, U, SGSVIS);
    else return C3D_EINVAL;
    if (smagc)
        for (int J = 1; J <= g.N2M; J++) smagc[J - 1] = g.SMAGC[J];
    return 0;
}

// The SGS-flux contributions alone: HH (0:M1,0:M2,0:M3,3) is zeroed, then receives the
// terms RHS1/2/3 subtract from HH for the given SGSVIS (wall planes as passed).
int orc_sgs_rhs(void *h, const double *U, const double *SGSVIS, double *HH) {
    Orc &g = *(Orc *)h;
    std::memset(HH, 0, (size_t)g.su3 * 3 * sizeof(double));
    sgs_rhs1(g, U, HH, SGSVIS);
    sgs_rhs2_vis22(g, U, HH, SGSVIS);
    sgs_rhs2(g, U, HH, SGSVIS);
    sgs_rhs3(g, U, HH, SGSVIS);
    return 0;
}

// The operators of c3d_op_apply in the reference's arithmetic: the compact solves by
// bordered LU (CTDMA11/CTDMA33, compact3d.f:8952-9046) with the right-hand sides of
// RHS1 loops 20/50, the y stencils of RHS1 loop 10 / RHS2 loop 10, and GETDP.  F and X
// are (0:M1,0:M2,0:M3); X receives J = 1..N2M (2..N2M for DY1) and zeros elsewhere.
int orc_operator(void *h, int op, const double *F, double *X) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double DX1 = g.DX1, DX3 = g.DX3, DX1Q = g.DX1Q, DX3Q = g.DX3Q;
    std::memset(X, 0, (size_t)g.su3 * sizeof(double));
    auto f = [&](int i, int j, int k) { return F[g.iu(i, j, k)]; };
    ConstLine L;
    if (op >= 1 && op <= 3) {
        L.set(N1M, 1.0, op == 1 ? 22.0 : op == 2 ? 10.0 : 6.0, 1.0);
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++) {
            std::vector<double> D(N1M + 1), Y(N1M + 1);
            for (int J = 1; J <= N2M; J++) {
                for (int I = 1; I <= N1M; I++) {
                    const int IP = g.IPA[I], IM = g.IMA[I];
                    if (op == 1) D[I] = 24. * DX1 * (f(IP, J, K) - f(I, J, K));
                    else if (op == 2) D[I] = 12. * DX1Q * (f(IM, J, K) - 2. * f(I, J, K) + f(IP, J, K));
                    else D[I] = 4. * (f(I, J, K) + f(IP, J, K));
                }
                ctdma_bordered(N1M, L.A.data(), L.B.data(), L.C.data(), D.data(), Y.data());
                for (int I = 1; I <= N1M; I++) X[g.iu(I, J, K)] = Y[I];
            }
        }
    } else if (op >= 4 && op <= 6) {
        L.set(N3M, 1.0, op == 4 ? 22.0 : op == 5 ? 10.0 : 6.0, 1.0);
#pragma omp parallel for
        for (int I = 1; I <= N1M; I++) {
            std::vector<double> D(N3M + 1), Y(N3M + 1);
            for (int J = 1; J <= N2M; J++) {
                for (int K = 1; K <= N3M; K++) {
                    const int KP = g.KPA[K], KM = g.KMA[K];
                    if (op == 4) D[K] = 24. * DX3 * (f(I, J, KP) - f(I, J, K));
                    else if (op == 5) D[K] = 12. * DX3Q * (f(I, J, KM) - 2. * f(I, J, K) + f(I, J, KP));
                    else D[K] = 4. * (f(I, J, K) + f(I, J, KP));
                }
                ctdma_bordered(N3M, L.A.data(), L.B.data(), L.C.data(), D.data(), Y.data());
                for (int K = 1; K <= N3M; K++) X[g.iu(I, J, K)] = Y[K];
            }
        }
    } else if (op == 7 || op == 8) {
#pragma omp parallel for
        for (int K = 1; K <= N3M; K++)
            for (int J = (op == 7 ? 2 : 1); J <= N2M; J++)
                for (int I = 1; I <= N1M; I++) {
                    if (op == 7) X[g.iu(I, J, K)] = (f(I, J, K) - f(I, J - 1, K)) / g.H[J];
                    else X[g.iu(I, J, K)] = g.HP[J] * f(I, J + 1, K) - g.HC[J] * f(I, J, K) + g.HM[J] * f(I, J - 1, K);
                }
    } else if (op == 9) {
        std::vector<double> RDP((size_t)g.sp2 * g.N3, 0.0), DP((size_t)g.sp2 * g.N3, 0.0);
        for (int K = 1; K <= N3M; K++)
            for (int J = 1; J <= N2M; J++)
                for (int I = 1; I <= N1M; I++) RDP[g.ip(I, J, K)] = f(I, J, K);
        getdp(g, DP.data(), RDP.data());
        for (int K = 1; K <= N3M; K++)
            for (int J = 1; J <= N2M; J++)
                for (int I = 1; I <= N1M; I++) X[g.iu(I, J, K)] = DP[g.ip(I, J, K)];
    } else {
        return C3D_EINVAL;
    }
    return 0;
}

// WALLMODEL_INSTANT alone on U (TAUW, TAUB, WSM(1) are updated in the handle).
int orc_wallmodel(void *h, const double *U) { return wallmodel(*(Orc *)h, U); }

// GETUP (compact3d.f:879-960).  U, P, HH, SGSVIS are Fortran arrays (SGSVIS may be null;
// an internal array is used then).  With an SGS model (FILES != 0) the driver's WALLSS
// call that precedes GETUP when WMODEL == 0 (compact3d.f:125) is folded in here, so
// SGSCS sees the wall shear of the current field as in the reference's time loop.
int orc_getup(void *h, double *U, double *P, double *HH, double *SGSVIS, int NTIME, double DT,
              double *PRESG, double *PRESG3) {
    Orc &g = *(Orc *)h;
    (void)NTIME;
    if (g.FILES < 0 || g.FILES > 3 || g.WMODEL < 0 || g.WMODEL > 5) return C3D_EINVAL;
    if (g.WMODEL == 4 && g.N3M > g.N1M) return C3D_EINVAL;   // WERNER indexes INDX(N1M) with K
    const int N1 = g.N1, N2 = g.N2, N3 = g.N3;
    double *UH = g.UH.data(), *HH2 = g.HH2.data();
    if (g.FILES != 0 && !SGSVIS) {
        g.SGS.assign((size_t)g.su3, 0.0);
        SGSVIS = g.SGS.data();
    }
    if (g.FILES != 0 && g.WMODEL == 0) wallss_common(g, U, g.WSM);
    for (int NV = 1; NV <= 3; NV++) {
#pragma omp parallel for
        for (int K = 1; K <= N3; K++)
            for (int J = 1; J <= N2; J++)
                for (int I = 1; I <= N1; I++) UH[g.iuc(I, J, K, NV)] = 0.0;
    }
#pragma omp parallel for
    for (int K = 1; K <= N3; K++)
        for (int J = 1; J <= N2; J++)
            for (int I = 1; I <= N1; I++) g.DP[g.ip(I, J, K)] = 0.0;
    if (SGSVIS) {
#pragma omp parallel for
        for (int K = 1; K <= N3; K++)
            for (int J = 0; J <= N2; J++)
                for (int I = 1; I <= N1; I++) SGSVIS[g.iu(I, J, K)] = 0.0;
    }
    for (int NV = 1; NV <= 3; NV++) {
#pragma omp parallel for
        for (int K = 1; K <= N3; K++)
            for (int J = 1; J <= N2; J++)
                for (int I = 1; I <= N1; I++) {
                    long id = g.iuc(I, J, K, NV);
                    HH2[id] = HH[id];
                    HH[id] = 0.0;
                }
    }
    if (g.FILES == 1) sgsdy(g, U, SGSVIS);
    if (g.FILES == 2) sgscs(g, U, SGSVIS);
    if (g.FILES == 3) sgssd(g, U, SGSVIS);
    int status = 0;
    if (g.FILES != 0) {   // WALL_MODEL (compact3d.f:1952-2026)
        if (g.WMODEL == 0) {
            g.IFWALL = 0;
            wallss_common(g, U, g.WSM);
        } else {
            status = wallmodel(g, U, P, NTIME, DT, *PRESG, *PRESG3);
            g.IFWALL = 1;
        }
    }
    const double *SV = g.FILES != 0 ? SGSVIS : nullptr;
    bcond(g, U, SGSVIS);
    // UHCALC
    rhs1(g, U, P, HH, HH2, g.RUH1.data(), *PRESG, SV);
    rhs2(g, U, P, HH, HH2, g.RUH2.data(), SV);
    rhs3(g, U, P, HH, HH2, g.RUH3.data(), *PRESG3, SV);
    getuh(g, U, UH, g.RUH1.data(), 1, DT);
    getuh(g, U, UH, g.RUH2.data(), 2, DT);
    getuh(g, U, UH, g.RUH3.data(), 3, DT);
    // end of GETUH3: UH = U + UH
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) {
                UH[g.iuc(I, J, K, 1)] = U[g.iuc(I, J, K, 1)] + UH[g.iuc(I, J, K, 1)];
                UH[g.iuc(I, J, K, 3)] = U[g.iuc(I, J, K, 3)] + UH[g.iuc(I, J, K, 3)];
            }
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 2; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) UH[g.iuc(I, J, K, 2)] = U[g.iuc(I, J, K, 2)] + UH[g.iuc(I, J, K, 2)];
    // DPCALC
    rhsdp(g, g.RDP.data(), UH, DT);
    getdp(g, g.DP.data(), g.RDP.data());
    // UPCALC
    upcalc(g, U, P, UH, g.DP.data(), DT, PRESG, PRESG3, true);
    return status;
}

// Pressure projection of U (RHSDP + GETDP + UPCALC with UH = U, DT = 1, no bulk forcing);
// used to make a synthetic initial condition discretely divergence-free.
int orc_project(void *h, double *U) {
    Orc &g = *(Orc *)h;
    bcond(g, U, nullptr);
    std::vector<double> UH(U, U + g.su3 * 3);
    rhsdp(g, g.RDP.data(), UH.data(), 1.0);
    getdp(g, g.DP.data(), g.RDP.data());
    upcalc(g, U, nullptr, UH.data(), g.DP.data(), 1.0, nullptr, nullptr, false);
    return 0;
}

// Individual stages, for unit tests.
int orc_bcond(void *h, double *U) {
    bcond(*(Orc *)h, U, nullptr);
    return 0;
}
int orc_getdp(void *h, const double *RDP, double *DP) {
    getdp(*(Orc *)h, DP, RDP);
    return 0;
}
int orc_rhsdp(void *h, const double *UH, double DT, double *RDP) {
    rhsdp(*(Orc *)h, RDP, UH, DT);
    return 0;
}

// DIVCHECK (compact3d.f:9049-9131)
double orc_divcheck(void *h, const double *U) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double DX1 = g.DX1, DX3 = g.DX3;
    std::vector<double> DIV((size_t)N1M * N2M * N3M);
    auto div = [&](int i, int j, int k) -> double & {
        return DIV[(i - 1) + (size_t)N1M * ((j - 1) + (size_t)N2M * (k - 1))];
    };
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++)
                div(I, J, K) = (U[g.iuc(I, J + 1, K, 2)] - U[g.iuc(I, J, K, 2)]) / g.DY[J];
    ConstLine L22x, L22z;
    L22x.set(N1M, 1.0, 22.0, 1.0);
    L22z.set(N3M, 1.0, 22.0, 1.0);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        std::vector<double> D1(N1M + 1), X1(N1M + 1);
        for (int J = 1; J <= N2M; J++) {
            for (int I = 1; I <= N1M - 1; I++) D1[I] = 24. * DX1 * (U[g.iuc(I + 1, J, K, 1)] - U[g.iuc(I, J, K, 1)]);
            D1[N1M] = 24. * DX1 * (U[g.iuc(1, J, K, 1)] - U[g.iuc(N1M, J, K, 1)]);
            ctdma_bordered(N1M, L22x.A.data(), L22x.B.data(), L22x.C.data(), D1.data(), X1.data());
            for (int I = 1; I <= N1M; I++) div(I, J, K) = div(I, J, K) + X1[I];
        }
    }
    std::vector<double> mx(N1M + 1, 0.0);
#pragma omp parallel for
    for (int I = 1; I <= N1M; I++) {
        std::vector<double> D3(N3M + 1), X3(N3M + 1);
        double m = 0.0;
        for (int J = 1; J <= N2M; J++) {
            for (int K = 1; K <= N3M - 1; K++) D3[K] = 24. * DX3 * (U[g.iuc(I, J, K + 1, 3)] - U[g.iuc(I, J, K, 3)]);
            D3[N3M] = 24. * DX3 * (U[g.iuc(I, J, 1, 3)] - U[g.iuc(I, J, N3M, 3)]);
            ctdma_bordered(N3M, L22z.A.data(), L22z.B.data(), L22z.C.data(), D3.data(), X3.data());
            for (int K = 1; K <= N3M; K++) {
                div(I, J, K) = div(I, J, K) + X3[K];
                m = std::max(std::fabs(div(I, J, K)), m);
            }
        }
        mx[I] = m;
    }
    double DIVMAX = 0.0;
    for (int I = 1; I <= N1M; I++) DIVMAX = std::max(mx[I], DIVMAX);
    return DIVMAX;
}

// CFL (compact3d.f:9138-9169)
double orc_cfl(void *h, const double *U) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    std::vector<double> mk(N3M + 1, 0.0);
#pragma omp parallel for
    for (int K = 1; K <= N3M; K++) {
        int KP = g.KPA[K];
        double m = 0.0;
        for (int J = 1; J <= N2M; J++) {
            int JP = J + 1;
            for (int I = 1; I <= N1M; I++) {
                int IP = g.IPA[I];
                double CFLL = std::fabs(U[g.iuc(I, J, K, 1)] + U[g.iuc(IP, J, K, 1)]) * 0.5 * g.DX1 +
                              std::fabs(U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5 / g.DY[J] +
                              std::fabs(U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, KP, 3)]) * 0.5 * g.DX3;
                m = std::max(m, CFLL);
            }
        }
        mk[K] = m;
    }
    double CFLM = 0.0;
    for (int K = 1; K <= N3M; K++) CFLM = std::max(CFLM, mk[K]);
    return CFLM;
}

// CHKMF (compact3d.f:9463-9503)
void orc_chkmf(void *h, const double *U, double *flow1, double *flow3) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    double F1 = 0.0, F3 = 0.0;
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) F1 = F1 + U[g.iuc(1, J, K, 1)] * g.DY[J] / g.DX3 / g.DX1;
    F1 = F1 / g.ALX / g.ALZ;
    for (int K = 1; K <= N3M; K++)
        for (int J = 1; J <= N2M; J++)
            for (int I = 1; I <= N1M; I++) F3 = F3 + U[g.iuc(I, J, 1, 3)] * g.DY[J] / g.DX1 / g.DX3;
    F3 = F3 / g.ALX / g.ALZ;
    *flow1 = F1;
    *flow3 = F3;
}

// WALLSS (compact3d.f:11077-11143)
void orc_wallss(void *h, const double *U, double *wsm) { wallss_common(*(Orc *)h, U, wsm); }

// ENERGY's plane statistics (compact3d.f:10003-10232), 29 per plane J = 1..N2M into
// out[(J-1)*29 + q]: 0-2 VM (cell-centre u, v, w), 3 PM, 4-6 WM (vorticity), 7-12 VRMS
// (uu, vv, ww, uv, uw, vw), 13 PRMS (pp), 14 PV (pv), 15-17 WRMS (vorticity squares),
// 18 U2V (uuv), 19 VW2 (vww), 20-22 VSKEW and 23-25 VFLAT (third and fourth central
// moments), 26-28 DUDY, DVDY, DWDY.  Plane means over K, I in that order, as the loops.
// ENERGY's 1-D spectra and two-point correlations (compact3d.f:10243-10515).  VM(J,L)
// and VRMS(J,L) = <v_L v_L> are the plane statistics of the cell-centre velocities
// (10095-10133, V at (J, J+1)); VMO (3 N2M, J fastest; null: VM) is the mean the spectra
// subtract.  XSPCTR(I,J,L) = sum_K |DFT_x(v_L - VMO)(I-1)|^2 / N1M / (PI DX1) / N3M over the
// x lines and ZSPCTR(K,J,L) likewise along z (/ N3M / (PI DX3) / N1M).  The correlations
// use VP = v_L - VM with V at (J, JPA(J)) (JPA(N2M) = N2M) and the points N1H = N1M/2+1,
// N3H = N3M/2+1: RXX(I,J,L) = sum_K VP(N1H,J,K) VP(I,J,K) / N3M / (VRMS - VM^2),
// RZZ(K,J,L) = sum_I VP(I,J,N3H) VP(I,J,K) / N1M / (VRMS - VM^2) and RXY(I,J,L) =
// sum_K VP(N1H,1,K) VP(I,J,K) / N3M / sqrt(VRMS - VM^2)(J) / sqrt(VRMS - VM^2)(1).
// Outputs are Fortran (N,N2M,3) arrays; any may be null.
void orc_plane_spectra(void *h, const double *U, const double *VMO, double *XS, double *ZS, double *RXX,
                       double *RZZ, double *RXY) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double NXZ = 1.0 / (double)(N1M * N3M), PI = std::acos(-1.0);
    std::vector<double> VM((size_t)(N2M + 1) * 4, 0.0), VRMS((size_t)(N2M + 1) * 4, 0.0);
    auto vm = [&](int J, int L) -> double & { return VM[(size_t)J * 4 + L]; };
    auto vr = [&](int J, int L) -> double & { return VRMS[(size_t)J * 4 + L]; };
    auto vc = [&](int I, int J, int K, int L, int JP) {   // cell-centre velocity
        if (L == 1) return (U[g.iuc(I, J, K, 1)] + U[g.iuc(g.IPA[I], J, K, 1)]) * 0.5;
        if (L == 2) return (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
        return (U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, g.KPA[K], 3)]) * 0.5;
    };
    for (int J = 1; J <= N2M; J++) {
        double s[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++)
                for (int L = 1; L <= 3; L++) {
                    const double v = vc(I, J, K, L, J + 1);
                    s[L] = s[L] + v;
                    q[L] = q[L] + v * v;
                }
        for (int L = 1; L <= 3; L++) {
            vm(J, L) = s[L] * NXZ;
            vr(J, L) = q[L] * NXZ;
        }
    }
    auto vmo = [&](int J, int L) { return VMO ? VMO[(size_t)(L - 1) * N2M + (J - 1)] : vm(J, L); };
    if (XS) {
        const double FS = PI * g.DX1;
        std::vector<cplx> c(N1M);
        for (int L = 1; L <= 3; L++)
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> acc(N1M, 0.0);
                for (int K = 1; K <= N3M; K++) {
                    for (int I = 1; I <= N1M; I++) c[I - 1] = cplx(vc(I, J, K, L, J + 1) - vmo(J, L), 0.0);
                    fft1d(N1M, -1, c.data(), 1);
                    for (int I = 0; I < N1M; I++) acc[I] = acc[I] + std::norm(c[I]) / N1M / FS;
                }
                for (int I = 0; I < N1M; I++) XS[I + (size_t)N1M * ((J - 1) + (size_t)N2M * (L - 1))] = acc[I] / (double)N3M;
            }
    }
    if (ZS) {
        const double FS = PI * g.DX3;
        std::vector<cplx> c(N3M);
        for (int L = 1; L <= 3; L++)
            for (int J = 1; J <= N2M; J++) {
                std::vector<double> acc(N3M, 0.0);
                for (int I = 1; I <= N1M; I++) {
                    for (int K = 1; K <= N3M; K++) c[K - 1] = cplx(vc(I, J, K, L, J + 1) - vmo(J, L), 0.0);
                    fft1d(N3M, -1, c.data(), 1);
                    for (int K = 0; K < N3M; K++) acc[K] = acc[K] + std::norm(c[K]) / N3M / FS;
                }
                for (int K = 0; K < N3M; K++) ZS[K + (size_t)N3M * ((J - 1) + (size_t)N2M * (L - 1))] = acc[K] / (double)N1M;
            }
    }
    const int N1H = N1M / 2 + 1, N3H = N3M / 2 + 1;
    auto vp = [&](int I, int J, int K, int L) { return vc(I, J, K, L, g.JPA[J]) - vm(J, L); };
    for (int L = 1; L <= 3; L++)
        for (int J = 1; J <= N2M; J++) {
            const double var = vr(J, L) - vm(J, L) * vm(J, L);
            if (RXX)
                for (int I = 1; I <= N1M; I++) {
                    double r = 0.0;
                    for (int K = 1; K <= N3M; K++) r = r + vp(N1H, J, K, L) * vp(I, J, K, L);
                    RXX[(I - 1) + (size_t)N1M * ((J - 1) + (size_t)N2M * (L - 1))] = r / (double)N3M / var;
                }
            if (RZZ)
                for (int K = 1; K <= N3M; K++) {
                    double r = 0.0;
                    for (int I = 1; I <= N1M; I++) r = r + vp(I, J, N3H, L) * vp(I, J, K, L);
                    RZZ[(K - 1) + (size_t)N3M * ((J - 1) + (size_t)N2M * (L - 1))] = r / (double)N1M / var;
                }
            if (RXY) {
                const double var1 = vr(1, L) - vm(1, L) * vm(1, L);
                for (int I = 1; I <= N1M; I++) {
                    double r = 0.0;
                    for (int K = 1; K <= N3M; K++) r = r + vp(N1H, 1, K, L) * vp(I, J, K, L);
                    RXY[(I - 1) + (size_t)N1M * ((J - 1) + (size_t)N2M * (L - 1))] =
                        r / (double)N3M / std::sqrt(var) / std::sqrt(var1);
                }
            }
        }
}

// ENERGY's quadrant analysis (compact3d.f:10560-10604): out[(J-1)*8 + q], Q(J,1..4) =
// -sum(u'v') / (N1M N3M) per sign quadrant of (u', v'), QP(J,1..4) = point counts /
// (N1M N3M); u' = u_c - VMP(J,1), v' = v_c - VMP(J,2) (VMP 2 N2M, J fastest; null: 0).
void orc_plane_quadrants(void *h, const double *U, const double *VMP, double *out) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double NXZ = 1.0 / (double)(N1M * N3M);
    for (int J = 1; J <= N2M; J++) {
        const int JP = J + 1;
        const double m1 = VMP ? VMP[J - 1] : 0.0, m2 = VMP ? VMP[N2M + J - 1] : 0.0;
        double UV[4] = {0, 0, 0, 0}, UVP[4] = {0, 0, 0, 0};
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                const double V1 = (U[g.iuc(I, J, K, 1)] + U[g.iuc(IP, J, K, 1)]) * 0.5;
                const double V2 = (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
                const double V1P = V1 - m1, V2P = V2 - m2;
                int q = -1;
                if (V1P > 0.0 && V2P > 0.0) q = 0;
                if (V1P < 0.0 && V2P > 0.0) q = 1;
                if (V1P < 0.0 && V2P < 0.0) q = 2;
                if (V1P > 0.0 && V2P < 0.0) q = 3;
                if (q >= 0) {
                    UV[q] = UV[q] + V1P * V2P;
                    UVP[q] = UVP[q] + 1.0;
                }
            }
        for (int q = 0; q < 4; q++) {
            out[(size_t)(J - 1) * 8 + q] = -UV[q] * NXZ;
            out[(size_t)(J - 1) * 8 + 4 + q] = UVP[q] * NXZ;
        }
    }
}

// ENERGY's wall-stress spectrum (compact3d.f:10394-10416): SPECTAUW(I,K,1) =
// |DFT2(TAUW(.,.,1) - UTAU^2)(I-1,K-1)|^2 / N1M / N3M / (PI DX3) / (PI DX1), Fortran
// (N1M, N3M); UTAU as the driver holds it (sqrt of the averaged wall stress).
void orc_wall_spectrum(void *h, double UTAU, double *out) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N3M = g.N3M;
    const double PI = std::acos(-1.0), FS = PI * g.DX1, FS1 = PI * g.DX3;
    std::vector<cplx> c((size_t)N1M * N3M);
    for (int K = 1; K <= N3M; K++)
        for (int I = 1; I <= N1M; I++) c[(I - 1) + (size_t)N1M * (K - 1)] = cplx(g.TAUW[g.itw(I, K, 1)] - UTAU * UTAU, 0.0);
    dft2d(N1M, N3M, c.data(), -1);
    for (size_t q = 0; q < c.size(); q++) out[q] = std::norm(c[q]) / N1M / N3M / FS1 / FS;
}

// ENERGY's 3-D two-point correlation (compact3d.f:10524-10556): RXYZ(I,J,K,L) =
// VP(N1H,N2H,N3H,L) VP(I,J,K,L) / sqrt(VRMS - VM^2)(J) / sqrt(VRMS - VM^2)(N2H), VP as in
// orc_plane_spectra; N2H = N2M/2 + 1 with ALY = 1, N2M/4 + 1 otherwise.  Fortran
// (N1M, N2M, N3M, 3).
void orc_corr3d(void *h, const double *U, double *out) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M;
    const double NXZ = 1.0 / (double)(N1M * N3M);
    auto vc = [&](int I, int J, int K, int L, int JP) {
        if (L == 1) return (U[g.iuc(I, J, K, 1)] + U[g.iuc(g.IPA[I], J, K, 1)]) * 0.5;
        if (L == 2) return (U[g.iuc(I, J, K, 2)] + U[g.iuc(I, JP, K, 2)]) * 0.5;
        return (U[g.iuc(I, J, K, 3)] + U[g.iuc(I, J, g.KPA[K], 3)]) * 0.5;
    };
    std::vector<double> VM((size_t)(N2M + 1) * 4, 0.0), VR((size_t)(N2M + 1) * 4, 0.0);
    for (int J = 1; J <= N2M; J++) {
        double s[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
        for (int K = 1; K <= N3M; K++)
            for (int I = 1; I <= N1M; I++)
                for (int L = 1; L <= 3; L++) {
                    const double v = vc(I, J, K, L, J + 1);
                    s[L] = s[L] + v;
                    q[L] = q[L] + v * v;
                }
        for (int L = 1; L <= 3; L++) {
            VM[(size_t)J * 4 + L] = s[L] * NXZ;
            VR[(size_t)J * 4 + L] = q[L] * NXZ;
        }
    }
    const int N1H = N1M / 2 + 1, N3H = N3M / 2 + 1, N2H = g.ALY == 1.0 ? N2M / 2 + 1 : N2M / 4 + 1;
    auto vp = [&](int I, int J, int K, int L) { return vc(I, J, K, L, g.JPA[J]) - VM[(size_t)J * 4 + L]; };
    for (int L = 1; L <= 3; L++) {
        const double ref = vp(N1H, N2H, N3H, L);
        const double sh = std::sqrt(VR[(size_t)N2H * 4 + L] - VM[(size_t)N2H * 4 + L] * VM[(size_t)N2H * 4 + L]);
        for (int K = 1; K <= N3M; K++)
            for (int J = 1; J <= N2M; J++) {
                const double sj = std::sqrt(VR[(size_t)J * 4 + L] - VM[(size_t)J * 4 + L] * VM[(size_t)J * 4 + L]);
                for (int I = 1; I <= N1M; I++)
                    out[(I - 1) + (size_t)N1M * ((J - 1) + (size_t)N2M * ((K - 1) + (size_t)N3M * (L - 1)))] =
                        ref * vp(I, J, K, L) / sj / sh;
            }
    }
}

void orc_plane_stats(void *h, const double *U, const double *P, double *out) {
    Orc &g = *(Orc *)h;
    const int N1M = g.N1M, N2M = g.N2M, N3M = g.N3M, N2 = g.N2;
    const double NXZ = 1.0 / (double)(N1M * N3M), DX1 = g.DX1, DX3 = g.DX3;
    const double *DY = g.DY.data(), *H = g.H.data();
    auto u = [&](int i, int j, int k, int c) { return U[g.iuc(i, j, k, c)]; };
    auto p = [&](int i, int j, int k) { return P[g.ip(i, j, k)]; };
    std::vector<double> VOR((size_t)3 * N1M * N2M * N3M);
    auto vor = [&](int i, int j, int k, int c) -> double & {
        return VOR[(((size_t)(c - 1) * N3M + (k - 1)) * N2M + (j - 1)) * N1M + (i - 1)];
    };
    for (int K = 1; K <= N3M; K++) {   // loop 10: vorticity at the cell centres
        const int KP = g.KPA[K], KM = g.KMA[K];
        for (int J = 1; J <= N2M; J++) {
            const int JP = J + 1, JM = J - 1;
            const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I], IM = g.IMA[I];
                double U1KP = 0.5 * (u(I, J, KP, 1) + u(IP, J, KP, 1));
                double U1KM = 0.5 * (u(I, J, KM, 1) + u(IP, J, KM, 1));
                double U2KP = 0.5 * (u(I, J, KP, 2) + u(I, JP, KP, 2));
                double U2KM = 0.5 * (u(I, J, KM, 2) + u(I, JP, KM, 2));
                double U2IP = 0.5 * (u(IP, J, K, 2) + u(IP, JP, K, 2));
                double U2IM = 0.5 * (u(IM, J, K, 2) + u(IM, JP, K, 2));
                double U3IP = 0.5 * (u(IP, J, K, 3) + u(IP, J, KP, 3));
                double U3IM = 0.5 * (u(IM, J, K, 3) + u(IM, J, KP, 3));
                double U1JP = 0.5 * (u(I, JP, K, 1) + u(IP, JP, K, 1));
                double U1JC = 0.5 * (u(I, J, K, 1) + u(IP, J, K, 1));
                double U1JM = 0.5 * (u(I, JM, K, 1) + u(IP, JM, K, 1));
                double U12 = 0.5 / H[JP] * (DY[JP] * U1JC + DY[J] * U1JP);
                double U11 = 0.5 / H[J] * (DY[J] * U1JM + DY[JM] * U1JC);
                U12 = U12 * FJUP + (1. - FJUP) * (u(I, N2, K, 1) + u(IP, N2, K, 1)) * 0.5;
                U11 = U11 * FJUM + (1. - FJUM) * (u(I, 0, K, 1) + u(IP, 0, K, 1)) * 0.5;
                double U3JP = 0.5 * (u(I, JP, K, 3) + u(I, JP, KP, 3));
                double U3JC = 0.5 * (u(I, J, K, 3) + u(I, J, KP, 3));
                double U3JM = 0.5 * (u(I, JM, K, 3) + u(I, JM, KP, 3));
                double U32 = 0.5 / H[JP] * (DY[JP] * U3JC + DY[J] * U3JP);
                double U31 = 0.5 / H[J] * (DY[J] * U3JM + DY[JM] * U3JC);
                U32 = U32 * FJUP + (1. - FJUP) * (u(I, N2, K, 3) + u(I, N2, KP, 3)) * 0.5;
                U31 = U31 * FJUM + (1. - FJUM) * (u(I, 0, K, 3) + u(I, 0, KP, 3)) * 0.5;
                double DV3DX2 = (U32 - U31) / DY[J];
                double DV2DX3 = (U2KP - U2KM) * 0.5 * DX3;
                double DV3DX1 = (U3IP - U3IM) * 0.5 * DX1;
                double DV1DX3 = (U1KP - U1KM) * 0.5 * DX3;
                double DV2DX1 = (U2IP - U2IM) * 0.5 * DX1;
                double DV1DX2 = (U12 - U11) / DY[J];
                vor(I, J, K, 1) = DV3DX2 - DV2DX3;
                vor(I, J, K, 2) = DV1DX3 - DV3DX1;
                vor(I, J, K, 3) = DV2DX1 - DV1DX2;
            }
        }
    }
    for (int J = 1; J <= N2M; J++) {   // loops 20, 21 and 40
        const int JP = J + 1, JM = J - 1;
        double s[23] = {0.0};
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                double V1 = (u(I, J, K, 1) + u(IP, J, K, 1)) * 0.5;
                double V2 = (u(I, J, K, 2) + u(I, JP, K, 2)) * 0.5;
                double V3 = (u(I, J, K, 3) + u(I, J, KP, 3)) * 0.5;
                const double PP = p(I, J, K);
                s[0] = s[0] + V1; s[1] = s[1] + V2; s[2] = s[2] + V3; s[3] = s[3] + PP;
                s[4] = s[4] + vor(I, J, K, 1); s[5] = s[5] + vor(I, J, K, 2); s[6] = s[6] + vor(I, J, K, 3);
                s[7] = s[7] + V1 * V1; s[8] = s[8] + V2 * V2; s[9] = s[9] + V3 * V3;
                s[10] = s[10] + V1 * V2; s[11] = s[11] + V1 * V3; s[12] = s[12] + V2 * V3;
                s[13] = s[13] + PP * PP; s[14] = s[14] + PP * V2;
                s[15] = s[15] + vor(I, J, K, 1) * vor(I, J, K, 1);
                s[16] = s[16] + vor(I, J, K, 2) * vor(I, J, K, 2);
                s[17] = s[17] + vor(I, J, K, 3) * vor(I, J, K, 3);
                s[18] = s[18] + V1 * V1 * V2;
                s[19] = s[19] + V2 * V3 * V3;
            }
        }
        double *o = out + (size_t)(J - 1) * 29;
        for (int q = 0; q < 20; ++q) o[q] = s[q] * NXZ;
        double sk[6] = {0.0};
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                double V1 = (u(I, J, K, 1) + u(IP, J, K, 1)) * 0.5 - o[0];
                double V2 = (u(I, J, K, 2) + u(I, JP, K, 2)) * 0.5 - o[1];
                double V3 = (u(I, J, K, 3) + u(I, J, KP, 3)) * 0.5 - o[2];
                sk[0] = sk[0] + V1 * V1 * V1; sk[1] = sk[1] + V2 * V2 * V2; sk[2] = sk[2] + V3 * V3 * V3;
                sk[3] = sk[3] + V1 * V1 * V1 * V1; sk[4] = sk[4] + V2 * V2 * V2 * V2; sk[5] = sk[5] + V3 * V3 * V3 * V3;
            }
        }
        for (int q = 0; q < 6; ++q) o[20 + q] = sk[q] * NXZ;
        const double FJUM = g.FJMU[J], FJUP = g.FJPA[J];
        double du = 0.0, dv = 0.0, dw = 0.0;
        for (int K = 1; K <= N3M; K++) {
            const int KP = g.KPA[K];
            for (int I = 1; I <= N1M; I++) {
                const int IP = g.IPA[I];
                double U_JP = (u(I, JP, K, 1) + u(IP, JP, K, 1)) * 0.5;
                double U_JC = (u(I, J, K, 1) + u(IP, J, K, 1)) * 0.5;
                double U_JM = (u(I, JM, K, 1) + u(IP, JM, K, 1)) * 0.5;
                double W_JP = (u(I, JP, K, 3) + u(I, JP, KP, 3)) * 0.5;
                double W_JC = (u(I, J, K, 3) + u(I, J, KP, 3)) * 0.5;
                double W_JM = (u(I, JM, K, 3) + u(I, JM, KP, 3)) * 0.5;
                double U1 = FJUM * (1.0 / H[J] * (DY[J] * U_JM / 2.0 + DY[JM] * U_JC / 2.0)) +
                            (1. - FJUM) * (u(I, 0, K, 1) + u(IP, 0, K, 1)) * 0.5;
                double U2 = FJUP * (1.0 / H[JP] * (DY[J] * U_JP / 2.0 + DY[JP] * U_JC / 2.0)) +
                            (1. - FJUP) * (u(I, N2, K, 1) + u(IP, N2, K, 1)) * 0.5;
                double V1 = u(I, J, K, 2), V2 = u(I, JP, K, 2);
                double W1 = FJUM * (1.0 / H[J] * (DY[J] * W_JM / 2.0 + DY[JM] * W_JC / 2.0)) +
                            (1. - FJUM) * (u(I, 0, K, 3) + u(I, 0, KP, 3)) * 0.5;
                double W2 = FJUP * (1.0 / H[JP] * (DY[J] * W_JP / 2.0 + DY[JP] * W_JC / 2.0)) +
                            (1. - FJUP) * (u(I, N2, K, 3) + u(I, N2, KP, 3)) * 0.5;
                du = du + (U2 - U1) / DY[J];
                dv = dv + (V2 - V1) / DY[J];
                dw = dw + (W2 - W1) / DY[J];
            }
        }
        o[26] = du * NXZ;
        o[27] = dv * NXZ;
        o[28] = dw * NXZ;
    }
}

// ---- unit-level entry points ----
// CTDMA11 on one line with constant coefficients (a,b,c); d,x 0-based length n.
void orc_ctdma11(int n, double a, double b, double c, const double *d, double *x) {
    std::vector<double> A(n + 1, a), B(n + 1, b), C(n + 1, c), D(n + 1), X(n + 1);
    for (int i = 0; i < n; i++) D[i + 1] = d[i];
    ctdma_bordered(n, A.data(), B.data(), C.data(), D.data(), X.data());
    for (int i = 0; i < n; i++) x[i] = X[i + 1];
}
// CTDMA1J/CTDMA3I on one line (reciprocal form).
void orc_ctdma_recip(int n, double a, double b, double c, const double *d, double *x) {
    std::vector<double> A(n + 2, a), B(n + 2, b), C(n + 2, c), D(n + 2), X(n + 2);
    for (int i = 0; i < n; i++) D[i + 1] = d[i];
    ctdma_recip(1, n, A.data(), B.data(), C.data(), D.data(), X.data());
    for (int i = 0; i < n; i++) x[i] = X[i + 1];
}
// TDMAP on one line; arrays 0-based length n.
void orc_tdmap(int n, const double *a, const double *b, const double *c, const double *r, double *x) {
    std::vector<double> A(n + 1), B(n + 1), C(n + 1), R(n + 1), X(n + 1);
    for (int i = 0; i < n; i++) {
        A[i + 1] = a[i];
        B[i + 1] = b[i];
        C[i + 1] = c[i];
        R[i + 1] = r[i];
    }
    tdmap(A.data(), B.data(), C.data(), R.data(), n, X.data());
    for (int i = 0; i < n; i++) x[i] = X[i + 1];
}
// Complex FFT of n interleaved (re,im) values in place.
void orc_fft(int n, double *data, int sign) {
    fft1d(n, sign, (cplx *)data, 1);
}
// 2-D DFT of a Fortran complex array (n1 fastest), interleaved doubles.
void orc_dft2d(int n1, int n3, double *data, int sign) {
    dft2d(n1, n3, (cplx *)data, sign);
}
// Poisson metrics, for tests of the library's own copy.
void orc_poisson_metrics(void *h, double *ak1, double *ak3, double *pmj, double *pcj, double *ppj) {
    Orc &g = *(Orc *)h;
    for (int i = 1; i <= g.N1M; i++) ak1[i - 1] = g.AK1[i];
    for (int k = 1; k <= g.N3MH; k++) ak3[k - 1] = g.AK3[k];
    for (int j = 1; j <= g.N2M; j++) {
        pmj[j - 1] = g.PMJ[j];
        pcj[j - 1] = g.PCJ[j];
        ppj[j - 1] = g.PPJ[j];
    }
}

}  // extern "C"
