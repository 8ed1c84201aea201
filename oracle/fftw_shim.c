/* TEST INFRASTRUCTURE ONLY: the few FFTW 3 legacy-Fortran-interface routines that
 * compact3d.f calls (GETDP, compact3d.f:9305-9437), for the C translation of the
 * reference made by oracle/f77c.py.  FFTW itself is a third-party library that the
 * reference neither vendors nor pins; this file restates the transform FFTW documents
 * for dfftw_plan_dft_2d / dfftw_execute_dft:
 *
 *   out(p, q) = sum_{i<n0} sum_{k<n1} in(i, k) exp(sign * 2 pi sqrt(-1) (i p / n0 + k q / n1))
 *
 * with the Fortran (column-major) dimension order of the legacy interface (n0 is the
 * fastest index), sign = FFTW_FORWARD (-1) or FFTW_BACKWARD (+1), no normalisation.
 * Each dimension is transformed by a mixed-radix Cooley-Tukey recursion (radix 2, 3, 5,
 * any other prime factor summed directly), in double precision with twiddle factors
 * taken at the exact angle (m mod n) / n in long double.  The transform is re-entrant:
 * GETDP executes plans inside an OpenMP loop, so the scratch space is per thread.
 * Threads and planner flags are otherwise ignored.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

typedef struct {
    int n0, n1, sign;
    cplx *w0, *w1;   /* w[m] = exp(sign 2 pi i m / n) */
} plan2d;

static cplx *twiddles(int n, int sign) {
    cplx *w = malloc(sizeof(*w) * (size_t)n);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int m = 0; m < n; ++m) {
        long double a = 2.0L * pi * (long double)m / (long double)n;
        w[m] = (double)cosl(a) + (double)((long double)sign * sinl(a)) * I;
    }
    return w;
}

static int smallest_factor(int n) {
    if (n % 2 == 0) return 2;
    if (n % 3 == 0) return 3;
    if (n % 5 == 0) return 5;
    for (int f = 7; f * f <= n; f += 2)
        if (n % f == 0) return f;
    return n;
}

/* y[0..n) = DFT_n of x[0], x[s], ..., x[(n-1)s]; w is the length-N table and ws = N / n */
static void fft_rec(const cplx *x, long s, cplx *y, int n, const cplx *w, int ws, int N, cplx *tmp) {
    if (n == 1) { y[0] = x[0]; return; }
    const int p = smallest_factor(n), m = n / p;
    for (int r = 0; r < p; ++r) fft_rec(x + r * s, s * p, y + r * m, m, w, ws * p, N, tmp);
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) tmp[r] = y[r * m + k];
        for (int q = 0; q < p; ++q) {
            const long e = (long)(k + q * m);
            cplx acc = 0;
            for (int r = 0; r < p; ++r) acc += tmp[r] * w[((long)r * e % n) * ws % N];
            y[k + q * m] = acc;
        }
    }
}

static __thread cplx *t_buf = 0;
static __thread size_t t_cap = 0;
static cplx *scratch(size_t n) {
    if (n > t_cap) {
        free(t_buf);
        t_buf = malloc(sizeof(cplx) * n);
        t_cap = n;
    }
    return t_buf;
}

void f77_DFFTW_INIT_THREADS(int *iret) { *iret = 1; }
void f77_DFFTW_PLAN_WITH_NTHREADS(int *n) { (void)n; }
double f77_OMP_GET_MAX_THREADS(void) { return 1.0; }

void f77_DFFTW_PLAN_DFT_2D(long long *plan, int *n0, int *n1, void *in, void *out, int *sign, int *flags) {
    (void)in; (void)out; (void)flags;
    plan2d *p = malloc(sizeof(plan2d));
    p->n0 = *n0;
    p->n1 = *n1;
    p->sign = *sign;
    p->w0 = twiddles(*n0, *sign);
    p->w1 = twiddles(*n1, *sign);
    *plan = (long long)(size_t)p;
}

void f77_DFFTW_EXECUTE_DFT(long long *plan, void *in, void *out) {
    const plan2d *p = (const plan2d *)(size_t)*plan;
    const int n0 = p->n0, n1 = p->n1, nm = n0 > n1 ? n0 : n1;
    const cplx *x = in;
    cplx *y = out;
    cplx *buf = scratch((size_t)n0 * n1 + 3 * (size_t)nm);
    cplx *T = buf, *line = buf + (size_t)n0 * n1, *res = line + nm, *tmp = res + nm;
    /* along the first (fastest) dimension, into T */
    for (int k = 0; k < n1; ++k) fft_rec(x + (size_t)n0 * k, 1, T + (size_t)n0 * k, n0, p->w0, 1, n0, tmp);
    /* along the second dimension, into y */
    for (int q = 0; q < n0; ++q) {
        fft_rec(T + q, n0, res, n1, p->w1, 1, n1, tmp);
        for (int r = 0; r < n1; ++r) y[q + (size_t)n0 * r] = res[r];
    }
    (void)line;
}

void f77_DFFTW_DESTROY_PLAN(long long *plan) {
    plan2d *p = (plan2d *)(size_t)*plan;
    free(p->w0);
    free(p->w1);
    free(p);
}
