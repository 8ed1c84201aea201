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
 * It is evaluated by direct summation along each dimension in long double with twiddle
 * factors taken at the exact angle (m mod n) / n, so results are accurate to about one
 * unit of the double rounding of each output; threads and planner flags are ignored.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int n0, n1, sign;
    long double _Complex *w0, *w1, *tmp;
} plan2d;

static long double _Complex *twiddles(int n, int sign) {
    long double _Complex *w = malloc(sizeof(*w) * (size_t)n);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int m = 0; m < n; ++m) {
        long double a = 2.0L * pi * (long double)m / (long double)n;
        w[m] = cosl(a) + (long double)sign * sinl(a) * I;
    }
    return w;
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
    p->tmp = malloc(sizeof(long double _Complex) * (size_t)(*n0) * (size_t)(*n1));
    *plan = (long long)(size_t)p;
}

void f77_DFFTW_EXECUTE_DFT(long long *plan, void *in, void *out) {
    plan2d *p = (plan2d *)(size_t)*plan;
    const int n0 = p->n0, n1 = p->n1;
    const double _Complex *x = in;
    double _Complex *y = out;
    long double _Complex *t = p->tmp;
    /* along the first (fastest) dimension */
    for (int k = 0; k < n1; ++k)
        for (int q = 0; q < n0; ++q) {
            long double _Complex s = 0;
            for (int i = 0; i < n0; ++i) s += (long double _Complex)x[i + (size_t)n0 * k] * p->w0[((long)i * q) % n0];
            t[q + (size_t)n0 * k] = s;
        }
    /* along the second dimension */
    for (int q = 0; q < n0; ++q) {
        long double _Complex col[n1];
        for (int k = 0; k < n1; ++k) col[k] = t[q + (size_t)n0 * k];
        for (int r = 0; r < n1; ++r) {
            long double _Complex s = 0;
            for (int k = 0; k < n1; ++k) s += col[k] * p->w1[((long)k * r) % n1];
            y[q + (size_t)n0 * r] = (double _Complex)s;
        }
    }
}

void f77_DFFTW_DESTROY_PLAN(long long *plan) {
    plan2d *p = (plan2d *)(size_t)*plan;
    free(p->w0);
    free(p->w1);
    free(p->tmp);
    free(p);
}
