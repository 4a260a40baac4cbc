/* Separable direct DFT on a row-major n0 x n1 x n2 complex array (interleaved
 * re/im), X[k] = sum_n x[n] exp(sign 2 pi i k n / N) along each axis, with
 * exact-residue twiddles.  Shared by the FFTW3 stand-in used to build the
 * reference (oracle/shim/shim_impl.cpp) and by the CPU restatement
 * (oracle/lp_oracle.c), so both evaluate fftw_execute identically.
 * Test infrastructure only. */
#ifndef LP_ORACLE_DFT3_H
#define LP_ORACLE_DFT3_H
#include <math.h>
#include <stdlib.h>

static void lp_dft_axis(double *x, const int n[3], int axis, int sign)
{
    const int N = n[axis];
    double *wr = (double *)malloc(sizeof(double) * 2 * (size_t)N);
    double *wi = wr + N;
    for (int m = 0; m < N; ++m) {
        double ang = 2.0 * M_PI * (double)m / (double)N;
        wr[m] = cos(ang);
        wi[m] = sign * sin(ang);
    }
    long stride = 1;
    for (int a = 2; a > axis; --a) stride *= n[a];
    long outer = 1, inner = stride;
    for (int a = 0; a < axis; ++a) outer *= n[a];
    const long npencil = outer * inner;
#pragma omp parallel
    {
        double *tr = (double *)malloc(sizeof(double) * 2 * (size_t)N);
        double *ti = tr + N;
#pragma omp for schedule(static)
        for (long p = 0; p < npencil; ++p) {
            long o = p / inner, in_ = p % inner;
            double *base = x + 2 * (o * (long)N * stride + in_);
            for (int k = 0; k < N; ++k) {
                double sr = 0.0, si = 0.0;
                for (int j = 0; j < N; ++j) {
                    int m = (int)(((long)k * j) % N);
                    double xr = base[2 * j * stride], xi = base[2 * j * stride + 1];
                    sr += xr * wr[m] - xi * wi[m];
                    si += xr * wi[m] + xi * wr[m];
                }
                tr[k] = sr;
                ti[k] = si;
            }
            for (int k = 0; k < N; ++k) {
                base[2 * k * stride] = tr[k];
                base[2 * k * stride + 1] = ti[k];
            }
        }
        free(tr);
    }
    free(wr);
}

/* In-place unnormalised 3-D DFT, last axis first (the order is immaterial
 * mathematically; it is fixed so results are reproducible). */
static void lp_dft3_inplace(double *x, int n0, int n1, int n2, int sign)
{
    int n[3] = {n0, n1, n2};
    for (int axis = 2; axis >= 0; --axis) lp_dft_axis(x, n, axis, sign);
}
#endif
