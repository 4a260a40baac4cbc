// Implementations behind the FFTW3 and MKL-LAPACK stand-in headers in this
// directory.  They let the Landau-Poisson reference's own sources (read where
// they lie, never copied) compile and run here as a CPU test oracle.
//
// FFTW3 subset: fftw_plan_dft_3d + fftw_execute as an unnormalised separable
// direct DFT, X[k] = sum_n x[n] exp(sign 2 pi i k n / N) along each axis,
// row-major.  Used by fft3D/FS/ifft3D (source/collisionRoutines_1.cpp:163-276)
// on the in-place plans made at source/LP_ompi_1.cpp:247-248.
//
// LAPACK subset: dgetrf/dgetri/dgbtrf/dgbtrs over oracle/band_lu.h.
//
// Test infrastructure only; nothing in the shipped library links this file.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>

#include "fftw3.h"
#include "mkl_lapack.h"
#include "../band_lu.h"
#include "../dft3.h"

struct lp_shim_fftw_plan_s {
    int n[3];
    int sign;
    double *in;
    double *out;
};

extern "C" {

void *fftw_malloc(size_t n) {
    void *p = nullptr;
    if (posix_memalign(&p, 64, n ? n : 64) != 0) return nullptr;
    return p;
}
void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int) {}

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned) {
    fftw_plan p = new lp_shim_fftw_plan_s;
    p->n[0] = n0; p->n[1] = n1; p->n[2] = n2;
    p->sign = sign;
    p->in = &in[0][0];
    p->out = &out[0][0];
    return p;
}

void fftw_destroy_plan(fftw_plan p) { delete p; }

void fftw_execute(const fftw_plan p) {
    const long total = (long)p->n[0] * p->n[1] * p->n[2];
    if (p->out != p->in) std::memcpy(p->out, p->in, sizeof(double) * 2 * total);
    lp_dft3_inplace(p->out, p->n[0], p->n[1], p->n[2], p->sign);
}

void dgetrf(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info) {
    *info = lp_dgetf2(*m, *n, a, *lda, ipiv);
}

void dgetri(const int *n, double *a, const int *lda, const int *ipiv, double *work,
            const int *lwork, int *info) {
    std::vector<double> w(*n > 0 ? *n : 1);
    (void)work; (void)lwork;
    *info = lp_dgetri(*n, a, *lda, ipiv, w.data());
}

void dgbtrf(const int *m, const int *n, const int *kl, const int *ku, double *ab,
            const int *ldab, int *ipiv, int *info) {
    *info = lp_dgbtf2(*m, *n, *kl, *ku, ab, *ldab, ipiv);
}

void dgbtrs(const char *trans, const int *n, const int *kl, const int *ku, const int *nrhs,
            const double *ab, const int *ldab, const int *ipiv, double *b, const int *ldb,
            int *info) {
    *info = 0;
    if (*trans != 'N' && *trans != 'n') { *info = -1; return; }
    for (int r = 0; r < *nrhs; ++r)
        lp_dgbtrs_n(*n, *kl, *ku, ab, *ldab, ipiv, b + (long)r * (*ldb));
}

}  // extern "C"
