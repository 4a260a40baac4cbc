/* Stand-in for the four LAPACK routines the Landau-Poisson reference calls
 * through <mkl_lapack.h> (source/LP_ompi.h:25): dgetrf/dgetri on the 5x5
 * conservation Gram matrix (source/conservationRoutines.cpp:186-187) and
 * dgbtrf/dgbtrs on the LDG Poisson band matrix
 * (source/PoissonFunctions.cpp:1053, 1267).  Fortran calling convention,
 * column-major, LAPACK band storage.  Implemented in oracle/band_lu.h from the
 * published LAPACK algorithms (unblocked dgbtf2 / dgbtrs / dgetf2 / dgetri).
 * Test infrastructure only. */
#ifndef LP_SHIM_MKL_LAPACK_H
#define LP_SHIM_MKL_LAPACK_H
#ifdef __cplusplus
extern "C" {
#endif
void dgetrf(const int *m, const int *n, double *a, const int *lda, int *ipiv, int *info);
void dgetri(const int *n, double *a, const int *lda, const int *ipiv, double *work,
            const int *lwork, int *info);
void dgbtrf(const int *m, const int *n, const int *kl, const int *ku, double *ab,
            const int *ldab, int *ipiv, int *info);
void dgbtrs(const char *trans, const int *n, const int *kl, const int *ku, const int *nrhs,
            const double *ab, const int *ldab, const int *ipiv, double *b, const int *ldb,
            int *info);
#ifdef __cplusplus
}
#endif
#endif
