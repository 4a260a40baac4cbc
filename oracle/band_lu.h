/* Dense and banded LU factorisation with partial pivoting, restated from the
 * published LAPACK reference algorithms (unblocked DGETF2/DGETRI with
 * DTRTI2, DGBTF2 and DGBTRS with DTBSV), column-major, Fortran 1-based
 * indexing through the AB()/A() macros.
 *
 * Test infrastructure: used by the MKL stand-in (oracle/shim/shim_impl.cpp)
 * that lets the reference's own sources compile here, and by the CPU
 * restatement (oracle/lp_oracle.c).  The operation order of each routine
 * follows the LAPACK/BLAS reference code so that the factors and solutions
 * are reproducible across machines when compiled with -ffp-contract=off.
 *
 * Reference call sites: source/conservationRoutines.cpp:186-187 (5x5 dgetrf,
 * dgetri), source/PoissonFunctions.cpp:1053 (dgbtrf) and :1267 (dgbtrs).
 */
#ifndef LP_ORACLE_BAND_LU_H
#define LP_ORACLE_BAND_LU_H
#include <math.h>

#define LP_MIN(a, b) ((a) < (b) ? (a) : (b))
#define LP_MAX(a, b) ((a) > (b) ? (a) : (b))

/* LU of a general m x n matrix, column-major with leading dimension lda.
 * Returns LAPACK's INFO (0 or the first zero pivot, 1-based). */
static inline int lp_dgetf2(int m, int n, double *a, int lda, int *ipiv)
{
#define A_(i, j) a[((i) - 1) + (long)((j) - 1) * lda]
    int info = 0;
    for (int j = 1; j <= LP_MIN(m, n); ++j) {
        int jp = j;
        double amax = fabs(A_(j, j));
        for (int i = j + 1; i <= m; ++i) {
            double v = fabs(A_(i, j));
            if (v > amax) { amax = v; jp = i; }
        }
        ipiv[j - 1] = jp;
        if (A_(jp, j) != 0.0) {
            if (jp != j)
                for (int c = 1; c <= n; ++c) { double t = A_(j, c); A_(j, c) = A_(jp, c); A_(jp, c) = t; }
            if (j < m) {
                double r = 1.0 / A_(j, j);
                for (int i = j + 1; i <= m; ++i) A_(i, j) *= r;
            }
        } else if (info == 0) {
            info = j;
        }
        if (j < LP_MIN(m, n)) {
            for (int c = j + 1; c <= n; ++c) {
                double y = A_(j, c);
                if (y != 0.0) {
                    double t = -y;
                    for (int i = j + 1; i <= m; ++i) A_(i, c) += A_(i, j) * t;
                }
            }
        }
    }
    return info;
#undef A_
}

/* Inverse from the LU of lp_dgetf2 (DGETRI with the unblocked DTRTI2 path).
 * work must hold n doubles. */
static inline int lp_dgetri(int n, double *a, int lda, const int *ipiv, double *work)
{
#define A_(i, j) a[((i) - 1) + (long)((j) - 1) * lda]
    for (int j = 1; j <= n; ++j)
        if (A_(j, j) == 0.0) return j;
    /* inv(U) in place: DTRTI2 upper, non-unit. */
    for (int j = 1; j <= n; ++j) {
        A_(j, j) = 1.0 / A_(j, j);
        double ajj = -A_(j, j);
        /* x := triu(A(1:j-1,1:j-1)) * A(1:j-1, j)   (DTRMV upper, no-trans) */
        for (int jj = 1; jj <= j - 1; ++jj) {
            double xj = A_(jj, j);
            if (xj != 0.0) {
                double t = xj;
                for (int i = 1; i <= jj - 1; ++i) A_(i, j) += t * A_(i, jj);
                A_(jj, j) = A_(jj, j) * A_(jj, jj);
            }
        }
        for (int i = 1; i <= j - 1; ++i) A_(i, j) *= ajj;
    }
    /* Solve inv(A) * L = inv(U). */
    for (int j = n; j >= 1; --j) {
        for (int i = j + 1; i <= n; ++i) { work[i - 1] = A_(i, j); A_(i, j) = 0.0; }
        if (j < n) {
            for (int jj = j + 1; jj <= n; ++jj) {
                double t = -work[jj - 1];
                if (work[jj - 1] != 0.0)
                    for (int i = 1; i <= n; ++i) A_(i, j) += t * A_(i, jj);
            }
        }
    }
    /* Undo the row interchanges as column interchanges. */
    for (int j = n - 1; j >= 1; --j) {
        int jp = ipiv[j - 1];
        if (jp != j)
            for (int i = 1; i <= n; ++i) { double t = A_(i, j); A_(i, j) = A_(i, jp); A_(i, jp) = t; }
    }
    return 0;
#undef A_
}

/* Band LU with partial pivoting (DGBTF2).  ab is ldab x n, ldab >= 2kl+ku+1,
 * A(i,j) stored at AB(kl+ku+1+i-j, j).  Returns LAPACK's INFO. */
static inline int lp_dgbtf2(int m, int n, int kl, int ku, double *ab, int ldab, int *ipiv)
{
#define AB(i, j) ab[((i) - 1) + (long)((j) - 1) * ldab]
    int info = 0;
    int kv = ku + kl;
    for (int j = ku + 2; j <= LP_MIN(kv, n); ++j)
        for (int i = kv - j + 2; i <= kl; ++i) AB(i, j) = 0.0;
    int ju = 1;
    for (int j = 1; j <= LP_MIN(m, n); ++j) {
        if (j + kv <= n)
            for (int i = 1; i <= kl; ++i) AB(i, j + kv) = 0.0;
        int km = LP_MIN(kl, m - j);
        int jp = 1;
        double amax = fabs(AB(kv + 1, j));
        for (int i = 2; i <= km + 1; ++i) {
            double v = fabs(AB(kv + i, j));
            if (v > amax) { amax = v; jp = i; }
        }
        ipiv[j - 1] = jp + j - 1;
        if (AB(kv + jp, j) != 0.0) {
            ju = LP_MAX(ju, LP_MIN(j + ku + jp - 1, n));
            if (jp != 1)
                for (int c = 0; c <= ju - j; ++c) {
                    double t = AB(kv + jp - c, j + c);
                    AB(kv + jp - c, j + c) = AB(kv + 1 - c, j + c);
                    AB(kv + 1 - c, j + c) = t;
                }
            if (km > 0) {
                double r = 1.0 / AB(kv + 1, j);
                for (int i = 1; i <= km; ++i) AB(kv + 1 + i, j) *= r;
                if (ju > j) {
                    for (int c = 1; c <= ju - j; ++c) {
                        double y = AB(kv - c + 1, j + c);
                        if (y != 0.0) {
                            double t = -y;
                            for (int i = 1; i <= km; ++i)
                                AB(kv + i - c + 1, j + c) += AB(kv + 1 + i, j) * t;
                        }
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
    }
    return info;
#undef AB
}

/* Solve A x = b with the factors of lp_dgbtf2, one right-hand side, no
 * transpose (DGBTRS 'N' followed by DTBSV upper). b is overwritten. */
static inline void lp_dgbtrs_n(int n, int kl, int ku, const double *ab, int ldab,
                               const int *ipiv, double *b)
{
#define AB(i, j) ab[((i) - 1) + (long)((j) - 1) * ldab]
    int kd = ku + kl + 1;
    if (kl > 0) {
        for (int j = 1; j <= n - 1; ++j) {
            int lm = LP_MIN(kl, n - j);
            int l = ipiv[j - 1];
            if (l != j) { double t = b[l - 1]; b[l - 1] = b[j - 1]; b[j - 1] = t; }
            double bj = b[j - 1];
            if (bj != 0.0) {
                double t = -bj;
                for (int i = 1; i <= lm; ++i) b[j + i - 1] += AB(kd + i, j) * t;
            }
        }
    }
    int k = kl + ku;
    int kplus1 = k + 1;
    for (int j = n; j >= 1; --j) {
        if (b[j - 1] != 0.0) {
            int l = kplus1 - j;
            b[j - 1] = b[j - 1] / AB(kplus1, j);
            double t = b[j - 1];
            for (int i = j - 1; i >= LP_MAX(1, j - k); --i) b[i - 1] = b[i - 1] - t * AB(l + i, j);
        }
    }
#undef AB
}

#endif
