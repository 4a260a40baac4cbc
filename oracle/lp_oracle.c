/* CPU restatement of the Landau-Poisson reference's hot path: the test
 * oracle.  TEST INFRASTRUCTURE ONLY -- the shipped GPU library never links or
 * calls this file (see lp_oracle.h for who may).
 *
 * Each function cites the reference routine it restates (paths relative to
 * the reference checkout).  Where the golden vectors are compared bit for
 * bit, the expression order of the reference is kept and the file is compiled
 * with -ffp-contract=off; the direct DFT behind fftw_execute is the same code
 * the FFTW3 stand-in uses (dft3.h).
 *
 * Abbreviations used in citations:
 *   C = source/collisionRoutines_1.cpp   K = source/conservationRoutines.cpp
 *   A = source/advection_1.cpp           P = source/PoissonFunctions.cpp
 *   M = source/LP_ompi_1.cpp             S = source/SetInit_1.cpp
 *   MC = source/MomentCalculations.cpp
 */
#include "lp_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "band_lu.h"
#include "dft3.h"

/* 5-point Gauss-Legendre rule on [-1,1] with the decimal values the reference
 * uses (A:12-13). */
static const double GW[5] = {0.5688888888888889, 0.4786286704993665, 0.4786286704993665,
                             0.2369268850561891, 0.2369268850561891};
static const double GX[5] = {0., -0.5384693101056831, 0.5384693101056831, -0.9061798459386640,
                             0.9061798459386640};

typedef struct {
    int nx, ny, ndim, kl, ku, ldab;
    double *ab;
    int *ipiv;
    double dxp, dyp, xc, xd;
    double *cx; /* cell centres CX[1..nx] */
    double acvx[3][3], acvy[3][3], acyrr[3][3], acyrl[3][3], acxrr[3][3], acxrl[3][3];
} pois_t;

struct lpo_ctx {
    lpo_params p;
    int nv3, n3, ncell;
    long size;
    double PI, dv, dx, dy, scalev, scaleL, scale, scale3, L_v, R_v, L_eta, h_eta, h_v;
    double *v, *eta, *wt;
    double *sh;           /* n3 x 6: Shat00, Shat01, Shat02, Shat11, Shat12, Shat22 */
    double *ah;           /* n3: sqrt(8/pi)(R r - sin R r)/(R r) */
    unsigned char *rzero; /* n3: |omega| == 0 */
    double *c1, *c2;      /* 5 x n3 */
    double cct[25];
    double cct_lin[4];    /* inverse 2x2 Gram matrix of rows C1[0], C1[4] (two-species variant) */
    int *nodecell;        /* n: DG cell of spectral node */
    double *tt;           /* 3 x n x nv complex: T0, T1, T2 per (k, j) */
    pois_t ps;
};

static inline double gridv(const lpo_ctx *c, double m) { return (-c->p.lv + (m + 0.5) * c->dv); }
static inline double gridx(const lpo_ctx *c, double m) { return (m + 0.5) * c->dx; }

/* ---------------------------------------------------------------- weights */
/* S1hat, S233hat, S213hat (C:10-28). */
static double s1hat(const lpo_ctx *c, double k1, double k2, double k3)
{
    const double PI = c->PI, R = c->R_v;
    if (k1 == 0. && k2 == 0. && k3 == 0.) return sqrt(1. / (2 * PI)) * R * R;
    return sqrt(2.0 / PI) * (1 - cos(R * sqrt(k1 * k1 + k2 * k2 + k3 * k3))) / (k1 * k1 + k2 * k2 + k3 * k3);
}
static double s233hat(const lpo_ctx *c, double k1, double k2, double k3)
{
    const double PI = c->PI, R = c->R_v;
    double r = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
    if (r == 0.) return sqrt(1. / (2. * PI)) * R * R / 3.;
    return sqrt(2. / PI) *
           ((k1 * k1 + k2 * k2) * (R * r - sin(R * r)) / (R * r) -
            k3 * k3 * (R * r + R * r * cos(R * r) - 2. * sin(R * r)) / (R * r)) /
           pow(r, 4.);
}
static double s213hat(const lpo_ctx *c, double k1, double k2, double k3)
{
    const double PI = c->PI, R = c->R_v;
    double r = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
    if (k1 == 0. || k3 == 0.) return 0.;
    return -sqrt(2 / PI) * k1 * k3 * (2. * R * r + R * r * cos(R * r) - 3. * sin(R * r)) / (R * pow(r, 5.));
}

/* The omega-only part of gHat3 (C:30-53, C:67): the symmetric matrix Shat and
 * the r-dependent leading term. */
static void omega_tables(lpo_ctx *c)
{
    const int n = c->p.n;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < c->n3; ++t) {
        int l = t / (n * n), m = (t / n) % n, q = t % n;
        double k1 = c->eta[l], k2 = c->eta[m], k3 = c->eta[q];
        double r = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        double *s = c->sh + 6 * (long)t;
        s[0] = s1hat(c, k1, k2, k3) - s233hat(c, k2, k3, k1);
        s[3] = s1hat(c, k1, k2, k3) - s233hat(c, k1, k3, k2);
        s[5] = s1hat(c, k1, k2, k3) - s233hat(c, k1, k2, k3);
        s[1] = -s213hat(c, k1, k3, k2);
        s[2] = -s213hat(c, k1, k2, k3);
        s[4] = -s213hat(c, k2, k1, k3);
        c->rzero[t] = (r == 0.);
        c->ah[t] = (r == 0.) ? 0. : (sqrt(8. / c->PI)) * (c->R_v * r - sin(c->R_v * r)) / (c->R_v * r);
    }
}

/* gHat3(eta_xi, eta_omega) (C:30-69), evaluated from the omega tables with
 * the reference's summation order over (i, j). */
static inline double weight_of(const lpo_ctx *c, int xi, int om)
{
    const int n = c->p.n;
    int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
    int l = om / (n * n), m = (om / n) % n, q = om % n;
    const double *s = c->sh + 6 * (long)om;
    double d0 = c->eta[i] - c->eta[l], d1 = c->eta[j] - c->eta[m], d2 = c->eta[k] - c->eta[q];
    double res = 0.;
    res += s[0] * d0 * d0; res += s[1] * d0 * d1; res += s[2] * d0 * d2;
    res += s[1] * d1 * d0; res += s[3] * d1 * d1; res += s[4] * d1 * d2;
    res += s[2] * d2 * d0; res += s[4] * d2 * d1; res += s[5] * d2 * d2;
    if (c->rzero[om]) return -res;
    return c->ah[om] - res;
}

double lpo_weight(const lpo_ctx *c, int xi, int om) { return weight_of(c, xi, om); }

/* The omega tables weight_of reads (C:30-69): ahat (n3), Shat (n3 x 6: 00, 01,
 * 02, 11, 12, 22) and the nodes |omega| == 0, whose weight omits ahat. */
void lpo_omega_tables(const lpo_ctx *c, double *ah, double *sh, unsigned char *rz)
{
    memcpy(ah, c->ah, sizeof(double) * (size_t)c->n3);
    memcpy(sh, c->sh, sizeof(double) * 6 * (size_t)c->n3);
    memcpy(rz, c->rzero, (size_t)c->n3);
}

/* ---------------------------------------------------------- conservation */
static double sinc_(double x) { return x == 0.0 ? 1.0 : sin(x) / x; }

/* createCCtAndPivot (K:133-209): constraint rows and the inverse Gram matrix. */
static void cons_tables(lpo_ctx *c)
{
    const int n = c->p.n, n3 = c->n3;
    const double L = c->L_v;
    const double *eta = c->eta;
    for (int t = 0; t < n3; ++t) {
        int k = t % n, j = ((t - k) % (n * n)) / n, i = (t - k - j * n) / (n * n);
        double a1, a2, a3;
        c->c1[0 * n3 + t] = sinc_(L * eta[i]) * sinc_(L * eta[j]) * sinc_(L * eta[k]);
        c->c1[1 * n3 + t] = 0.; c->c1[2 * n3 + t] = 0.; c->c1[3 * n3 + t] = 0.;
        if (eta[i] != 0) a1 = ((eta[i] * eta[i] * L * L - 2) * sin(eta[i] * L) + 2 * eta[i] * L * cos(eta[i] * L)) / (eta[i] * eta[i] * eta[i] * L);
        else a1 = L * L / 3.;
        if (eta[j] != 0) a2 = ((eta[j] * eta[j] * L * L - 2) * sin(eta[j] * L) + 2 * eta[j] * L * cos(eta[j] * L)) / (eta[j] * eta[j] * eta[j] * L);
        else a2 = L * L / 3.;
        if (eta[k] != 0) a3 = ((eta[k] * eta[k] * L * L - 2) * sin(eta[k] * L) + 2 * eta[k] * L * cos(eta[k] * L)) / (eta[k] * eta[k] * eta[k] * L);
        else a3 = L * L / 3.;
        c->c1[4 * n3 + t] = 0.5 * (a1 * sinc_(L * eta[j]) * sinc_(L * eta[k]) + a2 * sinc_(L * eta[i]) * sinc_(L * eta[k]) + a3 * sinc_(L * eta[i]) * sinc_(L * eta[j]));
        c->c2[0 * n3 + t] = 0.;
        c->c2[1 * n3 + t] = (eta[i] != 0) ? -sinc_(L * eta[j]) * sinc_(L * eta[k]) * (sinc_(eta[i] * L) - cos(eta[i] * L)) / eta[i] : 0.;
        c->c2[2 * n3 + t] = (eta[j] != 0) ? -sinc_(L * eta[i]) * sinc_(L * eta[k]) * (sinc_(eta[j] * L) - cos(eta[j] * L)) / eta[j] : 0.;
        c->c2[3 * n3 + t] = (eta[k] != 0) ? -sinc_(L * eta[i]) * sinc_(L * eta[j]) * (sinc_(eta[k] * L) - cos(eta[k] * L)) / eta[k] : 0.;
        c->c2[4 * n3 + t] = 0.;
    }
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            double s = 0.;
            for (int k = 0; k < n3; ++k) s += c->c1[i * n3 + k] * c->c1[j * n3 + k] + c->c2[i * n3 + k] * c->c2[j * n3 + k];
            c->cct[i * 5 + j] = s;
        }
    int piv[5];
    double work[5];
    lp_dgetf2(5, 5, c->cct, 5, piv);
    lp_dgetri(5, c->cct, 5, piv, work);
    /* CCt_linear (K:190-199): rows C1[0] and C1[4] (C2[0] = C2[4] = 0) */
    double t = 0., t1 = 0., t2 = 0.;
    for (int k = 0; k < n3; ++k) {
        t += c->c1[0 * n3 + k] * c->c1[0 * n3 + k] + c->c2[0 * n3 + k] * c->c2[0 * n3 + k];
        t1 += c->c1[0 * n3 + k] * c->c1[4 * n3 + k] + c->c2[0 * n3 + k] * c->c2[4 * n3 + k];
        t2 += c->c1[4 * n3 + k] * c->c1[4 * n3 + k] + c->c2[4 * n3 + k] * c->c2[4 * n3 + k];
    }
    c->cct_lin[0] = t; c->cct_lin[1] = t1; c->cct_lin[2] = t1; c->cct_lin[3] = t2;
    int piv2[2];
    double work2[2];
    lp_dgetf2(2, 2, c->cct_lin, 2, piv2);
    lp_dgetri(2, c->cct_lin, 2, piv2, work2);
}

void lpo_cons(const lpo_ctx *c, double *c1, double *c2, double *cct)
{
    memcpy(c1, c->c1, sizeof(double) * 5 * c->n3);
    memcpy(c2, c->c2, sizeof(double) * 5 * c->n3);
    memcpy(cct, c->cct, sizeof(double) * 25);
}

/* conserveAllMoments + solveWithCCt (K:100-129, K:7-57). */
void lpo_conserve(const lpo_ctx *c, double *q)
{
    const int n3 = c->n3;
    double t[5] = {0, 0, 0, 0, 0}, lam[5];
    for (int k = 0; k < n3; ++k) {
        t[0] += q[2 * (long)k] * c->c1[0 * n3 + k];
        t[1] += q[2 * (long)k + 1] * c->c2[1 * n3 + k];
        t[2] += q[2 * (long)k + 1] * c->c2[2 * n3 + k];
        t[3] += q[2 * (long)k + 1] * c->c2[3 * n3 + k];
        t[4] += q[2 * (long)k] * c->c1[4 * n3 + k];
    }
    for (int i = 0; i < 5; ++i) {
        double s = 0.;
        for (int j = 0; j < 5; ++j) s += c->cct[j + i * 5] * t[j];
        lam[i] = s;
    }
    for (int k = 0; k < n3; ++k) {
        q[2 * (long)k] -= (c->c1[0 * n3 + k] * lam[0] + c->c1[4 * n3 + k] * lam[4]);
        q[2 * (long)k + 1] -= (c->c2[1 * n3 + k] * lam[1] + c->c2[2 * n3 + k] * lam[2] + c->c2[3 * n3 + k] * lam[3]);
    }
}

/* -------------------------------------------------------------- transforms */
/* fft3D (C:163-197). */
void lpo_fft3d(const lpo_ctx *c, const double *in, double *out)
{
    const int n = c->p.n;
    const long n3 = c->n3;
    double *tmp = (double *)malloc(sizeof(double) * 2 * n3);
    const double hv = c->h_v;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                long idx = k + n * (j + (long)n * i);
                double sum = ((double)i + (double)j + (double)k) * c->L_eta * hv;
                double w = c->scale3 * hv * hv * hv * c->wt[i] * c->wt[j] * c->wt[k];
                tmp[2 * idx] = w * (cos(sum) * in[2 * idx] - sin(sum) * in[2 * idx + 1]);
                tmp[2 * idx + 1] = w * (cos(sum) * in[2 * idx + 1] + sin(sum) * in[2 * idx]);
            }
    lp_dft3_inplace(tmp, n, n, n, -1);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                long idx = k + n * (j + (long)n * i);
                double sum = c->L_v * (c->eta[i] + c->eta[j] + c->eta[k]);
                out[2 * idx] = (cos(sum) * tmp[2 * idx] - sin(sum) * tmp[2 * idx + 1]);
                out[2 * idx + 1] = (cos(sum) * tmp[2 * idx + 1] + sin(sum) * tmp[2 * idx]);
            }
    free(tmp);
}

/* FS (C:241-276). */
void lpo_fs(const lpo_ctx *c, const double *in, double *out)
{
    const int n = c->p.n;
    const long n3 = c->n3;
    double *tmp = (double *)malloc(sizeof(double) * 2 * n3);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                long idx = k + n * (j + (long)n * i);
                double sum = -(((double)i + (double)j + (double)k) * c->L_v * c->h_eta);
                tmp[2 * idx] = (cos(sum) * in[2 * idx] - sin(sum) * in[2 * idx + 1]);
                tmp[2 * idx + 1] = (cos(sum) * in[2 * idx + 1] + sin(sum) * in[2 * idx]);
            }
    lp_dft3_inplace(tmp, n, n, n, +1);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                long idx = k + n * (j + (long)n * i);
                double sum = -(c->L_eta * (c->v[i] + c->v[j] + c->v[k]));
                out[2 * idx] = (cos(sum) * tmp[2 * idx] - sin(sum) * tmp[2 * idx + 1]) / c->scaleL / c->scale3;
                out[2 * idx + 1] = (cos(sum) * tmp[2 * idx + 1] + sin(sum) * tmp[2 * idx]) / c->scaleL / c->scale3;
            }
    free(tmp);
}

/* -------------------------------------------------------------- ComputeQ */
/* ComputeQ (C:739-822): forward transform of the real node values, then the
 * windowed weighted sum over omega for every xi. */
void lpo_compute_q(const lpo_ctx *c, const double *f, double *qhat)
{
    const int n = c->p.n, h = n / 2;
    const long n3 = c->n3;
    double *fin = (double *)calloc(2 * n3, sizeof(double));
    double *F = (double *)malloc(sizeof(double) * 2 * n3);
    for (long i = 0; i < n3; ++i) fin[2 * i] = f[i];
    lpo_fft3d(c, fin, F);
    const double pre = c->h_eta * c->h_eta * c->h_eta;
    const double *wt = c->wt;
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                int si = i < h ? 0 : i - h + 1, ei = i < h ? i + h + 1 : n;
                int sj = j < h ? 0 : j - h + 1, ej = j < h ? j + h + 1 : n;
                int sk = k < h ? 0 : k - h + 1, ek = k < h ? k + h + 1 : n;
                int xi = k + n * (j + n * i);
                double t0 = 0., t1 = 0.;
                for (int l = si; l < ei; ++l)
                    for (int m = sj; m < ej; ++m)
                        for (int q = sk; q < ek; ++q) {
                            int x = i + h - l, y = j + h - m, z = k + h - q;
                            long o = q + n * (m + (long)n * l), u = z + n * (y + (long)n * x);
                            double w = weight_of(c, xi, (int)o);
                            t0 += pre * wt[l] * wt[m] * wt[q] * w * (F[2 * o] * F[2 * u] - F[2 * o + 1] * F[2 * u + 1]);
                            t1 += pre * wt[l] * wt[m] * wt[q] * w * (F[2 * o] * F[2 * u + 1] + F[2 * o + 1] * F[2 * u]);
                        }
                qhat[2 * (long)xi] = t0;
                qhat[2 * (long)xi + 1] = t1;
            }
    }
    free(fin);
    free(F);
}

/* ------------------------------------------------- two-species (linear) term */
/* gHat3_linear(eta_xi, eta_omega) (C:71-96): -sum_ij Shat_ij(omega) xi_i (xi_j - omega_j)
 * in the reference's (i, j) order. */
static inline double weight_lin_of(const lpo_ctx *c, int xi, int om)
{
    const int n = c->p.n;
    const double z[3] = {c->eta[xi / (n * n)], c->eta[(xi / n) % n], c->eta[xi % n]};
    const double kk[3] = {c->eta[om / (n * n)], c->eta[(om / n) % n], c->eta[om % n]};
    const double *s = c->sh + 6 * (long)om;
    const double S[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    double r = 0.;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r += S[i][j] * z[i] * (z[j] - kk[j]);
    return -r;
}

double lpo_weight_lin(const lpo_ctx *c, int xi, int om) { return weight_lin_of(c, xi, om); }

/* ComputeQ of the two-species variant (C:551-635): qhat = Q(f,f) plus the
 * linear term sum cw scale3 Wlin(xi, w) F(xi + n/2 - w), qhat_lin = that term. */
void lpo_compute_q_lin(const lpo_ctx *c, const double *f, double *qhat, double *qlin)
{
    const int n = c->p.n, h = n / 2;
    const long n3 = c->n3;
    double *fin = (double *)calloc(2 * n3, sizeof(double));
    double *F = (double *)malloc(sizeof(double) * 2 * n3);
    for (long i = 0; i < n3; ++i) fin[2 * i] = f[i];
    lpo_fft3d(c, fin, F);
    const double pre = c->h_eta * c->h_eta * c->h_eta, s3 = c->scale3;
    const double *wt = c->wt;
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                int si = i < h ? 0 : i - h + 1, ei = i < h ? i + h + 1 : n;
                int sj = j < h ? 0 : j - h + 1, ej = j < h ? j + h + 1 : n;
                int sk = k < h ? 0 : k - h + 1, ek = k < h ? k + h + 1 : n;
                int xi = k + n * (j + n * i);
                double t0 = 0., t1 = 0., t01 = 0., t11 = 0.;
                for (int l = si; l < ei; ++l)
                    for (int m = sj; m < ej; ++m)
                        for (int q = sk; q < ek; ++q) {
                            int x = i + h - l, y = j + h - m, z = k + h - q;
                            long o = q + n * (m + (long)n * l), u = z + n * (y + (long)n * x);
                            double w = weight_of(c, xi, (int)o), wl = weight_lin_of(c, xi, (int)o);
                            t0 += pre * wt[l] * wt[m] * wt[q] * (w * (F[2 * o] * F[2 * u] - F[2 * o + 1] * F[2 * u + 1]) + s3 * wl * F[2 * u]);
                            t1 += pre * wt[l] * wt[m] * wt[q] * (w * (F[2 * o] * F[2 * u + 1] + F[2 * o + 1] * F[2 * u]) + s3 * wl * F[2 * u + 1]);
                            t01 += pre * wt[l] * wt[m] * wt[q] * s3 * wl * F[2 * u];
                            t11 += pre * wt[l] * wt[m] * wt[q] * s3 * wl * F[2 * u + 1];
                        }
                qhat[2 * (long)xi] = t0;
                qhat[2 * (long)xi + 1] = t1;
                qlin[2 * (long)xi] = t01;
                qlin[2 * (long)xi + 1] = t11;
            }
    }
    free(fin);
    free(F);
}

/* conserveAllMoments of the two-species variant (K:63-98): qhat with the 5
 * constraints, qhat_lin's real part with mass and energy (CCt_linear). */
void lpo_conserve_lin(const lpo_ctx *c, double *q, double *ql)
{
    const int n3 = c->n3;
    lpo_conserve(c, q);
    double t0 = 0., t1 = 0.;
    for (int k = 0; k < n3; ++k) {
        t0 += ql[2 * (long)k] * c->c1[0 * n3 + k];
        t1 += ql[2 * (long)k] * c->c1[4 * n3 + k];
    }
    const double l0 = c->cct_lin[0] * t0 + c->cct_lin[1] * t1, l1 = c->cct_lin[2] * t0 + c->cct_lin[3] * t1;
    for (int k = 0; k < n3; ++k) ql[2 * (long)k] -= (c->c1[0 * n3 + k] * l0 + c->c1[4 * n3 + k] * l1);
}

void lpo_cct_lin(const lpo_ctx *c, double *out4) { memcpy(out4, c->cct_lin, sizeof(double) * 4); }

/* A stage's conserved mode array: ComputeQ and conserveAllMoments, and in the
 * two-species variant the conserved linear part added (C:656-698). */
static void stage_q(const lpo_ctx *c, const double *f1, double *q)
{
    if (c->p.linear_ei) {
        double *ql = (double *)malloc(sizeof(double) * 2 * c->n3);
        lpo_compute_q_lin(c, f1, q, ql);
        lpo_conserve_lin(c, q, ql);
        for (long i = 0; i < 2 * (long)c->n3; ++i) q[i] += ql[i];
        free(ql);
    } else {
        lpo_compute_q(c, f1, q);
        lpo_conserve(c, q);
    }
}

/* ------------------------------------------------------------ projection */
/* Per-axis factors of IntModes (C:364-505): T0 = int_cell e^{i eta v} dv,
 * T1 = int_cell e^{i eta v} (v-v_j)/dv dv, T2 = int_cell e^{i eta v} ((v-v_j)/dv)^2 dv,
 * with the reference's closed forms and eta == 0 branches. */
static void proj_tables(lpo_ctx *c)
{
    const int n = c->p.n, nv = c->p.nv;
    const double dv = c->dv;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < nv; ++j) {
            double e = c->eta[k];
            double gp = gridv(c, j + 0.5), gm = gridv(c, j - 0.5), gj = gridv(c, (double)j);
            double t0r, t0i, t1r, t1i, t2r, t2i;
            if (e != 0.) {
                t0r = (sin(e * gp) - sin(e * gm)) / e;
                t0i = (cos(e * gm) - cos(e * gp)) / e;
                t1r = ((gp * sin(e * gp) - gm * sin(e * gm)) / e + (cos(e * gp) - cos(e * gm)) / e / e - gj * t0r) / dv;
                t1i = ((sin(e * gp) - sin(e * gm)) / e / e + (gm * cos(e * gm) - gp * cos(e * gp)) / e - gj * t0i) / dv;
                double ar = (gp * sin(e * gp) - gm * sin(e * gm)) / e + (cos(e * gp) - cos(e * gm)) / e / e;
                double ai = (sin(e * gp) - sin(e * gm)) / e / e + (gm * cos(e * gm) - gp * cos(e * gp)) / e;
                t2r = ((gp * gp * sin(e * gp) - gm * gm * sin(e * gm) - 2 * ai) / e - 2 * gj * ar + gj * gj * t0r) / dv / dv;
                t2i = ((gm * gm * cos(e * gm) - gp * gp * cos(e * gp) + 2 * ar) / e - 2 * gj * ai + gj * gj * t0i) / dv / dv;
            } else {
                t0r = dv; t0i = 0.;
                t1r = 0.; t1i = 0.;
                t2r = dv / 12.; t2i = 0.;
            }
            double *T = c->tt;
            long b = (long)k * nv + j, stride = (long)n * nv;
            T[2 * b] = t0r; T[2 * b + 1] = t0i;
            T[2 * (stride + b)] = t1r; T[2 * (stride + b) + 1] = t1i;
            T[2 * (2 * stride + b)] = t2r; T[2 * (2 * stride + b) + 1] = t2i;
        }
}

static inline const double *tfac(const lpo_ctx *c, int which, int k, int j)
{
    return c->tt + 2 * ((long)which * c->p.n * c->p.nv + (long)k * c->p.nv + j);
}

/* IntModes (C:364-505) assembled from the per-axis factors in the reference's
 * complex-multiplication order. */
void lpo_intmodes(const lpo_ctx *c, int k1, int k2, int k3, int j1, int j2, int j3, double *r)
{
    const double *a1 = tfac(c, 0, k1, j1), *a2 = tfac(c, 0, k2, j2), *a3 = tfac(c, 0, k3, j3);
    const double *b1 = tfac(c, 1, k1, j1), *b2 = tfac(c, 1, k2, j2), *b3 = tfac(c, 1, k3, j3);
    const double *d1 = tfac(c, 2, k1, j1), *d2 = tfac(c, 2, k2, j2), *d3 = tfac(c, 2, k3, j3);
    /* l = 0 */
    r[0] = a3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - a3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    r[1] = a3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + a3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    /* l = 1 */
    r[2] = a3[0] * (b1[0] * a2[0] - b1[1] * a2[1]) - a3[1] * (b1[0] * a2[1] + a2[0] * b1[1]);
    r[3] = a3[0] * (b1[0] * a2[1] + a2[0] * b1[1]) + a3[1] * (b1[0] * a2[0] - b1[1] * a2[1]);
    /* l = 2 */
    r[4] = a3[0] * (a1[0] * b2[0] - a1[1] * b2[1]) - a3[1] * (a1[0] * b2[1] + b2[0] * a1[1]);
    r[5] = a3[0] * (a1[0] * b2[1] + b2[0] * a1[1]) + a3[1] * (a1[0] * b2[0] - a1[1] * b2[1]);
    /* l = 3 */
    r[6] = b3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - b3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    r[7] = b3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + b3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    /* l = 4 */
    double p1r = a3[0] * (d1[0] * a2[0] - d1[1] * a2[1]) - a3[1] * (d1[0] * a2[1] + a2[0] * d1[1]);
    double p1i = a3[0] * (d1[0] * a2[1] + a2[0] * d1[1]) + a3[1] * (d1[0] * a2[0] - d1[1] * a2[1]);
    double p2r = a3[0] * (a1[0] * d2[0] - a1[1] * d2[1]) - a3[1] * (a1[0] * d2[1] + d2[0] * a1[1]);
    double p2i = a3[0] * (a1[0] * d2[1] + d2[0] * a1[1]) + a3[1] * (a1[0] * d2[0] - a1[1] * d2[1]);
    double p3r = d3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - d3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    double p3i = d3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + d3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    r[8] = p1r + p2r + p3r;
    r[9] = p1i + p2i + p3i;
}

/* IntModes evaluated from scratch for every (mode, v-cell) pair, computing
 * the sines and cosines of each axis factor on every call as the reference
 * does (C:364-505); same values as lpo_intmodes, at the reference's cost. */
static void axis_factors(const lpo_ctx *c, int k, int j, double *t0, double *t1, double *t2)
{
    const double e = c->eta[k], dv = c->dv;
    const double gp = gridv(c, j + 0.5), gm = gridv(c, j - 0.5), gj = gridv(c, (double)j);
    if (e != 0.) {
        t0[0] = (sin(e * gp) - sin(e * gm)) / e;
        t0[1] = (cos(e * gm) - cos(e * gp)) / e;
        t1[0] = ((gp * sin(e * gp) - gm * sin(e * gm)) / e + (cos(e * gp) - cos(e * gm)) / e / e - gj * t0[0]) / dv;
        t1[1] = ((sin(e * gp) - sin(e * gm)) / e / e + (gm * cos(e * gm) - gp * cos(e * gp)) / e - gj * t0[1]) / dv;
        double ar = (gp * sin(e * gp) - gm * sin(e * gm)) / e + (cos(e * gp) - cos(e * gm)) / e / e;
        double ai = (sin(e * gp) - sin(e * gm)) / e / e + (gm * cos(e * gm) - gp * cos(e * gp)) / e;
        t2[0] = ((gp * gp * sin(e * gp) - gm * gm * sin(e * gm) - 2 * ai) / e - 2 * gj * ar + gj * gj * t0[0]) / dv / dv;
        t2[1] = ((gm * gm * cos(e * gm) - gp * gp * cos(e * gp) + 2 * ar) / e - 2 * gj * ai + gj * gj * t0[1]) / dv / dv;
    } else {
        t0[0] = dv; t0[1] = 0.; t1[0] = 0.; t1[1] = 0.; t2[0] = dv / 12.; t2[1] = 0.;
    }
}

static void intmodes_trig(const lpo_ctx *c, int k1, int k2, int k3, int j1, int j2, int j3, double *r)
{
    double a1[2], a2[2], a3[2], b1[2], b2[2], b3[2], d1[2], d2[2], d3[2];
    axis_factors(c, k1, j1, a1, b1, d1);
    axis_factors(c, k2, j2, a2, b2, d2);
    axis_factors(c, k3, j3, a3, b3, d3);
    r[0] = a3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - a3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    r[1] = a3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + a3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    r[2] = a3[0] * (b1[0] * a2[0] - b1[1] * a2[1]) - a3[1] * (b1[0] * a2[1] + a2[0] * b1[1]);
    r[3] = a3[0] * (b1[0] * a2[1] + a2[0] * b1[1]) + a3[1] * (b1[0] * a2[0] - b1[1] * a2[1]);
    r[4] = a3[0] * (a1[0] * b2[0] - a1[1] * b2[1]) - a3[1] * (a1[0] * b2[1] + b2[0] * a1[1]);
    r[5] = a3[0] * (a1[0] * b2[1] + b2[0] * a1[1]) + a3[1] * (a1[0] * b2[0] - a1[1] * b2[1]);
    r[6] = b3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - b3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    r[7] = b3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + b3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    double p1r = a3[0] * (d1[0] * a2[0] - d1[1] * a2[1]) - a3[1] * (d1[0] * a2[1] + a2[0] * d1[1]);
    double p1i = a3[0] * (d1[0] * a2[1] + a2[0] * d1[1]) + a3[1] * (d1[0] * a2[0] - d1[1] * a2[1]);
    double p2r = a3[0] * (a1[0] * d2[0] - a1[1] * d2[1]) - a3[1] * (a1[0] * d2[1] + d2[0] * a1[1]);
    double p2i = a3[0] * (a1[0] * d2[1] + d2[0] * a1[1]) + a3[1] * (a1[0] * d2[0] - a1[1] * d2[1]);
    double p3r = d3[0] * (a1[0] * a2[0] - a1[1] * a2[1]) - d3[1] * (a1[0] * a2[1] + a2[0] * a1[1]);
    double p3i = d3[0] * (a1[0] * a2[1] + a2[0] * a1[1]) + d3[1] * (a1[0] * a2[0] - a1[1] * a2[1]);
    r[8] = p1r + p2r + p3r;
    r[9] = p1i + p2i + p3i;
}

/* Separable evaluation of tp_l(j) = Re sum_k IntM_l(k, j) Qc(k): three
 * successive per-axis contractions of the complex mode array Qc. */
static void project_separable(const lpo_ctx *c, const double *qc, double *tp /* nv3 x 5 */)
{
    const int n = c->p.n, nv = c->p.nv;
    /* Y[a][k1][k2][j3] = sum_k3 T_a(k3, j3) qc[k1][k2][k3] */
    long ny = (long)n * n * nv, nz = (long)n * nv * nv;
    double *Y = (double *)malloc(sizeof(double) * 2 * 3 * ny);
    double *Z = (double *)malloc(sizeof(double) * 2 * 5 * nz);
    for (int a = 0; a < 3; ++a)
        for (int k1 = 0; k1 < n; ++k1)
            for (int k2 = 0; k2 < n; ++k2)
                for (int j3 = 0; j3 < nv; ++j3) {
                    double sr = 0., si = 0.;
                    for (int k3 = 0; k3 < n; ++k3) {
                        const double *t = tfac(c, a, k3, j3);
                        const double *q = qc + 2 * ((long)(k1 * n + k2) * n + k3);
                        sr += t[0] * q[0] - t[1] * q[1];
                        si += t[0] * q[1] + t[1] * q[0];
                    }
                    long o = (((long)a * n + k1) * n + k2) * nv + j3;
                    Y[2 * o] = sr; Y[2 * o + 1] = si;
                }
    /* Z[p][k1][j2][j3], p indexes (axis3 factor a, axis2 factor b):
     * 0:(0,0) 1:(0,1) 2:(0,2) 3:(1,0) 4:(2,0) */
    static const int PA[5] = {0, 0, 0, 1, 2}, PB[5] = {0, 1, 2, 0, 0};
    for (int p = 0; p < 5; ++p)
        for (int k1 = 0; k1 < n; ++k1)
            for (int j2 = 0; j2 < nv; ++j2)
                for (int j3 = 0; j3 < nv; ++j3) {
                    double sr = 0., si = 0.;
                    for (int k2 = 0; k2 < n; ++k2) {
                        const double *t = tfac(c, PB[p], k2, j2);
                        const double *y = Y + 2 * ((((long)PA[p] * n + k1) * n + k2) * nv + j3);
                        sr += t[0] * y[0] - t[1] * y[1];
                        si += t[0] * y[1] + t[1] * y[0];
                    }
                    long o = (((long)p * n + k1) * nv + j2) * nv + j3;
                    Z[2 * o] = sr; Z[2 * o + 1] = si;
                }
    /* tp_l = Re sum_k1 T_c(k1, j1) Z[p]; l=0:(c0,p0) l=1:(c1,p0) l=2:(c0,p1)
     * l=3:(c0,p3) l=4: (c2,p0)+(c0,p2)+(c0,p4) */
    for (int j1 = 0; j1 < nv; ++j1)
        for (int j2 = 0; j2 < nv; ++j2)
            for (int j3 = 0; j3 < nv; ++j3) {
                double acc[7] = {0, 0, 0, 0, 0, 0, 0};
                static const int CT[7] = {0, 1, 0, 0, 2, 0, 0}, ZP[7] = {0, 0, 1, 3, 0, 2, 4};
                for (int k1 = 0; k1 < n; ++k1)
                    for (int e = 0; e < 7; ++e) {
                        const double *t = tfac(c, CT[e], k1, j1);
                        const double *z = Z + 2 * ((((long)ZP[e] * n + k1) * nv + j2) * nv + j3);
                        acc[e] += t[0] * z[0] - t[1] * z[1];
                    }
                double *o = tp + 5 * ((long)(j1 * nv + j2) * nv + j3);
                o[0] = acc[0]; o[1] = acc[1]; o[2] = acc[2]; o[3] = acc[3];
                o[4] = acc[4] + acc[5] + acc[6];
            }
    free(Y);
    free(Z);
}

/* RK4 (C:824-906): three conserved re-evaluations of Q on node values, the
 * non-classical combination 1/2 qhat + (Q1+Q2+Q3)/6 (defect F10, kept), DG
 * projection and the {phi0, phi6} mass-matrix inverse.  With LPO_FIX_F1 the
 * state is read from slots {0,3,4,5,6} of the cell's 7-coefficient records;
 * otherwise from the stride-6 slots {0,2,3,4,5} of the compiled reference
 * (C:894-898), where ucell must then be the whole state and cell its index. */
static void rk4_impl(const lpo_ctx *c, const double *f, const double *qhat, const double *U,
                     long ubase, int stride, const int *slot, double *du, int direct)
{
    const long n3 = c->n3;
    const int nv = c->p.nv, nv3 = c->nv3;
    const double dt = c->p.dt, nu = c->p.nu;
    double *out = (double *)malloc(sizeof(double) * 2 * n3);
    double *Qn = (double *)malloc(sizeof(double) * n3);
    double *Q1n = (double *)malloc(sizeof(double) * n3);
    double *f1 = (double *)malloc(sizeof(double) * n3);
    double *q1 = (double *)malloc(sizeof(double) * 2 * n3);
    double *q2 = (double *)malloc(sizeof(double) * 2 * n3);
    double *q3 = (double *)malloc(sizeof(double) * 2 * n3);
    double *qc = (double *)malloc(sizeof(double) * 2 * n3);
    lpo_fs(c, qhat, out);
    for (long i = 0; i < n3; ++i) { Qn[i] = out[2 * i]; f1[i] = f[i] + dt * Qn[i] * nu; }
    stage_q(c, f1, q1);
    lpo_fs(c, q1, out);
    for (long i = 0; i < n3; ++i) { Q1n[i] = out[2 * i]; f1[i] = f[i] + 0.5 * dt * Qn[i] * nu + 0.5 * dt * Q1n[i] * nu; }
    stage_q(c, f1, q2);
    lpo_fs(c, q2, out);
    for (long i = 0; i < n3; ++i) { Q1n[i] = out[2 * i]; f1[i] = f[i] + 0.5 * dt * Qn[i] * nu + 0.5 * dt * Q1n[i] * nu; }
    stage_q(c, f1, q3);
    for (long i = 0; i < n3; ++i) {
        qc[2 * i] = nu * (0.5 * qhat[2 * i] + (q1[2 * i] + q2[2 * i] + q3[2 * i]) / 6.);
        qc[2 * i + 1] = nu * (0.5 * qhat[2 * i + 1] + (q1[2 * i + 1] + q2[2 * i + 1] + q3[2 * i + 1]) / 6.);
    }
    double *tp = (double *)malloc(sizeof(double) * 5 * nv3);
    if (direct) {
        const int n = c->p.n;
#pragma omp parallel for schedule(dynamic)
        for (int kt = 0; kt < nv3; ++kt) {
            int j3 = kt % nv, j2 = ((kt - j3) / nv) % nv, j1 = (kt - j3 - nv * j2) / (nv * nv);
            double a[5] = {0, 0, 0, 0, 0}, im[10];
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    for (int k = 0; k < n; ++k) {
                        long ke = k + n * (j + (long)n * i);
                        if (direct == 2) intmodes_trig(c, i, j, k, j1, j2, j3, im);
                        else lpo_intmodes(c, i, j, k, j1, j2, j3, im);
                        double qr = qc[2 * ke], qi = qc[2 * ke + 1];
                        for (int l = 0; l < 5; ++l) a[l] += im[2 * l] * qr - im[2 * l + 1] * qi;
                    }
            for (int l = 0; l < 5; ++l) tp[5 * (long)kt + l] = a[l];
        }
    } else {
        project_separable(c, qc, tp);
    }
    const double s = c->scalev, sL = c->scaleL, s3 = c->scale3;
    for (int kt = 0; kt < nv3; ++kt) {
        const double *u = U + (ubase + kt) * stride;
        const double *t = tp + 5 * (long)kt;
        double p0 = u[slot[0]] + u[slot[4]] / 4. + dt * t[0] / s / sL / s3;
        double p2 = u[slot[1]] + dt * t[1] * 12. / s / sL / s3;
        double p3 = u[slot[2]] + dt * t[2] * 12. / s / sL / s3;
        double p4 = u[slot[3]] + dt * t[3] * 12. / s / sL / s3;
        double p5 = u[slot[0]] / 4. + u[slot[4]] * 19. / 240. + dt * t[4] / s / sL / s3;
        double *d = du + 5 * (long)kt;
        d[0] = 19 * p0 / 4. - 15 * p5;
        d[4] = 60 * p5 - 15 * p0;
        d[1] = p2; d[2] = p3; d[3] = p4;
    }
    free(tp); free(out); free(Qn); free(Q1n); free(f1); free(q1); free(q2); free(q3); free(qc);
}

void lpo_rk4(const lpo_ctx *c, const double *f, const double *qhat, const double *ucell, double *du,
             int direct)
{
    static const int fixed_slots[5] = {0, 3, 4, 5, 6};
    rk4_impl(c, f, qhat, ucell, 0, 7, fixed_slots, du, direct);
}

/* RK4 of the two-species variant (C:637-737) for spatial cell `cell` of the
 * state U: the conserved qhat and qhat_lin are added first; with LPO_FIX_F1
 * the stride-7 slots, else the compiled reference's stride-6 reads. */
void lpo_rk4_lin(const lpo_ctx *c, const double *f, const double *qhat, const double *qlin, const double *U,
                 int cell, double *du, int direct)
{
    static const int fixed_slots[5] = {0, 3, 4, 5, 6};
    static const int ref_slots[5] = {0, 2, 3, 4, 5};
    const long n3 = c->n3;
    double *q0 = (double *)malloc(sizeof(double) * 2 * n3);
    for (long i = 0; i < 2 * n3; ++i) q0[i] = qhat[i] + qlin[i];
    if (c->p.fixes & LPO_FIX_F1) rk4_impl(c, f, q0, U + 7 * (long)cell * c->nv3, 0, 7, fixed_slots, du, direct);
    else rk4_impl(c, f, q0, U, (long)cell * c->nv3, 6, ref_slots, du, direct);
    free(q0);
}

/* -------------------------------------------------------- DG <-> nodes */
/* setInit_spectral: the DG polynomial of the cell containing each
 * spectral node, evaluated at the node.  Slot 2 is the compiled reference's
 * v1-slope slot (defect F2); LPO_FIX_F2 uses slot 3. */
void lpo_nodes(const lpo_ctx *c, const double *U, int cell, double *f)
{
    const int n = c->p.n, nv = c->p.nv;
    const double dv = c->dv;
    const int s1 = (c->p.fixes & LPO_FIX_F2) ? 3 : 2;
    for (int l = 0; l < n; ++l) {
        int j1 = c->nodecell[l];
        for (int m = 0; m < n; ++m) {
            int j2 = c->nodecell[m];
            for (int q = 0; q < n; ++q) {
                int j3 = c->nodecell[q];
                long k = (long)cell * c->nv3 + (j1 * nv * nv + j2 * nv + j3);
                const double *u = U + 7 * k;
                double g1 = gridv(c, (double)j1), g2 = gridv(c, (double)j2), g3 = gridv(c, (double)j3);
                f[l * n * n + m * n + q] = u[0] + u[s1] * (c->v[l] - g1) / dv + u[4] * (c->v[m] - g2) / dv +
                                           u[5] * (c->v[q] - g3) / dv +
                                           u[6] * (((c->v[l] - g1) / dv) * ((c->v[l] - g1) / dv) +
                                                   ((c->v[m] - g2) / dv) * ((c->v[m] - g2) / dv) +
                                                   ((c->v[q] - g3) / dv) * ((c->v[q] - g3) / dv));
            }
        }
    }
}

/* Collision step of every spatial cell (M:500-568 with F1/F3 as configured):
 * nodes, ComputeQ, conserve, RK4, and the scatter of dU into slots
 * {0,3,4,5,6}.  All cells read the pre-collision state. */
int lpo_collide(const lpo_ctx *c, double *U, int direct)
{
    const int nv3 = c->nv3;
    const long n3 = c->n3;
    int ncol = (c->p.fixes & LPO_FIX_F3) ? c->ncell : (c->p.nx1 < c->ncell ? c->p.nx1 : c->ncell);
    double *du = (double *)malloc(sizeof(double) * 5 * (size_t)nv3 * ncol);
    double *f = (double *)malloc(sizeof(double) * n3);
    double *q = (double *)malloc(sizeof(double) * 2 * n3);
    static const int fixed_slots[5] = {0, 3, 4, 5, 6};
    static const int ref_slots[5] = {0, 2, 3, 4, 5};
    for (int s = 0; s < ncol; ++s) {
        lpo_nodes(c, U, s, f);
        stage_q(c, f, q);
        if (c->p.fixes & LPO_FIX_F1)
            rk4_impl(c, f, q, U + 7 * (long)s * nv3, 0, 7, fixed_slots, du + 5 * (long)s * nv3, direct);
        else
            rk4_impl(c, f, q, U, (long)s * nv3, 6, ref_slots, du + 5 * (long)s * nv3, direct);
    }
    for (long k = 0; k < (long)ncol * nv3; ++k) {
        U[7 * k + 0] = du[5 * k];
        U[7 * k + 6] = du[5 * k + 4];
        U[7 * k + 3] = du[5 * k + 1];
        U[7 * k + 4] = du[5 * k + 2];
        U[7 * k + 5] = du[5 * k + 3];
    }
    free(du); free(f); free(q);
    return 0;
}

/* ------------------------------------------------------- initial state */
static double maxw(double v1, double v2, double v3, double T, double PI)
{
    double r2 = v1 * v1 + v2 * v2 + v3 * v3;
    return exp(-r2 / (2 * T)) / (2 * PI * T * sqrt(2 * T * PI)); /* Mw */
}

/* SetInit_LD: 5-point Gauss projection of (1 + A cos kx) f_v(v)
 * onto the 7-coefficient basis.  kind 0 uses the reference's Mw (T = 0.9,
 * defect F6); kind 1 the unit Maxwellian; kind 2 the two-stream profile
 * (M(v - u e1) + M(v + u e1)) / 2 with unit-temperature M. */
void lpo_set_init(const lpo_ctx *c, double *U, int kind, double u)
{
    const int nv = c->p.nv, nx1 = c->p.nx1, nx2 = c->p.nx2;
    const double a = c->p.a_amp, cw = c->p.k_wave, dv = c->dv, dx = c->dx, PI = c->PI;
    memset(U, 0, sizeof(double) * 7 * (size_t)c->size);
    for (int j1 = 0; j1 < nv; ++j1)
        for (int j2 = 0; j2 < nv; ++j2)
            for (int j3 = 0; j3 < nv; ++j3) {
                double t0 = 0., t1 = 0., t2 = 0., t3 = 0., t4 = 0.;
                for (int m1 = 0; m1 < 5; ++m1)
                    for (int m2 = 0; m2 < 5; ++m2)
                        for (int m3 = 0; m3 < 5; ++m3) {
                            double x1 = gridv(c, (double)j1) + 0.5 * dv * GX[m1];
                            double x2 = gridv(c, (double)j2) + 0.5 * dv * GX[m2];
                            double x3 = gridv(c, (double)j3) + 0.5 * dv * GX[m3];
                            double fv;
                            if (kind == 0) fv = maxw(x1, x2, x3, 0.9, PI);
                            else if (kind == 1) fv = maxw(x1, x2, x3, 1.0, PI);
                            else fv = 0.5 * (maxw(x1 - u, x2, x3, 1.0, PI) + maxw(x1 + u, x2, x3, 1.0, PI));
                            double tp = GW[m1] * GW[m2] * GW[m3] * fv;
                            t0 += tp;
                            t1 += tp * 0.5 * GX[m1];
                            t2 += tp * 0.5 * GX[m2];
                            t3 += tp * 0.5 * GX[m3];
                            t4 += tp * 0.25 * (GX[m1] * GX[m1] + GX[m2] * GX[m2] + GX[m3] * GX[m3]);
                        }
                t0 = t0 * 0.5 * 0.5 * 0.5; t1 = t1 * 0.5 * 0.5 * 0.5; t2 = t2 * 0.5 * 0.5 * 0.5;
                t3 = t3 * 0.5 * 0.5 * 0.5; t4 = t4 * 0.5 * 0.5 * 0.5;
                for (int i1 = 0; i1 < nx1; ++i1)
                    for (int i2 = 0; i2 < nx2; ++i2) {
                        long k = (long)i1 * nx2 * c->nv3 + (long)i2 * c->nv3 + (j1 * nv * nv + j2 * nv + j3);
                        double sp = sin(cw * gridx(c, i1 + 0.5)), sm = sin(cw * gridx(c, i1 - 0.5));
                        double tp0 = (dx + (sp - sm) * a / cw) * t0 / dx;
                        double tp5 = (dx + (sp - sm) * a / cw) * t4 / dx;
                        U[7 * k + 0] = 19 * tp0 / 4. - 15 * tp5;
                        U[7 * k + 6] = 60 * tp5 - 15 * tp0;
                        U[7 * k + 1] = (0.5 * (sp + sm) + (cos(cw * gridx(c, i1 + 0.5)) - cos(cw * gridx(c, i1 - 0.5))) / (cw * dx)) * (a / cw) * t0 * 12. / dx;
                        U[7 * k + 3] = (dx + (sp - sm) * a / cw) * t1 * 12 / dx;
                        U[7 * k + 4] = (dx + (sp - sm) * a / cw) * t2 * 12 / dx;
                        U[7 * k + 5] = (dx + (sp - sm) * a / cw) * t3 * 12 / dx;
                    }
            }
}

/* ------------------------------------------------------------- Poisson */
static double fle(int k, double x)
{
    if (k == 0) return 1.0;
    if (k == 1) return x;
    if (k == 2) return x * x - 1. / 12.;
    return 0.;
}
static double fled(int k, double x)
{
    (void)x;
    if (k == 0) return 0.;
    if (k == 1) return 1.;
    return 2. * x;
}

/* LDG P1 Poisson set-up on an nx x ny grid of the
 * rectangle [0,Lx] x [0,Lx] with the reference's boundary treatment; block
 * placement is generic in ny (the reference's ii-ladder at P:814-1016 assumes
 * ny >= 2, defect F7).  The band matrix is factored with lp_dgbtf2. */
static void pois_setup(lpo_ctx *c)
{
    pois_t *ps = &c->ps;
    const int NXp = c->p.nx1, NYp = c->p.nx2;
    ps->nx = NXp; ps->ny = NYp;
    const double xlength = c->p.lx, ylength = c->p.lx;
    double *DX = (double *)calloc(NXp + 2, sizeof(double));
    double *DY = (double *)calloc(NYp + 2, sizeof(double));
    double *CX = (double *)calloc(NXp + 2, sizeof(double));
    double *CY = (double *)calloc(NYp + 2, sizeof(double));
    for (int i = 1; i <= NXp; ++i) DX[i] = xlength / ((double)NXp);
    for (int j = 1; j <= NYp; ++j) DY[j] = ylength / ((double)NYp);
    CX[1] = 0. + DX[1] / 2.;
    for (int i = 2; i <= NXp; ++i) CX[i] = CX[i - 1] + DX[i - 1] / 2. + DX[i] / 2.;
    CY[1] = 0. + DY[1] / 2.;
    for (int j = 2; j <= NYp; ++j) CY[j] = CY[j - 1] + DY[j - 1] / 2. + DY[j] / 2.;
    double xa = CX[1] - DX[1] / 2., xb = CX[NXp] + DX[NXp] / 2.;
    double xc = xa + (xb - xa) / 2., xd = xa + (xb - xa) / 2.;
    ps->xc = xc; ps->xd = xd;
    ps->dxp = DX[1]; ps->dyp = DY[1];

    /* Quadrature and basis values: two Gauss points. */
    const double s3 = sqrt(3.0) / 6.0;
    double gp[3] = {0., -s3, s3}, gw[3] = {0., 0.5, 0.5};
    double gaut[3][3];
    for (int l = 1; l <= 2; ++l)
        for (int ll = 1; ll <= 2; ++ll) gaut[l][ll] = gw[l] * gw[ll];
    const double ai[3] = {1., 12.0, 12.0};
    double bl[3][3], br[3][3], bb[3][3], bt[3][3], cxv[3][3][3], cyv[3][3][3], cxy[3][3][3];
    /* mode order: 0 -> (0,0), 1 -> x-degree 1, 2 -> y-degree 1 */
    static const int DXG[3] = {0, 1, 0}, DYG[3] = {0, 0, 1};
    for (int l = 1; l <= 2; ++l)
        for (int md = 0; md < 3; ++md) {
            bl[md][l] = fle(DXG[md], -0.5) * fle(DYG[md], gp[l]);
            br[md][l] = fle(DXG[md], 0.5) * fle(DYG[md], gp[l]);
            bb[md][l] = fle(DYG[md], -0.5) * fle(DXG[md], gp[l]);
            bt[md][l] = fle(DYG[md], 0.5) * fle(DXG[md], gp[l]);
        }
    for (int l = 1; l <= 2; ++l)
        for (int ll = 1; ll <= 2; ++ll)
            for (int md = 0; md < 3; ++md) {
                cxv[md][l][ll] = fled(DXG[md], gp[l]) * fle(DYG[md], gp[ll]);
                cyv[md][l][ll] = fle(DXG[md], gp[l]) * fled(DYG[md], gp[ll]);
                cxy[md][l][ll] = fle(DXG[md], gp[l]) * fle(DYG[md], gp[ll]);
            }
    double cvx[3][3], cvy[3][3], cyll[3][3], cylr[3][3], cyrl[3][3], cyrr[3][3], cxll[3][3], cxlr[3][3],
        cxrl[3][3], cxrr[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            cvx[i][j] = 0.; cvy[i][j] = 0.;
            for (int kx = 1; kx <= 2; ++kx)
                for (int ky = 1; ky <= 2; ++ky) {
                    cvx[i][j] = cvx[i][j] - cxy[j][kx][ky] * cxv[i][kx][ky] * gaut[kx][ky];
                    cvy[i][j] = cvy[i][j] - cxy[j][kx][ky] * cyv[i][kx][ky] * gaut[kx][ky];
                }
        }
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            cyll[i][j] = cylr[i][j] = cyrl[i][j] = cyrr[i][j] = 0.;
            cxll[i][j] = cxlr[i][j] = cxrl[i][j] = cxrr[i][j] = 0.;
            for (int g = 1; g <= 2; ++g) {
                cyll[i][j] = cyll[i][j] + bl[i][g] * bl[j][g] * gw[g];
                cylr[i][j] = cylr[i][j] + br[i][g] * bl[j][g] * gw[g];
                cyrl[i][j] = cyrl[i][j] + bl[i][g] * br[j][g] * gw[g];
                cyrr[i][j] = cyrr[i][j] + br[i][g] * br[j][g] * gw[g];
                cxll[i][j] = cxll[i][j] + bb[i][g] * bb[j][g] * gw[g];
                cxlr[i][j] = cxlr[i][j] + bt[i][g] * bb[j][g] * gw[g];
                cxrl[i][j] = cxrl[i][j] + bb[i][g] * bt[j][g] * gw[g];
                cxrr[i][j] = cxrr[i][j] + bt[i][g] * bt[j][g] * gw[g];
            }
        }
    double acvx[3][3], acvy[3][3], acyll[3][3], acylr[3][3], acyrl[3][3], acyrr[3][3], acxll[3][3],
        acxlr[3][3], acxrl[3][3], acxrr[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            acvx[i][j] = ai[i] * cvx[i][j]; acvy[i][j] = ai[i] * cvy[i][j];
            acyll[i][j] = ai[i] * cyll[i][j]; acylr[i][j] = ai[i] * cylr[i][j];
            acyrl[i][j] = ai[i] * cyrl[i][j]; acyrr[i][j] = ai[i] * cyrr[i][j];
            acxll[i][j] = ai[i] * cxll[i][j]; acxlr[i][j] = ai[i] * cxlr[i][j];
            acxrr[i][j] = ai[i] * cxrr[i][j]; acxrl[i][j] = ai[i] * cxrl[i][j];
        }
    (void)acyll; (void)acylr; (void)acxll; (void)acxlr;
    memcpy(ps->acvx, acvx, sizeof(acvx)); memcpy(ps->acvy, acvy, sizeof(acvy));
    memcpy(ps->acyrr, acyrr, sizeof(acyrr)); memcpy(ps->acyrl, acyrl, sizeof(acyrl));
    memcpy(ps->acxrr, acxrr, sizeof(acxrr)); memcpy(ps->acxrl, acxrl, sizeof(acxrl));

    const double c11 = 1.;
    const int nsub = (NYp + 1) * 3 - 1, nsuper = nsub;
    const int ldab = 2 * nsub + nsuper + 1, m1 = nsub + nsuper + 1;
    const int ndim = 3 * NXp * NYp;
    ps->kl = nsub; ps->ku = nsuper; ps->ldab = ldab; ps->ndim = ndim;
    ps->ab = (double *)calloc((size_t)ldab * ndim, sizeof(double));
    ps->ipiv = (int *)calloc(ndim, sizeof(int));
#define ABP(r, col) ps->ab[((r) - 1) + (long)((col) - 1) * ldab]
    /* eps == 1 everywhere inside (CDS); outside the grid the reference's
     * static arrays are zero, which only reaches blocks it then overrides. */
    for (int ix = 1; ix <= NXp; ++ix)
        for (int jy = 1; jy <= NYp; ++jy) {
            int ii = (ix - 1) * NYp + jy;
            double col[3][3], cob[3][3], coc[3][3], cott[3][3], cor[3][3];
            const int top = (jy == NYp), right = (ix == NXp);
            const int gate = (CX[ix] >= xc && CX[ix] <= xd);
            const double ep = 1., epr = right ? 0. : 1., ept = top ? 0. : 1.;
            const double dxr = DX[ix + 1], dyt = DY[jy + 1];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double vcol = 0., vcob = 0., vcoc = 0., vcott = 0., vcor = 0.;
                    for (int k = 0; k < 3; ++k) {
                        vcol = vcol - (cvx[i][k] - cyll[i][k]) * ep * acyrl[k][j] * DY[jy] / DX[ix];
                        vcob = vcob - (cvy[i][k] - cxll[i][k]) * ep * acxrl[k][j] * DX[ix] / DY[jy];
                        if (!top) vcott = vcott + cxlr[i][k] * ept * (acvy[k][j] + acxrr[k][j]) * DX[ix] / dyt;
                        if (!right) vcor = vcor + cylr[i][k] * (acvx[k][j] + acyrr[k][j]) * epr * DY[jy] / dxr;
                        if (!top && !right)
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr - cxlr[i][k] * acxrl[k][j] * ept * DX[ix] / dyt;
                    }
                    vcol = vcol - c11 * cyrl[i][j] * DY[jy];
                    vcob = vcob - c11 * cxrl[i][j] * DX[ix];
                    vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                    vcott = vcott - c11 * cxlr[i][j] * DX[ix];
                    vcor = vcor - c11 * cylr[i][j] * DY[jy];
                    /* Neumann at the top, outside the gate. */
                    if (top && !right && !gate) {
                        vcoc = 0.;
                        for (int k = 0; k < 3; ++k)
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr;
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * cxll[i][j] * DX[ix];
                    }
                    /* Dirichlet gate at the top. */
                    if (top && gate) {
                        vcoc = 0.; vcob = 0.;
                        for (int k = 0; k < 3; ++k) {
                            vcob = vcob - (cvy[i][k] - cxll[i][k] + cxrr[i][k]) * ep * acxrl[k][j] * DX[ix] / DY[jy];
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k] + cxrr[i][k]) * ep * acvy[k][j] * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr;
                        }
                        vcob = vcob - c11 * cxrl[i][j] * DX[ix];
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                    }
                    if (jy == NYp - 1 && gate) {
                        vcott = 0.;
                        for (int k = 0; k < 3; ++k) vcott = vcott + cxlr[i][k] * ept * acvy[k][j] * DX[ix] / dyt;
                        vcott = vcott - c11 * cxlr[i][j] * DX[ix];
                    }
                    /* Dirichlet on the right. */
                    if (right && !top) {
                        vcoc = 0.; vcol = 0.;
                        for (int k = 0; k < 3; ++k) {
                            vcol = vcol - (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acyrl[k][j] * DY[jy] / DX[ix];
                            vcoc = vcoc + (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                   (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acvx[k][j] * DY[jy] / DX[ix] -
                                   cxlr[i][k] * acxrl[k][j] * ept * DX[ix] / dyt;
                        }
                        vcol = vcol - c11 * cyrl[i][j] * DY[jy];
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                    }
                    if (right && top) {
                        vcoc = 0.; vcol = 0.;
                        for (int k = 0; k < 3; ++k) {
                            vcol = vcol - (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acyrl[k][j] * DY[jy] / DX[ix];
                            vcoc = vcoc + (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                   (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acvx[k][j] * DY[jy] / DX[ix];
                        }
                        vcol = vcol - c11 * cyrl[i][j] * DY[jy];
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * cxll[i][j] * DX[ix];
                    }
                    if (ix == NXp - 1) {
                        vcor = 0.;
                        for (int k = 0; k < 3; ++k) vcor = vcor + cylr[i][k] * acvx[k][j] * epr * DY[jy] / dxr;
                        vcor = vcor - c11 * cylr[i][j] * DY[jy];
                    }
                    if (jy == 1) { /* bottom */
                        for (int k = 0; k < 3; ++k)
                            vcoc = vcoc - (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                   cvy[i][k] * ep * (acvy[k][j] + acxrr[k][j] - acxll[k][j]) * DX[ix] / DY[jy];
                        vcoc = vcoc - c11 * cxll[i][j] * DX[ix];
                    }
                    col[i][j] = vcol; cob[i][j] = vcob; coc[i][j] = vcoc; cott[i][j] = vcott; cor[i][j] = vcor;
                }
            /* Band placement: A(row, colm) at AB(m1 + row - colm, colm). */
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    int irow = (ii - 1) * 3 + j + 1;
                    int icol;
                    icol = (ii - 1) * 3 + k + 1; ABP(irow - icol + m1, icol) = coc[j][k];
                    if (jy > 1) { icol = (ii - 2) * 3 + k + 1; ABP(irow - icol + m1, icol) = cob[j][k]; }
                    if (jy < NYp) { icol = ii * 3 + k + 1; ABP(irow - icol + m1, icol) = cott[j][k]; }
                    if (ix < NXp) { icol = (ii - 1 + NYp) * 3 + k + 1; ABP(irow - icol + m1, icol) = cor[j][k]; }
                    if (ix > 1) { icol = (ii - 1 - NYp) * 3 + k + 1; ABP(irow - icol + m1, icol) = col[j][k]; }
                }
        }
#undef ABP
    lp_dgbtf2(ndim, ndim, nsub, nsuper, ps->ab, ldab, ps->ipiv);
    ps->cx = CX;
    free(DX); free(DY); free(CY);
}

void lpo_band(const lpo_ctx *c, int *dims, double *ab, int *ipiv)
{
    dims[0] = c->ps.ndim; dims[1] = c->ps.kl; dims[2] = c->ps.ku; dims[3] = c->ps.ldab;
    if (ab) memcpy(ab, c->ps.ab, sizeof(double) * (size_t)c->ps.ldab * c->ps.ndim);
    if (ipiv) memcpy(ipiv, c->ps.ipiv, sizeof(int) * c->ps.ndim);
}

/* pois2d: charge moments, right-hand side, band solve, field
 * reconstruction and the cell integrals used by the advection.  Cells are
 * indexed ii = (ix-1)*ny + (jy-1) throughout (defect F8 used nx there). */
/* Charge moments of spatial cells [s0, s1): rt[3*(s-s0)+m]. */
void lpo_charge(const lpo_ctx *c, const double *U, int s0, int s1, double *rt)
{
    const int nv = c->p.nv;
    for (int s = s0; s < s1; ++s) {
        double r0 = 0., r1 = 0., r2 = 0.;
        for (int j1 = 0; j1 < nv; ++j1)
            for (int j2 = 0; j2 < nv; ++j2)
                for (int j3 = 0; j3 < nv; ++j3) {
                    long k = (long)s * c->nv3 + j1 * nv * nv + j2 * nv + j3;
                    r0 += c->scalev * (U[7 * k + 0] + 0.25 * U[7 * k + 6]);
                    r1 += c->scalev * U[7 * k + 1];
                    r2 += c->scalev * U[7 * k + 2];
                }
        const int ii = s - s0;
        rt[3 * ii] = r0; rt[3 * ii + 1] = r1; rt[3 * ii + 2] = r2;
    }
}

void lpo_poisson(const lpo_ctx *c, const double *U, double *potc, double *phix, double *phiy,
                 double *fields)
{
    const int nc = c->ps.nx * c->ps.ny;
    double *rt = (double *)calloc(3 * (size_t)nc, sizeof(double));
    lpo_charge(c, U, 0, nc, rt);
    lpo_poisson_rt(c, rt, potc, phix, phiy, fields);
    free(rt);
}

/* The rest of pois2d from given charge moments rt (3 per spatial cell). */
void lpo_poisson_rt(const lpo_ctx *c, const double *rt, double *potc, double *phix, double *phiy,
                    double *fields)
{
    const pois_t *ps = &c->ps;
    const int NXp = ps->nx, NYp = ps->ny;
    const int nc = NXp * NYp;
    double *b = (double *)calloc(ps->ndim, sizeof(double));
    const double PEP = 1., DOP = 1., DXv = ps->dxp, DYv = ps->dyp;
    for (int ii = 0; ii < nc; ++ii) {
        /* boundary data are zero, so only the charge terms remain */
        b[3 * ii + 0] = PEP * (rt[3 * ii] - DOP) * DXv * DYv;
        b[3 * ii + 1] = PEP * rt[3 * ii + 1] * DXv * DYv / 12.;
        b[3 * ii + 2] = PEP * rt[3 * ii + 2] * DXv * DYv / 12.;
    }
    lp_dgbtrs_n(ps->ndim, ps->kl, ps->ku, ps->ab, ps->ldab, ps->ipiv, b);
    for (int i = 0; i < 3 * nc; ++i) potc[i] = b[i];
    /* E_x */
    for (int ix = 1; ix <= NXp; ++ix)
        for (int jy = 1; jy <= NYp; ++jy) {
            int ii = (ix - 1) * NYp + jy - 1, il = (ix - 2) * NYp + jy - 1;
            for (int k = 0; k < 3; ++k) {
                double s = 0.;
                if (ix == 1) {
                    for (int kk = 0; kk < 3; ++kk) s = s + (ps->acvx[k][kk] + ps->acyrr[k][kk]) * potc[3 * ii + kk];
                    s = s - ps->acyrl[k][0] * 0.;
                } else if (ix == NXp) {
                    for (int kk = 0; kk < 3; ++kk) s = s + ps->acvx[k][kk] * potc[3 * ii + kk] - ps->acyrl[k][kk] * potc[3 * il + kk];
                    s = s + ps->acyrr[k][0] * 0.;
                } else {
                    for (int kk = 0; kk < 3; ++kk)
                        s = s + (ps->acvx[k][kk] + ps->acyrr[k][kk]) * potc[3 * ii + kk] - ps->acyrl[k][kk] * potc[3 * il + kk];
                }
                phix[3 * ii + k] = -s / DXv;
            }
        }
    /* E_y */
    for (int ix = 1; ix <= NXp; ++ix)
        for (int jy = 1; jy <= NYp; ++jy) {
            int ii = (ix - 1) * NYp + jy - 1, il = (ix - 1) * NYp + jy - 2;
            const int gate = (ps->cx[ix] >= ps->xc && ps->cx[ix] <= ps->xd);
            for (int k = 0; k < 3; ++k) {
                double s = 0.;
                if (jy == 1) {
                    phiy[3 * ii + k] = (k == 0) ? -potc[3 * ii + 2] / DYv : 0.;
                    continue;
                }
                if (jy == NYp && gate) {
                    for (int kk = 0; kk < 3; ++kk) s = s + ps->acvy[k][kk] * potc[3 * ii + kk] - ps->acxrl[k][kk] * potc[3 * il + kk];
                    s = s + ps->acxrr[k][0] * 0.;
                } else {
                    for (int kk = 0; kk < 3; ++kk)
                        s = s + (ps->acvy[k][kk] + ps->acxrr[k][kk]) * potc[3 * ii + kk] - ps->acxrl[k][kk] * potc[3 * il + kk];
                }
                phiy[3 * ii + k] = -s / DYv;
            }
        }
    if (fields) {
        for (int ii = 0; ii < nc; ++ii) {
            double *F = fields;
            F[0 * nc + ii] = phix[3 * ii];
            F[1 * nc + ii] = phix[3 * ii + 1] / 12.;
            F[2 * nc + ii] = phix[3 * ii + 2] / 12.;
            F[3 * nc + ii] = phix[3 * ii] / 12.;
            F[4 * nc + ii] = 0.;
            F[5 * nc + ii] = phix[3 * ii] / 12.;
            F[6 * nc + ii] = phiy[3 * ii];
            F[7 * nc + ii] = phiy[3 * ii + 1] / 12.;
            F[8 * nc + ii] = phiy[3 * ii + 2] / 12.;
            F[9 * nc + ii] = phiy[3 * ii] / 12.;
            F[10 * nc + ii] = 0.;
            F[11 * nc + ii] = phiy[3 * ii] / 12.;
            F[12 * nc + ii] = phix[3 * ii] > 0. ? 1. : -1.;
            F[13 * nc + ii] = phiy[3 * ii] > 0. ? 1. : -1.;
        }
    }
    free(b);
}

/* ----------------------------------------------------------- advection */
/* Right-hand side H of one DG record (A:213-405 for I1, I2, I3, I5 and the
 * combination at A:455-467); H[2] is 0 (defect F4). */
static void flux_h(const lpo_ctx *c, const double *U, long k, const double *IE, const double *IXE,
                   const double *IXXE, double *H)
{
    const int nv = c->p.nv, nx1 = c->p.nx1, nx2 = c->p.nx2;
    const long sv = c->nv3;
    const double dv = c->dv;
    const long jm = k % sv, s = (k - jm) / sv;
    const int j3 = (int)(jm % nv), j2 = (int)(((jm - j3) % ((long)nv * nv)) / nv),
              j1 = (int)((jm - j3 - j2 * nv) / ((long)nv * nv));
    const int i2 = (int)(s % nx2), i1 = (int)((s - i2) / nx2);
    const double G = gridv(c, (double)j1);
    const double *u = U + 7 * k;
    /* I3 neighbours (x1 upwind by sign of v1, periodic). */
    long kr3, kl3;
    double ur3, ul3;
    if (j1 < nv / 2) {
        int iir = i1 + 1;
        if (iir == nx1) iir = 0;
        kr3 = (long)iir * nx2 * sv + (long)i2 * sv + jm;
        kl3 = k;
        ur3 = -U[kr3 * 7 + 1];
        ul3 = -U[kl3 * 7 + 1];
    } else {
        int iil = i1 - 1;
        if (iil == -1) iil = nx1 - 1;
        kr3 = k;
        kl3 = (long)iil * nx2 * sv + (long)i2 * sv + jm;
        ur3 = U[kr3 * 7 + 1];
        ul3 = U[kl3 * 7 + 1];
    }
    const double *R3 = U + 7 * kr3, *L3 = U + 7 * kl3;
    /* I5 neighbours (v1 upwind by sign of the cell-average E_x, zero inflow).
     * pois2d leaves cell averages of E_x in IE_X, IXE_X, IXXE_X
     * where the weak form needs cell integrals (the 1-D field code at A:180
     * uses intE, the integral); LPO_FIX_F12 scales them by dx. */
    const double fs = (c->p.fixes & LPO_FIX_F12) ? c->dx : 1.;
    const double ie = IE[s] * fs, ixe = IXE[s] * fs, ixxe = IXXE[s] * fs;
    int j1r, j1l;
    long kr5, kl5;
    double ur5 = 0., ul5 = 0.;
    if (ie > 0) {
        j1r = j1 + 1; j1l = j1;
        kr5 = s * sv + (j1r * nv * nv + j2 * nv + j3);
        kl5 = k;
        if (j1r < nv) ur5 = -U[kr5 * 7 + 3];
        ul5 = -U[kl5 * 7 + 3];
    } else {
        j1r = j1; j1l = j1 - 1;
        kr5 = k;
        kl5 = s * sv + (j1l * nv * nv + j2 * nv + j3);
        ur5 = U[kr5 * 7 + 3];
        if (j1l > -1) ul5 = U[kl5 * 7 + 3];
    }
    const int hasr = j1r < nv, hasl = j1l > -1;
    const double *R5 = hasr ? U + 7 * kr5 : NULL, *L5 = hasl ? U + 7 * kl5 : NULL;
    static const int LS[6] = {0, 1, 3, 4, 5, 6};
    double tp[6];
    for (int q = 0; q < 6; ++q) {
        const int l = LS[q];
        double i1v = 0., i2v = 0., i3v = 0., i5v = 0.;
        if (l == 1) i1v = dv * dv * dv * (G * u[0] + dv * u[3] / 12. + u[6] * G / 4.);
        if (l == 3) i2v = (((u[0] + u[6] / 4.) * ie + u[1] * ixe) * c->scalev) / dv;
        else if (l == 6) i2v = u[3] * dv * dv * ie / 6.;
        switch (l) {
        case 0: i3v = dv * dv * dv * ((R3[0] + 0.5 * ur3 - L3[0] - 0.5 * ul3) * G + (R3[3] - L3[3]) * dv / 12. + (R3[6] - L3[6]) * G / 4.); break;
        case 1: i3v = 0.5 * dv * dv * dv * ((R3[0] + 0.5 * ur3 + L3[0] + 0.5 * ul3) * G + (R3[3] + L3[3]) * dv / 12. + (R3[6] + L3[6]) * G / 4.); break;
        case 3: i3v = dv * dv * (((R3[0] - L3[0]) * dv * dv + (ur3 - ul3) * 0.5 * dv * dv + (R3[3] - L3[3]) * dv * G) / 12. + (R3[6] - L3[6]) * dv * dv * 19. / 720.); break;
        case 4: i3v = (R3[4] - L3[4]) * G * dv * dv * dv / 12.; break;
        case 5: i3v = (R3[5] - L3[5]) * G * dv * dv * dv / 12.; break;
        case 6: i3v = dv * dv * dv * ((R3[0] + 0.5 * ur3 - L3[0] - 0.5 * ul3) * G / 4. + (R3[3] - L3[3]) * dv * 19. / 720. + (R3[6] - L3[6]) * G * 19. / 240.); break;
        }
        switch (l) {
        case 0:
            if (hasr && hasl) i5v = dv * dv * (R5[0] + 0.5 * ur5 + R5[6] * 5. / 12. - L5[0] - 0.5 * ul5 - L5[6] * 5. / 12.) * ie + dv * dv * (R5[1] - L5[1]) * ixe;
            else if (hasr) i5v = dv * dv * (R5[0] + 0.5 * ur5 + R5[6] * 5. / 12.) * ie + dv * dv * R5[1] * ixe;
            else if (hasl) i5v = dv * dv * (-L5[0] - 0.5 * ul5 - L5[6] * 5. / 12.) * ie - dv * dv * L5[1] * ixe;
            break;
        case 1:
            if (hasr && hasl) i5v = dv * dv * ((R5[0] + 0.5 * ur5 + R5[6] * 5. / 12. - L5[0] - 0.5 * ul5 - L5[6] * 5. / 12.) * ixe + (R5[1] - L5[1]) * ixxe);
            else if (hasr) i5v = dv * dv * ((R5[0] + 0.5 * ur5 + R5[6] * 5. / 12.) * ixe + R5[1] * ixxe);
            else if (hasl) i5v = dv * dv * ((-L5[0] - 0.5 * ul5 - L5[6] * 5. / 12.) * ixe - L5[1] * ixxe);
            break;
        case 3:
            if (hasr && hasl) i5v = 0.5 * (dv * dv * (R5[0] + 0.5 * ur5 + R5[6] * 5. / 12. + L5[0] + 0.5 * ul5 + L5[6] * 5. / 12.) * ie + dv * dv * (R5[1] + L5[1]) * ixe);
            else if (hasr) i5v = 0.5 * (dv * dv * (R5[0] + 0.5 * ur5 + R5[6] * 5. / 12.) * ie + dv * dv * R5[1] * ixe);
            else if (hasl) i5v = 0.5 * (dv * dv * (L5[0] + 0.5 * ul5 + L5[6] * 5. / 12.) * ie + dv * dv * L5[1] * ixe);
            break;
        case 4:
            if (hasr && hasl) i5v = (R5[4] - L5[4]) * ie * dv * dv / 12.;
            else if (hasr) i5v = R5[4] * ie * dv * dv / 12.;
            else if (hasl) i5v = -L5[4] * ie * dv * dv / 12.;
            break;
        case 5:
            if (hasr && hasl) i5v = (R5[5] - L5[5]) * ie * dv * dv / 12.;
            else if (hasr) i5v = R5[5] * ie * dv * dv / 12.;
            else if (hasl) i5v = -L5[5] * ie * dv * dv / 12.;
            break;
        case 6:
            if (hasr && hasl) i5v = dv * dv * (((R5[0] + 0.5 * ur5 - L5[0] - 0.5 * ul5) * 5. / 12. + (R5[6] - L5[6]) * 133. / 720.) * ie + (R5[1] - L5[1]) * ixe * 5. / 12.);
            else if (hasr) i5v = dv * dv * (((R5[0] + 0.5 * ur5) * 5. / 12. + R5[6] * 133. / 720.) * ie + R5[1] * ixe * 5. / 12.);
            else if (hasl) i5v = -dv * dv * (((L5[0] + 0.5 * ul5) * 5. / 12. + L5[6] * 133. / 720.) * ie + L5[1] * ixe * 5. / 12.);
            break;
        }
        tp[q] = i1v - i2v - i3v + i5v;
    }
    const double dx = c->dx, sv3 = c->scalev;
    H[0] = (19 * tp[0] / 4. - 15 * tp[5]) / dx / sv3;
    H[6] = (60 * tp[5] - 15 * tp[0]) / dx / sv3;
    H[1] = tp[1] * 12. / dx / sv3;
    H[2] = 0.;
    H[3] = tp[2] * 12. / dx / sv3;
    H[4] = tp[3] * 12. / dx / sv3;
    H[5] = tp[4] * 12. / dx / sv3;
}

/* Cell sizes of a slab of a larger grid: its own geometry gives lx / nx1
 * of the slab, which can differ from the grid's in the last bit. */
void lpo_set_cell_size(lpo_ctx *c, double dx, double dy)
{
    c->dx = dx;
    c->dy = dy;
}

/* One SSP-RK3 stage (A:455-581) with given field integrals fields14 (the
 * 14 x ncell output of pois2d): Uout = combination(U0, Us, H(Us)). */
void lpo_rk3_stage(const lpo_ctx *c, const double *U0, const double *Us, const double *fl, int stage,
                   double *Uout)
{
    const long size = c->size, nc = c->ncell;
    const double dt = c->p.dt;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < size; ++k) {
        double H[7];
        flux_h(c, Us, k, fl, fl + nc, fl + 3 * nc, H);
        for (int l = 0; l < 7; ++l) {
            if (stage == 0) Uout[7 * k + l] = U0[7 * k + l] + dt * H[l];
            else if (stage == 1) Uout[7 * k + l] = 0.75 * U0[7 * k + l] + 0.25 * Us[7 * k + l] + 0.25 * dt * H[l];
            else Uout[7 * k + l] = U0[7 * k + l] / 3. + Us[7 * k + l] * 2. / 3. + dt * H[l] * 2. / 3.;
        }
    }
}

/* RK3 (A:428-601): SSP-RK3 with a Poisson solve before each stage. */
void lpo_rk3(const lpo_ctx *c, double *U)
{
    const long size = c->size, nc = c->ncell;
    double *U1 = (double *)malloc(sizeof(double) * 7 * size);
    double *Ut = (double *)malloc(sizeof(double) * 7 * size);
    double *potc = (double *)malloc(sizeof(double) * 3 * nc);
    double *px = (double *)malloc(sizeof(double) * 3 * nc);
    double *py = (double *)malloc(sizeof(double) * 3 * nc);
    double *fl = (double *)malloc(sizeof(double) * 14 * nc);
    const double dt = c->p.dt;
    for (int stage = 0; stage < 3; ++stage) {
        const double *Us = stage == 0 ? U : U1;
        lpo_poisson(c, Us, potc, px, py, fl);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < size; ++k) {
            double H[7];
            flux_h(c, Us, k, fl, fl + nc, fl + 3 * nc, H);
            for (int l = 0; l < 7; ++l) {
                if (stage == 0) Ut[7 * k + l] = U[7 * k + l] + dt * H[l];
                else if (stage == 1) Ut[7 * k + l] = 0.75 * U[7 * k + l] + 0.25 * U1[7 * k + l] + 0.25 * dt * H[l];
                else Ut[7 * k + l] = U[7 * k + l] / 3. + U1[7 * k + l] * 2. / 3. + dt * H[l] * 2. / 3.;
            }
        }
        if (stage < 2) memcpy(U1, Ut, sizeof(double) * 7 * size);
        else memcpy(U, Ut, sizeof(double) * 7 * size);
    }
    free(U1); free(Ut); free(potc); free(px); free(py); free(fl);
}

/* One time step of the driver loop (M:496-568): advection, then collisions
 * when nu > 0. */
void lpo_step(const lpo_ctx *c, double *U, int direct)
{
    lpo_rk3(c, U);
    if (c->p.nu > 0.) lpo_collide(c, U, direct);
}

/* Moments (MC:3-47, computeEleE): mass, momentum, kinetic and electric
 * energy.  Kinetic energy covers the first nx1 spatial cells as in the
 * reference unless LPO_FIX_F3. */
void lpo_moments(const lpo_ctx *c, const double *U, const double *phix, const double *phiy,
                 double *out)
{
    const int nv = c->p.nv;
    const long sv = c->nv3, size = c->size;
    const double dv = c->dv, dx = c->dx, dy = c->dy;
    double m = 0., a1 = 0., a2 = 0., a3 = 0., ke = 0.;
    for (long k = 0; k < size; ++k) m += U[k * 7 + 0] + U[k * 7 + 6] / 4.;
    for (long k = 0; k < size; ++k) {
        long j = k % sv;
        int j3 = (int)(j % nv), j2 = (int)(((j - j3) % ((long)nv * nv)) / nv), j1 = (int)((j - j3 - j2 * nv) / ((long)nv * nv));
        a1 += gridv(c, (double)j1) * dv * U[k * 7 + 0] + U[k * 7 + 3] * dv * dv / 12. + U[k * 7 + 6] * gridv(c, (double)j1) * dv / 4.;
        a2 += gridv(c, (double)j2) * dv * U[k * 7 + 0] + U[k * 7 + 4] * dv * dv / 12. + U[k * 7 + 6] * gridv(c, (double)j2) * dv / 4.;
        a3 += gridv(c, (double)j3) * dv * U[k * 7 + 0] + U[k * 7 + 5] * dv * dv / 12. + U[k * 7 + 6] * gridv(c, (double)j3) * dv / 4.;
    }
    long kend = (c->p.fixes & LPO_FIX_F3) ? size : (long)c->p.nx1 * sv;
    if (kend > size) kend = size;
    for (long k = 0; k < kend; ++k) {
        long j = k % sv;
        int j3 = (int)(j % nv), j2 = (int)(((j - j3) % ((long)nv * nv)) / nv), j1 = (int)((j - j3 - j2 * nv) / ((long)nv * nv));
        double g1 = gridv(c, (double)j1), g2 = gridv(c, (double)j2), g3 = gridv(c, (double)j3);
        double tp1 = g1 * g1 + g2 * g2 + g3 * g3;
        ke += U[k * 7 + 0] * (tp1 + dv * dv / 4.) * dv + (g1 * U[k * 7 + 3] + g2 * U[k * 7 + 4] + g3 * U[k * 7 + 5]) * dv * dv / 6. +
              U[k * 7 + 6] * (dv * dv * dv * 19. / 240. + tp1 * dv / 4.);
    }
    out[0] = m * dx * dy * c->scalev;
    out[1] = a1 * dx * dy * dv * dv;
    out[2] = a2 * dx * dy * dv * dv;
    out[3] = a3 * dx * dy * dv * dv;
    out[4] = 0.5 * (ke * (dx * dy * dv * dv));
    double e = 0.;
    for (long s = 0; s < c->ncell; ++s) {
        e += phix[3 * s] * phix[3 * s] + phiy[3 * s] * phiy[3 * s];
        e += (phix[3 * s + 1] * phix[3 * s + 1] + phiy[3 * s + 1] * phiy[3 * s + 1]) / 12;
        e += (phix[3 * s + 2] * phix[3 * s + 2] + phiy[3 * s + 2] * phiy[3 * s + 2]) / 12;
    }
    out[5] = 0.5 * (dx * dy) * e;
}

/* ------------------------------------------------------------- context */
int lpo_create(const lpo_params *p, lpo_ctx **out)
{
    if (!p || p->nx1 < 2 || p->nx2 < 1 || p->nv < 2 || p->n < 2 || (p->n % 2)) return 1;
    lpo_ctx *c = (lpo_ctx *)calloc(1, sizeof(lpo_ctx));
    c->p = *p;
    c->PI = M_PI;
    c->nv3 = p->nv * p->nv * p->nv;
    c->n3 = p->n * p->n * p->n;
    c->ncell = p->nx1 * p->nx2;
    c->size = (long)c->ncell * c->nv3;
    /* M:38-40, M:66, M:270-284 */
    c->dv = 2. * p->lv / p->nv;
    c->dx = p->lx / p->nx1;
    c->dy = p->lx / p->nx2;
    c->scaleL = 8 * p->lv * p->lv * p->lv;
    c->scalev = c->dv * c->dv * c->dv;
    c->scale = 1.0 / sqrt(2.0 * M_PI);
    c->scale3 = pow(c->scale, 3.0);
    c->L_v = p->lv;
    c->R_v = p->lv;
    c->L_eta = 0.5 * (double)(p->n - 1) * c->PI / c->L_v;
    c->h_v = 2.0 * c->L_v / (double)(p->n - 1);
    c->h_eta = 2.0 * c->L_eta / (double)(p->n);
    const int n = p->n;
    c->v = (double *)malloc(sizeof(double) * n);
    c->eta = (double *)malloc(sizeof(double) * n);
    c->wt = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) {
        c->eta[i] = -c->L_eta + (double)i * c->h_eta;
        c->v[i] = -c->L_v + (double)i * c->h_v;
    }
    if ((p->fixes & LPO_FIX_F11) && fabs(c->eta[n / 2]) < 1e-12 * c->L_eta) c->eta[n / 2] = 0.;
    c->wt[0] = 0.5;
    c->wt[n - 1] = 0.5;
    for (int i = 1; i < n - 1; ++i) c->wt[i] = 1.0;
    c->nodecell = (int *)malloc(sizeof(int) * n);
    for (int l = 0; l < n; ++l) {
        int j = (int)((l * c->h_v) / c->dv);
        if (j == p->nv) j = p->nv - 1;
        c->nodecell[l] = j;
    }
    c->sh = (double *)malloc(sizeof(double) * 6 * c->n3);
    c->ah = (double *)malloc(sizeof(double) * c->n3);
    c->rzero = (unsigned char *)malloc(c->n3);
    omega_tables(c);
    c->c1 = (double *)malloc(sizeof(double) * 5 * c->n3);
    c->c2 = (double *)malloc(sizeof(double) * 5 * c->n3);
    cons_tables(c);
    c->tt = (double *)malloc(sizeof(double) * 2 * 3 * n * p->nv);
    proj_tables(c);
    pois_setup(c);
    *out = c;
    return 0;
}

void lpo_destroy(lpo_ctx *c)
{
    if (!c) return;
    free(c->v); free(c->eta); free(c->wt); free(c->sh); free(c->ah); free(c->rzero);
    free(c->c1); free(c->c2); free(c->nodecell); free(c->tt);
    free(c->ps.ab); free(c->ps.ipiv); free(c->ps.cx);
    free(c);
}

void lpo_grids(const lpo_ctx *c, double *v, double *eta, double *wt, double *sc)
{
    const int n = c->p.n;
    if (v) memcpy(v, c->v, sizeof(double) * n);
    if (eta) memcpy(eta, c->eta, sizeof(double) * n);
    if (wt) memcpy(wt, c->wt, sizeof(double) * n);
    if (sc) {
        double s[14] = {c->L_eta, c->h_eta, c->h_v, c->L_v, c->R_v, c->scale, c->scale3,
                        c->scaleL, c->scalev, c->dv, c->dx, c->p.lx, c->p.lv, c->dy};
        memcpy(sc, s, sizeof(s));
    }
}


/* Entropy int f log f (EntropyCalculations.cpp:11-65): 5-point Gauss rule in
 * x1, v1, v2, v3 over the records of the first nx1 spatial cells (cells
 * s < nx1, as the reference's loop i < Nx), f > 0 only. */
double lpo_entropy(const lpo_ctx *c, const double *U)
{
    static const double wt5[5] = {0.5688888888888889, 0.4786286704993665, 0.4786286704993665,
                                  0.2369268850561891, 0.2369268850561891};
    static const double vt5[5] = {0., -0.5384693101056831, 0.5384693101056831, -0.9061798459386640,
                                  0.9061798459386640};
    const int nv = c->p.nv;
    const double dv = c->dv, dx = c->dx;
    long ncell = (c->p.fixes & LPO_FIX_F3) ? (long)c->p.nx1 * c->p.nx2 : c->p.nx1;
    if (ncell > (long)c->p.nx1 * c->p.nx2) ncell = (long)c->p.nx1 * c->p.nx2;
    double ent = 0.;
    for (long i = 0; i < ncell; ++i)
        for (int j1 = 0; j1 < nv; ++j1)
            for (int j2 = 0; j2 < nv; ++j2)
                for (int j3 = 0; j3 < nv; ++j3) {
                    const long k = i * c->nv3 + ((long)j1 * nv + j2) * nv + j3;
                    const double *u = U + 7 * k;
                    for (int nx = 0; nx < 5; ++nx)
                        for (int a = 0; a < 5; ++a)
                            for (int b = 0; b < 5; ++b)
                                for (int e = 0; e < 5; ++e) {
                                    const double xd = 0.5 * vt5[nx] * dx / dx, v1 = 0.5 * vt5[a] * dv / dv,
                                                 v2 = 0.5 * vt5[b] * dv / dv, v3 = 0.5 * vt5[e] * dv / dv;
                                    const double f = u[0] + u[1] * xd + u[3] * v1 + u[4] * v2 + u[5] * v3 +
                                                     u[6] * (v1 * v1 + v2 * v2 + v3 * v3);
                                    if (f > 0) ent += wt5[nx] * wt5[a] * wt5[b] * wt5[e] * f * log(f);
                                }
                }
    return ent * 0.5 * dv * 0.5 * dv * 0.5 * dv * 0.5 * dx;
}

/* The (x1, v1) marginal of PrintMarginal / f_marg2D_x1v1
 * (MarginalCreation.cpp:35-61, 174-197) at 4 x 4 points per cell pair:
 * out[(i1*4 + a) * (nv*4) + j1*4 + b]. */
void lpo_marginal_x1v1(const lpo_ctx *c, const double *U, double *out)
{
    const int nv = c->p.nv, nx1 = c->p.nx1, nx2 = c->p.nx2;
    const double dv = c->dv, dx = c->dx;
    const double ddx = dx / 4, ddv = dv / 4;
    long o = 0;
    /* sample positions as the reference forms them: left cell edge plus
     * multiples of a quarter cell, then the offset from the centre */
    for (int i1 = 0; i1 < nx1; ++i1)
        for (int a = 0; a < 4; ++a) {
            const double x1 = (((double)i1 - 0.5) + 0.5) * dx + a * ddx;
            const double xd = x1 - ((double)i1 + 0.5) * dx;
            for (int j1 = 0; j1 < nv; ++j1)
                for (int b = 0; b < 4; ++b) {
                    const double v1 = gridv(c, (double)j1 - 0.5) + b * ddv;
                    const double vd = v1 - gridv(c, (double)j1);
                    double r = 0.;
                    for (int i2 = 0; i2 < nx2; ++i2)
                        for (int jj = 0; jj < nv * nv; ++jj) {
                            const double *u = U + 7 * (((long)i1 * nx2 + i2) * c->nv3 + (long)j1 * nv * nv + jj);
                            r += dx * dv * dv * u[0] + dv * dv * u[1] * xd + dx * dv * u[3] * vd +
                                 dx * u[6] * (vd * vd + dv * dv / 6.);
                        }
                    out[o++] = r;
                }
        }
}
