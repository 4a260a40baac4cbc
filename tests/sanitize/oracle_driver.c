/* Runs the CPU oracle's routines on small cases; built with AddressSanitizer
 * and UndefinedBehaviorSanitizer by tests/test_host_sanitizers.py, which
 * fails on any sanitizer report or non-zero exit.  Test infrastructure. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "lp_oracle.h"

static int finite_all(const double *x, long n) {
    for (long i = 0; i < n; ++i)
        if (!isfinite(x[i])) return 0;
    return 1;
}

static int run(int nx1, int nx2, int nv, int n, double lv, unsigned fixes, int linear_ei) {
    lpo_params p = {nx1, nx2, nv, n, lv, 4.0 * 3.14159265358979323846, 0.05, 0.01, 0.3, 0.5, fixes, linear_ei};
    lpo_ctx *c = NULL;
    if (lpo_create(&p, &c) != 0 || !c) return 1;
    const long n3 = (long)n * n * n, nv3 = (long)nv * nv * nv, ncell = (long)nx1 * nx2, size = ncell * nv3;
    double *U = calloc((size_t)size * 7, sizeof(double)), *f = calloc((size_t)n3, sizeof(double));
    double *q = calloc((size_t)n3 * 2, sizeof(double)), *q2 = calloc((size_t)n3 * 2, sizeof(double));
    double *tmp = calloc((size_t)n3 * 2, sizeof(double)), *du = calloc((size_t)nv3 * 5, sizeof(double));
    double *c1 = calloc((size_t)5 * n3, sizeof(double)), *c2 = calloc((size_t)5 * n3, sizeof(double));
    double v[64], eta[64], wt[64], sc[14], cct[25], im[10], m6[6], cct4[4];
    double *potc = calloc((size_t)3 * ncell, sizeof(double)), *phix = calloc((size_t)3 * ncell, sizeof(double));
    double *phiy = calloc((size_t)3 * ncell, sizeof(double)), *fl = calloc((size_t)14 * ncell, sizeof(double));
    double *marg = calloc((size_t)nx1 * 4 * nv * 4, sizeof(double));
    int ok = 1;
    lpo_grids(c, v, eta, wt, sc);
    lpo_cons(c, c1, c2, cct);
    lpo_set_init(c, U, 2, 2.0);
    lpo_set_init(c, U, 1, 0.0);
    lpo_nodes(c, U, 0, f);
    for (long i = 0; i < n3; ++i) { tmp[2 * i] = f[i]; tmp[2 * i + 1] = 0.0; }
    lpo_fft3d(c, tmp, q2);
    lpo_fs(c, q2, tmp);
    (void)lpo_weight(c, 0, (int)(n3 - 1));
    lpo_compute_q(c, f, q);
    lpo_conserve(c, q);
    lpo_intmodes(c, 1, 2, 3, 0, nv - 1, nv / 2, im);
    lpo_rk4(c, f, q, U, du, 1);
    lpo_rk4(c, f, q, U, du, 0);
    ok &= finite_all(du, nv3 * 5);
    lpo_poisson(c, U, potc, phix, phiy, fl);
    lpo_moments(c, U, phix, phiy, m6);
    (void)lpo_entropy(c, U);
    lpo_marginal_x1v1(c, U, marg);
    lpo_rk3(c, U);
    ok &= lpo_collide(c, U, 0) == 0;
    lpo_step(c, U, 0);
    ok &= finite_all(U, size * 7);
    if (linear_ei) {
        (void)lpo_weight_lin(c, 1, 2);
        lpo_compute_q_lin(c, f, q, q2);
        lpo_conserve_lin(c, q, q2);
        lpo_cct_lin(c, cct4);
        lpo_rk4_lin(c, f, q, q2, U, 0, du, 0);
        ok &= finite_all(du, nv3 * 5);
    }
    int dims[4];
    lpo_band(c, dims, NULL, NULL);
    double *ab = calloc((size_t)dims[0] * dims[3], sizeof(double));
    int *ipiv = calloc((size_t)dims[0], sizeof(int));
    lpo_band(c, dims, ab, ipiv);
    free(ab); free(ipiv);
    free(U); free(f); free(q); free(q2); free(tmp); free(du); free(c1); free(c2);
    free(potc); free(phix); free(phiy); free(fl); free(marg);
    lpo_destroy(c);
    return ok ? 0 : 2;
}

int main(void) {
    int r = 0;
    r |= run(2, 2, 4, 8, 5.25, 0u, 0);
    r |= run(4, 1, 6, 8, 5.25, LPO_FIX_DEFAULT, 0);
    r |= run(3, 1, 4, 16, 6.0, LPO_FIX_DEFAULT, 0);
    r |= run(2, 2, 4, 8, 5.25, LPO_FIX_F2 | LPO_FIX_F3, 1);
    if (r) { fprintf(stderr, "oracle driver: status %d\n", r); return r; }
    printf("ok\n");
    return 0;
}
