/* CPU restatement of the Landau-Poisson reference's hot path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arms of bench.py may load this library, and only
 * as the checker or the timed CPU baseline; the shipped GPU library never
 * links or calls it.
 *
 * Geometry is generic: nx1 x nx2 spatial cells (nx2 = nx1 reproduces the
 * reference's 2-D layout; nx2 = 1 is the 1-D reduction), nv^3 DG velocity
 * cells with 7 coefficients each (AoS, stride 7), n^3 spectral nodes.
 * Cell index s = i1*nx2 + i2; DG record k = s*nv^3 + (j1*nv + j2)*nv + j3.
 *
 * Pinning: every routine is checked against golden vectors produced by the
 * reference's own sources built here (oracle/build_ref.sh,
 * tests/golden/make_golden.py).
 */
#ifndef LP_ORACLE_H
#define LP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Fixes of reference defects, one flag each (the same bits as LP_FIX_* of
 * lp_gb300.h); with a flag clear the oracle keeps the reference's behaviour. */
#define LPO_FIX_F1 1u   /* RK4 reads the stride-7 slots {0,3,4,5,6} */
#define LPO_FIX_F2 2u   /* setInit_spectral uses slot 3 as the v1 slope */
#define LPO_FIX_F3 4u   /* collide every spatial cell, not only s < nx1 */
#define LPO_FIX_F11 8u  /* snap the middle Fourier node eta[n/2] to exactly 0 */
#define LPO_FIX_F12 16u /* the DG flux takes cell integrals of E_x (dx x averages) */
#define LPO_FIX_DEFAULT (LPO_FIX_F1 | LPO_FIX_F2 | LPO_FIX_F3 | LPO_FIX_F11 | LPO_FIX_F12)

typedef struct {
    int nx1, nx2, nv, n;
    double lv, lx, nu, dt, a_amp, k_wave;
    unsigned fixes;
    int linear_ei; /* 1: the two-species variant (FullandLinear) */
} lpo_params;

typedef struct lpo_ctx lpo_ctx;

int lpo_create(const lpo_params *p, lpo_ctx **out);
void lpo_destroy(lpo_ctx *c);
/* sc = {L_eta, h_eta, h_v, L_v, R_v, scale, scale3, scaleL, scalev, dv, dx, Lx, Lv, dy} */
void lpo_grids(const lpo_ctx *c, double *v, double *eta, double *wt, double *sc);
void lpo_cons(const lpo_ctx *c, double *c1, double *c2, double *cct);
double lpo_weight(const lpo_ctx *c, int xi, int om);
void lpo_omega_tables(const lpo_ctx *c, double *ah, double *sh, unsigned char *rz);
void lpo_fft3d(const lpo_ctx *c, const double *in, double *out);
void lpo_fs(const lpo_ctx *c, const double *in, double *out);
void lpo_compute_q(const lpo_ctx *c, const double *f, double *qhat);
void lpo_conserve(const lpo_ctx *c, double *qhat);
void lpo_intmodes(const lpo_ctx *c, int k1, int k2, int k3, int j1, int j2, int j3, double *out10);
/* RK4 of one spatial cell: f (n^3 node values), conserved qhat, the cell's
 * nv^3*7 state and its nv^3*5 output.  direct=1 sums IntModes over every
 * (mode, v-cell) pair from precomputed axis factors; direct=2 recomputes the
 * factors' sines and cosines on every call as the reference does (its cost);
 * direct=0 uses the separable form. */
void lpo_rk4(const lpo_ctx *c, const double *f, const double *qhat, const double *ucell,
             double *du, int direct);
void lpo_nodes(const lpo_ctx *c, const double *U, int cell, double *f);
/* kind 0: reference Landau-damping IC (T=0.9 Maxwellian), 1: unit Maxwellian,
 * 2: two-stream with drift u (param) */
void lpo_set_init(const lpo_ctx *c, double *U, int kind, double u);
void lpo_poisson(const lpo_ctx *c, const double *U, double *potc, double *phix, double *phiy,
                 double *fields14);
void lpo_rk3(const lpo_ctx *c, double *U);
/* Pieces of pois2d and RK3 for a slab of spatial cells: the charge moments
 * of cells [s0, s1) (3 per cell), the solve from given charges of every
 * cell, and one SSP-RK3 stage (0, 1, 2) with given field integrals. */
void lpo_charge(const lpo_ctx *c, const double *U, int s0, int s1, double *rt);
void lpo_poisson_rt(const lpo_ctx *c, const double *rt, double *potc, double *phix, double *phiy,
                    double *fields14);
void lpo_rk3_stage(const lpo_ctx *c, const double *U0, const double *Us, const double *fields14, int stage,
                   double *Uout);
/* Overrides the cell sizes (a slab context takes the whole grid's). */
void lpo_set_cell_size(lpo_ctx *c, double dx, double dy);
int lpo_collide(const lpo_ctx *c, double *U, int direct);
void lpo_step(const lpo_ctx *c, double *U, int direct);
void lpo_moments(const lpo_ctx *c, const double *U, const double *phix, const double *phiy,
                 double *out6);
void lpo_band(const lpo_ctx *c, int *dims, double *ab, int *ipiv);
double lpo_entropy(const lpo_ctx *c, const double *U);
/* two-species variant (FullandLinear) */
double lpo_weight_lin(const lpo_ctx *c, int xi, int om);
void lpo_compute_q_lin(const lpo_ctx *c, const double *f, double *qhat, double *qlin);
void lpo_conserve_lin(const lpo_ctx *c, double *q, double *qlin);
void lpo_cct_lin(const lpo_ctx *c, double *out4);
void lpo_rk4_lin(const lpo_ctx *c, const double *f, const double *qhat, const double *qlin, const double *U,
                 int cell, double *du, int direct);
void lpo_marginal_x1v1(const lpo_ctx *c, const double *U, double *out);

#ifdef __cplusplus
}
#endif
#endif
