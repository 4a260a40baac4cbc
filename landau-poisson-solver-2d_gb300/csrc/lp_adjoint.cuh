// Launchers of the adjoint kernels (lp_adjoint.cu): vector-Jacobian products
// of the FP64 collision step, advection step, Poisson solve and field energy.
#pragma once

#include "lp_kernels.cuh"

namespace lp {

// lam_F(a) = sum_xi lam_q(xi) P(xi, pair of a) conj(F(xi + n/2 - a)) (the
// transpose of the weighted contraction of ComputeQ linearised at F).
cudaError_t launch_qvjp(const double2 *F, const double2 *lq, const double *P, const int *pair_off, int n, int Bp,
                        double2 *lF, cudaStream_t st);
// The same VJP as correlations of lam_q with the conjugated a_p = C_p F and
// b_p = w_p F of the convolution form, by M = 3n/2-point DFTs along the
// three axes (lp_corr.cu): Cp the seven omega factors [7][n^3], Wf (M x n)
// and Wi (n x M, the 1/M and the output shift folded in) per-axis matrices,
// scratch of corr_scratch_elems(n) values; cells [0, B) of the Bp-strided
// arrays, in chunks of corr_cells().
int corr_cells();
size_t corr_scratch_elems(int n);
void corr_tables(const double *shat, const double *ahat, const double *cw, double h_eta, int n, std::vector<double> &Cp,
                 std::vector<double> &Wf, std::vector<double> &Wi);
cudaError_t launch_qvjp_corr(const double2 *F, const double2 *lq, const double *Cp, const double2 *Wf,
                             const double2 *Wi, int n, int Bp, int B, double2 *lF, double2 *scratch,
                             cudaStream_t st);
// Transpose of the DG projection: lam_tp [5][nv^3][Bp] -> lam_Qc [n^3][Bp]
// (lZ, lY scratch as the forward's Z, Y).
cudaError_t launch_project_vjp(const double *ltp, const double *tf, int n, int nv, int Bp, double2 *lZ, double2 *lY,
                               double2 *lQ, cudaStream_t st);
// Transpose of the collided coefficients' update and scatter for cells
// [c0, c0+B): lam_out (7 per record) -> lam_tp and the direct part of lam_in.
cudaError_t launch_collide_out_vjp(const double *lout, int nv, int c0, int B, int Bp, double dt, double kfac,
                                   double *ltp, double *lin, cudaStream_t st);
// lam_in += transpose of the node sampling (nfirst/ncount: the spectral
// nodes inside each DG velocity cell along one axis).
cudaError_t launch_nodes_vjp(const double *lf, int nv, int n, int c0, int B, int Bp, int slot1, const int *nfirst,
                             const int *ncount, const double *nodeoff, double *lin, cudaStream_t st);
cudaError_t launch_axpby(double *y, double a, const double *x, double b, long long n, cudaStream_t st);
cudaError_t launch_caxpby(double2 *y, double a, const double2 *x, double b, long long n, cudaStream_t st);
cudaError_t launch_add_re(double *y, double a, const double2 *x, double b, long long n, cudaStream_t st);
cudaError_t launch_dot_cell(const double *x, const double *y, long long npt, int Bp, int B, double scale, double *out,
                            cudaStream_t st);
cudaError_t launch_cdot_cell(const double2 *x, const double2 *y, long long npt, int Bp, int B, double scale,
                             double *out, cudaStream_t st);
cudaError_t launch_qsum(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, long long n,
                        double2 *out, cudaStream_t st);
// lamV += (dH/dV)^T lamH, lamF[3 per cell] += (dH/dE)^T lamH at V with fields.
cudaError_t launch_flux_vjp(const AdvectDev &ad, const double *V, const double *fields, const double *lamH,
                            double *lamV, double *lamF, cudaStream_t st);
cudaError_t launch_scale(double *y, const double *x, double c, long long n, cudaStream_t st);
// lam of the charge moments from the field adjoints (lamF, lphix, lphiy
// optional) with the dense inverse Ainv of the LDG matrix.
cudaError_t launch_poisson_vjp(const PoissonDev &pd, const double *lamF, const double *lphix, const double *lphiy,
                               const double *Ainv, double *lrt, cudaStream_t st);
cudaError_t launch_charge_vjp(const double *lrt, long long size, int nv3, double scalev, double *lamU,
                              cudaStream_t st);
cudaError_t launch_field_energy(const double *phix, const double *phiy, int nc, double dxdy, double *J,
                                double *lphix, double *lphiy, cudaStream_t st);

}  // namespace lp
