// Kernel launchers of the GB300 Landau-Poisson hot path (sm_103a).
//
// Spectral arrays are "cell-minor": element (point, cell) of an n^3 x Bp
// array sits at point*Bp + cell, Bp a multiple of 32, so the 32 lanes of a
// warp are 32 spatial cells and every load is coalesced.  The state U keeps
// the reference's AoS layout of 7 doubles per record.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace lp {

#ifdef __CUDACC__
// Every kernel of the library starts with this: under a programmatic
// dependency (the step graphs' kernel-to-kernel edges, which let a grid be
// launched while the previous one still runs) it returns once the grids this
// one depends on have completed and their writes are visible, so no kernel
// reads anything before its predecessors are done.  Under an ordinary launch
// it returns at once.
__device__ __forceinline__ void lp_grid_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif

template <typename R> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

// Pair table of the windowed weight contraction: for each xi, ceil(cnt/2)
// pairs (omega, u = xi + n/2 - omega) with the combined weight
// cw(omega) W(xi,omega) + cw(u) W(xi,u) (one term on the diagonal).
cudaError_t launch_pairs(const double *eta, const double *shat, const double *ahat,
                         const unsigned char *rzero, const double *cw, const int *pair_off, int n,
                         double *P64, float *P32, unsigned *PI, cudaStream_t st);

// Node values of cells [c0, c0+B) of U, written to f[n^3][Bp] (R precision).
template <typename R>
cudaError_t launch_nodes(const double *U, int nv, int n, int c0, int B, int Bp, int slot1,
                         const int *nodecell, const double *nodeoff, double dv, R *f,
                         cudaStream_t st);

// A per-axis transform factored as out[a] = post[a] sum_i w^((a i) mod n) pre[i] in[i]
// (FP32, passed by value to the kernels; n <= 32).  sign -1: w = exp(-2 pi i / n),
// the forward transform; +1: the inverse.  With one, the FP32 passes for n in
// {8, 16, 24, 32} run as register FFTs instead of the dense matrix M.
struct DftFac {
    float2 pre[32], post[32], w[32];
    int n = 0, sign = 0;
};

// Forward transform (fft3D with the phases folded into per-axis matrices):
// real f[n^3][Bp] -> complex F.  t1 is scratch of the same size as F.
template <typename R>
cudaError_t launch_fwd(const R *f, typename V2<R>::t *t1, typename V2<R>::t *F, const R *M, int n,
                       int Bp, cudaStream_t st, const DftFac *fac = nullptr);

// Per-cell collision frequency and time step of the cells of one pass
// (indexed by the cell's lane position 0..Bp-1); nullptr: the scalars.
struct Rates {
    const double *nu = nullptr;
    const double *dt = nullptr;
};

// Inverse transform FS of q (FP64 complex), real part only, fused with the
// RK4 stage update of the node values: stage 0 stores Q = Re FS(q) in qn and
// writes f1 = f + dt Q nu; stages 1, 2 write f1 = f + dt/2 Q nu + dt/2 Re FS(q) nu.
// cf/lamc (n in {8, 16, 24, 32}): q has not been projected by
// conserveAllMoments; q -= C^T lambda is applied in R precision on load (cf:
// the nonzero constraint rows C1[0], C2[1..3], C1[4] as FP32, lamc: [5][Bp]).
template <typename R>
cudaError_t launch_fs_stage(const double2 *q, typename V2<R>::t *t1, typename V2<R>::t *t2,
                            const R *M, int n, int Bp, int stage, double dt, double nu,
                            const R *f, R *qn, R *f1, cudaStream_t st, Rates rates = Rates{},
                            const float *cf = nullptr, const double *lamc = nullptr,
                            const DftFac *fac = nullptr);
// The same from an FP32 mode array (mixed path, n in {8, 16, 24, 32}).
cudaError_t launch_fs_stage32(const float2 *q, float2 *t1, float2 *t2, const float *M, int n, int Bp, int stage,
                              double dt, double nu, const float *f, float *qn, float *f1, cudaStream_t st,
                              Rates rates, const float *cf, const double *lamc, const DftFac *fac = nullptr);
// One FP32 RK4 stage from its mode array to the next transformed node values
// F: the inverse transform, the node-value stage and the forward transform,
// with the last inverse and first forward passes (both along the slowest
// axis) fused so that the stage's node values stay on chip; without the
// per-axis factors (fi, ff) the two transforms run in turn through f1.
cudaError_t launch_fs_fwd32(const float2 *q, float2 *t1, float2 *t2, float2 *F, const float *Mi, const float *M,
                            int n, int Bp, int stage, double dt, double nu, const float *f, float *qn, float *f1,
                            cudaStream_t st, Rates rates, const float *cf, const double *lamc,
                            const DftFac *fi = nullptr, const DftFac *ff = nullptr);

// Inverse transform FS of q, full complex output (for the reference-shaped FS).
template <typename R>
cudaError_t launch_fs_full(const double2 *q, typename V2<R>::t *t1, typename V2<R>::t *t2,
                           typename V2<R>::t *out, const R *M, int n, int Bp, cudaStream_t st);

// Forward transform of complex input (for the reference-shaped fft3D).
template <typename R>
cudaError_t launch_fwd_complex(const typename V2<R>::t *in, typename V2<R>::t *t1,
                               typename V2<R>::t *F, const R *M, int n, int Bp, cudaStream_t st);

// q(xi) = sum_pairs P F(omega) F(u) for every xi and cell.
template <typename R>
cudaError_t launch_computeq(const typename V2<R>::t *F, const R *P, const unsigned *PI,
                            const int *pair_off, int n3, int Bp, double2 *q, cudaStream_t st);

// Two-species variant: the linear weight table (per xi, every window entry),
// its contraction ql(xi) = sum Wl F(xi + n/2 - omega), and q += ql.
cudaError_t launch_lin_weights(const double *eta, const double *shat, const double *cw, const long long *win_off, int n,
                               double scale3, double *W64, float *W32, cudaStream_t st);
template <typename R>
cudaError_t launch_qlin(const typename V2<R>::t *F, const R *Wl, const long long *win_off, int n, int Bp, double2 *ql,
                        cudaStream_t st);
cudaError_t launch_qadd(double2 *q, const double2 *ql, long long total, cudaStream_t st);

// Line-tiled FP32 contraction (mixed path, n in {8, 16, 24, 32}): one warp
// per (output line (i, j), k-tile, 32 cells); the symmetric plane pairs
// {(l, m), (i+n/2-l, j+n/2-m)} of the window keep both F lines in registers
// and every term A(k') B(k+n/2-k') takes one combined weight.  Per-plane
// partial sums are added to a Kahan-compensated FP32 accumulator.
bool lines_supported(int n);
long long lines_table_floats(int n, std::vector<long long> &line_off);
cudaError_t launch_lines_table(const double *eta, const double *shat, const double *ahat,
                               const unsigned char *rzero, const double *cw, const long long *line_off,
                               int n, float *W, cudaStream_t st);
// warps (2 or 4): warps of a block splitting the plane pairs of one line.
// Odd k-tiles go to st_odd (nullptr: st); the caller orders st_odd after
// the tile inputs and joins it back (the tiles write disjoint outputs).
cudaError_t launch_computeq_lines(const float2 *F, const float *W, const long long *line_off, int n,
                                  int Bp, double2 *q, cudaStream_t st, int warps = 2,
                                  cudaStream_t st_odd = nullptr);

// Mixed path, convolution form of the same contraction (lp_fftq.cu): the
// weight splits into seven omega-factors C[7][n^3] times polynomials in u,
// so q is a sum of seven windowed convolutions, evaluated with M = 3n/2
// point DFTs along axes 2 and 3 and summed directly along axis 1.
template <typename C> struct FftTwT {
    C fw[48];  // exp(-2 pi i q2 k1 / M) at q2 * 6 + k1
    C fa[48];  // fw exp(2 pi i k1 / 3): the a-side, output shift n/2
    C iv[48];  // conj(fw) / M
};
using FftTw = FftTwT<float2>;
using FftTw64 = FftTwT<double2>;
bool fftq_supported(int n);
FftTw fftq_twiddles(int n);
FftTw64 fftq_twiddles64(int n);
void fftq_coefficients(const double *shat, const double *ahat, const double *cw, double h_eta, int n,
                       std::vector<float> &C);
void fftq_coefficients64(const double *shat, const double *ahat, const double *cw, double h_eta, int n,
                         std::vector<double> &C);
size_t fftq_gh_elems(int n, int Bs);       // axis-1 sums and inverse axis-2 outputs
size_t fftq_scratch_elems(int n, int Bs);  // float2 elements for Bs cells
// Cells [c0, c0 + Bc) of F and q (stride Bp); Bc and c0 multiples of 32,
// Bc <= Bs, the cells of the scratch.  form 1 (fused, lp_fqf.cu): the axis-3
// DFTs into X1, then the axis-2 DFTs, axis-1 sums and inverse axis-2 DFTs
// in one kernel that keeps the axis-2 spectra on chip, then Z2; form 0
// (three-pass): X1/X2, Y and Z1 as separate kernels through DRAM, then Z2.
// stage -1 runs every kernel; 0, 2, 3, 4 only one of them (form 1: X1, the
// fused kernel, nothing, Z2; form 0: X1/X2, Y, Z1, Z2; 1 launches nothing),
// on the scratch a full run left.  q32: the mode array is written as FP32
// complex there instead of q.  err: set by the fused kernel when one of its
// bounded waits runs out.
// conserveAllMoments' sums formed by the convolution form's last kernel as it
// writes an FP32 mode array: each thread sums its outputs times the
// constraint rows (cf, FP32 [5][n^3]) in FP32, each block adds its threads'
// sums in FP64 into part[block][5][Bp] (the layout of the chunk partials of
// launch_conserve, with fftq_cons_blocks(n) chunks).
struct ConsFused {
    const float *cf = nullptr;
    double *part = nullptr;
};
// Blocks of the last kernel per group of 32 cells (the chunks of part).
int fftq_cons_blocks(int n);

cudaError_t launch_computeq_fft(const float2 *F, const float *C, const FftTw &tw, int n, int Bp, int c0, int Bc,
                                float2 *scratch, int Bs, double2 *q, cudaStream_t st, int stage = -1,
                                float2 *q32 = nullptr, const ConsFused *cons = nullptr, int form = 0,
                                int *err = nullptr);
// FP64 path, the same contraction in FP64 (the three-pass kernels at
// double precision): F and q FP64 complex, C the seven omega-factors in FP64,
// scratch of fftq_scratch_elems64(n, Bs) double2 elements.  Where the node
// grid is uniform (eta[n/2] exactly 0) its sums agree with the direct
// weighted sum of the pair form to 1e-14 (relative L2).
size_t fftq_scratch_elems64(int n, int Bs);
cudaError_t launch_computeq_fft64(const double2 *F, const double *C, const FftTw64 &tw, int n, int Bp, int c0,
                                  int Bc, double2 *scratch, int Bs, double2 *q, cudaStream_t st);
// The fused form's stages 0 and 2 (lp_fqf.cu) on X1 and H of the scratch,
// and the X1 elements it needs for Bs cells.
cudaError_t launch_fq_fused(int n, const float2 *F, const float *C, const FftTw &tw, int Bp, int c0, int Bc,
                            float2 *X1, float2 *H, int Bs, cudaStream_t st, int stage, int *err);
size_t fq_fused_x1_elems(int n, int Bs);

// Moment-conserving projection of q in place (FP64).
// apply = false: only the multipliers lam[5][Bp] (the correction is left to
// the consumers of q).
cudaError_t launch_conserve(double2 *q, const double *c1, const double *c2, const double *cct_inv,
                            int n3, int Bp, double *part, int nchunk, double *lam,
                            cudaStream_t st, bool apply = true);
// The multipliers lam[5][Bp] from chunk partials part[nchunk][5][Bp].
cudaError_t launch_cons_lambda(const double *part, int nchunk, const double *cct_inv, int Bp, double *lam,
                               cudaStream_t st);

// Final RK4 combination, DG projection and mass-matrix inverse: writes
// dU[B][nv^3][5] for cells [c0, c0+B).  Qc, Y, Z are scratch.
template <typename R>
cudaError_t launch_project(const double2 *q0, const double2 *q1, const double2 *q2,
                           const double2 *q3, double nu, const R *tfac, int n, int nv, int Bp,
                           int B, int c0, const double *U, int ustride, const int *uslot,
                           double dt, double scalev, double scaleL, double scale3,
                           typename V2<R>::t *Qc, typename V2<R>::t *Y, typename V2<R>::t *Z,
                           double *dU, cudaStream_t st, Rates rates = Rates{});

// Mixed path: reconcile the 5 DG moments of each cell's increment with their
// FP64 values from the mode array (minimal-norm 5x5 Lagrange correction), in
// two parts: the FP64 target moments from q0..q3 (independent of the DG
// projection, so they can run beside it) and, once dU exists, its actual
// moments, the multipliers and (apply) the correction of dU.  tpart nullptr
// in launch_moment_finish: the target moments are zero.
cudaError_t launch_moment_target(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3,
                                 double nu, const double *gmom, int n3, int Bp, int nchunk, double *tpart,
                                 cudaStream_t st, Rates rates = Rates{});
cudaError_t launch_moment_finish(const double *tpart, int nchunk, const double *U, int nv, double dv, double lv,
                                 int c0, int B, int Bp, int nrc, double *apart, const double *gm_inv, double scale,
                                 double kfac, double *lam, double *dU, cudaStream_t st, Rates rates = Rates{},
                                 bool apply = true);

// Mixed path with LP_FIX_F1 fixed: DG projection of the RK4 combination
// into the coefficient increments Inc[kt][5][Bp] (no state read) with
// per-block partial sums of their DG moments, part[blocks][5][Bp]; the
// multipliers from those partials (tpart as in launch_moment_finish); and
// U slots {0,3,4,5,6} += increment + moment correction.
int project_inc_blocks(int n, int nv);
// cf/lam4 (n in {8, 16, 24, 32}): the q_s were not projected; their
// corrections with lam4[s][5][Bp] are applied in FP32 on load.  q32: the
// four mode arrays are FP32 complex (q0..q3 unused).  tc_tab (the table of
// pj3_tc_table on the device) runs the axis-3 pass on the tensor cores where
// pj3_tc_supported, tc_tab1 (pj1_tc_table) the axis-1 pass where
// pj1_tc_supported, with tc_err their device error flag.
cudaError_t launch_project_inc(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, double nu,
                               const float *tfac, int n, int nv, int Bp, int B, double dt, double scalev,
                               double scaleL, double scale3, float2 *Qc, float2 *Y, float2 *Z, float *Inc,
                               double *part, double lv, double dv, cudaStream_t st, Rates rates = Rates{},
                               const float *cf = nullptr, const double *lam4 = nullptr,
                               float2 *const *q32 = nullptr, const float *tc_tab = nullptr,
                               int *tc_err = nullptr, const float *tc_tab1 = nullptr);
cudaError_t launch_lambda_inc(const double *tpart, int nchunk, const double *part, int n, int nv, int B, int Bp,
                              const double *gm_inv, double scale, double kfac, double *lam, cudaStream_t st,
                              Rates rates = Rates{});
cudaError_t launch_scatter_inc(const float *Inc, int Bp, int B, int nv, int c0, double *U, const double *lam,
                               double dv, double lv, cudaStream_t st);

// U slots {0,3,4,5,6} of cells [c0, c0+B) <- dU; with lam (the mixed path's
// moment multipliers of launch_moment_fix with apply = false) the correction
// is added on the way.
cudaError_t launch_scatter(const double *dU, int nv3, int c0, int B, double *U, cudaStream_t st,
                           const double *lam = nullptr, int nv = 0, double dv = 0., double lv = 0.);

// ---- advection and Poisson ----
// Charge moments of every spatial cell summed in the reference's record order
// (scalev included): rt[3*ncell].
cudaError_t launch_charge(const double *U, int ncell, int nv3, double scalev, double *rt,
                          cudaStream_t st);
// FP32 copy of the state (size records of 7) and, when part != nullptr, the
// charge partial sums of every block of 128 records: part[3 * size/128].
cudaError_t launch_state_f32(const double *U, long long size, float *Uf, double *part, cudaStream_t st);

struct PoissonDev {
    int nx, ny, ndim, kl, ku, ldab;
    const double *ab;
    const int *ipiv;
    double dxp, dyp;
    const unsigned char *gate;  // per x1 cell, 1-based
    double blk[6][9];           // acvx, acyrr, acyrl, acvy, acxrr, acxrl
    // fast variant (mixed path): reciprocals of the band diagonal (nullptr:
    // the host's operations, divisions included), of dxp and dyp, and the
    // factor applied to the summed charge partials
    const double *rdiag;
    double rdxp, rdyp, cscale;
    int staged;  // set by the launcher: band factors copied to shared memory
};
// rt: 3 charge sums per cell (npart = 1) or npart block partials per cell.
cudaError_t launch_poisson(const PoissonDev &pd, const double *rt, int npart, double *b, double *potc,
                           double *phix, double *phiy, double *fields, cudaStream_t st);

struct AdvectDev {
    int nx1, nx2, nv;
    long long size;
    double lv, dv, dx, scalev, dt;
    double rdv, inv;  // 1/dv and 1/dx/scalev
    float dt_f;       // dt in FP32 (mixed-path stage copies)
    double dt6;       // dt/6 (mixed-path final stage)
    double fscale;    // factor of the field integrals in the flux: dx with
                      // LP_FIX_F12 (cell integrals), else 1 (the reference's averages)
    struct {
        float lv, dv, rdv, scalev, inv, fscale;
    } f;              // FP32 copies for the FP32 flux
};
// One SSP-RK3 stage: Uout = combination(U0, Us, H).  H is evaluated in FP64
// from Us when Uin_f32 is nullptr, else in FP32 from the FP32 stage values
// Uin_f32.  Uout_f32 (optional) receives an FP32 copy of Uout and part
// (optional) the charge partial sums of Uout per block of 128 records.
cudaError_t launch_flux_stage(const AdvectDev &ad, const double *U0, const double *Us, const float *Uin_f32,
                              const double *fields, int stage, double *Uout, float *Uout_f32, double *part,
                              cudaStream_t st);

// ---- axis-3 DG projection pass on the tensor cores (lp_pjtc.cu) ----
// Columns of the shared GEMM operand (6 nv rounded up to a multiple of 16).
int pj3_tc_np(int nv);
// n in {8, 16, 24, 32}, 6 nv <= 256, Bp a multiple of 32.
bool pj3_tc_supported(int n, int nv, int Bp);
size_t pj3_tc_table_floats(int n, int nv);
size_t pj3_tc_smem(int n, int nv);
// The shared operand from the per-axis factors tfac ([3][n][nv] complex FP32):
// TF32 head then tail, in the MMA's shared-memory layout.
void pj3_tc_table(const float *tfac, int n, int nv, std::vector<float> &out);
// k_pj3 on the tensor cores: the same inputs and output Y; err (device) is
// set to 1 or 2 when a bounded wait for the shared operand or the MMAs ran out.
template <typename QT>
cudaError_t launch_pj3_tc(const QT *q0, const QT *q1, const QT *q2, const QT *q3, double nu, const double *cnu,
                          const float *btab, int n, int nv, int Bp, float2 *Y, const float *cf, const double *lam4,
                          int *err, cudaStream_t st);

// The axis-2 pass (k_pj2) on the tensor cores with the axis-3 pass's table:
// n in {8, 16, 24, 32}, nv in {8, 16, 24}, Bp a multiple of 32.
bool pj2_tc_supported(int n, int nv, int Bp);
size_t pj2_tc_smem(int n, int nv);
cudaError_t launch_pj2_tc(const float2 *Y, const float *btab, int n, int nv, int Bp, float2 *Z, int *err,
                          cudaStream_t st);
// The axis-1 pass (k_pj1's increments and moment partials) on the tensor
// cores: n in {8, 16, 24, 32}, even nv <= 32, Bp a multiple of 32.
int pj1_tc_nvp(int nv);
bool pj1_tc_supported(int n, int nv, int Bp);
size_t pj1_tc_table_floats(int n, int nv);
size_t pj1_tc_smem(int n, int nv);
void pj1_tc_table(const float *tfac, int n, int nv, std::vector<float> &out);
cudaError_t launch_pj1_tc(const float2 *Z, const float *btab, int n, int nv, int Bp, int B, double dt, double kfac,
                          const double *cdt, double dv, double lv, float *Inc, double *part, int *err,
                          cudaStream_t st);

// ---- mixed-path advection (increment form of SSP-RK3, FP32 fluxes) ----
// FP32 copy of the state and FP64 charge partials of every group of 128
// records (part[3 * size/128]).
cudaError_t launch_state_f32_grp(const double *U, long long size, float *Uf, double *part, cudaStream_t st);
// Stage s in {0, 1, 2}: H from Uin (FP32 copy of U_s); stages 0, 1 update the
// FP32 running sum S, write the FP32 copy of U_{s+1} and the FP32 charge
// partials of S (ipart); stage 2 adds dt/6 (S + 4 H2) to the FP64 state U.
cudaError_t launch_flux_inc(const AdvectDev &ad, int stage, const float *Uin, const float *Uf0,
                            const double *fields, float *S, float *Uoutf, double *U, float *ipart,
                            cudaStream_t st);
// Poisson solve from charge partials base + iscale * inc (npart groups per
// cell; inc may be nullptr) with the dense inverse Ainv (ndim x ndim,
// row-major): potential into potc, fields as launch_poisson.  b is scratch.
cudaError_t launch_poisson_dense(const PoissonDev &pd, const double *base, const float *inc, double iscale,
                                 int npart, const double *Ainv, double *b, double *potc, double *phix,
                                 double *phiy, double *fields, cudaStream_t st);

// ---- diagnostics ----
// Block partial sums of int f log f over records [0, kend) (5-point Gauss
// rule; multiply the sum by (dv/2)^3 dx/2).
cudaError_t launch_entropy(const double *U, long long kend, double *part, int nblk, cudaStream_t st);
// The reference's (x1, v1) marginal at 4 x 4 points per cell pair:
// out[nx1*4][nv*4].
cudaError_t launch_marginal_x1v1(const double *U, int nx1, int nx2, int nv, double dx, double dv, double lv,
                                 double *out, cudaStream_t st);

// FMA-throughput microbenchmarks (FP32 packed f32x2 and FP64).
cudaError_t launch_fma_peak(bool fp64, int blocks, int iters, double *sink, cudaStream_t st);

// Block partial sums of the moments (mass, p1, p2, p3, kinetic energy).
cudaError_t launch_moments(const double *U, long long size, long long kend, int nv, double lv,
                           double dv, double *part, int nblk, cudaStream_t st);

}  // namespace lp
