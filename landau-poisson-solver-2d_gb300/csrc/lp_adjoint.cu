// Adjoint (vector-Jacobian products) of the FP64 hot path: one collision
// step, one SSP-RK3 advection step with its three LDG Poisson solves, and the
// field energy.  Conventions: a real array's adjoint is the gradient; for a
// complex array z the adjoint lam holds dL/dRe z + i dL/dIm z, so for a
// complex-linear map z -> A z the adjoint map is lam -> A^H lam, and for
// z -> Re(A z) with real output it is lam -> A^H lam as well.  Spectral
// arrays are cell-minor (point * Bp + cell) like the forward kernels.
#include "lp_adjoint.cuh"

namespace lp {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// ---------------------------------------------------------------- ComputeQ VJP
// q(xi) = sum_pairs P(xi, {w, u}) F(w) F(u), u = xi + n/2 - w, so
// lam_F(a) = sum_xi lam_q(xi) P(xi, pair of a) conj(F(xi + n/2 - a)), twice
// for the self-paired middle of a window.  One thread per (a, cell), the
// xi loop over the box where xi + n/2 - a lies in the grid (a correlation).
__global__ void k_qvjp(const double2 *__restrict__ F, const double2 *__restrict__ lq, const double *__restrict__ P,
                       const int *__restrict__ pair_off, int n, int Bp, double2 *__restrict__ lF) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int n3 = n * n * n, h = n / 2;
    if (tid >= (long long)n3 * Bp) return;
    const int c = (int)(tid % Bp), a = (int)(tid / Bp);
    const int a0 = a / (n * n), a1 = (a / n) % n, a2 = a % n;
    const int lo0 = max(0, a0 - h), hi0 = min(n - 1, a0 - h + n - 1);
    const int lo1 = max(0, a1 - h), hi1 = min(n - 1, a1 - h + n - 1);
    const int lo2 = max(0, a2 - h), hi2 = min(n - 1, a2 - h + n - 1);
    double sr = 0., si = 0.;
    for (int i = lo0; i <= hi0; ++i) {
        const int si0 = i < h ? 0 : i - h + 1, ni = i < h ? i + h + 1 : 3 * h - 1 - i;
        for (int j = lo1; j <= hi1; ++j) {
            const int sj = j < h ? 0 : j - h + 1, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
            for (int k = lo2; k <= hi2; ++k) {
                const int sk = k < h ? 0 : k - h + 1, nk = k < h ? k + h + 1 : 3 * h - 1 - k;
                const int xi = (i * n + j) * n + k, cnt = ni * nj * nk;
                const int L = ((a0 - si0) * nj + (a1 - sj)) * nk + (a2 - sk), Lu = cnt - 1 - L;
                const int off = pair_off[xi], npair = pair_off[xi + 1] - off;
                double w = P[off + (L < npair ? L : Lu)];
                if (L == Lu) w *= 2.;
                const int u = ((i + h - a0) * n + (j + h - a1)) * n + (k + h - a2);
                const double2 t = cmulc(lq[(long long)xi * Bp + c], F[(long long)u * Bp + c]);
                sr += w * t.x;
                si += w * t.y;
            }
        }
    }
    lF[tid] = make_double2(sr, si);
}

// ---------------------------------------------------------------- DG projection transposes
// Forward: Y_a = T_a(axis 3) Qc; Z_p = T(axis 2) Y; tp = Re T(axis 1) Z with
// (axis-1, axis-2, axis-3) factors tp0 (0,0,0), tp2 (1,0,0), tp3 (0,1,0),
// tp4 (0,0,1), tp5 (2,0,0) + (0,2,0) + (0,0,2).  lam_tp: [5][nv^3][Bp] for
// (tp0, tp2, tp3, tp4, tp5).
__global__ void k_projT1(const double *__restrict__ ltp, const double *__restrict__ tf, int n, int nv, int Bp,
                         double2 *__restrict__ lZ) {
    lp_grid_wait();
    // lZ[p][k1][j2][j3]: p0 = T0 tp0 + T1 tp2 + T2 tp5, p1 = T0 tp3, p2 = T0 tp5, p3 = T0 tp4, p4 = T0 tp5
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nv2 = (long long)nv * nv, nv3 = nv2 * nv;
    if (tid >= (long long)n * nv2 * Bp) return;
    const int c = (int)(tid % Bp);
    long long r = tid / Bp;
    const int j23 = (int)(r % nv2), k1 = (int)(r / nv2);
    double2 z[5] = {};
    for (int j1 = 0; j1 < nv; ++j1) {
        const long long rec = j1 * nv2 + j23;
        const double l0 = ltp[(0 * nv3 + rec) * Bp + c], l2 = ltp[(1 * nv3 + rec) * Bp + c];
        const double l3 = ltp[(2 * nv3 + rec) * Bp + c], l4 = ltp[(3 * nv3 + rec) * Bp + c];
        const double l5 = ltp[(4 * nv3 + rec) * Bp + c];
        const double *t0 = tf + 2 * ((0 * n + k1) * nv + j1), *t1 = tf + 2 * ((1 * n + k1) * nv + j1);
        const double *t2 = tf + 2 * ((2 * n + k1) * nv + j1);
        // conj(t) * lam for a real lam
        z[0].x += t0[0] * l0 + t1[0] * l2 + t2[0] * l5;
        z[0].y -= t0[1] * l0 + t1[1] * l2 + t2[1] * l5;
        z[1].x += t0[0] * l3; z[1].y -= t0[1] * l3;
        z[2].x += t0[0] * l5; z[2].y -= t0[1] * l5;
        z[3].x += t0[0] * l4; z[3].y -= t0[1] * l4;
        z[4].x += t0[0] * l5; z[4].y -= t0[1] * l5;
    }
    for (int p = 0; p < 5; ++p) lZ[(((long long)p * n + k1) * nv2 + j23) * Bp + c] = z[p];
}

__global__ void k_projT2(const double2 *__restrict__ lZ, const double *__restrict__ tf, int n, int nv, int Bp,
                         double2 *__restrict__ lY) {
    lp_grid_wait();
    // lY[a][k1][k2][j3]: a0 = T0 Z0 + T1 Z1 + T2 Z2, a1 = T0 Z3, a2 = T0 Z4 (conjugated factors)
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)n * n * nv * Bp) return;
    const int c = (int)(tid % Bp);
    long long r = tid / Bp;
    const int j3 = (int)(r % nv);
    r /= nv;
    const int k2 = (int)(r % n), k1 = (int)(r / n);
    double2 y[3] = {};
    for (int j2 = 0; j2 < nv; ++j2) {
        double2 zz[5];
        for (int p = 0; p < 5; ++p) zz[p] = lZ[((((long long)p * n + k1) * nv + j2) * nv + j3) * Bp + c];
        const double2 t0 = make_double2(tf[2 * ((0 * n + k2) * nv + j2)], tf[2 * ((0 * n + k2) * nv + j2) + 1]);
        const double2 t1 = make_double2(tf[2 * ((1 * n + k2) * nv + j2)], tf[2 * ((1 * n + k2) * nv + j2) + 1]);
        const double2 t2 = make_double2(tf[2 * ((2 * n + k2) * nv + j2)], tf[2 * ((2 * n + k2) * nv + j2) + 1]);
        double2 v;
        v = cmulc(zz[0], t0); y[0].x += v.x; y[0].y += v.y;
        v = cmulc(zz[1], t1); y[0].x += v.x; y[0].y += v.y;
        v = cmulc(zz[2], t2); y[0].x += v.x; y[0].y += v.y;
        v = cmulc(zz[3], t0); y[1].x += v.x; y[1].y += v.y;
        v = cmulc(zz[4], t0); y[2].x += v.x; y[2].y += v.y;
    }
    for (int a = 0; a < 3; ++a) lY[((((long long)a * n + k1) * n + k2) * nv + j3) * Bp + c] = y[a];
}

__global__ void k_projT3(const double2 *__restrict__ lY, const double *__restrict__ tf, int n, int nv, int Bp,
                         double2 *__restrict__ lQ) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)n * n * n * Bp) return;
    const int c = (int)(tid % Bp);
    long long r = tid / Bp;
    const int k3 = (int)(r % n);
    r /= n;
    const int k2 = (int)(r % n), k1 = (int)(r / n);
    double2 s = make_double2(0., 0.);
    for (int j3 = 0; j3 < nv; ++j3)
        for (int a = 0; a < 3; ++a) {
            const double2 t = make_double2(tf[2 * ((a * n + k3) * nv + j3)], tf[2 * ((a * n + k3) * nv + j3) + 1]);
            const double2 v = cmulc(lY[((((long long)a * n + k1) * n + k2) * nv + j3) * Bp + c], t);
            s.x += v.x; s.y += v.y;
        }
    lQ[tid] = s;
}

// ---------------------------------------------------------------- collision output / nodes
// dU of k_proj1 and the scatter into slots {0,3,4,5,6} (F1 fixed): lam_out
// (7 per record) -> lam_tp (5 per v-cell, cell-minor) and the direct part of
// lam_in (slots 1, 2 pass through).
__global__ void k_collide_out_vjp(const double *__restrict__ lout, int nv, int c0, int B, int Bp, double dt,
                                  double kfac, double *__restrict__ ltp, double *__restrict__ lin) {
    lp_grid_wait();
    const long long nv3 = (long long)nv * nv * nv;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= nv3 * Bp) return;
    const int c = (int)(tid % Bp);
    const long long kt = tid / Bp;
    double *lt = ltp + kt * Bp + c;
    if (c >= B) {
        for (int e = 0; e < 5; ++e) lt[e * nv3 * Bp] = 0.;
        return;
    }
    const long long rec = (long long)(c0 + c) * nv3 + kt;
    const double *lo = lout + 7 * rec;
    double *li = lin + 7 * rec;
    // d0 = 19 p0/4 - 15 p5, d4 = 60 p5 - 15 p0, d1..d3 = p2..p4
    const double lp0 = 19. / 4. * lo[0] - 15. * lo[6], lp5 = -15. * lo[0] + 60. * lo[6];
    const double lp2 = lo[3], lp3 = lo[4], lp4 = lo[5];
    // p0 = u0 + u6/4 + dt tp0 kfac, p5 = u0/4 + u6 19/240 + dt tp5 kfac, p2.. = u3.. + 12 dt tp kfac
    li[0] = lp0 + 0.25 * lp5;
    li[6] = 0.25 * lp0 + 19. / 240. * lp5;
    li[3] = lp2; li[4] = lp3; li[5] = lp4;
    li[1] = lo[1]; li[2] = lo[2];
    const double s = dt * kfac;
    lt[0] = s * lp0;
    lt[1 * nv3 * Bp] = 12. * s * lp2;
    lt[2 * nv3 * Bp] = 12. * s * lp3;
    lt[3 * nv3 * Bp] = 12. * s * lp4;
    lt[4 * nv3 * Bp] = s * lp5;
}

// Transpose of setInit_spectral (k_nodes_t): every DG record gathers the
// adjoints of the spectral nodes inside its velocity cell.
__global__ void k_nodes_vjp(const double *__restrict__ lf, int nv, int n, int c0, int B, int Bp, int slot1,
                            const int *__restrict__ nfirst, const int *__restrict__ ncount,
                            const double *__restrict__ nodeoff, double *__restrict__ lin) {
    lp_grid_wait();
    const long long nv3 = (long long)nv * nv * nv;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= nv3 * B) return;
    const int c = (int)(tid % B);
    const long long kt = tid / B;
    const int j3 = (int)(kt % nv), j2 = (int)((kt / nv) % nv), j1 = (int)(kt / ((long long)nv * nv));
    double s0 = 0., s1 = 0., s4 = 0., s5 = 0., s6 = 0.;
    for (int l = nfirst[j1]; l < nfirst[j1] + ncount[j1]; ++l)
        for (int m = nfirst[j2]; m < nfirst[j2] + ncount[j2]; ++m)
            for (int q = nfirst[j3]; q < nfirst[j3] + ncount[j3]; ++q) {
                const double g = lf[(((long long)l * n + m) * n + q) * Bp + c];
                const double a = nodeoff[l], b = nodeoff[m], e = nodeoff[q];
                s0 += g; s1 += g * a; s4 += g * b; s5 += g * e; s6 += g * (a * a + b * b + e * e);
            }
    double *li = lin + 7 * ((long long)(c0 + c) * nv3 + kt);
    li[0] += s0; li[slot1] += s1; li[4] += s4; li[5] += s5; li[6] += s6;
}

// ---------------------------------------------------------------- elementwise helpers (cell-minor)
// y = a*y + b*x for real arrays (a == 0: y is not read)
__global__ void k_axpby(double *__restrict__ y, double a, const double *__restrict__ x, double b, long long n) {
    lp_grid_wait();
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a == 0. ? b * x[i] : a * y[i] + b * x[i];
}
// y = a*y + b*x for complex arrays (a == 0: y is not read)
__global__ void k_caxpby(double2 *__restrict__ y, double a, const double2 *__restrict__ x, double b, long long n) {
    lp_grid_wait();
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 v = x[i];
    if (a == 0.) y[i] = make_double2(b * v.x, b * v.y);
    else y[i] = make_double2(a * y[i].x + b * v.x, a * y[i].y + b * v.y);
}
// y (real) = a*y + b*Re x (a == 0: y is not read)
__global__ void k_add_re(double *__restrict__ y, double a, const double2 *__restrict__ x, double b, long long n) {
    lp_grid_wait();
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a == 0. ? b * x[i].x : a * y[i] + b * x[i].x;
}
// out[c] += scale * sum_pt x[pt][c] y[pt][c] (real) over cells c < B; one warp per cell
__global__ void k_dot_cell(const double *__restrict__ x, const double *__restrict__ y, long long npt, int Bp, int B,
                           double scale, double *__restrict__ out) {
    lp_grid_wait();
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= B) return;
    double s = 0.;
    for (long long p = lane; p < npt; p += 32) s += x[p * Bp + c] * y[p * Bp + c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (lane == 0) out[c] += scale * s;
}
// out[c] += scale * Re sum_pt conj(x) y (complex)
__global__ void k_cdot_cell(const double2 *__restrict__ x, const double2 *__restrict__ y, long long npt, int Bp,
                            int B, double scale, double *__restrict__ out) {
    lp_grid_wait();
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= B) return;
    double s = 0.;
    for (long long p = lane; p < npt; p += 32) {
        const double2 a = x[p * Bp + c], b = y[p * Bp + c];
        s += a.x * b.x + a.y * b.y;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (lane == 0) out[c] += scale * s;
}
// Qc / nu = q0/2 + (q1 + q2 + q3)/6
__global__ void k_qsum(const double2 *__restrict__ q0, const double2 *__restrict__ q1, const double2 *__restrict__ q2,
                       const double2 *__restrict__ q3, long long n, double2 *__restrict__ out) {
    lp_grid_wait();
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 a = q0[i], b = q1[i], d = q2[i], e = q3[i];
    out[i] = make_double2(0.5 * a.x + (b.x + d.x + e.x) / 6., 0.5 * a.y + (b.y + d.y + e.y) / 6.);
}

// ---------------------------------------------------------------- advection VJP
// Transpose of one flux evaluation H(V, E) (flux_rhs in FP64; A:184-405) at
// record k: given lam_H (the adjoint of H[k]), adds (dH_k/dV)^T lam_H into
// lam_V (own, x1 and v1 neighbours; FP64 atomics) and (dH_k/dE)^T lam_H into
// the per-cell field adjoints lam_f = (ie, ixe, ixxe) per cell.
__global__ void k_flux_vjp(AdvectDev ad, const double *__restrict__ V, const double *__restrict__ fields,
                           const double *__restrict__ lamH, double *__restrict__ lamV, double *__restrict__ lamF) {
    lp_grid_wait();
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= ad.size) return;
    const int nv = ad.nv;
    const long long sv = (long long)nv * nv * nv;
    const long long jm = k % sv, s = k / sv;
    const int j3 = (int)(jm % nv), j2 = (int)((jm / nv) % nv), j1 = (int)(jm / ((long long)nv * nv));
    const int i2 = (int)(s % ad.nx2), i1 = (int)(s / ad.nx2);
    const double dv = ad.dv, dv2 = dv * dv, dv3 = dv2 * dv, dv4 = dv3 * dv;
    const double G = -ad.lv + (j1 + 0.5) * ad.dv;
    const double *lh = lamH + 7 * k;
    const double inv = ad.inv;
    // lam of tp0..tp5 (tp2 = l3, tp3 = l4, tp4 = l5, tp5 = l6)
    const double m0 = inv * (19. / 4. * lh[0] - 15. * lh[6]), m5 = inv * (-15. * lh[0] + 60. * lh[6]);
    const double m1 = 12. * inv * lh[1], m2 = 12. * inv * lh[3], m3 = 12. * inv * lh[4], m4 = 12. * inv * lh[5];
    const double *u = V + 7 * k;
    // x1 direction (I3)
    long long kR3, kL3;
    double s3;
    if (j1 < nv / 2) {
        int iir = i1 + 1;
        if (iir == ad.nx1) iir = 0;
        kR3 = (long long)iir * ad.nx2 * sv + (long long)i2 * sv + jm; kL3 = k; s3 = -1.;
    } else {
        int iil = i1 - 1;
        if (iil == -1) iil = ad.nx1 - 1;
        kL3 = (long long)iil * ad.nx2 * sv + (long long)i2 * sv + jm; kR3 = k; s3 = 1.;
    }
    const double gAd = -(m0 * dv3 * G + m2 * dv4 / 12. + m5 * dv3 * G / 4.), gAs = -0.5 * m1 * dv3 * G;
    const double g3d = -(m0 * dv4 / 12. + m2 * dv3 * G / 12. + m5 * dv4 * 19. / 720.), g3s = -0.5 * m1 * dv4 / 12.;
    const double g6d = -(m0 * dv3 * G / 4. + m2 * dv4 * 19. / 720. + m5 * dv3 * G * 19. / 240.), g6s = -0.5 * m1 * dv3 * G / 4.;
    const double g4d = -m3 * G * dv3 / 12., g5d = -m4 * G * dv3 / 12.;
    {
        double *lr = lamV + 7 * kR3, *ll = lamV + 7 * kL3;
        const double gAR = gAd + gAs, gAL = -gAd + gAs;
        atomicAdd(lr + 0, gAR); atomicAdd(lr + 1, 0.5 * s3 * gAR);
        atomicAdd(ll + 0, gAL); atomicAdd(ll + 1, 0.5 * s3 * gAL);
        atomicAdd(lr + 3, g3d + g3s); atomicAdd(ll + 3, -g3d + g3s);
        atomicAdd(lr + 6, g6d + g6s); atomicAdd(ll + 6, -g6d + g6s);
        atomicAdd(lr + 4, g4d); atomicAdd(ll + 4, -g4d);
        atomicAdd(lr + 5, g5d); atomicAdd(ll + 5, -g5d);
    }
    // v1 direction (I5), upwind by the sign of the cell-average E_x
    const long long nc = (long long)ad.nx1 * ad.nx2;
    const double fs = ad.fscale;  // dx with LP_FIX_F12, else 1
    const double ie = fields[s] * fs, ixe = fields[nc + s] * fs, ixxe = fields[3 * nc + s] * fs;
    long long kR5 = -1, kL5 = -1;
    double s5;
    if (ie > 0) {
        if (j1 + 1 < nv) kR5 = s * sv + ((long long)(j1 + 1) * nv * nv + j2 * nv + j3);
        kL5 = k; s5 = -1.;
    } else {
        kR5 = k;
        if (j1 - 1 > -1) kL5 = s * sv + ((long long)(j1 - 1) * nv * nv + j2 * nv + j3);
        s5 = 1.;
    }
    double R5[7] = {0, 0, 0, 0, 0, 0, 0}, L5[7] = {0, 0, 0, 0, 0, 0, 0};
    if (kR5 >= 0) for (int q = 0; q < 7; ++q) R5[q] = V[7 * kR5 + q];
    if (kL5 >= 0) for (int q = 0; q < 7; ++q) L5[q] = V[7 * kL5 + q];
    const double hAd = m0 * dv2 * ie + m1 * dv2 * ixe, hAs = 0.5 * m2 * dv2 * ie;
    const double h1d = m0 * dv2 * ixe + m1 * dv2 * ixxe + m5 * dv2 * ixe * 5. / 12., h1s = 0.5 * m2 * dv2 * ixe;
    const double h4d = m3 * dv2 * ie / 12., h5d = m4 * dv2 * ie / 12.;
    const double hBd = m5 * dv2 * ie * 5. / 12., h6d = m5 * dv2 * ie * 133. / 720.;
    auto side = [&](double *l, double hA, double hB, double h1, double h6, double h4, double h5) {
        atomicAdd(l + 0, hA + hB);
        atomicAdd(l + 3, 0.5 * s5 * (hA + hB));
        atomicAdd(l + 6, 5. / 12. * hA + h6);
        atomicAdd(l + 1, h1);
        atomicAdd(l + 4, h4);
        atomicAdd(l + 5, h5);
    };
    if (kR5 >= 0) side(lamV + 7 * kR5, hAd + hAs, hBd, h1d + h1s, h6d, h4d, h5d);
    if (kL5 >= 0) side(lamV + 7 * kL5, -hAd + hAs, -hBd, -h1d + h1s, -h6d, -h4d, -h5d);
    // I1 and I2 (own record)
    const double sv_dv = ad.scalev * ad.rdv;
    double *lo = lamV + 7 * k;
    atomicAdd(lo + 0, m1 * dv3 * G - m2 * ie * sv_dv);
    atomicAdd(lo + 3, m1 * dv4 / 12. - m5 * dv2 * ie / 6.);
    atomicAdd(lo + 6, m1 * dv3 * G / 4. - m2 * ie * sv_dv / 4.);
    atomicAdd(lo + 1, -m2 * ixe * sv_dv);
    // field adjoints
    const double A5R = R5[0] + 0.5 * s5 * R5[3] + 5. / 12. * R5[6], A5L = L5[0] + 0.5 * s5 * L5[3] + 5. / 12. * L5[6];
    const double B5R = R5[0] + 0.5 * s5 * R5[3], B5L = L5[0] + 0.5 * s5 * L5[3];
    const double lie = m0 * dv2 * (A5R - A5L) + 0.5 * m2 * dv2 * (A5R + A5L) + m3 * dv2 / 12. * (R5[4] - L5[4]) +
                       m4 * dv2 / 12. * (R5[5] - L5[5]) +
                       m5 * dv2 * (5. / 12. * (B5R - B5L) + 133. / 720. * (R5[6] - L5[6])) -
                       m2 * (u[0] + u[6] / 4.) * sv_dv - m5 * u[3] * dv2 / 6.;
    const double lixe = m0 * dv2 * (R5[1] - L5[1]) + m1 * dv2 * (A5R - A5L) + 0.5 * m2 * dv2 * (R5[1] + L5[1]) +
                        m5 * dv2 * 5. / 12. * (R5[1] - L5[1]) - m2 * u[1] * sv_dv;
    const double lixxe = m1 * dv2 * (R5[1] - L5[1]);
    atomicAdd(lamF + 3 * s + 0, fs * lie);
    atomicAdd(lamF + 3 * s + 1, fs * lixe);
    atomicAdd(lamF + 3 * s + 2, fs * lixxe);
}

// lam_H = c * lam_out for every record (stage adjoint source)
__global__ void k_scale(double *__restrict__ y, const double *__restrict__ x, double c, long long n) {
    lp_grid_wait();
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) y[i] = c * x[i];
}

// ---------------------------------------------------------------- Poisson VJP (one block)
// fields (ie, ixe, ixxe per cell) and lam of phix, phiy -> lam of the charge
// moments rt (3 per cell): through the field reconstruction,
// the dense inverse of the LDG matrix (transposed) and the right-hand side.
__global__ void k_poisson_vjp(PoissonDev pd, const double *__restrict__ lamF, const double *__restrict__ lphix,
                              const double *__restrict__ lphiy, const double *__restrict__ Ainv,
                              double *__restrict__ lrt) {
    lp_grid_wait();
    extern __shared__ double sm[];
    const int nc = pd.nx * pd.ny, nd = pd.ndim, t = threadIdx.x;
    double *lpx = sm, *lpy = sm + 3 * nc, *lb = sm + 6 * nc;
    for (int ii = t; ii < nc; ii += blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            lpx[3 * ii + k] = lphix ? lphix[3 * ii + k] : 0.;
            lpy[3 * ii + k] = lphiy ? lphiy[3 * ii + k] : 0.;
        }
        if (lamF) {  // ie = phix0, ixe = phix1/12, ixxe = phix0/12
            lpx[3 * ii] += lamF[3 * ii] + lamF[3 * ii + 2] / 12.;
            lpx[3 * ii + 1] += lamF[3 * ii + 1] / 12.;
        }
    }
    __syncthreads();
    const double *acvx = pd.blk[0], *acyrr = pd.blk[1], *acyrl = pd.blk[2];
    const double *acvy = pd.blk[3], *acxrr = pd.blk[4], *acxrl = pd.blk[5];
    for (int ii = t; ii < nc; ii += blockDim.x) {
        const int ix = ii / pd.ny + 1, jy = ii % pd.ny + 1;
        for (int kk = 0; kk < 3; ++kk) {
            double g = 0.;
            // own E_x rows: phix[ii][k] = -(1/dxp) (sum (acvx + [ix<nx] acyrr) b_ii - [ix>1] acyrl b_left)
            for (int k = 0; k < 3; ++k) {
                const double cf = acvx[3 * k + kk] + (ix == pd.nx ? 0. : acyrr[3 * k + kk]);
                g -= cf * pd.rdxp * lpx[3 * ii + k];
            }
            // right neighbour's E_x uses this cell as its left cell
            if (ix < pd.nx) {
                const int ir = ii + pd.ny;
                for (int k = 0; k < 3; ++k) g += acyrl[3 * k + kk] * pd.rdxp * lpx[3 * ir + k];
            }
            // own E_y rows
            if (jy == 1) {
                if (kk == 2) g -= pd.rdyp * lpy[3 * ii];
            } else {
                const bool top = (jy == pd.ny && pd.gate[ix]);
                for (int k = 0; k < 3; ++k) {
                    const double cf = acvy[3 * k + kk] + (top ? 0. : acxrr[3 * k + kk]);
                    g -= cf * pd.rdyp * lpy[3 * ii + k];
                }
            }
            // the cell above uses this cell as its lower cell (jy + 1 > 1)
            if (jy < pd.ny) {
                const int ia = ii + 1;
                for (int k = 0; k < 3; ++k) g += acxrl[3 * k + kk] * pd.rdyp * lpy[3 * ia + k];
            }
            lb[3 * ii + kk] = g;
        }
    }
    __syncthreads();
    // lam_rhs = Ainv^T lam_b, then the right-hand side's scaling
    for (int j = t; j < nd; j += blockDim.x) {
        double s = 0.;
        for (int i = 0; i < nd; ++i) s += Ainv[(long long)i * nd + j] * lb[i];
        const double dd = pd.dxp * pd.dyp;
        lrt[j] = (j % 3 == 0) ? s * dd : s * dd / 12.;
    }
}

// lam_U[rec] += scalev * (lam_rt0, lam_rt1, lam_rt2) on slots (0 and 6/4, 1, 2)
__global__ void k_charge_vjp(const double *__restrict__ lrt, long long size, int nv3, double scalev,
                             double *__restrict__ lamU) {
    lp_grid_wait();
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= size) return;
    const long long s = k / nv3;
    const double a = scalev * lrt[3 * s], b = scalev * lrt[3 * s + 1], c = scalev * lrt[3 * s + 2];
    double *l = lamU + 7 * k;
    l[0] += a; l[6] += 0.25 * a; l[1] += b; l[2] += c;
}

// J = 1/2 dx dy sum (E0^2 + (E1^2 + E2^2)/12) over E_x and E_y and its
// gradient with respect to phix, phiy (one block).
__global__ void k_field_energy(const double *__restrict__ phix, const double *__restrict__ phiy, int nc, double dxdy,
                               double *__restrict__ J, double *__restrict__ lphix, double *__restrict__ lphiy) {
    lp_grid_wait();
    __shared__ double red[256];
    const int t = threadIdx.x;
    double s = 0.;
    for (int ii = t; ii < nc; ii += blockDim.x) {
        const double *px = phix + 3 * ii, *py = phiy + 3 * ii;
        s += px[0] * px[0] + py[0] * py[0] + (px[1] * px[1] + py[1] * py[1] + px[2] * px[2] + py[2] * py[2]) / 12.;
        if (lphix) {
            lphix[3 * ii] = dxdy * px[0]; lphix[3 * ii + 1] = dxdy * px[1] / 12.; lphix[3 * ii + 2] = dxdy * px[2] / 12.;
            lphiy[3 * ii] = dxdy * py[0]; lphiy[3 * ii + 1] = dxdy * py[1] / 12.; lphiy[3 * ii + 2] = dxdy * py[2] / 12.;
        }
    }
    red[t] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) red[t] += red[t + w];
        __syncthreads();
    }
    if (t == 0) *J = 0.5 * dxdy * red[0];
}

inline dim3 g1(long long total, int block) { return dim3((unsigned)((total + block - 1) / block)); }

}  // namespace

// =============================================================== launchers
cudaError_t launch_qvjp(const double2 *F, const double2 *lq, const double *P, const int *pair_off, int n, int Bp,
                        double2 *lF, cudaStream_t st) {
    k_qvjp<<<g1((long long)n * n * n * Bp, 128), 128, 0, st>>>(F, lq, P, pair_off, n, Bp, lF);
    return cudaGetLastError();
}

cudaError_t launch_project_vjp(const double *ltp, const double *tf, int n, int nv, int Bp, double2 *lZ, double2 *lY,
                               double2 *lQ, cudaStream_t st) {
    k_projT1<<<g1((long long)n * nv * nv * Bp, 128), 128, 0, st>>>(ltp, tf, n, nv, Bp, lZ);
    k_projT2<<<g1((long long)n * n * nv * Bp, 128), 128, 0, st>>>(lZ, tf, n, nv, Bp, lY);
    k_projT3<<<g1((long long)n * n * n * Bp, 128), 128, 0, st>>>(lY, tf, n, nv, Bp, lQ);
    return cudaGetLastError();
}

cudaError_t launch_collide_out_vjp(const double *lout, int nv, int c0, int B, int Bp, double dt, double kfac,
                                   double *ltp, double *lin, cudaStream_t st) {
    const long long nv3 = (long long)nv * nv * nv;
    k_collide_out_vjp<<<g1(nv3 * Bp, 128), 128, 0, st>>>(lout, nv, c0, B, Bp, dt, kfac, ltp, lin);
    return cudaGetLastError();
}

cudaError_t launch_nodes_vjp(const double *lf, int nv, int n, int c0, int B, int Bp, int slot1, const int *nfirst,
                             const int *ncount, const double *nodeoff, double *lin, cudaStream_t st) {
    const long long nv3 = (long long)nv * nv * nv;
    k_nodes_vjp<<<g1(nv3 * B, 128), 128, 0, st>>>(lf, nv, n, c0, B, Bp, slot1, nfirst, ncount, nodeoff, lin);
    return cudaGetLastError();
}

cudaError_t launch_axpby(double *y, double a, const double *x, double b, long long n, cudaStream_t st) {
    k_axpby<<<g1(n, 256), 256, 0, st>>>(y, a, x, b, n);
    return cudaGetLastError();
}
cudaError_t launch_caxpby(double2 *y, double a, const double2 *x, double b, long long n, cudaStream_t st) {
    k_caxpby<<<g1(n, 256), 256, 0, st>>>(y, a, x, b, n);
    return cudaGetLastError();
}
cudaError_t launch_add_re(double *y, double a, const double2 *x, double b, long long n, cudaStream_t st) {
    k_add_re<<<g1(n, 256), 256, 0, st>>>(y, a, x, b, n);
    return cudaGetLastError();
}
cudaError_t launch_dot_cell(const double *x, const double *y, long long npt, int Bp, int B, double scale, double *out,
                            cudaStream_t st) {
    k_dot_cell<<<(B + 7) / 8, 256, 0, st>>>(x, y, npt, Bp, B, scale, out);
    return cudaGetLastError();
}
cudaError_t launch_cdot_cell(const double2 *x, const double2 *y, long long npt, int Bp, int B, double scale,
                             double *out, cudaStream_t st) {
    k_cdot_cell<<<(B + 7) / 8, 256, 0, st>>>(x, y, npt, Bp, B, scale, out);
    return cudaGetLastError();
}
cudaError_t launch_qsum(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, long long n,
                        double2 *out, cudaStream_t st) {
    k_qsum<<<g1(n, 256), 256, 0, st>>>(q0, q1, q2, q3, n, out);
    return cudaGetLastError();
}

cudaError_t launch_flux_vjp(const AdvectDev &ad, const double *V, const double *fields, const double *lamH,
                            double *lamV, double *lamF, cudaStream_t st) {
    k_flux_vjp<<<g1(ad.size, 128), 128, 0, st>>>(ad, V, fields, lamH, lamV, lamF);
    return cudaGetLastError();
}
cudaError_t launch_scale(double *y, const double *x, double c, long long n, cudaStream_t st) {
    k_scale<<<g1(n, 256), 256, 0, st>>>(y, x, c, n);
    return cudaGetLastError();
}
cudaError_t launch_poisson_vjp(const PoissonDev &pd, const double *lamF, const double *lphix, const double *lphiy,
                               const double *Ainv, double *lrt, cudaStream_t st) {
    const int nc = pd.nx * pd.ny;
    const size_t smem = sizeof(double) * (size_t)(9 * nc);
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k_poisson_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_poisson_vjp<<<1, 256, smem, st>>>(pd, lamF, lphix, lphiy, Ainv, lrt);
    return cudaGetLastError();
}
cudaError_t launch_charge_vjp(const double *lrt, long long size, int nv3, double scalev, double *lamU,
                              cudaStream_t st) {
    k_charge_vjp<<<g1(size, 256), 256, 0, st>>>(lrt, size, nv3, scalev, lamU);
    return cudaGetLastError();
}
cudaError_t launch_field_energy(const double *phix, const double *phiy, int nc, double dxdy, double *J,
                                double *lphix, double *lphiy, cudaStream_t st) {
    k_field_energy<<<1, 256, 0, st>>>(phix, phiy, nc, dxdy, J, lphix, lphiy);
    return cudaGetLastError();
}

}  // namespace lp
