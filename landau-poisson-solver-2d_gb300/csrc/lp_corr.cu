// The vector-Jacobian product of ComputeQ's weighted sum
// (source/collisionRoutines_1.cpp:739-822) as correlations, in FP64.
//
// With the weight split of the convolution form (lp_fftq.cu),
//   q(xi) = sum_p sum_omega a_p(omega) b_p(u),   u = xi + h - omega,
//   a_p = C_p F (C_p the seven omega factors), b_p = w_p F (w_p(u) = 1,
//   (u_i - h)^2 or (u_i - h)(u_j - h)),
// the linearisation at F is dq(xi) = sum_p sum_omega [C_p dF(omega) b_p(u) +
// a_p(omega) w_p(u) dF(u)], a complex-linear map, whose adjoint is
//   lam_F(x) = sum_p [ C_p(x) R[b_p](x) + w_p(x) R[a_p](x) ],
//   R[g](x) = sum_xi lam_q(xi) conj(g(xi + h - x))   (xi + h - x on the grid),
// fourteen correlations of lam_q with the conjugated arrays.  Each is a
// product of M = 3n/2-point DFTs along the three axes: with the arrays zero-
// padded to M points, the indices xi + h - x that fall outside [0, n) land
// where lam_q is zero, so R[g] = IDFT( DFT(lam_q) conj(DFT(g)) e^{-2 pi i
// (k1 + k2 + k3) h / M} ) on x in [0, n)^3, and h / M = 1/3.
//
// The transforms are separable passes of per-axis DFT matrices (FP64,
// M x n forward; n x M inverse with the 1/M and the phase folded in); cells
// go through in chunks of kCorrCells, their arrays cell-minor.
#include "lp_adjoint.cuh"

#include <cmath>

namespace lp {
namespace {

constexpr int kCorrCells = 32;

__device__ __forceinline__ double2 cmulc2(double2 a, double2 b) {  // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// out = Mat (dout x din) applied along axis `ax` of `in` (dims d0 x d1 x d2,
// cell-minor with kCorrCells cells); one thread per (output point, cell)
__global__ void k_sep_pass(const double2 *__restrict__ in, int d0, int d1, int d2, int ax,
                           const double2 *__restrict__ Mat, int dout, double2 *__restrict__ out) {
    lp_grid_wait();
    int e[3] = {d0, d1, d2};
    const int din = e[ax];
    e[ax] = dout;
    const long long npt = (long long)e[0] * e[1] * e[2];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= npt * kCorrCells) return;
    const int c = (int)(tid % kCorrCells);
    long long p = tid / kCorrCells;
    const int o2 = (int)(p % e[2]);
    p /= e[2];
    const int o1 = (int)(p % e[1]), o0 = (int)(p / e[1]);
    const int o[3] = {o0, o1, o2};
    // input stride of axis ax and the input offset of the pencil
    const long long st[3] = {(long long)d1 * d2, (long long)d2, 1};
    long long base = 0;
    for (int a = 0; a < 3; ++a)
        if (a != ax) base += o[a] * st[a];
    const int oi = o[ax];
    double sr = 0., si = 0.;
    for (int s = 0; s < din; ++s) {
        const double2 m = Mat[(long long)oi * din + s];
        const double2 x = in[(base + s * st[ax]) * kCorrCells + c];
        sr += m.x * x.x - m.y * x.y;
        si += m.x * x.y + m.y * x.x;
    }
    out[tid] = make_double2(sr, si);
}

// g = C_p F (kind 0) or w_p F (kind 1) for cells [c0, c0 + kCorrCells) of F
// (stride Bp); lam (kind 2): g = lam_q of those cells
__global__ void k_corr_make(const double2 *__restrict__ src, int Bp, int c0, int B, const double *__restrict__ Cp,
                            int p, int n, int kind, double2 *__restrict__ g) {
    lp_grid_wait();
    const long long n3 = (long long)n * n * n;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= n3 * kCorrCells) return;
    const int c = (int)(tid % kCorrCells);
    const long long pt = tid / kCorrCells;
    double2 v = make_double2(0., 0.);
    if (c0 + c < B) v = src[pt * Bp + c0 + c];
    double s = 1.;
    if (kind == 0) {
        s = Cp[(long long)p * n3 + pt];
    } else if (kind == 1 && p > 0) {
        const int h = n / 2, i = (int)(pt / ((long long)n * n)), j = (int)((pt / n) % n), k = (int)(pt % n);
        const double u[3] = {(double)(i - h), (double)(j - h), (double)(k - h)};
        // p = 1..6: u0^2, u1^2, u2^2, u0 u1, u0 u2, u1 u2
        static constexpr int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
        s = u[ia[p - 1]] * u[ib[p - 1]];
    }
    g[tid] = make_double2(s * v.x, s * v.y);
}

// G = L conj(G), elementwise
__global__ void k_corr_prod(const double2 *__restrict__ L, double2 *__restrict__ G, long long nel) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid < nel) G[tid] = cmulc2(L[tid], G[tid]);
}

// acc (+)= coefficient(x) R(x): C_p(x) for a correlation with b_p (kind 0),
// w_p(x) for one with a_p (kind 1)
__global__ void k_corr_acc(const double2 *__restrict__ R, const double *__restrict__ Cp, int p, int n, int kind,
                           bool first, double2 *__restrict__ acc) {
    lp_grid_wait();
    const long long n3 = (long long)n * n * n;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= n3 * kCorrCells) return;
    const long long pt = tid / kCorrCells;
    double s = 1.;
    if (kind == 0) {
        s = Cp[(long long)p * n3 + pt];
    } else if (p > 0) {
        const int h = n / 2, i = (int)(pt / ((long long)n * n)), j = (int)((pt / n) % n), k = (int)(pt % n);
        const double u[3] = {(double)(i - h), (double)(j - h), (double)(k - h)};
        static constexpr int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
        s = u[ia[p - 1]] * u[ib[p - 1]];
    }
    const double2 r = R[tid];
    const double2 a = first ? make_double2(0., 0.) : acc[tid];
    acc[tid] = make_double2(a.x + s * r.x, a.y + s * r.y);
}

__global__ void k_corr_store(const double2 *__restrict__ acc, int n, int Bp, int c0, int B, double2 *__restrict__ lF) {
    lp_grid_wait();
    const long long n3 = (long long)n * n * n;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= n3 * kCorrCells) return;
    const int c = (int)(tid % kCorrCells);
    if (c0 + c < B) lF[(tid / kCorrCells) * Bp + c0 + c] = acc[tid];
}

inline unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

int corr_cells() { return kCorrCells; }

size_t corr_scratch_elems(int n) {
    const size_t M = 3 * (size_t)n / 2, m3 = M * M * M, n3 = (size_t)n * n * n;
    return (3 * m3 + n3) * kCorrCells;
}

void corr_tables(const double *shat, const double *ahat, const double *cw, double h_eta, int n, std::vector<double> &Cp,
                 std::vector<double> &Wf, std::vector<double> &Wi) {
    const size_t n3 = (size_t)n * n * n;
    const int M = 3 * n / 2;
    Cp.assign(7 * n3, 0.);
    const double h2 = h_eta * h_eta;
    // the pairs of lp_fftq.cu: (ahat, 1), (S00, u0^2), (S11, u1^2), (S22, u2^2),
    // (S01, u0 u1), (S02, u0 u2), (S12, u1 u2); shat per omega: S00, S01, S02, S11, S12, S22
    static const int sidx[6] = {0, 3, 5, 1, 2, 4};
    static const double mult[6] = {1., 1., 1., 2., 2., 2.};
    for (size_t o = 0; o < n3; ++o) {
        Cp[o] = cw[o] * ahat[o];
        for (int p = 0; p < 6; ++p) Cp[(p + 1) * n3 + o] = -mult[p] * h2 * cw[o] * shat[6 * o + sidx[p]];
    }
    const double PI = std::acos(-1.0);
    Wf.assign(2 * (size_t)M * n, 0.);
    Wi.assign(2 * (size_t)n * M, 0.);
    for (int k = 0; k < M; ++k)
        for (int s = 0; s < n; ++s) {
            const double a = -2. * PI * ((long long)k * s % M) / M;
            Wf[2 * ((size_t)k * n + s)] = std::cos(a);
            Wf[2 * ((size_t)k * n + s) + 1] = std::sin(a);
        }
    for (int x = 0; x < n; ++x)
        for (int k = 0; k < M; ++k) {
            // e^{2 pi i k x / M} e^{-2 pi i k / 3} / M
            const double a = 2. * PI * ((long long)k * x % M) / M - 2. * PI * (k % 3) / 3.;
            Wi[2 * ((size_t)x * M + k)] = std::cos(a) / M;
            Wi[2 * ((size_t)x * M + k) + 1] = std::sin(a) / M;
        }
}

cudaError_t launch_qvjp_corr(const double2 *F, const double2 *lq, const double *Cp, const double2 *Wf,
                             const double2 *Wi, int n, int Bp, int B, double2 *lF, double2 *scratch,
                             cudaStream_t st) {
    const int M = 3 * n / 2;
    const long long m3 = (long long)M * M * M, n3 = (long long)n * n * n, CB = kCorrCells;
    double2 *L = scratch, *S1 = L + m3 * CB, *S2 = S1 + m3 * CB, *acc = S2 + m3 * CB;
    auto fwd = [&](double2 *g) {  // g (n^3) -> S2 (M^3) through S1
        k_sep_pass<<<blocks((long long)n * n * M * CB), 256, 0, st>>>(g, n, n, n, 2, Wf, M, S1);
        k_sep_pass<<<blocks((long long)n * M * M * CB), 256, 0, st>>>(S1, n, n, M, 1, Wf, M, S2);
        k_sep_pass<<<blocks(m3 * CB), 256, 0, st>>>(S2, n, M, M, 0, Wf, M, S1);
        return S1;
    };
    for (int c0 = 0; c0 < B; c0 += (int)CB) {
        // DFT of lam_q
        k_corr_make<<<blocks(n3 * CB), 256, 0, st>>>(lq, Bp, c0, B, nullptr, 0, n, 2, acc);
        double2 *G = fwd(acc);
        cudaMemcpyAsync(L, G, sizeof(double2) * m3 * CB, cudaMemcpyDeviceToDevice, st);
        bool first = true;
        for (int p = 0; p < 7; ++p)
            for (int kind = 0; kind < 2; ++kind) {
                // the array correlated with lam: a_p (kind 0 makes C_p F, its R
                // takes w_p) or b_p (kind 1 makes w_p F, its R takes C_p)
                k_corr_make<<<blocks(n3 * CB), 256, 0, st>>>(F, Bp, c0, B, Cp, p, n, kind, S2);
                double2 *Gp = fwd(S2);  // in S1
                k_corr_prod<<<blocks(m3 * CB), 256, 0, st>>>(L, Gp, m3 * CB);
                k_sep_pass<<<blocks((long long)n * M * M * CB), 256, 0, st>>>(Gp, M, M, M, 0, Wi, n, S2);
                k_sep_pass<<<blocks((long long)n * n * M * CB), 256, 0, st>>>(S2, n, M, M, 1, Wi, n, S1);
                k_sep_pass<<<blocks(n3 * CB), 256, 0, st>>>(S1, n, n, M, 2, Wi, n, S2);
                k_corr_acc<<<blocks(n3 * CB), 256, 0, st>>>(S2, Cp, p, n, kind == 0 ? 1 : 0, first, acc + 0);
                first = false;
            }
        k_corr_store<<<blocks(n3 * CB), 256, 0, st>>>(acc, n, Bp, c0, B, lF);
    }
    return cudaGetLastError();
}

}  // namespace lp
