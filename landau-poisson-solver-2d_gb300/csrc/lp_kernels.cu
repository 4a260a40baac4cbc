// CUDA kernels of the GB300 Landau-Poisson hot path (sm_103a).
// Citations are to the reference checkout:
//   C = source/collisionRoutines_1.cpp   K = source/conservationRoutines.cpp
//   A = source/advection_1.cpp           P = source/PoissonFunctions.cpp
//   S = source/SetInit_1.cpp             MC = source/MomentCalculations.cpp
#include "lp_kernels.cuh"
#include "lp_dev.cuh"

#include <algorithm>
#include <cstdint>
#include <type_traits>

namespace lp {
namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename R> __device__ __forceinline__ typename V2<R>::t mk2(R x, R y);
template <> __device__ __forceinline__ double2 mk2<double>(double x, double y) { return make_double2(x, y); }
template <> __device__ __forceinline__ float2 mk2<float>(float x, float y) { return make_float2(x, y); }

template <typename R> __device__ __forceinline__ typename V2<R>::t ld2(const R *p) { return mk2<R>(*p, R(0)); }
template <typename R> __device__ __forceinline__ typename V2<R>::t ld2(const typename V2<R>::t *p) { return *p; }
template <typename R> __device__ __forceinline__ typename V2<R>::t ld2c(const double2 *p) {
    double2 v = *p;
    return mk2<R>((R)v.x, (R)v.y);
}

inline dim3 grid1(long long total, int block) { return dim3((unsigned)((total + block - 1) / block)); }

// ---------------------------------------------------------------- pairs
// gHat3(eta_xi, eta_omega) (C:30-69) from the omega tables, in the reference's
// order and without FMA contraction, so the value equals the host's.
__device__ double weight_dev(const double *eta, const double *shat, const double *ahat,
                             const unsigned char *rzero, int n, int i, int j, int k, int o) {
    const int l = o / (n * n), m = (o / n) % n, q = o % n;
    const double *s = shat + 6 * (long long)o;
    const double d0 = __dsub_rn(eta[i], eta[l]), d1 = __dsub_rn(eta[j], eta[m]), d2 = __dsub_rn(eta[k], eta[q]);
    double r = 0.0;
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[0], d0), d0));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[1], d0), d1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[2], d0), d2));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[1], d1), d0));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[3], d1), d1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[4], d1), d2));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[2], d2), d0));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[4], d2), d1));
    r = __dadd_rn(r, __dmul_rn(__dmul_rn(s[5], d2), d2));
    return rzero[o] ? -r : __dsub_rn(ahat[o], r);
}

__global__ void k_pairs(const double *__restrict__ eta, const double *__restrict__ shat,
                        const double *__restrict__ ahat, const unsigned char *__restrict__ rzero,
                        const double *__restrict__ cw, const int *__restrict__ pair_off, int n,
                        double *__restrict__ P64, float *__restrict__ P32, unsigned *__restrict__ PI) {
    lp_grid_wait();
    const int xi = blockIdx.x, h = n / 2;
    const int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
    // window of omega where u = xi + n/2 - omega lies in the grid (C:764-789)
    const int si = i < h ? 0 : i - h + 1, ni = i < h ? i + h + 1 : 3 * h - 1 - i;
    const int sj = j < h ? 0 : j - h + 1, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
    const int sk = k < h ? 0 : k - h + 1, nk = k < h ? k + h + 1 : 3 * h - 1 - k;
    const int cnt = ni * nj * nk, off = pair_off[xi], npair = pair_off[xi + 1] - off;
    for (int L = threadIdx.x; L < npair; L += blockDim.x) {
        const int l = si + L / (nj * nk), m = sj + (L / nk) % nj, q = sk + L % nk;
        const int Lu = cnt - 1 - L;
        const int lu = si + Lu / (nj * nk), mu = sj + (Lu / nk) % nj, qu = sk + Lu % nk;
        const int om = (l * n + m) * n + q, uu = (lu * n + mu) * n + qu;
        double w = __dmul_rn(cw[om], weight_dev(eta, shat, ahat, rzero, n, i, j, k, om));
        if (Lu != L) w = __dadd_rn(w, __dmul_rn(cw[uu], weight_dev(eta, shat, ahat, rzero, n, i, j, k, uu)));
        if (P64) P64[off + L] = w;
        if (P32) P32[off + L] = (float)w;
        PI[off + L] = (unsigned)om | ((unsigned)uu << 16);
    }
}

// ---------------------------------------------------------------- two-species linear term
// gHat3_linear(eta_xi, eta_omega) = -sum_ij Shat_ij(omega) xi_i (xi_j - omega_j)
// (C:71-96) in the reference's (i, j) order, without FMA.
__device__ double weight_lin_dev(const double *eta, const double *shat, int n, int i, int j, int k, int o) {
    const int l = o / (n * n), m = (o / n) % n, q = o % n;
    const double *s = shat + 6 * (long long)o;
    const double S[3][3] = {{s[0], s[1], s[2]}, {s[1], s[3], s[4]}, {s[2], s[4], s[5]}};
    const double z[3] = {eta[i], eta[j], eta[k]}, w[3] = {eta[l], eta[m], eta[q]};
    double r = 0.;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) r = __dadd_rn(r, __dmul_rn(__dmul_rn(S[a][b], z[a]), __dsub_rn(z[b], w[b])));
    return -r;
}

// Linear weight table: for every xi, all window entries L (row-major over the
// window box) hold cw(omega) scale3 gHat3_linear(eta_xi, eta_omega), the
// factor of F(xi + n/2 - omega) in ComputeQ's linear term (C:614-621).
__global__ void k_lin_weights(const double *__restrict__ eta, const double *__restrict__ shat,
                              const double *__restrict__ cw, const long long *__restrict__ win_off, int n,
                              double scale3, double *__restrict__ W64, float *__restrict__ W32) {
    lp_grid_wait();
    const int xi = blockIdx.x, h = n / 2;
    const int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
    const int si = i < h ? 0 : i - h + 1, sj = j < h ? 0 : j - h + 1, sk = k < h ? 0 : k - h + 1;
    const int nj = j < h ? j + h + 1 : 3 * h - 1 - j, nk = k < h ? k + h + 1 : 3 * h - 1 - k;
    const long long off = win_off[xi], cnt = win_off[xi + 1] - off;
    for (long long L = threadIdx.x; L < cnt; L += blockDim.x) {
        const int l = si + (int)(L / (nj * nk)), m = sj + (int)((L / nk) % nj), q = sk + (int)(L % nk);
        const int o = (l * n + m) * n + q;
        const double w = __dmul_rn(__dmul_rn(cw[o], scale3), weight_lin_dev(eta, shat, n, i, j, k, o));
        if (W64) W64[off + L] = w;
        if (W32) W32[off + L] = (float)w;
    }
}

// ql(xi) = sum over the window of Wl F(xi + n/2 - omega), one thread per (xi,
// cell), cell-minor.  FP64: one sequential sum in the window's order with
// _rn operations; FP32: each window line summed in FP32 and the lines added
// to a Kahan-compensated FP32 sum.
template <typename R>
__global__ void k_qlin(const typename V2<R>::t *__restrict__ F, const R *__restrict__ Wl,
                       const long long *__restrict__ win_off, int n, int Bp, double2 *__restrict__ ql) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int n3 = n * n * n, h = n / 2;
    if (tid >= (long long)n3 * Bp) return;
    const int c = (int)(tid % Bp), xi = (int)(tid / Bp);
    const int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
    const int si = i < h ? 0 : i - h + 1, ni = i < h ? i + h + 1 : 3 * h - 1 - i;
    const int sj = j < h ? 0 : j - h + 1, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
    const int sk = k < h ? 0 : k - h + 1, nk = k < h ? k + h + 1 : 3 * h - 1 - k;
    const R *w = Wl + win_off[xi];
    if constexpr (std::is_same<R, double>::value) {
        double sr = 0., sim = 0.;
        for (int a = 0; a < ni; ++a)
            for (int b = 0; b < nj; ++b) {
                const int x = i + h - (si + a), y = j + h - (sj + b);
                const double2 *Fl = F + ((long long)(x * n + y) * n) * Bp + c;
                const double *wl = w + (a * nj + b) * nk;
                for (int e = 0; e < nk; ++e) {
                    const double2 f = Fl[(long long)(k + h - (sk + e)) * Bp];
                    sr = __dadd_rn(sr, __dmul_rn(wl[e], f.x));
                    sim = __dadd_rn(sim, __dmul_rn(wl[e], f.y));
                }
            }
        ql[tid] = make_double2(sr, sim);
    } else {
        float sr = 0.f, sim = 0.f, cr = 0.f, ci = 0.f;
        for (int a = 0; a < ni; ++a)
            for (int b = 0; b < nj; ++b) {
                const int x = i + h - (si + a), y = j + h - (sj + b);
                const float2 *Fl = F + ((long long)(x * n + y) * n) * Bp + c;
                const float *wl = w + (a * nj + b) * nk;
                float pr = 0.f, pim = 0.f;
                for (int e = 0; e < nk; ++e) {
                    const float2 f = Fl[(long long)(k + h - (sk + e)) * Bp];
                    pr = fmaf(wl[e], f.x, pr);
                    pim = fmaf(wl[e], f.y, pim);
                }
                float yr = pr - cr, tr = sr + yr;
                cr = (tr - sr) - yr; sr = tr;
                float yi = pim - ci, ti = sim + yi;
                ci = (ti - sim) - yi; sim = ti;
            }
        ql[tid] = make_double2((double)sr - (double)cr, (double)sim - (double)ci);
    }
}

// q += ql (the two-species stage's mode array, C:656-698)
__global__ void k_qadd(double2 *__restrict__ q, const double2 *__restrict__ ql, long long total) {
    lp_grid_wait();
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < total) { const double2 a = q[t], b = ql[t]; q[t] = make_double2(a.x + b.x, a.y + b.y); }
}

// ---------------------------------------------------------------- nodes
// setInit_spectral for a batch of cells, cell-minor output
// (n <= 32): a block takes one (l, m) node pair and 32 cells; a warp takes
// four cells with the lanes along q, so the lanes read consecutive records of
// one cell, and the values go out cell-minor through a shared tile.
template <typename R>
__global__ void __launch_bounds__(256) k_nodes_t(const double *__restrict__ U, int nv, int n, int c0, int B, int Bp,
                                                 int slot1, const int *__restrict__ nodecell,
                                                 const double *__restrict__ nodeoff, R *__restrict__ f) {
    lp_grid_wait();
    __shared__ R tile[32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lm = blockIdx.x, l = lm / n, m = lm - l * n, cb = blockIdx.y * 32;
    const int j1 = nodecell[l], j2 = nodecell[m];
    const double a = nodeoff[l], b = nodeoff[m];
    const int q = lane < n ? lane : n - 1;
    const int j3 = nodecell[q];
    const double e = nodeoff[q];
    const long long nv3 = (long long)nv * nv * nv, rec = (j1 * nv + j2) * nv + j3;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int cc = w + 8 * i;
        R v = R(0);
        if (cb + cc < B) {
            const double *u = U + 7 * ((long long)(c0 + cb + cc) * nv3 + rec);
            const double val = u[0] + u[slot1] * a + u[4] * b + u[5] * e + u[6] * (a * a + b * b + e * e);
            v = (R)val;
        }
        tile[lane][cc] = v;
    }
    __syncthreads();
    R *out = f + (long long)lm * n * Bp + cb + lane;
    for (int qq = w; qq < n; qq += 8) out[(long long)qq * Bp] = tile[qq][lane];
}

// ---------------------------------------------------------------- DFT pass
// out(pencil)[p][c] = sum_a M[p][a] in(pencil)[a][c] along axis ax of an
// n x n x n x Bp array; M holds the per-axis DFT with the fft3D/FS phases and
// scalings folded in.  Block (32 cells, n outputs) over kDftPencils pencils
// in turn: M is staged in shared memory once per block, and the next
// pencil's element is loaded into a register while the current one is
// computed (pencils alternate between two shared buffers).
// OUT 0: complex store.  OUT 1: FS stage epilogue on the real part.
constexpr int kDftPencils = 4;

template <typename R, typename TIn, int OUT>
__global__ void k_dft(const TIn *__restrict__ in, typename V2<R>::t *__restrict__ out,
                      const R *__restrict__ M, int n, int ax, int Bp, int stage, R dt, R nu,
                      const R *__restrict__ f, R *__restrict__ qn, R *__restrict__ f1,
                      const double *__restrict__ cnu, const double *__restrict__ cdt) {
    lp_grid_wait();
    using C = typename V2<R>::t;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *Ms = reinterpret_cast<C *>(smem_raw);
    C *pen = Ms + n * n;  // [2][n][32]
    const int cl = threadIdx.x, p = threadIdx.y;
    const int c = blockIdx.y * 32 + cl;
    const int pid0 = blockIdx.x * kDftPencils, pend = min(n * n, pid0 + kDftPencils);
    for (int t = threadIdx.y * 32 + threadIdx.x; t < n * n; t += 32 * n) Ms[t] = mk2<R>(M[2 * t], M[2 * t + 1]);
    auto offset = [&](int pid) -> long long {
        long long base, stride;
        if (ax == 2) { base = (long long)pid * n * Bp; stride = Bp; }
        else if (ax == 1) { const int i0 = pid / n, i2 = pid % n; base = ((long long)i0 * n * n + i2) * Bp; stride = (long long)n * Bp; }
        else { base = (long long)pid * Bp; stride = (long long)n * n * Bp; }
        return base + p * stride + c;
    };
    auto load = [&](long long o) -> C {
        if constexpr (std::is_same<TIn, double2>::value) return ld2c<R>(in + o);
        else return ld2<R>(in + o);
    };
    R dtc = dt, nuc = nu;
    if (OUT == 1 && cnu) { nuc = (R)cnu[c]; dtc = (R)cdt[c]; }
    long long o = offset(pid0);
    C v = load(o);
    for (int pid = pid0, j = 0; pid < pend; ++pid, ++j) {
        C *pb = pen + (j & 1) * n * 32;
        pb[p * 32 + cl] = v;
        const long long onext = pid + 1 < pend ? offset(pid + 1) : o;
        if (pid + 1 < pend) v = load(onext);
        __syncthreads();
        R sr = R(0), si = R(0);
#pragma unroll 4
        for (int a = 0; a < n; ++a) {
            const C m = Ms[p * n + a], x = pb[a * 32 + cl];
            sr += m.x * x.x - m.y * x.y;
            si += m.x * x.y + m.y * x.x;
        }
        if constexpr (OUT == 0) {
            out[o] = mk2<R>(sr, si);
        } else {
            // RK4 node-value stages (C:831-862); per-cell nu and dt when given.
            if (stage == 0) {
                qn[o] = sr;
                f1[o] = f[o] + dtc * sr * nuc;
            } else {
                f1[o] = f[o] + R(0.5) * dtc * qn[o] * nuc + R(0.5) * dtc * sr * nuc;
            }
        }
        o = onext;
    }
}

// The same pass for n in {8, 16, 24, 32}: OG threads per (pencil, cell),
// each holding the pencil's n inputs in registers and forming n / OG of the
// outputs (in pairs) from M in shared memory (broadcast reads); the pass
// needs one block barrier (after staging M) instead of one per pencil.
// cf/lamc (pencils along the last axis only): the input is a mode array whose
// conservation projection was not applied; x -= C^T lambda is applied on load
// in R precision (cf: the 5 nonzero constraint rows, lamc: [5][Bp]).
template <typename R, typename TIn, int OUT, int N, int PY, int OG>
__global__ void __launch_bounds__(32 * PY * OG) k_dftp(const TIn *__restrict__ in, typename V2<R>::t *__restrict__ out,
                                                       const R *__restrict__ M, int ax, int Bp, int stage, R dt,
                                                       R nu, const R *__restrict__ f, R *__restrict__ qn,
                                                       R *__restrict__ f1, const double *__restrict__ cnu,
                                                       const double *__restrict__ cdt, const float *__restrict__ cf,
                                                       const double *__restrict__ lamc) {
    lp_grid_wait();
    using C = typename V2<R>::t;
    constexpr int NO = N / OG;  // outputs per thread
    __shared__ C Ms[N * N];
    __shared__ float cfs[PY][5][N];  // constraint rows of the block's pencils (cf given)
    for (int t = threadIdx.y * 32 + threadIdx.x; t < N * N; t += 32 * PY * OG) Ms[t] = mk2<R>(M[2 * t], M[2 * t + 1]);
    if (cf) {
        constexpr int n3 = N * N * N;
        for (int t = threadIdx.y * 32 + threadIdx.x; t < PY * 5 * N; t += 32 * PY * OG) {
            const int pp = t / (5 * N), r = (t / N) % 5, i = t % N, p0 = blockIdx.x * PY + pp;
            cfs[pp][r][i] = p0 < N * N ? cf[r * n3 + p0 * N + i] : 0.f;
        }
    }
    __syncthreads();
    const int pid = blockIdx.x * PY + threadIdx.y / OG, og = threadIdx.y % OG;
    if (pid >= N * N) return;
    const int c = blockIdx.y * 32 + threadIdx.x;
    long long base, stride;
    if (ax == 2) { base = (long long)pid * N * Bp; stride = Bp; }
    else if (ax == 1) { const int i0 = pid / N, i2 = pid % N; base = ((long long)i0 * N * N + i2) * Bp; stride = (long long)N * Bp; }
    else { base = (long long)pid * Bp; stride = (long long)N * N * Bp; }
    base += c;
    C x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if constexpr (std::is_same<TIn, double2>::value) x[i] = ld2c<R>(in + base + i * stride);
        else x[i] = ld2<R>(in + base + i * stride);
    }
    if (cf) {
        const R l0 = (R)lamc[c], l1 = (R)lamc[Bp + c], l2 = (R)lamc[2 * Bp + c], l3 = (R)lamc[3 * Bp + c],
                l4 = (R)lamc[4 * Bp + c];
        const float(*r)[N] = cfs[threadIdx.y / OG];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            x[i].x -= (R)r[0][i] * l0 + (R)r[4][i] * l4;
            x[i].y -= (R)r[1][i] * l1 + (R)r[2][i] * l2 + (R)r[3][i] * l3;
        }
    }
    R dtc = dt, nuc = nu;
    if (OUT == 1 && cnu) { nuc = (R)cnu[c]; dtc = (R)cdt[c]; }
#pragma unroll
    for (int aa = 0; aa < NO; aa += 2) {
        const int a = og * NO + aa;
        R sr0 = R(0), si0 = R(0), sr1 = R(0), si1 = R(0);
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const C m0 = Ms[a * N + i], m1 = Ms[(a + 1) * N + i];
            sr0 += m0.x * x[i].x - m0.y * x[i].y;
            si0 += m0.x * x[i].y + m0.y * x[i].x;
            sr1 += m1.x * x[i].x - m1.y * x[i].y;
            si1 += m1.x * x[i].y + m1.y * x[i].x;
        }
        const long long o0 = base + a * stride, o1 = o0 + stride;
        if constexpr (OUT == 0) {
            out[o0] = mk2<R>(sr0, si0);
            out[o1] = mk2<R>(sr1, si1);
        } else {
            // RK4 node-value stages (C:831-862); per-cell nu and dt when given.
            if (stage == 0) {
                qn[o0] = sr0;
                f1[o0] = f[o0] + dtc * sr0 * nuc;
                qn[o1] = sr1;
                f1[o1] = f[o1] + dtc * sr1 * nuc;
            } else {
                f1[o0] = f[o0] + R(0.5) * dtc * qn[o0] * nuc + R(0.5) * dtc * sr0 * nuc;
                f1[o1] = f[o1] + R(0.5) * dtc * qn[o1] * nuc + R(0.5) * dtc * sr1 * nuc;
            }
        }
    }
}

// ---------------------------------------------------------------- register FFTs
// Length-N DFTs y[a] = sum_i r^(a i) x[i], r = exp(S 2 pi i / N), S = -1
// (forward) or +1 (inverse), on a register array: radices 2, 3, 4 and 8 in
// closed form and Cooley-Tukey N = N1 N2 (N1-point DFTs over the strided
// inputs, twiddles r^(a1 i2) from the factor table, N2-point DFTs) for
// N = 16 (4 x 4), 24 (3 x 8), 32 (4 x 8).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// z * (S i)
template <int S> __device__ __forceinline__ float2 mul_si(float2 z) {
    return S > 0 ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x);
}

template <int S> __device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}
template <int S> __device__ __forceinline__ void dft3(float2 &a, float2 &b, float2 &c) {
    constexpr float h3 = 0.8660254037844386f;  // sqrt(3) / 2
    const float2 t = cadd(b, c), d = mul_si<S>(csub(b, c));
    const float2 m = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
    a = cadd(a, t);
    b = make_float2(m.x + h3 * d.x, m.y + h3 * d.y);
    c = make_float2(m.x - h3 * d.x, m.y - h3 * d.y);
}
template <int S> __device__ __forceinline__ void dft4(float2 &a, float2 &b, float2 &c, float2 &d) {
    const float2 a0 = cadd(a, c), a1 = csub(a, c), b0 = cadd(b, d), b1 = mul_si<S>(csub(b, d));
    a = cadd(a0, b0);
    b = cadd(a1, b1);
    c = csub(a0, b0);
    d = csub(a1, b1);
}
template <int S> __device__ __forceinline__ void dft8(float2 (&v)[8]) {
    constexpr float r2 = 0.7071067811865476f;  // 1 / sqrt(2)
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<S>(e0, e1, e2, e3);
    dft4<S>(o0, o1, o2, o3);
    // o_k * r^k, r = exp(S 2 pi i / 8)
    const float2 s1 = cadd(o1, mul_si<S>(o1)), s3 = csub(mul_si<S>(o3), o3);
    o1 = make_float2(r2 * s1.x, r2 * s1.y);
    o2 = mul_si<S>(o2);
    o3 = make_float2(r2 * s3.x, r2 * s3.y);
    v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}
template <int K, int S> __device__ __forceinline__ void dft_small(float2 (&v)[K]) {
    if constexpr (K == 2) dft2<S>(v[0], v[1]);
    else if constexpr (K == 3) dft3<S>(v[0], v[1], v[2]);
    else if constexpr (K == 4) dft4<S>(v[0], v[1], v[2], v[3]);
    else dft8<S>(v);
}
template <int N> struct FftPlan;
template <> struct FftPlan<8> { static constexpr int N1 = 8, N2 = 1; };
template <> struct FftPlan<16> { static constexpr int N1 = 4, N2 = 4; };
template <> struct FftPlan<24> { static constexpr int N1 = 3, N2 = 8; };
template <> struct FftPlan<32> { static constexpr int N1 = 4, N2 = 8; };

// w: the factor table's roots, w[k] = exp(S 2 pi i k / N)
template <int N, int S> __device__ __forceinline__ void fft_reg(float2 (&x)[N], const float2 *w) {
    constexpr int N1 = FftPlan<N>::N1, N2 = FftPlan<N>::N2;
    if constexpr (N2 == 1) {
        dft_small<N1, S>(x);
    } else {
        float2 z[N];  // z[a1 N2 + i2]
#pragma unroll
        for (int i2 = 0; i2 < N2; ++i2) {
            float2 v[N1];
#pragma unroll
            for (int i1 = 0; i1 < N1; ++i1) v[i1] = x[N2 * i1 + i2];
            dft_small<N1, S>(v);
#pragma unroll
            for (int a1 = 0; a1 < N1; ++a1) z[a1 * N2 + i2] = (a1 * i2) % N ? cmulf(v[a1], w[(a1 * i2) % N]) : v[a1];
        }
#pragma unroll
        for (int a1 = 0; a1 < N1; ++a1) {
            float2 v[N2];
#pragma unroll
            for (int i2 = 0; i2 < N2; ++i2) v[i2] = z[a1 * N2 + i2];
            dft_small<N2, S>(v);
#pragma unroll
            for (int a2 = 0; a2 < N2; ++a2) x[a1 + N1 * a2] = v[a2];
        }
    }
}

// The FP32 per-axis pass as a register FFT: one thread per (pencil, cell)
// holds the pencil, multiplies by pre, transforms and multiplies by post.
// OUT 0: complex store; OUT 1: the RK4 node-value stage on the real part.
// cf/lamc (axis 2 only): the lazy conservation correction on load.
template <typename TIn, int OUT, int N, int S, int PY>
__global__ void __launch_bounds__(32 * PY) k_fftf(const TIn *__restrict__ in, float2 *__restrict__ out,
                                                  const __grid_constant__ DftFac fac, int ax, int Bp, int stage,
                                                  float dt, float nu, const float *__restrict__ f,
                                                  float *__restrict__ qn, float *__restrict__ f1,
                                                  const double *__restrict__ cnu, const double *__restrict__ cdt,
                                                  const float *__restrict__ cf, const double *__restrict__ lamc) {
    lp_grid_wait();
    __shared__ float cfs[PY][5][N];
    if (cf) {
        constexpr int n3 = N * N * N;
        for (int t = threadIdx.y * 32 + threadIdx.x; t < PY * 5 * N; t += 32 * PY) {
            const int pp = t / (5 * N), r = (t / N) % 5, i = t % N, p0 = blockIdx.x * PY + pp;
            cfs[pp][r][i] = p0 < N * N ? cf[r * n3 + p0 * N + i] : 0.f;
        }
        __syncthreads();
    }
    const int pid = blockIdx.x * PY + threadIdx.y;
    if (pid >= N * N) return;
    const int c = blockIdx.y * 32 + threadIdx.x;
    long long base, stride;
    if (ax == 2) { base = (long long)pid * N * Bp; stride = Bp; }
    else if (ax == 1) { const int i0 = pid / N, i2 = pid % N; base = ((long long)i0 * N * N + i2) * Bp; stride = (long long)N * Bp; }
    else { base = (long long)pid * Bp; stride = (long long)N * N * Bp; }
    base += c;
    float2 x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if constexpr (std::is_same<TIn, double2>::value) x[i] = ld2c<float>(in + base + i * stride);
        else x[i] = ld2<float>(in + base + i * stride);
    }
    if (cf) {
        const float l0 = (float)lamc[c], l1 = (float)lamc[Bp + c], l2 = (float)lamc[2 * Bp + c],
                    l3 = (float)lamc[3 * Bp + c], l4 = (float)lamc[4 * Bp + c];
        const float(*r)[N] = cfs[threadIdx.y];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            x[i].x -= r[0][i] * l0 + r[4][i] * l4;
            x[i].y -= r[1][i] * l1 + r[2][i] * l2 + r[3][i] * l3;
        }
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
        if constexpr (std::is_same<TIn, float>::value) x[i] = make_float2(x[i].x * fac.pre[i].x, x[i].x * fac.pre[i].y);
        else x[i] = cmulf(x[i], fac.pre[i]);
    }
    fft_reg<N, S>(x, fac.w);
    float dtc = dt, nuc = nu;
    if (OUT == 1 && cnu) { nuc = (float)cnu[c]; dtc = (float)cdt[c]; }
#pragma unroll
    for (int a = 0; a < N; ++a) {
        const long long o = base + (long long)a * stride;
        if constexpr (OUT == 0) {
            out[o] = cmulf(x[a], fac.post[a]);
        } else {
            // RK4 node-value stages (C:831-862); per-cell nu and dt when given.
            const float sr = x[a].x * fac.post[a].x - x[a].y * fac.post[a].y;
            if (stage == 0) {
                qn[o] = sr;
                f1[o] = f[o] + dtc * sr * nuc;
            } else {
                f1[o] = f[o] + 0.5f * dtc * qn[o] * nuc + 0.5f * dtc * sr * nuc;
            }
        }
    }
}

// One RK4 node-value stage across the last inverse pass and the first
// forward pass, both along axis 0, as register FFTs, one thread per (pencil,
// cell): the inverse gives the stage's Q at the nodes (its real part), the
// node value (stage 0: qn = Q, v = f + dt nu Q; stages 1, 2:
// v = f + dt nu qn / 2 + dt nu Q / 2, C:831-862) and its forward transform.
template <int N, int PY>
__global__ void __launch_bounds__(32 * PY) k_fftf_fs(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                     const __grid_constant__ DftFac fi,
                                                     const __grid_constant__ DftFac ff, int Bp, int stage, float dt,
                                                     float nu, const float *__restrict__ f, float *__restrict__ qn,
                                                     const double *__restrict__ cnu, const double *__restrict__ cdt) {
    lp_grid_wait();
    const int pid = blockIdx.x * PY + threadIdx.y;
    if (pid >= N * N) return;
    const int c = blockIdx.y * 32 + threadIdx.x;
    const long long stride = (long long)N * N * Bp, base = (long long)pid * Bp + c;
    float2 x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = cmulf(in[base + i * stride], fi.pre[i]);
    fft_reg<N, 1>(x, fi.w);
    float dtc = dt, nuc = nu;
    if (cnu) { nuc = (float)cnu[c]; dtc = (float)cdt[c]; }
#pragma unroll
    for (int a = 0; a < N; ++a) {
        const long long o = base + (long long)a * stride;
        const float sr = x[a].x * fi.post[a].x - x[a].y * fi.post[a].y;
        float v;
        if (stage == 0) {
            qn[o] = sr;
            v = f[o] + dtc * sr * nuc;
        } else {
            v = f[o] + 0.5f * dtc * qn[o] * nuc + 0.5f * dtc * sr * nuc;
        }
        x[a] = make_float2(v * ff.pre[a].x, v * ff.pre[a].y);
    }
    fft_reg<N, -1>(x, ff.w);
#pragma unroll
    for (int a = 0; a < N; ++a) out[base + (long long)a * stride] = cmulf(x[a], ff.post[a]);
}

// The two slow axes of a transform through one (axis-0, axis-1) plane in
// shared memory: a block holds the plane of one axis-2 index for CB cells
// (rows of N CB values padded by 8 so that both pencil directions read
// conflict-free), one thread per (pencil, cell).
// STAGE: one RK4 node-value stage, from the axis-2 inverse output to the
// axis-2 forward input: axis-1 inverse FFT, axis-0 inverse FFT with the
// stage update (as k_fftf_fs) and axis-0 forward FFT, axis-1 forward FFT.
// !STAGE: the forward transform's axis-1 and axis-0 passes.
template <int N, int CB, bool STAGE>
__global__ void __launch_bounds__(CB * N) k_fftf_plane(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                       const __grid_constant__ DftFac fi,
                                                       const __grid_constant__ DftFac ff, int Bp, int stage,
                                                       float dt, float nu, const float *__restrict__ f,
                                                       float *__restrict__ qn, const double *__restrict__ cnu,
                                                       const double *__restrict__ cdt) {
    lp_grid_wait();
    constexpr int RS = N * CB + 8;  // row stride (float2) of the plane
    __shared__ float2 pl[N * RS];
    const int c = threadIdx.x, p = threadIdx.y, i2 = blockIdx.x, cb = blockIdx.y * CB;
    const long long s1 = (long long)N * Bp, s0 = (long long)N * N * Bp;
    const long long gcell = (long long)i2 * Bp + cb + c;
    // stage inputs of the axis-0 pencil (i1 = p) of this thread, fetched early
    float fv[N], qv[N];
    float dtc = dt, nuc = nu;
    if constexpr (STAGE) {
#pragma unroll
        for (int i0 = 0; i0 < N; ++i0) {
            const long long o = i0 * s0 + p * s1 + gcell;
            fv[i0] = f[o];
            qv[i0] = stage == 0 ? 0.f : qn[o];
        }
        if (cnu) { nuc = (float)cnu[cb + c]; dtc = (float)cdt[cb + c]; }
    }
    float2 x[N];
    // axis 1: the pencil (i0 = p, ., i2)
#pragma unroll
    for (int i1 = 0; i1 < N; ++i1) x[i1] = in[p * s0 + i1 * s1 + gcell];
    if constexpr (STAGE) {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = cmulf(x[i], fi.pre[i]);
        fft_reg<N, 1>(x, fi.w);
#pragma unroll
        for (int a = 0; a < N; ++a) x[a] = cmulf(x[a], fi.post[a]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = cmulf(x[i], ff.pre[i]);
        fft_reg<N, -1>(x, ff.w);
#pragma unroll
        for (int a = 0; a < N; ++a) x[a] = cmulf(x[a], ff.post[a]);
    }
#pragma unroll
    for (int i1 = 0; i1 < N; ++i1) pl[p * RS + i1 * CB + c] = x[i1];
    __syncthreads();
    // axis 0: the pencil (., i1 = p, i2)
#pragma unroll
    for (int i0 = 0; i0 < N; ++i0) x[i0] = pl[i0 * RS + p * CB + c];
    if constexpr (STAGE) {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = cmulf(x[i], fi.pre[i]);
        fft_reg<N, 1>(x, fi.w);
#pragma unroll
        for (int a = 0; a < N; ++a) {
            const float sr = x[a].x * fi.post[a].x - x[a].y * fi.post[a].y;
            float v;
            if (stage == 0) {
                qn[a * s0 + p * s1 + gcell] = sr;
                v = fv[a] + dtc * sr * nuc;
            } else {
                v = fv[a] + 0.5f * dtc * qv[a] * nuc + 0.5f * dtc * sr * nuc;
            }
            x[a] = make_float2(v * ff.pre[a].x, v * ff.pre[a].y);
        }
        fft_reg<N, -1>(x, ff.w);
#pragma unroll
        for (int a = 0; a < N; ++a) pl[a * RS + p * CB + c] = cmulf(x[a], ff.post[a]);
        __syncthreads();
        // axis 1 forward: the pencil (i0 = p, ., i2)
#pragma unroll
        for (int i1 = 0; i1 < N; ++i1) x[i1] = cmulf(pl[p * RS + i1 * CB + c], ff.pre[i1]);
        fft_reg<N, -1>(x, ff.w);
#pragma unroll
        for (int a = 0; a < N; ++a) out[p * s0 + a * s1 + gcell] = cmulf(x[a], ff.post[a]);
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = cmulf(x[i], ff.pre[i]);
        fft_reg<N, -1>(x, ff.w);
#pragma unroll
        for (int a = 0; a < N; ++a) out[a * s0 + p * s1 + gcell] = cmulf(x[a], ff.post[a]);
    }
}

template <int N, bool STAGE>
cudaError_t plane_launch(const float2 *in, float2 *out, const DftFac &fi, const DftFac &ff, int Bp, int stage,
                         double dt, double nu, const float *f, float *qn, cudaStream_t st, Rates rates) {
    constexpr int CB = 8;
    k_fftf_plane<N, CB, STAGE><<<dim3(N, Bp / CB), dim3(CB, N), 0, st>>>(in, out, fi, ff, Bp, stage, (float)dt,
                                                                         (float)nu, f, qn, rates.nu, rates.dt);
    return cudaGetLastError();
}

template <typename TIn, int OUT, int N>
cudaError_t fft_launch(const TIn *in, float2 *out, const DftFac &fac, int ax, int Bp, int stage, double dt,
                       double nu, const float *f, float *qn, float *f1, cudaStream_t st, Rates rates,
                       const float *cf, const double *lamc) {
    constexpr int PY = 4;
    dim3 grid((N * N + PY - 1) / PY, Bp / 32), block(32, PY);
    if (fac.sign < 0)
        k_fftf<TIn, OUT, N, -1, PY><<<grid, block, 0, st>>>(in, out, fac, ax, Bp, stage, (float)dt, (float)nu, f, qn,
                                                             f1, rates.nu, rates.dt, cf, lamc);
    else
        k_fftf<TIn, OUT, N, 1, PY><<<grid, block, 0, st>>>(in, out, fac, ax, Bp, stage, (float)dt, (float)nu, f, qn,
                                                            f1, rates.nu, rates.dt, cf, lamc);
    return cudaGetLastError();
}

template <typename R, typename TIn, int OUT, int N>
cudaError_t dftp_launch(const TIn *in, typename V2<R>::t *out, const R *M, int ax, int Bp, int stage, double dt,
                        double nu, const R *f, R *qn, R *f1, cudaStream_t st, Rates rates,
                        const float *cf = nullptr, const double *lamc = nullptr) {
    constexpr int PY = 2, OG = 4;
    if (cf && ax != 2) return cudaErrorInvalidValue;
    dim3 grid((N * N + PY - 1) / PY, Bp / 32), block(32, PY * OG);
    k_dftp<R, TIn, OUT, N, PY, OG><<<grid, block, 0, st>>>(in, out, M, ax, Bp, stage, (R)dt, (R)nu, f, qn, f1,
                                                           rates.nu, rates.dt, cf, lamc);
    return cudaGetLastError();
}

template <typename R, typename TIn, int OUT>
cudaError_t dft_pass(const TIn *in, typename V2<R>::t *out, const R *M, int n, int ax, int Bp, int stage,
                     double dt, double nu, const R *f, R *qn, R *f1, cudaStream_t st, Rates rates = Rates{},
                     const float *cf = nullptr, const double *lamc = nullptr, const DftFac *fac = nullptr) {
    using C = typename V2<R>::t;
    if constexpr (std::is_same<R, float>::value) {
        if (fac && fac->n == n) {
            if (cf && ax != 2) return cudaErrorInvalidValue;
            switch (n) {
            case 8: return fft_launch<TIn, OUT, 8>(in, out, *fac, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
            case 16: return fft_launch<TIn, OUT, 16>(in, out, *fac, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
            case 24: return fft_launch<TIn, OUT, 24>(in, out, *fac, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
            case 32: return fft_launch<TIn, OUT, 32>(in, out, *fac, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
            default: break;
            }
        }
    }
    switch (n) {
    case 8: return dftp_launch<R, TIn, OUT, 8>(in, out, M, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
    case 16: return dftp_launch<R, TIn, OUT, 16>(in, out, M, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
    case 24: return dftp_launch<R, TIn, OUT, 24>(in, out, M, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
    case 32: return dftp_launch<R, TIn, OUT, 32>(in, out, M, ax, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc);
    default: break;
    }
    if (cf) return cudaErrorInvalidValue;  // lazy conservation needs the register-pencil pass
    const size_t smem = sizeof(C) * (size_t)(n * n + 2 * 32 * n);
    dim3 grid((n * n + kDftPencils - 1) / kDftPencils, Bp / 32), block(32, n);
    k_dft<R, TIn, OUT><<<grid, block, smem, st>>>(in, out, M, n, ax, Bp, stage, (R)dt, (R)nu, f, qn, f1, rates.nu,
                                                  rates.dt);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- ComputeQ
// q(xi)[c] = sum over the pairs of xi of P * F(omega)[c] * F(u)[c]
// (C:739-822 with the two terms of each symmetric pair folded).  One warp per
// xi, lanes are cells; pair weights and packed indices are broadcast by
// shuffle from a coalesced load of 32 pairs.  Products accumulate in R over
// a chunk of 32 pairs, chunk sums in FP64.
template <typename R>
__global__ void __launch_bounds__(128) k_computeq(const typename V2<R>::t *__restrict__ F,
                                                  const R *__restrict__ P, const unsigned *__restrict__ PI,
                                                  const int *__restrict__ pair_off, int n3, int Bp,
                                                  double2 *__restrict__ q) {
    lp_grid_wait();
    using C = typename V2<R>::t;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int xi = blockIdx.x * 4 + warp;
    if (xi >= n3) return;
    const int c = blockIdx.y * 32 + lane;
    const int off = pair_off[xi], npair = pair_off[xi + 1] - off;
    const C *Fc = F + c;
    double ar = 0.0, ai = 0.0;
    for (int base = 0; base < npair; base += 32) {
        const int idx = base + lane;
        R pw = R(0);
        unsigned pk = 0u;
        if (idx < npair) { pw = P[off + idx]; pk = PI[off + idx]; }
        const int cnt = min(32, npair - base);
        R cr = R(0), ci = R(0);
#pragma unroll 4
        for (int s = 0; s < cnt; ++s) {
            const R ps = __shfl_sync(FULL, pw, s);
            const unsigned pks = __shfl_sync(FULL, pk, s);
            const C a = Fc[(long long)(pks & 0xffffu) * Bp];
            const C b = Fc[(long long)(pks >> 16) * Bp];
            const R pr = a.x * b.x - a.y * b.y;
            const R pim = a.x * b.y + a.y * b.x;
            cr = fma(ps, pr, cr);
            ci = fma(ps, pim, ci);
        }
        ar += (double)cr;
        ai += (double)ci;
    }
    q[(long long)xi * Bp + c] = make_double2(ar, ai);
}

// ---------------------------------------------------------------- line-tiled contraction
// For output xi = (i, j, k) the window of omega = (l, m, k') is a box; the
// planes (l, m) pair up under (l, m) -> (i+h-l, j+h-m) and, inside a pair,
// term (l, m, k') of one plane and term (i+h-l, j+h-m, k+h-k') of the other
// multiply the same product A(k') B(k+h-k') with A = F(l, m, .),
// B = F(i+h-l, j+h-m, .).  The weight table holds, per (line, plane pair,
// k-tile), the combined weights in (k, k') order, padded to 4 floats.
template <int N> __host__ __device__ constexpr int wlo(int k) { return k < N / 2 ? 0 : k - N / 2 + 1; }
template <int N> __host__ __device__ constexpr int whi(int k) { return k < N / 2 ? k + N / 2 + 1 : N; }
template <int N> __host__ __device__ constexpr int span_terms(int k0, int k1) {
    int s = 0;
    for (int k = k0; k < k1; ++k) s += whi<N>(k) - wlo<N>(k);
    return s;
}
__host__ __device__ constexpr int pad4(int x) { return (x + 3) & ~3; }
// floats of one tile's weights per plane pair, padded to 16 bytes
template <int N> __host__ __device__ constexpr int tile_floats(int k0, int k1) { return pad4(span_terms<N>(k0, k1)); }
template <int N, int KT> __host__ __device__ constexpr int tile_off(int t) {
    int s = 0;
    for (int u = 0; u < t; ++u) s += tile_floats<N>(u * KT, (u + 1) * KT);
    return s;
}
template <int N, int KT> __host__ __device__ constexpr int pp_floats() { return tile_off<N, KT>(N / KT); }
// Inside a tile the terms are stored k'-major (then k), so consecutive terms
// feed different accumulators: k' = n pairs with k in [n - N/2, n + N/2 - 1].
template <int N> __host__ __device__ constexpr int klo_of(int n, int K0) { return n - N / 2 > K0 ? n - N / 2 : K0; }
template <int N> __host__ __device__ constexpr int khi_of(int n, int K1) { return n + N / 2 - 1 < K1 - 1 ? n + N / 2 - 1 : K1 - 1; }
template <int N> __host__ __device__ constexpr int nmaj_before(int n, int K0, int K1) {
    int s = 0;
    for (int nn = 0; nn < n; ++nn) {
        const int c = khi_of<N>(nn, K1) - klo_of<N>(nn, K0) + 1;
        s += c > 0 ? c : 0;
    }
    return s;
}

template <int N> struct LinesCfg;
template <> struct LinesCfg<8> { static constexpr int KT = 8; };
template <> struct LinesCfg<16> { static constexpr int KT = 8; };
template <> struct LinesCfg<24> { static constexpr int KT = 12; };
template <> struct LinesCfg<32> { static constexpr int KT = 8; };

__device__ __forceinline__ float pick4(const float4 &v, int r) { return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w)); }


// One k-tile of output lines.  The LW warps of a block take the
// plane pairs of the same (line, tile, 32 cells) in turn; each warp stages
// the plane pair's two F lines in shared memory with cp.async (one buffer:
// every lane copies and reads only its own cell's column, and the copy of
// the next plane pair is issued when the current one has been consumed, its
// latency hidden by the other resident warps) and its weights (double
// buffered: the next plane pair's weights are copied during the computation).  Per plane pair, with a = A(k'), b = B(k+h-k') and
// weight w: U += (w a) (bx, by) and V += (w a) (by, bx) in packed FP32x2, so
// Re = U.x - U.y, Im = V.x + V.y; each plane pair's partials enter a
// Kahan-compensated FP32 accumulator, and the warps' results are summed in
// FP64 in a fixed order.
template <int N, int TILE, int LW>
__global__ void __launch_bounds__(32 * LW, 12 / LW) k_cq_lines(const float2 *__restrict__ F, const float *__restrict__ W,
                                                            const long long *__restrict__ line_off, int Bp,
                                                            double2 *__restrict__ q) {
    lp_grid_wait();
    constexpr int KT = LinesCfg<N>::KT, h = N / 2, K0 = TILE * KT;
    constexpr int TP = pp_floats<N, KT>(), TOFF = tile_off<N, KT>(TILE);
    constexpr int TT = tile_floats<N>(K0, K0 + KT);  // weight floats of this tile per plane pair
    extern __shared__ __align__(16) unsigned char lines_smem[];
    // per warp: [2 lines][N][32 lanes] float2; then per warp [2 buffers][TT]
    // weights; the reduction area reuses the space after the loop
    float2 *stage = reinterpret_cast<float2 *>(lines_smem);
    float *wstage = reinterpret_cast<float *>(lines_smem + sizeof(float2) * 2 * N * 32 * LW);
    double2 *red = reinterpret_cast<double2 *>(lines_smem);  // reuses the staging area after the loop
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *mybuf = stage + (long long)warp * 2 * N * 32;
    float *mywbuf = wstage + warp * 2 * TT;
    const int G = Bp / 32;
    // line_off holds N^2 + 1 weight offsets, then the lines longest first
    const int g = (int)(blockIdx.x % G), ij = (int)line_off[N * N + 1 + blockIdx.x / G];
    const int i = ij / N, j = ij % N;
    const int si = i < h ? 0 : i - h + 1, ni = i < h ? i + h + 1 : 3 * h - 1 - i;
    const int sj = j < h ? 0 : j - h + 1, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
    const int npp = (ni * nj + 1) / 2;
    const int c = g * 32 + lane;
    const float *wbase = W + line_off[ij] + TOFF;
    auto stage_lines = [&](int pp) {
        const int l = si + pp / nj, m = sj + pp % nj;
        const int x = i + h - l, y = j + h - m;
        const float2 *Al = F + (long long)((l * N + m) * N) * Bp + c;
        const float2 *Bl = F + (long long)((x * N + y) * N) * Bp + c;
        float2 *dA = mybuf + lane;
        float2 *dB = mybuf + N * 32 + lane;
#pragma unroll 4
        for (int n = 0; n < N; ++n) {
            cp_async8(dA + n * 32, Al + (long long)n * Bp);
            cp_async8(dB + n * 32, Bl + (long long)n * Bp);
        }
    };
    auto stage_w = [&](int pp, int buf) {
        const float *ws = wbase + (long long)pp * TP;
        float *wd = mywbuf + buf * TT;
        for (int q4 = lane; q4 < TT / 4; q4 += 32) cp_async16(wd + 4 * q4, ws + 4 * q4);
    };
    float sr[KT], sim[KT], cr[KT], ci[KT];
    unsigned long long U[KT], V[KT];
#pragma unroll
    for (int kk = 0; kk < KT; ++kk) { sr[kk] = 0.f; sim[kk] = 0.f; cr[kk] = 0.f; ci[kk] = 0.f; U[kk] = 0ull; V[kk] = 0ull; }
    if (warp < npp) {
        stage_lines(warp);
        stage_w(warp, 0);
    }
    cp_async_commit();
    int it = 0;
    for (int pp = warp; pp < npp; pp += LW, ++it) {
        const int nxt = pp + LW;
        cp_async_wait0();
        __syncwarp();
        // (issued before the line reads: the copy instructions order the
        // compiler's memory accesses, and the reads should sink to their uses)
        if (nxt < npp) stage_w(nxt, (it + 1) & 1);
        cp_async_commit();
        const float2 *sA = mybuf + lane;
        const float2 *sB = mybuf + N * 32 + lane;
        const float *wp = mywbuf + (it & 1) * TT;
        unsigned long long A[N], B[N], Bs[N];
#pragma unroll
        for (int n = 0; n < N; ++n) {
            const float2 a = sA[n * 32], b = sB[n * 32];
            A[n] = pk2(a.x, a.y);
            B[n] = pk2(b.x, b.y);
            Bs[n] = pk2(b.y, b.x);
        }
        float4 w4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int n = 0; n < N; ++n) {
#pragma unroll
            for (int k = klo_of<N>(n, K0); k <= khi_of<N>(n, K0 + KT); ++k) {
                const int t = nmaj_before<N>(n, K0, K0 + KT) + k - klo_of<N>(n, K0);
                if ((t & 3) == 0) w4 = *reinterpret_cast<const float4 *>(wp + t);
                const float wt = pick4(w4, t & 3);
                const unsigned long long wa = mul2(pk2(wt, wt), A[n]);
                U[k - K0] = fma2(wa, B[k + h - n], U[k - K0]);
                V[k - K0] = fma2(wa, Bs[k + h - n], V[k - K0]);
            }
        }
        // each plane pair's packed partials enter the Kahan sums (folding two
        // plane pairs per update measured no faster)
#pragma unroll
        for (int kk = 0; kk < KT; ++kk) {
            const float2 u2 = up2(U[kk]), v2 = up2(V[kk]);
            const float pr = u2.x - u2.y, pm = v2.x + v2.y;
            float yr = pr - cr[kk], tr = sr[kk] + yr;  // Kahan: s + (p - c)
            cr[kk] = (tr - sr[kk]) - yr; sr[kk] = tr;
            float yi = pm - ci[kk], ti = sim[kk] + yi;
            ci[kk] = (ti - sim[kk]) - yi; sim[kk] = ti;
            U[kk] = 0ull; V[kk] = 0ull;
        }
        __syncwarp();  // every lane is done with this plane pair's lines and weights
        if (nxt < npp) stage_lines(nxt);
        cp_async_commit();
    }
    cp_async_wait0();
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KT; ++kk)
        red[(warp * KT + kk) * 32 + lane] = make_double2((double)sr[kk] - (double)cr[kk], (double)sim[kk] - (double)ci[kk]);
    __syncthreads();
    for (int kk = warp; kk < KT; kk += LW) {
        double2 acc = red[kk * 32 + lane];
#pragma unroll
        for (int w = 1; w < LW; ++w) {
            const double2 v = red[(w * KT + kk) * 32 + lane];
            acc.x += v.x; acc.y += v.y;
        }
        q[(long long)((i * N + j) * N + K0 + kk) * Bp + c] = acc;
    }
}

template <int N, int T, int LW> constexpr size_t lines_smem_bytes() {
    constexpr int KT = LinesCfg<N>::KT;
    constexpr size_t staging = sizeof(float2) * 2 * N * 32 * LW +
                               sizeof(float) * 2 * tile_floats<N>(T * KT, T * KT + KT) * LW;
    constexpr size_t reduction = sizeof(double2) * LW * KT * 32;
    return staging > reduction ? staging : reduction;
}

template <int N>
__global__ void k_lines_table(const double *__restrict__ eta, const double *__restrict__ shat,
                              const double *__restrict__ ahat, const unsigned char *__restrict__ rzero,
                              const double *__restrict__ cw, const long long *__restrict__ line_off,
                              float *__restrict__ W) {
    lp_grid_wait();
    constexpr int KT = LinesCfg<N>::KT, NT = N / KT, h = N / 2, TP = pp_floats<N, KT>();
    const int ij = blockIdx.x, i = ij / N, j = ij % N;
    const int si = i < h ? 0 : i - h + 1, ni = i < h ? i + h + 1 : 3 * h - 1 - i;
    const int sj = j < h ? 0 : j - h + 1, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
    const int cntp = ni * nj, npp = (cntp + 1) / 2;
    float *out = W + line_off[ij];
    for (int idx = threadIdx.x; idx < npp * TP; idx += blockDim.x) {
        const int pp = idx / TP;
        int t = idx % TP;  // float offset inside the plane pair's block
        // locate (tile, k, k') of slot t
        int tile = 0;
        while (tile + 1 < NT && t >= tile_off<N, KT>(tile + 1)) ++tile;
        t -= tile_off<N, KT>(tile);  // term index inside the tile
        const int K0 = tile * KT, K1 = K0 + KT;
        int k = -1, kp = -1;
        for (int nn = 0; nn < N; ++nn) {
            const int lo = klo_of<N>(nn, K0), hi = khi_of<N>(nn, K1);
            const int cnt = hi - lo + 1 > 0 ? hi - lo + 1 : 0;
            if (t < cnt) { kp = nn; k = lo + t; break; }
            t -= cnt;
        }
        if (kp < 0) { out[idx] = 0.f; continue; }  // padding
        const int l = si + pp / nj, m = sj + pp % nj;
        const int x = i + h - l, y = j + h - m;
        const int xi_ = (i * N + j) * N + k;
        const int om = (l * N + m) * N + kp, uu = (x * N + y) * N + (k + h - kp);
        double wv = __dmul_rn(cw[om], weight_dev(eta, shat, ahat, rzero, N, i, j, k, om));
        if (2 * pp != cntp - 1) wv = __dadd_rn(wv, __dmul_rn(cw[uu], weight_dev(eta, shat, ahat, rzero, N, i, j, k, uu)));
        (void)xi_;
        out[idx] = (float)wv;
    }
}

// ---------------------------------------------------------------- conserve
// conserveAllMoments (K:100-129): t = C q (5 dot products), lam = (CC^T)^-1 t,
// q -= C^T lam.  Partial sums per chunk of points, then per cell.
template <typename QT>
__global__ void k_cons_partial(const QT *__restrict__ q, const double *__restrict__ c1,
                               const double *__restrict__ c2, int n3, int Bp, int nchunk,
                               double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[8][5][32];
    const int cl = threadIdx.x, y = threadIdx.y, c = blockIdx.y * 32 + cl, k = blockIdx.x;
    const int cs = (n3 + nchunk - 1) / nchunk, p0 = k * cs, p1 = min(n3, p0 + cs);
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0;
#pragma unroll 4
    for (int pt = p0 + y; pt < p1; pt += 8) {
        const QT w = q[(long long)pt * Bp + c];
        double2 v;
        if constexpr (std::is_same<QT, float2>::value)  // exact for normal numbers, off the FP64 pipe
            v = make_double2(f32_to_f64_bits(w.x), f32_to_f64_bits(w.y));
        else
            v = make_double2((double)w.x, (double)w.y);
        t0 += v.x * c1[pt];
        t1 += v.y * c2[n3 + pt];
        t2 += v.y * c2[2 * n3 + pt];
        t3 += v.y * c2[3 * n3 + pt];
        t4 += v.x * c1[4 * n3 + pt];
    }
    red[y][0][cl] = t0; red[y][1][cl] = t1; red[y][2][cl] = t2; red[y][3][cl] = t3; red[y][4][cl] = t4;
    __syncthreads();
    if (y < 5) {
        double s = 0;
        for (int yy = 0; yy < 8; ++yy) s += red[yy][y][cl];
        part[((long long)k * 5 + y) * Bp + c] = s;
    }
}

// One block of five warps per cell: warp j sums the chunk partials of
// constraint j (each lane a fixed strided subset, then a fixed butterfly of
// shuffles), and threads 0..4 form lambda_i = sum_j (C C^T)^-1[j + 5 i] t_j
// (solveWithCCt, K:49-55).  The FP64 dependency chains stay short: GB300's
// FP64 unit is narrow, and a block-wide tree with one thread solving the 5x5
// system spent most of its time waiting on FP64 results.
__global__ void __launch_bounds__(160) k_cons_lambda(const double *__restrict__ part, int nchunk,
                                                     const double *__restrict__ cct, int Bp,
                                                     double *__restrict__ lam) {
    lp_grid_wait();
    __shared__ double t5[5];
    const int c = blockIdx.x, lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    double v = 0.;
    for (int k = lane; k < nchunk; k += 32) v += part[((long long)k * 5 + j) * Bp + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) t5[j] = v;
    __syncthreads();
    if (threadIdx.x < 5) {
        const int i = threadIdx.x;
        double s = 0.;
#pragma unroll
        for (int q = 0; q < 5; ++q) s += cct[q + i * 5] * t5[q];
        lam[(long long)i * Bp + c] = s;
    }
}

__global__ void k_cons_apply(double2 *__restrict__ q, const double *__restrict__ c1,
                             const double *__restrict__ c2, const double *__restrict__ lam, int n3, int Bp) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)n3 * Bp) return;
    const int c = (int)(tid % Bp), pt = (int)(tid / Bp);
    const double l0 = lam[c], l1 = lam[Bp + c], l2 = lam[2 * Bp + c], l3 = lam[3 * Bp + c], l4 = lam[4 * Bp + c];
    double2 v = q[tid];
    v.x -= (c1[pt] * l0 + c1[4 * n3 + pt] * l4);
    v.y -= (c2[n3 + pt] * l1 + c2[2 * n3 + pt] * l2 + c2[3 * n3 + pt] * l3);
    q[tid] = v;
}

// ---------------------------------------------------------------- projection
// Qc = nu (q0/2 + (q1 + q2 + q3)/6) (C:878-879), the non-classical RK4
// combination of the reference (kept as specified).
template <typename R>
__global__ void k_qcomb(const double2 *__restrict__ q0, const double2 *__restrict__ q1,
                        const double2 *__restrict__ q2, const double2 *__restrict__ q3, double nu,
                        long long total, int Bp, const double *__restrict__ cnu,
                        typename V2<R>::t *__restrict__ Qc) {
    lp_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= total) return;
    if (cnu) nu = cnu[tid % Bp];
    const double2 a = q0[tid], b = q1[tid], d = q2[tid], e = q3[tid];
    constexpr double sixth = 1. / 6.;
    const double re = nu * (0.5 * a.x + (b.x + d.x + e.x) * sixth);
    const double im = nu * (0.5 * a.y + (b.y + d.y + e.y) * sixth);
    Qc[tid] = mk2<R>((R)re, (R)im);
}

// tp_l(j) = Re sum_k IntModes_l(k, j) Qc(k) (C:867-889) evaluated as three
// per-axis contractions with the factors T0, T1, T2 of IntModes (C:364-505).
// Each thread owns a chunk of JB output indices along the contracted axis,
// so every input element is read once per chunk.
constexpr int JB = 8;

template <typename R>
__global__ void k_proj3(const typename V2<R>::t *__restrict__ Qc, const R *__restrict__ tf, int n, int nv,
                        int Bp, typename V2<R>::t *__restrict__ Y) {
    lp_grid_wait();
    const int nch = (nv + JB - 1) / JB;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)n * n * nch * Bp;
    if (tid >= total) return;
    const int c = (int)(tid % Bp);
    long long r = tid / Bp;
    const int ch = (int)(r % nch); r /= nch;
    const int k2 = (int)(r % n), k1 = (int)(r / n);
    const int j0 = ch * JB;
    R s[3][JB][2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int jj = 0; jj < JB; ++jj) { s[a][jj][0] = 0; s[a][jj][1] = 0; }
    const long long qb = ((long long)(k1 * n + k2) * n) * Bp + c;
    for (int k3 = 0; k3 < n; ++k3) {
        const typename V2<R>::t x = Qc[qb + (long long)k3 * Bp];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int jj = 0; jj < JB; ++jj) {
                if (j0 + jj < nv) {
                    const R *t = tf + 2 * ((a * n + k3) * nv + j0 + jj);
                    s[a][jj][0] += t[0] * x.x - t[1] * x.y;
                    s[a][jj][1] += t[0] * x.y + t[1] * x.x;
                }
            }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int jj = 0; jj < JB; ++jj)
            if (j0 + jj < nv)
                Y[((((long long)a * n + k1) * n + k2) * nv + j0 + jj) * Bp + c] = mk2<R>(s[a][jj][0], s[a][jj][1]);
}

template <typename R>
__global__ void k_proj2(const typename V2<R>::t *__restrict__ Y, const R *__restrict__ tf, int n, int nv,
                        int Bp, typename V2<R>::t *__restrict__ Z) {
    lp_grid_wait();
    const int nch = (nv + JB - 1) / JB;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)n * nv * nch * Bp;
    if (tid >= total) return;
    const int c = (int)(tid % Bp);
    long long r = tid / Bp;
    const int j3 = (int)(r % nv); r /= nv;
    const int ch = (int)(r % nch), k1 = (int)(r / nch);
    const int j0 = ch * JB;
    // Z[p] with (axis-3 factor, axis-2 factor) = (0,0) (0,1) (0,2) (1,0) (2,0)
    R s[5][JB][2];
#pragma unroll
    for (int p = 0; p < 5; ++p)
#pragma unroll
        for (int jj = 0; jj < JB; ++jj) { s[p][jj][0] = 0; s[p][jj][1] = 0; }
    for (int k2 = 0; k2 < n; ++k2) {
        typename V2<R>::t y[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) y[a] = Y[((((long long)a * n + k1) * n + k2) * nv + j3) * Bp + c];
#pragma unroll
        for (int jj = 0; jj < JB; ++jj) {
            if (j0 + jj < nv) {
                const int j2 = j0 + jj;
                const R *t0 = tf + 2 * ((0 * n + k2) * nv + j2);
                const R *t1 = tf + 2 * ((1 * n + k2) * nv + j2);
                const R *t2 = tf + 2 * ((2 * n + k2) * nv + j2);
                s[0][jj][0] += t0[0] * y[0].x - t0[1] * y[0].y; s[0][jj][1] += t0[0] * y[0].y + t0[1] * y[0].x;
                s[1][jj][0] += t1[0] * y[0].x - t1[1] * y[0].y; s[1][jj][1] += t1[0] * y[0].y + t1[1] * y[0].x;
                s[2][jj][0] += t2[0] * y[0].x - t2[1] * y[0].y; s[2][jj][1] += t2[0] * y[0].y + t2[1] * y[0].x;
                s[3][jj][0] += t0[0] * y[1].x - t0[1] * y[1].y; s[3][jj][1] += t0[0] * y[1].y + t0[1] * y[1].x;
                s[4][jj][0] += t0[0] * y[2].x - t0[1] * y[2].y; s[4][jj][1] += t0[0] * y[2].y + t0[1] * y[2].x;
            }
        }
    }
#pragma unroll
    for (int p = 0; p < 5; ++p)
#pragma unroll
        for (int jj = 0; jj < JB; ++jj)
            if (j0 + jj < nv)
                Z[((((long long)p * n + k1) * nv + j0 + jj) * nv + j3) * Bp + c] = mk2<R>(s[p][jj][0], s[p][jj][1]);
}

// Last contraction, the mass-matrix inverse on {phi0, phi6} and the RK4
// update of the 5 collided coefficients (C:890-905).
template <typename R>
__global__ void k_proj1(const typename V2<R>::t *__restrict__ Z, const R *__restrict__ tf, int n, int nv,
                        int Bp, int B, int c0, const double *__restrict__ U, int ustride, int4 us, int us4,
                        double dt, double kfac, const double *__restrict__ cdt, double *__restrict__ dU) {
    lp_grid_wait();
    const int nch = (nv + JB - 1) / JB;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nv3 = (long long)nv * nv * nv;
    if (tid >= (long long)nv * nv * nch * Bp) return;
    const int c = (int)(tid % Bp);
    if (c >= B) return;
    if (cdt) dt = cdt[c];
    long long r = tid / Bp;
    const int j3 = (int)(r % nv); r /= nv;
    const int j2 = (int)(r % nv), ch = (int)(r / nv);
    const int j0 = ch * JB;
    // l=0: T0 on Z0; l=1: T1 on Z0; l=2: T0 on Z1; l=3: T0 on Z3; l=4: T2 on Z0 + T0 on Z2 + T0 on Z4
    R a[7][JB];
#pragma unroll
    for (int e = 0; e < 7; ++e)
#pragma unroll
        for (int jj = 0; jj < JB; ++jj) a[e][jj] = 0;
    const long long zs = (long long)n * nv * nv * Bp;
    for (int k1 = 0; k1 < n; ++k1) {
        const long long zb = (((long long)k1 * nv + j2) * nv + j3) * Bp + c;
        const typename V2<R>::t z0 = Z[zb], z1 = Z[zb + zs], z2 = Z[zb + 2 * zs], z3 = Z[zb + 3 * zs], z4 = Z[zb + 4 * zs];
#pragma unroll
        for (int jj = 0; jj < JB; ++jj) {
            if (j0 + jj < nv) {
                const int j1 = j0 + jj;
                const R *t0 = tf + 2 * ((0 * n + k1) * nv + j1);
                const R *t1 = tf + 2 * ((1 * n + k1) * nv + j1);
                const R *t2 = tf + 2 * ((2 * n + k1) * nv + j1);
                a[0][jj] += t0[0] * z0.x - t0[1] * z0.y;
                a[1][jj] += t1[0] * z0.x - t1[1] * z0.y;
                a[2][jj] += t0[0] * z1.x - t0[1] * z1.y;
                a[3][jj] += t0[0] * z3.x - t0[1] * z3.y;
                a[4][jj] += t2[0] * z0.x - t2[1] * z0.y;
                a[5][jj] += t0[0] * z2.x - t0[1] * z2.y;
                a[6][jj] += t0[0] * z4.x - t0[1] * z4.y;
            }
        }
    }
#pragma unroll
    for (int jj = 0; jj < JB; ++jj) {
        if (j0 + jj >= nv) continue;
        const long long kt = ((long long)(j0 + jj) * nv + j2) * nv + j3;
        const double tp0 = (double)a[0][jj], tp2 = (double)a[1][jj], tp3 = (double)a[2][jj], tp4 = (double)a[3][jj];
        const double tp5 = (double)a[4][jj] + (double)a[5][jj] + (double)a[6][jj];
        const double *u = U + (long long)ustride * ((long long)(c0 + c) * nv3 + kt);
        const double p0 = u[us.x] + u[us4] * 0.25 + dt * tp0 * kfac;
        const double p2 = u[us.y] + dt * tp2 * 12. * kfac;
        const double p3 = u[us.z] + dt * tp3 * 12. * kfac;
        const double p4 = u[us.w] + dt * tp4 * 12. * kfac;
        const double p5 = u[us.x] * 0.25 + u[us4] * (19. / 240.) + dt * tp5 * kfac;
        double *d = dU + 5 * ((long long)c * nv3 + kt);
        d[0] = 19 * p0 * 0.25 - 15 * p5;
        d[4] = 60 * p5 - 15 * p0;
        d[1] = p2; d[2] = p3; d[3] = p4;
    }
}

// ---------------------------------------------------------------- moments of the increment
// Mixed path: the 5 DG moments of each cell's collision increment are
// evaluated in FP64 directly from the FP64 mode array (target) and from the
// projected coefficients (actual); the minimal-norm correction
// delta_j = Phi_j^T lambda, lambda = Gm^-1 (target - actual), then makes the
// coefficients carry exactly the FP64 moments.
__global__ void k_mom_target(const double2 *__restrict__ q0, const double2 *__restrict__ q1,
                             const double2 *__restrict__ q2, const double2 *__restrict__ q3, double nu,
                             const double *__restrict__ cnu, const double *__restrict__ gmom, int n3, int Bp,
                             int nchunk, double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[8][5][32];
    const int cl = threadIdx.x, y = threadIdx.y, c = blockIdx.y * 32 + cl, k = blockIdx.x;
    if (cnu) nu = cnu[c];
    const int cs = (n3 + nchunk - 1) / nchunk, p0 = k * cs, p1 = min(n3, p0 + cs);
    double t[5] = {0, 0, 0, 0, 0};
    for (int pt = p0 + y; pt < p1; pt += 8) {
        const long long o = (long long)pt * Bp + c;
        const double2 a = q0[o], b = q1[o], d = q2[o], e = q3[o];
        const double re = nu * (0.5 * a.x + (b.x + d.x + e.x) * (1. / 6.));
        const double im = nu * (0.5 * a.y + (b.y + d.y + e.y) * (1. / 6.));
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const double *g = gmom + 2 * ((long long)m * n3 + pt);
            t[m] += g[0] * re - g[1] * im;
        }
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) red[y][m][cl] = t[m];
    __syncthreads();
    if (y < 5) {
        double s = 0;
        for (int yy = 0; yy < 8; ++yy) s += red[yy][y][cl];
        part[((long long)k * 5 + y) * Bp + c] = s;
    }
}

__device__ __forceinline__ void phi_row(double dv, double lv, int nv, long long kt, double G[3], double &g2) {
    const int j3 = (int)(kt % nv), j2 = (int)((kt / nv) % nv), j1 = (int)(kt / ((long long)nv * nv));
    G[0] = -lv + (j1 + 0.5) * dv;
    G[1] = -lv + (j2 + 0.5) * dv;
    G[2] = -lv + (j3 + 0.5) * dv;
    g2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
}

// dv/12, dv/6, dv^2/4 and 19 dv^2/240 of the DG moment rows, computed once on the host
struct MomRow {
    double dv12, dv6, dv2q, c19;
};
inline MomRow mom_row(double dv) { return MomRow{dv / 12., dv / 6., dv * dv / 4., 19. * dv * dv / 240.}; }

__global__ void k_mom_actual(const double *__restrict__ dU, const double *__restrict__ U, int nv, double dv,
                             double lv, MomRow mr, int c0, int nrc, double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[5][256];
    const int cc = blockIdx.y, t = threadIdx.x;
    const long long nv3 = (long long)nv * nv * nv;
    const long long cs = (nv3 + nrc - 1) / nrc, r0 = blockIdx.x * cs, r1 = min(nv3, r0 + cs);
    double m[5] = {0, 0, 0, 0, 0};
    for (long long kt = r0 + t; kt < r1; kt += 256) {
        const double *a = dU + 5 * ((long long)cc * nv3 + kt);
        const double *u = U + 7 * ((long long)(c0 + cc) * nv3 + kt);
        const double d0 = a[0] - u[0], d1 = a[1] - u[3], d2 = a[2] - u[4], d3 = a[3] - u[5], d4 = a[4] - u[6];
        double G[3], g2;
        phi_row(dv, lv, nv, kt, G, g2);
        m[0] += d0 + 0.25 * d4;
        m[1] += G[0] * d0 + mr.dv12 * d1 + 0.25 * G[0] * d4;
        m[2] += G[1] * d0 + mr.dv12 * d2 + 0.25 * G[1] * d4;
        m[3] += G[2] * d0 + mr.dv12 * d3 + 0.25 * G[2] * d4;
        m[4] += (g2 + mr.dv2q) * d0 + mr.dv6 * (G[0] * d1 + G[1] * d2 + G[2] * d3) + (mr.c19 + 0.25 * g2) * d4;
    }
    for (int q = 0; q < 5; ++q) red[q][t] = m[q];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int q = 0; q < 5; ++q) red[q][t] += red[q][t + w];
        __syncthreads();
    }
    if (t < 5) part[((long long)cc * nrc + blockIdx.x) * 5 + t] = red[t][0];
}

// The multipliers of each cell: lambda = Gm^-1 (scale target - actual), the
// actual moments summed from nk partials at apart[c sc + k sk + m sm].
__global__ void k_mom_lambda(const double *__restrict__ tpart, int nchunk, const double *__restrict__ apart,
                             int nk, long long sc, long long sk, long long sm, const double *__restrict__ gm_inv,
                             double scale, double kfac, const double *__restrict__ cdt, int B, int Bp,
                             double *__restrict__ lam) {
    lp_grid_wait();
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= B) return;
    if (cdt) scale = cdt[c] * kfac;
    double tg[5] = {0, 0, 0, 0, 0}, ac[5] = {0, 0, 0, 0, 0};
    if (tpart)  // nullptr: the target moments are zero
        for (int k = lane; k < nchunk; k += 32)
            for (int m = 0; m < 5; ++m) tg[m] += tpart[((long long)k * 5 + m) * Bp + c];
    for (int k = lane; k < nk; k += 32)
        for (int m = 0; m < 5; ++m) ac[m] += apart[c * sc + k * sk + m * sm];
    for (int off = 16; off > 0; off >>= 1)
        for (int m = 0; m < 5; ++m) {
            tg[m] += __shfl_down_sync(FULL, tg[m], off);
            ac[m] += __shfl_down_sync(FULL, ac[m], off);
        }
    if (lane == 0) {
        double r[5];
        for (int m = 0; m < 5; ++m) r[m] = scale * tg[m] - ac[m];
        for (int i = 0; i < 5; ++i) {
            double sum = 0;
            for (int j = 0; j < 5; ++j) sum += gm_inv[i * 5 + j] * r[j];
            lam[5 * c + i] = sum;
        }
    }
}

// delta = Phi^T lambda added to the 5 coefficients a of record kt
// (columns of Phi: a0, a1, a2, a3, a4)
__device__ __forceinline__ void mom_correct(double a[5], const double *l, double dv, double lv, int nv, long long kt,
                                            const MomRow &mr) {
    double G[3], g2;
    phi_row(dv, lv, nv, kt, G, g2);
    a[0] += l[0] + G[0] * l[1] + G[1] * l[2] + G[2] * l[3] + (g2 + mr.dv2q) * l[4];
    a[1] += mr.dv12 * l[1] + mr.dv6 * G[0] * l[4];
    a[2] += mr.dv12 * l[2] + mr.dv6 * G[1] * l[4];
    a[3] += mr.dv12 * l[3] + mr.dv6 * G[2] * l[4];
    a[4] += 0.25 * l[0] + 0.25 * (G[0] * l[1] + G[1] * l[2] + G[2] * l[3]) + (mr.c19 + 0.25 * g2) * l[4];
}

__global__ void k_mom_apply(double *__restrict__ dU, const double *__restrict__ lam, int nv, double dv, double lv,
                            MomRow mr, long long nrec) {
    lp_grid_wait();
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const long long nv3 = (long long)nv * nv * nv;
    double *a = dU + 5 * r;
    double v[5] = {a[0], a[1], a[2], a[3], a[4]};
    mom_correct(v, lam + 5 * (r / nv3), dv, lv, nv, r % nv3, mr);
    for (int q = 0; q < 5; ++q) a[q] = v[q];
}

// dU into slots {0,3,4,5,6} (LP_ompi_1.cpp:522-532), with the mixed path's
// moment correction Phi^T lambda applied on the way when lam is given.
__global__ void k_scatter(const double *__restrict__ dU, long long nrec, long long r0, double *__restrict__ U,
                          const double *__restrict__ lam, int nv, double dv, double lv, MomRow mr) {
    lp_grid_wait();
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const double *dd = dU + 5 * r;
    double d[5] = {dd[0], dd[1], dd[2], dd[3], dd[4]};
    if (lam) {
        const long long nv3 = (long long)nv * nv * nv;
        mom_correct(d, lam + 5 * (r / nv3), dv, lv, nv, r % nv3, mr);
    }
    double *u = U + 7 * (r0 + r);
    u[0] = d[0]; u[6] = d[4]; u[3] = d[1]; u[4] = d[2]; u[5] = d[3];
}

// ---------------------------------------------------------------- mixed tail
// Mixed path with LP_FIX_F1 fixed.  The mass-matrix inverse of the last
// projection step maps the old coefficients to themselves (its u-terms
// cancel), so the increment of the 5 collided coefficients of a record is
// dt kfac (19/4 tp0 - 15 tp5, 12 tp2, 12 tp3, 12 tp4, 60 tp5 - 15 tp0) and
// needs no state.  k_proj1_inc writes it cell-minor, Inc[kt][5][Bp], with
// per-block partial sums of its 5 DG moments (part[cell][5][blk]);
// k_scatter_inc adds increment and moment correction to U through a
// shared-memory transpose, so both sides of the copy are coalesced.
constexpr int kIncWarps = 4, JBI = 4;

__global__ void __launch_bounds__(32 * kIncWarps)
    k_proj1_inc(const float2 *__restrict__ Z, const float *__restrict__ tf, int n, int nv, int Bp, int B, double dt,
                double kfac, const double *__restrict__ cdt, double dv, double lv, MomRow mr,
                float *__restrict__ Inc, double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[kIncWarps][5][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int c = blockIdx.y * 32 + lane;
    const int nch = (nv + JBI - 1) / JBI, W = nv * nv * nch;
    const int it = blockIdx.x * kIncWarps + w;
    double m[5] = {0, 0, 0, 0, 0};
    if (it < W && c < B) {
        const int j3 = it % nv, j2 = (it / nv) % nv, ch = it / (nv * nv);
        const int j0 = ch * JBI;
        const double s = (cdt ? cdt[c] : dt) * kfac;
        float a[7][JBI];
#pragma unroll
        for (int e = 0; e < 7; ++e)
#pragma unroll
            for (int jj = 0; jj < JBI; ++jj) a[e][jj] = 0.f;
        const long long zs = (long long)n * nv * nv * Bp;
        for (int k1 = 0; k1 < n; ++k1) {
            const long long zb = (((long long)k1 * nv + j2) * nv + j3) * Bp + c;
            const float2 z0 = Z[zb], z1 = Z[zb + zs], z2 = Z[zb + 2 * zs], z3 = Z[zb + 3 * zs], z4 = Z[zb + 4 * zs];
#pragma unroll
            for (int jj = 0; jj < JBI; ++jj) {
                if (j0 + jj < nv) {
                    const int j1 = j0 + jj;
                    const float *t0 = tf + 2 * ((0 * n + k1) * nv + j1);
                    const float *t1 = tf + 2 * ((1 * n + k1) * nv + j1);
                    const float *t2 = tf + 2 * ((2 * n + k1) * nv + j1);
                    a[0][jj] += t0[0] * z0.x - t0[1] * z0.y;
                    a[1][jj] += t1[0] * z0.x - t1[1] * z0.y;
                    a[2][jj] += t0[0] * z1.x - t0[1] * z1.y;
                    a[3][jj] += t0[0] * z3.x - t0[1] * z3.y;
                    a[4][jj] += t2[0] * z0.x - t2[1] * z0.y;
                    a[5][jj] += t0[0] * z2.x - t0[1] * z2.y;
                    a[6][jj] += t0[0] * z4.x - t0[1] * z4.y;
                }
            }
        }
        const double G2 = -lv + (j2 + 0.5) * dv, G3 = -lv + (j3 + 0.5) * dv;
#pragma unroll
        for (int jj = 0; jj < JBI; ++jj) {
            if (j0 + jj >= nv) continue;
            const int j1 = j0 + jj;
            const long long kt = ((long long)j1 * nv + j2) * nv + j3;
            const double tp0 = a[0][jj], tp2 = a[1][jj], tp3 = a[2][jj], tp4 = a[3][jj];
            const double tp5 = (double)a[4][jj] + (double)a[5][jj] + (double)a[6][jj];
            // stored in FP32; the moments are those of the stored values
            const float f0 = (float)(s * (4.75 * tp0 - 15. * tp5)), f4 = (float)(s * (60. * tp5 - 15. * tp0));
            const float f1 = (float)(12. * s * tp2), f2 = (float)(12. * s * tp3), f3 = (float)(12. * s * tp4);
            float *o = Inc + kt * 5 * Bp + c;
            o[0] = f0; o[Bp] = f1; o[2 * Bp] = f2; o[3 * Bp] = f3; o[4 * Bp] = f4;
            const double d0 = f32_to_f64_bits(f0), d1 = f32_to_f64_bits(f1), d2 = f32_to_f64_bits(f2),
                         d3 = f32_to_f64_bits(f3), d4 = f32_to_f64_bits(f4);
            const double G1 = -lv + (j1 + 0.5) * dv, g2 = G1 * G1 + G2 * G2 + G3 * G3;
            m[0] += d0 + 0.25 * d4;
            m[1] += G1 * d0 + mr.dv12 * d1 + 0.25 * G1 * d4;
            m[2] += G2 * d0 + mr.dv12 * d2 + 0.25 * G2 * d4;
            m[3] += G3 * d0 + mr.dv12 * d3 + 0.25 * G3 * d4;
            m[4] += (g2 + mr.dv2q) * d0 + mr.dv6 * (G1 * d1 + G2 * d2 + G3 * d3) + (mr.c19 + 0.25 * g2) * d4;
        }
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) red[w][q][lane] = m[q];
    __syncthreads();
    if (w == 0 && c < Bp) {
        for (int q = 0; q < 5; ++q) {
            double t = 0.;
            for (int v = 0; v < kIncWarps; ++v) t += red[v][q][lane];
            part[((long long)c * 5 + q) * gridDim.x + blockIdx.x] = t;
        }
    }
}

// out_j = sum_k T(k, j) x_k for j = 0..nv-1 (nv even), two j per 16-byte
// factor load: A += T * Re x, B += T * Im x with the pencil's broadcast pairs
// xr[k] = (Re x_k, Re x_k), xi[k] = (Im x_k, Im x_k); out = (A.x - B.y, A.y + B.x).
template <int N>
__device__ __forceinline__ void proj_pairs(const unsigned long long (&xr)[N], const unsigned long long (&xi)[N],
                                           const float2 *T, int nv, float2 *out, long long ostride) {
    for (int j = 0; j < nv; j += 2) {
        unsigned long long A0 = 0ull, B0 = 0ull, A1 = 0ull, B1 = 0ull;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const ulonglong2 tt = *reinterpret_cast<const ulonglong2 *>(T + k * nv + j);
            A0 = fma2(tt.x, xr[k], A0);
            B0 = fma2(tt.x, xi[k], B0);
            A1 = fma2(tt.y, xr[k], A1);
            B1 = fma2(tt.y, xi[k], B1);
        }
        const float2 a0 = up2(A0), b0 = up2(B0), a1 = up2(A1), b1 = up2(B1);
        out[(long long)j * ostride] = make_float2(a0.x - b0.y, a0.y + b0.x);
        out[(long long)(j + 1) * ostride] = make_float2(a1.x - b1.y, a1.y + b1.x);
    }
}

// The same projection for n in {8, 16, 24, 32}, one thread per (pencil,
// cell) with the pencil's n inputs in registers and the per-axis factors
// T0, T1, T2 ([3][n][nv] complex) in shared memory (broadcast reads):
//   k_pj3  RK4 combination of q0..q3 (FP64 in, FP32 out) and the axis-3 pass,
//   k_pj2  the axis-2 pass into the five combinations Z0..Z4,
//   k_pj1  the axis-1 pass into the increments and their moment partials.
// cf/lam4: the q_s were not projected by conserveAllMoments; each gets its
// correction q_s -= C^T lambda_s (lam4[s][5][Bp]) in FP32 on load, and the
// combination is formed in FP32.
template <int N, typename QT>
__global__ void __launch_bounds__(128) k_pj3(const QT *__restrict__ q0, const QT *__restrict__ q1,
                                             const QT *__restrict__ q2, const QT *__restrict__ q3,
                                             double nu, const double *__restrict__ cnu, const float *__restrict__ tf,
                                             int nv, int Bp, float2 *__restrict__ Y, const float *__restrict__ cf,
                                             const double *__restrict__ lam4) {
    lp_grid_wait();
    extern __shared__ float2 Ts[];
    for (int t = threadIdx.y * 32 + threadIdx.x; t < 3 * N * nv; t += 128) Ts[t] = make_float2(tf[2 * t], tf[2 * t + 1]);
    __syncthreads();
    const int pid = blockIdx.x * 4 + threadIdx.y;  // (k1, k2)
    if (pid >= N * N) return;
    const int c = blockIdx.y * 32 + threadIdx.x;
    if (cnu) nu = cnu[c];
    float2 x[N];
    const long long b = (long long)pid * N * Bp + c;
    if (cf) {
        constexpr int n3 = N * N * N;
        float l[4][5];
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int j = 0; j < 5; ++j) l[s][j] = (float)lam4[(s * 5 + j) * Bp + c];
        const float nuf = (float)nu;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const long long o = b + (long long)k * Bp;
            const int pt = pid * N + k;
            const float r0 = cf[pt], r1 = cf[n3 + pt], r2 = cf[2 * n3 + pt], r3 = cf[3 * n3 + pt], r4 = cf[4 * n3 + pt];
            const QT qs[4] = {q0[o], q1[o], q2[o], q3[o]};
            float2 v[4];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                v[s].x = (float)qs[s].x - (r0 * l[s][0] + r4 * l[s][4]);
                v[s].y = (float)qs[s].y - (r1 * l[s][1] + r2 * l[s][2] + r3 * l[s][3]);
            }
            x[k] = make_float2(nuf * (0.5f * v[0].x + (v[1].x + v[2].x + v[3].x) * (1.f / 6.f)),
                               nuf * (0.5f * v[0].y + (v[1].y + v[2].y + v[3].y) * (1.f / 6.f)));
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const long long o = b + (long long)k * Bp;
            const QT a = q0[o], e = q1[o], d = q2[o], g = q3[o];
            x[k] = make_float2((float)(nu * (0.5 * a.x + (e.x + d.x + g.x) * (1. / 6.))),
                               (float)(nu * (0.5 * a.y + (e.y + d.y + g.y) * (1. / 6.))));
        }
    }
    if ((nv & 1) == 0) {
        unsigned long long xr[N], xi[N];
#pragma unroll
        for (int k = 0; k < N; ++k) { xr[k] = pk2(x[k].x, x[k].x); xi[k] = pk2(x[k].y, x[k].y); }
        for (int a = 0; a < 3; ++a)
            proj_pairs<N>(xr, xi, Ts + a * N * nv, nv, Y + ((long long)a * N * N + pid) * nv * Bp + c, Bp);
        return;
    }
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < nv; ++j) {
            const float2 *t = Ts + a * N * nv + j;
            float sr = 0.f, si = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const float2 m = t[k * nv];
                sr += m.x * x[k].x - m.y * x[k].y;
                si += m.x * x[k].y + m.y * x[k].x;
            }
            Y[(((long long)a * N * N + pid) * nv + j) * Bp + c] = make_float2(sr, si);
        }
}

// Z[p][k1][j2][j3] with (axis-3, axis-2 factor) = (0,0) (0,1) (0,2) (1,0) (2,0)
template <int N>
__global__ void __launch_bounds__(128) k_pj2(const float2 *__restrict__ Y, const float *__restrict__ tf, int nv,
                                             int Bp, float2 *__restrict__ Z) {
    lp_grid_wait();
    extern __shared__ float2 Ts[];
    for (int t = threadIdx.y * 32 + threadIdx.x; t < 3 * N * nv; t += 128) Ts[t] = make_float2(tf[2 * t], tf[2 * t + 1]);
    __syncthreads();
    const int pid = blockIdx.x * 4 + threadIdx.y;  // (k1, j3)
    if (pid >= N * nv) return;
    const int k1 = pid / nv, j3 = pid - k1 * nv;
    const int c = blockIdx.y * 32 + threadIdx.x;
    const long long ys = (long long)N * N * nv * Bp, zs = (long long)N * nv * nv * Bp;
    if ((nv & 1) == 0) {
        for (int a = 0; a < 3; ++a) {
            unsigned long long xr[N], xi[N];
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const float2 v = Y[a * ys + (((long long)k1 * N + k) * nv + j3) * Bp + c];
                xr[k] = pk2(v.x, v.x);
                xi[k] = pk2(v.y, v.y);
            }
            const int nf = a == 0 ? 3 : 1;
            for (int f = 0; f < nf; ++f) {
                const int p = a == 0 ? f : 2 + a;
                proj_pairs<N>(xr, xi, Ts + f * N * nv, nv, Z + p * zs + ((long long)k1 * nv * nv + j3) * Bp + c,
                              (long long)nv * Bp);
            }
        }
        return;
    }
    for (int a = 0; a < 3; ++a) {
        float2 x[N];
#pragma unroll
        for (int k = 0; k < N; ++k) x[k] = Y[a * ys + (((long long)k1 * N + k) * nv + j3) * Bp + c];
        const int nf = a == 0 ? 3 : 1;
        for (int f = 0; f < nf; ++f) {
            const int p = a == 0 ? f : 2 + a;
            for (int j = 0; j < nv; ++j) {
                const float2 *t = Ts + f * N * nv + j;
                float sr = 0.f, si = 0.f;
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    const float2 m = t[k * nv];
                    sr += m.x * x[k].x - m.y * x[k].y;
                    si += m.x * x[k].y + m.y * x[k].x;
                }
                Z[p * zs + (((long long)k1 * nv + j) * nv + j3) * Bp + c] = make_float2(sr, si);
            }
        }
    }
}


// Per (j2, j3, cell) pencil, four warps each take a group of JG consecutive
// j1 outputs (JG even, 4 JG >= nv).  The block's five source pencils Z0..Z4
// along k1 (two pencils x 32 cells) are staged in shared memory by one burst
// of cp.async copies; for each source the sums over k1 run with packed FP32
// FMAs, P += T(k1, j1) * z(k1) element-wise (Re (T z) = P.x - P.y), the
// factors read for two consecutive j1 per 16-byte load when nv is even.
// The sums of each j1 give the increment (see k_proj1_inc), written
// cell-minor, and the block's moment partials.
constexpr int kPj1Warps = 8, kPj1Pen = 2, kPj1Groups = kPj1Warps / kPj1Pen, kPj1Max = 8;
inline size_t pj1_smem(int N, int nv) {
    return sizeof(float2) * ((size_t)3 * N * nv + (size_t)kPj1Pen * 5 * N * 32);
}
template <int N, bool EVEN, int JG, int MINB = 1>
__global__ void __launch_bounds__(32 * kPj1Warps, MINB) k_pj1(const float2 *__restrict__ Z, const float *__restrict__ tf,
                                                        int nv, int Bp, int B, double dt, double kfac,
                                                        const double *__restrict__ cdt, double dv, double lv,
                                                        MomRow mr, float *__restrict__ Inc, double *__restrict__ part) {
    lp_grid_wait();
    extern __shared__ __align__(16) float2 Ts[];  // [3][N][nv], then the pencils [kPj1Pen][5][N][32]
    float2 *Zs = Ts + 3 * N * nv;
    __shared__ double red[kPj1Warps][5][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long zs = (long long)N * nv * nv * Bp, ks = (long long)nv * nv * Bp;
    for (int t = threadIdx.x; t < kPj1Pen * 5 * N * 16; t += 32 * kPj1Warps) {
        const int c2 = t & 15, r = t >> 4, k = r % N, p = (r / N) % 5, q = r / (5 * N);
        const int pq = blockIdx.x * kPj1Pen + q;
        if (pq < nv * nv)
            cp_async16(Zs + r * 32 + 2 * c2, Z + p * zs + k * ks + (long long)pq * Bp + blockIdx.y * 32 + 2 * c2);
    }
    cp_async_commit();
    for (int t = threadIdx.x; t < 3 * N * nv; t += 32 * kPj1Warps) Ts[t] = make_float2(tf[2 * t], tf[2 * t + 1]);
    cp_async_wait0();
    __syncthreads();
    const int pp = w / kPj1Groups, g = w - pp * kPj1Groups;
    const int pid = blockIdx.x * kPj1Pen + pp;
    const int c = blockIdx.y * 32 + lane;
    const int jg = JG, j0 = g * jg;
    double m[5] = {0, 0, 0, 0, 0};
    if (pid < nv * nv && c < B && j0 < nv) {
        const int j2 = pid / nv, j3 = pid - j2 * nv;
        const float2 *zp = Zs + pp * 5 * N * 32 + lane;
        // a[0], a[1]: T0, T1 sums of Z0; a[2], a[3]: T0 sums of Z1, Z3;
        // a[4]: T2 sum of Z0 plus the T0 sums of Z2 and Z4 (in that order)
        float a[5][JG];
#pragma unroll 1
        for (int p = 0; p < 5; ++p) {
            const int ntab = p == 0 ? 3 : 1;
            unsigned long long P[3][JG];
#pragma unroll
            for (int tb = 0; tb < 3; ++tb)
#pragma unroll
                for (int jj = 0; jj < JG; ++jj) P[tb][jj] = 0ull;
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const float2 zk = zp[(p * N + k) * 32];
                const unsigned long long zv = pk2(zk.x, zk.y);
#pragma unroll
                for (int tb = 0; tb < 3; ++tb) {
                    if (tb >= ntab) break;
#pragma unroll
                    for (int jj = 0; jj < JG; jj += 2) {
                        const int j1 = j0 + jj;
                        const float2 *T = Ts + tb * N * nv + k * nv + j1;
                        if constexpr (EVEN) {
                            const ulonglong2 tt = *reinterpret_cast<const ulonglong2 *>(T);
                            P[tb][jj] = fma2(tt.x, zv, P[tb][jj]);
                            P[tb][jj + 1] = fma2(tt.y, zv, P[tb][jj + 1]);
                        } else {
                            const float2 t0 = j1 < nv ? T[0] : make_float2(0.f, 0.f);
                            const float2 t1 = j1 + 1 < nv ? T[1] : make_float2(0.f, 0.f);
                            P[tb][jj] = fma2(pk2(t0.x, t0.y), zv, P[tb][jj]);
                            P[tb][jj + 1] = fma2(pk2(t1.x, t1.y), zv, P[tb][jj + 1]);
                        }
                    }
                }
            }
#pragma unroll
            for (int jj = 0; jj < JG; ++jj) {
                float v[3];
#pragma unroll
                for (int tb = 0; tb < 3; ++tb) {
                    const float2 pv = up2(P[tb][jj]);
                    v[tb] = pv.x - pv.y;
                }
                if (p == 0) { a[0][jj] = v[0]; a[1][jj] = v[1]; a[4][jj] = v[2]; }
                else if (p == 1) a[2][jj] = v[0];
                else if (p == 3) a[3][jj] = v[0];
                else a[4][jj] += v[0];
            }
        }
        const float sf = (float)((cdt ? cdt[c] : dt) * kfac);
        const double G2 = -lv + (j2 + 0.5) * dv, G3 = -lv + (j3 + 0.5) * dv;
        // Sums over this thread's j1 = j0 + jj of d_q, jj d_q (q = 0, 1, 4) and
        // jj^2 d_q (q = 0, 4) as FP32 pairs, exact to ~2^-44 of their terms:
        // with G1 = G10 + jj dv, sum G1 d = G10 S + dv T and
        // sum G1^2 d = G10^2 S + 2 G10 dv T + dv^2 V follow in FP64 once.
        DFSum S[5], T0, T1, T4, V0, V4;
#pragma unroll
        for (int jj = 0; jj < JG; ++jj) {
            const int j1 = j0 + jj;
            if (j1 >= nv) break;
            // the increment in FP32 (its inputs are FP32 sums), stored in FP32
            const float tp5 = a[4][jj];
            const float d0 = sf * (4.75f * a[0][jj] - 15.f * tp5), d4 = sf * (60.f * tp5 - 15.f * a[0][jj]);
            const float d1 = 12.f * sf * a[1][jj], d2 = 12.f * sf * a[2][jj], d3 = 12.f * sf * a[3][jj];
            const long long kt = ((long long)j1 * nv + j2) * nv + j3;
            float *o = Inc + kt * 5 * Bp + c;
            o[0] = d0; o[Bp] = d1; o[2 * Bp] = d2; o[3 * Bp] = d3; o[4 * Bp] = d4;
            S[0].add(d0); S[1].add(d1); S[2].add(d2); S[3].add(d3); S[4].add(d4);
            const float w1 = (float)jj, w2 = (float)(jj * jj);
            T0.addw(w1, d0); T1.addw(w1, d1); T4.addw(w1, d4);
            V0.addw(w2, d0); V4.addw(w2, d4);
        }
        const double G10 = -lv + (j0 + 0.5) * dv, G100 = G10 * G10, dv2 = dv * dv;
        const double S0 = S[0].get(), S1 = S[1].get(), S4 = S[4].get(), T0d = T0.get(), T1d = T1.get(),
                     T4d = T4.get();
        const double A0 = G10 * S0 + dv * T0d, A1 = G10 * S1 + dv * T1d, A4 = G10 * S4 + dv * T4d;
        const double B0 = G100 * S0 + 2. * G10 * dv * T0d + dv2 * V0.get();
        const double B4 = G100 * S4 + 2. * G10 * dv * T4d + dv2 * V4.get();
        const double S2 = S[2].get(), S3 = S[3].get();
        const double S04 = S0 + 0.25 * S4, G2233 = G2 * G2 + G3 * G3;
        m[0] = S04;
        m[1] = A0 + mr.dv12 * S1 + 0.25 * A4;
        m[2] = G2 * S04 + mr.dv12 * S2;
        m[3] = G3 * S04 + mr.dv12 * S3;
        m[4] = B0 + (G2233 + mr.dv2q) * S0 + mr.dv6 * (A1 + G2 * S2 + G3 * S3) + mr.c19 * S4 + 0.25 * B4 +
               0.25 * G2233 * S4;
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) red[w][q][lane] = m[q];
    __syncthreads();
    if (w == 0 && c < Bp)
        for (int q = 0; q < 5; ++q) {
            double t = 0.;
            for (int v = 0; v < kPj1Warps; ++v) t += red[v][q][lane];
            part[((long long)c * 5 + q) * gridDim.x + blockIdx.x] = t;
        }
}

template <int N, int JG>
cudaError_t pj1_launch(dim3 g1, const float2 *Z, const float *tfac, int nv, int Bp, int B, double dt, double kfac,
                       const double *cdt, double dv, double lv, float *Inc, double *part, cudaStream_t st) {
    const size_t sm = pj1_smem(N, nv);
    cudaError_t e;
    // two blocks per SM (at most 128 registers) up to six outputs per thread
    constexpr int MB = JG <= 6 ? 2 : 1;
    if (nv % 2 == 0) {
        if ((e = cudaFuncSetAttribute(k_pj1<N, true, JG, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)))
            return e;
        k_pj1<N, true, JG, MB><<<g1, 32 * kPj1Warps, sm, st>>>(Z, tfac, nv, Bp, B, dt, kfac, cdt, dv, lv,
                                                               mom_row(dv), Inc, part);
    } else {
        if ((e = cudaFuncSetAttribute(k_pj1<N, false, JG, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sm)))
            return e;
        k_pj1<N, false, JG, MB><<<g1, 32 * kPj1Warps, sm, st>>>(Z, tfac, nv, Bp, B, dt, kfac, cdt, dv, lv,
                                                                mom_row(dv), Inc, part);
    }
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_pj(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, double nu,
                      const float *tfac, int nv, int Bp, int B, double dt, double kfac, float2 *Y, float2 *Z,
                      float *Inc, double *part, double lv, double dv, cudaStream_t st, Rates rates,
                      const float *cf, const double *lam4, float2 *const *q32, const float *tc_tab, int *tc_err,
                      const float *tc_tab1) {
    const size_t ts = sizeof(float2) * 3 * N * nv;
    if (nv > kPj1Groups * kPj1Max) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_pj3<N, double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ts))) return e;
    if ((e = cudaFuncSetAttribute(k_pj3<N, float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ts))) return e;
    if ((e = cudaFuncSetAttribute(k_pj2<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ts))) return e;
    if (tc_tab && pj3_tc_supported(N, nv, Bp)) {
        // the axis-3 pass as a GEMM on the tensor cores (lp_pjtc.cu)
        e = q32 ? launch_pj3_tc<float2>(q32[0], q32[1], q32[2], q32[3], nu, rates.nu, tc_tab, N, nv, Bp, Y, cf, lam4,
                                        tc_err, st)
                : launch_pj3_tc<double2>(q0, q1, q2, q3, nu, rates.nu, tc_tab, N, nv, Bp, Y, cf, lam4, tc_err, st);
        if (e) return e;
    } else if (q32)
        k_pj3<N, float2><<<dim3((N * N + 3) / 4, Bp / 32), dim3(32, 4), ts, st>>>(
            q32[0], q32[1], q32[2], q32[3], nu, rates.nu, tfac, nv, Bp, Y, cf, lam4);
    else
        k_pj3<N, double2><<<dim3((N * N + 3) / 4, Bp / 32), dim3(32, 4), ts, st>>>(q0, q1, q2, q3, nu, rates.nu, tfac,
                                                                                nv, Bp, Y, cf, lam4);
    if (tc_tab && pj2_tc_supported(N, nv, Bp)) {
        // the axis-2 pass on the tensor cores (lp_pjtc.cu), with the axis-3 table
        if ((e = launch_pj2_tc(Y, tc_tab, N, nv, Bp, Z, tc_err, st))) return e;
    } else {
        k_pj2<N><<<dim3((N * nv + 3) / 4, Bp / 32), dim3(32, 4), ts, st>>>(Y, tfac, nv, Bp, Z);
    }
    if (tc_tab1 && pj1_tc_supported(N, nv, Bp)) {
        // the axis-1 pass as GEMMs on the tensor cores (lp_pjtc.cu)
        return launch_pj1_tc(Z, tc_tab1, N, nv, Bp, B, dt, kfac, rates.dt, dv, lv, Inc, part, tc_err, st);
    }
    const dim3 g1((nv * nv + kPj1Pen - 1) / kPj1Pen, Bp / 32);
    const int jg = 2 * ((nv + 2 * kPj1Groups - 1) / (2 * kPj1Groups));
    switch (jg) {
    case 2: e = pj1_launch<N, 2>(g1, Z, tfac, nv, Bp, B, dt, kfac, rates.dt, dv, lv, Inc, part, st); break;
    case 4: e = pj1_launch<N, 4>(g1, Z, tfac, nv, Bp, B, dt, kfac, rates.dt, dv, lv, Inc, part, st); break;
    case 6: e = pj1_launch<N, 6>(g1, Z, tfac, nv, Bp, B, dt, kfac, rates.dt, dv, lv, Inc, part, st); break;
    default: e = pj1_launch<N, 8>(g1, Z, tfac, nv, Bp, B, dt, kfac, rates.dt, dv, lv, Inc, part, st); break;
    }
    if (e) return e;
    return cudaGetLastError();
}

constexpr int kScatRec = 32;  // records per tile (x 32 cells)
constexpr size_t kScatSmem = sizeof(double) * (kScatRec * 5 * 33 + 32 * 5 + 8 * 7 * kScatRec);
__global__ void __launch_bounds__(256) k_scatter_inc(const float *__restrict__ Inc, int Bp, int B, int nv, int c0,
                                                     double *__restrict__ U, const double *__restrict__ lam,
                                                     double dv, double lv, MomRow mr) {
    lp_grid_wait();
    extern __shared__ double ssm[];
    double(*S)[5][33] = reinterpret_cast<double(*)[5][33]>(ssm);  // [record][coefficient][cell]
    // the cells' multipliers, converted to FP32 once here (the correction is
    // formed in FP32; a conversion per record would load GB300's narrow FP64 pipe)
    float(*L)[5] = reinterpret_cast<float(*)[5]>(ssm + kScatRec * 5 * 33);
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    double *ut = ssm + kScatRec * 5 * 33 + 32 * 5 + w * 7 * kScatRec;  // this warp's records of U
    const int nv3 = nv * nv * nv;
    const int kt0 = blockIdx.x * kScatRec;
    const int nrec = min(kScatRec, nv3 - kt0);
    const int cb = blockIdx.y * 32;
    // rows (record, coefficient) of 32 cells: coalesced along the cells; all
    // loads of a thread are issued before the first shared-memory store
    float v[kScatRec * 5 / 8];
#pragma unroll
    for (int j = 0; j < kScatRec * 5 / 8; ++j) {
        const int row = w + 8 * j, r = row / 5, q = row - r * 5;
        v[j] = (r < nrec && cb + lane < B) ? Inc[((long long)(kt0 + r) * 5 + q) * Bp + cb + lane] : 0.f;
    }
#pragma unroll
    for (int j = 0; j < kScatRec * 5 / 8; ++j) {
        const int row = w + 8 * j, r = row / 5, q = row - r * 5;
        S[r][q][lane] = f32_to_f64_bits(v[j]);
    }
    if (t < 160) {
        const int cc = t / 5, q = t - cc * 5;
        L[cc][q] = (lam && cb + cc < B) ? (float)lam[5 * (cb + cc) + q] : 0.f;
    }
    __syncthreads();
    const int kt = kt0 + lane, j3 = kt % nv, j2 = (kt / nv) % nv, j1 = kt / (nv * nv);
    // the correction Phi^T lambda in FP32: it is ~1e-7 of the increment, so
    // its rounding moves the moments by ~1e-15 of the increment's
    const float fdv = (float)dv, flv = (float)lv;
    const float G[3] = {-flv + (j1 + 0.5f) * fdv, -flv + (j2 + 0.5f) * fdv, -flv + (j3 + 0.5f) * fdv};
    const float g2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
    const float dv12 = (float)mr.dv12, dv6 = (float)mr.dv6, dv2q = (float)mr.dv2q, c19 = (float)mr.c19;
    // one cell per warp pass: its nrec records are 7 nrec contiguous doubles of U
    for (int cc = w; cc < 32 && cb + cc < B; cc += 8) {
        double *ug = U + 7 * ((long long)(c0 + cb + cc) * nv3 + kt0);
        if (nrec == kScatRec) {
            double x[7];
#pragma unroll
            for (int j = 0; j < 7; ++j) x[j] = ug[lane + 32 * j];
#pragma unroll
            for (int j = 0; j < 7; ++j) ut[lane + 32 * j] = x[j];
        } else {
            for (int k = lane; k < 7 * nrec; k += 32) ut[k] = ug[k];
        }
        __syncwarp();
        if (lane < nrec) {
            double a[5] = {S[lane][0][cc], S[lane][1][cc], S[lane][2][cc], S[lane][3][cc], S[lane][4][cc]};
            if (lam) {  // Phi^T lambda (mom_correct with the cell centre of this lane's record)
                const float l0 = L[cc][0], l1 = L[cc][1], l2 = L[cc][2], l3 = L[cc][3], l4 = L[cc][4];
                const float gl = G[0] * l1 + G[1] * l2 + G[2] * l3;
                a[0] += f32_to_f64_bits(l0 + gl + (g2 + dv2q) * l4);
                a[1] += f32_to_f64_bits(dv12 * l1 + dv6 * G[0] * l4);
                a[2] += f32_to_f64_bits(dv12 * l2 + dv6 * G[1] * l4);
                a[3] += f32_to_f64_bits(dv12 * l3 + dv6 * G[2] * l4);
                a[4] += f32_to_f64_bits(0.25f * l0 + 0.25f * gl + (c19 + 0.25f * g2) * l4);
            }
            double *u = ut + 7 * lane;
            u[0] += a[0]; u[3] += a[1]; u[4] += a[2]; u[5] += a[3]; u[6] += a[4];
        }
        __syncwarp();
        if (nrec == kScatRec) {
#pragma unroll
            for (int j = 0; j < 7; ++j) ug[lane + 32 * j] = ut[lane + 32 * j];
        } else {
            for (int k = lane; k < 7 * nrec; k += 32) ug[k] = ut[k];
        }
        __syncwarp();
    }
}

// The multipliers of one cell per block from the partials part[c][5][nk]
// (coalesced) and, when given, the target partials tpart[nchunk][5][Bp].
__global__ void __launch_bounds__(160) k_lambda_inc(const double *__restrict__ tpart, int nchunk,
                                                    const double *__restrict__ part, int nk,
                                                    const double *__restrict__ gm_inv, double scale, double kfac,
                                                    const double *__restrict__ cdt, int Bp,
                                                    double *__restrict__ lam) {
    lp_grid_wait();
    // one block of five warps per cell: warp m sums moment m of the
    // increments' partials (and of the target's, two-species operator) over
    // a fixed strided subset per lane and a fixed butterfly of shuffles;
    // threads 0..4 then solve with the inverse Gram matrix.  The FP64
    // dependency chains stay short on GB300's narrow FP64 unit.
    __shared__ double r5[5];
    const int c = blockIdx.x, lane = threadIdx.x & 31, m = threadIdx.x >> 5;
    const double *pc = part + ((long long)c * 5 + m) * nk;
    double ac = 0., tg = 0.;
    for (int k = lane; k < nk; k += 32) ac += pc[k];
    if (tpart)
        for (int k = lane; k < nchunk; k += 32) tg += tpart[((long long)k * 5 + m) * Bp + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ac += __shfl_xor_sync(0xffffffffu, ac, o);
        tg += __shfl_xor_sync(0xffffffffu, tg, o);
    }
    if (lane == 0) {
        const double sc = cdt ? cdt[c] * kfac : scale;
        r5[m] = sc * tg - ac;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        const int i = threadIdx.x;
        double sum = 0.;
#pragma unroll
        for (int j = 0; j < 5; ++j) sum += gm_inv[i * 5 + j] * r5[j];
        lam[5 * c + i] = sum;
    }
}

// ---------------------------------------------------------------- Poisson
// Charge moments per spatial cell: the sums over the cell's
// records of scalev (U0 + U6/4), scalev U1 and scalev U2.  The right-hand
// side of the Poisson problem is the small difference rho - 1, so the
// summation order matters at the 1e-12 level.  k_charge_seq accumulates each
// moment in one thread in the reference's record order without FMA, which
// gives the reference's sums bit for bit: warp 0 sums one chunk of terms
// while the other warps stage the next chunk in shared memory.
constexpr int kChargeChunk = 1024;
__global__ void __launch_bounds__(256) k_charge_seq(const double *__restrict__ U, int nv3, double scalev,
                                                   double *__restrict__ rt) {
    lp_grid_wait();
    __shared__ double term[2][3][kChargeChunk];
    const int s = blockIdx.x, t = threadIdx.x;
    const double *base = U + 7 * (long long)s * nv3;
    const int nchunk = (nv3 + kChargeChunk - 1) / kChargeChunk;
    auto stage = [&](int ch, int tid, int nthr) {
        const int c0 = ch * kChargeChunk, len = min(kChargeChunk, nv3 - c0);
        for (int j = tid; j < len; j += nthr) {
            const double *u = base + 7 * (long long)(c0 + j);
            term[ch & 1][0][j] = __dmul_rn(scalev, __dadd_rn(u[0], __dmul_rn(0.25, u[6])));
            term[ch & 1][1][j] = __dmul_rn(scalev, u[1]);
            term[ch & 1][2][j] = __dmul_rn(scalev, u[2]);
        }
    };
    stage(0, t, blockDim.x);
    __syncthreads();
    double acc = 0.0;
    for (int ch = 0; ch < nchunk; ++ch) {
        if (t < 32) {
            if (t < 3) {
                const int len = min(kChargeChunk, nv3 - ch * kChargeChunk);
                const double *tt = term[ch & 1][t];
#pragma unroll 8
                for (int j = 0; j < len; ++j) acc = __dadd_rn(acc, tt[j]);
            }
        } else if (ch + 1 < nchunk) {
            stage(ch + 1, t - 32, blockDim.x - 32);
        }
        __syncthreads();
    }
    if (t < 3) rt[3 * s + t] = acc;
}

// Block sums of (U0 + U6/4, U1, U2) over 128 consecutive records, written to
// part[blockIdx.x][3] in a fixed order; the Poisson kernel adds a cell's
// blocks in order and scales by scalev (the mixed path's charge).
__device__ __forceinline__ void charge_block_sum(double a0, double a1, double a2, double *__restrict__ part) {
    __shared__ double red[3][4];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    const int t = threadIdx.x;
    if ((t & 31) == 0) { red[0][t >> 5] = a0; red[1][t >> 5] = a1; red[2][t >> 5] = a2; }
    __syncthreads();
    if (t < 3) part[3 * (long long)blockIdx.x + t] = (red[t][0] + red[t][1]) + (red[t][2] + red[t][3]);
}

// FP32 copy of the state for the FP32 flux, with the charge partial sums of
// the same records (one record per thread, 128 records per block).
__global__ void __launch_bounds__(128) k_state_f32(const double *__restrict__ U, long long size,
                                                  float *__restrict__ Uf, double *__restrict__ part) {
    lp_grid_wait();
    const long long k = blockIdx.x * 128ll + threadIdx.x;
    double a0 = 0., a1 = 0., a2 = 0.;
    if (k < size) {
        const double *u = U + 7 * k;
        double v[7];
#pragma unroll
        for (int l = 0; l < 7; ++l) { v[l] = u[l]; Uf[7 * k + l] = (float)v[l]; }
        a0 = v[0] + 0.25 * v[6]; a1 = v[1]; a2 = v[2];
    }
    if (part) charge_block_sum(a0, a1, a2, part);
}

// pois2d in one block: right-hand side, the band solve of DGBTRS
// replayed on one warp in the host factorisation's operation order, field
// reconstruction and the cell integrals used by the advection.  With
// pd.rdiag == nullptr every operation is the host's, without FMA (the
// reference's result bit for bit); otherwise (mixed path) divisions become
// products with precomputed reciprocals and the charge comes as npart block
// partial sums per cell.
__global__ void k_poisson(PoissonDev pd, const double *__restrict__ rt, int npart, double *__restrict__ bg,
                          double *__restrict__ potc, double *__restrict__ phix, double *__restrict__ phiy,
                          double *__restrict__ fields) {
    lp_grid_wait();
    extern __shared__ double b[];
    const int t = threadIdx.x, nc = pd.nx * pd.ny, nd = pd.ndim;
    const bool fast = pd.rdiag != nullptr;
    // shared memory: b[nd], the band factors (when they fit), the pivots
    double *sab = b + nd;
    int *spiv = reinterpret_cast<int *>(sab + (pd.staged ? (size_t)pd.ldab * nd : 0));
    if (pd.staged)
        for (long long i = t; i < (long long)pd.ldab * nd; i += blockDim.x) sab[i] = pd.ab[i];
    for (int i = t; i < nd; i += blockDim.x) spiv[i] = pd.ipiv[i];
    const double *AB = pd.staged ? sab : pd.ab;
    for (int ii = t; ii < nc; ii += blockDim.x) {
        const double DXv = pd.dxp, DYv = pd.dyp;
        if (!fast) {
            b[3 * ii] = __dmul_rn(__dmul_rn(__dsub_rn(rt[3 * ii], 1.0), DXv), DYv);
            b[3 * ii + 1] = __ddiv_rn(__dmul_rn(__dmul_rn(rt[3 * ii + 1], DXv), DYv), 12.);
            b[3 * ii + 2] = __ddiv_rn(__dmul_rn(__dmul_rn(rt[3 * ii + 2], DXv), DYv), 12.);
        } else {
            double r0 = 0., r1 = 0., r2 = 0.;
            const double *pp = rt + 3 * (long long)ii * npart;
            for (int p = 0; p < npart; ++p) { r0 += pp[3 * p]; r1 += pp[3 * p + 1]; r2 += pp[3 * p + 2]; }
            b[3 * ii] = (r0 * pd.cscale - 1.0) * DXv * DYv;
            b[3 * ii + 1] = r1 * pd.cscale * DXv * DYv * (1. / 12.);
            b[3 * ii + 2] = r2 * pd.cscale * DXv * DYv * (1. / 12.);
        }
    }
    __syncthreads();
    const int ldab = pd.ldab;
#define ABD(i, j) AB[((i) - 1) + (long long)((j) - 1) * ldab]
    if (t < 32) {
        const int kd = pd.ku + pd.kl + 1;
        for (int j = 1; j <= nd - 1; ++j) {
            const int lm = min(pd.kl, nd - j);
            const int l = spiv[j - 1];
            if (t == 0 && l != j) { const double tmp = b[l - 1]; b[l - 1] = b[j - 1]; b[j - 1] = tmp; }
            __syncwarp();
            const double bj = b[j - 1];
            if (bj != 0.0) {
                const double tt = -bj;
                for (int i = 1 + t; i <= lm; i += 32) b[j + i - 1] = __dadd_rn(b[j + i - 1], __dmul_rn(ABD(kd + i, j), tt));
            }
            __syncwarp();
        }
        const int k = pd.kl + pd.ku, kplus1 = k + 1;
        for (int j = nd; j >= 1; --j) {
            const double bj = b[j - 1];
            __syncwarp();
            if (bj != 0.0) {
                const int l = kplus1 - j;
                const double xj = fast ? bj * pd.rdiag[j - 1] : __ddiv_rn(bj, ABD(kplus1, j));
                const int ilo = max(1, j - k);
                for (int i = j - 1 - t; i >= ilo; i -= 32) b[i - 1] = __dsub_rn(b[i - 1], __dmul_rn(xj, ABD(l + i, j)));
                if (t == 0) b[j - 1] = xj;
            }
            __syncwarp();
        }
    }
#undef ABD
    __syncthreads();
    for (int i = t; i < nd; i += blockDim.x) { potc[i] = b[i]; bg[i] = b[i]; }
    __syncthreads();
    const double *acvx = pd.blk[0], *acyrr = pd.blk[1], *acyrl = pd.blk[2];
    const double *acvy = pd.blk[3], *acxrr = pd.blk[4], *acxrl = pd.blk[5];
    const double rdxp = pd.rdxp, rdyp = pd.rdyp;
    auto div = [&](double a, double d, double rd) { return fast ? a * rd : __ddiv_rn(a, d); };
    for (int ii = t; ii < nc; ii += blockDim.x) {
        const int ix = ii / pd.ny + 1, jy = ii % pd.ny + 1;
        const int il = ii - pd.ny, ib = ii - 1;
        for (int k = 0; k < 3; ++k) {  // E_x
            double s = 0.;
            if (ix == 1) {
                for (int kk = 0; kk < 3; ++kk) s = __dadd_rn(s, __dmul_rn(__dadd_rn(acvx[3 * k + kk], acyrr[3 * k + kk]), b[3 * ii + kk]));
                s = __dsub_rn(s, __dmul_rn(acyrl[3 * k], 0.));
            } else if (ix == pd.nx) {
                for (int kk = 0; kk < 3; ++kk)
                    s = __dsub_rn(__dadd_rn(s, __dmul_rn(acvx[3 * k + kk], b[3 * ii + kk])), __dmul_rn(acyrl[3 * k + kk], b[3 * il + kk]));
                s = __dadd_rn(s, __dmul_rn(acyrr[3 * k], 0.));
            } else {
                for (int kk = 0; kk < 3; ++kk)
                    s = __dsub_rn(__dadd_rn(s, __dmul_rn(__dadd_rn(acvx[3 * k + kk], acyrr[3 * k + kk]), b[3 * ii + kk])),
                                  __dmul_rn(acyrl[3 * k + kk], b[3 * il + kk]));
            }
            phix[3 * ii + k] = div(-s, pd.dxp, rdxp);
        }
        for (int k = 0; k < 3; ++k) {  // E_y
            double s = 0.;
            if (jy == 1) {
                phiy[3 * ii + k] = (k == 0) ? div(-b[3 * ii + 2], pd.dyp, rdyp) : 0.;
                continue;
            }
            if (jy == pd.ny && pd.gate[ix]) {
                for (int kk = 0; kk < 3; ++kk)
                    s = __dsub_rn(__dadd_rn(s, __dmul_rn(acvy[3 * k + kk], b[3 * ii + kk])), __dmul_rn(acxrl[3 * k + kk], b[3 * ib + kk]));
                s = __dadd_rn(s, __dmul_rn(acxrr[3 * k], 0.));
            } else {
                for (int kk = 0; kk < 3; ++kk)
                    s = __dsub_rn(__dadd_rn(s, __dmul_rn(__dadd_rn(acvy[3 * k + kk], acxrr[3 * k + kk]), b[3 * ii + kk])),
                                  __dmul_rn(acxrl[3 * k + kk], b[3 * ib + kk]));
            }
            phiy[3 * ii + k] = div(-s, pd.dyp, rdyp);
        }
        // cell integrals of the field
        const double ex0 = phix[3 * ii], ex1 = phix[3 * ii + 1], ex2 = phix[3 * ii + 2];
        const double ey0 = phiy[3 * ii], ey1 = phiy[3 * ii + 1], ey2 = phiy[3 * ii + 2];
        constexpr double r12 = 1. / 12.;
        fields[0 * nc + ii] = ex0;
        fields[1 * nc + ii] = div(ex1, 12., r12);
        fields[2 * nc + ii] = div(ex2, 12., r12);
        fields[3 * nc + ii] = div(ex0, 12., r12);
        fields[4 * nc + ii] = 0.;
        fields[5 * nc + ii] = div(ex0, 12., r12);
        fields[6 * nc + ii] = ey0;
        fields[7 * nc + ii] = div(ey1, 12., r12);
        fields[8 * nc + ii] = div(ey2, 12., r12);
        fields[9 * nc + ii] = div(ey0, 12., r12);
        fields[10 * nc + ii] = 0.;
        fields[11 * nc + ii] = div(ey0, 12., r12);
        fields[12 * nc + ii] = ex0 > 0. ? 1. : -1.;
        fields[13 * nc + ii] = ey0 > 0. ? 1. : -1.;
    }
}


// ---------------------------------------------------------------- advection
// Right-hand side H of record k (I1, I2, I3, I5 at A:213-405 combined as at
// A:455-467; H[2] = 0) in arithmetic T from stage values of type S.  Constant
// divisions are products with reciprocals (within 2 ulp of the reference's).
template <typename T, typename S>
__device__ __forceinline__ void flux_rhs(const AdvectDev &ad, const S *__restrict__ Us,
                                         const double *__restrict__ fields, long long k, T H[7]) {
    const int nv = ad.nv;
    const long long sv = (long long)nv * nv * nv;
    // record decomposition in 32-bit arithmetic (the launcher keeps size < 2^31)
    const int k32 = (int)k, sv32 = (int)sv, nvv = nv * nv;
    const int jm32 = k32 % sv32, s32 = k32 / sv32;
    const long long jm = jm32, s = s32;
    const int j3 = jm32 % nv, j2 = (jm32 / nv) % nv, j1 = jm32 / nvv;
    const int i2 = s32 % ad.nx2, i1 = s32 / ad.nx2;
    // FP32 evaluation takes its constants from the FP32 copies and converts
    // the FP64 fields by bit manipulation, so no FP64 instruction is issued
    constexpr bool F32 = std::is_same<T, float>::value;
    const T dv = F32 ? (T)ad.f.dv : (T)ad.dv, rdv = F32 ? (T)ad.f.rdv : (T)ad.rdv;
    const T G = F32 ? (T)(-ad.f.lv + ((float)j1 + 0.5f) * ad.f.dv) : (T)(-ad.lv + (j1 + 0.5) * ad.dv);
    const T i12 = T(1. / 12.), i720_19 = T(19. / 720.), i240_19 = T(19. / 240.), i5_12 = T(5. / 12.),
            i720_133 = T(133. / 720.), i6 = T(1. / 6.), h = T(0.5), q4 = T(0.25);
    T u[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) u[q] = (T)Us[7 * k + q];
    // x1 upwind neighbours by the sign of v1, periodic (I3).
    T R3[7], L3[7], ur3, ul3;
    if (j1 < nv / 2) {
        int iir = i1 + 1;
        if (iir == ad.nx1) iir = 0;
        const long long kr3 = (long long)iir * ad.nx2 * sv + (long long)i2 * sv + jm;
#pragma unroll
        for (int q = 0; q < 7; ++q) { R3[q] = (T)Us[7 * kr3 + q]; L3[q] = u[q]; }
        ur3 = -R3[1];
        ul3 = -L3[1];
    } else {
        int iil = i1 - 1;
        if (iil == -1) iil = ad.nx1 - 1;
        const long long kl3 = (long long)iil * ad.nx2 * sv + (long long)i2 * sv + jm;
#pragma unroll
        for (int q = 0; q < 7; ++q) { L3[q] = (T)Us[7 * kl3 + q]; R3[q] = u[q]; }
        ur3 = R3[1];
        ul3 = L3[1];
    }
    // v1 upwind neighbours by the sign of the cell-average E_x, no inflow (I5).
    const long long nc = (long long)ad.nx1 * ad.nx2;
    const double ie_d = fields[s];
    T ie, ixe, ixxe;
    // the reference's field terms are cell averages; with LP_FIX_F12 they are
    // scaled to the cell integrals the DG weak form needs (fscale = dx)
    if constexpr (F32) {
        const float fs = ad.f.fscale;
        ie = f64_to_f32_bits(ie_d) * fs; ixe = f64_to_f32_bits(fields[nc + s]) * fs;
        ixxe = f64_to_f32_bits(fields[3 * nc + s]) * fs;
    } else {
        const double fs = ad.fscale;
        ie = ie_d * fs; ixe = fields[nc + s] * fs; ixxe = fields[3 * nc + s] * fs;
    }
    // ie > 0 from the bit pattern (a positive double is a positive integer)
    const bool ie_pos = F32 ? (__double_as_longlong(ie_d) > 0) : (ie_d > 0);
    T R5[7], L5[7], ur5 = T(0), ul5 = T(0);
    bool hasr, hasl;
    if (ie_pos) {
        hasr = j1 + 1 < nv;
        hasl = true;
        const long long kr5 = s * sv + ((long long)(j1 + 1) * nv * nv + j2 * nv + j3);
#pragma unroll
        for (int q = 0; q < 7; ++q) { R5[q] = hasr ? (T)Us[7 * kr5 + q] : T(0); L5[q] = u[q]; }
        if (hasr) ur5 = -R5[3];
        ul5 = -L5[3];
    } else {
        hasr = true;
        hasl = j1 - 1 > -1;
        const long long kl5 = s * sv + ((long long)(j1 - 1) * nv * nv + j2 * nv + j3);
#pragma unroll
        for (int q = 0; q < 7; ++q) { L5[q] = hasl ? (T)Us[7 * kl5 + q] : T(0); R5[q] = u[q]; }
        ur5 = R5[3];
        if (hasl) ul5 = L5[3];
    }
    const T dv2 = dv * dv, dv3 = dv * dv * dv;
    T tp[6];
    // l = 0
    {
        T i3 = dv3 * ((R3[0] + h * ur3 - L3[0] - h * ul3) * G + (R3[3] - L3[3]) * dv * i12 + (R3[6] - L3[6]) * G * q4);
        T i5 = T(0);
        if (hasr && hasl) i5 = dv2 * (R5[0] + h * ur5 + R5[6] * i5_12 - L5[0] - h * ul5 - L5[6] * i5_12) * ie + dv2 * (R5[1] - L5[1]) * ixe;
        else if (hasr) i5 = dv2 * (R5[0] + h * ur5 + R5[6] * i5_12) * ie + dv2 * R5[1] * ixe;
        else if (hasl) i5 = dv2 * (-L5[0] - h * ul5 - L5[6] * i5_12) * ie - dv2 * L5[1] * ixe;
        tp[0] = -i3 + i5;
    }
    // l = 1
    {
        T i1v = dv3 * (G * u[0] + dv * u[3] * i12 + u[6] * G * q4);
        T i3 = h * dv3 * ((R3[0] + h * ur3 + L3[0] + h * ul3) * G + (R3[3] + L3[3]) * dv * i12 + (R3[6] + L3[6]) * G * q4);
        T i5 = T(0);
        if (hasr && hasl) i5 = dv2 * ((R5[0] + h * ur5 + R5[6] * i5_12 - L5[0] - h * ul5 - L5[6] * i5_12) * ixe + (R5[1] - L5[1]) * ixxe);
        else if (hasr) i5 = dv2 * ((R5[0] + h * ur5 + R5[6] * i5_12) * ixe + R5[1] * ixxe);
        else if (hasl) i5 = dv2 * ((-L5[0] - h * ul5 - L5[6] * i5_12) * ixe - L5[1] * ixxe);
        tp[1] = i1v - i3 + i5;
    }
    // l = 3 (v1 slope)
    {
        T i2 = (((u[0] + u[6] * q4) * ie + u[1] * ixe) * (F32 ? (T)ad.f.scalev : (T)ad.scalev)) * rdv;
        T i3 = dv2 * (((R3[0] - L3[0]) * dv2 + (ur3 - ul3) * h * dv2 + (R3[3] - L3[3]) * dv * G) * i12 + (R3[6] - L3[6]) * dv2 * i720_19);
        T i5 = T(0);
        if (hasr && hasl) i5 = h * (dv2 * (R5[0] + h * ur5 + R5[6] * i5_12 + L5[0] + h * ul5 + L5[6] * i5_12) * ie + dv2 * (R5[1] + L5[1]) * ixe);
        else if (hasr) i5 = h * (dv2 * (R5[0] + h * ur5 + R5[6] * i5_12) * ie + dv2 * R5[1] * ixe);
        else if (hasl) i5 = h * (dv2 * (L5[0] + h * ul5 + L5[6] * i5_12) * ie + dv2 * L5[1] * ixe);
        tp[2] = -i2 - i3 + i5;
    }
    // l = 4, 5 (v2, v3 slopes)
#pragma unroll
    for (int q = 4; q <= 5; ++q) {
        T i3 = (R3[q] - L3[q]) * G * dv3 * i12;
        T i5 = T(0);
        if (hasr && hasl) i5 = (R5[q] - L5[q]) * ie * dv2 * i12;
        else if (hasr) i5 = R5[q] * ie * dv2 * i12;
        else if (hasl) i5 = -L5[q] * ie * dv2 * i12;
        tp[q - 1] = -i3 + i5;
    }
    // l = 6 (|v|^2 mode)
    {
        T i2 = u[3] * dv2 * ie * i6;
        T i3 = dv3 * ((R3[0] + h * ur3 - L3[0] - h * ul3) * G * q4 + (R3[3] - L3[3]) * dv * i720_19 + (R3[6] - L3[6]) * G * i240_19);
        T i5 = T(0);
        if (hasr && hasl) i5 = dv2 * (((R5[0] + h * ur5 - L5[0] - h * ul5) * i5_12 + (R5[6] - L5[6]) * i720_133) * ie + (R5[1] - L5[1]) * ixe * i5_12);
        else if (hasr) i5 = dv2 * (((R5[0] + h * ur5) * i5_12 + R5[6] * i720_133) * ie + R5[1] * ixe * i5_12);
        else if (hasl) i5 = -dv2 * (((L5[0] + h * ul5) * i5_12 + L5[6] * i720_133) * ie + L5[1] * ixe * i5_12);
        tp[5] = -i2 - i3 + i5;
    }
    const T inv = F32 ? (T)ad.f.inv : (T)ad.inv, c12 = T(12);
    H[0] = (T(19) * tp[0] * q4 - T(15) * tp[5]) * inv;
    H[6] = (T(60) * tp[5] - T(15) * tp[0]) * inv;
    H[1] = tp[1] * c12 * inv;
    H[2] = T(0);
    H[3] = tp[2] * c12 * inv;
    H[4] = tp[3] * c12 * inv;
    H[5] = tp[4] * c12 * inv;
}

// One SSP-RK3 stage (A:469, A:527, A:581): H from the stage values Uin (type
// S, evaluated in T), the combination with U0 and Us in FP64.  Optionally
// writes an FP32 copy of the result (the next stage's Uin) and the charge
// partial sums of the result per block of 128 records (the next Poisson
// solve's right-hand side); both need the records of a block to belong to
// one spatial cell (nv^3 a multiple of 128).
template <typename T, typename S>
__global__ void __launch_bounds__(128) k_flux(AdvectDev ad, const double *__restrict__ U0, const double *__restrict__ Us,
                                             const S *__restrict__ Uin, const double *__restrict__ fields, int stage,
                                             double *__restrict__ Uout, float *__restrict__ Uoutf,
                                             double *__restrict__ part) {
    lp_grid_wait();
    const long long k = blockIdx.x * 128ll + threadIdx.x;
    double a0 = 0., a1 = 0., a2 = 0.;
    if (k < ad.size) {
        T H[7];
        flux_rhs<T, S>(ad, Uin, fields, k, H);
        const double dt = ad.dt;
        const double *u0 = U0 + 7 * k, *u = Us + 7 * k;
        double r[7];
#pragma unroll
        for (int l = 0; l < 7; ++l) {
            const double hl = (double)H[l];
            if (stage == 0) r[l] = u0[l] + dt * hl;
            else if (stage == 1) r[l] = 0.75 * u0[l] + 0.25 * u[l] + 0.25 * dt * hl;
            else r[l] = u0[l] * (1. / 3.) + u[l] * (2. / 3.) + dt * hl * (2. / 3.);
        }
        double *o = Uout + 7 * k;
#pragma unroll
        for (int l = 0; l < 7; ++l) o[l] = r[l];
        if (Uoutf) {
#pragma unroll
            for (int l = 0; l < 7; ++l) Uoutf[7 * k + l] = (float)r[l];
        }
        a0 = r[0] + 0.25 * r[6]; a1 = r[1]; a2 = r[2];
    }
    if (part) charge_block_sum(a0, a1, a2, part);
}

// ---------------------------------------------------------------- mixed-path advection
// FP32 copy of the state and the FP64 charge moments of every group of 128
// consecutive records (one warp per group, four records per lane):
// part[3 * group] = (sum U0 + U6/4, sum U1, sum U2).
__global__ void __launch_bounds__(128) k_state_f32_grp(const double *__restrict__ U, long long size,
                                                      float *__restrict__ Uf, double *__restrict__ part) {
    lp_grid_wait();
    const int lane = threadIdx.x & 31;
    const long long g = blockIdx.x * 4ll + (threadIdx.x >> 5);
    double a0 = 0., a1 = 0., a2 = 0.;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const long long k = g * 128 + j * 32 + lane;
        if (k < size) {
            const double *u = U + 7 * k;
            double v[7];
#pragma unroll
            for (int l = 0; l < 7; ++l) { v[l] = u[l]; Uf[7 * k + l] = f64_to_f32_bits(v[l]); }
            a0 += v[0] + 0.25 * v[6]; a1 += v[1]; a2 += v[2];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0 && g * 128 < size) { part[3 * g] = a0; part[3 * g + 1] = a1; part[3 * g + 2] = a2; }
}

// Mixed path, increment form of SSP-RK3 (the reference's stages A:469-581 in
// exact arithmetic): with H_s = H(U_s) evaluated in FP32,
//   U1 = U + dt H0,   U2 = U + dt/4 (H0 + H1),   U_new = U + dt/6 (H0 + H1 + 4 H2).
// Stages 0 and 1 read the FP32 copy of U_s (own and neighbour records), keep
// the running FP32 sum S of the H's, write the FP32 copy Uf0 + c S of the next
// stage's values and the FP32 sums of S over every group of 128 records (the
// charge moments are linear: rho(U_{s+1}) = rho(U) + c sum S).  Only stage 2
// touches the FP64 state: U += dt/6 (S + 4 H2).
template <int STAGE>
__global__ void __launch_bounds__(128) k_flux_inc(AdvectDev ad, const float *__restrict__ Uin,
                                                 const float *__restrict__ Uf0, const double *__restrict__ fields,
                                                 float *__restrict__ S, float *__restrict__ Uoutf,
                                                 double *__restrict__ U, float *__restrict__ ipart) {
    lp_grid_wait();
    const long long k = blockIdx.x * 128ll + threadIdx.x;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (k < ad.size) {
        float H[7];
        flux_rhs<float, float>(ad, Uin, fields, k, H);
        if (STAGE < 2) {
            const float c = STAGE == 0 ? ad.dt_f : 0.25f * ad.dt_f;
            float s[7];
#pragma unroll
            for (int l = 0; l < 7; ++l) {
                s[l] = STAGE == 0 ? H[l] : S[7 * k + l] + H[l];
                S[7 * k + l] = s[l];
                Uoutf[7 * k + l] = Uf0[7 * k + l] + c * s[l];
            }
            a0 = s[0] + 0.25f * s[6]; a1 = s[1]; a2 = s[2];
        } else {
            double *u = U + 7 * k;
#pragma unroll
            for (int l = 0; l < 7; ++l) u[l] += ad.dt6 * f32_to_f64_bits(S[7 * k + l] + 4.f * H[l]);
        }
    }
    if (STAGE < 2) {
        __shared__ float red[3][4];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        }
        const int t = threadIdx.x;
        if ((t & 31) == 0) { red[0][t >> 5] = a0; red[1][t >> 5] = a1; red[2][t >> 5] = a2; }
        __syncthreads();
        if (t < 3) ipart[3 * (long long)blockIdx.x + t] = (red[t][0] + red[t][1]) + (red[t][2] + red[t][3]);
    }
}

// Mixed-path Poisson solve in three kernels: the right-hand side from the
// group partials (one warp per cell), x = A^-1 b with the dense inverse of
// the LDG matrix (one warp per row), and the field reconstruction and cell
// integrals (one thread per cell; pois2d P:1292-1467).
__global__ void k_prhs(PoissonDev pd, const double *__restrict__ base, const float *__restrict__ inc,
                       double iscale, int npart, double *__restrict__ b) {
    lp_grid_wait();
    const int lane = threadIdx.x & 31;
    const int ii = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (ii >= pd.nx * pd.ny) return;
    double r[3] = {0., 0., 0.}, d[3] = {0., 0., 0.};
    for (int p = lane; p < npart; p += 32)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            r[m] += base[3 * ((long long)ii * npart + p) + m];
            if (inc) d[m] += (double)inc[3 * ((long long)ii * npart + p) + m];
        }
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        double v = r[m] + iscale * d[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        r[m] = v * pd.cscale;
    }
    if (lane == 0) {
        const double DXv = pd.dxp, DYv = pd.dyp;
        b[3 * ii] = (r[0] - 1.0) * DXv * DYv;
        b[3 * ii + 1] = r[1] * DXv * DYv * (1. / 12.);
        b[3 * ii + 2] = r[2] * DXv * DYv * (1. / 12.);
    }
}

__global__ void k_psolve_dense(const double *__restrict__ Ainv, const double *__restrict__ b, int nd,
                               double *__restrict__ x) {
    lp_grid_wait();
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= nd) return;
    const double *a = Ainv + (long long)row * nd;
    double s = 0.;
    for (int j = lane; j < nd; j += 32) s += a[j] * b[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = s;
}

__global__ void k_pfields(PoissonDev pd, const double *__restrict__ b, double *__restrict__ phix,
                          double *__restrict__ phiy, double *__restrict__ fields) {
    lp_grid_wait();
    const int nc = pd.nx * pd.ny;
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= nc) return;
    const double *acvx = pd.blk[0], *acyrr = pd.blk[1], *acyrl = pd.blk[2];
    const double *acvy = pd.blk[3], *acxrr = pd.blk[4], *acxrl = pd.blk[5];
    const int ix = ii / pd.ny + 1, jy = ii % pd.ny + 1;
    const int il = ii - pd.ny, ib = ii - 1;
    double ex[3], ey[3];
    for (int k = 0; k < 3; ++k) {  // E_x
        double s = 0.;
        for (int kk = 0; kk < 3; ++kk) {
            const double bc = b[3 * ii + kk];
            if (ix == 1) s += (acvx[3 * k + kk] + acyrr[3 * k + kk]) * bc;
            else if (ix == pd.nx) s += acvx[3 * k + kk] * bc - acyrl[3 * k + kk] * b[3 * il + kk];
            else s += (acvx[3 * k + kk] + acyrr[3 * k + kk]) * bc - acyrl[3 * k + kk] * b[3 * il + kk];
        }
        ex[k] = -s * pd.rdxp;
    }
    for (int k = 0; k < 3; ++k) {  // E_y
        if (jy == 1) { ey[k] = (k == 0) ? -b[3 * ii + 2] * pd.rdyp : 0.; continue; }
        double s = 0.;
        const bool top = (jy == pd.ny && pd.gate[ix]);
        for (int kk = 0; kk < 3; ++kk) {
            const double bc = b[3 * ii + kk];
            if (top) s += acvy[3 * k + kk] * bc - acxrl[3 * k + kk] * b[3 * ib + kk];
            else s += (acvy[3 * k + kk] + acxrr[3 * k + kk]) * bc - acxrl[3 * k + kk] * b[3 * ib + kk];
        }
        ey[k] = -s * pd.rdyp;
    }
    constexpr double r12 = 1. / 12.;
    for (int k = 0; k < 3; ++k) { phix[3 * ii + k] = ex[k]; phiy[3 * ii + k] = ey[k]; }
    fields[0 * nc + ii] = ex[0];
    fields[1 * nc + ii] = ex[1] * r12;
    fields[2 * nc + ii] = ex[2] * r12;
    fields[3 * nc + ii] = ex[0] * r12;
    fields[4 * nc + ii] = 0.;
    fields[5 * nc + ii] = ex[0] * r12;
    fields[6 * nc + ii] = ey[0];
    fields[7 * nc + ii] = ey[1] * r12;
    fields[8 * nc + ii] = ey[2] * r12;
    fields[9 * nc + ii] = ey[0] * r12;
    fields[10 * nc + ii] = 0.;
    fields[11 * nc + ii] = ey[0] * r12;
    fields[12 * nc + ii] = ex[0] > 0. ? 1. : -1.;
    fields[13 * nc + ii] = ey[0] > 0. ? 1. : -1.;
}

// ---------------------------------------------------------------- diagnostics
// Entropy int f log f (computeEntropy, EntropyCalculations.cpp:11-65): the
// 5-point Gauss-Legendre rule in x1, v1, v2, v3 of every record, f > 0 only
// (the x2 slope is not sampled, as in the reference).  f and f log f in FP32
// (a diagnostic; within 1e-6 of the FP64 sum), per-record sums added in FP64.
__constant__ float c_gl_x[5] = {0.f, -0.5384693101056831f, 0.5384693101056831f, -0.9061798459386640f,
                                0.9061798459386640f};
__constant__ float c_gl_w[5] = {0.5688888888888889f, 0.4786286704993665f, 0.4786286704993665f,
                                0.2369268850561891f, 0.2369268850561891f};
__global__ void __launch_bounds__(256) k_entropy(const double *__restrict__ U, long long kend,
                                                double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[256];
    double acc = 0.;
    for (long long k = blockIdx.x * 256ll + threadIdx.x; k < kend; k += 256ll * gridDim.x) {
        const double *u = U + 7 * k;
        const float u0 = (float)u[0], u1 = (float)u[1], u3 = (float)u[3], u4 = (float)u[4], u5 = (float)u[5],
                    u6 = (float)u[6];
        float s = 0.f;
        for (int a = 0; a < 5; ++a) {
            const float fa = u0 + u1 * 0.5f * c_gl_x[a];
            for (int p = 0; p < 5; ++p) {
                const float b1 = 0.5f * c_gl_x[p];
                const float fp = fa + u3 * b1, wp = c_gl_w[a] * c_gl_w[p];
                for (int q = 0; q < 5; ++q) {
                    const float b2 = 0.5f * c_gl_x[q];
                    const float fq = fp + u4 * b2, wq = wp * c_gl_w[q], s12 = b1 * b1 + b2 * b2;
                    for (int r = 0; r < 5; ++r) {
                        const float b3 = 0.5f * c_gl_x[r];
                        const float f = fq + u5 * b3 + u6 * (s12 + b3 * b3);
                        if (f > 0.f) s += wq * c_gl_w[r] * f * __logf(f);
                    }
                }
            }
        }
        acc += (double)s;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Marginal in (x1, v1) at 4 x 4 points per (x1 cell, v1 cell) (PrintMarginal
// with f_marg2D_x1v1, MarginalCreation.cpp:35-61, 174-197): at x1 = x_i1 +
// (-1/2 + a/4) dx, v1 = v_j1 + (-1/2 + b/4) dv, the sum over the x2 cells
// and the (v2, v3) cells of dx dv^2 U0 + dv^2 U1 (x1 - x_i1) + dx dv U3 (v1 -
// v_j1) + dx U6 ((v1 - v_j1)^2 + dv^2/6) -- dx times the (v2, v3) marginal.
// out[(i1*4 + a) * (nv*4) + j1*4 + b].
__global__ void k_marginal_x1v1(const double *__restrict__ U, int nx1, int nx2, int nv, double dx, double dv,
                                double lv, double *__restrict__ out) {
    lp_grid_wait();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int npv = nv * 4;
    if (t >= nx1 * 4 * npv) return;
    const int row = t / npv, col = t % npv;
    const int i1 = row / 4, a = row % 4, j1 = col / 4, b = col % 4;
    // positions formed as the reference does (left edge + quarter cells, minus the centre)
    const double xd = __dsub_rn(__dadd_rn(__dmul_rn(((double)i1 - 0.5) + 0.5, dx), __dmul_rn((double)a, dx / 4)),
                                __dmul_rn((double)i1 + 0.5, dx));
    const double v1 = __dadd_rn(__dadd_rn(-lv, __dmul_rn(((double)j1 - 0.5) + 0.5, dv)), __dmul_rn((double)b, dv / 4));
    const double vd = __dsub_rn(v1, __dadd_rn(-lv, __dmul_rn((double)j1 + 0.5, dv)));
    const long long nv3 = (long long)nv * nv * nv;
    double r = 0.;
    for (int i2 = 0; i2 < nx2; ++i2)
        for (int jj = 0; jj < nv * nv; ++jj) {
            const double *u = U + 7 * (((long long)i1 * nx2 + i2) * nv3 + (long long)j1 * nv * nv + jj);
            // the reference's expression order, without FMA
            double t0 = __dmul_rn(__dmul_rn(__dmul_rn(dx, dv), dv), u[0]);
            t0 = __dadd_rn(t0, __dmul_rn(__dmul_rn(__dmul_rn(dv, dv), u[1]), xd));
            t0 = __dadd_rn(t0, __dmul_rn(__dmul_rn(__dmul_rn(dx, dv), u[3]), vd));
            t0 = __dadd_rn(t0, __dmul_rn(__dmul_rn(dx, u[6]), __dadd_rn(__dmul_rn(vd, vd), __ddiv_rn(__dmul_rn(dv, dv), 6.))));
            r = __dadd_rn(r, t0);
        }
    out[t] = r;
}

// ---------------------------------------------------------------- FMA peaks
// Eight independent dependent chains per thread of packed FP32x2 FMAs (two
// FMAs each) or of FP64 FMAs; the result is written so nothing is elided.
__global__ void k_fma_f32(int iters, double *sink) {
    lp_grid_wait();
    unsigned long long a[8], b = pk2(1.0000001f, 0.9999999f), c = pk2(1e-7f, -1e-7f);
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = pk2((float)threadIdx.x + q, (float)blockIdx.x);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = fma2(a[q], b, c);
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) { const float2 v = up2(a[q]); sum += v.x + v.y; }
    if (sum == 1234.5f) sink[0] = sum;
}
__global__ void k_fma_f64(int iters, double *sink) {
    lp_grid_wait();
    double a[8];
    const double b = 1.0000000001, c = 1e-12;
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = threadIdx.x + q + blockIdx.x;
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int q = 0; q < 8; ++q) a[q] = fma(a[q], b, c);
    double sum = 0.;
#pragma unroll
    for (int q = 0; q < 8; ++q) sum += a[q];
    if (sum == 1234.5) sink[0] = sum;
}

// ---------------------------------------------------------------- moments
__global__ void k_moments(const double *__restrict__ U, long long size, long long kend, int nv, double lv,
                          double dv, double *__restrict__ part) {
    lp_grid_wait();
    __shared__ double red[5][256];
    const int t = threadIdx.x;
    double m = 0, a1 = 0, a2 = 0, a3 = 0, ke = 0;
    const long long sv = (long long)nv * nv * nv;
    for (long long k = blockIdx.x * 256LL + t; k < size; k += (long long)gridDim.x * 256) {
        const double *u = U + 7 * k;
        const long long j = k % sv;
        const int j3 = (int)(j % nv), j2 = (int)((j / nv) % nv), j1 = (int)(j / ((long long)nv * nv));
        const double g1 = -lv + (j1 + 0.5) * dv, g2 = -lv + (j2 + 0.5) * dv, g3 = -lv + (j3 + 0.5) * dv;
        m += u[0] + u[6] / 4.;
        a1 += g1 * dv * u[0] + u[3] * dv * dv / 12. + u[6] * g1 * dv / 4.;
        a2 += g2 * dv * u[0] + u[4] * dv * dv / 12. + u[6] * g2 * dv / 4.;
        a3 += g3 * dv * u[0] + u[5] * dv * dv / 12. + u[6] * g3 * dv / 4.;
        if (k < kend) {
            const double tp1 = g1 * g1 + g2 * g2 + g3 * g3;
            ke += u[0] * (tp1 + dv * dv / 4.) * dv + (g1 * u[3] + g2 * u[4] + g3 * u[5]) * dv * dv / 6. +
                  u[6] * (dv * dv * dv * 19. / 240. + tp1 * dv / 4.);
        }
    }
    red[0][t] = m; red[1][t] = a1; red[2][t] = a2; red[3][t] = a3; red[4][t] = ke;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int q = 0; q < 5; ++q) red[q][t] += red[q][t + w];
        __syncthreads();
    }
    if (t < 5) part[blockIdx.x * 5 + t] = red[t][0];
}

}  // namespace

// =============================================================== launchers
cudaError_t launch_lin_weights(const double *eta, const double *shat, const double *cw, const long long *win_off, int n,
                               double scale3, double *W64, float *W32, cudaStream_t st) {
    k_lin_weights<<<n * n * n, 256, 0, st>>>(eta, shat, cw, win_off, n, scale3, W64, W32);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_qlin(const typename V2<R>::t *F, const R *Wl, const long long *win_off, int n, int Bp, double2 *ql,
                        cudaStream_t st) {
    k_qlin<R><<<grid1((long long)n * n * n * Bp, 128), 128, 0, st>>>(F, Wl, win_off, n, Bp, ql);
    return cudaGetLastError();
}
template cudaError_t launch_qlin<double>(const double2 *, const double *, const long long *, int, int, double2 *,
                                         cudaStream_t);
template cudaError_t launch_qlin<float>(const float2 *, const float *, const long long *, int, int, double2 *,
                                        cudaStream_t);

cudaError_t launch_qadd(double2 *q, const double2 *ql, long long total, cudaStream_t st) {
    k_qadd<<<grid1(total, 256), 256, 0, st>>>(q, ql, total);
    return cudaGetLastError();
}

cudaError_t launch_pairs(const double *eta, const double *shat, const double *ahat, const unsigned char *rzero,
                         const double *cw, const int *pair_off, int n, double *P64, float *P32, unsigned *PI,
                         cudaStream_t st) {
    k_pairs<<<n * n * n, 256, 0, st>>>(eta, shat, ahat, rzero, cw, pair_off, n, P64, P32, PI);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_nodes(const double *U, int nv, int n, int c0, int B, int Bp, int slot1, const int *nodecell,
                         const double *nodeoff, double dv, R *f, cudaStream_t st) {
    if (n > 32) return cudaErrorInvalidValue;
    k_nodes_t<R><<<dim3(n * n, Bp / 32), 256, 0, st>>>(U, nv, n, c0, B, Bp, slot1, nodecell, nodeoff, f);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_fwd(const R *f, typename V2<R>::t *t1, typename V2<R>::t *F, const R *M, int n, int Bp,
                       cudaStream_t st, const DftFac *fac) {
    using C = typename V2<R>::t;
    cudaError_t e;
    if constexpr (std::is_same<R, float>::value) {
        if (fac && fac->n == n && fac->sign < 0 && (n == 8 || n == 16 || n == 24)) {
            // axis 2, then axes 1 and 0 through one shared-memory plane
            if ((e = dft_pass<R, R, 0>(f, t1, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr,
                                       nullptr, fac)))
                return e;
            switch (n) {
            case 8: return plane_launch<8, false>(t1, F, *fac, *fac, Bp, 0, 0, 0, nullptr, nullptr, st, Rates{});
            case 16: return plane_launch<16, false>(t1, F, *fac, *fac, Bp, 0, 0, 0, nullptr, nullptr, st, Rates{});
            default: return plane_launch<24, false>(t1, F, *fac, *fac, Bp, 0, 0, 0, nullptr, nullptr, st, Rates{});
            }
        }
    }
    if ((e = dft_pass<R, R, 0>(f, F, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr, nullptr,
                               fac)))
        return e;
    if ((e = dft_pass<R, C, 0>(F, t1, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr, nullptr,
                               fac)))
        return e;
    return dft_pass<R, C, 0>(t1, F, M, n, 0, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr, nullptr,
                             fac);
}

template <typename R>
cudaError_t launch_fwd_complex(const typename V2<R>::t *in, typename V2<R>::t *t1, typename V2<R>::t *F,
                               const R *M, int n, int Bp, cudaStream_t st) {
    using C = typename V2<R>::t;
    cudaError_t e;
    if ((e = dft_pass<R, C, 0>(in, F, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st))) return e;
    if ((e = dft_pass<R, C, 0>(F, t1, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st))) return e;
    return dft_pass<R, C, 0>(t1, F, M, n, 0, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st);
}

template <typename R>
cudaError_t launch_fs_stage(const double2 *q, typename V2<R>::t *t1, typename V2<R>::t *t2, const R *M, int n,
                            int Bp, int stage, double dt, double nu, const R *f, R *qn, R *f1, cudaStream_t st,
                            Rates rates, const float *cf, const double *lamc, const DftFac *fac) {
    using C = typename V2<R>::t;
    cudaError_t e;
    if ((e = dft_pass<R, double2, 0>(q, t1, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, cf, lamc,
                                     fac)))
        return e;
    if ((e = dft_pass<R, C, 0>(t1, t2, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr, nullptr,
                               fac)))
        return e;
    return dft_pass<R, C, 1>(t2, nullptr, M, n, 0, Bp, stage, dt, nu, f, qn, f1, st, rates, nullptr, nullptr, fac);
}

cudaError_t launch_fs_stage32(const float2 *q, float2 *t1, float2 *t2, const float *M, int n, int Bp, int stage,
                              double dt, double nu, const float *f, float *qn, float *f1, cudaStream_t st,
                              Rates rates, const float *cf, const double *lamc, const DftFac *fac) {
    cudaError_t e;
    if ((e = dft_pass<float, float2, 0>(q, t1, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, cf,
                                        lamc, fac)))
        return e;
    if ((e = dft_pass<float, float2, 0>(t1, t2, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr,
                                        nullptr, fac)))
        return e;
    return dft_pass<float, float2, 1>(t2, nullptr, M, n, 0, Bp, stage, dt, nu, f, qn, f1, st, rates, nullptr, nullptr,
                                      fac);
}

cudaError_t launch_fs_fwd32(const float2 *q, float2 *t1, float2 *t2, float2 *F, const float *Mi, const float *M,
                            int n, int Bp, int stage, double dt, double nu, const float *f, float *qn, float *f1,
                            cudaStream_t st, Rates rates, const float *cf, const double *lamc, const DftFac *fi,
                            const DftFac *ff) {
    cudaError_t e;
    if (fi && ff && fi->n == n && ff->n == n && fi->sign > 0 && ff->sign < 0 &&
        (n == 8 || n == 16 || n == 24 || n == 32)) {
        if ((e = dft_pass<float, float2, 0>(q, t1, Mi, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, cf,
                                            lamc, fi)))
            return e;
        if (n <= 24) {
            // axes 1 and 0 of the stage through one shared-memory plane
            switch (n) {
            case 8: e = plane_launch<8, true>(t1, t2, *fi, *ff, Bp, stage, dt, nu, f, qn, st, rates); break;
            case 16: e = plane_launch<16, true>(t1, t2, *fi, *ff, Bp, stage, dt, nu, f, qn, st, rates); break;
            default: e = plane_launch<24, true>(t1, t2, *fi, *ff, Bp, stage, dt, nu, f, qn, st, rates); break;
            }
            if (e) return e;
            return dft_pass<float, float2, 0>(t2, F, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{},
                                              nullptr, nullptr, ff);
        }
        if ((e = dft_pass<float, float2, 0>(t1, t2, Mi, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{},
                                            nullptr, nullptr, fi)))
            return e;
        constexpr int PY = 4;
        const dim3 grid(n * n / PY, Bp / 32), block(32, PY);
        switch (n) {
        case 8: k_fftf_fs<8, PY><<<grid, block, 0, st>>>(t2, t1, *fi, *ff, Bp, stage, (float)dt, (float)nu, f, qn, rates.nu, rates.dt); break;
        case 16: k_fftf_fs<16, PY><<<grid, block, 0, st>>>(t2, t1, *fi, *ff, Bp, stage, (float)dt, (float)nu, f, qn, rates.nu, rates.dt); break;
        case 24: k_fftf_fs<24, PY><<<grid, block, 0, st>>>(t2, t1, *fi, *ff, Bp, stage, (float)dt, (float)nu, f, qn, rates.nu, rates.dt); break;
        default: k_fftf_fs<32, PY><<<grid, block, 0, st>>>(t2, t1, *fi, *ff, Bp, stage, (float)dt, (float)nu, f, qn, rates.nu, rates.dt); break;
        }
        if ((e = cudaGetLastError())) return e;
        if ((e = dft_pass<float, float2, 0>(t1, t2, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{},
                                            nullptr, nullptr, ff)))
            return e;
        return dft_pass<float, float2, 0>(t2, F, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st, Rates{}, nullptr,
                                          nullptr, ff);
    }
    // without the factors: the inverse passes into f1, then the forward transform
    if ((e = launch_fs_stage32(q, t1, t2, Mi, n, Bp, stage, dt, nu, f, qn, f1, st, rates, cf, lamc))) return e;
    return launch_fwd<float>(f1, t1, F, M, n, Bp, st);
}

template <typename R>
cudaError_t launch_fs_full(const double2 *q, typename V2<R>::t *t1, typename V2<R>::t *t2,
                           typename V2<R>::t *out, const R *M, int n, int Bp, cudaStream_t st) {
    using C = typename V2<R>::t;
    cudaError_t e;
    if ((e = dft_pass<R, double2, 0>(q, t1, M, n, 2, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st))) return e;
    if ((e = dft_pass<R, C, 0>(t1, t2, M, n, 1, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st))) return e;
    return dft_pass<R, C, 0>(t2, out, M, n, 0, Bp, 0, 0, 0, nullptr, nullptr, nullptr, st);
}

template <typename R>
cudaError_t launch_computeq(const typename V2<R>::t *F, const R *P, const unsigned *PI, const int *pair_off,
                            int n3, int Bp, double2 *q, cudaStream_t st) {
    dim3 grid((n3 + 3) / 4, Bp / 32);
    k_computeq<R><<<grid, 128, 0, st>>>(F, P, PI, pair_off, n3, Bp, q);
    return cudaGetLastError();
}

bool lines_supported(int n) { return n == 8 || n == 16 || n == 24 || n == 32; }

namespace {
template <int N> long long lines_offsets(std::vector<long long> &line_off) {
    constexpr int KT = LinesCfg<N>::KT, h = N / 2, TP = pp_floats<N, KT>();
    line_off.assign((size_t)N * N + 1, 0);
    for (int ij = 0; ij < N * N; ++ij) {
        const int i = ij / N, j = ij % N;
        const int ni = i < h ? i + h + 1 : 3 * h - 1 - i, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
        line_off[ij + 1] = line_off[ij] + (long long)((ni * nj + 1) / 2) * TP;
    }
    // then the lines in order of decreasing plane-pair count: blocks are
    // dispatched longest first, so the last wave holds the short lines
    std::vector<int> order(N * N);
    for (int ij = 0; ij < N * N; ++ij) order[ij] = ij;
    std::stable_sort(order.begin(), order.end(), [](int a, int b) {
        auto npp = [](int ij) {
            const int i = ij / N, j = ij % N;
            const int ni = i < h ? i + h + 1 : 3 * h - 1 - i, nj = j < h ? j + h + 1 : 3 * h - 1 - j;
            return (ni * nj + 1) / 2;
        };
        return npp(a) > npp(b);
    });
    for (int r = 0; r < N * N; ++r) line_off.push_back(order[r]);
    return line_off[(size_t)N * N];
}
}  // namespace

long long lines_table_floats(int n, std::vector<long long> &line_off) {
    switch (n) {
    case 8: return lines_offsets<8>(line_off);
    case 16: return lines_offsets<16>(line_off);
    case 24: return lines_offsets<24>(line_off);
    case 32: return lines_offsets<32>(line_off);
    default: return 0;
    }
}

cudaError_t launch_lines_table(const double *eta, const double *shat, const double *ahat, const unsigned char *rzero,
                               const double *cw, const long long *line_off, int n, float *W, cudaStream_t st) {
    switch (n) {
    case 8: k_lines_table<8><<<64, 256, 0, st>>>(eta, shat, ahat, rzero, cw, line_off, W); break;
    case 16: k_lines_table<16><<<256, 256, 0, st>>>(eta, shat, ahat, rzero, cw, line_off, W); break;
    case 24: k_lines_table<24><<<576, 256, 0, st>>>(eta, shat, ahat, rzero, cw, line_off, W); break;
    case 32: k_lines_table<32><<<1024, 256, 0, st>>>(eta, shat, ahat, rzero, cw, line_off, W); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

namespace {
template <int N, int T, int LW>
void launch_tiles(const float2 *F, const float *W, const long long *line_off, int Bp, double2 *q, cudaStream_t st,
                  cudaStream_t st_odd) {
    constexpr int NT = N / LinesCfg<N>::KT;
    if constexpr (T < NT) {
        const unsigned blocks = (unsigned)((long long)N * N * (Bp / 32));
        constexpr size_t smem = lines_smem_bytes<N, T, LW>();
        static bool attr_set = false;  // one attribute call per instantiation
        if (!attr_set) {
            cudaFuncSetAttribute(k_cq_lines<N, T, LW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr_set = true;
        }
        k_cq_lines<N, T, LW><<<blocks, 32 * LW, smem, (T & 1) ? st_odd : st>>>(F, W, line_off, Bp, q);
        launch_tiles<N, T + 1, LW>(F, W, line_off, Bp, q, st, st_odd);
    }
}

template <int LW>
cudaError_t computeq_lines(const float2 *F, const float *W, const long long *line_off, int n, int Bp, double2 *q,
                           cudaStream_t st, cudaStream_t st_odd) {
    switch (n) {
    case 8: launch_tiles<8, 0, LW>(F, W, line_off, Bp, q, st, st_odd); break;
    case 16: launch_tiles<16, 0, LW>(F, W, line_off, Bp, q, st, st_odd); break;
    case 24: launch_tiles<24, 0, LW>(F, W, line_off, Bp, q, st, st_odd); break;
    case 32: launch_tiles<32, 0, LW>(F, W, line_off, Bp, q, st, st_odd); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_computeq_lines(const float2 *F, const float *W, const long long *line_off, int n, int Bp,
                                  double2 *q, cudaStream_t st, int warps, cudaStream_t st_odd) {
    if (!st_odd) st_odd = st;
    if (warps == 4) return computeq_lines<4>(F, W, line_off, n, Bp, q, st, st_odd);
    if (warps == 2) return computeq_lines<2>(F, W, line_off, n, Bp, q, st, st_odd);
    return cudaErrorInvalidValue;
}

cudaError_t launch_conserve(double2 *q, const double *c1, const double *c2, const double *cct_inv, int n3, int Bp,
                            double *part, int nchunk, double *lam, cudaStream_t st, bool apply) {
    k_cons_partial<double2><<<dim3(nchunk, Bp / 32), dim3(32, 8), 0, st>>>(q, c1, c2, n3, Bp, nchunk, part);
    k_cons_lambda<<<Bp, 160, 0, st>>>(part, nchunk, cct_inv, Bp, lam);
    if (apply) k_cons_apply<<<grid1((long long)n3 * Bp, 256), 256, 0, st>>>(q, c1, c2, lam, n3, Bp);
    return cudaGetLastError();
}

cudaError_t launch_cons_lambda(const double *part, int nchunk, const double *cct_inv, int Bp, double *lam,
                               cudaStream_t st) {
    k_cons_lambda<<<Bp, 160, 0, st>>>(part, nchunk, cct_inv, Bp, lam);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_project(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, double nu,
                           const R *tfac, int n, int nv, int Bp, int B, int c0, const double *U, int ustride,
                           const int *uslot, double dt, double scalev, double scaleL, double scale3,
                           typename V2<R>::t *Qc, typename V2<R>::t *Y, typename V2<R>::t *Z, double *dU,
                           cudaStream_t st, Rates rates) {
    const long long n3 = (long long)n * n * n;
    k_qcomb<R><<<grid1(n3 * Bp, 256), 256, 0, st>>>(q0, q1, q2, q3, nu, n3 * Bp, Bp, rates.nu, Qc);
    const int nch = (nv + JB - 1) / JB;
    k_proj3<R><<<grid1((long long)n * n * nch * Bp, 128), 128, 0, st>>>(Qc, tfac, n, nv, Bp, Y);
    k_proj2<R><<<grid1((long long)n * nv * nch * Bp, 128), 128, 0, st>>>(Y, tfac, n, nv, Bp, Z);
    const double kfac = 1. / scalev / scaleL / scale3;
    int4 us = make_int4(uslot[0], uslot[1], uslot[2], uslot[3]);
    k_proj1<R><<<grid1((long long)nv * nv * nch * Bp, 128), 128, 0, st>>>(Z, tfac, n, nv, Bp, B, c0, U, ustride, us,
                                                                             uslot[4], dt, kfac, rates.dt, dU);
    return cudaGetLastError();
}

cudaError_t launch_moment_target(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3,
                                 double nu, const double *gmom, int n3, int Bp, int nchunk, double *tpart,
                                 cudaStream_t st, Rates rates) {
    k_mom_target<<<dim3(nchunk, Bp / 32), dim3(32, 8), 0, st>>>(q0, q1, q2, q3, nu, rates.nu, gmom, n3, Bp, nchunk,
                                                               tpart);
    return cudaGetLastError();
}

cudaError_t launch_moment_finish(const double *tpart, int nchunk, const double *U, int nv, double dv, double lv,
                                 int c0, int B, int Bp, int nrc, double *apart, const double *gm_inv, double scale,
                                 double kfac, double *lam, double *dU, cudaStream_t st, Rates rates, bool apply) {
    const MomRow mr = mom_row(dv);
    k_mom_actual<<<dim3(nrc, B), 256, 0, st>>>(dU, U, nv, dv, lv, mr, c0, nrc, apart);
    k_mom_lambda<<<(B + 3) / 4, 128, 0, st>>>(tpart, nchunk, apart, nrc, (long long)nrc * 5, 5, 1, gm_inv, scale,
                                              kfac, rates.dt, B, Bp, lam);
    if (apply) {
        const long long nrec = (long long)B * nv * nv * nv;
        k_mom_apply<<<grid1(nrec, 256), 256, 0, st>>>(dU, lam, nv, dv, lv, mr, nrec);
    }
    return cudaGetLastError();
}

int project_inc_blocks(int n, int nv) {
    if (n == 8 || n == 16 || n == 24 || n == 32) return (nv * nv + kPj1Pen - 1) / kPj1Pen;  // k_pj1
    return (nv * nv * ((nv + JBI - 1) / JBI) + kIncWarps - 1) / kIncWarps;
}

cudaError_t launch_project_inc(const double2 *q0, const double2 *q1, const double2 *q2, const double2 *q3, double nu,
                               const float *tfac, int n, int nv, int Bp, int B, double dt, double scalev,
                               double scaleL, double scale3, float2 *Qc, float2 *Y, float2 *Z, float *Inc,
                               double *part, double lv, double dv, cudaStream_t st, Rates rates, const float *cf,
                               const double *lam4, float2 *const *q32, const float *tc_tab, int *tc_err,
                               const float *tc_tab1) {
    const double kfac = 1. / scalev / scaleL / scale3;
    switch (n) {
    case 8: return launch_pj<8>(q0, q1, q2, q3, nu, tfac, nv, Bp, B, dt, kfac, Y, Z, Inc, part, lv, dv, st, rates, cf, lam4, q32, tc_tab, tc_err, tc_tab1);
    case 16: return launch_pj<16>(q0, q1, q2, q3, nu, tfac, nv, Bp, B, dt, kfac, Y, Z, Inc, part, lv, dv, st, rates, cf, lam4, q32, tc_tab, tc_err, tc_tab1);
    case 24: return launch_pj<24>(q0, q1, q2, q3, nu, tfac, nv, Bp, B, dt, kfac, Y, Z, Inc, part, lv, dv, st, rates, cf, lam4, q32, tc_tab, tc_err, tc_tab1);
    case 32: return launch_pj<32>(q0, q1, q2, q3, nu, tfac, nv, Bp, B, dt, kfac, Y, Z, Inc, part, lv, dv, st, rates, cf, lam4, q32, tc_tab, tc_err, tc_tab1);
    default: break;
    }
    if (cf || q32) return cudaErrorInvalidValue;  // lazy conservation needs the register-pencil passes
    const long long n3 = (long long)n * n * n;
    k_qcomb<float><<<grid1(n3 * Bp, 256), 256, 0, st>>>(q0, q1, q2, q3, nu, n3 * Bp, Bp, rates.nu, Qc);
    const int nch = (nv + JB - 1) / JB;
    k_proj3<float><<<grid1((long long)n * n * nch * Bp, 128), 128, 0, st>>>(Qc, tfac, n, nv, Bp, Y);
    k_proj2<float><<<grid1((long long)n * nv * nch * Bp, 128), 128, 0, st>>>(Y, tfac, n, nv, Bp, Z);
    k_proj1_inc<<<dim3(project_inc_blocks(n, nv), Bp / 32), 32 * kIncWarps, 0, st>>>(
        Z, tfac, n, nv, Bp, B, dt, kfac, rates.dt, dv, lv, mom_row(dv), Inc, part);
    return cudaGetLastError();
}

cudaError_t launch_lambda_inc(const double *tpart, int nchunk, const double *part, int n, int nv, int B, int Bp,
                              const double *gm_inv, double scale, double kfac, double *lam, cudaStream_t st,
                              Rates rates) {
    k_lambda_inc<<<B, 160, 0, st>>>(tpart, nchunk, part, project_inc_blocks(n, nv), gm_inv, scale, kfac, rates.dt, Bp,
                                    lam);
    return cudaGetLastError();
}

cudaError_t launch_scatter_inc(const float *Inc, int Bp, int B, int nv, int c0, double *U, const double *lam,
                               double dv, double lv, cudaStream_t st) {
    const long long nv3 = (long long)nv * nv * nv;
    const cudaError_t e = cudaFuncSetAttribute(k_scatter_inc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kScatSmem);
    if (e != cudaSuccess) return e;
    k_scatter_inc<<<dim3((unsigned)((nv3 + kScatRec - 1) / kScatRec), Bp / 32), 256, kScatSmem, st>>>(
        Inc, Bp, B, nv, c0, U, lam, dv, lv, mom_row(dv));
    return cudaGetLastError();
}

cudaError_t launch_scatter(const double *dU, int nv3, int c0, int B, double *U, cudaStream_t st, const double *lam,
                           int nv, double dv, double lv) {
    const long long nrec = (long long)B * nv3;
    k_scatter<<<grid1(nrec, 256), 256, 0, st>>>(dU, nrec, (long long)c0 * nv3, U, lam, nv, dv, lv, mom_row(dv));
    return cudaGetLastError();
}

cudaError_t launch_charge(const double *U, int ncell, int nv3, double scalev, double *rt, cudaStream_t st) {
    k_charge_seq<<<ncell, 256, 0, st>>>(U, nv3, scalev, rt);
    return cudaGetLastError();
}

cudaError_t launch_state_f32(const double *U, long long size, float *Uf, double *part, cudaStream_t st) {
    k_state_f32<<<grid1(size, 128), 128, 0, st>>>(U, size, Uf, part);
    return cudaGetLastError();
}

cudaError_t launch_poisson(const PoissonDev &pd, const double *rt, int npart, double *b, double *potc, double *phix,
                           double *phiy, double *fields, cudaStream_t st) {
    // the band solve is a dependent chain over ndim columns: read the band
    // factors from shared memory when they fit
    PoissonDev d = pd;
    const size_t base = (sizeof(double) + sizeof(int)) * (size_t)pd.ndim;
    const size_t band = sizeof(double) * (size_t)pd.ldab * pd.ndim;
    d.staged = (base + band <= 200 * 1024) ? 1 : 0;
    const size_t smem = base + (d.staged ? band : 0);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_poisson, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_poisson<<<1, 256, smem, st>>>(d, rt, npart, b, potc, phix, phiy, fields);
    return cudaGetLastError();
}

cudaError_t launch_flux_stage(const AdvectDev &ad, const double *U0, const double *Us, const float *Uin_f32,
                              const double *fields, int stage, double *Uout, float *Uout_f32, double *part,
                              cudaStream_t st) {
    if (ad.size >= (1ll << 31)) return cudaErrorInvalidValue;  // 32-bit record indexing in flux_rhs
    if (Uin_f32)
        k_flux<float, float><<<grid1(ad.size, 128), 128, 0, st>>>(ad, U0, Us, Uin_f32, fields, stage, Uout, Uout_f32,
                                                                 part);
    else
        k_flux<double, double><<<grid1(ad.size, 128), 128, 0, st>>>(ad, U0, Us, Us, fields, stage, Uout, Uout_f32,
                                                                   part);
    return cudaGetLastError();
}

cudaError_t launch_state_f32_grp(const double *U, long long size, float *Uf, double *part, cudaStream_t st) {
    k_state_f32_grp<<<grid1(size, 512), 128, 0, st>>>(U, size, Uf, part);
    return cudaGetLastError();
}

cudaError_t launch_flux_inc(const AdvectDev &ad, int stage, const float *Uin, const float *Uf0,
                            const double *fields, float *S, float *Uoutf, double *U, float *ipart,
                            cudaStream_t st) {
    if (ad.size >= (1ll << 31)) return cudaErrorInvalidValue;  // 32-bit record indexing in flux_rhs
    const dim3 g = grid1(ad.size, 128);
    if (stage == 0) k_flux_inc<0><<<g, 128, 0, st>>>(ad, Uin, Uf0, fields, S, Uoutf, U, ipart);
    else if (stage == 1) k_flux_inc<1><<<g, 128, 0, st>>>(ad, Uin, Uf0, fields, S, Uoutf, U, ipart);
    else k_flux_inc<2><<<g, 128, 0, st>>>(ad, Uin, Uf0, fields, S, Uoutf, U, ipart);
    return cudaGetLastError();
}

cudaError_t launch_poisson_dense(const PoissonDev &pd, const double *base, const float *inc, double iscale,
                                 int npart, const double *Ainv, double *b, double *potc, double *phix,
                                 double *phiy, double *fields, cudaStream_t st) {
    const int nc = pd.nx * pd.ny;
    k_prhs<<<(nc + 7) / 8, 256, 0, st>>>(pd, base, inc, iscale, npart, b);
    k_psolve_dense<<<(pd.ndim + 7) / 8, 256, 0, st>>>(Ainv, b, pd.ndim, potc);
    k_pfields<<<(nc + 127) / 128, 128, 0, st>>>(pd, potc, phix, phiy, fields);
    return cudaGetLastError();
}

cudaError_t launch_entropy(const double *U, long long kend, double *part, int nblk, cudaStream_t st) {
    k_entropy<<<nblk, 256, 0, st>>>(U, kend, part);
    return cudaGetLastError();
}

cudaError_t launch_marginal_x1v1(const double *U, int nx1, int nx2, int nv, double dx, double dv, double lv,
                                 double *out, cudaStream_t st) {
    const int total = nx1 * 4 * nv * 4;
    k_marginal_x1v1<<<(total + 127) / 128, 128, 0, st>>>(U, nx1, nx2, nv, dx, dv, lv, out);
    return cudaGetLastError();
}

cudaError_t launch_fma_peak(bool fp64, int blocks, int iters, double *sink, cudaStream_t st) {
    if (fp64) k_fma_f64<<<blocks, 256, 0, st>>>(iters, sink);
    else k_fma_f32<<<blocks, 256, 0, st>>>(iters, sink);
    return cudaGetLastError();
}

cudaError_t launch_moments(const double *U, long long size, long long kend, int nv, double lv, double dv,
                           double *part, int nblk, cudaStream_t st) {
    k_moments<<<nblk, 256, 0, st>>>(U, size, kend, nv, lv, dv, part);
    return cudaGetLastError();
}

// explicit instantiations
#define LP_INST(R)                                                                                              \
    template cudaError_t launch_nodes<R>(const double *, int, int, int, int, int, int, const int *,             \
                                         const double *, double, R *, cudaStream_t);                            \
    template cudaError_t launch_fwd<R>(const R *, V2<R>::t *, V2<R>::t *, const R *, int, int, cudaStream_t,    \
                                       const DftFac *);                                                         \
    template cudaError_t launch_fwd_complex<R>(const V2<R>::t *, V2<R>::t *, V2<R>::t *, const R *, int, int,   \
                                               cudaStream_t);                                                   \
    template cudaError_t launch_fs_stage<R>(const double2 *, V2<R>::t *, V2<R>::t *, const R *, int, int, int,  \
                                            double, double, const R *, R *, R *, cudaStream_t, Rates,           \
                                            const float *, const double *, const DftFac *);                     \
    template cudaError_t launch_fs_full<R>(const double2 *, V2<R>::t *, V2<R>::t *, V2<R>::t *, const R *, int, \
                                           int, cudaStream_t);                                                  \
    template cudaError_t launch_computeq<R>(const V2<R>::t *, const R *, const unsigned *, const int *, int,    \
                                            int, double2 *, cudaStream_t);                                      \
    template cudaError_t launch_project<R>(const double2 *, const double2 *, const double2 *, const double2 *,  \
                                           double, const R *, int, int, int, int, int, const double *, int,     \
                                           const int *, double, double, double, double, V2<R>::t *,             \
                                           V2<R>::t *, V2<R>::t *, double *, cudaStream_t, Rates);
LP_INST(double)
LP_INST(float)
#undef LP_INST

}  // namespace lp
