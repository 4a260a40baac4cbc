// ComputeQ of the mixed path as a sum of seven windowed convolutions.
//
// The reference's weight (source/collisionRoutines_1.cpp:30-69, used at
// C:739-822) is gHat3(xi, omega) = ahat(omega) - d^T Shat(omega) d with
// d = eta(xi) - eta(omega).  On the uniform eta grid d = (u - h) h_eta where
// u = xi + h - omega is the index of the second factor F(u), so every term
// of the windowed sum
//
//     Qhat(xi) = sum_omega cw(omega) gHat3(xi, omega) F(omega) F(u)
//
// splits into a function of omega times a function of u:
//
//     Qhat = sum_p (a_p * b_p)(xi + h),   p = 0..6,
//     a_0 = cw ahat F,                    b_0 = F,
//     a_ij = -c_ij h_eta^2 cw Shat_ij F,  b_ij = (u_i - h)(u_j - h) F,
//
// with c_ii = 1, c_ij = 2 (i < j) and * the linear convolution on the n^3
// grid.  The output window xi + h in [h, n + h) of a linear convolution of
// two length-n sequences is free of wrap-around on a cyclic grid of
// M = 3n/2 points, so along axes 2 and 3 the convolutions are products of
// M-point DFTs of the zero-padded arrays, and along axis 1 they are summed
// directly (the direct sum along one axis costs less than a third of the
// forward and inverse transforms it replaces):
//
//   X1  axis-3 DFT of the 7 a-arrays and of F (u3-h)^e, e = 0, 1, 2;
//   X2  axis-2 DFT of the 7 a-arrays and of the 6 (e2, e3) b-combinations
//       (X1 and X2 in one kernel, the X1 outputs held in shared memory);
//   Y   per (k2, k3): sum_p sum_l a_p(l) (u1-h)^e1 b_p(u1), u1 = i + h - l;
//   Z1  inverse axis-2 DFT, only the n outputs xi2 + h;
//   Z2  inverse axis-3 DFT, only the n outputs xi3 + h, written as FP64.
//
// The shift by h of the output window is the factor exp(2 pi i k h / M) =
// exp(2 pi i k / 3) on the a-side spectra.  The M-point DFTs factor as
// M = 6 S (S = n/4): S six-point DFTs of the 4 non-zero inputs, twiddles,
// six S-point DFTs; the inverse is the conjugate transpose with only 4 of
// the 6 outputs of its last stage kept.  A thread transforms one pencil of
// one cell; the 32 lanes of a warp are 32 cells, so every load and store is
// coalesced on the cell-minor arrays.  Arithmetic is FP32.
#include "lp_kernels.cuh"
#include "lp_dev.cuh"
#include "lp_fft.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace lp {
namespace {

constexpr int kPY = 4;  // pencils per block (blockDim.y); blockDim.x = 32 cells

// X1 and X2 fused per (axis-1 plane l, CB cells, X1 array t = blockIdx.z):
// the plane's axis-3 DFTs go to shared memory ([m][k3][CB cells]) and the
// axis-2 DFTs read them from there, so the X1 outputs never reach DRAM.
// blockDim = (CB cells, PY threads), each thread taking pencils ty,
// ty + PY, ... of both phases.
template <int N, int PY, int CB>
__global__ void __launch_bounds__(CB * PY) k_fq_x12(const float2 *__restrict__ F, const float *__restrict__ C,
                                                    int Bp, int c0, float2 *__restrict__ X, int Bs, FftTw tw) {
    lp_grid_wait();
    constexpr int n = N, h = N / 2, M = 3 * N / 2;
    extern __shared__ float2 t3[];  // [m][k3][CB]
    const int tx = threadIdx.x, ty = threadIdx.y, l = blockIdx.x, t = blockIdx.z;
    const int cell = blockIdx.y * CB + tx;
    const size_t as = (size_t)n * M * M * Bs, os = (size_t)M * Bs;  // array and k2 strides of X
    {
        // axis-3 DFTs of the (l, m) pencils of array t
        for (int m = ty; m < n; m += PY) {
            const float2 *src = F + ((size_t)l * n + m) * n * Bp + c0 + cell;
            float2 x[N];
            float2 *row = t3 + m * M * CB + tx;
            auto put = [&](int k, float2 v) { row[k * CB] = v; };
            if (t < 7) {
                // n contiguous, 16-byte aligned weights: n / 4 vector loads
                const float4 *cp =
                    reinterpret_cast<const float4 *>(C + (size_t)t * n * n * n + ((size_t)l * n + m) * n);
#pragma unroll
                for (int q4 = 0; q4 < n / 4; ++q4) {
                    const float4 w = __ldg(cp + q4);
                    x[4 * q4] = cscale(src[(size_t)(4 * q4) * Bp], w.x);
                    x[4 * q4 + 1] = cscale(src[(size_t)(4 * q4 + 1) * Bp], w.y);
                    x[4 * q4 + 2] = cscale(src[(size_t)(4 * q4 + 2) * Bp], w.z);
                    x[4 * q4 + 3] = cscale(src[(size_t)(4 * q4 + 3) * Bp], w.w);
                }
                fwd_pencil_st<N, true>(x, tw.fa, put);
            } else {
#pragma unroll
                for (int q = 0; q < n; ++q) x[q] = cscale(src[(size_t)q * Bp], poww(q, h, t - 7));
                fwd_pencil_st<N, false>(x, tw.fw, put);
            }
        }
        __syncthreads();
        // axis-2 DFTs of the (l, k3) pencils into X
        for (int k3 = ty; k3 < M; k3 += PY) {
            float2 x[N];
#pragma unroll
            for (int m = 0; m < n; ++m) x[m] = t3[(m * M + k3) * CB + tx];
            float2 *dst = X + ((size_t)l * M * M + k3) * Bs + cell;
            if (t < 7) {
                float2 *d = dst + t * as;
                fwd_pencil_st<N, true>(x, tw.fa, [&](int k, float2 v) { d[(size_t)k * os] = v; });
            } else {
                // b-side: the X1 array 7 + e3 gives the combinations (e2, e3)
                // at arrays 7 (0,0), 8 (2,0), 10 (1,0) | 11 (0,1), 12 (1,1) | 9 (0,2)
                const int e3 = t - 7;
                const int no = e3 == 0 ? 3 : (e3 == 1 ? 2 : 1);
                for (int o = 0; o < no; ++o) {
                    const int e2 = e3 == 0 ? (o == 0 ? 0 : (o == 1 ? 2 : 1)) : (e3 == 1 ? o : 0);
                    const int arr = e3 == 0 ? (o == 0 ? 7 : (o == 1 ? 8 : 10)) : (e3 == 1 ? 11 + o : 9);
                    float2 xw[N];
#pragma unroll
                    for (int m = 0; m < n; ++m) xw[m] = e2 ? cscale(x[m], poww(m, h, e2)) : x[m];
                    float2 *d = dst + arr * as;
                    fwd_pencil_st<N, false>(xw, tw.fw, [&](int k, float2 v) { d[(size_t)k * os] = v; });
                }
            }
        }
    }
}

// Y: the direct convolution along axis 1 for the outputs i in
// [I0, I0 + NI) of one (k2, k3) pencil, summed over the seven pairs.
// Pair p takes the b-array Y00 (p = 0, 1), Y20, Y02, Y10, Y01, Y11 (p = 2..6)
// weighted by (u1 - h)^e1, e1 = 2 for p = 1, 1 for p = 4, 5, else 0.
// The 2n values of a pair (b-array along u1, a-array along l) are copied
// into shared memory with cp.async, two pairs in flight: the copies of pair
// p + 1 run while pair p is summed.  Every thread copies and reads only its
// own column (sm + v * threads), so no block barrier is needed.
// Complex products use packed FMAs with split accumulators:
// A += Re(a) b, B += Im(a) b, a b = (A.x - B.y, A.y + B.x).
template <int N>
__device__ __forceinline__ void y_issue(const float2 *__restrict__ base, size_t ps, int p, float2 *sm, int nt) {
    const int sy = (p == 0 || p == 1) ? 7 : p + 6;
#pragma unroll
    for (int u = 0; u < N; ++u) cp_async8(sm + u * nt, base + ((size_t)sy * N + u) * ps);
#pragma unroll
    for (int l = 0; l < N; ++l) cp_async8(sm + (N + l) * nt, base + ((size_t)p * N + l) * ps);
    cp_async_commit();
}

template <int N, int NI, int I0>
__device__ __forceinline__ void y_part(const float2 *__restrict__ base, size_t ps, float2 *__restrict__ dst,
                                       size_t os, float2 *sm, int nt) {
    constexpr int n = N, h = N / 2;
    unsigned long long A[NI], B[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) A[i] = B[i] = 0ull;
    y_issue<N>(base, ps, 0, sm, nt);
#pragma unroll 1
    for (int p = 0; p < 7; ++p) {
        float2 *cur = sm + (p & 1) * 2 * N * nt;
        if (p + 1 < 7) {
            y_issue<N>(base, ps, p + 1, sm + ((p + 1) & 1) * 2 * N * nt, nt);
            cp_async_wait1();
        } else {
            cp_async_wait0();
        }
        const int e1 = (p == 1) ? 2 : ((p == 4 || p == 5) ? 1 : 0);
        unsigned long long yb[N];
#pragma unroll
        for (int u = 0; u < n; ++u) {
            const float2 v = cscale(cur[u * nt], poww(u, h, e1));
            yb[u] = pk2(v.x, v.y);
        }
#pragma unroll
        for (int l = 0; l < n; ++l) {
            // outputs i with u = i + h - l in [0, n)
            if (l - h >= I0 + NI || l + h <= I0) continue;
            const float2 a = cur[(N + l) * nt];
            const unsigned long long ar = pk2(a.x, a.x), ai = pk2(a.y, a.y);
#pragma unroll
            for (int ii = 0; ii < NI; ++ii) {
                const int u = I0 + ii + h - l;
                if (u >= 0 && u < n) {
                    A[ii] = fma2(ar, yb[u], A[ii]);
                    B[ii] = fma2(ai, yb[u], B[ii]);
                }
            }
        }
    }
#pragma unroll
    for (int ii = 0; ii < NI; ++ii) {
        const float2 a = up2(A[ii]), b = up2(B[ii]);
        dst[(size_t)ii * os] = make_float2(a.x - b.y, a.y + b.x);
    }
}

// blockIdx.z selects the output half when NI = N / 2.  G is [n][M][M][Bs].
// Dynamic shared memory: 2 stages x 2N values x blockDim threads.
template <int N, int NI, int PY>
__global__ void __launch_bounds__(32 * PY) k_fq_y(const float2 *__restrict__ X, int Bs, float2 *__restrict__ G) {
    lp_grid_wait();
    constexpr int M = 3 * N / 2;
    extern __shared__ float2 ysm[];
    const int pen = blockIdx.x * PY + threadIdx.y;
    if (pen >= M * M) return;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    const size_t ps = (size_t)M * M * Bs;  // stride of the axis-1 index
    const float2 *base = X + (size_t)pen * Bs + cell;
    float2 *dst = G + (size_t)pen * Bs + cell;
    float2 *sm = ysm + threadIdx.y * 32 + threadIdx.x;
    constexpr int nt = 32 * PY;
    if (NI == N || blockIdx.z == 0) {
        y_part<N, NI, 0>(base, ps, dst, ps, sm, nt);
    } else {
        y_part<N, NI, (NI < N ? NI : 0)>(base, ps, dst + (size_t)NI * ps, ps, sm, nt);
    }
}

// Z1: inverse axis-2 DFT of the (i, k3) pencils, outputs xi2 in [0, n).
// H is [n][n][M][Bs].
template <int N>
__global__ void __launch_bounds__(32 * kPY) k_fq_z1(const float2 *__restrict__ G, int Bs, float2 *__restrict__ H,
                                                    FftTw tw) {
    lp_grid_wait();
    constexpr int n = N, M = 3 * N / 2;
    const int pen = blockIdx.x * kPY + threadIdx.y;
    if (pen >= n * M) return;
    const int i = pen / M, k3 = pen - i * M;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    const float2 *src = G + ((size_t)i * M * M + k3) * Bs + cell;
    float2 g[M], x[N];
#pragma unroll
    for (int k = 0; k < M; ++k) g[k] = src[(size_t)k * M * Bs];
    inv_pencil<N>(g, x, tw.iv);
    float2 *dst = H + ((size_t)i * n * M + k3) * Bs + cell;
#pragma unroll
    for (int j = 0; j < n; ++j) dst[(size_t)j * M * Bs] = x[j];
}

// Z2: inverse axis-3 DFT of the (i, j) pencils into q (stride Bp), FP64
// or FP32 complex.  CONS (FP32 output): each block's constraint sums of its
// outputs (ConsFused).
template <int N, typename QT, bool CONS>
__global__ void __launch_bounds__(32 * kPY) k_fq_z2(const float2 *__restrict__ H, int Bs, QT *__restrict__ q,
                                                    int Bp, int c0, FftTw tw, ConsFused cons) {
    lp_grid_wait();
    constexpr int n = N, M = 3 * N / 2;
    const int pen = blockIdx.x * kPY + threadIdx.y;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    float t[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (pen < n * n) {
        const float2 *src = H + (size_t)pen * M * Bs + cell;
        float2 g[M], x[N];
#pragma unroll
        for (int k = 0; k < M; ++k) g[k] = src[(size_t)k * Bs];
        inv_pencil<N>(g, x, tw.iv);
        QT *dst = q + (size_t)pen * n * Bp + c0 + cell;
#pragma unroll
        for (int k = 0; k < n; ++k) {
            if constexpr (std::is_same<QT, double2>::value) dst[(size_t)k * Bp] = make_double2((double)x[k].x, (double)x[k].y);
            else dst[(size_t)k * Bp] = x[k];
        }
        if constexpr (CONS) {
            constexpr int n3 = N * N * N;
            const float *cr = cons.cf + pen * n;
#pragma unroll
            for (int k = 0; k < n; ++k) {
                t[0] = fmaf(x[k].x, cr[k], t[0]);
                t[1] = fmaf(x[k].y, cr[n3 + k], t[1]);
                t[2] = fmaf(x[k].y, cr[2 * n3 + k], t[2]);
                t[3] = fmaf(x[k].y, cr[3 * n3 + k], t[3]);
                t[4] = fmaf(x[k].x, cr[4 * n3 + k], t[4]);
            }
        }
    }
    if constexpr (CONS) {
        __shared__ double red[kPY][5][32];
        const int lane = threadIdx.x, y = threadIdx.y;
#pragma unroll
        for (int r = 0; r < 5; ++r) red[y][r][lane] = f32_to_f64_bits(t[r]);
        __syncthreads();
        if (y == 0) {
            const long long c = c0 + cell;
            for (int r = 0; r < 5; ++r) {
                double s = 0.;
                for (int yy = 0; yy < kPY; ++yy) s += red[yy][r][lane];
                cons.part[((long long)blockIdx.x * 5 + r) * Bp + c] = s;
            }
        }
    }
}

template <int N>
cudaError_t launch_fq(const float2 *F, const float *C, const FftTw &tw, int Bp, int c0, int Bc, float2 *scratch,
                      int Bs, double2 *q, cudaStream_t st, int stage, float2 *q32, const ConsFused *cons, int form,
                      int *err) {
    constexpr int n = N, M = 3 * N / 2;
    constexpr int NI = N;  // outputs per thread in Y (one pass: X is read once)
    float2 *G = scratch, *H = scratch + (size_t)n * M * M * Bs, *X = scratch + fftq_gh_elems(n, Bs);
    const dim3 blk(32, kPY);
    const int gc = Bc / 32;
    if (form == 1) {
        // axis-3 DFTs into X1 (stage 0); axis-2 DFTs, axis-1 sums and
        // inverse axis-2 DFTs on chip into H (stage 2)
        if (stage < 0 || stage == 0 || stage == 2) {
            const cudaError_t e = launch_fq_fused(n, F, C, tw, Bp, c0, Bc, X, H, Bs, st, stage, err);
            if (e != cudaSuccess) return e;
        }
    } else {
        // X1 and X2 in one pass (stage 1 then has nothing left to do): 16
        // cells per block up to n = 24, 8 at n = 32 (a plane of 16 cells
        // would take 196 KB of shared memory)
        constexpr int CB = (N == 32) ? 8 : 16;
        constexpr int PX = (N == 24) ? 12 : (N == 32 ? 16 : M / 2);
        if (stage < 0 || stage == 0) {
            const size_t smem = sizeof(float2) * n * M * CB;
            const cudaError_t e =
                cudaFuncSetAttribute(k_fq_x12<N, PX, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            k_fq_x12<N, PX, CB><<<dim3(n, Bc / CB, 10), dim3(CB, PX), smem, st>>>(F, C, Bp, c0, X, Bs, tw);
        }
        if (stage < 0 || stage == 2) {
            constexpr int PY = (N >= 32) ? 2 : 4;
            const size_t smem = sizeof(float2) * 2 * 2 * N * 32 * PY;
            // opt-in above 48 KB of dynamic shared memory (per device, so on every call)
            const cudaError_t e = cudaFuncSetAttribute(k_fq_y<N, NI, PY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)smem);
            if (e != cudaSuccess) return e;
            k_fq_y<N, NI, PY><<<dim3((M * M + PY - 1) / PY, gc, N / NI), dim3(32, PY), smem, st>>>(X, Bs, G);
        }
        if (stage < 0 || stage == 3) k_fq_z1<N><<<dim3((n * M + kPY - 1) / kPY, gc, 1), blk, 0, st>>>(G, Bs, H, tw);
    }
    if (stage < 0 || stage == 4) {
        const dim3 g2((n * n + kPY - 1) / kPY, gc, 1);
        if (q32 && cons) k_fq_z2<N, float2, true><<<g2, blk, 0, st>>>(H, Bs, q32, Bp, c0, tw, *cons);
        else if (q32) k_fq_z2<N, float2, false><<<g2, blk, 0, st>>>(H, Bs, q32, Bp, c0, tw, ConsFused{});
        else k_fq_z2<N, double2, false><<<g2, blk, 0, st>>>(H, Bs, q, Bp, c0, tw, ConsFused{});
    }
    return cudaGetLastError();
}

}  // namespace

bool fftq_supported(int n) { return n == 8 || n == 16 || n == 24 || n == 32; }
int fftq_cons_blocks(int n) { return (n * n + kPY - 1) / kPY; }

size_t fftq_gh_elems(int n, int Bs) {
    const size_t M = 3 * (size_t)n / 2;
    return (size_t)n * M * (M + n) * Bs;
}

size_t fftq_scratch_elems(int n, int Bs) {
    const size_t M = 3 * (size_t)n / 2;
    return fftq_gh_elems(n, Bs) + std::max((size_t)13 * n * M * M * Bs, fq_fused_x1_elems(n, Bs));
}

FftTw fftq_twiddles(int n) {
    FftTw t{};
    const int M = 3 * n / 2, S = n / 4;
    const double PI = std::acos(-1.0);
    for (int q2 = 0; q2 < S; ++q2)
        for (int k1 = 0; k1 < 6; ++k1) {
            const double a = -2. * PI * q2 * k1 / M, ph = 2. * PI * k1 / 3.;
            t.fw[q2 * 6 + k1] = make_float2((float)std::cos(a), (float)std::sin(a));
            t.fa[q2 * 6 + k1] = make_float2((float)std::cos(a + ph), (float)std::sin(a + ph));
            t.iv[q2 * 6 + k1] = make_float2((float)(std::cos(a) / M), (float)(-std::sin(a) / M));
        }
    return t;
}

void fftq_coefficients(const double *shat, const double *ahat, const double *cw, double h_eta, int n,
                       std::vector<float> &C) {
    const size_t n3 = (size_t)n * n * n;
    C.assign(7 * n3, 0.f);
    const double h2 = h_eta * h_eta;
    // pairs: (ahat, 1), (S00, u1^2), (S11, u2^2), (S22, u3^2), (S01, u1 u2), (S02, u1 u3), (S12, u2 u3);
    // shat per omega: S00, S01, S02, S11, S12, S22
    static const int sidx[6] = {0, 3, 5, 1, 2, 4};
    static const double mult[6] = {1., 1., 1., 2., 2., 2.};
    for (size_t o = 0; o < n3; ++o) {
        C[o] = (float)(cw[o] * ahat[o]);
        for (int p = 0; p < 6; ++p) C[(p + 1) * n3 + o] = (float)(-mult[p] * h2 * cw[o] * shat[6 * o + sidx[p]]);
    }
}

cudaError_t launch_computeq_fft(const float2 *F, const float *C, const FftTw &tw, int n, int Bp, int c0, int Bc,
                                float2 *scratch, int Bs, double2 *q, cudaStream_t st, int stage, float2 *q32,
                                const ConsFused *cons, int form, int *err) {
    if (Bc <= 0 || Bc % 32 || Bc > Bs || c0 % 32 || c0 + Bc > Bp || stage < -1 || stage > 4)
        return cudaErrorInvalidValue;
    if (cons && (!q32 || !cons->cf || !cons->part)) return cudaErrorInvalidValue;
    if (form != 0 && form != 1) return cudaErrorInvalidValue;
    switch (n) {
    case 8: return launch_fq<8>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st, stage, q32, cons, form, err);
    case 16: return launch_fq<16>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st, stage, q32, cons, form, err);
    case 24: return launch_fq<24>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st, stage, q32, cons, form, err);
    case 32: return launch_fq<32>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st, stage, q32, cons, form, err);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace lp
