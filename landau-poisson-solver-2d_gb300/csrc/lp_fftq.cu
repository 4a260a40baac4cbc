// ComputeQ as a sum of seven windowed convolutions (the mixed path in FP32,
// the FP64 path in FP64).
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
//   Z2  inverse axis-3 DFT, only the n outputs xi3 + h, written as FP64
//       (or FP32 for the mixed path's lazily conserved stages).
//
// The shift by h of the output window is the factor exp(2 pi i k h / M) =
// exp(2 pi i k / 3) on the a-side spectra.  The M-point DFTs factor as
// M = 6 S (S = n/4): S six-point DFTs of the 4 non-zero inputs, twiddles,
// six S-point DFTs; the inverse is the conjugate transpose with only 4 of
// the 6 outputs of its last stage kept.  A thread transforms one pencil of
// one cell; the 32 lanes of a warp are 32 cells, so every load and store is
// coalesced on the cell-minor arrays.  The kernels are templates on the real
// type: FP32 for the mixed path (packed f32x2 FMAs in Y), FP64 for the FP64
// path (Y in four output parts, its accumulators in registers).
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
template <typename R, int N, int PY, int CB>
__global__ void __launch_bounds__(CB * PY)
    k_fq_x12(const typename V2<R>::t *__restrict__ F, const R *__restrict__ C, int Bp, int c0,
             typename V2<R>::t *__restrict__ X, int Bs, FftTwT<typename V2<R>::t> tw) {
    lp_grid_wait();
    using Cp = typename V2<R>::t;
    constexpr int n = N, h = N / 2, M = 3 * N / 2;
    extern __shared__ __align__(16) unsigned char x12_smem[];
    Cp *t3 = reinterpret_cast<Cp *>(x12_smem);  // [m][k3][CB]
    const int tx = threadIdx.x, ty = threadIdx.y, l = blockIdx.x, t = blockIdx.z;
    const int cell = blockIdx.y * CB + tx;
    const size_t as = (size_t)n * M * M * Bs, os = (size_t)M * Bs;  // array and k2 strides of X
    {
        // axis-3 DFTs of the (l, m) pencils of array t
        for (int m = ty; m < n; m += PY) {
            const Cp *src = F + ((size_t)l * n + m) * n * Bp + c0 + cell;
            Cp x[N];
            Cp *row = t3 + m * M * CB + tx;
            auto put = [&](int k, Cp v) { row[k * CB] = v; };
            if (t < 7) {
                // n contiguous, 16-byte aligned weights: 16-byte vector loads
                const R *cw = C + (size_t)t * n * n * n + ((size_t)l * n + m) * n;
                if constexpr (std::is_same<R, float>::value) {
                    const float4 *cp = reinterpret_cast<const float4 *>(cw);
#pragma unroll
                    for (int q4 = 0; q4 < n / 4; ++q4) {
                        const float4 w = __ldg(cp + q4);
                        x[4 * q4] = cscale(src[(size_t)(4 * q4) * Bp], w.x);
                        x[4 * q4 + 1] = cscale(src[(size_t)(4 * q4 + 1) * Bp], w.y);
                        x[4 * q4 + 2] = cscale(src[(size_t)(4 * q4 + 2) * Bp], w.z);
                        x[4 * q4 + 3] = cscale(src[(size_t)(4 * q4 + 3) * Bp], w.w);
                    }
                } else {
                    const double2 *cp = reinterpret_cast<const double2 *>(cw);
#pragma unroll
                    for (int q2 = 0; q2 < n / 2; ++q2) {
                        const double2 w = __ldg(cp + q2);
                        x[2 * q2] = cscale(src[(size_t)(2 * q2) * Bp], w.x);
                        x[2 * q2 + 1] = cscale(src[(size_t)(2 * q2 + 1) * Bp], w.y);
                    }
                }
                fwd_pencil_st<N, true>(x, tw.fa, put);
            } else {
#pragma unroll
                for (int q = 0; q < n; ++q) x[q] = cscale(src[(size_t)q * Bp], poww<R>(q, h, t - 7));
                fwd_pencil_st<N, false>(x, tw.fw, put);
            }
        }
        __syncthreads();
        // axis-2 DFTs of the (l, k3) pencils into X
        for (int k3 = ty; k3 < M; k3 += PY) {
            Cp x[N];
#pragma unroll
            for (int m = 0; m < n; ++m) x[m] = t3[(m * M + k3) * CB + tx];
            Cp *dst = X + ((size_t)l * M * M + k3) * Bs + cell;
            if (t < 7) {
                Cp *d = dst + t * as;
                fwd_pencil_st<N, true>(x, tw.fa, [&](int k, Cp v) { d[(size_t)k * os] = v; });
            } else {
                // b-side: the X1 array 7 + e3 gives the combinations (e2, e3)
                // at arrays 7 (0,0), 8 (2,0), 10 (1,0) | 11 (0,1), 12 (1,1) | 9 (0,2)
                const int e3 = t - 7;
                const int no = e3 == 0 ? 3 : (e3 == 1 ? 2 : 1);
                for (int o = 0; o < no; ++o) {
                    const int e2 = e3 == 0 ? (o == 0 ? 0 : (o == 1 ? 2 : 1)) : (e3 == 1 ? o : 0);
                    const int arr = e3 == 0 ? (o == 0 ? 7 : (o == 1 ? 8 : 10)) : (e3 == 1 ? 11 + o : 9);
                    Cp xw[N];
#pragma unroll
                    for (int m = 0; m < n; ++m) xw[m] = e2 ? cscale(x[m], poww<R>(m, h, e2)) : x[m];
                    Cp *d = dst + arr * as;
                    fwd_pencil_st<N, false>(xw, tw.fw, [&](int k, Cp v) { d[(size_t)k * os] = v; });
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
// Complex products use split accumulators (packed FMAs in FP32):
// A += Re(a) b, B += Im(a) b, a b = (A.x - B.y, A.y + B.x).
template <typename R, int N>
__device__ __forceinline__ void y_issue(const typename V2<R>::t *__restrict__ base, size_t ps, int p,
                                        typename V2<R>::t *sm, int nt) {
    const int sy = (p == 0 || p == 1) ? 7 : p + 6;
    auto cpy = [](void *d, const void *g) {
        if constexpr (std::is_same<R, float>::value) cp_async8(d, g);
        else cp_async16(d, g);
    };
#pragma unroll
    for (int u = 0; u < N; ++u) cpy(sm + u * nt, base + ((size_t)sy * N + u) * ps);
#pragma unroll
    for (int l = 0; l < N; ++l) cpy(sm + (N + l) * nt, base + ((size_t)p * N + l) * ps);
    cp_async_commit();
}

template <typename R, int N, int NI, int I0>
__device__ __forceinline__ void y_part(const typename V2<R>::t *__restrict__ base, size_t ps,
                                       typename V2<R>::t *__restrict__ dst, size_t os, typename V2<R>::t *sm,
                                       int nt) {
    using Cp = typename V2<R>::t;
    constexpr int n = N, h = N / 2;
    constexpr bool F32 = std::is_same<R, float>::value;
    // FP32: packed FMAs on (re, im) pairs; FP64: the same products one by one
    using Acc = typename std::conditional<F32, unsigned long long, double2>::type;
    Acc A[NI], B[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) {
        if constexpr (F32) A[i] = B[i] = 0ull;
        else A[i] = B[i] = make_double2(0., 0.);
    }
    y_issue<R, N>(base, ps, 0, sm, nt);
#pragma unroll 1
    for (int p = 0; p < 7; ++p) {
        Cp *cur = sm + (p & 1) * 2 * N * nt;
        if (p + 1 < 7) {
            y_issue<R, N>(base, ps, p + 1, sm + ((p + 1) & 1) * 2 * N * nt, nt);
            cp_async_wait1();
        } else {
            cp_async_wait0();
        }
        const int e1 = (p == 1) ? 2 : ((p == 4 || p == 5) ? 1 : 0);
        Acc yb[N];
#pragma unroll
        for (int u = 0; u < n; ++u) {
            const Cp v = cscale(cur[u * nt], poww<R>(u, h, e1));
            if constexpr (F32) yb[u] = pk2(v.x, v.y);
            else yb[u] = v;
        }
#pragma unroll
        for (int l = 0; l < n; ++l) {
            // outputs i with u = i + h - l in [0, n)
            if (l - h >= I0 + NI || l + h <= I0) continue;
            const Cp a = cur[(N + l) * nt];
            if constexpr (F32) {
                const unsigned long long ar = pk2(a.x, a.x), ai = pk2(a.y, a.y);
#pragma unroll
                for (int ii = 0; ii < NI; ++ii) {
                    const int u = I0 + ii + h - l;
                    if (u >= 0 && u < n) {
                        A[ii] = fma2(ar, yb[u], A[ii]);
                        B[ii] = fma2(ai, yb[u], B[ii]);
                    }
                }
            } else {
#pragma unroll
                for (int ii = 0; ii < NI; ++ii) {
                    const int u = I0 + ii + h - l;
                    if (u >= 0 && u < n) {
                        A[ii].x = fma(a.x, yb[u].x, A[ii].x);
                        A[ii].y = fma(a.x, yb[u].y, A[ii].y);
                        B[ii].x = fma(a.y, yb[u].x, B[ii].x);
                        B[ii].y = fma(a.y, yb[u].y, B[ii].y);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int ii = 0; ii < NI; ++ii) {
        if constexpr (F32) {
            const float2 a = up2(A[ii]), b = up2(B[ii]);
            dst[(size_t)ii * os] = make_float2(a.x - b.y, a.y + b.x);
        } else {
            dst[(size_t)ii * os] = make_double2(A[ii].x - B[ii].y, A[ii].y + B[ii].x);
        }
    }
}

// blockIdx.z selects the part of the outputs, [z NI, (z + 1) NI), when
// NI < N (N / NI in {1, 2, 4}).  G is [n][M][M][Bs].  Dynamic shared memory:
// 2 stages x 2N values x blockDim threads.
template <typename R, int N, int NI, int PY>
__global__ void __launch_bounds__(32 * PY)
    k_fq_y(const typename V2<R>::t *__restrict__ X, int Bs, typename V2<R>::t *__restrict__ G) {
    lp_grid_wait();
    using Cp = typename V2<R>::t;
    static_assert(N % NI == 0 && (N / NI == 1 || N / NI == 2 || N / NI == 4), "one, two or four output parts");
    constexpr int M = 3 * N / 2;
    extern __shared__ __align__(16) unsigned char y_smem[];
    const int pen = blockIdx.x * PY + threadIdx.y;
    if (pen >= M * M) return;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    const size_t ps = (size_t)M * M * Bs;  // stride of the axis-1 index
    const Cp *base = X + (size_t)pen * Bs + cell;
    Cp *dst = G + (size_t)pen * Bs + cell;
    Cp *sm = reinterpret_cast<Cp *>(y_smem) + threadIdx.y * 32 + threadIdx.x;
    constexpr int nt = 32 * PY;
    const int z = blockIdx.z;
    if (z == 0) y_part<R, N, NI, 0>(base, ps, dst, ps, sm, nt);
    if constexpr (N / NI >= 2) {
        if (z == 1) y_part<R, N, NI, NI>(base, ps, dst + (size_t)NI * ps, ps, sm, nt);
    }
    if constexpr (N / NI == 4) {
        if (z == 2) y_part<R, N, NI, 2 * NI>(base, ps, dst + (size_t)2 * NI * ps, ps, sm, nt);
        if (z == 3) y_part<R, N, NI, 3 * NI>(base, ps, dst + (size_t)3 * NI * ps, ps, sm, nt);
    }
}

// Z1: inverse axis-2 DFT of the (i, k3) pencils, outputs xi2 in [0, n).
// H is [n][n][M][Bs].
template <typename R, int N>
__global__ void __launch_bounds__(32 * kPY)
    k_fq_z1(const typename V2<R>::t *__restrict__ G, int Bs, typename V2<R>::t *__restrict__ H,
            FftTwT<typename V2<R>::t> tw) {
    lp_grid_wait();
    using Cp = typename V2<R>::t;
    constexpr int n = N, M = 3 * N / 2;
    const int pen = blockIdx.x * kPY + threadIdx.y;
    if (pen >= n * M) return;
    const int i = pen / M, k3 = pen - i * M;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    const Cp *src = G + ((size_t)i * M * M + k3) * Bs + cell;
    Cp g[M], x[N];
#pragma unroll
    for (int k = 0; k < M; ++k) g[k] = src[(size_t)k * M * Bs];
    inv_pencil<N>(g, x, tw.iv);
    Cp *dst = H + ((size_t)i * n * M + k3) * Bs + cell;
#pragma unroll
    for (int j = 0; j < n; ++j) dst[(size_t)j * M * Bs] = x[j];
}

// Z2: inverse axis-3 DFT of the (i, j) pencils into q (stride Bp), FP64
// or FP32 complex.  CONS (FP32 output): each block's constraint sums of its
// outputs (ConsFused).
template <typename R, int N, typename QT, bool CONS>
__global__ void __launch_bounds__(32 * kPY)
    k_fq_z2(const typename V2<R>::t *__restrict__ H, int Bs, QT *__restrict__ q, int Bp, int c0,
            FftTwT<typename V2<R>::t> tw, ConsFused cons) {
    lp_grid_wait();
    using Cp = typename V2<R>::t;
    static_assert(!CONS || std::is_same<R, float>::value, "the fused sums are those of an FP32 mode array");
    constexpr int n = N, M = 3 * N / 2;
    const int pen = blockIdx.x * kPY + threadIdx.y;
    const int cell = blockIdx.y * 32 + threadIdx.x;
    float t[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (pen < n * n) {
        const Cp *src = H + (size_t)pen * M * Bs + cell;
        Cp g[M], x[N];
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
                cudaFuncSetAttribute(k_fq_x12<float, N, PX, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            k_fq_x12<float, N, PX, CB><<<dim3(n, Bc / CB, 10), dim3(CB, PX), smem, st>>>(F, C, Bp, c0, X, Bs, tw);
        }
        if (stage < 0 || stage == 2) {
            constexpr int PY = (N >= 32) ? 2 : 4;
            const size_t smem = sizeof(float2) * 2 * 2 * N * 32 * PY;
            // opt-in above 48 KB of dynamic shared memory (per device, so on every call)
            const cudaError_t e = cudaFuncSetAttribute(k_fq_y<float, N, NI, PY>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            k_fq_y<float, N, NI, PY><<<dim3((M * M + PY - 1) / PY, gc, N / NI), dim3(32, PY), smem, st>>>(X, Bs, G);
        }
        if (stage < 0 || stage == 3)
            k_fq_z1<float, N><<<dim3((n * M + kPY - 1) / kPY, gc, 1), blk, 0, st>>>(G, Bs, H, tw);
    }
    if (stage < 0 || stage == 4) {
        const dim3 g2((n * n + kPY - 1) / kPY, gc, 1);
        if (q32 && cons) k_fq_z2<float, N, float2, true><<<g2, blk, 0, st>>>(H, Bs, q32, Bp, c0, tw, *cons);
        else if (q32) k_fq_z2<float, N, float2, false><<<g2, blk, 0, st>>>(H, Bs, q32, Bp, c0, tw, ConsFused{});
        else k_fq_z2<float, N, double2, false><<<g2, blk, 0, st>>>(H, Bs, q, Bp, c0, tw, ConsFused{});
    }
    return cudaGetLastError();
}

// The three-pass form in FP64 (the FP64 path): the same kernels at double
// precision.  The axis-1 sums run in four output parts of n / 4 (the FP64
// accumulators and b-values of a full pencil would not fit in registers).
// Dynamic shared memory at n = 24: 216 KB for X1/X2 (16 cells), 192 KB
// for Y.
template <int N>
cudaError_t launch_fq64(const double2 *F, const double *C, const FftTw64 &tw, int Bp, int c0, int Bc,
                        double2 *scratch, int Bs, double2 *q, cudaStream_t st) {
    constexpr int n = N, M = 3 * N / 2, NI = N / 4;
    double2 *G = scratch, *H = scratch + (size_t)n * M * M * Bs, *X = scratch + fftq_gh_elems(n, Bs);
    const dim3 blk(32, kPY);
    const int gc = Bc / 32;
    {
        constexpr int CB = (N == 32) ? 8 : 16;
        constexpr int PX = (N == 24) ? 12 : (N == 32 ? 16 : M / 2);
        const size_t smem = sizeof(double2) * n * M * CB;
        const cudaError_t e =
            cudaFuncSetAttribute(k_fq_x12<double, N, PX, CB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_fq_x12<double, N, PX, CB><<<dim3(n, Bc / CB, 10), dim3(CB, PX), smem, st>>>(F, C, Bp, c0, X, Bs, tw);
    }
    {
        constexpr int PY = (N >= 32) ? 2 : 4;
        const size_t smem = sizeof(double2) * 2 * 2 * N * 32 * PY;
        const cudaError_t e =
            cudaFuncSetAttribute(k_fq_y<double, N, NI, PY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_fq_y<double, N, NI, PY><<<dim3((M * M + PY - 1) / PY, gc, N / NI), dim3(32, PY), smem, st>>>(X, Bs, G);
    }
    k_fq_z1<double, N><<<dim3((n * M + kPY - 1) / kPY, gc, 1), blk, 0, st>>>(G, Bs, H, tw);
    k_fq_z2<double, N, double2, false>
        <<<dim3((n * n + kPY - 1) / kPY, gc, 1), blk, 0, st>>>(H, Bs, q, Bp, c0, tw, ConsFused{});
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

size_t fftq_scratch_elems64(int n, int Bs) {
    const size_t M = 3 * (size_t)n / 2;
    return fftq_gh_elems(n, Bs) + (size_t)13 * n * M * M * Bs;
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

FftTw64 fftq_twiddles64(int n) {
    FftTw64 t{};
    const int M = 3 * n / 2, S = n / 4;
    const double PI = std::acos(-1.0);
    for (int q2 = 0; q2 < S; ++q2)
        for (int k1 = 0; k1 < 6; ++k1) {
            const double a = -2. * PI * q2 * k1 / M, ph = 2. * PI * k1 / 3.;
            t.fw[q2 * 6 + k1] = make_double2(std::cos(a), std::sin(a));
            t.fa[q2 * 6 + k1] = make_double2(std::cos(a + ph), std::sin(a + ph));
            t.iv[q2 * 6 + k1] = make_double2(std::cos(a) / M, -std::sin(a) / M);
        }
    return t;
}

namespace {
template <typename T>
void coefficients(const double *shat, const double *ahat, const double *cw, double h_eta, int n, std::vector<T> &C) {
    const size_t n3 = (size_t)n * n * n;
    C.assign(7 * n3, T(0));
    const double h2 = h_eta * h_eta;
    // pairs: (ahat, 1), (S00, u1^2), (S11, u2^2), (S22, u3^2), (S01, u1 u2), (S02, u1 u3), (S12, u2 u3);
    // shat per omega: S00, S01, S02, S11, S12, S22
    static const int sidx[6] = {0, 3, 5, 1, 2, 4};
    static const double mult[6] = {1., 1., 1., 2., 2., 2.};
    for (size_t o = 0; o < n3; ++o) {
        C[o] = (T)(cw[o] * ahat[o]);
        for (int p = 0; p < 6; ++p) C[(p + 1) * n3 + o] = (T)(-mult[p] * h2 * cw[o] * shat[6 * o + sidx[p]]);
    }
}
}  // namespace

void fftq_coefficients(const double *shat, const double *ahat, const double *cw, double h_eta, int n,
                       std::vector<float> &C) {
    coefficients(shat, ahat, cw, h_eta, n, C);
}

void fftq_coefficients64(const double *shat, const double *ahat, const double *cw, double h_eta, int n,
                         std::vector<double> &C) {
    coefficients(shat, ahat, cw, h_eta, n, C);
}

cudaError_t launch_computeq_fft64(const double2 *F, const double *C, const FftTw64 &tw, int n, int Bp, int c0,
                                  int Bc, double2 *scratch, int Bs, double2 *q, cudaStream_t st) {
    if (Bc <= 0 || Bc % 32 || Bc > Bs || c0 % 32 || c0 + Bc > Bp) return cudaErrorInvalidValue;
    switch (n) {
    case 8: return launch_fq64<8>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st);
    case 16: return launch_fq64<16>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st);
    case 24: return launch_fq64<24>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st);
    case 32: return launch_fq64<32>(F, C, tw, Bp, c0, Bc, scratch, Bs, q, st);
    default: return cudaErrorInvalidValue;
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
