// Register FFT building blocks of the convolution form of ComputeQ (FP32
// complex): three-, four-, six- and S-point DFTs, the forward M-point DFT
// (M = 3n/2 = 6S) of n inputs zero-padded to M, and its inverse keeping the
// first n outputs.  Shared by the convolution kernels of lp_fftq.cu and
// lp_fqf.cu.
#pragma once

namespace lp {
namespace {

constexpr float kC3 = 0.866025403784438646763723170752936183f;  // sqrt(3)/2
constexpr float kR2 = 0.707106781186547524400844362104849039f;  // 1/sqrt(2)

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// -i z (forward) or +i z (inverse)
template <bool INV> __device__ __forceinline__ float2 rot(float2 z) {
    return INV ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x);
}

// Three-point DFT, sign of the exponent negative (forward) or positive.
template <bool INV> __device__ __forceinline__ void dft3(float2 a, float2 b, float2 c, float2 &X0, float2 &X1,
                                                         float2 &X2) {
    const float2 s = cadd(b, c), d = csub(b, c);
    X0 = cadd(a, s);
    const float2 t = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
    const float2 e = cscale(rot<INV>(d), kC3);
    X1 = cadd(t, e);
    X2 = csub(t, e);
}
// the same with c = 0
template <bool INV> __device__ __forceinline__ void dft3_2(float2 a, float2 b, float2 &X0, float2 &X1, float2 &X2) {
    X0 = cadd(a, b);
    const float2 t = make_float2(a.x - 0.5f * b.x, a.y - 0.5f * b.y);
    const float2 e = cscale(rot<INV>(b), kC3);
    X1 = cadd(t, e);
    X2 = csub(t, e);
}

// Six-point DFT as two three-point DFTs (even / odd inputs).  NIN = 4: the
// inputs x4, x5 are zero.  NOUT = 4: only X0..X3 are formed.
template <bool INV, int NIN, int NOUT> __device__ __forceinline__ void dft6(const float2 (&x)[6], float2 (&X)[6]) {
    float2 E0, E1, E2, O0, O1, O2;
    if (NIN == 4) {
        dft3_2<INV>(x[0], x[2], E0, E1, E2);
        dft3_2<INV>(x[1], x[3], O0, O1, O2);
    } else {
        dft3<INV>(x[0], x[2], x[4], E0, E1, E2);
        dft3<INV>(x[1], x[3], x[5], O0, O1, O2);
    }
    const float2 w1 = make_float2(0.5f, INV ? kC3 : -kC3), w2 = make_float2(-0.5f, INV ? kC3 : -kC3);
    const float2 p1 = cmul(O1, w1), p2 = cmul(O2, w2);
    X[0] = cadd(E0, O0);
    X[1] = cadd(E1, p1);
    X[2] = cadd(E2, p2);
    X[3] = csub(E0, O0);
    if (NOUT == 6) {
        X[4] = csub(E1, p1);
        X[5] = csub(E2, p2);
    }
}

template <bool INV> __device__ __forceinline__ void dft4(float2 a, float2 b, float2 c, float2 d, float2 &X0,
                                                         float2 &X1, float2 &X2, float2 &X3) {
    const float2 s0 = cadd(a, c), d0 = csub(a, c), s1 = cadd(b, d), e = rot<INV>(csub(b, d));
    X0 = cadd(s0, s1);
    X2 = csub(s0, s1);
    X1 = cadd(d0, e);
    X3 = csub(d0, e);
}

// In-place S-point DFT, S in {2, 4, 6, 8}.
template <int S, bool INV> __device__ __forceinline__ void dftS(float2 (&x)[S]) {
    if constexpr (S == 2) {
        const float2 a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = csub(a, b);
    } else if constexpr (S == 4) {
        float2 X0, X1, X2, X3;
        dft4<INV>(x[0], x[1], x[2], x[3], X0, X1, X2, X3);
        x[0] = X0; x[1] = X1; x[2] = X2; x[3] = X3;
    } else if constexpr (S == 6) {
        float2 X[6];
        dft6<INV, 6, 6>(x, X);
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = X[k];
    } else {
        static_assert(S == 8, "S-point DFT for S in {2, 4, 6, 8}");
        float2 E[4], O[4];
        dft4<INV>(x[0], x[2], x[4], x[6], E[0], E[1], E[2], E[3]);
        dft4<INV>(x[1], x[3], x[5], x[7], O[0], O[1], O[2], O[3]);
        const float2 w1 = make_float2(kR2, INV ? kR2 : -kR2), w3 = make_float2(-kR2, INV ? kR2 : -kR2);
        const float2 p[4] = {O[0], cmul(O[1], w1), rot<INV>(O[2]), cmul(O[3], w3)};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x[k] = cadd(E[k], p[k]);
            x[k + 4] = csub(E[k], p[k]);
        }
    }
}

// Forward M-point DFT (M = 3n/2 = 6S) of n inputs zero-padded to M:
// X[k1 + 6 k2] = sum_q2 exp(-2 pi i q2 k2 / S) tw[q2][k1]
//                sum_q1 x[S q1 + q2] exp(-2 pi i q1 k1 / 6).
// tw is exp(-2 pi i q2 k1 / M), times exp(2 pi i k1 / 3) on the a-side.
template <int N, bool PHASE> __device__ __forceinline__ void fwd_pencil(const float2 (&x)[N],
                                                                        float2 (&X)[3 * N / 2],
                                                                        const float2 *tw) {
    constexpr int S = N / 4;
    float2 Y[S][6];
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2) {
        const float2 in[6] = {x[q2], x[S + q2], x[2 * S + q2], x[3 * S + q2], make_float2(0.f, 0.f),
                              make_float2(0.f, 0.f)};
        dft6<false, 4, 6>(in, Y[q2]);
    }
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2)
#pragma unroll
        for (int k1 = 1; k1 < 6; ++k1)
            if (PHASE || q2 > 0) Y[q2][k1] = cmul(Y[q2][k1], tw[q2 * 6 + k1]);
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
        float2 col[S];
#pragma unroll
        for (int q2 = 0; q2 < S; ++q2) col[q2] = Y[q2][k1];
        dftS<S, false>(col);
#pragma unroll
        for (int k2 = 0; k2 < S; ++k2) X[k1 + 6 * k2] = col[k2];
    }
}

// The same transform handing each output to st(k, value) as soon as it is
// formed (the outputs need no registers of their own).
template <int N, bool PHASE, typename Store>
__device__ __forceinline__ void fwd_pencil_st(const float2 (&x)[N], const float2 *tw, Store st) {
    constexpr int S = N / 4;
    float2 Y[S][6];
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2) {
        const float2 in[6] = {x[q2], x[S + q2], x[2 * S + q2], x[3 * S + q2], make_float2(0.f, 0.f),
                              make_float2(0.f, 0.f)};
        dft6<false, 4, 6>(in, Y[q2]);
    }
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2)
#pragma unroll
        for (int k1 = 1; k1 < 6; ++k1)
            if (PHASE || q2 > 0) Y[q2][k1] = cmul(Y[q2][k1], tw[q2 * 6 + k1]);
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
        float2 col[S];
#pragma unroll
        for (int q2 = 0; q2 < S; ++q2) col[q2] = Y[q2][k1];
        dftS<S, false>(col);
#pragma unroll
        for (int k2 = 0; k2 < S; ++k2) st(k1 + 6 * k2, col[k2]);
    }
}

// Inverse: x[s] = sum_k G[k] exp(2 pi i k s / M) / M for s in [0, n), the
// conjugate transpose of fwd_pencil without the phase; iv holds
// conj(tw[q2][k1]) / M.
template <int N> __device__ __forceinline__ void inv_pencil(const float2 (&G)[3 * N / 2], float2 (&x)[N],
                                                            const float2 *iv) {
    constexpr int S = N / 4;
    float2 Z[6][S];
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
#pragma unroll
        for (int k2 = 0; k2 < S; ++k2) Z[k1][k2] = G[k1 + 6 * k2];
        dftS<S, true>(Z[k1]);
    }
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1)
#pragma unroll
        for (int q2 = 0; q2 < S; ++q2) Z[k1][q2] = cmul(Z[k1][q2], iv[q2 * 6 + k1]);
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2) {
        const float2 in[6] = {Z[0][q2], Z[1][q2], Z[2][q2], Z[3][q2], Z[4][q2], Z[5][q2]};
        float2 out[6];
        dft6<true, 6, 4>(in, out);
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) x[S * q1 + q2] = out[q1];
    }
}

// (u - h)^e for e in {0, 1, 2}
__device__ __forceinline__ float poww(int u, int h, int e) {
    const float d = (float)(u - h);
    return e == 0 ? 1.f : (e == 1 ? d : d * d);
}

}  // namespace
}  // namespace lp
