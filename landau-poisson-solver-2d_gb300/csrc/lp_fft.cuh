// Register FFT building blocks of the convolution form of ComputeQ (FP32 or
// FP64 complex): three-, four-, six- and S-point DFTs, the forward M-point DFT
// (M = 3n/2 = 6S) of n inputs zero-padded to M, and its inverse keeping the
// first n outputs.  Shared by the convolution kernels of lp_fftq.cu and
// lp_fqf.cu.
#pragma once

namespace lp {
namespace {

// The complex type of a precision (float2 or double2): its real type, a
// constructor and the constants of the small DFTs.  The FP32 constants are
// the float literals themselves, so the FP32 kernels' arithmetic does not
// depend on this template layer.
template <typename C> struct Cx;
template <> struct Cx<float2> {
    using R = float;
    static __device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }
    static constexpr float c3 = 0.866025403784438646763723170752936183f;  // sqrt(3)/2
    static constexpr float r2 = 0.707106781186547524400844362104849039f;  // 1/sqrt(2)
};
template <> struct Cx<double2> {
    using R = double;
    static __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
    static constexpr double c3 = 0.866025403784438646763723170752936183;
    static constexpr double r2 = 0.707106781186547524400844362104849039;
};

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return Cx<C>::mk(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return Cx<C>::mk(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cscale(C a, typename Cx<C>::R s) {
    return Cx<C>::mk(a.x * s, a.y * s);
}
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return Cx<C>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// -i z (forward) or +i z (inverse)
template <bool INV, typename C> __device__ __forceinline__ C rot(C z) {
    return INV ? Cx<C>::mk(-z.y, z.x) : Cx<C>::mk(z.y, -z.x);
}

// Three-point DFT, sign of the exponent negative (forward) or positive.
template <bool INV, typename C> __device__ __forceinline__ void dft3(C a, C b, C c, C &X0, C &X1, C &X2) {
    using R = typename Cx<C>::R;
    const C s = cadd(b, c), d = csub(b, c);
    X0 = cadd(a, s);
    const C t = Cx<C>::mk(a.x - R(0.5) * s.x, a.y - R(0.5) * s.y);
    const C e = cscale(rot<INV>(d), Cx<C>::c3);
    X1 = cadd(t, e);
    X2 = csub(t, e);
}
// the same with c = 0
template <bool INV, typename C> __device__ __forceinline__ void dft3_2(C a, C b, C &X0, C &X1, C &X2) {
    using R = typename Cx<C>::R;
    X0 = cadd(a, b);
    const C t = Cx<C>::mk(a.x - R(0.5) * b.x, a.y - R(0.5) * b.y);
    const C e = cscale(rot<INV>(b), Cx<C>::c3);
    X1 = cadd(t, e);
    X2 = csub(t, e);
}

// Six-point DFT as two three-point DFTs (even / odd inputs).  NIN = 4: the
// inputs x4, x5 are zero.  NOUT = 4: only X0..X3 are formed.
template <bool INV, int NIN, int NOUT, typename C> __device__ __forceinline__ void dft6(const C (&x)[6], C (&X)[6]) {
    using R = typename Cx<C>::R;
    C E0, E1, E2, O0, O1, O2;
    if (NIN == 4) {
        dft3_2<INV>(x[0], x[2], E0, E1, E2);
        dft3_2<INV>(x[1], x[3], O0, O1, O2);
    } else {
        dft3<INV>(x[0], x[2], x[4], E0, E1, E2);
        dft3<INV>(x[1], x[3], x[5], O0, O1, O2);
    }
    const C w1 = Cx<C>::mk(R(0.5), INV ? Cx<C>::c3 : -Cx<C>::c3),
            w2 = Cx<C>::mk(R(-0.5), INV ? Cx<C>::c3 : -Cx<C>::c3);
    const C p1 = cmul(O1, w1), p2 = cmul(O2, w2);
    X[0] = cadd(E0, O0);
    X[1] = cadd(E1, p1);
    X[2] = cadd(E2, p2);
    X[3] = csub(E0, O0);
    if (NOUT == 6) {
        X[4] = csub(E1, p1);
        X[5] = csub(E2, p2);
    }
}

template <bool INV, typename C> __device__ __forceinline__ void dft4(C a, C b, C c, C d, C &X0, C &X1, C &X2, C &X3) {
    const C s0 = cadd(a, c), d0 = csub(a, c), s1 = cadd(b, d), e = rot<INV>(csub(b, d));
    X0 = cadd(s0, s1);
    X2 = csub(s0, s1);
    X1 = cadd(d0, e);
    X3 = csub(d0, e);
}

// In-place S-point DFT, S in {2, 4, 6, 8}.
template <int S, bool INV, typename C> __device__ __forceinline__ void dftS(C (&x)[S]) {
    if constexpr (S == 2) {
        const C a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = csub(a, b);
    } else if constexpr (S == 4) {
        C X0, X1, X2, X3;
        dft4<INV>(x[0], x[1], x[2], x[3], X0, X1, X2, X3);
        x[0] = X0; x[1] = X1; x[2] = X2; x[3] = X3;
    } else if constexpr (S == 6) {
        C X[6];
        dft6<INV, 6, 6>(x, X);
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = X[k];
    } else {
        static_assert(S == 8, "S-point DFT for S in {2, 4, 6, 8}");
        constexpr auto r2 = Cx<C>::r2;
        C E[4], O[4];
        dft4<INV>(x[0], x[2], x[4], x[6], E[0], E[1], E[2], E[3]);
        dft4<INV>(x[1], x[3], x[5], x[7], O[0], O[1], O[2], O[3]);
        const C w1 = Cx<C>::mk(r2, INV ? r2 : -r2), w3 = Cx<C>::mk(-r2, INV ? r2 : -r2);
        const C p[4] = {O[0], cmul(O[1], w1), rot<INV>(O[2]), cmul(O[3], w3)};
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
template <int N, bool PHASE, typename C>
__device__ __forceinline__ void fwd_pencil(const C (&x)[N], C (&X)[3 * N / 2], const C *tw) {
    constexpr int S = N / 4;
    const C z = Cx<C>::mk(0, 0);
    C Y[S][6];
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2) {
        const C in[6] = {x[q2], x[S + q2], x[2 * S + q2], x[3 * S + q2], z, z};
        dft6<false, 4, 6>(in, Y[q2]);
    }
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2)
#pragma unroll
        for (int k1 = 1; k1 < 6; ++k1)
            if (PHASE || q2 > 0) Y[q2][k1] = cmul(Y[q2][k1], tw[q2 * 6 + k1]);
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
        C col[S];
#pragma unroll
        for (int q2 = 0; q2 < S; ++q2) col[q2] = Y[q2][k1];
        dftS<S, false>(col);
#pragma unroll
        for (int k2 = 0; k2 < S; ++k2) X[k1 + 6 * k2] = col[k2];
    }
}

// The same transform handing each output to st(k, value) as soon as it is
// formed (the outputs need no registers of their own).
template <int N, bool PHASE, typename C, typename Store>
__device__ __forceinline__ void fwd_pencil_st(const C (&x)[N], const C *tw, Store st) {
    constexpr int S = N / 4;
    const C z = Cx<C>::mk(0, 0);
    C Y[S][6];
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2) {
        const C in[6] = {x[q2], x[S + q2], x[2 * S + q2], x[3 * S + q2], z, z};
        dft6<false, 4, 6>(in, Y[q2]);
    }
#pragma unroll
    for (int q2 = 0; q2 < S; ++q2)
#pragma unroll
        for (int k1 = 1; k1 < 6; ++k1)
            if (PHASE || q2 > 0) Y[q2][k1] = cmul(Y[q2][k1], tw[q2 * 6 + k1]);
#pragma unroll
    for (int k1 = 0; k1 < 6; ++k1) {
        C col[S];
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
template <int N, typename C>
__device__ __forceinline__ void inv_pencil(const C (&G)[3 * N / 2], C (&x)[N], const C *iv) {
    constexpr int S = N / 4;
    C Z[6][S];
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
        const C in[6] = {Z[0][q2], Z[1][q2], Z[2][q2], Z[3][q2], Z[4][q2], Z[5][q2]};
        C out[6];
        dft6<true, 6, 4>(in, out);
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) x[S * q1 + q2] = out[q1];
    }
}

// (u - h)^e for e in {0, 1, 2}
template <typename R = float> __device__ __forceinline__ R poww(int u, int h, int e) {
    const R d = (R)(u - h);
    return e == 0 ? R(1) : (e == 1 ? d : d * d);
}

}  // namespace
}  // namespace lp
